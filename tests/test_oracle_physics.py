"""The oracle's rain physics against an independent float64 restatement.

The oracle restates rs.cl in FP32 operation for operation; nothing from the
reference runs here, so its advance path has no golden vectors.  This file
restates the same kernels once more, in float64 numpy, straight from the
mathematics of rs.cl (wind_table_index rs.cl:123-176, read_imagef with the
clamp-to-edge linear sampler rs.cl:8, bg_atts rs.cl:533-580, el_atts
rs.cl:653-739, compute_ellipsoid_rcs rs.cl:268-280, rand rs.cl:35-44), and
checks that the oracle's FP32 step agrees within FP32 rounding: a
transcription error in the oracle (a wrong index, sign, constant or lane)
shows up as a gross difference.  Scatterers within a rounding distance of a
decision (the box faces, a table cell edge) are left out of the comparison.
"""
import math

import numpy as np
import pytest

from simradar_gb300 import synth


def wind_index64(pos, wd, sd):
    """Stretched grid: copysign(s0-2, p_rel) log1p(s4-6 |p_rel|) + s8-10,
    p_rel relative to the box centre in x and y, to 0 in z."""
    c = np.array([sd[8] + 0.5 * sd[12], sd[9] + 0.5 * sd[13], 0.0])
    prel = pos[:, :3].astype(np.float64) - c
    w = wd.astype(np.float64)
    return np.copysign(w[0:3], prel) * np.log1p(w[4:7] * np.abs(prel)) + w[8:11]


def read_image3d64(vol, coord):
    """read_imagef, unnormalised coordinates, CLK_ADDRESS_CLAMP_TO_EDGE,
    CLK_FILTER_LINEAR: i0 = floor(u - 0.5), weight frac(u - 0.5)."""
    nz, ny, nx = vol.shape[:3]
    out = np.zeros((coord.shape[0], 4))
    idx, wts = [], []
    for u, n in zip(coord.T, (nx, ny, nz)):
        t = u - 0.5
        i0 = np.floor(t)
        a = t - i0
        i0 = i0.astype(np.int64)
        idx.append((np.clip(i0, 0, n - 1), np.clip(i0 + 1, 0, n - 1)))
        wts.append((1.0 - a, a))
    v = vol.astype(np.float64)
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = wts[0][dx] * wts[1][dy] * wts[2][dz]
                out += w[:, None] * v[idx[2][dz], idx[1][dy], idx[0][dx]]
    return out


def ellipsoid_rcs64(pos, table, desc):
    """Nearest table entry by radius, then (hh, hh + (vv - hh) cos^2 beta),
    beta the elevation of the scatterer.  The entry is an integer decision on
    fma(radius, s0, s1) in FP32 (the radii sit on the table's nodes), so the
    index is formed as the reference forms it: one FP32 rounding of the exact
    product-sum."""
    fma32 = (pos[:, 3].astype(np.float64) * np.float64(desc[0]) + np.float64(desc[1])).astype(np.float32)
    fidx = np.clip(fma32.astype(np.float64), 0.0, float(desc[2]))
    idx = fidx.astype(np.int64)
    xz = table[idx].astype(np.float64)
    beta = np.arctan2(pos[:, 2], np.hypot(pos[:, 0], pos[:, 1]))
    cb2 = np.cos(beta) ** 2
    return np.stack([xz[:, 0], xz[:, 1], xz[:, 0] + (xz[:, 2] - xz[:, 0]) * cb2,
                     xz[:, 1] + (xz[:, 3] - xz[:, 1]) * cb2], axis=1), fidx


def rand64(seed):
    """seed = (seed * 16807) & 0x7fffffff lane by lane; value seed / (2^31 - 1)."""
    s = (seed.astype(np.uint64) * np.uint64(16807)) & np.uint64(0x7FFFFFFF)
    return s.astype(np.uint32), s.astype(np.float64) / 2147483647.0


def outside64(p, sd):
    o = np.array(sd[8:11], np.float64)
    e = o + np.array(sd[12:15], np.float64)
    return np.any((p[:, :3] <= o) | (p[:, :3] >= e), axis=1)


def near_face(p, sd, tol):
    o = np.array(sd[8:11], np.float64)
    e = o + np.array(sd[12:15], np.float64)
    return np.any((np.abs(p[:, :3] - o) < tol) | (np.abs(p[:, :3] - e) < tol), axis=1)


def step64(S, state, sd, dragged, bounded, p_look):
    """One bg_atts / el_atts step of every background scatterer in float64.
    The wind is looked up at p_look: the oracle's FP32 positions, so that the
    rounding of the position (0.12 mm at 2 km, a 6e-5 texel shift) does not
    move the lookup; the position update is compared on its own."""
    pos = state["pos"].astype(np.float64)
    vel = state["vel"].astype(np.float64)
    dt = float(sd[11])
    p = pos.copy()
    p[:, :3] += vel[:, :3] * dt
    out = outside64(p, sd)
    seed, r = rand64(state["rnd"])
    resp = p.copy()
    resp[:, :3] = r[:, :3] * np.array(sd[12:15], np.float64) + np.array(sd[8:11], np.float64)
    bg = read_image3d64(S.les[0].uvwt, wind_index64(p_look, S.les_desc, sd))
    if dragged:
        dv = bg - vel
        dva = np.linalg.norm(dv[:, :3], axis=1)
        re = 6.7308e4 * (2.0 * p[:, 3]) * dva
        with np.errstate(divide="ignore", invalid="ignore"):
            cd = 24.0 / re + 6.0 / (1.0 + np.sqrt(re)) + 0.4
        k = 0.5 * 1.225 * cd * (0.003006012 / p[:, 3]) * dva
        dudt = k[:, None] * dv + np.array([0.0, 0.0, -9.8, 0.0])
        v = vel.copy()
        v[:, :3] += dudt[:, :3] * dt
        if bounded:
            big = np.linalg.norm(v, axis=1) > np.maximum(1.0, 3.0 * np.linalg.norm(bg, axis=1))
            v[big, :3] = bg[big, :3] + np.array([0.0, 0.0, -9.8]) * dt
            v[big, 3] = bg[big, 3]
        slow = dva <= 1.0e-3
        v[slow, :3] = vel[slow, :3] + np.array([0.0, 0.0, -9.8]) * dt
        v[slow, 3] = vel[slow, 3]
    else:
        v = bg
    rcs, fidx = ellipsoid_rcs64(p_look, S.ell, S.ell_desc)
    return p, v, rcs, out, resp, seed, fidx


@pytest.mark.parametrize("concept", [synth.CONCEPT_DBU, 0])
def test_rain_step_against_float64(oracle_lib, concept):
    O = oracle_lib
    S = synth.make_scene(num_rain=20000, les_count=1, concept=concept, seed=99)
    # give the scatterers a velocity so that drag, bounding and respawn all occur
    rng = np.random.default_rng(5)
    S.state["vel"][:, :3] = rng.uniform(-30.0, 30.0, (S.num_scats, 3)).astype(np.float32)
    S.state["pos"][:200, 0] = np.float32(S.box[0] + 0.01)
    S.state["vel"][:200, 0] = -20.0
    sd = synth.pulse_sim_desc(S, 3)
    st = O.OracleState(S.state)
    O.advance_time(st, S, S.counts, S.les[0], sd)
    dragged = bool(concept & synth.CONCEPT_DRAGGED)
    bounded = bool(concept & synth.CONCEPT_BOUNDED)
    p, v, rcs, out, resp, seed, fidx = step64(S, S.state, sd, dragged, bounded, st.s["pos"].astype(np.float64))
    skip = near_face(p, sd, 1e-3)
    assert out.sum() >= 150 and (~out & ~skip).sum() > 15000
    # respawned: positions from the RNG, velocity zero, seed advanced, rcs kept
    m = out & ~skip
    assert np.array_equal(st.s["rnd"][m], seed[m])
    assert np.allclose(st.s["pos"][m, :3], resp[m, :3], rtol=1e-6, atol=1e-3)
    assert np.all(st.s["vel"][m] == 0.0)
    assert np.array_equal(st.s["rcs"][m], S.state["rcs"][m])
    # advected: position, velocity and backscatter within FP32 rounding
    m = ~out & ~skip
    assert np.array_equal(st.s["rnd"][m], S.state["rnd"][m])
    assert np.allclose(st.s["pos"][m], p[m], rtol=1e-6, atol=1e-4)
    dv = np.abs(st.s["vel"][m] - v[m])
    assert np.all(dv <= 1e-4 * np.abs(v[m]) + 2e-4), "velocity: max diff %g" % dv.max()
    dr = np.abs(st.s["rcs"][m] - rcs[m])
    assert np.all(dr <= 1e-5 * np.abs(rcs[m]).max(axis=1, keepdims=True) + 1e-30), "rcs: max diff %g" % dr.max()


def test_wind_lookup_against_float64(oracle_lib):
    """bg_atts returns the wind itself (vel = read_imagef(uvwt, index)): the
    LES index and the trilinear filter against float64 over a spread of
    positions, including ones outside the LES domain (edge clamping)."""
    O = oracle_lib
    S = synth.make_scene(num_rain=5000, les_count=1, concept=0, seed=3)
    ox, oy, oz, sx, sy, sz = S.box
    rng = np.random.default_rng(7)
    S.state["pos"][:, 0] = rng.uniform(ox + 1, ox + sx - 1, S.num_scats)
    S.state["pos"][:, 1] = rng.uniform(oy + 1, oy + sy - 1, S.num_scats)
    S.state["pos"][:, 2] = rng.uniform(oz + 1, oz + sz - 1, S.num_scats)
    S.state["vel"][:] = 0.0
    sd = synth.pulse_sim_desc(S, 0)
    st = O.OracleState(S.state)
    O.advance_time(st, S, S.counts, S.les[0], sd)
    ref = read_image3d64(S.les[0].uvwt, wind_index64(st.s["pos"], S.les_desc, sd))
    d = np.abs(st.s["vel"] - ref)
    assert np.all(d <= 1e-5 * np.abs(ref).max() + 1e-6), "wind: max diff %g" % d.max()
    assert math.isfinite(float(d.max()))


# ---------------------------------------------------------------- debris
def qmul(l, r):
    """quat_mult (rs.cl:54-60), (x, y, z, w) rows."""
    lx, ly, lz, lw = l.T
    rx, ry, rz, rw = r.T
    return np.stack([lw * rx - lz * ry + ly * rz + lx * rw,
                     lw * ry + lz * rx + ly * rw - lx * rz,
                     lw * rz + lz * rw - ly * rx + lx * ry,
                     lw * rw - lz * rz - ly * ry - lx * rx], axis=1)


def qconj(q):
    return q * np.array([-1.0, -1.0, -1.0, 1.0])


def qrot(v, q):
    return qmul(qmul(q, v), qconj(q))


def normalize4(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def read_image2d64(img, u, v):
    ny, nx = img.shape[:2]
    out = np.zeros((u.shape[0], 4))
    idx, wts = [], []
    for c, n in ((u, nx), (v, ny)):
        t = c - 0.5
        i0 = np.floor(t)
        a = t - i0
        i0 = i0.astype(np.int64)
        idx.append((np.clip(i0, 0, n - 1), np.clip(i0 + 1, 0, n - 1)))
        wts.append((1.0 - a, a))
    im = img.astype(np.float64)
    for dx in (0, 1):
        for dy in (0, 1):
            out += (wts[0][dx] * wts[1][dy])[:, None] * im[idx[1][dy], idx[0][dx]]
    return out


def debris_rcs64(pos, ori, re, im, rd, cross_pol):
    """compute_debris_rcs (rs.cl:282-359)."""
    el = np.arctan2(pos[:, 2], np.hypot(pos[:, 0], pos[:, 1]))
    az = np.arctan2(pos[:, 0], pos[:, 1])
    se, ce = np.sin(0.5 * (el + np.pi / 2)), np.cos(0.5 * (el + np.pi / 2))
    sa, ca = np.sin(0.5 * az), np.cos(0.5 * az)
    oc = (np.stack([-se, ce, se, ce], axis=1) * ca[:, None] + np.stack([ce, se, ce, -se], axis=1) * sa[:, None]) \
        * math.sqrt(0.5)
    R = qmul(ori, oc)
    q = np.stack([R[:, 0], R[:, 2], -R[:, 1], R[:, 3]], axis=1)
    qx, qy, qz, qw = q.T
    barg = qw * qw + qz * qz - qy * qy - qx * qx
    lump = (barg > 0.999847) | (barg < -0.999847)
    alpha = np.where(lump, 0.0, np.arctan2(qy * qz - qw * qx, qx * qz + qw * qy))
    beta = np.where(lump, 0.0, np.arccos(np.clip(barg, -1, 1)))
    gamma = np.where(lump, np.sign(qz) * np.arccos(np.clip(qw, -1, 1)) * 2.0,
                     np.arctan2(qy * qz + qw * qx, qw * qy - qx * qz))
    u = alpha * rd[0] + rd[4]
    v = beta * rd[1] + rd[5]
    r_, i_ = read_image2d64(re, u, v), read_image2d64(im, u, v)
    cg, sg = np.cos(gamma), np.sin(gamma)
    hh_r = cg * (cg * r_[:, 0] - r_[:, 2] * sg) - sg * (cg * r_[:, 2] - r_[:, 1] * sg)
    hh_i = cg * (cg * i_[:, 0] - i_[:, 2] * sg) - sg * (cg * i_[:, 2] - i_[:, 1] * sg)
    vv_r = cg * (cg * r_[:, 1] + r_[:, 2] * sg) + sg * (cg * r_[:, 2] + r_[:, 0] * sg)
    vv_i = cg * (cg * i_[:, 1] + i_[:, 2] * sg) + sg * (cg * i_[:, 2] + i_[:, 0] * sg)
    ss = np.stack([hh_r, hh_i, vv_r, vv_i], axis=1)
    if cross_pol:
        hv_r = cg * (cg * r_[:, 2] + r_[:, 0] * sg) - sg * (cg * r_[:, 1] + r_[:, 2] * sg)
        hv_i = cg * (cg * i_[:, 2] + i_[:, 0] * sg) - sg * (cg * i_[:, 1] + i_[:, 2] * sg)
        vh_r = cg * (cg * r_[:, 2] - r_[:, 1] * sg) + sg * (cg * r_[:, 0] - r_[:, 2] * sg)
        vh_i = cg * (cg * i_[:, 2] - i_[:, 1] * sg) + sg * (cg * i_[:, 0] - i_[:, 2] * sg)
        ss = ss + np.stack([vh_r, vh_i, hv_r, hv_i], axis=1)
    near = np.abs(np.abs(barg) - 0.999847) < 1e-5
    return ss, near


@pytest.mark.parametrize("concept", [synth.CONCEPT_DBU, synth.CONCEPT_DBU | synth.CONCEPT_CROSS_POL])
def test_debris_step_against_float64(oracle_lib, concept):
    """db_atts (rs.cl:744-907) for scatterers that are not respawned: the
    attitude update, the ADM force and torque (compute_dudt_dwdt
    rs.cl:195-261), the bounded velocity, the tumble and the debris RCS,
    against float64; lookups at the oracle's FP32 position and attitude."""
    O = oracle_lib
    S = synth.make_scene(num_rain=16, debris=[(synth.OBJ_LEAF, 3000), (synth.OBJ_BRICK, 3000)], les_count=1,
                         concept=concept, seed=11)
    rng = np.random.default_rng(8)
    n = S.num_scats
    S.state["vel"][:, :3] = rng.uniform(-15.0, 15.0, (n, 3)).astype(np.float32)
    q = rng.standard_normal((n, 4))
    S.state["ori"][:] = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    t = np.concatenate([rng.normal(0, 0.02, (n, 3)), np.ones((n, 1))], axis=1)
    S.state["tum"][:] = (t / np.linalg.norm(t, axis=1, keepdims=True)).astype(np.float32)
    sd = synth.pulse_sim_desc(S, 5)
    st = O.OracleState(S.state)
    O.advance_time(st, S, S.counts, S.les[0], sd)
    dt = float(sd[11])
    cross = bool(concept & synth.CONCEPT_CROSS_POL)
    origin = S.counts[0]
    for t_i, cnt in enumerate(S.counts[1:]):
        sl = slice(origin, origin + cnt)
        origin += cnt
        cd_img, cm_img, ad = S.adm[t_i]
        re, im, rd = S.rcs_tables[t_i]
        pos0 = S.state["pos"][sl].astype(np.float64)
        vel0 = S.state["vel"][sl].astype(np.float64)
        ori_in = S.state["ori"][sl].astype(np.float64)
        tum_in = S.state["tum"][sl].astype(np.float64)
        ori = normalize4(qmul(ori_in, tum_in))
        p = pos0.copy()
        p[:, :3] += vel0[:, :3] * dt
        out = outside64(p, sd) | near_face(p, sd, 1e-3)
        P32, O32 = st.s["pos"][sl].astype(np.float64), st.s["ori"][sl].astype(np.float64)
        assert np.allclose(O32[~out], ori[~out], rtol=0, atol=2e-6)
        assert np.allclose(P32[~out], p[~out], rtol=1e-6, atol=1e-4)
        bg = read_image3d64(S.les[0].uvwt, wind_index64(P32, S.les_desc, sd))
        ur = bg - vel0
        uh = qrot(normalize4(ur), qconj(O32))
        beta = np.arccos(np.clip(uh[:, 0], -1, 1))
        alpha = np.arctan2(uh[:, 2], uh[:, 1])
        neg = alpha < 0
        alpha = np.where(neg, np.pi + alpha, alpha)
        beta = np.where(neg, -beta, beta)
        cd = read_image2d64(cd_img, beta * ad[0] + ad[4], alpha * ad[1] + ad[5])
        cm = read_image2d64(cm_img, beta * ad[0] + ad[4], alpha * ad[1] + ad[5])
        Ta = float(ad[15])
        u2 = np.sum(ur[:, :3] ** 2, axis=1)
        dudt = Ta * u2[:, None] * qrot(cd, O32) + np.array([0.0, 0.0, -9.8, 0.0])
        inv = np.array([ad[12], ad[13], ad[14], 0.0], np.float64)
        dwdt = np.radians(Ta * u2[:, None] * inv * cm)
        vxy = vel0[:, :2] + dudt[:, :2] * dt
        lhs, rhs = np.linalg.norm(vxy, axis=1), 3.0 * np.linalg.norm(bg[:, :2], axis=1)
        bnd = lhs > rhs
        vel = vel0 + dudt * np.array([dt, dt, dt, 0.0])
        vel[bnd, :2] = bg[bnd, :2]
        dw = dwdt * np.array([dt, dt, dt, 0.0])
        c, s = np.cos(dw), np.sin(dw)
        tum = normalize4(np.stack([c[:, 0] * s[:, 1] * s[:, 2] + s[:, 0] * c[:, 1] * c[:, 2],
                                   c[:, 0] * s[:, 1] * c[:, 2] - s[:, 0] * c[:, 1] * s[:, 2],
                                   c[:, 0] * c[:, 1] * s[:, 2] + s[:, 0] * s[:, 1] * c[:, 2],
                                   c[:, 0] * c[:, 1] * c[:, 2] - s[:, 0] * s[:, 1] * s[:, 2]], axis=1))
        rcs, near = debris_rcs64(P32, O32, re, im, rd, cross)
        # leave out rounding-sized neighbourhoods of the branch decisions
        ill = (np.abs(uh[:, 0]) > 0.9999) | (np.abs(np.arctan2(uh[:, 2], uh[:, 1])) < 1e-4) | \
            (np.abs(lhs - rhs) < 1e-4 * (rhs + 1e-3)) | near
        m = ~out & ~ill
        assert m.sum() > 0.8 * cnt
        V, T, X = st.s["vel"][sl][m], st.s["tum"][sl][m], st.s["rcs"][sl][m]
        dv = np.abs(V - vel[m])
        assert np.all(dv <= 1e-5 * np.abs(vel[m]) + 1e-4), "type %d velocity: max diff %g" % (t_i, dv.max())
        assert np.all(np.abs(T - tum[m]) <= 1e-5), "type %d tumble: max diff %g" % (t_i, np.abs(T - tum[m]).max())
        scale = np.abs(rcs[m]).max(axis=1, keepdims=True) + 1e-30
        dx = np.abs(X - rcs[m]) / scale
        assert np.all(dx <= 1e-3), "type %d rcs: max rel diff %g" % (t_i, dx.max())
