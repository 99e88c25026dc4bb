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
