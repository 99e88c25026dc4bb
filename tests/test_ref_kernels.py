"""The oracle's kernels against the reference's own rs.cl (CPU tests).

oracle/ref/Makefile compiles the reference's kernel source rs.cl itself,
unmodified, as C++ through oracle/ref/clc/opencl_c.hpp (vector types,
swizzles, built-ins, the linear clamp-to-edge sampler, work groups meeting at
barriers).  The built-ins whose results the OpenCL specification leaves to
the device (the elementary functions, length, normalize, the filter's
arithmetic) are fixed as the oracle fixes them; everything rs.cl spells out
-- operation order, constants, branches, lane arithmetic, the reduction trees
of the pulse -- is the reference's own.  These tests run both on the same
inputs and require the same bits:

  * every advance kernel (el_atts, bg_atts, fp_atts, db_atts with the three
    debris-flux-field placements, db_rcs) over several steps with respawns:
    positions, velocities, orientations, tumbles, seeds and backscatter bit
    for bit, except lanes 2 and 3 of the rain drops' backscatter, where the
    oracle (and the backend) form cos^2 of the elevation as |xy|^2 / |xyz|^2
    instead of cos(atan2(z, |xy|))^2: within 4e-7 relative;
  * scat_sig_aux, make_pulse_pass_1 and the three pass-2 kernels in every
    launch plan RS_make_pulse_params makes (pulse, sig and aux bit for bit);
  * pop;
  * rs.c's recorded sessions run again with the device executing rs.cl: the
    recorded state (made with the oracle's kernels) bit for bit but for the
    rain backscatter and the signals formed from it, the pulses within 1e-6
    of their largest gate.

The GPU tests hold the backend to the oracle bit for bit, so these pin the
backend's state to the reference's kernel source.  They need the reference
tree (the build reads rs.cl where it lies) and are skipped without it.
"""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refbind
from simradar_gb300 import synth

pytestmark = pytest.mark.skipif(not refbind.available(), reason="the reference tree is not present")

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("pos", "vel", "ori", "tum", "rnd", "rcs")
RAIN_RCS_REL = 4e-7


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def rscl():
    return refbind.rscl()


def push_to_edges(S, n_rain=64, n_deb=16):
    """Scatterers just inside the box moving out: the next step respawns them."""
    ox, oy, oz, sx, sy, sz = S.box
    pos, vel = S.state["pos"], S.state["vel"]
    pos[:n_rain, 0] = np.float32(ox) + np.float32(1e-3)
    vel[:n_rain, 0] = -5.0
    pos[n_rain:2 * n_rain, 2] = np.float32(oz + sz) - np.float32(1e-3)
    vel[n_rain:2 * n_rain, 2] = 5.0
    if len(S.counts) > 1:
        d0 = S.counts[0]
        pos[d0:d0 + n_deb, 1] = np.float32(oy) + np.float32(1e-3)
        vel[d0:d0 + n_deb, 1] = -5.0


def concept_desc(S, k, concept):
    sd = synth.pulse_sim_desc(S, k)
    sd[5] = np.frombuffer(np.uint32(concept).tobytes(), np.float32)[0]
    return sd


def assert_advance_equal(a, b, n_rain, what):
    for f in FIELDS:
        if f == "rcs":
            continue
        d = (bits(a.s[f]) != bits(b.s[f])).any(axis=1)
        assert not d.any(), "%s: %s differs at %d entries (first %d)" % (what, f, d.sum(), np.argmax(d))
    ra, rb = a.s["rcs"], b.s["rcs"]
    assert np.array_equal(bits(ra[n_rain:]), bits(rb[n_rain:])), what + ": debris backscatter"
    assert np.array_equal(bits(ra[:n_rain, :2]), bits(rb[:n_rain, :2])), what + ": rain backscatter lanes 0-1"
    x, y = ra[:n_rain, 2:].astype(np.float64), rb[:n_rain, 2:].astype(np.float64)
    rel = np.abs(x - y) / np.maximum(np.abs(x), 1e-38)
    assert rel.max() <= RAIN_RCS_REL, "%s: rain backscatter lanes 2-3 %.3g" % (what, rel.max())


@pytest.mark.parametrize("concept", [synth.CONCEPT_DBU, 0, synth.CONCEPT_BOUNDED, synth.CONCEPT_FIXED_POS,
                                     synth.CONCEPT_DRAGGED | synth.CONCEPT_CROSS_POL,
                                     synth.CONCEPT_DBU | synth.CONCEPT_VERTICAL])
def test_advance_kernels_match_rs_cl(rscl, concept):
    """el_atts (D, with and without B), bg_atts, fp_atts (F) and db_atts for
    three debris types (with cross-pol), five steps with respawns."""
    S = synth.make_scene(num_rain=20000, debris=[(synth.OBJ_LEAF, 512), (synth.OBJ_WOODBOARD_2X4, 512),
                                                  (synth.OBJ_BRICK, 512)], les_count=1, concept=concept)
    push_to_edges(S)
    a, b = O.OracleState(S.state), O.OracleState(S.state)
    for k in range(5):
        sd = concept_desc(S, k, concept)
        O.advance_time(a, S, S.counts, S.les[0], sd)
        O.advance_time(b, S, S.counts, S.les[0], sd, L=rscl)
        assert_advance_equal(a, b, S.counts[0], "concept %d step %d" % (concept, k))
    if not concept & synth.CONCEPT_FIXED_POS:
        respawned = (bits(a.s["rnd"]) != bits(S.state["rnd"])).any(axis=1)
        assert respawned[:S.counts[0]].sum() >= 64 and respawned[S.counts[0]:].sum() >= 16


def test_uniform_les_grid_matches_rs_cl(rscl):
    """wind_table_index's uniform branch (rs.cl:152-173: fma(pos, scale,
    origin)) with the LES volume spread over the scan box, el_atts and
    db_atts."""
    S = synth.make_scene(num_rain=8000, debris=[(synth.OBJ_LEAF, 300), (synth.OBJ_BRICK, 300)], les_count=1)
    push_to_edges(S)
    ox, oy, oz, sx, sy, sz = S.box
    n = (S.les_cfg.nx, S.les_cfg.ny, S.les_cfg.nz)
    desc = np.zeros(16, np.float32)   # spacing code 0 (uniform) in lane 7
    for ax, (o, size) in enumerate(((ox, sx), (oy, sy), (oz, sz))):
        desc[ax] = np.float32(n[ax] / size)
        desc[4 + ax] = np.float32(-o * n[ax] / size)
    desc[3] = S.les_desc[3]
    S.les_desc = desc
    a, b = O.OracleState(S.state), O.OracleState(S.state)
    for k in range(4):
        sd = concept_desc(S, k, synth.CONCEPT_DBU)
        O.advance_time(a, S, S.counts, S.les[0], sd)
        O.advance_time(b, S, S.counts, S.les[0], sd, L=rscl)
        assert_advance_equal(a, b, S.counts[0], "uniform LES step %d" % k)
    assert not np.array_equal(bits(a.s["vel"]), bits(S.state["vel"]))


@pytest.mark.parametrize("mode", [0.0, 1.0, 2.0])
def test_debris_flux_field_matches_rs_cl(rscl, mode):
    """db_atts's respawn from the debris flux field (rs.cl:795-835): plain,
    stretched-grid (mode 1) and domain-scaled (mode 2) placement."""
    concept = synth.CONCEPT_DBU | synth.CONCEPT_DFF
    S = synth.make_scene(num_rain=2000, debris=[(synth.OBJ_LEAF, 400), (synth.OBJ_BRICK, 400)], les_count=1,
                         concept=concept, seed=41)
    push_to_edges(S, n_rain=100, n_deb=200)
    S.dff = np.linspace(0.0, 8.999, 2048).astype(np.float32)   # 3 x 3 cells
    S.dff_desc = np.zeros(16, np.float32)
    S.dff_desc[0] = S.dff_desc[1] = np.float32(1.0 / 3.0)
    S.dff_desc[4] = S.dff_desc[5] = 1.02
    S.dff_desc[8] = S.dff_desc[9] = 2.0
    S.dff_desc[13] = 3.0
    S.dff_desc[14] = mode
    S.dff_desc[15] = 2047.0
    a, b = O.OracleState(S.state), O.OracleState(S.state)
    for k in range(3):
        sd = concept_desc(S, k, concept)
        O.advance_time(a, S, S.counts, S.les[0], sd)
        O.advance_time(b, S, S.counts, S.les[0], sd, L=rscl)
        assert_advance_equal(a, b, S.counts[0], "DFF mode %g step %d" % (mode, k))
    deb = slice(S.counts[0], S.num_scats)
    assert (bits(a.s["rnd"][deb]) != bits(S.state["rnd"][deb])).any(axis=1).sum() >= 100


def test_debris_rcs_matches_rs_cl(rscl):
    """db_rcs (rs.cl:909-919), cross-pol on."""
    concept = synth.CONCEPT_DBU | synth.CONCEPT_CROSS_POL
    S = synth.make_scene(num_rain=256, debris=[(synth.OBJ_LEAF, 700), (synth.OBJ_BRICK, 300)], les_count=1,
                         concept=concept)
    a, b = O.OracleState(S.state), O.OracleState(S.state)
    sd = concept_desc(S, 3, concept)
    O.db_rcs(a, S, S.counts, sd)
    O.db_rcs(b, S, S.counts, sd, L=rscl)
    assert np.array_equal(bits(a.s["rcs"]), bits(b.s["rcs"]))
    assert not np.array_equal(bits(a.s["rcs"]), bits(S.state["rcs"]))


@pytest.mark.parametrize("n, maxg, swap", [(20000, 1024, 1), (20000, 256, 0), (20000, 256, 1), (128, 1024, 1),
                                           (4096, 1024, 0), (62, 1024, 1), (131072, 1024, 1), (3000, 1024, 1)])
def test_pulse_kernels_match_rs_cl(rscl, n, maxg, swap):
    """scat_sig_aux, make_pulse_pass_1 and pass 2 under the plan
    RS_make_pulse_params makes for n scatterers and a work-group limit of
    maxg (every pass-2 method, rs.c's kernel-name swap on and off, and the
    31-wide work group of n = 62 whose tree reads past its gate column)."""
    S = synth.make_scene(num_rain=n, les_count=1)
    a, b = O.OracleState(S.state), O.OracleState(S.state)
    for k in (3, 7):
        sd = synth.pulse_sim_desc(S, k)
        pa = O.make_pulse(a, S, sd, max_work_group_size=maxg, name_swap=swap)
        pb = O.make_pulse(b, S, sd, max_work_group_size=maxg, name_swap=swap, L=rscl)
        assert np.array_equal(bits(pa), bits(pb)), "pulse %d" % k
        assert np.array_equal(bits(a.s["sig"]), bits(b.s["sig"]))
        assert np.array_equal(bits(a.s["aux"]), bits(b.s["aux"]))
        assert np.abs(pa).max() > 0


def test_pop_matches_rs_cl(rscl):
    """pop (rs.cl:1444-1453)."""
    n = 100000
    sd = np.zeros(16, np.float32)
    sd[0:3] = synth.beam_unit(3.0, 10.0)
    outs = []
    for L in (O.lib(), rscl):
        rcs, aux, pos = (np.zeros((n, 4), np.float32) for _ in range(3))
        L.or_pop(O.fp(rcs), O.fp(aux), O.fp(pos), O.fp(sd), n)
        outs.append((rcs, aux, pos))
    for x, y in zip(*outs):
        assert np.array_equal(bits(x), bits(y))


@pytest.fixture(scope="module")
def tables_home(tmp_path_factory):
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_ref_session import write_tables
    home = str(tmp_path_factory.mktemp("rscl_home"))
    write_tables(home)
    return home


@pytest.mark.parametrize("name", ["ref_session_dbu", "ref_session_bg", "ref_session_dff", "ref_session_vpr"])
def test_rs_c_session_with_rs_cl_kernels(tables_home, tmp_path, name):
    """rs.c's recorded session run again with the device executing the
    reference's rs.cl: the same event list, the same final positions,
    velocities, orientations, tumbles, aux and seeds bit for bit; the rain
    backscatter (and the signals and pulses formed from it) within the
    bound of its cos^2 formula."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_ref_session import SESSIONS as ARGS
    with np.load(os.path.join(HERE, "golden", name + ".npz")) as z:
        R = {k: z[k] for k in z.files}
    N = refbind.run_session(str(tmp_path / "s.bin"), tables_home, kernels="rscl", **ARGS[name])
    assert int(N["failed"]) == 0
    near = {"pulse_raw", "pulse_merged", "pulse_abs", "pulse_direct", "final_rcs_every8", "final_sig_every8",
            "final_hash"}
    for k, v in N.items():
        if k not in near:
            assert np.array_equal(np.asarray(v), R[k]), k
    fields = ["pos", "vel", "ori", "tum", "aux", "rcs", "sig", "rnd"]
    for i, f in enumerate(fields):
        if f not in ("rcs", "sig"):
            assert int(N["final_hash"][i]) == int(R["final_hash"][i]), f
    for f in ("rcs", "sig"):
        x = R["final_%s_every8" % f].astype(np.float64)
        y = N["final_%s_every8" % f].astype(np.float64)
        assert np.all(np.abs(x - y) <= 4e-7 * np.abs(x)), f
    for k in ("pulse_raw", "pulse_merged"):
        x, y = R[k].astype(np.float64), N[k].astype(np.float64)
        scale = np.abs(x).reshape(x.shape[0], -1).max(axis=1)
        err = np.abs(x - y).reshape(x.shape[0], -1).max(axis=1)
        assert np.all(err <= 1e-6 * scale), "%s: %.3g" % (k, (err / scale).max())
