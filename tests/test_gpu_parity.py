"""GPU parity: the sm_103a backend (through its C ABI) against the CPU oracle.

State evolution (positions, velocities, orientations, tumbles, RCS, respawn
seeds) must be bit-exact.  Pulses are sums over scatterers and gates of a
bit-identical signal times a bit-identical gate weight, taken in a different
order (and with the product fused into the running sum where the kernel
holds two scatterers per lane), so they agree within the FP32 summation
bound stated in PULSE_TOL below.
"""
import numpy as np
import pytest

from simradar_gb300 import synth

pytestmark = pytest.mark.gpu

# |gpu - oracle| <= PULSE_TOL * sum_i |w_i sig_i| per gate and lane.  Both are
# FP32 sums of the same contributions; the classical bound for reordering n
# terms is (n - 1) eps sum|x|, and with n ~ 1e4-1e5 per gate the observed
# differences sit near sqrt(n) eps, so 2e-5 (about 170 eps) is the bound
# checked here.
PULSE_TOL = 2.0e-5

STATE_FIELDS = ("pos", "vel", "ori", "tum", "rcs", "rnd")


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def assert_state_equal(gpu, ref, fields=STATE_FIELDS, where=""):
    for f in fields:
        g, r = bits(gpu[f]), bits(ref[f])
        bad = np.nonzero((g != r).any(axis=1))[0]
        assert bad.size == 0, "%s%s: %d scatterers differ, first %s: gpu %s oracle %s" % (
            where, f, bad.size, bad[:5], gpu[f][bad[0]], ref[f][bad[0]])


def push_to_edges(S, n_rain=64, n_deb=16):
    """Put some scatterers just inside the box moving out, so the next step
    respawns them (exercises the RNG path)."""
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


@pytest.fixture(scope="module")
def scene_db():
    S = synth.make_scene(num_rain=20000, debris=[(synth.OBJ_LEAF, 512), (synth.OBJ_WOODBOARD_2X4, 512),
                                                  (synth.OBJ_BRICK, 512)], les_count=2)
    push_to_edges(S)
    return S


def run_pair(backend, oracle_lib, S, steps, concept=None, precision=0, check_each=True):
    O = oracle_lib
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    W.set_precision(precision)
    st = O.OracleState(S.state)
    pulses = []
    for k in range(steps):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        if concept is not None:
            sd[5] = synth.fbits(concept)
        if k == 0:
            sd[11] = 0.0   # the warm pass of RS_populate runs with PRT = 0 (rs.c:4940-4946)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        r = O.make_pulse(st, S, sd)
        r64, ab = O.make_pulse_f64(st, S, sd, return_abs=True)
        pulses.append((g, r, r64, ab))
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
        if check_each:
            assert_state_equal(W.download(STATE_FIELDS), st.s, where="step %d " % k)
    return W, st, pulses


def test_math_bitexact(backend, oracle_lib):
    rng = np.random.default_rng(7)
    cases = [
        (0, rng.uniform(-20, 20, 100000), None), (1, rng.uniform(-20, 20, 100000), None),
        (0, rng.uniform(1e5, 4e6, 100000), None), (1, rng.uniform(1e5, 4e6, 100000), None),
        (2, np.exp(rng.uniform(-20, 20, 100000)), None), (3, rng.uniform(-0.9, 50, 100000), None),
        (4, rng.uniform(-1, 1, 100000), None), (5, rng.uniform(-5, 5, 100000), rng.uniform(-5, 5, 100000)),
        (6, rng.uniform(-90, 90, 100000), None), (7, rng.uniform(0.5, 20, 100000), rng.uniform(-20, 5, 100000)),
    ]
    for fn, a, b in cases:
        a = a.astype(np.float32)
        b = b.astype(np.float32) if b is not None else None
        g = backend.eval_math(fn, a, b)
        c = oracle_lib.eval_math(fn, a, b)
        assert np.array_equal(bits(g), bits(c)), "math fn %d differs on %d inputs" % (fn, int((bits(g) != bits(c)).sum()))


def _ulp_walk(x, k):
    """x moved k representable floats (k < 0: down)."""
    x = np.float32(x)
    for _ in range(abs(int(k))):
        x = np.nextafter(x, np.float32(-np.inf if k < 0 else np.inf), dtype=np.float32)
    return x


def test_triangle_weight_matches_table_lerp(backend, oracle_lib):
    """The pulse kernel's closed-form weight on the reference's triangle
    table against the table lerp of make_pulse_pass_1 (rs.cl:1196-1209):
    bit-identical on random distances and on every float within 40 ulps of
    the breakpoints -dr, 0 and +dr (the corners of its two index
    computations), for several gate widths."""
    rng = np.random.default_rng(11)
    d_all, s_all = [], []
    for dr in (30.0, 25.0, 15.0, 7.5, 1.0, 0.3, 150.0, 3.0e-3):
        s = np.float32(np.float32(1.0) / np.float32(dr))
        d = list(rng.uniform(-2.5 * dr, 2.5 * dr, 200000).astype(np.float32))
        for c in (-dr, dr):
            d += [_ulp_walk(c, k) for k in range(-40, 41)]
        d += list((np.float32(dr) * np.float32(2.0) ** -np.arange(1, 60, dtype=np.float32)).astype(np.float32))
        d += list(-(np.float32(dr) * np.float32(2.0) ** -np.arange(1, 60, dtype=np.float32)).astype(np.float32))
        d += [np.float32(0.0), np.float32(-0.0), np.float32(np.nan), np.float32(np.inf), np.float32(-np.inf)]
        d_all += d
        s_all += [s] * len(d)
    a = np.array(d_all, np.float32)
    b = np.array(s_all, np.float32)
    g = backend.eval_math(8, a, b)
    c = oracle_lib.eval_math(8, a, b)
    assert np.array_equal(bits(g), bits(c)), "triangle weight differs on %d of %d inputs" % (
        int((bits(g) != bits(c)).sum()), a.size)


def test_compensated_phase_sine_cosine(backend):
    """The compensated pulse's sine and cosine of the two-way phase k r
    (reduce_pio2_df + sincos_df, as double-floats) against double, for
    ranges near the radar and 30 km out (phases to 4.2e6 rad), and for
    ranges placed on multiples of pi/2 / k and of 1/128 rad past them (the
    reduction's and the table's nodes and midpoints): within 1e-13.  The
    plain FP32 form, for scale, is off by up to a quarter at 30 km."""
    rng = np.random.default_rng(17)
    k = np.float32(4.0 * np.pi / 0.1)
    r = [rng.uniform(1.0, 50.0, 50000), rng.uniform(1800.0, 2500.0, 100000),
         rng.uniform(31000.0, 33000.0, 100000)]
    n = np.arange(1, 2600000, 997, dtype=np.float64)
    r.append(n * (np.pi / 2) / float(k))
    r.append((n * (np.pi / 2) + (np.arange(n.size) % 205 - 102) / 128.0) / float(k))
    a = np.concatenate(r).astype(np.float32)
    b = np.full_like(a, k)
    for fn in (9, 10):
        e = np.abs(backend.eval_math(fn, a, b).astype(np.float64))
        assert e.max() <= 1.0e-13, "fn %d: %.3g at r = %r" % (fn, e.max(), a[np.argmax(e)])
    far = a > 30000.0
    assert np.abs(backend.eval_math(11, a[far], b[far])).max() > 0.05


def test_advance_dbu_bitexact(backend, oracle_lib, scene_db):
    """Concept DBU (el_atts, bounded) rain + three debris types, 6 steps."""
    W, st, _ = run_pair(backend, oracle_lib, scene_db, 6)
    # respawns happened and were reproduced
    assert (bits(st.s["rnd"]) != bits(scene_db.state["rnd"])).any(axis=1).sum() >= 64
    W.close()


@pytest.mark.parametrize("concept", [0, synth.CONCEPT_BOUNDED, synth.CONCEPT_FIXED_POS,
                                     synth.CONCEPT_DRAGGED | synth.CONCEPT_CROSS_POL])
def test_advance_concepts_bitexact(backend, oracle_lib, scene_db, concept):
    """bg_atts (no D), fp_atts (F), el_atts without bounding, cross-pol debris."""
    W, st, _ = run_pair(backend, oracle_lib, scene_db, 3, concept=concept)
    W.close()


def test_pulse_plain_matches_oracle(backend, oracle_lib, scene_db):
    """Against the reference's own summation order (pass 1 + pass 2) and
    against the exact sum of the same FP32 contributions."""
    S = scene_db
    O = oracle_lib
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    st = O.OracleState(S.state)
    for k in range(4):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        assert np.isfinite(g).all()
        direct, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
        assert_pulse_close(g, O.make_pulse(st, S, sd), ab, "pulse %d vs reference order" % k)
        assert_pulse_close(g, direct, ab, "pulse %d vs exact sum" % k)
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
    W.close()


def test_pulse_f64_matches_cpu_f64(backend, oracle_lib, scene_db):
    W, st, pulses = run_pair(backend, oracle_lib, scene_db, 2, precision=2, check_each=False)
    for g, r, r64, ab in pulses:
        assert np.all(np.abs(g - r64) <= 1e-6 * ab + 1e-30)
    W.close()


# Compensated form against FP64: every factor of every term is a
# double-float and the sums are error-free, so the pulse reaches the FP64
# pulse of the same state to the FP32 rounding of its output (6e-8 of a
# component) plus the double-float's own precision (the range to 2^-48, a
# phase error of ~1e-8 rad at 30 km, which shows only where a gate's terms
# cancel by 1e4 or more).  Asserted per gate and lane, raw (every gate with
# a non-zero FP64 value, whatever its terms do): |gpu - fp64| <= COMP_REL
# |gate| (the gate's complex magnitude per polarization), and <= COMP_TIGHT
# |gate| on gates whose terms cancel by less than 100x.
COMP_REL = 1.0e-5
COMP_TIGHT = 2.0e-7


def assert_comp_close(g, r64, ab, what=""):
    mag = np.hypot(r64[:, 0::2], r64[:, 1::2]).repeat(2, axis=1)
    err = np.abs(g.astype(np.float64) - r64)
    zero = mag == 0
    assert np.all(err[zero] == 0.0), "%s: non-zero output on a gate with no contribution" % what
    nz = ~zero
    rel = err[nz] / mag[nz]
    if rel.size:
        k = np.argmax(rel)
        where = tuple(np.argwhere(nz)[k])
        assert rel[k] <= COMP_REL, "%s: relative error %.3g at (gate, lane) %s, |gate| %r sum|x| %r" % (
            what, rel[k], where, mag[where], ab[where])
    well = nz & (ab <= 100.0 * mag)
    if well.any():
        assert (err[well] / mag[well]).max() <= COMP_TIGHT, "%s: %.3g on a well-conditioned gate" % (
            what, (err[well] / mag[well]).max())


def test_pulse_compensated_error(backend, oracle_lib, scene_db):
    """Compensated form: per-gate relative I/Q error <= 1e-5 against FP64 on
    every gate, <= 2e-7 where the terms cancel by less than 100x."""
    W, st, pulses = run_pair(backend, oracle_lib, scene_db, 3, precision=1, check_each=False)
    for k, (g, r, r64, ab) in enumerate(pulses):
        assert_comp_close(g, r64, ab, "pulse %d" % k)
    W.close()


def test_compensated_moments_and_per_gate(backend, oracle_lib, scene_db):
    """The compensated form's two ways of summing on the triangle -- each
    term into its range interval as two moments, or weighed into every gate
    it reaches -- both within the bound against FP64, and the same pulse
    within one FP32 rounding of its components, in the caller's order (the
    first pulse) and in spatial order."""
    O = oracle_lib
    S = scene_db
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    W.set_precision(1)
    st = O.OracleState(S.state)
    for k in range(3):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        r64, ab = O.make_pulse_f64(st, S, sd, return_abs=True)
        got = {}
        for mom in (1, 0):
            W.set_moments(mom)
            W.make_pulse(sd)
            got[mom] = W.download_pulse(1.0)
            assert_comp_close(got[mom], r64, ab, "pulse %d moments %d" % (k, mom))
        a, b = got[1].astype(np.float64), got[0].astype(np.float64)
        assert np.all(np.abs(a - b) <= 1.2e-7 * np.maximum(np.abs(a), np.abs(b))), "pulse %d" % k
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
    W.close()


@pytest.mark.parametrize("concept", [synth.CONCEPT_DBU, 0])
def test_advance_two_per_thread(backend, oracle_lib, scene_db, concept):
    """Two background scatterers per advance thread (rsc_set_advance_shape)
    advance the state bit for bit as the oracle does, el_atts and bg_atts,
    respawns included."""
    O = oracle_lib
    S = scene_db
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    W.set_advance_shape(2)
    st = O.OracleState(S.state)
    for k in range(4):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        sd[5] = synth.fbits(concept)
        W.make_pulse(sd)
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
        assert_state_equal(W.download(STATE_FIELDS), st.s, where="step %d " % k)
    assert (bits(st.s["rnd"]) != bits(S.state["rnd"])).any(axis=1).sum() >= 64
    W.close()


def test_dense_gate_path(backend, oracle_lib):
    """A range weight with non-zero edges reaches every gate (dense path)."""
    S = synth.make_scene(num_rain=5000, les_count=1)
    S.range_w = np.array([0.25, 1.0, 0.5], dtype=np.float32)
    W, st, pulses = run_pair(backend, oracle_lib, S, 2, check_each=True)
    for g, r, r64, ab in pulses:
        assert np.all(np.abs(g - r) <= PULSE_TOL * ab + 1e-30)
    W.close()


def assert_pulse_close(g, r, ab, what=""):
    lim = PULSE_TOL * ab + 1e-30
    d = np.abs(g.astype(np.float64) - r.astype(np.float64))
    bad = np.argwhere(d > lim)
    assert bad.size == 0, "%s: %d values beyond tolerance; first (gate, lane) %s gpu %r oracle %r abs-sum %r" % (
        what, len(bad), tuple(bad[0]), g[tuple(bad[0])], r[tuple(bad[0])], ab[tuple(bad[0])])


@pytest.mark.parametrize("n", [1, 31, 33, 64, 65, 1025])
def test_small_and_ragged_sizes(backend, oracle_lib, n):
    """Below 128 scatterers the reference's pass-1 work group is count / 2
    wide; its tree reduction is only right for powers of two (31, 65: it adds
    the next gate's entries) and count 1 divides by zero in
    RS_make_pulse_params.  The GPU is compared with the exact sum of the
    reference's FP32 contributions for every size, and with the reference's
    own summation where that plan is valid."""
    O = oracle_lib
    S = synth.make_scene(num_rain=n, les_count=1)
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    st = O.OracleState(S.state)
    for k in range(3):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        direct, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
        assert_pulse_close(g, direct, ab, "n=%d pulse %d vs exact sum" % (n, k))
        if O.reference_plan_valid(n):
            assert_pulse_close(g, O.make_pulse(st, S, sd), ab, "n=%d pulse %d vs reference order" % (n, k))
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
        assert_state_equal(W.download(STATE_FIELDS), st.s, where="n=%d step %d " % (n, k))
    W.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_non_finite_scatterers(backend, oracle_lib, precision):
    """A scatterer with a non-finite backscatter reaches every gate, as in
    make_pulse_pass_1 (0 x NaN is NaN): the values the oracle's exact sum
    makes non-finite are non-finite on the GPU, in the caller's order and in
    spatial order (the grouped kernel hands such warps to the one-scatterer
    path), and every other value stays within the summation bound."""
    O = oracle_lib
    S = synth.make_scene(num_rain=20000, les_count=1, seed=77)
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    W.set_precision(precision)
    st = O.OracleState(S.state)
    sd0 = synth.pulse_sim_desc(S, 0)
    for sorted_state in (False, True):
        if sorted_state:
            W.advance_time(pop, 0, sd0)   # the first advance puts the state in spatial order
            O.advance_time(st, S, S.counts, S.les[0], sd0)
            assert W.sort_count >= 1
        cur = W.download(("pos", "rcs"))
        rcs, pos = cur["rcs"].copy(), cur["pos"].copy()
        rcs[123, 0] = np.float32(np.nan)          # the H lanes of every gate
        W.upload(0, rcs=rcs, pos=pos)
        st.s["rcs"][:] = rcs
        sd = synth.pulse_sim_desc(S, 3)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        direct, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
        where = "sorted" if sorted_state else "caller order"
        assert np.array_equal(np.isfinite(g), np.isfinite(direct)), where
        assert np.isnan(direct[:, :2]).all() and np.isfinite(direct[:, 2:]).all(), where
        ok = np.isfinite(direct)
        if precision == 0:
            assert_pulse_close(np.where(ok, g, 0.0), np.where(ok, direct, 0.0), np.where(ok, ab, 0.0), where)
        else:
            r64, ab64 = O.make_pulse_f64(st, S, sd, return_abs=True)
            assert_comp_close(np.where(ok, g, 0.0), np.where(ok, r64, 0.0), np.where(ok, ab64, 0.0), where)
        rcs[123, 0] = np.float32(1.0)
        W.upload(0, rcs=rcs)
        st.s["rcs"][:] = rcs
    W.close()


def test_download_forms_sig_aux(backend, oracle_lib, scene_db):
    """RS_download returns aux / sig as scat_sig_aux wrote them (bit-exact),
    whether the pulse kernel wrote them or they are formed on download."""
    for materialize in (False, True):
        S = scene_db
        W = backend.Worker(0)
        synth.load_worker(W, S)
        W.set_materialize(materialize)
        st = oracle_lib.OracleState(S.state)
        sd = synth.pulse_sim_desc(S, 3)
        W.make_pulse(sd)
        oracle_lib.make_pulse(st, S, sd)
        out = W.download(("aux", "sig"))
        assert_state_equal(out, st.s, fields=("aux", "sig"))
        W.close()


def test_les_slot_swap(backend, oracle_lib):
    """Advance on LES slot 1 (a different volume) after an asynchronous upload."""
    S = synth.make_scene(num_rain=8000, les_count=2)
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S, les_slot_volumes=(0,))
    W.set_les(1, S.les[1].uvwt, S.les[1].cpxx, S.les_desc, asynchronous=True)
    st = oracle_lib.OracleState(S.state)
    sd = synth.pulse_sim_desc(S, 0)
    for slot in (1, 0, 1):
        W.advance_time(pop, slot, sd)
        oracle_lib.advance_time(st, S, S.counts, S.les[slot], sd)
    assert_state_equal(W.download(STATE_FIELDS), st.s)
    W.close()


def test_debris_rcs_refresh(backend, oracle_lib, scene_db):
    S = scene_db
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    st = oracle_lib.OracleState(S.state)
    sd = synth.pulse_sim_desc(S, 5)
    W.update_debris_rcs(pop, sd)
    oracle_lib.db_rcs(st, S, S.counts, sd)
    assert_state_equal(W.download(("rcs",)), st.s, fields=("rcs",))
    W.close()


def test_errors_are_status_codes(backend):
    W = backend.Worker(0)
    with pytest.raises(backend.BackendError):
        W.make_pulse(np.zeros(16, np.float32))        # before malloc
    with pytest.raises(backend.BackendError):
        W.malloc(10, 0.0, 1.0, 100000)                 # too many gates
    W.malloc(100, 1000.0, 15.0, 8)
    with pytest.raises(backend.BackendError):
        W.set_les(2, np.zeros((2, 2, 2, 4), np.float32), None, np.zeros(16, np.float32))
    with pytest.raises(backend.BackendError):
        W.upload(99, pos=np.zeros((5, 4), np.float32))  # beyond the arrays
    W.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_fused_step_matches_separate(backend, oracle_lib, scene_db, precision):
    """advance_time followed by make_pulse in one kernel (set_fused_step) gives
    the state of the separate kernels bit for bit and the same pulses within
    the summation bound; the oracle agrees."""
    O = oracle_lib
    S = scene_db
    pop = synth.population(S)
    Wf, Ws = backend.Worker(0), backend.Worker(0)
    for W in (Wf, Ws):
        synth.load_worker(W, S)
        W.set_precision(precision)
    Wf.set_fused_step(True)
    Ws.set_fused_step(False)
    st = O.OracleState(S.state)
    for k in range(5):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        Wf.make_pulse(sd)
        Ws.make_pulse(sd)
        gf, gs = Wf.download_pulse(1.0), Ws.download_pulse(1.0)
        direct, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
        if precision == 0:
            assert_pulse_close(gf, direct, ab, "fused pulse %d" % k)
            assert_pulse_close(gs, direct, ab, "separate pulse %d" % k)
        else:
            r64, ab64 = O.make_pulse_f64(st, S, sd, return_abs=True)
            assert_comp_close(gf, r64, ab64, "fused compensated pulse %d" % k)
        Wf.advance_time(pop, 0, sd)
        Ws.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
    a, b = Wf.download(STATE_FIELDS), Ws.download(STATE_FIELDS)
    for f in STATE_FIELDS:
        assert np.array_equal(bits(a[f]), bits(b[f])), f
    assert_state_equal(a, st.s, where="fused ")
    Wf.close()
    Ws.close()


def test_download_pulse_async(backend, scene_db):
    """The queued copy holds the same pulse as the blocking read (which
    applies the gain), for pulses queued back to back between advances."""
    S = scene_db
    W = backend.Worker(0)
    synth.load_worker(W, S)
    pop = synth.population(S)
    outs = np.zeros((3, S.range_count, 4), np.float32)
    refs = []
    for k in range(3):
        sd = synth.pulse_sim_desc(S, k)
        W.make_pulse(sd)
        W.download_pulse_async(outs[k])
        W.synchronize()
        refs.append(W.download_pulse(2.0))
        W.advance_time(pop, 0, sd)
    for k in range(3):
        assert np.any(outs[k] != 0.0)
        assert np.array_equal(outs[k] * np.float32(2.0), refs[k]), k
    W.close()


def test_download_pulse_async_queued(backend, scene_db):
    """Pulses copied asynchronously into page-locked buffers while the host
    queues the following steps: each buffer holds its own step's pulse (the
    next pulse kernel waits for the copy) and the state ends bit-identical,
    compared with a second worker that reads every pulse with a blocking
    download (no overlap between its steps)."""
    torch = pytest.importorskip("torch")
    S = scene_db
    pop = synth.population(S)
    A, B = backend.Worker(0), backend.Worker(0)
    for W in (A, B):
        synth.load_worker(W, S)
    K = 8
    ring = torch.empty((K, S.range_count, 4), dtype=torch.float32).pin_memory().numpy()
    refs = []
    for k in range(K):
        sd = synth.pulse_sim_desc(S, 5 * k)
        A.make_pulse(sd)
        A.download_pulse_async(ring[k])
        A.advance_time(pop, 0, sd)
        B.make_pulse(sd)
        refs.append(B.download_pulse(1.0))
        B.advance_time(pop, 0, sd)
    A.synchronize()
    for k in range(K):
        scale = float(np.abs(refs[k]).max())
        assert scale > 0.0
        np.testing.assert_allclose(ring[k], refs[k], rtol=1e-4, atol=1e-5 * scale, err_msg=str(k))
    # the queued steps (pulses and advances overlapping on their two
    # streams) leave the same state as the stepped ones
    assert_state_equal(A.download(STATE_FIELDS), B.download(STATE_FIELDS), where="queued vs stepped ")
    A.close()
    B.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_max_gates(backend, oracle_lib, precision):
    """RSC_MAX_GATES (512) gates: the largest shared-memory bins of every
    precision mode; the gates beyond the box stay exactly zero."""
    O = oracle_lib
    S = synth.make_scene(num_rain=30000, gates=512, les_count=1, seed=21)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    W.set_precision(precision)
    st = O.OracleState(S.state)
    pop = synth.population(S)
    for k in range(2):
        sd = synth.pulse_sim_desc(S, k)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        assert g.shape == (512, 4) and np.isfinite(g).all()
        if precision == 0:
            d, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
            assert_pulse_close(g, d, ab, "512 gates pulse %d" % k)
        else:
            r64, ab = O.make_pulse_f64(st, S, sd, return_abs=True)
            if precision == 1:
                assert_comp_close(g, r64, ab, "512 gates compensated pulse %d" % k)
            else:
                assert np.all(np.abs(g - r64) <= 1e-6 * ab + 1e-30)
        assert np.all(g[60:] == 0.0)
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
    assert_state_equal(W.download(STATE_FIELDS), st.s, where="512 gates ")
    W.close()


def test_debris_only(backend, oracle_lib):
    """No background scatterers at all: two debris types only."""
    O = oracle_lib
    S = synth.make_scene(num_rain=0, debris=[(synth.OBJ_LEAF, 700), (synth.OBJ_BRICK, 300)], les_count=1, seed=31)
    push_to_edges(S, n_rain=0, n_deb=40)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    st = O.OracleState(S.state)
    pop = synth.population(S)
    for k in range(3):
        sd = synth.pulse_sim_desc(S, k)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        d, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
        assert_pulse_close(g, d, ab, "debris-only pulse %d" % k)
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
        assert_state_equal(W.download(STATE_FIELDS), st.s, where="debris-only step %d " % k)
    W.close()


@pytest.mark.parametrize("mode", [0.0, 1.0, 2.0])
def test_debris_flux_field_respawn(backend, oracle_lib, mode):
    """Concept C (debris flux from velocity, rs.cl:795-835): respawned debris
    take their cell from the inverse-CDF table, placed plainly, on the
    stretched grid (mode 1) or scaled to the domain (mode 2)."""
    O = oracle_lib
    S = synth.make_scene(num_rain=2000, debris=[(synth.OBJ_LEAF, 400), (synth.OBJ_BRICK, 400)], les_count=1,
                         concept=synth.CONCEPT_DBU | synth.CONCEPT_DFF, seed=41)
    push_to_edges(S, n_rain=100, n_deb=200)
    icdf = np.linspace(0.0, 8.999, 2048).astype(np.float32)   # 3 x 3 cells
    desc = np.zeros(16, np.float32)
    desc[0] = desc[1] = np.float32(1.0 / 3.0)
    desc[4] = desc[5] = 1.02
    desc[8] = desc[9] = 2.0
    desc[13] = 3.0
    desc[14] = mode
    desc[15] = 2047.0
    S.dff, S.dff_desc = icdf, desc
    W = backend.Worker(0)
    synth.load_worker(W, S)
    for slot in (0, 1):
        W.set_dff(slot, icdf, desc)
    st = O.OracleState(S.state)
    pop = synth.population(S)
    for k in range(3):
        sd = synth.pulse_sim_desc(S, k)
        W.make_pulse(sd)
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
        assert_state_equal(W.download(STATE_FIELDS), st.s, where="DFF mode %g step %d " % (mode, k))
    # debris respawned from the table sit at the minimum height
    deb = slice(S.counts[0], S.num_scats)
    moved = (st.s["rnd"][deb] != S.state["rnd"][deb]).any(axis=1)
    assert moved.sum() >= 100
    W.close()


def test_host_fault_injection(backend, oracle_lib):
    """Failures made on the host, none of them touching a kernel: an
    allocation the device refuses, calls before their tables, a table whose
    descriptor points past its end, a debris type naming a missing table.
    Each returns its status and the worker keeps working afterwards."""
    O = oracle_lib
    W = backend.Worker(0)
    with pytest.raises(backend.BackendError) as e:
        W.malloc(2 ** 42, 1000.0, 15.0, 8)              # 70 TB: cudaMalloc refuses
    assert e.value.status == -3
    S = synth.make_scene(num_rain=5000, debris=[(synth.OBJ_LEAF, 64)], les_count=1, seed=5)
    W.malloc(S.num_scats, S.range_start, S.range_delta, S.range_count)
    W.upload(0, **S.state)
    sd = synth.pulse_sim_desc(S, 0)
    with pytest.raises(backend.BackendError) as e:
        W.make_pulse(sd)                                # no range / angular weights yet
    assert e.value.status == -4
    bad = S.range_desc.copy()
    bad[2] = 5.0                                        # max index past the 3-entry table
    with pytest.raises(backend.BackendError) as e:
        W.set_range_weight(S.range_w, bad)
    assert e.value.status == -1
    W.set_range_weight(S.range_w, S.range_desc)
    W.set_angular_weight(S.ang_w, S.ang_desc)
    W.set_rcs_ellipsoid(S.ell, S.ell_desc)
    pop = synth.population(S)
    with pytest.raises(backend.BackendError) as e:
        W.advance_time(pop, 0, sd)                      # no LES volume yet
    assert e.value.status == -4
    W.set_les(0, S.les[0].uvwt, S.les[0].cpxx, S.les_desc)
    with pytest.raises(backend.BackendError) as e:
        W.advance_time(pop, 0, sd)                      # the leaf's ADM table is missing
    assert e.value.status == -4
    for t, (cd, cm, ad) in enumerate(S.adm):
        W.set_adm(t, cd, cm, ad)
    for t, (re, im, rd) in enumerate(S.rcs_tables):
        W.set_rcs(t, re, im, rd)
    # after all of that, a normal step matches the oracle
    st = O.OracleState(S.state)
    W.make_pulse(sd)
    g = W.download_pulse(1.0)
    d, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
    assert_pulse_close(g, d, ab, "after the failures")
    W.advance_time(pop, 0, sd)
    O.advance_time(st, S, S.counts, S.les[0], sd)
    assert_state_equal(W.download(STATE_FIELDS), st.s, where="after the failures ")
    W.close()
