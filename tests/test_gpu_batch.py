"""GPU parity of the batching form: many instances stepped by three launches
per step (the pulse, the background advance and the debris advance, each for
all of them), with and without a CUDA graph.

Every instance must evolve bit for bit as the oracle does for it alone, and
its pulses must agree with the exact FP32 sum within the same bound as the
one-instance path (PULSE_TOL of test_gpu_parity).
"""
import numpy as np
import pytest

from simradar_gb300 import synth

from test_gpu_parity import (STATE_FIELDS, assert_comp_close, assert_pulse_close, assert_state_equal, bits,
                             push_to_edges)

pytestmark = pytest.mark.gpu


def _scenes():
    """Uneven instances: sizes from 1 to 20k, different debris mixes, gate
    counts, scans and concepts (one scene's LES volumes shared by all)."""
    A = synth.make_scene(num_rain=20000, debris=[(synth.OBJ_LEAF, 256), (synth.OBJ_WOODBOARD_2X4, 256),
                                                 (synth.OBJ_BRICK, 256)], les_count=2, seed=11)
    push_to_edges(A)
    B = synth.make_scene(num_rain=3000, gates=24, gate_spacing=20.0, concept=0, with_tables=False, seed=12,
                         scan=synth.rhi_positions(2.0, 0.5, 20.0, 0.5))
    C = synth.make_scene(num_rain=1, with_tables=False, seed=13)
    D = synth.make_scene(num_rain=65, debris=[(synth.OBJ_BRICK, 1000)], with_tables=False, seed=14,
                         concept=synth.CONCEPT_DRAGGED | synth.CONCEPT_CROSS_POL)
    for S in (B, C, D):
        S.les, S.les_cfg, S.les_desc = A.les, A.les_cfg, A.les_desc
    return [A, B, C, D]


@pytest.fixture(scope="module")
def scenes():
    return _scenes()


def _workers(backend, scenes, precision=0):
    ws = []
    for S in scenes:
        W = backend.Worker(0)
        synth.load_worker(W, S)
        W.set_precision(precision)
        ws.append(W)
    return ws


def _steps(scenes, k0, count, les_of=lambda k: 0):
    sims = np.zeros((count, len(scenes), 16), np.float32)
    les = np.zeros((count, len(scenes)), np.int32)
    for j in range(count):
        k = k0 + j
        for i, S in enumerate(scenes):
            sims[j, i] = synth.pulse_sim_desc(S, k + i, tic=k * 1e-3)
            les[j, i] = les_of(k)
    return sims, les


def test_batch_matches_oracle(backend, oracle_lib, scenes):
    """Six steps in two graph runs of three, with a LES slot swap in the
    second: state bit-exact and pulses within the summation bound, for every
    instance."""
    O = oracle_lib
    ws = _workers(backend, scenes)
    B = backend.Batch(ws)
    B.set_populations([synth.population(S) for S in scenes])
    sts = [O.OracleState(S.state) for S in scenes]
    les_of = lambda k: 0 if k < 4 else 1
    for k0 in (0, 3):
        sims, les = _steps(scenes, k0, 3, les_of)
        pulses = B.run(sims, les, use_graph=True)
        for j in range(3):
            for i, S in enumerate(scenes):
                sd = sims[j, i]
                direct, ab = O.make_pulse_direct(sts[i], S, sd, return_abs=True)
                g = pulses[j, i, :S.range_count]
                assert np.isfinite(g).all()
                assert_pulse_close(g, direct, ab, "instance %d step %d" % (i, k0 + j))
                O.advance_time(sts[i], S, S.counts, S.les[les[j, i]], sd)
        for i, W in enumerate(ws):
            assert_state_equal(W.download(STATE_FIELDS), sts[i].s, where="instance %d after step %d " % (i, k0 + 2))
    assert B.launch_count == 18   # per step: pulse, background advance, debris advance
    # respawns happened in the big instance and were reproduced
    assert (bits(sts[0].s["rnd"]) != bits(scenes[0].state["rnd"])).any(axis=1).sum() >= 64
    B.close()
    for W in ws:
        W.close()


def test_batch_les_refill(backend, oracle_lib, scenes):
    """An LES slot refilled on the copy stream between runs is what the next
    run that reads it sees: slot 1 is refilled with volume 0 while the
    instances step on slot 0, then they step on slot 1."""
    O = oracle_lib
    sub = [scenes[0], scenes[3]]
    ws = _workers(backend, sub)
    B = backend.Batch(ws)
    B.set_populations([synth.population(S) for S in sub])
    sts = [O.OracleState(S.state) for S in sub]
    sims, les = _steps(sub, 0, 2)
    B.run(sims, les, download=False, wait=False)
    v = sub[0].les[0]
    for i in range(len(sub)):
        B.set_les_async(i, 1, v.uvwt, v.cpxx)
    sims2, les2 = _steps(sub, 2, 2, les_of=lambda k: 1)
    B.run(sims2, les2)
    B.synchronize()
    for i, S in enumerate(sub):
        for j in range(2):
            O.advance_time(sts[i], S, S.counts, S.les[0], sims[j, i])
        for j in range(2):
            O.advance_time(sts[i], S, S.counts, S.les[0], sims2[j, i])
        assert_state_equal(ws[i].download(STATE_FIELDS), sts[i].s, where="instance %d " % i)
    B.close()
    for W in ws:
        W.close()


def test_batch_graph_equals_stream(backend, scenes):
    """The captured graph and the stream-ordered launches give the same state
    bit for bit, and the same pulses within the summation bound."""
    wa = _workers(backend, scenes)
    wb = _workers(backend, scenes)
    Ba, Bb = backend.Batch(wa), backend.Batch(wb)
    pops = [synth.population(S) for S in scenes]
    Ba.set_populations(pops)
    Bb.set_populations(pops)
    for k0 in (0, 2, 4):
        sims, les = _steps(scenes, k0, 2)
        pa = Ba.run(sims, les, use_graph=True)
        pb = Bb.run(sims, les, use_graph=False)
        scale = np.abs(pb).max(axis=(2, 3), keepdims=True) + 1e-30
        assert np.all(np.abs(pa - pb) <= 1e-4 * scale)
    for x, y in zip(wa, wb):
        sa, sb = x.download(STATE_FIELDS), y.download(STATE_FIELDS)
        for f in STATE_FIELDS:
            assert np.array_equal(bits(sa[f]), bits(sb[f])), f
    for o in [Ba, Bb] + wa + wb:
        o.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_persistent_equals_graph(backend, oracle_lib, scenes, precision):
    """The persistent form -- every step of a run in one launch -- against
    the three-launch graph over runs of 3, 1 and 2 steps (odd runs leave the
    state in the other pos / rcs pair): the state bit for bit, the pulses
    within the summation bound, one launch per run; and the state after the
    runs is the oracle's."""
    O = oracle_lib
    wa = _workers(backend, scenes, precision=precision)
    wb = _workers(backend, scenes, precision=precision)
    Ba, Bb = backend.Batch(wa), backend.Batch(wb)
    pops = [synth.population(S) for S in scenes]
    Ba.set_populations(pops)
    Bb.set_populations(pops)
    Ba.set_precision(precision)
    Bb.set_precision(precision)
    Bb.set_persistent(True)
    sts = [O.OracleState(S.state) for S in scenes]
    k0 = 0
    for run in (3, 1, 2):
        sims, les = _steps(scenes, k0, run)
        n0 = Bb.launch_count
        pa = Ba.run(sims, les, use_graph=True)
        pb = Bb.run(sims, les)
        assert Bb.launch_count - n0 == 1
        scale = np.abs(pa).max(axis=(2, 3), keepdims=True) + 1e-30
        assert np.all(np.isfinite(pb))
        assert np.all(np.abs(pa - pb) <= 1e-4 * scale), np.abs(pa - pb).max()
        for j in range(run):
            for i, S in enumerate(scenes):
                O.advance_time(sts[i], S, S.counts, S.les[0], sims[j, i])
        for x, y in zip(wa, wb):
            sa, sb = x.download(STATE_FIELDS), y.download(STATE_FIELDS)
            for f in STATE_FIELDS:
                assert np.array_equal(bits(sa[f]), bits(sb[f])), (f, k0)
        k0 += run
    for i, W in enumerate(wb):
        assert_state_equal(W.download(STATE_FIELDS), sts[i].s, where="instance %d " % i)
    for o in [Ba, Bb] + wa + wb:
        o.close()


def test_batch_advance_shapes(backend, scenes):
    """The batched background advance at every block size and residency the
    autotuner tries leaves the same state bit for bit, with the same pulses
    (up to the order of the FP64 grid sums)."""
    pops = [synth.population(S) for S in scenes]
    ref = None
    for shape in ((128, 0), (64, 0), (256, 4), (128, 8)):
        ws = _workers(backend, scenes)
        B = backend.Batch(ws)
        B.set_populations(pops)
        B.set_advance_shape(*shape)
        assert B.advance_shape == shape
        sims, les = _steps(scenes, 0, 3)
        p = B.run(sims, les)
        st = [W.download(STATE_FIELDS) for W in ws]
        if ref is None:
            ref = (p, st)
        else:
            scale = np.abs(ref[0]).max(axis=(2, 3), keepdims=True) + 1e-30
            assert np.all(np.abs(p - ref[0]) <= 1e-6 * scale), shape
            for a, r in zip(st, ref[1]):
                for f in STATE_FIELDS:
                    assert np.array_equal(bits(a[f]), bits(r[f])), (shape, f)
        for o in [B] + ws:
            o.close()


def test_batch_autotune_and_compensated(backend, oracle_lib, scenes):
    """The autotuner picks a reachable shape and leaves the state alone; the
    compensated form in a batch keeps its bound against FP64."""
    O = oracle_lib
    ws = _workers(backend, scenes, precision=1)
    B = backend.Batch(ws)
    B.set_populations([synth.population(S) for S in scenes])
    B.set_precision(1)
    sims, les = _steps(scenes, 0, 2)
    warps, per_sm = B.autotune(sims[0])
    assert warps in (4, 8, 16) and 1 <= per_sm <= 4
    threads, adv_per_sm = B.advance_shape
    assert threads in (64, 128, 256) and adv_per_sm in (0, 1024 // threads)
    for i, W in enumerate(ws):
        assert_state_equal(W.download(STATE_FIELDS), scenes[i].state, where="instance %d after autotune " % i)
    sts = [O.OracleState(S.state) for S in scenes]
    pulses = B.run(sims, les)
    for j in range(2):
        for i, S in enumerate(scenes):
            r64, ab = O.make_pulse_f64(sts[i], S, sims[j, i], return_abs=True)
            assert_comp_close(pulses[j, i, :S.range_count], r64, ab, "instance %d step %d" % (i, j))
            O.advance_time(sts[i], S, S.counts, S.les[0], sims[j, i])
    for i, W in enumerate(ws):
        assert_state_equal(W.download(STATE_FIELDS), sts[i].s, where="instance %d " % i)
    B.close()
    for W in ws:
        W.close()


def test_worker_autotune(backend, scenes):
    S = scenes[0]
    W = backend.Worker(0)
    synth.load_worker(W, S)
    sd = synth.pulse_sim_desc(S, 0)
    W.make_pulse(sd)
    ref = W.download_pulse(1.0)
    warps, per_sm = W.autotune(sd)
    assert warps in (4, 8, 16) and 1 <= per_sm <= 4
    W.make_pulse(sd)
    g = W.download_pulse(1.0)
    assert np.all(np.abs(g - ref) <= 1e-4 * np.abs(ref).max())
    # shapes set by hand (one warp per block up to the largest that fits)
    for shape in ((1, 1), (8, 3), (16, 4), (0, 0)):
        W.set_pulse_shape(*shape)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        assert np.all(np.abs(g - ref) <= 1e-4 * np.abs(ref).max()), shape
    with pytest.raises(backend.BackendError):
        W.set_pulse_shape(17, 1)
    assert_state_equal(W.download(STATE_FIELDS), S.state, where="after autotune ")
    W.close()


def test_batch_errors(backend, scenes):
    """Bad descriptors are refused with a status, before any launch."""
    ws = _workers(backend, scenes[1:3])
    B = backend.Batch(ws)
    sims, les = _steps(scenes[1:3], 0, 2)
    with pytest.raises(backend.BackendError):   # populations not set
        B.run(sims, les)
    B.set_populations([synth.population(S) for S in scenes[1:3]])
    bad = les.copy()
    bad[1, 0] = 2                               # no such LES slot
    with pytest.raises(backend.BackendError):
        B.run(sims, bad)
    bad_sims = sims.copy()
    bad_sims[1, 1, 5] = synth.fbits(synth.CONCEPT_FIXED_POS)   # concept changes within the run
    with pytest.raises(backend.BackendError):
        B.run(bad_sims, les)
    with pytest.raises(backend.BackendError):
        B.set_precision(7)
    with pytest.raises(backend.BackendError):
        backend.Batch([ws[0], ws[0]])
    assert B.launch_count == 0
    B.close()
    for W in ws:
        W.close()


def test_partial_population_batch_and_worker(backend, oracle_lib):
    """Scatterers outside the population (here the last debris type) keep
    their position and backscatter while the others advance into the other
    pos / rcs pair, and they still take part in every pulse: batch runs of an
    odd step count interleaved with one-worker steps on the advance stream,
    with spatial sorts between them."""
    O = oracle_lib
    S = synth.make_scene(num_rain=6000, debris=[(synth.OBJ_LEAF, 256), (synth.OBJ_WOODBOARD_2X4, 256),
                                                (synth.OBJ_BRICK, 256)], les_count=1, seed=21)
    push_to_edges(S)
    counts = list(S.counts)
    counts[-1] = 0
    pop = backend.Population.make(counts)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    W.set_sort_interval(2)
    B = backend.Batch([W])
    B.set_populations([pop])
    st = O.OracleState(S.state)
    k = 0

    def check_pulse(g, sd, where):
        direct, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
        assert np.isfinite(g).all()
        assert_pulse_close(g, direct, ab, where)

    for rnd in range(2):
        sims = np.stack([synth.pulse_sim_desc(S, k + j, tic=(k + j) * 1e-3) for j in range(3)])[:, None, :]
        pulses = B.run(sims, np.zeros((3, 1), np.int32), use_graph=rnd == 1)
        for j in range(3):
            check_pulse(pulses[j, 0, :S.range_count], sims[j, 0], "batch step %d" % (k + j))
            O.advance_time(st, S, counts, S.les[0], sims[j, 0])
        k += 3
        for _ in range(2):
            sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
            W.make_pulse(sd)
            check_pulse(W.download_pulse(1.0), sd, "worker step %d" % k)
            W.advance_time(pop, 0, sd)
            O.advance_time(st, S, counts, S.les[0], sd)
            k += 1
        assert_state_equal(W.download(STATE_FIELDS), st.s, where="after step %d " % (k - 1))
    # the last type never moved
    lo = sum(counts)
    assert np.array_equal(bits(st.s["pos"][lo:]), bits(S.state["pos"][lo:]))
    B.close()
    W.close()


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_mixed_instances_odd_runs(backend, oracle_lib, use_graph):
    """A debris-only instance, one whose last debris type lies outside its
    population and one plain instance, stepped in runs of 1 and 3 steps (each
    run leaves the state in the other pos / rcs pair): every instance bit-exact
    against the oracle and its pulses within the summation bound."""
    O = oracle_lib
    A = synth.make_scene(num_rain=0, debris=[(synth.OBJ_LEAF, 700), (synth.OBJ_BRICK, 300)], les_count=1, seed=41)
    push_to_edges(A, n_rain=0, n_deb=40)
    B = synth.make_scene(num_rain=9000, debris=[(synth.OBJ_LEAF, 200), (synth.OBJ_BRICK, 200)], with_tables=False,
                         seed=42)
    C = synth.make_scene(num_rain=4000, with_tables=False, seed=43)
    for S in (B, C):
        S.les, S.les_cfg, S.les_desc = A.les, A.les_cfg, A.les_desc
    scenes = [A, B, C]
    counts = [list(S.counts) for S in scenes]
    counts[1][-1] = 0
    pops = [backend.Population.make(c) for c in counts]
    ws = []
    for S in scenes:
        W = backend.Worker(0)
        synth.load_worker(W, S)
        ws.append(W)
    Bt = backend.Batch(ws)
    Bt.set_populations(pops)
    sts = [O.OracleState(S.state) for S in scenes]
    k0 = 0
    for run in (1, 3, 1):
        sims, les = _steps(scenes, k0, run)
        pulses = Bt.run(sims, les, use_graph=use_graph)
        for j in range(run):
            for i, S in enumerate(scenes):
                direct, ab = O.make_pulse_direct(sts[i], S, sims[j, i], return_abs=True)
                assert_pulse_close(pulses[j, i, :S.range_count], direct, ab, "instance %d step %d" % (i, k0 + j))
                O.advance_time(sts[i], S, counts[i], S.les[0], sims[j, i])
        for i, W in enumerate(ws):
            assert_state_equal(W.download(STATE_FIELDS), sts[i].s, where="instance %d after step %d " % (i, k0 + run - 1))
        k0 += run
    Bt.close()
    for W in ws:
        W.close()
