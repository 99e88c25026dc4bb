"""The reference's workloads as parity cases on the GPU, at their own sizes,
through the C ABI against the oracle:

* 131,072 rain scatterers, concept DBU, PPI 3.0 deg -12..12 deg / 0.24 deg,
  40 gates: all 100 pulses of that run, the state bit-exact and every pulse
  within the FP32 summation bound of the reference's own order;
* the README-scale workload (1,998,848 rain + 1024 each of leaf, 2x4 board
  and brick): a few pulses, the same checks;
* 8,388,608 rain with the box and the gates 30 km out, 64 pulses: the state
  bit-exact, the plain pulse against the reference's order and the
  compensated pulse against the FP64 pulse of the same state;
* 33,554,432 rain + 131,072 debris on a 352 x 352 x 160 LES, RHI, as a
  batch of one in the compensated form;
* the 64-instance batching workload (synth.batch_workload).
"""
import numpy as np
import pytest

from simradar_gb300 import synth

from test_gpu_parity import STATE_FIELDS, assert_comp_close, assert_pulse_close, assert_state_equal

pytestmark = pytest.mark.gpu


def step_against_oracle(backend, O, S, pulses, check_every, compensated_every=0):
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    st = O.OracleState(S.state)
    for k in range(pulses):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        W.make_pulse(sd)
        g = W.download_pulse(1.0)
        assert np.isfinite(g).all(), "pulse %d" % k
        r = O.make_pulse(st, S, sd)
        r64, ab = O.make_pulse_f64(st, S, sd, return_abs=True)
        assert_pulse_close(g, r, ab, "pulse %d vs the reference's order" % k)
        if compensated_every and k % compensated_every == 0:
            W.set_precision(1)
            W.make_pulse(sd)
            assert_comp_close(W.download_pulse(1.0), r64, ab, "compensated pulse %d" % k)
            W.set_precision(0)
        W.advance_time(pop, 0, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
        if (k + 1) % check_every == 0 or k == pulses - 1:
            assert_state_equal(W.download(STATE_FIELDS), st.s, where="after pulse %d " % k)
    W.close()
    return st


def test_ppi_131072_all_pulses(backend, oracle_lib):
    S = synth.make_scene(num_rain=131072, gates=40)
    assert len(S.scan) == 101
    st = step_against_oracle(backend, oracle_lib, S, 100, check_every=25, compensated_every=33)
    # the run moved every scatterer and respawned some
    assert (st.s["pos"] != S.state["pos"]).any(axis=1).all()


def test_readme_scale(backend, oracle_lib):
    S = synth.make_scene(num_rain=1998848, gates=40,
                         debris=[(synth.OBJ_LEAF, 1024), (synth.OBJ_WOODBOARD_2X4, 1024), (synth.OBJ_BRICK, 1024)])
    step_against_oracle(backend, oracle_lib, S, 4, check_every=2, compensated_every=3)


def test_8m_gates_30km(backend, oracle_lib):
    """64 pulses: the compensated pulse of every one against the FP64 pulse
    (per-gate relative error <= 1e-5 raw, 2e-7 where the terms cancel by
    less than 100x), the plain one against the reference's order."""
    S = synth.make_scene(num_rain=8388608, gates=40, les_count=1, range_offset=30000.0, seed=4242,
                         scan=synth.ppi_positions(0.7, -0.6, 0.6, 0.012))
    step_against_oracle(backend, oracle_lib, S, 64, check_every=32, compensated_every=1)


def test_33m_batch_of_one(backend, oracle_lib):
    """33,554,432 rain + 131,072 debris, LES 352 x 352 x 160, RHI 0.5-20 deg,
    compensated form, run as a batch of one (the streaming form): two steps,
    the state bit-exact, both pulses against the FP64 pulse."""
    O = oracle_lib
    cfg = synth.LESConfig(nx=352, ny=352, nz=160)
    S = synth.make_scene(num_rain=33554432, gates=40, les_cfg=cfg, les_count=1, seed=777,
                         debris=[(synth.OBJ_LEAF, 43691), (synth.OBJ_WOODBOARD_2X4, 43691), (synth.OBJ_BRICK, 43690)],
                         scan=synth.rhi_positions(0.0, 0.5, 20.0, 0.02))
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S, les_slot_volumes=(0,))
    st = O.OracleState(S.state)
    S.state = None
    B = backend.Batch([W])
    B.set_populations([pop])
    B.set_precision(1)
    sims = np.stack([synth.pulse_sim_desc(S, k, tic=k * 1e-3) for k in range(2)])[:, None, :]
    pulses = B.run(sims, np.zeros((2, 1), np.int32), use_graph=True)
    for k in range(2):
        r64, ab = O.make_pulse_f64(st, S, sims[k, 0], return_abs=True)
        assert_comp_close(pulses[k, 0, :40], r64, ab, "step %d" % k)
        O.advance_time(st, S, S.counts, S.les[0], sims[k, 0])
    assert_state_equal(W.download(STATE_FIELDS), st.s, where="after two steps ")
    B.close()
    W.close()


def test_64_instances_batched(backend, oracle_lib):
    """The batching workload (64 instances, 53.5 M scatterers in all, sizes
    log-uniform 65,536-4,194,304, PPI / RHI mix), compensated, one graph run
    of two steps: every instance's state bit-exact, every pulse against its
    FP64 pulse."""
    O = oracle_lib
    scenes = synth.batch_workload(64)
    ws, sts = [], []
    for S in scenes:
        W = backend.Worker(0)
        synth.load_worker(W, S)
        ws.append(W)
        sts.append(O.OracleState(S.state))
        S.state = None
    B = backend.Batch(ws)
    B.set_populations([synth.population(S) for S in scenes])
    B.set_precision(1)
    steps = 2
    sims = np.zeros((steps, len(scenes), 16), np.float32)
    for j in range(steps):
        for i, S in enumerate(scenes):
            sims[j, i] = synth.pulse_sim_desc(S, j, tic=j * 1e-3)
    pulses = B.run(sims, np.zeros((steps, len(scenes)), np.int32), use_graph=True)
    for i, S in enumerate(scenes):
        for j in range(steps):
            r64, ab = O.make_pulse_f64(sts[i], S, sims[j, i], return_abs=True)
            assert_comp_close(pulses[j, i, :S.range_count], r64, ab, "instance %d step %d" % (i, j))
            O.advance_time(sts[i], S, S.counts, S.les[0], sims[j, i])
        assert_state_equal(ws[i].download(STATE_FIELDS), sts[i].s, where="instance %d " % i)
    B.close()
    for W in ws:
        W.close()
