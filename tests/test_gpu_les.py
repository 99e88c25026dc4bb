"""LES frames from files to the device (rsc_les_upload_async): the raw planes
copied on the worker's copy stream and remapped by k_les_remap give the same
scatterer state, bit for bit, as the oracle advancing on the frame that the
backend's host reader returns (rsc_les_read, pinned bit for bit to les.c by
tests/test_ref_loaders.py), with the upload queued behind and ahead of
advances that read the slot."""
import numpy as np
import pytest

from simradar_gb300 import rsc, synth

from test_gpu_parity import STATE_FIELDS, assert_state_equal, push_to_edges

pytestmark = pytest.mark.gpu


class Vol:
    def __init__(self, uvwt, cpxx):
        self.uvwt, self.cpxx = uvwt, cpxx


def scene_and_folder(tmp_path, config, concept=synth.CONCEPT_DBU, frames=4):
    cfg = synth.LESConfig(nx=96, ny=96, nz=48)
    S = synth.make_scene(num_rain=30000, debris=[(synth.OBJ_LEAF, 512)], les_cfg=cfg, les_count=frames,
                         concept=concept)
    rng = np.random.default_rng(9)
    for v in S.les:
        v.cpxx[..., 0] = rng.uniform(-14.0, -12.0, v.cpxx.shape[:3])
    push_to_edges(S)
    d = str(tmp_path / config)
    synth.write_les_folder(d, cfg, S.les, config=config)
    return S, d


def oracle_volume(d, config, n):
    """Frame n as the host reader gives it (a reader of its own, so that the
    device upload's reads are not disturbed)."""
    with rsc.LESSource(d, config) as src:
        uvwt, cpxx, _ = src.read(n)
    return Vol(uvwt, cpxx)


@pytest.mark.parametrize("config", ["suctvort", "flat"])
def test_upload_matches_oracle(backend, oracle_lib, tmp_path, config):
    concept = synth.CONCEPT_DBU if config == "suctvort" else synth.CONCEPT_FIXED_POS
    S, d = scene_and_folder(tmp_path, config, concept)
    src = backend.LESSource(d, config)
    desc = src.descriptor()
    if config == "suctvort":
        assert np.array_equal(desc.view(np.uint32), S.les_cfg.desc().view(np.uint32))
    S.les_desc = desc
    pop = synth.population(S)
    W = backend.Worker(0)
    synth.load_worker(W, S, les_slot_volumes=())
    t0 = src.upload_async(W, 0, 0)
    assert t0 == 0.0
    st = oracle_lib.OracleState(S.state)
    vols = {0: oracle_volume(d, config, 0)}
    slot_frame = {0: 0}
    # (slot read by the advance, upload before it: (slot, frame) or None)
    plan = [(0, (1, 1)), (0, None), (1, None), (1, (1, 2)), (1, (0, 3)), (0, None), (1, None)]
    for k, (slot, up) in enumerate(plan):
        if up is not None:
            s_up, f_up = up
            assert src.upload_async(W, s_up, f_up) == np.float32(f_up * float(S.les_cfg.tp))
            slot_frame[s_up] = f_up
            vols.setdefault(f_up, oracle_volume(d, config, f_up))
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        W.advance_time(pop, slot, sd)
        W.make_pulse(sd)
        oracle_lib.advance_time(st, S, S.counts, vols[slot_frame[slot]], sd)
    assert_state_equal(W.download(STATE_FIELDS), st.s, where=config + " ")
    W.close()
    src.close()


def test_upload_beside_set_les(backend, tmp_path):
    """The same frames through rsc_les_upload_async and through rsc_set_les of
    the host-remapped frame give the same state and pulses."""
    S, d = scene_and_folder(tmp_path, "suctvort")
    src = backend.LESSource(d, "suctvort")
    S.les_desc = src.descriptor()
    pop = synth.population(S)
    A, B = backend.Worker(0), backend.Worker(0)
    for W in (A, B):
        synth.load_worker(W, S, les_slot_volumes=())
    src.upload_async(A, 0, 0)
    uvwt, cpxx, _ = src.read(0)
    B.set_les(0, uvwt, cpxx, S.les_desc)
    for k in range(8):
        sd = synth.pulse_sim_desc(S, k, tic=k * 1e-3)
        slot = (k // 2) % 2
        if k % 2 == 1:
            # refill the other slot while this one is in use
            f = (k // 2 + 1) % 4
            src.upload_async(A, 1 - slot, f)
            uvwt, cpxx, _ = src.read(f)
            B.set_les(1 - slot, uvwt, cpxx, S.les_desc)
        for W in (A, B):
            W.advance_time(pop, slot, sd)
            W.make_pulse(sd)
        # same state, same kernel: the pulses differ only by the order of
        # the FP32 atomic additions
        ga, gb = A.download_pulse(1.0), B.download_pulse(1.0)
        np.testing.assert_allclose(ga, gb, rtol=1e-4, atol=1e-5 * float(np.abs(gb).max()), err_msg=str(k))
    assert_state_equal(A.download(STATE_FIELDS), B.download(STATE_FIELDS))
    A.close()
    B.close()
    src.close()


def test_batch_reads_uploaded_slot(backend, oracle_lib, tmp_path):
    """A batch run that reads a slot filled by rsc_les_upload_async waits for
    the upload: two instances, one of them switching to the uploaded frame."""
    S, d = scene_and_folder(tmp_path, "suctvort")
    src = backend.LESSource(d, "suctvort")
    S.les_desc = src.descriptor()
    T = synth.make_scene(num_rain=5000, les_cfg=S.les_cfg, with_tables=False, seed=31)
    T.les, T.les_desc = S.les, S.les_desc
    scenes = (S, T)
    ws = []
    for X in scenes:
        W = backend.Worker(0)
        synth.load_worker(W, X, les_slot_volumes=())
        src.upload_async(W, 0, 0)
        ws.append(W)
    B = backend.Batch(ws)
    B.set_populations([synth.population(X) for X in scenes])
    sts = [oracle_lib.OracleState(X.state) for X in scenes]
    vols = {f: oracle_volume(d, "suctvort", f) for f in (0, 2)}
    src.upload_async(ws[0], 1, 2)   # instance 0, slot 1 <- frame 2, queued before the run
    steps = 3
    sims = np.zeros((steps, 2, 16), np.float32)
    les = np.zeros((steps, 2), np.int32)
    for j in range(steps):
        for i, X in enumerate(scenes):
            sims[j, i] = synth.pulse_sim_desc(X, j + i, tic=j * 1e-3)
        les[j, 0] = 1
    B.run(sims, les, use_graph=True)
    B.synchronize()
    for j in range(steps):
        for i, X in enumerate(scenes):
            oracle_lib.advance_time(sts[i], X, X.counts, vols[2 if i == 0 else 0], sims[j, i])
    for i, W in enumerate(ws):
        assert_state_equal(W.download(STATE_FIELDS), sts[i].s, where="instance %d " % i)
    B.close()
    for W in ws:
        W.close()
    src.close()
