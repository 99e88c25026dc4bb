"""rsc_make_pulse_noalloc: the pulse entry point that allocates no device
memory, for callers that cannot call cudaMalloc (a real-time pulse loop, a
host whose device memory another allocator owns, code recording work where
allocation is forbidden).  Through the C ABI, on the caller's own device
buffers, two calls in a row must agree with the oracle's pulse and with
rsc_make_pulse on the same state within the pulse tolerance of the parity
tests, on the triangle range weight (sparse gate window) and on a table with
non-zero edges (every gate).

This file sorts last so that a run stopping at the first failure has run
every other test first.
"""
import ctypes

import numpy as np
import pytest

from simradar_gb300 import synth

pytestmark = pytest.mark.gpu

PULSE_TOL = 2.0e-5   # same bound as tests/test_gpu_parity.py


def _bind(lib):
    f = ctypes.POINTER(ctypes.c_float)
    fn = lib.rsc_make_pulse_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, f, ctypes.c_uint32, f, f, ctypes.c_uint32, f,
                   ctypes.c_float, ctypes.c_float, ctypes.c_uint32, f, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _scene(dense):
    S = synth.make_scene(num_rain=30000, debris=[(synth.OBJ_LEAF, 256)], les_count=1)
    if dense:
        # a range weight with non-zero edges: every gate is visited (the
        # dense path) instead of the triangle's sparse window
        S.range_w = np.array([0.25, 1.0, 0.5], np.float32)
    return S


@pytest.mark.parametrize("dense", [False, True], ids=["triangle", "dense"])
def test_noalloc_matches_oracle_and_worker(backend, oracle_lib, dense):
    """Two calls in a row on the caller's own device buffers: each pulse
    against the oracle's exact sum of the reference's FP32 terms and against
    rsc_make_pulse of the same state."""
    torch = pytest.importorskip("torch")
    lib = backend.load_library()
    noalloc = _bind(lib)
    S = _scene(dense)
    W = backend.Worker(0)
    synth.load_worker(W, S)
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(S.state["pos"]).to(dev).contiguous()
    rcs = torch.from_numpy(S.state["rcs"]).to(dev).contiguous()
    pulse = torch.full((S.range_count, 4), float("nan"), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = oracle_lib.OracleState(S.state)
    for call, k in enumerate((4, 11)):
        sd = synth.pulse_sim_desc(S, k)
        W.make_pulse(sd)
        worker = W.download_pulse(1.0).astype(np.float64)
        rc = noalloc(pos.data_ptr(), rcs.data_ptr(), S.num_scats, _fp(S.range_w), S.range_w.size, _fp(S.range_desc),
                     _fp(S.ang_w), S.ang_w.size, _fp(S.ang_desc), float(S.range_start), float(S.range_delta),
                     S.range_count, _fp(sd), pulse.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.rsc_last_error()
        torch.cuda.synchronize(dev)
        got = pulse.cpu().numpy().astype(np.float64)
        exact, ab = oracle_lib.make_pulse_direct(st, S, sd, return_abs=True)
        assert np.isfinite(got).all(), "call %d" % call
        assert np.any(got != 0.0), "call %d" % call
        assert np.all(np.abs(got - exact) <= PULSE_TOL * ab + 1e-30), "call %d vs the oracle" % call
        assert np.all(np.abs(got - worker) <= PULSE_TOL * ab + 1e-30), "call %d vs rsc_make_pulse" % call
    W.close()


def test_noalloc_rejects_sizes_beyond_its_limits(backend):
    lib = backend.load_library()
    noalloc = _bind(lib)
    one = np.zeros(4, np.float32)
    sd = np.zeros(16, np.float32)
    w = np.array([0.0, 1.0, 0.0], np.float32)
    d = np.array([1.0, 1.0, 2.0, 0.0], np.float32)
    rc = noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 10, _fp(w), 3, _fp(d), _fp(w), 3, _fp(d), 0.0, 1.0,
                 129, _fp(sd), ctypes.c_void_p(16), None)
    assert rc == -1 and b"128" in lib.rsc_last_error()
    big = np.zeros(65, np.float32)
    rc = noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 10, _fp(big), 65, _fp(d), _fp(w), 3, _fp(d), 0.0, 1.0,
                 8, _fp(sd), ctypes.c_void_p(16), None)
    assert rc == -1 and b"64" in lib.rsc_last_error()
    # a descriptor whose max index is not a finite index inside the table
    for bad in (np.inf, np.nan, 3.0, 1.0e30):
        dd = np.array([1.0, 1.0, bad, 0.0], np.float32)
        rc = noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 10, _fp(w), 3, _fp(dd), _fp(w), 3, _fp(d), 0.0, 1.0,
                     8, _fp(sd), ctypes.c_void_p(16), None)
        assert rc == -1 and b"max index" in lib.rsc_last_error(), bad
    del one
