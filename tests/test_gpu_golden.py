"""The GPU backend (through its C ABI) against the committed golden fixture:
state after four steps bit for bit, pulses within the FP32 summation bound
of the exact sum, the FP64 mode within 1e-6 of the FP64 sum, one-instance and
batched paths."""
import numpy as np
import pytest

import golden_fixture as G
from simradar_gb300 import synth
from test_gpu_parity import PULSE_TOL, assert_comp_close

pytestmark = pytest.mark.gpu


def _worker(backend, S, precision=0):
    W = backend.Worker(0)
    synth.load_worker(W, S)
    W.set_precision(precision)
    return W


def _bits_equal(W, E, where):
    out = W.download(G.STATE_FIELDS)
    for f in G.STATE_FIELDS:
        assert np.array_equal(out[f].view(np.uint32), E["out_" + f].view(np.uint32)), where + f


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_golden_worker(backend, precision):
    S = G.load()
    E = S.expected
    W = _worker(backend, S, precision)
    pop = synth.population(S)
    for k, sd in enumerate(S.sim_descs):
        W.make_pulse(sd)
        g = W.download_pulse(1.0).astype(np.float64)
        if precision == 0:
            assert np.all(np.abs(g - E["pulse_direct"][k]) <= PULSE_TOL * E["pulse_abs"][k] + 1e-30), k
        elif precision == 1:
            assert_comp_close(g, E["pulse_f64"][k], E["pulse_f64_abs"][k], "golden pulse %d" % k)
        else:
            assert np.all(np.abs(g - E["pulse_f64"][k]) <= 1e-6 * E["pulse_f64_abs"][k] + 1e-30), k
        W.advance_time(pop, 0, sd)
    _bits_equal(W, E, "worker precision %d: " % precision)
    W.close()


def test_golden_batch(backend):
    S = G.load()
    E = S.expected
    W = _worker(backend, S)
    B = backend.Batch([W])
    B.set_populations([synth.population(S)])
    sims = S.sim_descs[:, None, :]
    out = B.run(sims, np.zeros((len(sims), 1), np.int32))
    for k in range(len(sims)):
        g = out[k, 0, :S.range_count].astype(np.float64)
        assert np.all(np.abs(g - E["pulse_direct"][k]) <= PULSE_TOL * E["pulse_abs"][k] + 1e-30), k
    _bits_equal(W, E, "batch: ")
    B.close()
    W.close()
