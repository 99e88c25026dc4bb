"""The GPU backend, through its C ABI, against the reference's own known
answers (no oracle in between):

* test_make_pulse.c (test_make_pulse.c:553-653): the `pop` fixture
  (rs.cl:1444-1453), a {0, 1, 0} range weight over [-25, 25] m, a
  {0, .7, 1, .7, 0} angular weight at 10 degree steps, 9 gates from 1 m every
  0.25 m; every pulse form must pass the reference's CPU loop check.
* test_clreduce.c (test_clreduce.c:95-179): the `ramp` fill i mod 32 over
  2^21 elements sums to 32,505,856 per lane.  Here the ramp is the
  backscatter of 2^21 scatterers at range 1 m on the beam axis with unit
  weights and zero phase, so gate 0 must hold that sum exactly in all four
  lanes (integer partial sums stay exact through the per-warp FP32 bins and
  the FP64 accumulator).
"""
import numpy as np
import pytest

from test_oracle import F, assert_kat, kat_cpu_pulse, kat_setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_make_pulse_known_answer_on_gpu(backend, oracle_lib, precision):
    n, sd, rw, rwd, aw, awd = kat_setup()
    G, r0, dr = 9, F(1.0), F(0.25)
    rcs = np.zeros((n, 4), np.float32)
    aux = np.zeros((n, 4), np.float32)
    pos = np.zeros((n, 4), np.float32)
    oracle_lib.lib().or_pop(oracle_lib.fp(rcs), oracle_lib.fp(aux), oracle_lib.fp(pos), oracle_lib.fp(sd), n)
    W = backend.Worker(0)
    W.malloc(n, float(r0), float(dr), G)
    W.set_range_weight(rw, rwd)
    W.set_angular_weight(aw, awd)
    W.upload(0, pos=pos, rcs=rcs, aux=aux)
    W.set_precision(precision)
    W.make_pulse(sd)
    pulse = W.download_pulse(1.0)
    r_a = np.sqrt((pos[:, 0] * pos[:, 0] + pos[:, 1] * pos[:, 1] + pos[:, 2] * pos[:, 2]).astype(np.float32))
    cpu = kat_cpu_pulse(pos, rcs, r_a.astype(np.float32), sd, rw, rwd, aw, awd, G, r0, dr)
    assert_kat(pulse, cpu)
    W.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_reduce_ramp_known_answer(backend, precision):
    n = 1 << 21
    G = 4
    W = backend.Worker(0)
    W.malloc(n, 1.0, 0.25, G)
    rw = np.array([0.0, 1.0, 0.0], np.float32)
    xs = F(F(1.0) / F(25.0))
    W.set_range_weight(rw, np.array([xs, F(F(25.0) * xs), F(2.0), 0.0], np.float32))
    W.set_angular_weight(np.ones(4, np.float32), np.array([1.0, 0.0, 3.0, 0.0], np.float32))
    pos = np.zeros((n, 4), np.float32)
    pos[:, 1] = 1.0                                   # range 1 m on the beam axis
    ramp = (np.arange(n) % 32).astype(np.float32)     # test_clreduce.c's ramp
    rcs = np.repeat(ramp[:, None], 4, axis=1)
    W.upload(0, pos=pos, rcs=rcs)
    W.set_precision(precision)
    sd = np.zeros(16, np.float32)
    sd[1] = 1.0                                       # beam along +y, wave number 0: zero phase
    W.make_pulse(sd)
    pulse = W.download_pulse(1.0)
    assert int(ramp.sum(dtype=np.float64)) == 32505856
    assert np.all(pulse[0] == np.float32(32505856.0)), pulse[0]
    W.close()
