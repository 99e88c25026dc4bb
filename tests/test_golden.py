"""The oracle against the committed golden fixture (tests/golden/): the
state after four steps bit for bit, the reference-order pulse bit for bit,
the exact and FP64 sums to double-precision rounding."""
import numpy as np

import golden_fixture as G


def test_oracle_reproduces_golden(oracle_lib):
    O = oracle_lib
    S = G.load()
    st = O.OracleState(S.state)
    E = S.expected
    for k, sd in enumerate(S.sim_descs):
        d, a = O.make_pulse_direct(st, S, sd, return_abs=True)
        e = O.make_pulse_f64(st, S, sd)
        r = O.make_pulse(st, S, sd)
        assert np.array_equal(r.view(np.uint32), E["pulse_ref"][k].view(np.uint32)), "reference-order pulse %d" % k
        assert np.all(np.abs(d - E["pulse_direct"][k]) <= 1e-12 * E["pulse_abs"][k] + 1e-300), "exact sum %d" % k
        assert np.all(np.abs(e - E["pulse_f64"][k]) <= 1e-12 * E["pulse_f64_abs"][k] + 1e-300), "fp64 sum %d" % k
        assert np.allclose(a, E["pulse_abs"][k], rtol=1e-12, atol=0)
        O.advance_time(st, S, S.counts, S.les[0], sd)
    for f in G.STATE_FIELDS:
        assert np.array_equal(st.s[f].view(np.uint32), E["out_" + f].view(np.uint32)), f
    # the fixture exercises respawns
    assert (E["out_rnd"] != S.state["rnd"]).any(axis=1).sum() >= 16
