"""rsc_populate_upload: the state generated in blocks and copied while the
next block is generated equals the host generation, slot for slot; the
backend then steps it as any uploaded state."""
import numpy as np
import pytest

from simradar_gb300 import rsc, synth

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "ori", "tum", "aux", "rcs", "rnd")


def test_populate_upload_equals_host(backend):
    S = synth.make_scene(num_rain=1_500_000, debris=[(synth.OBJ_LEAF, 5000), (synth.OBJ_BRICK, 5000)],
                         les_count=1, with_tables=True, seed=3)
    ox, oy, oz, sx, sy, sz = S.box
    args = rsc.PopulateArgs.make(19760520, S.concept, (ox, oy, oz), (sx, sy, sz), S.counts, S.dsd_r, S.dsd_cdf)
    host, pop_h = rsc.populate_host(args, S.num_scats)
    W = backend.Worker(0)
    synth.load_worker(W, S)            # tables and an unrelated state, replaced below
    pop_d = rsc.populate_upload(W, args)
    got = W.download(FIELDS)
    for f in FIELDS:
        assert np.array_equal(got[f].view(np.uint32), host[f].view(np.uint32)), f
    assert np.array_equal(pop_d, pop_h)
    # and it steps: one pulse and one advance on the populated state
    sd = synth.pulse_sim_desc(S, 0)
    W.make_pulse(sd)
    assert np.isfinite(W.download_pulse(1.0)).all()
    W.advance_time(synth.population(S), 0, sd)
    assert np.isfinite(W.download(("pos",))["pos"]).all()
    W.close()
