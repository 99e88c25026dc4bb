"""Loader of the golden fixture tests/golden/scene_small.npz (made by
tests/golden/make_golden.py) as a scene the oracle and the backend take."""
import os

import numpy as np

from simradar_gb300 import synth

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scene_small.npz")
STATE_FIELDS = ("pos", "vel", "ori", "tum", "rcs", "rnd")


def load():
    z = np.load(PATH)
    S = synth.Scene()
    S.counts = [int(c) for c in z["counts"]]
    S.num_scats = int(sum(S.counts))
    S.box = tuple(float(v) for v in z["box"])
    rs, rd, rc = z["range"]
    S.range_start, S.range_delta, S.range_count = np.float32(rs), np.float32(rd), int(rc)
    S.range_w, S.range_desc = z["range_w"], z["range_desc"]
    S.ang_w, S.ang_desc = z["ang_w"], z["ang_desc"]
    S.ell, S.ell_desc = z["ell"], z["ell_desc"]
    S.les_desc = z["les_desc"]
    S.les = [synth.LESVolume(z["les0_uvwt"], z["les0_cpxx"])]
    n_types = len(S.counts) - 1
    S.adm = [(z["adm%d_cd" % t], z["adm%d_cm" % t], z["adm%d_desc" % t]) for t in range(n_types)]
    S.rcs_tables = [(z["rcs%d_re" % t], z["rcs%d_im" % t], z["rcs%d_desc" % t]) for t in range(n_types)]
    S.state = {f: z["in_" + f].copy() for f in ("pos", "vel", "ori", "tum", "aux", "rcs", "sig", "rnd")}
    S.sim_descs = z["sim_descs"]
    S.expected = {k: z[k] for k in z.files if k.startswith("pulse_") or k.startswith("out_")}
    return S
