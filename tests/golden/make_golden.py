"""Generate the golden fixture tests/golden/scene_small.npz.

A seeded small scene with every table the path reads (LES 20x20x10 stretched
with a wide base spacing so the box lies inside it, ADM / RCS images 25x13 for
three debris types, the standard range and angular weights, the ellipsoid
table), 512 rain + 3 x 32 debris scatterers, some of them placed at the box
edges moving out so that respawns (the RNG) are exercised, and four steps of
the oracle: the reference-order pulse, the exact and FP64 sums with their
absolute sums, and the state after the last step.

The fixture pins the oracle and the GPU against regressions; it is made by
the oracle, not by the reference (whose OpenCL path does not run here).  A
deliberate change of the shared elementary functions (rsmath.h) changes the
state bits on both sides at once; the fixture is then made again with this
script.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from simradar_gb300 import synth  # noqa: E402

STEPS = 4
FIELDS = ("pos", "vel", "ori", "tum", "aux", "rcs", "sig", "rnd")


def scene():
    cfg = synth.LESConfig(nx=20, ny=20, nz=10, ax=60.0, ay=60.0, az=90.0)
    S = synth.make_scene(num_rain=512, debris=[(synth.OBJ_LEAF, 32), (synth.OBJ_WOODBOARD_2X4, 32),
                                               (synth.OBJ_BRICK, 32)],
                         les_cfg=cfg, les_count=2, seed=20240607, les_seed=5)
    S.adm = [synth.adm_table(o, seed=100 + t, nb=25, na=13) for t, o in enumerate(S.debris_objs)]
    S.rcs_tables = [synth.rcs_table(seed=200 + t, na=25, nb=13) for t in range(len(S.debris_objs))]
    ox, oy, oz, sx, sy, sz = S.box
    pos, vel = S.state["pos"], S.state["vel"]
    pos[:16, 0] = np.float32(ox) + np.float32(1e-3)
    vel[:16, 0] = -5.0
    pos[16:32, 2] = np.float32(oz + sz) - np.float32(1e-3)
    vel[16:32, 2] = 5.0
    d0 = S.counts[0]
    pos[d0:d0 + 8, 1] = np.float32(oy) + np.float32(1e-3)
    vel[d0:d0 + 8, 1] = -5.0
    return S


def sim_descs(S):
    out = []
    for k in range(STEPS):
        sd = synth.pulse_sim_desc(S, 3 * k + 40, tic=k * 1e-3)
        out.append(sd)
    return np.stack(out)


def main():
    O.build()
    S = scene()
    sds = sim_descs(S)
    st = O.OracleState(S.state)
    ref, direct, dabs, f64, fabs_ = [], [], [], [], []
    for k in range(STEPS):
        sd = sds[k]
        d, a = O.make_pulse_direct(st, S, sd, return_abs=True)
        e, b = O.make_pulse_f64(st, S, sd, return_abs=True)
        ref.append(O.make_pulse(st, S, sd))
        direct.append(d)
        dabs.append(a)
        f64.append(e)
        fabs_.append(b)
        O.advance_time(st, S, S.counts, S.les[0], sd)
    arrays = dict(
        sim_descs=sds, counts=np.array(S.counts, np.int64), box=np.array(S.box, np.float64),
        range=np.array([S.range_start, S.range_delta, S.range_count], np.float64),
        range_w=S.range_w, range_desc=S.range_desc, ang_w=S.ang_w, ang_desc=S.ang_desc,
        ell=S.ell, ell_desc=S.ell_desc, les_desc=S.les_desc,
        les0_uvwt=S.les[0].uvwt, les0_cpxx=S.les[0].cpxx,
        pulse_ref=np.stack(ref), pulse_direct=np.stack(direct), pulse_abs=np.stack(dabs),
        pulse_f64=np.stack(f64), pulse_f64_abs=np.stack(fabs_))
    for t, (cd, cm, ad) in enumerate(S.adm):
        arrays["adm%d_cd" % t], arrays["adm%d_cm" % t], arrays["adm%d_desc" % t] = cd, cm, ad
    for t, (re, im, rd) in enumerate(S.rcs_tables):
        arrays["rcs%d_re" % t], arrays["rcs%d_im" % t], arrays["rcs%d_desc" % t] = re, im, rd
    for f in FIELDS:
        arrays["in_" + f] = S.state[f]
        if f not in ("aux", "sig"):
            arrays["out_" + f] = st.s[f]
    path = os.path.join(HERE, "scene_small.npz")
    np.savez_compressed(path, **arrays)
    resp = int((st.s["rnd"] != S.state["rnd"]).any(axis=1).sum())
    print("wrote %s (%d bytes): %d scatterers, %d steps, %d respawned, pulse max %.3g" % (
        path, os.path.getsize(path), S.num_scats, STEPS, resp, np.abs(np.stack(direct)).max()))


if __name__ == "__main__":
    main()
