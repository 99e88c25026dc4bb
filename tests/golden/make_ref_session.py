"""Record sessions of the reference host (rs.c) as golden fixtures.

rs.c, les.c, adm.c, rcs.c, obj.c, pos.c and log.c are compiled unmodified
from the reference tree with this project's OpenCL shim over the CPU oracle
(oracle/ref/Makefile), and oracle/_ref/refdrive runs simradar's session
(RS_init ... RS_suggest_scan_domain, RS_add_debris, RS_populate, warm-up
advances, then make_pulse / download_pulse_only / merge / advance_time /
advance_beam per pulse) on a reduced density.  The tables folder it reads
is written by synth.write_tables_folder, whose content is the same bytes on
every host, so the GPU test can write it again where the reference tree is
absent.  Each fixture holds what rs.c derived and sent to the device (tables,
descriptors, population layout, the event list with every descriptor), the
pulses it read back, and hashes of the uploaded state, of every LES frame
and of the final state (tests/test_ref_session.py, tests/test_gpu_ref_session.py).
ref_session_dbu_rscl is the DBU session with the device running the
reference's own rs.cl kernels rather than the oracle's.

    python tests/golden/make_ref_session.py [session ...]
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refbind  # noqa: E402
from simradar_gb300 import synth  # noqa: E402

# name: refdrive arguments.  Concepts (rs_enum.h:127-137): 26 = dragged +
# bounded + uniform-DSD (simradar's default DBU); 9 = bounded + cross-pol
# (bg_atts for the background); 154 = DBU + debris flux from velocity (rs.c
# derives the flux field from every LES frame it sets, rs.c:3106-3111, and
# respawned debris take their cell from it); 90 = DBU + vertically pointing
# radar (rs.c's scan box and gates for a radar looking up, rs.c:1602-1640,
# rs.c:2143-2160, rs.c:5830-5860).
SESSIONS = {
    "ref_session_dbu": dict(density=0.3, pulses=40, warmup=130, seed=19760520, gate=30.0,
                            scan="P:3.0,-12:12:0.24", concept=26,
                            debris=[(synth.OBJ_LEAF, 256), (synth.OBJ_WOODBOARD_2X4, 256), (synth.OBJ_BRICK, 256)]),
    "ref_session_bg": dict(density=0.2, pulses=24, warmup=0, seed=4321, gate=15.0,
                           scan="R:2.0,1:15:0.5", concept=9, debris=[(synth.OBJ_BRICK, 300)]),
    "ref_session_dff": dict(density=0.1, pulses=16, warmup=400, seed=2468, gate=30.0,
                            scan="P:3.0,-12:12:0.24", concept=154,
                            debris=[(synth.OBJ_LEAF, 512), (synth.OBJ_BRICK, 512)]),
    "ref_session_vpr": dict(density=0.3, pulses=24, warmup=60, seed=97531, gate=30.0,
                            scan="P:90.0,0:360:1.0", concept=90, debris=[(synth.OBJ_LEAF, 128)]),
}
# The same DBU session with the shim's device running the reference's own
# rs.cl (compiled for the CPU through oracle/ref/clc/opencl_c.hpp) instead of
# the oracle's restatement of its kernels.
SESSIONS["ref_session_dbu_rscl"] = dict(SESSIONS["ref_session_dbu"], kernels="rscl")
TABLES = dict(seed=7, volumes_per_file=10, adm_dims=(37, 19), rcs_dims=(37, 19))


def write_tables(home):
    synth.write_tables_folder(os.path.join(home, "Documents", "tables"), **TABLES)


def record(name, home, work):
    args = SESSIONS[name]
    R = refbind.run_session(os.path.join(work, name + ".bin"), home, **args)
    if int(R["failed"]):
        raise RuntimeError("refdrive reported failed checks for " + name)
    meta = {"density": args["density"], "pulses": args["pulses"], "warmup": args["warmup"], "gate": args["gate"],
            "scan": args["scan"], "concept": args["concept"], "kernels": args.get("kernels", "oracle"),
            "debris": np.array(args["debris"], np.int64).reshape(-1, 2),
            "tables_seed": TABLES["seed"], "tables_volumes_per_file": TABLES["volumes_per_file"],
            "tables_adm_dims": np.array(TABLES["adm_dims"]), "tables_rcs_dims": np.array(TABLES["rcs_dims"])}
    out = {k: np.asarray(v) for k, v in R.items()}
    out.update({"meta_" + k: np.asarray(v) for k, v in meta.items()})
    return out


def main():
    names = sys.argv[1:] or list(SESSIONS)   # record all, or the sessions named
    refbind.build()
    with tempfile.TemporaryDirectory() as home, tempfile.TemporaryDirectory() as work:
        write_tables(home)
        for name in names:
            out = record(name, home, work)
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print("%s: %d scatterers, %d gates, %d events -> %s (%d bytes)" % (
                name, int(out["num_scats"]), int(out["range_count"]), len(out["ev_kind"]), path,
                os.path.getsize(path)))


if __name__ == "__main__":
    main()
