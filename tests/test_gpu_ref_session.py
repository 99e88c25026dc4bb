"""The recorded sessions of the reference host, replayed on the GPU by a C
host through the C ABI (tests/c/host_loop.c, compiled here with gcc against
include/rsc.h and libsimradar_gb300.so).

The host makes the calls rs.c makes after the integration:
the worker, the tables and descriptors rs.c derived, the LES frames read by
the backend's reader from the same tables folder (rewritten here, the same
bytes) with the first one set synchronously and the swap uploaded on the copy
stream, RS_populate's draws made on the device, then every advance, debris
RCS refresh and pulse with the descriptor rs.c gave its kernels.  Checked
against the recording:

  * the LES descriptor bit for bit, every LES frame read (hash), the state
    after populate (hash);
  * the final state -- pos, vel, ori, tum, aux, rcs, sig, rnd -- bit for bit
    (ref_session_dbu_rscl, recorded with the device running the reference's
    own rs.cl: bit for bit but for the rain backscatter and the signals
    formed from it, within 4e-7);
  * every pulse read back within 2e-5 of the per-gate sum of |term| against
    both the pulse rs.c read back and the exact sum of its terms, and the
    merged, scaled pulse with the gain of RS_merge_pulse_tmp.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import refbind
from simradar_gb300 import build as B

from test_ref_session import ALL_SESSIONS, FIELDS, SESSIONS, SESSIONS_RSCL, load, write_session_tables

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def host_loop(tmp_path_factory, backend):
    exe = str(tmp_path_factory.mktemp("host") / "host_loop")
    libdir = os.path.dirname(B.LIB)
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-o", exe, os.path.join(HERE, "c", "host_loop.c"), "-L", libdir, "-lsimradar_gb300",
                    "-Wl,-rpath," + libdir, "-lm"], check=True)
    return exe


@pytest.fixture(scope="module")
def tables(tmp_path_factory):
    home = str(tmp_path_factory.mktemp("refhome"))
    return write_session_tables(home, load(SESSIONS[0]))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name", ALL_SESSIONS)
def test_c_host_replays_rs_c_session(name, host_loop, tables, tmp_path):
    R = load(name)
    sess = str(tmp_path / "session.bin")
    out = str(tmp_path / "out.bin")
    refbind.write_session(sess, {k: v for k, v in R.items() if not k.startswith("meta_")})
    p = subprocess.run([host_loop, sess, tables, out], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    O = refbind.read_session(out)
    assert int(O["launches"]) > 0
    # inputs
    assert np.array_equal(bits(O["les_desc"]), bits(R["les_desc"]))
    assert np.array_equal(O["les_hash"], R["les_hash"])
    assert np.array_equal(O["upload_hash"], R["init_hash"])
    # pulses
    ab = R["pulse_abs"].astype(np.float64)
    raw = O["pulse_raw"].astype(np.float64)
    for ref in (R["pulse_raw"].astype(np.float64), R["pulse_direct"]):
        err = np.abs(raw - ref)
        worst = np.unravel_index(np.argmax(err - 2e-5 * ab), err.shape)
        assert np.all(err <= 2e-5 * ab + 1e-30), (worst, raw[worst], ref[worst], ab[worst])
    gain = float(np.abs(R["pulse_merged"]).max() / max(np.abs(R["pulse_raw"]).max(), 1e-30))
    err = np.abs(O["pulse_merged"].astype(np.float64) - R["pulse_merged"].astype(np.float64))
    assert np.all(err <= 2e-5 * ab * gain * 1.0001 + 1e-30)
    # the final state, bit for bit; against a session run on the reference's
    # own rs.cl, the rain backscatter (|xy|^2 / |xyz|^2 here, cos(atan2)^2
    # there) and the signals formed from it within 4e-7
    near = ("rcs", "sig") if name in SESSIONS_RSCL else ()
    bad = []
    for i, f in enumerate(FIELDS):
        if f in near:
            x = R["final_%s_every8" % f].astype(np.float64)
            y = O["final_%s_every8" % f].astype(np.float64)
            if not np.all(np.abs(x - y) <= 4e-7 * np.abs(x)):
                bad.append("%s beyond 4e-7" % f)
            continue
        if int(O["final_hash"][i]) != int(R["final_hash"][i]):
            g, r = O["final_%s_every8" % f].view(np.uint32), R["final_%s_every8" % f].view(np.uint32)
            rows = np.nonzero((g != r).any(axis=1))[0]
            bad.append("%s (sampled rows differing: %d, first %s)" % (f, rows.size, rows[:4]))
    assert not bad, "final state differs from rs.c's: " + "; ".join(bad)
