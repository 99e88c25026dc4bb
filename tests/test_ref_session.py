"""Sessions of the reference host (rs.c) recorded in tests/golden/ref_session_*.npz.

tests/golden/make_ref_session.py ran the unmodified rs.c (with les.c, adm.c,
rcs.c, obj.c, pos.c) over this project's OpenCL shim on the CPU oracle and
recorded what rs.c derived and sent to the device and what it read back.
These CPU tests check against those recordings:

  * that this build's restatements of rs.c's host derivations give the same
    bits: the range and angular weights, the drop RCS table, the ADM / RCS /
    LES descriptors, the per-pulse beam vectors, and RS_populate's initial
    state (rsc_populate_host, the backend's own);
  * that the oracle's Python orchestration (oracle/oracle.py, the checker of
    every GPU parity test) replays rs.c's event list to the same pulses and
    the same final state, bit for bit (with the debris flux field tables rs.c
    derived from each LES frame in the session with that concept);
  * for ref_session_dbu_rscl, recorded with the device running the
    reference's own rs.cl, that the replay gives the same final state bit
    for bit but for the rain backscatter and the signals formed from it;
  * where the reference tree is present, that the recording is reproduced.
"""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refbind
from simradar_gb300 import rsc, synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
SESSIONS = ["ref_session_dbu", "ref_session_bg", "ref_session_dff", "ref_session_vpr"]
# recorded with the device running the reference's own rs.cl kernels
SESSIONS_RSCL = ["ref_session_dbu_rscl"]
ALL_SESSIONS = SESSIONS + SESSIONS_RSCL
FIELDS = ["pos", "vel", "ori", "tum", "aux", "rcs", "sig", "rnd"]
EV_LES, EV_ADVANCE, EV_DEBRIS_RCS, EV_PULSE, EV_UPLOAD = 1, 2, 3, 4, 5


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


class SessionScene:
    """The tables of a recorded session in the form oracle.py takes."""

    def __init__(self, R):
        self.range_count = int(R["range_count"])
        self.range_start = np.float32(R["range_start"])
        self.range_delta = np.float32(R["range_delta"])
        self.range_w, self.range_desc = R["range_weight"], R["range_weight_desc"]
        self.ang_w, self.ang_desc = R["angular_weight"], R["angular_weight_desc"]
        self.ell, self.ell_desc = R["rcs_ellipsoid"].reshape(-1, 4), R["rcs_ellipsoid_desc"]
        self.les_desc = R["les_desc"]
        self.adm = [(R["adm_cd_%d" % a], R["adm_cm_%d" % a], R["adm_desc_%d" % a]) for a in range(int(R["adm_count"]))]
        self.rcs_tables = [(R["rcs_real_%d" % r], R["rcs_imag_%d" % r], R["rcs_desc_%d" % r])
                           for r in range(int(R["rcs_count"]))]
        self.counts = [int(c) for c in R["counts"][:int(R["num_types"])]]
        self.dff, self.dff_desc = None, np.zeros(16, np.float32)

    def use_dff(self, R, index):
        """The debris flux field table (and descriptor) an advance read."""
        if index >= 0:
            self.dff, self.dff_desc = R["dff_tables"][index], R["dff_descs"][index]


def populate_args(R):
    dom = R["domain"]
    return rsc.PopulateArgs.make(int(R["random_seed"]), int(R["sim_concept"]), dom[:3], dom[3:],
                                 [int(c) for c in R["counts"][:int(R["num_types"])]], R["dsd_r"], R["dsd_cdf"])


def write_session_tables(home, R):
    synth.write_tables_folder(os.path.join(home, "Documents", "tables"), seed=int(R["meta_tables_seed"]),
                              volumes_per_file=int(R["meta_tables_volumes_per_file"]),
                              adm_dims=tuple(int(v) for v in R["meta_tables_adm_dims"]),
                              rcs_dims=tuple(int(v) for v in R["meta_tables_rcs_dims"]))
    return os.path.join(home, "Documents", "tables", "les", "suctvort")


@pytest.fixture(scope="module")
def tables_home(tmp_path_factory):
    """The sessions' tables folder, written again (the same bytes)."""
    home = str(tmp_path_factory.mktemp("refhome"))
    les_dir = write_session_tables(home, load(SESSIONS[0]))
    return home, les_dir


@pytest.mark.parametrize("name", ALL_SESSIONS)
def test_recording_is_consistent(name):
    R = load(name)
    assert int(R["failed"]) == 0 and int(R["uploads"]) == 1
    kinds = R["ev_kind"]
    pulses = [i for i in np.nonzero(kinds == EV_PULSE)[0] if R["ev_int"][i, 0] >= 0]
    assert len(pulses) == int(R["meta_pulses"]) == R["pulse_raw"].shape[0]
    n_adv = int(np.sum(kinds == EV_ADVANCE))
    assert n_adv == 1 + int(R["meta_warmup"]) + int(R["meta_pulses"])   # RS_populate's warm step
    # every pulse rs.c read back is the sum of its oracle terms within FP32 rounding
    err = np.abs(R["pulse_raw"].astype(np.float64) - R["pulse_direct"])
    assert np.all(err <= 2e-5 * R["pulse_abs"] + 1e-30)
    gain = np.float32(np.float32(np.float32(10.0) ** np.float32(np.float32(0.1) * R["antenna_gain_dbi"])) *
                      np.sqrt(R["tx_power_watt"], dtype=np.float32) / np.float32(4.0 * math.pi) *
                      np.float32(1.0e6))
    np.testing.assert_allclose(R["pulse_merged"], R["pulse_raw"] * gain, rtol=2e-6, atol=0)


@pytest.mark.parametrize("name", ALL_SESSIONS)
def test_populate_is_rs_populate(name):
    """rsc_populate_host (the backend's RS_populate) against the state rs.c
    uploaded, bit for bit."""
    R = load(name)
    arr, pop = rsc.populate_host(populate_args(R), int(R["num_scats"]))
    for i, f in enumerate(FIELDS):
        assert refbind.fnv1a(arr[f]) == int(R["init_hash"][i]), f
    assert np.array_equal(pop.astype(np.uint64), R["dsd_pop"])


@pytest.mark.parametrize("name", ALL_SESSIONS)
def test_host_tables_match_synth(name):
    """The tables and descriptors the tests and the bench build with synth
    against the ones rs.c made for the same radar."""
    R = load(name)
    k = np.float32(4.0 * math.pi / float(R["lambda"]))
    dr = np.float32(np.float32(0.5) * np.float32(3.0e8) * np.float32(0.2e-6))
    w, d = synth.range_weight_triangle(dr, user=k)
    assert np.array_equal(bits(w), bits(R["range_weight"])) and np.array_equal(bits(d), bits(R["range_weight_desc"]))
    w, d = synth.angular_weight_standard(1.0)
    assert np.array_equal(bits(d), bits(R["angular_weight_desc"]))
    np.testing.assert_allclose(w, R["angular_weight"], rtol=0, atol=4e-7)
    # the drop RCS table (FP64 host table rounded once) with the session's DSD
    sd = R["ev_desc"][np.nonzero(R["ev_kind"] == EV_PULSE)[0][0]]
    diam = 2.0 * R["dsd_r"].astype(np.float64)
    _, pdf, cdf, _ = synth.marshall_palmer(diam.astype(np.float32))
    assert np.array_equal(bits(cdf), bits(R["dsd_cdf"]))
    ell, ed = synth.ellipsoid_rcs_table(sd[4], sd[6], int(R["sim_concept"]), R["dsd_r"], pdf)
    assert np.array_equal(bits(ed), bits(R["rcs_ellipsoid_desc"]))
    np.testing.assert_allclose(ell, R["rcs_ellipsoid"].reshape(-1, 4), rtol=2e-7, atol=0)
    # LES descriptor of the 176 x 176 x 80 suctvort grid
    assert np.array_equal(bits(synth.LESConfig().desc()), bits(R["les_desc"]))
    # ADM / RCS descriptors for the tables' dimensions and each object
    objs = [int(o) for o, _ in R["meta_debris"]]
    nb, na = (int(v) for v in R["meta_tables_adm_dims"])
    for a, obj in enumerate(objs):
        _, _, ad = synth.adm_table(obj, seed=1, nb=nb, na=na)
        assert np.array_equal(bits(ad), bits(R["adm_desc_%d" % a])), (obj, ad, R["adm_desc_%d" % a])
    na_r, nb_r = (int(v) for v in R["meta_tables_rcs_dims"])
    for r in range(len(objs)):
        _, _, rd = synth.rcs_table(seed=1, na=na_r, nb=nb_r)
        assert np.array_equal(bits(rd), bits(R["rcs_desc_%d" % r]))


@pytest.mark.parametrize("name", ALL_SESSIONS)
def test_beam_positions_match(name):
    """The beam unit vector of every pulse descriptor against synth's
    RS_set_beam_pos of the scan's positions.  Loop pulse k sees position k:
    RS_populate advances the beam to position 0 before its warm pulse, and
    the loop advances it after each pulse.  (With no warm-up advance between
    them, rs.c forms no new pulse for loop pulse 0 -- the signal needs no
    update -- and reads back RS_populate's.)  Bit for bit, except with the
    beam at 90 degrees elevation: there cos(el) is 4e-8, and the C
    library's cosf / sinf and numpy's float32 ones give the horizontal
    components within 2 ulps of each other (the GPU replays take rs.c's own
    descriptors)."""
    R = load(name)
    scan = str(R["meta_scan"])
    mode, rest = scan.split(":", 1)
    a, b = rest.split(",", 1)
    lo, hi, step = (float(v) for v in b.split(":"))
    pos = synth.ppi_positions(float(a), lo, hi, step) if mode == "P" else synth.rhi_positions(float(a), lo, hi, step)
    for i in np.nonzero(R["ev_kind"] == EV_PULSE)[0]:
        k = int(R["ev_int"][i, 0])
        az, el = pos[max(k, 0) % len(pos)]
        want = np.array(synth.beam_unit(az, el), np.float32)
        got = R["ev_desc"][i, :3]
        if el == 90.0:
            ulps = np.abs(bits(got).astype(np.int64) - bits(want).astype(np.int64))
            assert np.all(ulps <= 2) and bits(got)[2] == bits(want)[2], (k, got, want)
        else:
            assert np.array_equal(bits(got), bits(want)), (k, got, want)


def replay_oracle(R, les_dir):
    """Replay rs.c's event list with oracle.py; returns the pulses read back
    and the final state."""
    S = SessionScene(R)
    state, _ = rsc.populate_host(populate_args(R), int(R["num_scats"]))
    st = None
    vols = {}
    pulses = np.zeros_like(R["pulse_raw"])
    with rsc.LESSource(les_dir, "suctvort") as src:
        for kind, ints, desc in zip(R["ev_kind"], R["ev_int"], R["ev_desc"]):
            if kind == EV_UPLOAD:
                st = O.OracleState(state)
            elif kind == EV_LES:
                uvwt, cpxx, _ = src.read(int(ints[1]))
                vols[int(ints[0])] = synth.LESVolume(uvwt, cpxx)
            elif kind == EV_ADVANCE:
                S.use_dff(R, int(ints[3]))
                O.advance_time(st, S, S.counts, vols[int(ints[0])], desc)
            elif kind == EV_DEBRIS_RCS:
                O.db_rcs(st, S, S.counts, desc)
            elif kind == EV_PULSE:
                p = O.make_pulse(st, S, desc)
                if ints[0] >= 0:
                    pulses[int(ints[0])] = p
    return pulses, st


@pytest.mark.parametrize("name", SESSIONS)
def test_oracle_replays_rs_c(name, tables_home):
    R = load(name)
    _, les_dir = tables_home
    pulses, st = replay_oracle(R, les_dir)
    assert np.array_equal(bits(pulses), bits(R["pulse_raw"]))
    for i, f in enumerate(FIELDS):
        assert refbind.fnv1a(st.s[f]) == int(R["final_hash"][i]), f
        assert np.array_equal(st.s[f][::8].view(np.uint32), R["final_%s_every8" % f].view(np.uint32)), f


def assert_state_near_rs_cl(st_s, R):
    """The final state against a session run on rs.cl: bit for bit but for
    the rain backscatter (the oracle's cos^2 of the elevation is
    |xy|^2 / |xyz|^2, rs.cl's cos(atan2(z, |xy|))^2) and the signals formed
    from it, which agree within 4e-7 relative."""
    for i, f in enumerate(FIELDS):
        if f in ("rcs", "sig"):
            x = R["final_%s_every8" % f].astype(np.float64)
            y = st_s[f][::8].astype(np.float64)
            assert np.all(np.abs(x - y) <= 4e-7 * np.abs(x)), f
        else:
            assert refbind.fnv1a(st_s[f]) == int(R["final_hash"][i]), f


def assert_pulses_near(got, R):
    """Pulses within 2e-5 of the per-gate sum of |term| of the recording."""
    ab = R["pulse_abs"].astype(np.float64)
    err = np.abs(got.astype(np.float64) - R["pulse_raw"].astype(np.float64))
    assert np.all(err <= 2e-5 * ab + 1e-30), float((err / (ab + 1e-30)).max())


@pytest.mark.parametrize("name", SESSIONS_RSCL)
def test_oracle_replays_rs_cl_session(name, tables_home):
    """rs.c's session run with the reference's own rs.cl kernels, replayed by
    the oracle's Python orchestration: the same final positions, velocities,
    orientations, tumbles, aux and seeds, bit for bit."""
    R = load(name)
    assert str(R["meta_kernels"]) == "rscl"
    _, les_dir = tables_home
    pulses, st = replay_oracle(R, les_dir)
    assert_pulses_near(pulses, R)
    assert_state_near_rs_cl(st.s, R)


@pytest.mark.skipif(not refbind.available(), reason="the reference tree is not present")
@pytest.mark.parametrize("name", ALL_SESSIONS)
def test_recording_reproduces(name, tables_home, tmp_path):
    """rs.c run again gives the recorded session (the oracle sums of |term|
    are per-thread double sums: compared to 1e-12)."""
    import sys
    sys.path.insert(0, GOLDEN)
    from make_ref_session import SESSIONS as ARGS
    home, _ = tables_home
    R = load(name)
    N = refbind.run_session(str(tmp_path / "s.bin"), home, **ARGS[name])
    for k, v in N.items():
        want = R[k]
        if k in ("pulse_abs", "pulse_direct"):
            np.testing.assert_allclose(v, want, rtol=1e-12, atol=0)
        else:
            assert np.array_equal(np.asarray(v), want), k
