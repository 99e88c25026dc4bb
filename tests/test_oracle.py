"""The oracle against the reference's own known-answer material.

* test_make_pulse.c's CPU-vs-device check (test_make_pulse.c:553-653): the
  `pop` fixture (rs.cl:1444-1453), a {0, 1, 0} range weight over [-25, 25] m,
  a {0, .7, 1, .7, 0} angular weight at 10 degree steps, 9 gates from 1 m every
  0.25 m; the device path (scat_sig_aux + pass 1 + pass 2 with 64 x 64 work
  items) must match a direct per-gate loop within the reference's 1e-3.
* RS_make_pulse_params (rs.c:1284-1386): the launch plans for the sizes the
  reference runs and the pass-2 kernel each selects.
* rand (rs.cl:35-44): the 31-bit masked 16807 multiply, lane by lane.
* the three pass-2 bodies agree with each other on the same pass-1 output.
"""
import math

import numpy as np
import pytest

F = np.float32


def read_table(table, last, index):
    """rs.c:358-374, vectorised in float32."""
    index = index.astype(np.float32)
    last = int(last)
    fl = np.floor(index)
    alpha = (index - fl).astype(np.float32)
    i = np.clip(fl, 0, last).astype(np.int64)
    i1 = np.clip(i + 1, 0, last)
    t = np.asarray(table, dtype=np.float32)
    out = (t[i] + alpha * (t[i1] - t[i])).astype(np.float32)
    out = np.where(index <= 0.0, t[0], out)
    out = np.where(fl >= last, t[int(last)], out)
    return out.astype(np.float32)


def kat_setup(num_elem=1079196):
    groups = 64
    nice = int(math.ceil(num_elem / groups / 2)) * groups * 2
    sd = np.zeros(16, dtype=np.float32)
    sd[0], sd[1], sd[2] = 0.0, 1.0, 0.0
    sd[4] = F(4.0 * math.pi / float(F(0.1)))
    rw = np.array([0.0, 1.0, 0.0], dtype=np.float32)
    xs = F(F(1.0) / F(25.0))
    rwd = np.array([xs, F(F(25.0) * xs), F(2.0), 0.0], dtype=np.float32)
    aw = np.array([0.0, 0.7, 1.0, 0.7, 0.0], dtype=np.float32)

    def deg2rad(d):
        return F(F(d) * F(0.01745329251994))
    awd = np.array([F(F(1.0) / deg2rad(10.0)), F(F(F(-deg2rad(-20.0)) * F(1.0)) / deg2rad(10.0)), F(4.0), 0.0],
                   dtype=np.float32)
    return nice, sd, rw, rwd, aw, awd


def test_make_pulse_known_answer(oracle_lib):
    O = oracle_lib
    n, sd, rw, rwd, aw, awd = kat_setup()
    G, r0, dr = 9, F(1.0), F(0.25)
    rcs = np.zeros((n, 4), np.float32)
    aux = np.zeros((n, 4), np.float32)
    pos = np.zeros((n, 4), np.float32)
    L = O.lib()
    L.or_pop(O.fp(rcs), O.fp(aux), O.fp(pos), O.fp(sd), n)
    # the fixture itself (rs.cl:1444-1453)
    k = np.arange(n, dtype=np.uint32)
    assert np.array_equal(pos[:, 0], (k % 9).astype(np.float32) - F(4.0))
    assert np.array_equal(pos[:, 1], (k.astype(np.float32) / F(90000.0) + F(1.0)).astype(np.float32))
    assert np.all(rcs == np.array([1.0, 0.5, 1.0, 0.5], np.float32))
    # device path with test_make_pulse's parameters and direct kernel names
    sig = np.zeros_like(rcs)
    pulse = np.zeros((G, 4), np.float32)
    rc = L.or_make_pulse(O.fp(pulse), O.fp(sig), O.fp(aux), O.fp(pos), O.fp(rcs), n, n, O.fp(aw), O.fp(awd),
                         O.fp(rw), O.fp(rwd), float(r0), float(dr), G, O.fp(sd), 64, 64, 49152, 0)
    assert rc == 0
    cpu = kat_cpu_pulse(pos, rcs, aux[:, 0], sd, rw, rwd, aw, awd, G, r0, dr)
    assert_kat(pulse, cpu)


def kat_cpu_pulse(pos, rcs, r_a, sd, rw, rwd, aw, awd, G, r0, dr):
    """The CPU loop of test_make_pulse.c:553-583 (float32, sequential sums)."""
    ang = np.arccos(((sd[0] * pos[:, 0] + sd[1] * pos[:, 1] + sd[2] * pos[:, 2]) / r_a).astype(np.float32))
    w_a = read_table(aw, awd[2], (ang * awd[0] + awd[1]).astype(np.float32))
    atten = np.power(r_a, F(-2.0)).astype(np.float32)
    ph = (r_a * sd[4]).astype(np.float32)
    c, s = np.cos(ph).astype(np.float32), np.sin(ph).astype(np.float32)
    sig_cpu = np.stack([rcs[:, 0] * c - rcs[:, 1] * (-s), rcs[:, 1] * c + rcs[:, 0] * (-s),
                        rcs[:, 2] * c - rcs[:, 3] * (-s), rcs[:, 3] * c + rcs[:, 2] * (-s)], axis=1) * atten[:, None]
    cpu = np.zeros((G, 4), np.float32)
    for ir in range(G):
        r = F(F(ir) * dr + r0)
        w_r = read_table(rw, rwd[2], ((r_a - r) * rwd[0] + rwd[1]).astype(np.float32))
        contrib = (sig_cpu * (w_r * w_a)[:, None]).astype(np.float32)
        cpu[ir] = np.cumsum(contrib, axis=0, dtype=np.float32)[-1]
    return cpu


def assert_kat(pulse, cpu):
    """The reference's green / red rule (test_make_pulse.c:640-646) on gate
    lane 0, and a tighter check of all four lanes."""
    delta = (cpu[:, 0] - pulse[:, 0]) / np.maximum(1.0, pulse[:, 0])
    square = cpu[:, 0] ** 2 + cpu[:, 1] ** 2
    assert np.all(delta / np.maximum(1.0, square) < 1e-3)
    assert np.allclose(pulse, cpu, rtol=2e-3, atol=1e-3 * np.abs(cpu).max())


@pytest.mark.parametrize("count,gsm,maxg,G,method,groups,local", [
    (1998848 + 3072, 64, 1024, 40, "range", 1024, 64),     # README scale, NVIDIA-like device
    (131072, 64, 1024, 40, "range", 1024, 64),
    (1079296, 64, 64, 9, "local", 64, 64),                  # test_make_pulse
    (128, 64, 1024, 40, "range", 1, 64),
    (128, 64, 1024, 4, "universal", 1, 64),
])
def test_make_pulse_params(oracle_lib, count, gsm, maxg, G, method, groups, local):
    import ctypes
    O = oracle_lib

    class P(ctypes.Structure):
        _fields_ = [("num_scats", ctypes.c_uint32), ("user_max_groups", ctypes.c_uint32),
                    ("user_max_work_items", ctypes.c_uint32), ("pass_2_method", ctypes.c_uint32),
                    ("range_count", ctypes.c_uint32), ("range_start", ctypes.c_float), ("range_delta", ctypes.c_float),
                    ("entry_counts", ctypes.c_uint32 * 2), ("group_counts", ctypes.c_uint32 * 2),
                    ("global_", ctypes.c_size_t * 2), ("local", ctypes.c_size_t * 2),
                    ("local_mem_size", ctypes.c_size_t * 2)]
    L = O.lib()
    L.or_make_pulse_params.argtypes = [ctypes.POINTER(P), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_uint32]
    L.or_make_pulse_params.restype = ctypes.c_int
    p = P()
    assert L.or_make_pulse_params(ctypes.byref(p), count, gsm, maxg, 49152, 1000.0, 15.0, G) == 0
    names = {0: "universal", 1: "range", 2: "local"}
    assert names[p.pass_2_method] == method
    assert p.group_counts[0] == groups
    assert p.local[0] == local
    assert p.entry_counts[1] == groups * G


def test_rand_lcg(oracle_lib):
    """rand() of rs.cl:35-44 is observable through a bg_atts respawn: one
    scatterer outside the box gets pos = r * size + origin with
    r = ((seed * 16807) & 0x7fffffff) / 2^31 per lane."""
    O = oracle_lib
    seeds = np.array([[1, 2147483646, 123456789, 0x7fffffff]], dtype=np.uint32)
    pos = np.array([[-10.0, 0.0, 0.0, 1e-3]], np.float32)
    vel = np.zeros((1, 4), np.float32)
    rcs = np.zeros((1, 4), np.float32)
    sd = np.zeros(16, np.float32)
    sd[8:11] = 0.0
    sd[12:15] = 1.0
    sd[11] = 1e-3
    wd = np.zeros(16, np.float32)
    uv = np.zeros((1, 1, 1, 4), np.float32)
    ell = np.zeros((1, 4), np.float32)
    ed = np.zeros(4, np.float32)
    L = O.lib()
    L.or_bg_atts(O.fp(pos), O.fp(vel), O.fp(rcs), O.up(seeds), O.image(uv), O.fp(wd), O.fp(ell), O.fp(ed), O.fp(sd), 0, 1)
    s0 = np.array([1, 2147483646, 123456789, 0x7fffffff], dtype=np.uint64)
    s1 = (s0 * 16807) % (1 << 32) & 0x7fffffff
    assert seeds[0].tolist() == s1.tolist()
    r = (s1.astype(np.float32) * F(1.0 / 2147483648.0)).astype(np.float32)
    assert np.array_equal(pos[0, :3], (r[:3] * F(1.0) + F(0.0)).astype(np.float32))


def test_pass2_bodies_agree(oracle_lib):
    """The three pass-2 bodies sum the same pass-1 partials (FP32 tolerance)."""
    O = oracle_lib
    from simradar_gb300 import synth
    S = synth.make_scene(num_rain=200000, les_count=1)
    st = O.OracleState(S.state)
    sd = synth.pulse_sim_desc(S, 10)
    outs = []
    # max work group sizes that select range (1024), local (64 groups with G=4 -> 2G <= 64) and universal
    for maxg in (1024, 256):
        for swap in (0, 1):
            outs.append(O.make_pulse(st, S, sd, max_work_group_size=maxg, name_swap=swap))
    ref, ab = O.make_pulse_f64(st, S, sd, return_abs=True)
    for p in outs:
        assert np.all(np.abs(p - ref) <= 5e-3 * ab + 1e-30)
    for p in outs[1:]:
        assert np.all(np.abs(p - outs[0]) <= 5e-5 * ab + 1e-30)


def test_reference_order_matches_exact_sum(oracle_lib):
    """pass 1 + pass 2 in the reference's order equals the exact sum of its own
    FP32 contributions within the FP32 reordering bound, for the plan sizes
    the reference runs (power-of-two work groups)."""
    O = oracle_lib
    from simradar_gb300 import synth
    for n in (128, 4096, 131072):
        S = synth.make_scene(num_rain=n, les_count=1)
        st = O.OracleState(S.state)
        sd = synth.pulse_sim_desc(S, 7)
        p = O.make_pulse(st, S, sd)
        direct, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
        assert np.all(np.abs(p - direct) <= 2e-5 * ab + 1e-30), n


def test_reference_tree_quirk_below_128(oracle_lib):
    """With 62 scatterers the pass-1 work group is 31 wide and the reference's
    tree reduction (rs.cl:1224-1290) folds entries of the next gate's column
    into a gate: its pulse then differs from the exact sum of its own
    contributions, and the backend follows the exact sum."""
    O = oracle_lib
    from simradar_gb300 import synth
    assert not O.reference_plan_valid(62) and O.reference_plan_valid(64)
    S = synth.make_scene(num_rain=62, les_count=1)
    st = O.OracleState(S.state)
    # point the beam at the scatterers so the sums are not negligible
    p = S.state["pos"][:, :3].astype(np.float64).mean(axis=0)
    sd = S.sim_desc.copy()
    sd[0:3] = (p / np.linalg.norm(p)).astype(np.float32)
    ref = O.make_pulse(st, S, sd)
    direct, ab = O.make_pulse_direct(st, S, sd, return_abs=True)
    assert np.any(np.abs(ref - direct) > 1e-3 * ab + 1e-30)
    assert O.lib().or_make_pulse_params.restype is not None
