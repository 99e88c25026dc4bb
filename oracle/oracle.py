"""ctypes binding of the CPU oracle (oracle/build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the simradar_gb300 package.  The oracle
is a plain-C restatement of rs.cl (see rsoracle.c); this module marshals
numpy arrays into it and strings the kernels together the way rs.c's
RS_advance_time (rs.c:5325-5388) and RS_make_pulse (rs.c:5563-5573) do.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")

_f = ctypes.POINTER(ctypes.c_float)
_d = ctypes.POINTER(ctypes.c_double)
_u = ctypes.POINTER(ctypes.c_uint32)
S_, U32, I_ = ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int


class Image(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        img = Image
        L.or_el_atts.argtypes = [_f, _f, _f, _u, img, _f, _f, _f, _f, S_, S_]
        L.or_bg_atts.argtypes = [_f, _f, _f, _u, img, _f, _f, _f, _f, S_, S_]
        L.or_fp_atts.argtypes = [_f, _f, _f, img, img, _f, _f, S_, S_]
        L.or_db_atts.argtypes = [_f, _f, _f, _f, _f, _u, img, _f, img, img, _f, img, img, _f, _f, _f, _f, S_, S_]
        L.or_db_rcs.argtypes = [_f, _f, _f, img, img, _f, _f, S_, S_]
        L.or_scat_sig_aux.argtypes = [_f, _f, _f, _f, _f, _f, _f, S_]
        L.or_pop.argtypes = [_f, _f, _f, _f, S_]
        L.or_make_pulse.argtypes = [_f, _f, _f, _f, _f, S_, S_, _f, _f, _f, _f, ctypes.c_float, ctypes.c_float, U32,
                                    _f, U32, U32, U32, I_]
        L.or_make_pulse.restype = I_
        L.or_make_pulse_f64.argtypes = [_d, _d, _f, _f, S_, _f, _f, _f, _f, ctypes.c_double, ctypes.c_double, U32, _f]
        L.or_make_pulse_direct.argtypes = [_d, _d, _f, _f, S_, _f, _f, _f, _f, ctypes.c_float, ctypes.c_float, U32,
                                           _f]
        L.or_eval_math.argtypes = [I_, _f, _f, _f, S_]
        L.or_num_threads.restype = I_
        _lib = L
    return _lib


def fp(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_f)


def up(a):
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_u)


def image(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim == 4:
        nz, ny, nx = a.shape[:3]
    else:
        nz = 1
        ny, nx = a.shape[:2]
    im = Image(a.ctypes.data, nx, ny, nz)
    im._keep = a
    return im


def num_threads():
    return lib().or_num_threads()


def eval_math(fn, a, b=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b if b is not None else a, dtype=np.float32)
    out = np.empty_like(a)
    lib().or_eval_math(int(fn), fp(a), fp(b), fp(out), a.size)
    return out


class OracleState:
    """Host copy of the attribute arrays, advanced by the oracle kernels."""

    def __init__(self, state):
        self.s = {k: np.ascontiguousarray(v).copy() for k, v in state.items()}

    def __getitem__(self, k):
        return self.s[k]


def advance_time(st, S, pop_counts, les_vol, sim_desc, L=None):
    """RS_advance_time's launches (rs.c:5325-5374) on the oracle.  Type 0 uses
    el_atts / fp_atts / bg_atts by concept; debris type k uses ADM / RCS table
    k - 1; the DFF slot is unused unless concept C is set.  L: another library
    with the oracle's entry points (refbind.rscl(), the reference's rs.cl)."""
    L = L or lib()
    s = st.s
    sd = np.ascontiguousarray(sim_desc, dtype=np.float32)
    concept = int(np.frombuffer(sd[5:6].tobytes(), dtype=np.uint32)[0])
    uv = image(les_vol.uvwt)
    cp = image(les_vol.cpxx)
    wd = np.ascontiguousarray(S.les_desc, dtype=np.float32)
    origin = 0
    n0 = pop_counts[0]
    if n0:
        if concept & (1 << 1):
            L.or_el_atts(fp(s["pos"]), fp(s["vel"]), fp(s["rcs"]), up(s["rnd"]), uv, fp(wd), fp(S.ell), fp(S.ell_desc),
                         fp(sd), origin, n0)
        elif concept & (1 << 5):
            L.or_fp_atts(fp(s["pos"]), fp(s["vel"]), fp(s["rcs"]), uv, cp, fp(wd), fp(sd), origin, n0)
        else:
            L.or_bg_atts(fp(s["pos"]), fp(s["vel"]), fp(s["rcs"]), up(s["rnd"]), uv, fp(wd), fp(S.ell), fp(S.ell_desc),
                         fp(sd), origin, n0)
    origin += n0
    dff = getattr(S, "dff", None)
    dff_desc = getattr(S, "dff_desc", np.zeros(16, np.float32))
    dff_arr = dff if dff is not None else np.zeros(1, np.float32)
    for t in range(1, len(pop_counts)):
        n = pop_counts[t]
        if n:
            cd, cm, ad = S.adm[t - 1]
            re, im, rd = S.rcs_tables[t - 1]
            L.or_db_atts(fp(s["pos"]), fp(s["ori"]), fp(s["vel"]), fp(s["tum"]), fp(s["rcs"]), up(s["rnd"]), uv, fp(wd),
                         image(cd), image(cm), fp(ad), image(re), image(im), fp(rd), fp(dff_arr), fp(dff_desc), fp(sd),
                         origin, n)
        origin += n


def db_rcs(st, S, pop_counts, sim_desc, L=None):
    L = L or lib()
    s = st.s
    sd = np.ascontiguousarray(sim_desc, dtype=np.float32)
    origin = pop_counts[0]
    for t in range(1, len(pop_counts)):
        n = pop_counts[t]
        if n:
            re, im, rd = S.rcs_tables[t - 1]
            L.or_db_rcs(fp(s["pos"]), fp(s["ori"]), fp(s["rcs"]), image(re), image(im), fp(rd), fp(sd), origin, n)
        origin += n


def make_pulse(st, S, sim_desc, group_size_multiple=64, max_work_group_size=1024, local_mem=49152, name_swap=1,
               L=None):
    """scat_sig_aux + pass 1 + pass 2 as RS_make_pulse enqueues them; returns the
    unscaled pulse (range_count, 4).  Updates sig / aux in the state."""
    L = L or lib()
    s = st.s
    N = s["pos"].shape[0]
    pulse = np.zeros((S.range_count, 4), dtype=np.float32)
    sd = np.ascontiguousarray(sim_desc, dtype=np.float32)
    rc = L.or_make_pulse(fp(pulse), fp(s["sig"]), fp(s["aux"]), fp(s["pos"]), fp(s["rcs"]), N, N, fp(S.ang_w),
                         fp(S.ang_desc), fp(S.range_w), fp(S.range_desc), float(S.range_start), float(S.range_delta),
                         S.range_count, fp(sd), group_size_multiple, max_work_group_size, local_mem, name_swap)
    if rc != 0:
        raise RuntimeError("or_make_pulse failed: %d" % rc)
    return pulse


def make_pulse_direct(st, S, sim_desc, return_abs=False):
    """The reference's FP32 contributions summed exactly (double), every gate."""
    L = lib()
    s = st.s
    N = s["pos"].shape[0]
    out = np.zeros((S.range_count, 4), dtype=np.float64)
    ab = np.zeros((S.range_count, 4), dtype=np.float64)
    sd = np.ascontiguousarray(sim_desc, dtype=np.float32)
    L.or_make_pulse_direct(out.ctypes.data_as(_d), ab.ctypes.data_as(_d), fp(s["pos"]), fp(s["rcs"]), N, fp(S.ang_w),
                           fp(S.ang_desc), fp(S.range_w), fp(S.range_desc), float(S.range_start),
                           float(S.range_delta), S.range_count, fp(sd))
    return (out, ab) if return_abs else out


def reference_plan_valid(n, group_size_multiple=64):
    """make_pulse_pass_1's tree needs a power-of-two work-group size
    (count / 2 when count < 2 * 64) and RS_make_pulse_params needs count >= 2."""
    if n < 2:
        return False
    wi = group_size_multiple if n > 2 * group_size_multiple else n // 2
    return wi & (wi - 1) == 0


def make_pulse_f64(st, S, sim_desc, return_abs=False):
    """FP64 pulse of the current FP32 state (gate origins in FP64)."""
    L = lib()
    s = st.s
    N = s["pos"].shape[0]
    out = np.zeros((S.range_count, 4), dtype=np.float64)
    ab = np.zeros((S.range_count, 4), dtype=np.float64)
    sd = np.ascontiguousarray(sim_desc, dtype=np.float32)
    L.or_make_pulse_f64(out.ctypes.data_as(_d), ab.ctypes.data_as(_d), fp(s["pos"]), fp(s["rcs"]), N, fp(S.ang_w),
                        fp(S.ang_desc), fp(S.range_w), fp(S.range_desc), float(S.range_start), float(S.range_delta),
                        S.range_count, fp(sd))
    return (out, ab) if return_abs else out
