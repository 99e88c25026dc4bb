"""ctypes binding of the reference's own host code (oracle/_ref/libref.so) and
the reader of the session records oracle/_ref/refdrive writes.

TEST INFRASTRUCTURE ONLY: imported by tests/ and tests/golden/, never by the
simradar_gb300 package.

oracle/ref/Makefile compiles the reference's C modules unmodified from the
reference tree (les.c, pos.c, adm.c, rcs.c, obj.c, log.c and rs.c, the last
against this project's OpenCL shim over the CPU oracle), and its kernel
source rs.cl as C++ through oracle/ref/clc/opencl_c.hpp (`rscl()`).  They can
be built only where the reference tree is present; `available()` says
whether it is.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "libref.so")
DRIVE = os.path.join(REF_DIR, "refdrive")
REFERENCE = os.environ.get("SIMRADAR_REFERENCE", "/root/reference")

_f = ctypes.POINTER(ctypes.c_float)
_u = ctypes.POINTER(ctypes.c_uint32)


def available():
    """True when the reference tree is here (the build can run)."""
    return os.path.exists(os.path.join(REFERENCE, "rs.c"))


def build():
    if not available():
        raise RuntimeError("the reference tree is not present; oracle/_ref cannot be built")
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + REFERENCE], check=True,
                   stdout=subprocess.DEVNULL)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or not os.path.exists(DRIVE):
            build()
        L = ctypes.CDLL(LIB)
        L.ref_les_frame.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, _f, _f, _u, _f]
        L.ref_pos_angles.argtypes = [ctypes.c_char_p, ctypes.c_int, _f, _f]
        L.ref_adm_table.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _u, _f, _f]
        L.ref_rcs_table.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _u, _f]
        L.ref_obj_table.argtypes = [ctypes.c_int, _f, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.ref_les_descriptor.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _f]
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(_f) if a is not None else None


def les_frame(parent, config, frame):
    """les.c's LES_get_frame of <parent>/tables/les/<config>: (uvwt, cpxx) as
    (nz, ny, nx, 4) float32, and the constants dict."""
    L = lib()
    dims = np.zeros(3, np.uint32)
    consts = np.zeros(10, np.float32)
    rc = L.ref_les_frame(parent.encode(), config.encode(), frame, None, None, dims.ctypes.data_as(_u), _fp(consts))
    if rc != 0:
        raise RuntimeError("LES_init_with_config_path / LES_get_frame failed (%d)" % rc)
    nx, ny, nz = (int(v) for v in dims)
    uvwt = np.zeros((nz, ny, nx, 4), np.float32)
    cpxx = np.zeros((nz, ny, nx, 4), np.float32)
    rc = L.ref_les_frame(parent.encode(), config.encode(), frame, _fp(uvwt), _fp(cpxx), dims.ctypes.data_as(_u),
                         _fp(consts))
    if rc != 0:
        raise RuntimeError("LES_get_frame failed (%d)" % rc)
    keys = ("tr", "tp", "ax", "ay", "az", "rx", "ry", "rz", "is_stretched", "frames")
    return uvwt, cpxx, dict(zip(keys, (float(v) for v in consts)))


def pos_angles(scan, count):
    """pos.c's POS_get_next_angles, `count` times: (az, el) float32 arrays."""
    az = np.zeros(count, np.float32)
    el = np.zeros(count, np.float32)
    rc = lib().ref_pos_angles(scan.encode(), count, _fp(az), _fp(el))
    if rc != 0:
        raise RuntimeError("POS_init_with_string failed")
    return az, el


def adm_table(path, name):
    """adm.c's ADM_get_table of <path>/adm/<name>.adm: (data (6, na, nb), phys)."""
    L = lib()
    dims = np.zeros(2, np.uint32)
    phys = np.zeros(9, np.float32)
    if L.ref_adm_table(path.encode(), name.encode(), dims.ctypes.data_as(_u), None, _fp(phys)) != 0:
        raise RuntimeError("ADM_get_table failed")
    nb, na = (int(v) for v in dims)
    data = np.zeros((6, na, nb), np.float32)
    L.ref_adm_table(path.encode(), name.encode(), dims.ctypes.data_as(_u), _fp(data), _fp(phys))
    return data, phys


def rcs_table(path, name):
    """rcs.c's RCS_get_table of <path>/rcs/<name>.rcs: data (6, nb, na)."""
    L = lib()
    dims = np.zeros(2, np.uint32)
    if L.ref_rcs_table(path.encode(), name.encode(), dims.ctypes.data_as(_u), None) != 0:
        raise RuntimeError("RCS_get_table failed")
    na, nb = (int(v) for v in dims)
    data = np.zeros((6, nb, na), np.float32)
    L.ref_rcs_table(path.encode(), name.encode(), dims.ctypes.data_as(_u), _fp(data))
    return data


def obj_table(obj_type):
    """obj.c's OBJ_get_table for a debris type (tables found from $HOME):
    (phys after ADM_dimension_set, adm table name, rcs table name)."""
    phys = np.zeros(9, np.float32)
    a = ctypes.create_string_buffer(1024)
    r = ctypes.create_string_buffer(1024)
    if lib().ref_obj_table(obj_type, _fp(phys), a, r, 1024) != 0:
        raise RuntimeError("OBJ_get_table failed")
    return phys, a.value.decode(), r.value.decode()


def les_descriptor(config):
    """rs.c's LES descriptor (RS_set_vel_data_to_config on frame 0) of the
    tables found from $HOME (set HOME before calling)."""
    desc = np.zeros(16, np.float32)
    rc = lib().ref_les_descriptor(REFERENCE.encode(), config.encode(), _fp(desc))
    if rc != 0:
        raise RuntimeError("RS_set_vel_data_to_config failed (%d)" % rc)
    return desc


# ------------------------------------------------- the reference's rs.cl
class _RsclLib:
    """The reference's rs.cl kernels compiled for the CPU (oracle/ref/rscl.h),
    under the oracle's entry-point names: oracle.advance_time / db_rcs /
    make_pulse(..., L=rscl()) run them where they would run the oracle's."""

    def __init__(self, L, O):
        self._L = L
        img = O.Image
        _s = ctypes.c_size_t
        f32, u32, i32 = ctypes.c_float, ctypes.c_uint32, ctypes.c_int
        sig = {
            "el_atts": [_f, _f, _f, _u, img, _f, _f, _f, _f, _s, _s],
            "bg_atts": [_f, _f, _f, _u, img, _f, _f, _f, _f, _s, _s],
            "fp_atts": [_f, _f, _f, img, img, _f, _f, _s, _s],
            "db_atts": [_f, _f, _f, _f, _f, _u, img, _f, img, img, _f, img, img, _f, _f, _f, _f, _s, _s],
            "db_rcs": [_f, _f, _f, img, img, _f, _f, _s, _s],
            "scat_sig_aux": [_f, _f, _f, _f, _f, _f, _f, _s],
            "pop": [_f, _f, _f, _f, _s],
            "make_pulse_pass_1": [_f, _f, _f, _s, _f, _f, f32, f32, u32, u32, u32, u32],
            "make_pulse_pass_2_local": [_f, _f, _s, u32, u32, _s, _s],
            "make_pulse_pass_2_range": [_f, _f, _s, u32, u32, _s, _s],
            "make_pulse_pass_2_group": [_f, _f, _s, u32, u32, _s, _s],
            "make_pulse": [_f, _f, _f, _f, _f, _s, _s, _f, _f, _f, _f, f32, f32, u32, _f, u32, u32, u32, i32],
        }
        for name, args in sig.items():
            fn = getattr(L, "rscl_" + name)
            fn.argtypes = args
            fn.restype = i32 if name == "make_pulse" else None

    def __getattr__(self, name):
        if name.startswith("or_"):
            return getattr(self._L, "rscl_" + name[3:])
        return getattr(self._L, name)


_rscl = None


def rscl():
    """The reference's rs.cl kernels behind the oracle's entry-point names."""
    global _rscl
    if _rscl is None:
        from . import oracle as O
        _rscl = _RsclLib(lib(), O)
    return _rscl


# ---------------------------------------------------------------- sessions
_DT = {"f4": np.float32, "u4": np.uint32, "i4": np.int32, "f8": np.float64, "u8": np.uint64}


def read_session(path):
    """The named arrays of a refdrive record file."""
    raw = open(path, "rb").read()
    if raw[:8] != b"RSREF001":
        raise ValueError("%s is not a refdrive record" % path)
    off = 8
    out = {}
    while off < len(raw):
        name = raw[off:off + 48].split(b"\0", 1)[0].decode()
        dtype = raw[off + 48:off + 56].split(b"\0", 1)[0].decode()
        ndim = int(np.frombuffer(raw, np.uint32, 1, off + 56)[0])
        shape = tuple(int(v) for v in np.frombuffer(raw, np.uint64, 4, off + 64)[:ndim])
        nbytes = int(np.frombuffer(raw, np.uint64, 1, off + 96)[0])
        off += 104
        a = np.frombuffer(raw, _DT[dtype], nbytes // np.dtype(_DT[dtype]).itemsize, off).copy()
        out[name] = a.reshape(shape) if ndim else a[0]
        off += nbytes
    return out


_CODE = {np.dtype(np.float32): "f4", np.dtype(np.uint32): "u4", np.dtype(np.int32): "i4",
         np.dtype(np.float64): "f8", np.dtype(np.uint64): "u8"}


def write_session(path, arrays):
    """Write named arrays as a record file (the format read_session reads and
    tests/c/host_loop.c takes); entries of other types are left out."""
    with open(path, "wb") as f:
        f.write(b"RSREF001")
        for name, v in arrays.items():
            a = np.asarray(v)
            if a.dtype not in _CODE:
                continue
            a = np.ascontiguousarray(a)
            shape = list(a.shape) + [0] * (4 - a.ndim)
            f.write(name.encode().ljust(48, b"\0") + _CODE[a.dtype].encode().ljust(8, b"\0"))
            f.write(np.array([a.ndim, 0], np.uint32).tobytes() + np.array(shape, np.uint64).tobytes())
            f.write(np.array([a.nbytes], np.uint64).tobytes() + a.tobytes())


def run_session(out_path, home, density=0.3, pulses=20, warmup=130, debris=(), seed=19760520, gate=30.0,
                scan="P:3.0,-12:12:0.24", concept=None, les="suctvort", threads=None, kernels="oracle"):
    """Run refdrive (rs.c on the CPU device of the OpenCL shim) with the tables
    under <home>/Documents/tables and return the record.  kernels: "oracle"
    (the device runs the oracle's restatement of each rs.cl kernel) or "rscl"
    (the reference's own rs.cl, compiled for the CPU)."""
    lib()
    cmd = [DRIVE, out_path, "--bundle", REFERENCE, "--density", repr(density), "--pulses", str(pulses),
           "--warmup", str(warmup), "--seed", str(seed), "--gate", repr(gate), "--scan", scan, "--les", les,
           "--kernels", kernels]
    if concept is not None:
        cmd += ["--concept", str(int(concept))]
    for t, n in debris:
        cmd += ["--debris", "%d:%d" % (t, n)]
    env = dict(os.environ, HOME=home)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    p = subprocess.run(cmd, env=env, cwd=home, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("refdrive failed (%d):\n%s\n%s" % (p.returncode, p.stdout[-2000:], p.stderr[-2000:]))
    return read_session(out_path)


def fnv1a(a):
    """The FNV-1a 64-bit hash refdrive uses, of an array's bytes."""
    b = np.frombuffer(np.ascontiguousarray(a).tobytes(), np.uint8)
    h = 14695981039346656037
    # chunked: the per-byte recurrence in Python over numpy slices
    prime = 1099511628211
    mask = (1 << 64) - 1
    for x in b.tolist():
        h = ((h ^ x) * prime) & mask
    return h
