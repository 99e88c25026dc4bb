"""ctypes binding of the backend C ABI (include/rsc.h).

The shared library is the product; this module only marshals numpy arrays
(float32 / uint32, C-contiguous) into the plain pointers the ABI takes.  There
is no other implementation behind it: if the library is missing, importing
the backend raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

RSC_OK = 0
RSC_MAX_TYPES = 8
RSC_MAX_GATES = 512
PULSE_PLAIN = 0
PULSE_COMPENSATED = 1
PULSE_F64 = 2

_f32p = ctypes.POINTER(ctypes.c_float)
_u32p = ctypes.POINTER(ctypes.c_uint32)


class BackendError(RuntimeError):
    """A backend call returned a negative status."""

    def __init__(self, status, message):
        super().__init__("rsc status %d: %s" % (status, message))
        self.status = status


class Population(ctypes.Structure):
    """rsc_population: per-type (origin, count) and the ADM / RCS table each
    debris type uses (RSWorker.origins / .counts, rs.h:160-161)."""

    _fields_ = [
        ("origins", ctypes.c_uint64 * RSC_MAX_TYPES),
        ("counts", ctypes.c_uint64 * RSC_MAX_TYPES),
        ("adm_index", ctypes.c_int32 * RSC_MAX_TYPES),
        ("rcs_index", ctypes.c_int32 * RSC_MAX_TYPES),
    ]

    @classmethod
    def make(cls, counts, origins=None, adm_index=None, rcs_index=None):
        p = cls()
        counts = list(counts) + [0] * (RSC_MAX_TYPES - len(counts))
        if origins is None:
            origins, acc = [], 0
            for c in counts:
                origins.append(acc)
                acc += c
        origins = list(origins) + [0] * (RSC_MAX_TYPES - len(origins))
        for k in range(RSC_MAX_TYPES):
            p.origins[k] = int(origins[k])
            p.counts[k] = int(counts[k])
            p.adm_index[k] = int(adm_index[k]) if adm_index is not None else max(k - 1, 0)
            p.rcs_index[k] = int(rcs_index[k]) if rcs_index is not None else max(k - 1, 0)
        return p


_lib = None


def library_path():
    return _build.LIB


def load_library():
    """Load libsimradar_gb300.so (built by simradar_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        raise ImportError("simradar_gb300 backend library not built: %s (run simradar_gb300.build.build())" % path)
    lib = ctypes.CDLL(path)
    P, I, S, U32, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_float
    sig = {
        "rsc_last_error": ([], ctypes.c_char_p),
        "rsc_device_count": ([ctypes.POINTER(I)], I),
        "rsc_worker_create": ([I, ctypes.POINTER(P)], I),
        "rsc_worker_free": ([P], I),
        "rsc_worker_malloc": ([P, S, F, F, U32], I),
        "rsc_set_range_weight": ([P, _f32p, U32, _f32p], I),
        "rsc_set_angular_weight": ([P, _f32p, U32, _f32p], I),
        "rsc_set_rcs_ellipsoid": ([P, _f32p, U32, _f32p], I),
        "rsc_set_les": ([P, I, _f32p, _f32p, U32, U32, U32, _f32p], I),
        "rsc_set_les_async": ([P, I, _f32p, _f32p, U32, U32, U32, _f32p], I),
        "rsc_set_adm": ([P, I, _f32p, _f32p, U32, U32, _f32p], I),
        "rsc_set_rcs": ([P, I, _f32p, _f32p, U32, U32, _f32p], I),
        "rsc_set_dff": ([P, I, _f32p, U32, _f32p], I),
        "rsc_upload": ([P, S, S, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _u32p], I),
        "rsc_download": ([P, S, S, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _u32p], I),
        "rsc_advance_time": ([P, ctypes.POINTER(Population), I, P], I),
        "rsc_update_debris_rcs": ([P, ctypes.POINTER(Population), _f32p], I),
        "rsc_make_pulse": ([P, P], I),
        "rsc_download_pulse": ([P, P, F], I),
        "rsc_synchronize": ([P], I),
        "rsc_download_pulse_async": ([P, P], I),
        "rsc_set_pulse_precision": ([P, I], I),
        "rsc_set_materialize_sig_aux": ([P, I], I),
        "rsc_set_pulse_moments": ([P, I], I),
        "rsc_launch_count": ([P, ctypes.POINTER(ctypes.c_uint64)], I),
        "rsc_get_stream": ([P, ctypes.POINTER(P)], I),
        "rsc_get_advance_stream": ([P, ctypes.POINTER(P)], I),
        "rsc_eval_math": ([I, _f32p, _f32p, _f32p, S], I),
        "rsc_autotune": ([P, _f32p, ctypes.POINTER(I), ctypes.POINTER(I)], I),
        "rsc_set_pulse_shape": ([P, I, I], I),
        "rsc_set_advance_shape": ([P, I], I),
        "rsc_set_sort_interval": ([P, I], I),
        "rsc_set_fused_step": ([P, I], I),
        "rsc_sort_count": ([P, ctypes.POINTER(ctypes.c_uint64)], I),
        "rsc_batch_create": ([ctypes.POINTER(P), I, ctypes.POINTER(P)], I),
        "rsc_batch_free": ([P], I),
        "rsc_batch_set_populations": ([P, ctypes.POINTER(Population)], I),
        "rsc_batch_set_precision": ([P, I], I),
        "rsc_batch_set_persistent": ([P, I], I),
        "rsc_batch_set_advance_shape": ([P, I, I], I),
        "rsc_batch_get_advance_shape": ([P, ctypes.POINTER(I), ctypes.POINTER(I)], I),
        "rsc_batch_autotune": ([P, _f32p], I),
        "rsc_batch_run": ([P, I, _f32p, ctypes.POINTER(ctypes.c_int32), _f32p, I], I),
        "rsc_batch_run_async": ([P, I, _f32p, ctypes.POINTER(ctypes.c_int32), _f32p, I], I),
        "rsc_batch_synchronize": ([P], I),
        "rsc_batch_set_les_async": ([P, I, I, _f32p, _f32p, U32, U32, U32], I),
        "rsc_batch_max_gates": ([P, ctypes.POINTER(I)], I),
        "rsc_batch_launch_count": ([P, ctypes.POINTER(ctypes.c_uint64)], I),
        "rsc_batch_get_stream": ([P, ctypes.POINTER(P)], I),
        "rsc_batch_get_shape": ([P, ctypes.POINTER(I), ctypes.POINTER(I)], I),
    }
    for name, (argtypes, restype) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = restype
    _lib = lib
    return lib


def _check(status):
    if status != RSC_OK:
        raise BackendError(status, load_library().rsc_last_error().decode(errors="replace"))


def _fp(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"], "expected C-contiguous float32"
    return a.ctypes.data_as(_f32p)


def _up(a):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"], "expected C-contiguous uint32"
    return a.ctypes.data_as(_u32p)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _addr(a):
    """Address of a C-contiguous float32 array (the per-pulse calls take
    plain addresses: cheaper than a ctypes pointer object)."""
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"], "expected C-contiguous float32"
    return a.ctypes.data


def device_count():
    n = ctypes.c_int(0)
    _check(load_library().rsc_device_count(ctypes.byref(n)))
    return n.value


def eval_math(fn, a, b=None):
    a = f32(a)
    b = f32(b) if b is not None else None
    out = np.empty_like(a)
    _check(load_library().rsc_eval_math(int(fn), _fp(a), _fp(b), _fp(out), a.size))
    return out


FIELDS = ("pos", "vel", "ori", "tum", "aux", "rcs", "sig", "rnd")


class Worker:
    """One GPU worker (RSWorker, rs.h:150-266) behind the C ABI."""

    def __init__(self, device=0):
        self._lib = load_library()
        h = ctypes.c_void_p()
        _check(self._lib.rsc_worker_create(int(device), ctypes.byref(h)))
        self._h = h
        self.num_scats = 0
        self.range_count = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rsc_worker_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --- allocation and tables -------------------------------------------
    def malloc(self, num_scats, range_start, range_delta, range_count):
        _check(self._lib.rsc_worker_malloc(self._h, int(num_scats), float(range_start), float(range_delta),
                                           int(range_count)))
        self.num_scats = int(num_scats)
        self.range_count = int(range_count)

    def set_range_weight(self, table, desc):
        t, d = f32(table), f32(desc)
        _check(self._lib.rsc_set_range_weight(self._h, _fp(t), t.size, _fp(d)))

    def set_angular_weight(self, table, desc):
        t, d = f32(table), f32(desc)
        _check(self._lib.rsc_set_angular_weight(self._h, _fp(t), t.size, _fp(d)))

    def set_rcs_ellipsoid(self, table4, desc):
        t, d = f32(table4), f32(desc)
        _check(self._lib.rsc_set_rcs_ellipsoid(self._h, _fp(t), t.size // 4, _fp(d)))

    def set_les(self, slot, uvwt, cpxx, desc, asynchronous=False):
        """uvwt, cpxx: (nz, ny, nx, 4) float32."""
        u = f32(uvwt)
        c = f32(cpxx) if cpxx is not None else None
        d = f32(desc)
        nz, ny, nx = u.shape[:3]
        fn = self._lib.rsc_set_les_async if asynchronous else self._lib.rsc_set_les
        _check(fn(self._h, int(slot), _fp(u), _fp(c), nx, ny, nz, _fp(d)))
        if asynchronous:
            self._keep = (u, c)

    def set_adm(self, index, cd, cm, desc):
        """cd, cm: (ny, nx, 4) float32 (x = beta, y = alpha)."""
        a, b, d = f32(cd), f32(cm), f32(desc)
        ny, nx = a.shape[:2]
        _check(self._lib.rsc_set_adm(self._h, int(index), _fp(a), _fp(b), nx, ny, _fp(d)))

    def set_rcs(self, index, real, imag, desc):
        """real, imag: (ny, nx, 4) float32 (x = alpha, y = beta)."""
        a, b, d = f32(real), f32(imag), f32(desc)
        ny, nx = a.shape[:2]
        _check(self._lib.rsc_set_rcs(self._h, int(index), _fp(a), _fp(b), nx, ny, _fp(d)))

    def set_dff(self, slot, icdf, desc):
        t, d = f32(icdf), f32(desc)
        _check(self._lib.rsc_set_dff(self._h, int(slot), _fp(t), t.size, _fp(d)))

    # --- state -----------------------------------------------------------
    def upload(self, offset=0, **arrays):
        count = None
        ptrs = []
        keep = []
        for f in FIELDS:
            a = arrays.get(f)
            if a is None:
                ptrs.append(None)
                continue
            a = np.ascontiguousarray(a, dtype=np.uint32 if f == "rnd" else np.float32)
            keep.append(a)
            n = a.size // 4
            if count is None:
                count = n
            elif count != n:
                raise ValueError("arrays of different lengths")
            ptrs.append(_up(a) if f == "rnd" else _fp(a))
        if count is None:
            return
        _check(self._lib.rsc_upload(self._h, int(offset), int(count), *ptrs))

    def download(self, fields=FIELDS, offset=0, count=None):
        if count is None:
            count = self.num_scats - offset
        out = {}
        ptrs = []
        for f in FIELDS:
            if f in fields:
                a = np.empty((count, 4), dtype=np.uint32 if f == "rnd" else np.float32)
                out[f] = a
                ptrs.append(_up(a) if f == "rnd" else _fp(a))
            else:
                ptrs.append(None)
        _check(self._lib.rsc_download(self._h, int(offset), int(count), *ptrs))
        return out

    # --- hot path --------------------------------------------------------
    def advance_time(self, pop, les_id, sim_desc):
        d = f32(sim_desc)
        _check(self._lib.rsc_advance_time(self._h, ctypes.byref(pop), int(les_id), _addr(d)))

    def update_debris_rcs(self, pop, sim_desc):
        d = f32(sim_desc)
        _check(self._lib.rsc_update_debris_rcs(self._h, ctypes.byref(pop), _fp(d)))

    def make_pulse(self, sim_desc):
        d = f32(sim_desc)
        _check(self._lib.rsc_make_pulse(self._h, _addr(d)))

    def download_pulse(self, gain=1.0, out=None):
        if out is None:
            out = np.empty((self.range_count, 4), dtype=np.float32)
        _check(self._lib.rsc_download_pulse(self._h, _addr(out), float(gain)))
        return out

    def download_pulse_async(self, out):
        """Queue the copy of the latest pulse (no gain) into `out`, a
        (range_count, 4) float32 array (page-locked for an asynchronous
        copy); it is complete after synchronize()."""
        assert out.shape == (self.range_count, 4)
        _check(self._lib.rsc_download_pulse_async(self._h, _addr(out)))

    def synchronize(self):
        _check(self._lib.rsc_synchronize(self._h))

    def set_precision(self, mode):
        _check(self._lib.rsc_set_pulse_precision(self._h, int(mode)))

    def set_materialize(self, enable):
        _check(self._lib.rsc_set_materialize_sig_aux(self._h, 1 if enable else 0))

    def set_moments(self, enable):
        """The compensated form's interval moments on or off (rsc_set_pulse_moments)."""
        _check(self._lib.rsc_set_pulse_moments(self._h, 1 if enable else 0))

    @property
    def launch_count(self):
        n = ctypes.c_uint64(0)
        _check(self._lib.rsc_launch_count(self._h, ctypes.byref(n)))
        return n.value

    @property
    def stream(self):
        s = ctypes.c_void_p()
        _check(self._lib.rsc_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    @property
    def advance_stream(self):
        """The stream advance_time issues on, beside the pulses."""
        s = ctypes.c_void_p()
        _check(self._lib.rsc_get_advance_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def set_sort_interval(self, steps):
        """Steps between re-sorts of the background range into spatial
        order (0: keep the caller's order)."""
        _check(self._lib.rsc_set_sort_interval(self._h, int(steps)))

    def set_fused_step(self, enable):
        """Run advance_time with the following make_pulse in one kernel."""
        _check(self._lib.rsc_set_fused_step(self._h, 1 if enable else 0))

    @property
    def sort_count(self):
        n = ctypes.c_uint64(0)
        _check(self._lib.rsc_sort_count(self._h, ctypes.byref(n)))
        return n.value

    def autotune(self, sim_desc):
        """Pick the pulse kernel's launch shape by timing (warps, blocks/SM)."""
        d = f32(sim_desc)
        wv, pv = ctypes.c_int(0), ctypes.c_int(0)
        _check(self._lib.rsc_autotune(self._h, _fp(d), ctypes.byref(wv), ctypes.byref(pv)))
        return wv.value, pv.value

    def set_pulse_shape(self, warps, blocks_per_sm):
        """Fix the pulse kernel's launch shape (0 = the largest that fits)."""
        _check(self._lib.rsc_set_pulse_shape(self._h, int(warps), int(blocks_per_sm)))

    def set_advance_shape(self, scatterers_per_thread):
        """Background scatterers per advance thread, 1 or 2 (rsc_set_advance_shape)."""
        _check(self._lib.rsc_set_advance_shape(self._h, int(scatterers_per_thread)))


class Batch:
    """Many workers stepped together: three launches per step for all of them
    (the batching form of include/rsc.h).  Keeps references to the workers so
    they outlive the batch."""

    def __init__(self, workers):
        self._lib = load_library()
        self.workers = list(workers)
        arr = (ctypes.c_void_p * len(self.workers))(*[w._h.value for w in self.workers])
        h = ctypes.c_void_p()
        _check(self._lib.rsc_batch_create(arr, len(self.workers), ctypes.byref(h)))
        self._h = h
        g = ctypes.c_int(0)
        _check(self._lib.rsc_batch_max_gates(self._h, ctypes.byref(g)))
        self.max_gates = g.value
        self._keep = []

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rsc_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_populations(self, pops):
        arr = (Population * len(self.workers))(*pops)
        _check(self._lib.rsc_batch_set_populations(self._h, arr))

    def set_precision(self, mode):
        _check(self._lib.rsc_batch_set_precision(self._h, int(mode)))

    def set_advance_shape(self, threads, blocks_per_sm=0):
        """The batched background advance's block size and resident blocks per SM."""
        _check(self._lib.rsc_batch_set_advance_shape(self._h, int(threads), int(blocks_per_sm)))

    @property
    def advance_shape(self):
        t, p = ctypes.c_int(0), ctypes.c_int(0)
        _check(self._lib.rsc_batch_get_advance_shape(self._h, ctypes.byref(t), ctypes.byref(p)))
        return t.value, p.value

    def set_persistent(self, enable):
        """Run every step of a run in one launch (rsc_batch_set_persistent)."""
        _check(self._lib.rsc_batch_set_persistent(self._h, 1 if enable else 0))

    def autotune(self, sim_descs):
        d = f32(sim_descs).reshape(len(self.workers), 16)
        _check(self._lib.rsc_batch_autotune(self._h, _fp(d)))
        return self.shape

    @property
    def shape(self):
        wv, pv = ctypes.c_int(0), ctypes.c_int(0)
        _check(self._lib.rsc_batch_get_shape(self._h, ctypes.byref(wv), ctypes.byref(pv)))
        return wv.value, pv.value

    def run(self, sim_descs, les_ids=None, out=None, use_graph=True, download=True, wait=True):
        """sim_descs: (steps, instances, 16).  Returns (steps, instances,
        max_gates, 4) pulses (no gain) when download is set.  With wait False
        the call returns once the work is queued; `out` (page-locked for an
        asynchronous copy) is filled by the time synchronize() returns."""
        d = f32(sim_descs)
        steps = d.shape[0]
        d = d.reshape(steps, len(self.workers), 16)
        if les_ids is None:
            les = np.zeros((steps, len(self.workers)), dtype=np.int32)
        else:
            les = np.ascontiguousarray(les_ids, dtype=np.int32).reshape(steps, len(self.workers))
        if download and out is None:
            out = np.empty((steps, len(self.workers), self.max_gates, 4), dtype=np.float32)
        fn = self._lib.rsc_batch_run if wait else self._lib.rsc_batch_run_async
        _check(fn(self._h, int(steps), _fp(d), les.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                  _fp(out) if download else None, 1 if use_graph else 0))
        return out if download else None

    def synchronize(self):
        _check(self._lib.rsc_batch_synchronize(self._h))
        self._keep = []

    def set_les_async(self, index, slot, uvwt, cpxx=None):
        """Refill an instance's LES slot on the batch's copy stream (the
        arrays must stay alive, and should be page-locked, until
        synchronize())."""
        u = f32(uvwt)
        c = f32(cpxx) if cpxx is not None else None
        nz, ny, nx = u.shape[:3]
        self._keep.append((u, c))
        _check(self._lib.rsc_batch_set_les_async(self._h, int(index), int(slot), _fp(u), _fp(c), nx, ny, nz))

    @property
    def launch_count(self):
        n = ctypes.c_uint64(0)
        _check(self._lib.rsc_batch_launch_count(self._h, ctypes.byref(n)))
        return n.value

    @property
    def stream(self):
        s = ctypes.c_void_p()
        _check(self._lib.rsc_batch_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0


class PopulateArgs(ctypes.Structure):
    """rsc_populate_args: what RS_populate reads from its handle."""
    _fields_ = [("seed", ctypes.c_uint32), ("sim_concept", ctypes.c_uint32),
                ("domain_origin", ctypes.c_float * 3), ("domain_size", ctypes.c_float * 3),
                ("num_types", ctypes.c_uint32),
                ("origins", ctypes.c_uint64 * RSC_MAX_TYPES), ("counts", ctypes.c_uint64 * RSC_MAX_TYPES),
                ("dsd_r", _f32p), ("dsd_cdf", _f32p), ("dsd_count", ctypes.c_uint32)]

    @classmethod
    def make(cls, seed, concept, origin, size, counts, dsd_r=None, dsd_cdf=None):
        a = cls()
        a.seed = int(seed) & 0xFFFFFFFF
        a.sim_concept = int(concept)
        for k in range(3):
            a.domain_origin[k] = float(origin[k])
            a.domain_size[k] = float(size[k])
        a.num_types = len(counts)
        acc = 0
        for k, c in enumerate(counts):
            a.origins[k] = acc
            a.counts[k] = int(c)
            acc += int(c)
        if dsd_r is not None:
            a._keep = (f32(dsd_r), f32(dsd_cdf))
            a.dsd_r, a.dsd_cdf = _fp(a._keep[0]), _fp(a._keep[1])
            a.dsd_count = len(dsd_r)
        return a


def _pop_lib():
    L = load_library()
    L.rsc_rand_sequence.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32)]
    L.rsc_populate_host.argtypes = [ctypes.POINTER(PopulateArgs), ctypes.c_size_t] + [_f32p] * 6 + \
        [_u32p, ctypes.POINTER(ctypes.c_uint32)]
    L.rsc_populate_upload.argtypes = [ctypes.c_void_p, ctypes.POINTER(PopulateArgs), ctypes.POINTER(ctypes.c_uint32)]
    L.rsc_populate_last_error.restype = ctypes.c_char_p
    return L


def rand_sequence(seed, count):
    """The first `count` values of glibc's rand() after srand(seed)."""
    L = _pop_lib()
    out = np.zeros(count, dtype=np.int32)
    st = L.rsc_rand_sequence(int(seed) & 0xFFFFFFFF, int(count), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    if st != RSC_OK:
        raise BackendError(st, L.rsc_populate_last_error().decode())
    return out


def populate_host(args, num_scats):
    """RS_populate's initial state as host arrays (dict of (num_scats, 4))."""
    L = _pop_lib()
    arr = {f: np.zeros((num_scats, 4), np.float32) for f in ("pos", "vel", "ori", "tum", "aux", "rcs")}
    arr["rnd"] = np.zeros((num_scats, 4), np.uint32)
    pop = np.zeros(max(1, args.dsd_count), np.uint32)
    st = L.rsc_populate_host(ctypes.byref(args), num_scats, _fp(arr["pos"]), _fp(arr["vel"]), _fp(arr["ori"]),
                             _fp(arr["tum"]), _fp(arr["aux"]), _fp(arr["rcs"]), _up(arr["rnd"]),
                             pop.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    if st != RSC_OK:
        raise BackendError(st, L.rsc_populate_last_error().decode())
    arr["sig"] = np.zeros((num_scats, 4), np.float32)
    return arr, pop[:args.dsd_count]


def populate_upload(worker, args):
    """Generate the initial state straight into an allocated worker."""
    L = _pop_lib()
    pop = np.zeros(max(1, args.dsd_count), np.uint32)
    _check(L.rsc_populate_upload(worker._h, ctypes.byref(args), pop.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
    return pop[:args.dsd_count]


class LESInfo(ctypes.Structure):
    """rsc_les_info: dimensions, frame count and constants of an LES folder."""
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32),
                ("files", ctypes.c_uint32), ("volumes_per_file", ctypes.c_uint32), ("frames", ctypes.c_uint32),
                ("is_stretched", ctypes.c_int32), ("p_for_cn2", ctypes.c_int32),
                ("tr", ctypes.c_float), ("tp", ctypes.c_float),
                ("v0", ctypes.c_float), ("p0", ctypes.c_float), ("t0", ctypes.c_float),
                ("ax", ctypes.c_float), ("ay", ctypes.c_float), ("az", ctypes.c_float),
                ("rx", ctypes.c_float), ("ry", ctypes.c_float), ("rz", ctypes.c_float)]


def _les_lib():
    L = load_library()
    P, I, U32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32
    for name, argtypes in {
        "rsc_les_open": [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(P)],
        "rsc_les_get_info": [P, ctypes.POINTER(LESInfo)],
        "rsc_les_grid": [P, _f32p, _f32p, _f32p],
        "rsc_les_descriptor": [ctypes.POINTER(LESInfo), _f32p],
        "rsc_les_read": [P, U32, _f32p, _f32p, _f32p],
        "rsc_les_prefetch": [P, U32],
        "rsc_les_upload_async": [P, P, I, U32, _f32p],
        "rsc_les_close": [P],
    }.items():
        fn = getattr(L, name)
        fn.argtypes = argtypes
        fn.restype = I
    L.rsc_les_last_error.restype = ctypes.c_char_p
    return L


class LESSource:
    """An LES folder of les.c (fort.10_2 + LES_mean_1_6_fnum<k>.dat) with a
    read-ahead thread: host frames (read) or device slots (upload_async)."""

    def __init__(self, directory, config="suctvort"):
        self._lib = _les_lib()
        self._h = ctypes.c_void_p()
        self._check(self._lib.rsc_les_open(os.fsencode(directory), config.encode(), ctypes.byref(self._h)))
        self.info = LESInfo()
        self._check(self._lib.rsc_les_get_info(self._h, ctypes.byref(self.info)))

    def _check(self, st):
        if st != RSC_OK:
            raise BackendError(st, self._lib.rsc_les_last_error().decode(errors="replace"))

    @property
    def shape(self):
        return (self.info.nz, self.info.ny, self.info.nx)

    @property
    def frames(self):
        return self.info.frames

    def descriptor(self):
        d = np.zeros(16, np.float32)
        self._check(self._lib.rsc_les_descriptor(ctypes.byref(self.info), _fp(d)))
        return d

    def grid(self):
        x, y, z = (np.zeros(self.shape, np.float32) for _ in range(3))
        self._check(self._lib.rsc_les_grid(self._h, _fp(x), _fp(y), _fp(z)))
        return x, y, z

    def read(self, frame):
        """(uvwt, cpxx, time) of a frame, remapped as les.c does."""
        uvwt = np.zeros(self.shape + (4,), np.float32)
        cpxx = np.zeros(self.shape + (4,), np.float32)
        t = ctypes.c_float(0.0)
        self._check(self._lib.rsc_les_read(self._h, int(frame), _fp(uvwt), _fp(cpxx), ctypes.byref(t)))
        return uvwt, cpxx, t.value

    def prefetch(self, frame):
        self._check(self._lib.rsc_les_prefetch(self._h, int(frame)))

    def upload_async(self, worker, slot, frame):
        """Frame into a worker's LES slot (copy stream + remap kernel); returns
        the frame's time stamp."""
        t = ctypes.c_float(0.0)
        _check(self._lib.rsc_les_upload_async(worker._h, self._h, int(slot), int(frame), ctypes.byref(t)))
        return t.value

    def close(self):
        if self._h:
            self._lib.rsc_les_close(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
