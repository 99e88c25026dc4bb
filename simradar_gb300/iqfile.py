"""Reader of simradar's .iq files (the layout of matlab/simradariq.m), and the
ctypes binding of the backend's background writer (rsc_iq_* in include/rsc.h)."""
import ctypes
import struct

import numpy as np

PARAM_NAMES = ("c", "prt", "loss", "lambda", "tx_power_watt", "antenna_gain_dbi", "antenna_bw_deg", "tau",
               "range_start", "range_end", "range_delta", "azimuth_start_deg", "azimuth_end_deg",
               "azimuth_delta_deg", "elevation_start_deg", "elevation_end_deg", "elevation_delta_deg",
               "domain_pad_factor", "body_per_cell", "prf", "va", "fn", "antenna_bw_rad", "dr")
HEADER_BYTES = 1024
PULSE_HEADER_BYTES = 32


class IQParams(ctypes.Structure):
    """rsc_iq_params: RSParams (rs_types.h:56-93)."""
    _fields_ = [(n, ctypes.c_float) for n in PARAM_NAMES] + [("range_count", ctypes.c_uint32)]


def read_iq(path):
    """The file header, the pulse headers and the I/Q samples of a .iq file:
    iq is (pulses, range_count, 4) float32 (Ih, Qh, Iv, Qv)."""
    with open(path, "rb") as f:
        raw = f.read()
    hdr = raw[:HEADER_BYTES]
    vals = struct.unpack_from("<24fI", hdr, 0)
    params = dict(zip(PARAM_NAMES, vals[:24]))
    params["range_count"] = vals[24]
    counts = list(struct.unpack_from("<8I", hdr, 100))
    scan_mode = hdr[132:148].split(b"\0", 1)[0].decode("ascii", "replace")
    scan = struct.unpack_from("<3f", hdr, 148)
    seed = struct.unpack_from("<I", hdr, 160)[0]
    G = params["range_count"]
    per = PULSE_HEADER_BYTES + 16 * G
    n = (len(raw) - HEADER_BYTES) // per
    body = np.frombuffer(raw, dtype=np.uint8, count=n * per, offset=HEADER_BYTES).reshape(n, per)
    ph = body[:, :12].copy().view("<f4").reshape(n, 3)
    iq = body[:, PULSE_HEADER_BYTES:].copy().view("<f4").reshape(n, G, 4)
    return {"params": params, "debris_counts": counts, "scan_mode": scan_mode, "scan_start": scan[0],
            "scan_end": scan[1], "scan_delta": scan[2], "seed": seed, "time": ph[:, 0], "el_deg": ph[:, 1],
            "az_deg": ph[:, 2], "iq": iq}


class IQWriter:
    """The backend's .iq writer (a background thread does the file I/O)."""

    def __init__(self, path, params, counts=(), scan_mode="", scan_start=0.0, scan_end=0.0, scan_delta=0.0, seed=0):
        from .rsc import load_library
        L = load_library()
        L.rsc_iq_open.argtypes = [ctypes.c_char_p, ctypes.POINTER(IQParams), ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.c_char_p, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint32,
                                  ctypes.POINTER(ctypes.c_void_p)]
        L.rsc_iq_write.argtypes = [ctypes.c_void_p, ctypes.c_uint32] + [ctypes.POINTER(ctypes.c_float)] * 4 + \
            [ctypes.c_uint32, ctypes.c_float]
        L.rsc_iq_flush.argtypes = [ctypes.c_void_p]
        L.rsc_iq_close.argtypes = [ctypes.c_void_p]
        L.rsc_iq_last_error.restype = ctypes.c_char_p
        self._L = L
        p = IQParams(**{k: float(params.get(k, 0.0)) for k in PARAM_NAMES})
        p.range_count = int(params["range_count"])
        c = (ctypes.c_uint32 * 8)(*([int(v) for v in counts] + [0] * (8 - len(counts))))
        h = ctypes.c_void_p()
        self._check(L.rsc_iq_open(path.encode(), ctypes.byref(p), c, scan_mode.encode(), float(scan_start),
                                  float(scan_end), float(scan_delta), int(seed), ctypes.byref(h)))
        self._h = h
        self.range_count = p.range_count

    def _check(self, status):
        if status != 0:
            raise RuntimeError("rsc_iq status %d: %s" % (status, self._L.rsc_iq_last_error().decode()))

    def write(self, pulses4, times=None, el_deg=None, az_deg=None, gain=1.0):
        """pulses4: (count, row_gates, 4) float32, row_gates >= range_count."""
        a = np.ascontiguousarray(pulses4, dtype=np.float32)
        count, row = a.shape[0], a.shape[1]
        fp = ctypes.POINTER(ctypes.c_float)
        arrs = [None if v is None else np.ascontiguousarray(v, dtype=np.float32) for v in (times, el_deg, az_deg)]
        ptr = [None if v is None else v.ctypes.data_as(fp) for v in arrs]
        self._check(self._L.rsc_iq_write(self._h, count, ptr[0], ptr[1], ptr[2], a.ctypes.data_as(fp), row,
                                         float(gain)))

    def flush(self):
        self._check(self._L.rsc_iq_flush(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._check(self._L.rsc_iq_close(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
