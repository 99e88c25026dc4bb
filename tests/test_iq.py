"""The .iq writer (rsc_iq_*): the layout of simradar.c's write_iq_file and
matlab/simradariq.m, byte offsets checked field by field; CPU only (the
writer is host code in the backend library)."""
import struct

import numpy as np

from simradar_gb300 import build, iqfile


def test_iq_file_layout(tmp_path):
    build.build()
    G = 40
    params = {n: float(i + 1) * 0.5 for i, n in enumerate(iqfile.PARAM_NAMES)}
    params["range_count"] = G
    rng = np.random.default_rng(1)
    blocks = [rng.standard_normal((100, 48, 4)).astype(np.float32) for _ in range(3)]
    path = str(tmp_path / "run.iq")
    with iqfile.IQWriter(path, params, counts=[1998848, 1024, 1024, 1024], scan_mode="PPI", scan_start=-12.0,
                         scan_end=12.0, scan_delta=0.24, seed=19760520) as w:
        for k, b in enumerate(blocks):
            t = np.arange(100, dtype=np.float32) * 1e-3 + k * 0.1
            w.write(b, times=t, el_deg=np.full(100, 3.0, np.float32), az_deg=np.linspace(-12, 12, 100), gain=2.0)
        w.flush()
    raw = open(path, "rb").read()
    assert len(raw) == 1024 + 300 * (32 + 16 * G)
    # field offsets of the 1024-byte header (rs_types.h RSParams, iq.h)
    assert struct.unpack_from("<f", raw, 0)[0] == 0.5 and struct.unpack_from("<f", raw, 92)[0] == 12.0
    assert struct.unpack_from("<I", raw, 96)[0] == G
    assert struct.unpack_from("<4I", raw, 100) == (1998848, 1024, 1024, 1024)
    assert raw[132:135] == b"PPI" and raw[135:148] == b"\0" * 13
    assert struct.unpack_from("<3f", raw, 148) == (-12.0, 12.0, np.float32(0.24))
    assert struct.unpack_from("<I", raw, 160)[0] == 19760520
    assert raw[164:1024] == b"\0" * (1024 - 164)
    d = iqfile.read_iq(path)
    assert d["params"]["range_count"] == G and d["params"]["dr"] == 12.0
    assert d["scan_mode"] == "PPI" and d["seed"] == 19760520
    iq = np.concatenate([b[:, :G] * np.float32(2.0) for b in blocks])
    assert np.array_equal(d["iq"], iq)
    assert np.allclose(d["time"][100:103], [0.1, 0.101, 0.102]) and np.all(d["el_deg"] == 3.0)
    # the pulse header pads to 32 bytes with zeros
    assert raw[1024 + 12:1024 + 32] == b"\0" * 20
