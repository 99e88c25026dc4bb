"""numpy restatement of the LES ingest of les.c (frame files -> uvwt / cpxx).

TEST INFRASTRUCTURE ONLY: imported by tests/ to check rsc_les_read and the
device remap of rsc_les_upload_async, never by the simradar_gb300 package.

Follows les.c:
  grid file fort.10_2          LES_enclosing_grid_create_from_file, les.c:477-518
  frame files and volume count LES_init_with_config_path, les.c:212-244
  constants by configuration   les.c:158-208 (tr = 50, les.c:139)
  frame offset and the reads   LES_background_read, les.c:350-386
  remap                        les.c:388-406
  descriptor                   RS_set_vel_data_to_LES_table, rs.c:3041-3078,
                               and RS_set_vel_data, rs.c:2944-2976
"""
import math
import os

import numpy as np

F = np.float32
FILE_VOLUMES = 10   # LES_file_nblock, les.c:12


def grid(directory):
    """(nx, ny, nz, x, y, z) of fort.10_2."""
    raw = np.fromfile(os.path.join(directory, "fort.10_2"), dtype=np.uint8)
    head = raw[:16].view(np.uint32)
    nx, ny, nz = int(head[1]), int(head[2]), int(head[3])
    n = nx * ny * nz
    off = 16
    axes = []
    for _ in range(3):
        off += 8
        axes.append(raw[off:off + 4 * n].view(np.float32).reshape(nz, ny, nx).copy())
        off += 4 * n
    return nx, ny, nz, axes[0], axes[1], axes[2]


def constants(config, x, y, z):
    """(v0, p0, t0, a[3], r[3], tp, stretched) of les.c:158-208."""
    c = config.lower()
    if c in ("suctvort", "suctvort_large"):
        v0 = F(100.0)
        return v0, F(v0 * v0), F(v0 * v0), [F(2.0)] * 3, [F(1.0212), F(1.0212), F(1.05)], F(2.0), True
    if c == "twocell":
        v0 = F(225.0)
        return v0, F(v0 * v0), F(v0 * v0), [F(1.0)] * 3, [F(1.0)] * 3, F(5.0), False
    if c == "flat":
        nz, ny, nx = x.shape
        xf, yf, zf = x.reshape(-1), y.reshape(-1), z.reshape(-1)
        r = [F(F(1.0e3) * F(xf[1] - xf[0])), F(F(1.0e3) * F(yf[nx] - yf[0])), F(F(1.0e3) * F(zf[nx * ny] - zf[0]))]
        return F(100.0), F(1.0), F(1.0e4), [F(0.0)] * 3, r, F(60.0), False
    v0 = F(100.0)
    return v0, F(v0 * v0), F(v0 * v0), [F(1.0)] * 3, [F(1.0)] * 3, F(5.0), False


def frame_files(directory):
    files = []
    while os.path.exists(os.path.join(directory, "LES_mean_1_6_fnum%d.dat" % (len(files) + 1))):
        files.append(os.path.join(directory, "LES_mean_1_6_fnum%d.dat" % (len(files) + 1)))
    return files


def volumes_per_file(directory):
    nx, ny, nz = grid(directory)[:3]
    size = os.path.getsize(frame_files(directory)[0])
    return size // (4 + 8 + nx * ny * nz * 5 * 4 + 8)


def frame(directory, config, n):
    """(uvwt, cpxx, time) of frame n, shapes (nz, ny, nx, 4)."""
    nx, ny, nz, x, y, z = grid(directory)
    nn = nx * ny * nz
    v0, p0, t0 = constants(config, x, y, z)[:3]
    path = frame_files(directory)[n // FILE_VOLUMES]
    per = 4 + 8 + 5 * (4 * nn + 8)
    off = 4 + (n % FILE_VOLUMES) * per
    with open(path, "rb") as f:
        f.seek(off)
        blob = f.read(per - 8)
    time = np.frombuffer(blob[:4], np.float32)[0]
    planes = []
    o = 12
    for _ in range(5):
        planes.append(np.frombuffer(blob[o:o + 4 * nn], np.float32).reshape(nz, ny, nx))
        o += 4 * nn + 8
    u, v, w, p, t = planes
    uvwt = np.stack([u * v0, v * v0, w * v0, t * t0], axis=-1).astype(np.float32)
    cpxx = np.zeros_like(uvwt)
    if config == "flat":   # case-sensitive in les.c:324
        cpxx[..., 0] = p * p0
    else:
        cpxx[..., 1] = p * p0
    return uvwt, cpxx, float(time)


def descriptor(config, nx, ny, nz, x=None, y=None, z=None):
    """The 16-float LES descriptor rs.c derives from the table constants."""
    _, _, _, a, r, _, stretched = constants(config, x, y, z)
    d = np.zeros(16, np.float32)
    n = (nx, ny, nz)
    if stretched:
        d[7] = np.array([7], np.uint32).view(np.float32)[0]
        for k in range(3):
            d[k] = F(1.0 / math.log(float(r[k])))
            d[4 + k] = F(F(r[k] - F(1.0)) / a[k])
            d[8 + k] = F(F(0.5) * F(n[k] - 1)) if k < 2 else F(0.0)
    else:
        for k in range(3):
            d[k] = F(F(1.0) / r[k])
            d[4 + k] = F(F(n[k] - 1) * F(0.5)) if k < 2 else F(0.0)
            d[8 + k] = F(F(n[k]) - F(1.0))
    d[3] = F(50.0)
    return d
