"""Synthetic, seeded inputs for the emulation loop.

The reference's data tables (LES wind volumes, debris ADM and RCS tables) are
a 15 GB archive that is not available, so every table here is synthetic and
seeded, with the shapes and value ranges of the real ones:

  LES   176 x 176 x 80 stretched grid (base 2 m, ratio 1.0212 horizontal,
        1.05 vertical), a Burgers-Rott vortex (50 m/s peak at a 100 m core
        radius, centred in the domain) plus seeded Gaussian turbulence
        (sigma 3 m/s); several time volumes.
  ADM   drag / moment coefficients on a 181 (beta) x 91 (alpha) grid, smooth
        low-order harmonics with seeded coefficients.
  RCS   complex hh / vv / hv on a 181 (alpha) x 91 (beta) grid, log-normal
        magnitude and uniform phase, lightly smoothed.
  DSD   Marshall-Palmer, N0 = 8000 m^-3 mm^-1, Lambda = 2300 m^-1.

The descriptors follow the reference host arithmetic (single precision where
rs.c uses float): RS_set_vel_data_to_LES_table (rs.c:3029-3126),
RS_set_adm_data_to_ADM_table (rs.c:3765-3812), RS_set_rcs_data_to_RCS_table
(rs.c:3975-4021), RS_set_range_weight_to_triangle (rs.c:2620-2623),
RS_set_angular_weight_to_standard (rs.c:2826-2852), RS_compute_rcs_ellipsoids
(rs.c:5922-6030), ADM_compute_properties (adm.c:279-304).
"""
import math
import os
import struct

import numpy as np

F = np.float32


def fbits(u):
    """A float whose bits are the uint32 u (the concept / spacing fields)."""
    return struct.unpack("<f", struct.pack("<I", u))[0]


# concept bits (rs_enum.h:127-137)
CONCEPT_CROSS_POL = 1
CONCEPT_DRAGGED = 1 << 1
CONCEPT_TRANSPARENT = 1 << 2
CONCEPT_BOUNDED = 1 << 3
CONCEPT_UNIFORM_DSD = 1 << 4
CONCEPT_FIXED_POS = 1 << 5
CONCEPT_VERTICAL = 1 << 6
CONCEPT_DFF = 1 << 7
CONCEPT_DBU = CONCEPT_DRAGGED | CONCEPT_BOUNDED | CONCEPT_UNIFORM_DSD  # simradar default (simradar.c:746-750)

SPACING_STRETCHED_XYZ = 7


# ---------------------------------------------------------------- LES tables
class LESVolume:
    """One LES time volume: uvwt and cpxx as (nz, ny, nx, 4) float32."""

    def __init__(self, uvwt, cpxx):
        self.uvwt = uvwt
        self.cpxx = cpxx


class LESConfig:
    def __init__(self, nx=176, ny=176, nz=80, ax=2.0, ay=2.0, az=2.0, rx=1.0212, ry=1.0212, rz=1.05, tr=50.0, tp=2.0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.ax, self.ay, self.az = F(ax), F(ay), F(az)
        self.rx, self.ry, self.rz = F(rx), F(ry), F(rz)
        self.tr, self.tp = F(tr), F(tp)

    def desc(self):
        """LES descriptor, stretched grid (rs.c:3041-3056, rs.c:2948-2975)."""
        d = np.zeros(16, dtype=np.float32)
        d[7] = fbits(SPACING_STRETCHED_XYZ)
        d[0] = F(1.0 / math.log(float(self.rx)))
        d[4] = F((self.rx - F(1.0)) / self.ax)
        d[8] = F(F(0.5) * F(self.nx - 1))
        d[1] = F(1.0 / math.log(float(self.ry)))
        d[5] = F((self.ry - F(1.0)) / self.ay)
        d[9] = F(F(0.5) * F(self.ny - 1))
        d[2] = F(1.0 / math.log(float(self.rz)))
        d[6] = F((self.rz - F(1.0)) / self.az)
        d[10] = F(0.0)
        d[3] = self.tr
        return d

    def node_positions(self):
        """Physical position of the texel centres relative to the domain centre
        (x, y) and the ground (z): the stretched index k maps to
        a / (r - 1) (r^|k - c| - 1); texel i sits at k = i + 0.5 because the
        unnormalized linear filter samples texel centres (rs.cl:8)."""
        def axis(n, a, r, centred):
            k = np.arange(n, dtype=np.float64) + 0.5
            a, r = float(a), float(r)
            if centred:
                c = 0.5 * (n - 1)
                return np.sign(k - c) * a / (r - 1.0) * (r ** np.abs(k - c) - 1.0)
            return a / (r - 1.0) * (r ** k - 1.0)
        return (axis(self.nx, self.ax, self.rx, True), axis(self.ny, self.ay, self.ry, True),
                axis(self.nz, self.az, self.rz, False))

    def half_width(self):
        """Usable half width / height of the domain (rs.c:5812-5815)."""
        w = F(self.ax * F(1.0 - F(float(self.rx)) ** F(0.5 * (self.nx - 3))) / F(1.0 - self.rx))
        h = F(self.az * F(1.0 - F(float(self.rz)) ** F(self.nz - 1)) / F(1.0 - self.rz))
        return float(w), float(h)


def les_volumes(cfg=None, count=10, seed=1, vmax=50.0, core=100.0, sigma=3.0, inflow=0.02):
    """Burgers-Rott vortex plus Gaussian turbulence on the stretched grid."""
    cfg = cfg or LESConfig()
    x, y, z = cfg.node_positions()
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    rho = np.sqrt(X * X + Y * Y)
    alpha = 1.25643
    rho_s = np.maximum(rho, 1e-6)
    vt = vmax * (1.0 + 1.0 / (2.0 * alpha)) * (core / rho_s) * (1.0 - np.exp(-alpha * rho_s ** 2 / core ** 2))
    ur = -inflow * rho
    cphi, sphi = X / rho_s, Y / rho_s
    u0 = -vt * sphi + ur * cphi
    v0 = vt * cphi + ur * sphi
    w0 = np.minimum(2.0 * inflow * Z, 15.0) * np.exp(-(rho / (3.0 * core)) ** 2)
    p0 = -1.0e3 * np.exp(-(rho / core) ** 2)
    vols = []
    rng = np.random.default_rng(seed)
    for _ in range(count):
        uvwt = np.zeros((cfg.nz, cfg.ny, cfg.nx, 4), dtype=np.float32)
        uvwt[..., 0] = u0 + sigma * rng.standard_normal(u0.shape)
        uvwt[..., 1] = v0 + sigma * rng.standard_normal(u0.shape)
        uvwt[..., 2] = w0 + sigma * rng.standard_normal(u0.shape)
        cpxx = np.zeros_like(uvwt)
        cpxx[..., 1] = p0
        vols.append(LESVolume(uvwt, cpxx))
    return cfg, vols


LES_SCALES = {"suctvort": (100.0, 1.0e4, 1.0e4), "suctvort_large": (100.0, 1.0e4, 1.0e4),
              "twocell": (225.0, 225.0 ** 2, 225.0 ** 2), "flat": (100.0, 1.0, 1.0e4)}


def write_les_folder(directory, cfg, vols, config="suctvort", volumes_per_file=10, node_km=None):
    """Write volumes in the files les.c reads (an LES folder): fort.10_2 with
    the node coordinates (km) and LES_mean_1_6_fnum<k>.dat with
    `volumes_per_file` volumes each, u v w p t divided by the configuration's
    scales (les.c:158-208), Fortran record markers around every field.  The
    synthetic stand-in for the LES tables the reference downloads."""
    os.makedirs(directory, exist_ok=True)
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    nn = nx * ny * nz
    if node_km is None:
        x, y, z = cfg.node_positions()
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        node_km = (X * 1e-3, Y * 1e-3, Z * 1e-3)

    def marker(n):
        return np.array([n], np.uint32).tobytes()

    with open(os.path.join(directory, "fort.10_2"), "wb") as f:
        f.write(marker(12) + np.array([nx, ny, nz], np.uint32).tobytes() + marker(12))
        for a in node_km:
            f.write(marker(4 * nn) + np.ascontiguousarray(a, np.float32).tobytes() + marker(4 * nn))
    v0, p0, t0 = LES_SCALES.get(config.lower(), (100.0, 1.0e4, 1.0e4))
    cn2 = config == "flat"
    for first in range(0, len(vols), volumes_per_file):
        path = os.path.join(directory, "LES_mean_1_6_fnum%d.dat" % (first // volumes_per_file + 1))
        with open(path, "wb") as f:
            f.write(marker(4))
            for k, vol in enumerate(vols[first:first + volumes_per_file]):
                t = np.float32((first + k) * float(cfg.tp))
                planes = [vol.uvwt[..., 0] / v0, vol.uvwt[..., 1] / v0, vol.uvwt[..., 2] / v0,
                          (vol.cpxx[..., 0] if cn2 else vol.cpxx[..., 1]) / p0, vol.uvwt[..., 3] / t0]
                f.write(t.tobytes() + marker(4) + marker(4 * nn))
                for j, a in enumerate(planes):
                    last = j == len(planes) - 1
                    f.write(np.ascontiguousarray(a, np.float32).tobytes() + marker(4 * nn) +
                            marker(4 if last else 4 * nn))


# ------------------------------------------- tables identical on every host
# The files below are made with integer hashing and the correctly rounded
# IEEE operations (+, -, *, /, sqrt) only -- no libm transcendental -- so the
# same call writes the same bytes on x86-64 and aarch64.  A session of the
# reference host recorded on one machine can then be replayed against its
# tables on another.

_SM_A = np.uint64(0x9E3779B97F4A7C15)
_SM_B = np.uint64(0xBF58476D1CE4E5B9)
_SM_C = np.uint64(0x94D049BB133111EB)


def hash_uniform(seed, n):
    """n float32 in [0, 1): splitmix64 of (seed << 32) + i, the top 24 bits
    times 2^-24 (exact in single precision)."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) << np.uint64(32)) + np.arange(n, dtype=np.uint64) + _SM_A
        z = (z ^ (z >> np.uint64(30))) * _SM_B
        z = (z ^ (z >> np.uint64(27))) * _SM_C
        z = z ^ (z >> np.uint64(31))
    return ((z >> np.uint64(40)).astype(np.float64) * 2.0 ** -24).astype(np.float32)


def _powers(r, k):
    """r ** k for integer k >= 0 by repeated multiplication (float64)."""
    out = np.ones(len(k), dtype=np.float64)
    p = 1.0
    table = [1.0]
    for _ in range(int(k.max()) if len(k) else 0):
        p = p * r
        table.append(p)
    for i, kk in enumerate(k):
        out[i] = table[int(kk)]
    return out


def exact_node_km(cfg):
    """Node coordinates (km) of the stretched grid, texel centres as in
    LESConfig.node_positions, formed without transcendental functions
    (half-integer powers as sqrt(r) times integer powers)."""
    def axis(n, a, r, centred):
        a, r = float(a), float(r)
        sr = math.sqrt(r)
        if centred:
            # k - c = i + 1 - n / 2 for even n, i + 1/2 - (n - 1) / 2 for odd n
            d2 = 2 * np.arange(n) + 1 - n          # 2 (k - c), an integer
            mag = np.abs(d2)
            whole = _powers(r, mag // 2)
            pw = np.where(mag % 2 == 1, whole * sr, whole)
            return np.sign(d2) * (a / (r - 1.0)) * (pw - 1.0)
        k2 = 2 * np.arange(n) + 1                   # 2 k for k = i + 1/2
        whole = _powers(r, k2 // 2)
        pw = np.where(k2 % 2 == 1, whole * sr, whole)
        return (a / (r - 1.0)) * (pw - 1.0)
    x = axis(cfg.nx, cfg.ax, cfg.rx, True)
    y = axis(cfg.ny, cfg.ay, cfg.ry, True)
    z = axis(cfg.nz, cfg.az, cfg.rz, False)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return X * 1e-3, Y * 1e-3, Z * 1e-3


def exact_les_volumes(cfg=None, count=2, seed=11, vmax=50.0, core=100.0, sigma=3.0):
    """LES volumes identical on every host: a Scully vortex (tangential speed
    2 vmax core rho / (rho^2 + core^2), peak vmax at rho = core, a rational
    function of the node position) with a weak updraft, plus uniform noise of
    standard deviation sigma from hash_uniform, per volume."""
    cfg = cfg or LESConfig()
    X, Y, Z = (a * 1e3 for a in exact_node_km(cfg))
    rho2 = X * X + Y * Y
    k = 2.0 * vmax * core / (rho2 + core * core)
    u0 = -k * Y
    v0 = k * X
    w0 = 0.05 * Z * core * core / (rho2 + core * core)
    p0 = -1.0e3 * core * core / (rho2 + core * core)
    n = cfg.nx * cfg.ny * cfg.nz
    amp = sigma * math.sqrt(12.0)
    vols = []
    for v in range(count):
        uvwt = np.zeros((cfg.nz, cfg.ny, cfg.nx, 4), dtype=np.float32)
        for c, base in enumerate((u0, v0, w0)):
            noise = (hash_uniform(seed * 1000 + 10 * v + c, n).astype(np.float64) - 0.5) * amp
            uvwt[..., c] = base + noise.reshape(base.shape)
        uvwt[..., 3] = (hash_uniform(seed * 1000 + 10 * v + 3, n).astype(np.float64) * 2.0 + 290.0).reshape(u0.shape)
        cpxx = np.zeros_like(uvwt)
        cpxx[..., 1] = p0
        vols.append(LESVolume(uvwt, cpxx))
    return cfg, vols


def write_adm_file(path, cd, cm):
    """An ADM table file as adm.c reads it (adm.c:168-209): uint16 nb, na,
    then cdx, cdy, cdz, cmx, cmy, cmz, na x nb floats each (beta fastest).
    cd, cm: (na, nb, 4) float32 images."""
    na, nb = cd.shape[:2]
    with open(path, "wb") as f:
        f.write(np.array([nb, na], np.uint16).tobytes())
        for img in (cd, cm):
            for c in range(3):
                f.write(np.ascontiguousarray(img[..., c], np.float32).tobytes())


def write_rcs_file(path, re, im):
    """An RCS table file as rcs.c reads it (rcs.c:197-239): uint16 na, nb,
    then hh, vv, hv real parts and hh, vv, hv imaginary parts, nb x na floats
    each (alpha fastest).  re, im: (nb, na, 4) float32 images with lanes
    (hh, vv, hv, 0)."""
    nb, na = re.shape[:2]
    with open(path, "wb") as f:
        f.write(np.array([na, nb], np.uint16).tobytes())
        for img in (re, im):
            for c in range(3):
                f.write(np.ascontiguousarray(img[..., c], np.float32).tobytes())


ADM_FILES = ("plate", "square_plate")                    # adm.h: ADMConfig*
RCS_FILES = ("leaf", "plate", "brick", "woodboard")      # rcs.h: RCSConfig* used by obj.c


def exact_adm_images(seed, nb=37, na=19):
    """(cd, cm) images (na, nb, 4), identical on every host: smooth drag
    coefficients (a quadratic of the table position) plus hashed noise."""
    a = np.arange(na, dtype=np.float64)[:, None] / (na - 1)
    b = np.arange(nb, dtype=np.float64)[None, :] / (nb - 1)
    cd = np.zeros((na, nb, 4), np.float32)
    cm = np.zeros((na, nb, 4), np.float32)
    for c in range(3):
        h = hash_uniform(seed * 100 + c, na * nb).astype(np.float64).reshape(na, nb)
        cd[..., c] = (0.6 - (0.5 * c + 1.0) * (a - 0.5) * (b - 0.5)) + 0.2 * (h - 0.5)
        h = hash_uniform(seed * 100 + 10 + c, na * nb).astype(np.float64).reshape(na, nb)
        cm[..., c] = 0.2 * (a - 0.5) * (b - 0.5) * (c + 1.0) + 0.05 * (h - 0.5)
    return cd, cm


def exact_rcs_images(seed, na=37, nb=19, level=1.0e-3):
    """(real, imag) images (nb, na, 4) with lanes (hh, vv, hv, 0), identical
    on every host: hashed values of magnitude ~level (hv a fifth of it)."""
    re = np.zeros((nb, na, 4), np.float32)
    im = np.zeros((nb, na, 4), np.float32)
    for c in range(3):
        s = 0.2 if c == 2 else 1.0
        re[..., c] = (level * s * (hash_uniform(seed * 100 + c, na * nb).astype(np.float64) * 2.0 - 1.0)).reshape(nb, na)
        im[..., c] = (level * s * (hash_uniform(seed * 100 + 10 + c, na * nb).astype(np.float64) * 2.0 - 1.0)).reshape(nb, na)
    return re, im


def write_tables_folder(root, les_cfg=None, les_vols=None, les_config="suctvort", volumes_per_file=10,
                        adm_dims=(37, 19), rcs_dims=(37, 19), seed=7):
    """The reference's tables folder (what it finds at ~/Documents/tables,
    les.c:71-126, adm.c:56-110, rcs.c:93-145): les/<config>/ with the grid and
    frame files, adm/<name>.adm and rcs/<name>.rcs for every table obj.c
    names.  All content is identical on every host (exact_* generators)."""
    if les_vols is None:
        les_cfg, les_vols = exact_les_volumes(les_cfg, count=2, seed=seed)
    write_les_folder(os.path.join(root, "les", les_config), les_cfg, les_vols, config=les_config,
                     volumes_per_file=volumes_per_file, node_km=exact_node_km(les_cfg))
    os.makedirs(os.path.join(root, "adm"), exist_ok=True)
    os.makedirs(os.path.join(root, "rcs"), exist_ok=True)
    for t, name in enumerate(ADM_FILES):
        cd, cm = exact_adm_images(seed + 10 + t, *adm_dims)
        write_adm_file(os.path.join(root, "adm", name + ".adm"), cd, cm)
    for t, name in enumerate(RCS_FILES):
        re, im = exact_rcs_images(seed + 20 + t, *rcs_dims)
        write_rcs_file(os.path.join(root, "rcs", name + ".rcs"), re, im)
    return les_cfg, les_vols


# ---------------------------------------------------------------- debris tables
OBJ_LEAF, OBJ_WOODBOARD_2X4, OBJ_BRICK = 1, 3, 6
# dimensions (m) and density (kg m^-3) per object (obj.c:102-148)
OBJ_DIMS = {
    OBJ_LEAF: (0.002, 0.04, 0.04, 1120.0),
    2: (0.001, 0.08, 0.06, 350.0),
    OBJ_WOODBOARD_2X4: (0.0508, 0.3048, 0.1016, 500.0),
    4: (0.1016, 0.3048, 0.2032, 500.0),
    5: (0.001, 1.0, 1.0, 7850.0),
    OBJ_BRICK: (0.065, 0.215, 0.1125, 2200.0),
}


def adm_properties(x, y, z, rho):
    """ADM_compute_properties (adm.c:279-304), single precision."""
    x, y, z, rho = F(x), F(y), F(z), F(rho)
    g, v0, rho_air = F(9.8), F(100.0), F(1.21)
    mass = x * y * z * rho
    ix = (y * y + z * z) * mass / F(12.0)
    iy = (x * x + z * z) * mass / F(12.0)
    iz = (x * x + y * y) * mass / F(12.0)
    Ta = rho_air * (y * z * v0 * v0) / (F(2.0) * mass * g)
    inv_x = (mass * x) / (ix * g * g)
    inv_y = (mass * y) / (iy * g * g)
    inv_z = (mass * z) / (iz * g * g)
    Ta = Ta * (g / (v0 * v0))
    return F(Ta), F(inv_x), F(inv_y), F(inv_z)


def adm_table(obj, seed, nb=181, na=91):
    """Synthetic ADM (cd, cm) images (ny = na alpha rows, nx = nb beta columns)
    and the descriptor of RS_set_adm_data_to_ADM_table / RS_set_adm_data."""
    rng = np.random.default_rng(seed)
    beta = np.linspace(-np.pi, np.pi, nb)
    alpha = np.linspace(0.0, np.pi, na)
    A, B = np.meshgrid(alpha, beta, indexing="ij")
    cd = np.zeros((na, nb, 4), dtype=np.float32)
    cm = np.zeros((na, nb, 4), dtype=np.float32)
    for c in range(3):
        a = rng.uniform(-1.0, 1.0, size=(3, 3))
        acc = np.zeros_like(A)
        for m in range(3):
            for n in range(3):
                acc += a[m, n] * np.cos(m * A + 0.3 * c) * np.cos(n * B + 0.7 * c)
        cd[..., c] = 0.5 * acc
        b = rng.uniform(-1.0, 1.0, size=(3, 3))
        acc = np.zeros_like(A)
        for m in range(3):
            for n in range(3):
                acc += b[m, n] * np.sin((m + 1) * A) * np.sin(n * B + 0.5 * c)
        cm[..., c] = 0.1 * acc
    desc = np.zeros(16, dtype=np.float32)
    xs = F((nb - 1) / (2.0 * math.pi))
    ys = F((na - 1) / math.pi)
    desc[0], desc[1] = xs, ys
    desc[4] = F(math.pi * float(xs) + 0.5)
    desc[5] = F(0.5)
    desc[8], desc[9] = F(nb - 1), F(na - 1)
    Ta, ix, iy, iz = adm_properties(*OBJ_DIMS[obj])
    desc[12], desc[13], desc[14], desc[15] = ix, iy, iz, Ta
    return cd, cm, desc


def rcs_table(seed, na=181, nb=91, level=1.0e-3):
    """Synthetic RCS (real, imag) images (ny = nb beta rows, nx = na alpha
    columns): log-normal magnitude, uniform phase, 3x3 smoothed; descriptor of
    RS_set_rcs_data_to_RCS_table / RS_set_rcs_data (no half-texel offset)."""
    rng = np.random.default_rng(seed)
    re = np.zeros((nb, na, 4), dtype=np.float32)
    im = np.zeros((nb, na, 4), dtype=np.float32)
    for c in range(3):
        mag = level * np.exp(0.5 * rng.standard_normal((nb, na))) * (0.2 if c == 2 else 1.0)
        ph = rng.uniform(-np.pi, np.pi, (nb, na))
        z = mag * np.exp(1j * ph)
        k = np.ones((3, 3)) / 9.0
        zp = np.pad(z, 1, mode="edge")
        zs = sum(k[i, j] * zp[i:i + nb, j:j + na] for i in range(3) for j in range(3))
        re[..., c] = zs.real
        im[..., c] = zs.imag
    desc = np.zeros(16, dtype=np.float32)
    xs = F((na - 1) / (2.0 * math.pi))
    desc[0] = xs
    desc[1] = F((nb - 1) / math.pi)
    desc[4] = F(math.pi * float(xs))
    desc[5] = F(0.0)
    desc[8], desc[9] = F(na - 1), F(nb - 1)
    return re, im, desc


# ---------------------------------------------------------------- radar tables
def range_weight_triangle(dr, user=0.0):
    """RS_set_range_weight_to_triangle (rs.c:2620-2623) via RS_set_range_weight."""
    dr = F(dr)
    dx = F(F(1.0) / dr)
    x0 = F(-(-dr) * dx)
    return np.array([0.0, 1.0, 0.0], dtype=np.float32), np.array([dx, x0, F(2.0), F(user)], dtype=np.float32)


def angular_weight_standard(beamwidth_deg):
    """RS_set_angular_weight_to_standard (rs.c:2826-2852): 32 samples of
    8 J2(c) / c^2 at 0.5 degree steps."""
    from scipy.special import jv
    bw_rad = F(float(F(F(beamwidth_deg) / F(180.0))) * math.pi)   # RS_update_computed_properties
    n = 32
    b = F(float(F(1.27)) * math.pi / float(bw_rad))
    delta = F(float(F(F(1.0) / F(360.0))) * math.pi)
    w = np.zeros(n, dtype=np.float32)
    for i in range(n):
        a = F(F(i) * delta)
        c = F(b * np.sin(a, dtype=np.float32))
        if i == 0:
            w[i] = 1.0
        elif i == n - 1:
            w[i] = 0.0
        else:
            w[i] = F(8.0 * jv(2, float(c)) / float(F(c * c)))
    dx = F(F(1.0) / delta)
    x0 = F(-F(0.0) * dx)
    return w, np.array([dx, x0, F(n - 1), F(0.0)], dtype=np.float32)


def ellipsoid_rcs_table(wave_number, drop_scale, concept=CONCEPT_DBU, dsd_r=None, dsd_pdf=None):
    """RS_compute_rcs_ellipsoids (rs.c:5922-6030): 96 drop sizes, FP64, rounded
    once; with concept U only the DSD bins are kept, scaled by sqrt(pdf / p)."""
    k0 = float(F(wave_number)) * 0.5
    eps0 = float(F(8.85418782e-12))
    er = np.array([78.669, 18.2257, 78.669, 18.2257])
    sc = k0 * k0 / (4.0 * float(F(1.0)) * math.pi * eps0) * float(F(1.0e-9)) * float(F(drop_scale))
    n = 96
    table = np.zeros((n, 4), dtype=np.float32)
    if not (concept & CONCEPT_TRANSPARENT):
        for i in range(n):
            d = 0.5 + i * 0.1
            d2, d3 = d * d, d * d * d
            d4 = d3 * d
            rba = 1.0048 + (0.0057e-1 * d) - (2.628e-2 * d2) + (3.682e-3 * d3) - (1.677e-4 * d4)
            rab = float(F(1.0)) / rba
            fsq = rab * rab - 1.0
            f = math.sqrt(fsq)
            lz = (1.0 + fsq) / fsq * (1.0 - math.atan(f) / f)
            lx = (1.0 - lz) * 0.5
            vol = math.pi * d3 / 6.0
            num = complex(vol * eps0, 0.0)
            nh = num * complex(er[0], er[1])
            nv = num * complex(er[2], er[3])
            dh = complex(lx * er[0] + 1.0, lx * er[1])
            dv = complex(lz * er[2] + 1.0, lz * er[3])
            ah, av = nh / dh, nv / dv
            table[i] = [sc * ah.real, sc * ah.imag, sc * av.real, sc * av.imag]
        if concept & CONCEPT_UNIFORM_DSD and dsd_r is not None:
            p = F(1.0) / F(len(dsd_r))
            copy = table.copy()
            table[:] = 0.0
            for r, pdf in zip(dsd_r, dsd_pdf):
                k = int(F(F(r) * F(20000.0))) - 5
                s = np.sqrt(F(F(pdf) / p), dtype=np.float32)
                table[k] = copy[k] * s
    dx = F(F(1.0) / F(0.05e-3))
    x0 = F(-F(0.25e-3) * dx)
    return table, np.array([dx, x0, F(n - 1), F(drop_scale)], dtype=np.float32)


def marshall_palmer(diameters_m, n0=8000.0, lam=2300.0):
    """RS_set_dsd_to_mp_with_sizes + RS_set_dsd (rs.c:2361-2463): radii, pdf, cdf
    and the drop concentration sum."""
    ds = np.asarray(diameters_m, dtype=np.float32)
    n = np.array([F(F(n0) * F(math.exp(-float(F(lam)) * float(d)))) for d in ds], dtype=np.float32)
    tot = F(0.0)
    for v in n:
        tot = F(tot + v)
    pdf = (n / tot).astype(np.float32)
    cdf = np.zeros_like(pdf)
    lo = F(0.0)
    for i in range(len(pdf)):
        cdf[i] = lo
        lo = F(lo + pdf[i])
    return (F(0.5) * ds).astype(np.float32), pdf, cdf, float(tot)


# ---------------------------------------------------------------- scenes
class Scene:
    """Everything one emulation needs: tables, descriptors, initial state,
    population layout and the per-pulse beam / simulation descriptors."""


def beam_unit(az_deg, el_deg):
    """RS_set_beam_pos (rs.c:2076-2085)."""
    el = F(F(el_deg) / F(180.0))
    az = F(F(az_deg) / F(180.0))
    el = F(float(el) * math.pi)
    az = F(float(az) * math.pi)
    return (F(np.cos(el, dtype=np.float32) * np.sin(az, dtype=np.float32)),
            F(np.cos(el, dtype=np.float32) * np.cos(az, dtype=np.float32)),
            F(np.sin(el, dtype=np.float32)))


def ppi_positions(el, az0, az1, daz):
    """POS_parse_from_string PPI branch (pos.c:80-110): positions until the
    azimuth reaches the end within a tenth of a step."""
    out = []
    f2 = F(az0)
    while True:
        out.append((float(f2), float(el)))
        f2 = F(f2 + F(daz))
        if not (abs(out[-1][0] - float(az1)) > 0.1 * float(F(daz))) or len(out) >= 10000:
            break
    return out


def rhi_positions(az, el0, el1, delv):
    out = []
    f2 = F(el0)
    while True:
        out.append((float(az), float(f2)))
        f2 = F(f2 + F(delv))
        if not (abs(out[-1][1] - float(el1)) > 0.1 * float(F(delv))) or len(out) >= 10000:
            break
    return out


def make_scene(num_rain=131072, debris=(), gate_spacing=15.0, gates=None, range_start=None, seed=19760520,
               les_cfg=None, les_count=2, concept=CONCEPT_DBU, scan=None, lam=0.1, prt=1.0e-3, tau=0.2e-6,
               beamwidth=1.0, dsd_diameters=None, box=None, range_offset=0.0, les_seed=1, with_tables=True,
               dsd_n0=8000.0):
    """A synthetic scene with the geometry of the reference's default box:
    R 1850-2420 m, azimuth +-8 deg, elevation 0-18 deg (RS_suggest_scan_domain
    for the suctvort LES, rs.c:5850-5877).  Positions are uniform in the box;
    seeds are uniform 31-bit integers.  `debris` is a list of (obj, count).
    `range_offset` moves the box (and the LES domain, which is centred on it)
    and the gates that far along +y: the 30 km case of the precision form,
    where the two-way phase 4 pi r / lambda is ~4e6 rad and one FP32 ulp of r
    is 2 mm.  `dsd_n0` is the Marshall-Palmer intercept (m^-3 mm^-1)."""
    S = Scene()
    rng = np.random.default_rng(seed)
    c = F(3.0e8)
    dr = F(F(0.5) * c * F(tau))
    S.lam, S.prt, S.concept = F(lam), F(prt), int(concept)
    S.les_cfg, vols = les_volumes(les_cfg, count=les_count, seed=les_seed) if with_tables else (les_cfg or LESConfig(), [])
    S.les = vols
    S.les_desc = S.les_cfg.desc()
    # box
    if box is None:
        r0, r1, a0, a1, e0, e1 = 1850.0, 2420.0, -8.0, 8.0, 0.0, 18.0
        rr = np.array([r0, r1])
        aa = np.radians(np.linspace(a0, a1, 33))
        ee = np.radians(np.linspace(e0, e1, 37))
        R, A, E = np.meshgrid(rr, aa, ee, indexing="ij")
        X = R * np.cos(E) * np.sin(A)
        Y = R * np.cos(E) * np.cos(A)
        Z = R * np.sin(E)
        box = (X.min(), Y.min() + range_offset, Z.min(), X.max() - X.min(), Y.max() - Y.min(), Z.max() - Z.min())
    S.box = tuple(float(F(v)) for v in box)
    ox, oy, oz, sx, sy, sz = S.box
    if range_start is None:
        range_start = 1850.0
    if gates is None:
        gates = int(round((2420.0 - 1850.0) / gate_spacing)) + 2
    S.range_start = F(range_start + range_offset)
    S.range_delta = F(gate_spacing)
    S.range_count = int(gates)
    S.dr = dr
    # DSD
    if dsd_diameters is None:
        dsd_diameters = np.arange(1, 11) * 0.5e-3
    S.dsd_r, S.dsd_pdf, S.dsd_cdf, S.dsd_nd = marshall_palmer(dsd_diameters, n0=dsd_n0)
    # population
    counts = [int(num_rain)] + [int(n) for _, n in debris]
    S.num_scats = int(sum(counts))
    S.counts = counts
    S.debris_objs = [o for o, _ in debris]
    N = S.num_scats
    pos = np.zeros((N, 4), dtype=np.float32)
    pos[:, 0] = rng.uniform(0.0, 1.0, N) * sx + ox
    pos[:, 1] = rng.uniform(0.0, 1.0, N) * sy + oy
    pos[:, 2] = rng.uniform(0.0, 1.0, N) * sz + oz
    bins = (rng.uniform(0.0, 1.0, num_rain) * len(S.dsd_r)).astype(np.int64)
    pos[:num_rain, 3] = S.dsd_r[bins]
    aux = np.zeros((N, 4), dtype=np.float32)
    aux[:, 1] = rng.uniform(0.0, 1.0, N)
    aux[:num_rain, 2] = (bins + 0.5) / len(S.dsd_r)
    aux[:, 3] = 1.0
    ori = np.zeros((N, 4), dtype=np.float32)
    ori[:] = [0.5, -0.5, -0.5, 0.5]
    tum = np.zeros((N, 4), dtype=np.float32)
    tum[:, 3] = 1.0
    rcs = np.zeros((N, 4), dtype=np.float32)
    rcs[:] = [1.0, 0.0, 1.0, 0.0]
    rnd = rng.integers(0, 2 ** 31, size=(N, 4), dtype=np.uint32)
    S.state = dict(pos=pos, vel=np.zeros((N, 4), np.float32), ori=ori, tum=tum, aux=aux, rcs=rcs,
                   sig=np.zeros((N, 4), np.float32), rnd=rnd)
    # simulation descriptor (rs_enum.h:93-110)
    vol = F(F(sx) * F(sy) * F(sz))
    drops_per_scat = F(F(vol * F(S.dsd_nd)) / F(num_rain)) if num_rain else F(1.0)
    sd = np.zeros(16, dtype=np.float32)
    sd[0], sd[1], sd[2] = beam_unit(0.0, 3.0)
    sd[3] = F(N)
    sd[4] = F(4.0 * math.pi / float(S.lam))
    sd[5] = fbits(S.concept)
    sd[6] = F(math.sqrt(float(drops_per_scat)))
    sd[8], sd[9], sd[10] = ox, oy, oz
    sd[11] = S.prt
    sd[12], sd[13], sd[14] = sx, sy, sz
    S.sim_desc = sd
    # radar tables
    S.range_w, S.range_desc = range_weight_triangle(dr, user=sd[4])
    S.ang_w, S.ang_desc = angular_weight_standard(beamwidth)
    S.ell, S.ell_desc = ellipsoid_rcs_table(sd[4], sd[6], S.concept, S.dsd_r, S.dsd_pdf)
    S.gain = F(float(F(F(10.0) ** F(F(0.1) * F(44.5))) * F(np.sqrt(F(50.0e3)))) / (4.0 * math.pi) * 1.0e6)
    # debris tables: type k uses ADM / RCS table k - 1
    S.adm, S.rcs_tables = [], []
    for t, obj in enumerate(S.debris_objs):
        S.adm.append(adm_table(obj, seed=100 + t))
        S.rcs_tables.append(rcs_table(seed=200 + t))
    # scan
    if scan is None:
        scan = ppi_positions(3.0, -12.0, 12.0, 0.24)
    S.scan = scan
    return S


def population(S):
    from .rsc import Population
    return Population.make(S.counts)


def pulse_sim_desc(S, k, tic=0.0):
    """sim_desc for pulse k of the scan (beam from the scan position)."""
    az, el = S.scan[k % len(S.scan)]
    sd = S.sim_desc.copy()
    sd[0], sd[1], sd[2] = beam_unit(az, el)
    sd[7] = F(tic)
    return sd


def load_worker(W, S, les_slot_volumes=(0, 1)):
    """Upload the scene's tables and state to a backend worker."""
    W.malloc(S.num_scats, S.range_start, S.range_delta, S.range_count)
    W.set_range_weight(S.range_w, S.range_desc)
    W.set_angular_weight(S.ang_w, S.ang_desc)
    W.set_rcs_ellipsoid(S.ell, S.ell_desc)
    for slot, v in enumerate(les_slot_volumes):
        if v < len(S.les):
            W.set_les(slot, S.les[v].uvwt, S.les[v].cpxx, S.les_desc)
    for t, (cd, cm, ad) in enumerate(S.adm):
        W.set_adm(t, cd, cm, ad)
    for t, (re, im, rd) in enumerate(S.rcs_tables):
        W.set_rcs(t, re, im, rd)
    W.upload(0, **S.state)


def batch_workload(count=64, seed=2024, gates=40):
    """The batching workload: `count` instances with scatterer counts
    log-uniform in [65,536, 4,194,304], 0-4096 debris of each of leaf, 2x4
    board and brick, Marshall-Palmer N0 uniform in [4000, 16000], PPI (even
    instances) and RHI (odd) scans, one LES volume shared by all."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(65536), math.log(4194304), count)).astype(np.int64)
    deb = rng.integers(0, 4097, size=(count, 3))
    n0 = rng.uniform(4000.0, 16000.0, count)
    base = make_scene(num_rain=1, les_count=1, with_tables=True)
    scenes = []
    for i in range(count):
        if i % 2 == 0:
            scan = ppi_positions(float(rng.uniform(1.0, 6.0)), -12.0, 12.0, 0.24)
        else:
            scan = rhi_positions(float(rng.uniform(-6.0, 6.0)), 0.5, 20.0, 0.2)
        debris = [(o, int(c)) for o, c in zip((OBJ_LEAF, OBJ_WOODBOARD_2X4, OBJ_BRICK), deb[i]) if c > 0]
        S = make_scene(num_rain=int(sizes[i]), debris=debris, gates=gates, les_count=1, with_tables=False,
                       seed=1000 + i, scan=scan, dsd_n0=float(n0[i]))
        S.les, S.les_cfg, S.les_desc = base.les, base.les_cfg, base.les_desc
        scenes.append(S)
    return scenes
