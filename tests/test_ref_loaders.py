"""The inputs of the emulation loop against the reference's own C code.

les.c, pos.c, adm.c, rcs.c, obj.c and rs.c are compiled unmodified from the
reference tree into oracle/_ref/libref.so (oracle/ref/Makefile), and their
results are compared with what this build reads, derives or restates:

  LES frames       les.c LES_get_frame        vs rsc_les_read (the backend's reader)
  LES descriptor   rs.c RS_set_vel_data_*     vs rsc_les_descriptor, synth.LESConfig.desc
  scan positions   pos.c POS_get_next_angles  vs synth.ppi_positions / rhi_positions
  ADM / RCS files  adm.c / rcs.c readers      vs the arrays synth writes
  debris physics   obj.c + adm.c constants    vs synth.adm_properties

Everything is bit for bit.  These tests need the reference tree (the build
compiles it where it lies) and no GPU; without the tree they skip.
"""
import math
import os

import numpy as np
import pytest

from oracle import refbind
from simradar_gb300 import rsc, synth

pytestmark = pytest.mark.skipif(not refbind.available(), reason="the reference tree is not present")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def les_tables(tmp_path, config, nx=24, ny=20, nz=12, volumes=3, seed=5):
    """A tables folder (<tmp>/tables/les/<config>) of exact volumes with
    non-zero t and cn2 lanes."""
    cfg = synth.LESConfig(nx=nx, ny=ny, nz=nz)
    _, vols = synth.exact_les_volumes(cfg, count=volumes, seed=seed)
    for v in vols:
        v.cpxx[..., 0] = (synth.hash_uniform(seed + 77, nx * ny * nz).reshape(nz, ny, nx) - 14.0)
    node_km = synth.exact_node_km(cfg)
    if config == "flat":
        x = (np.arange(nx) - 0.5 * (nx - 1)) * 0.01
        y = (np.arange(ny) - 0.5 * (ny - 1)) * 0.012
        z = np.arange(nz) * 0.005
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        node_km = (X, Y, Z)
    d = tmp_path / "tables" / "les" / config
    synth.write_les_folder(str(d), cfg, vols, config=config, node_km=node_km)
    return str(tmp_path), str(d), cfg, vols


@pytest.mark.parametrize("config", ["suctvort", "flat", "twocell", "other"])
def test_les_frames_match_les_c(tmp_path, config):
    parent, d, cfg, vols = les_tables(tmp_path, config)
    with rsc.LESSource(d, config) as src:
        I = src.info
        for n in (0, 2, 1):
            u_ref, c_ref, k = refbind.les_frame(parent, config, n)
            uvwt, cpxx, t = src.read(n)
            assert np.array_equal(bits(uvwt), bits(u_ref)), (config, n)
            assert np.array_equal(bits(cpxx), bits(c_ref)), (config, n)
        # the per-configuration constants of les.c:158-208
        assert np.float32(I.tp) == np.float32(k["tp"]) and np.float32(I.tr) == np.float32(k["tr"])
        for name in ("ax", "ay", "az", "rx", "ry", "rz"):
            assert np.float32(getattr(I, name)) == np.float32(k[name]), name
        assert bool(I.is_stretched) == bool(k["is_stretched"])
        assert I.frames == int(k["frames"])


@pytest.mark.parametrize("config", ["suctvort", "flat", "twocell"])
def test_les_descriptor_matches_rs_c(tmp_path, config, monkeypatch):
    """rsc_les_descriptor against RS_set_vel_data_to_LES_table + RS_set_vel_data
    run by rs.c on the same folder (found from $HOME as rs.c finds it)."""
    home = tmp_path / "home"
    les_tables(home / "Documents", config)
    monkeypatch.setenv("HOME", str(home))
    ref = refbind.les_descriptor(config)
    with rsc.LESSource(str(home / "Documents" / "tables" / "les" / config), config) as src:
        desc = src.descriptor()
    assert np.array_equal(bits(desc), bits(ref)), (desc, ref)
    if config == "suctvort":
        assert np.array_equal(bits(synth.LESConfig(nx=24, ny=20, nz=12).desc()), bits(ref))


@pytest.mark.parametrize("scan,count", [
    ("P:3.0,-12:12:0.24", 250),          # the PPI of the README run, wrapping around
    ("P:0.5,-8:8:0.5,1.5,8:-8:0.5", 80),  # two sweeps, the second reversed
    ("R:15.0,0.5:20:0.02", 1200),         # the RHI of the large instance, repeating
])
def test_scan_positions_match_pos_c(scan, count):
    az, el = refbind.pos_angles(scan, count)
    if scan.startswith("P:3.0"):
        pos = synth.ppi_positions(3.0, -12.0, 12.0, 0.24)
    elif scan.startswith("R:"):
        pos = synth.rhi_positions(15.0, 0.5, 20.0, 0.02)
    else:
        pos = None
    if pos is not None:
        want = np.array([pos[k % len(pos)] for k in range(count)], dtype=np.float32)
        assert np.array_equal(bits(az), bits(want[:, 0])), np.nonzero(az != want[:, 0])[0][:5]
        assert np.array_equal(bits(el), bits(want[:, 1])), np.nonzero(el != want[:, 1])[0][:5]
    assert np.isfinite(az).all() and np.isfinite(el).all()


def test_adm_and_rcs_files_match_readers(tmp_path):
    root = tmp_path / "tables"
    synth.write_tables_folder(str(root), les_cfg=synth.LESConfig(nx=8, ny=8, nz=6), volumes_per_file=10,
                              adm_dims=(37, 19), rcs_dims=(41, 23))
    for t, name in enumerate(synth.ADM_FILES):
        data, phys = refbind.adm_table(str(root), name)
        cd, cm = synth.exact_adm_images(7 + 10 + t, 37, 19)
        want = np.stack([cd[..., 0], cd[..., 1], cd[..., 2], cm[..., 0], cm[..., 1], cm[..., 2]])
        assert np.array_equal(bits(data), bits(want)), name
        # the default physics adm.c gives a table before obj.c resizes it
        Ta, ix, iy, iz = synth.adm_properties(0.002, 0.040, 0.040, 1120.0)
        assert np.array_equal(bits(phys[[5, 6, 7, 8]]), bits([Ta, ix, iy, iz]))
    for t, name in enumerate(synth.RCS_FILES):
        data = refbind.rcs_table(str(root), name)
        re, im = synth.exact_rcs_images(7 + 20 + t, 41, 23)
        want = np.stack([re[..., 0], re[..., 1], re[..., 2], im[..., 0], im[..., 1], im[..., 2]])
        assert np.array_equal(bits(data), bits(want)), name


@pytest.mark.parametrize("obj", sorted(synth.OBJ_DIMS))
def test_debris_physics_matches_obj_c(tmp_path, monkeypatch, obj):
    """OBJ_get_table's dimensions, density and the ADM constants Ta and
    1 / (In Ln) (adm.c:279-304 after ADM_dimension_set) against
    synth.adm_properties, which the ADM descriptors (slots 12-15) use."""
    home = tmp_path / "home"
    synth.write_tables_folder(str(home / "Documents" / "tables"), les_cfg=synth.LESConfig(nx=8, ny=8, nz=6))
    monkeypatch.setenv("HOME", str(home))
    monkeypatch.chdir(str(home))
    phys, adm_name, rcs_name = refbind.obj_table(obj)
    x, y, z, rho = synth.OBJ_DIMS[obj]
    assert np.array_equal(bits(phys[:4]), bits([x, y, z, rho]))
    Ta, ix, iy, iz = synth.adm_properties(x, y, z, rho)
    assert np.array_equal(bits(phys[5:9]), bits([Ta, ix, iy, iz])), (phys, (Ta, ix, iy, iz))
    assert adm_name in synth.ADM_FILES and rcs_name in synth.RCS_FILES
