"""The LES frame source on the host (rsc_les_open / _read / _descriptor):
files written in les.c's format are read back within a rounding of the
volumes written, in any order with the read-ahead thread, with the
configuration's constants and grid, and fail cleanly on bad frames.  The
bit-for-bit pin against les.c and rs.c themselves (frames, constants,
descriptor) is tests/test_ref_loaders.py.  No GPU involved."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))

from simradar_gb300 import rsc, synth  # noqa: E402


def small_folder(tmp_path, config="suctvort", volumes=13, nx=12, ny=10, nz=8, seed=3):
    cfg = synth.LESConfig(nx=nx, ny=ny, nz=nz)
    node_km = None
    if config == "flat":
        x = (np.arange(nx) - 0.5 * (nx - 1)) * 0.01
        y = (np.arange(ny) - 0.5 * (ny - 1)) * 0.012
        z = np.arange(nz) * 0.005
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        node_km = (X, Y, Z)
    _, vols = synth.les_volumes(cfg, count=volumes, seed=seed)
    rng = np.random.default_rng(seed)
    for v in vols:   # non-zero t and cn2 lanes too
        v.uvwt[..., 3] = rng.uniform(280.0, 300.0, v.uvwt.shape[:3])
        v.cpxx[..., 0] = rng.uniform(-14.0, -12.0, v.uvwt.shape[:3])
    d = str(tmp_path / config)
    synth.write_les_folder(d, cfg, vols, config=config, node_km=node_km)
    return d, cfg, vols


def test_read_returns_the_volumes_written(tmp_path):
    d, cfg, vols = small_folder(tmp_path)
    with rsc.LESSource(d, "suctvort") as src:
        I = src.info
        assert (I.nx, I.ny, I.nz) == (12, 10, 8)
        assert I.files == 2 and I.volumes_per_file == 10 and I.frames == 20
        assert I.is_stretched == 1 and I.p_for_cn2 == 0
        assert (I.v0, I.p0, I.t0, I.tp, I.tr) == (100.0, 1.0e4, 1.0e4, 2.0, 50.0)
        for n in (0, 1, 9, 10, 12, 5, 0, 11):
            uvwt, cpxx, t = src.read(n)
            assert t == np.float32(n * 2.0)
            # the scaled file values come back within a rounding of the volume written
            np.testing.assert_allclose(uvwt[..., :3], vols[n].uvwt[..., :3], rtol=1e-6, atol=1e-4)
            np.testing.assert_allclose(uvwt[..., 3], vols[n].uvwt[..., 3], rtol=1e-6, atol=0)
            np.testing.assert_allclose(cpxx[..., 1], vols[n].cpxx[..., 1], rtol=1e-6, atol=1e-4)
            assert np.all(cpxx[..., 0] == 0.0) and np.all(cpxx[..., 2:] == 0.0)


def test_frames_in_any_order_with_read_ahead(tmp_path):
    d, _, _ = small_folder(tmp_path, volumes=10)
    with rsc.LESSource(d, "suctvort") as src:
        want = {n: src.read(n)[0] for n in range(10)}
    rng = np.random.default_rng(5)
    with rsc.LESSource(d, "suctvort") as src:
        for n in list(range(10)) + list(rng.integers(0, 10, 40)):
            src.prefetch(int((n + 3) % 10))
            uvwt, _, _ = src.read(int(n))
            assert np.array_equal(uvwt, want[int(n)]), n


def test_descriptor_and_grid(tmp_path):
    d, cfg, _ = small_folder(tmp_path)
    with rsc.LESSource(d, "suctvort") as src:
        desc = src.descriptor()
        assert np.array_equal(desc.view(np.uint32), cfg.desc().view(np.uint32))
        x, y, z = src.grid()
        xs, ys, zs = cfg.node_positions()
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
        for got, want in ((x, X), (y, Y), (z, Z)):
            assert np.array_equal(got.reshape(-1), np.float32(want * 1e-3).reshape(-1))


def test_flat_config_puts_p_in_lane_0(tmp_path):
    d, _, vols = small_folder(tmp_path, config="flat", volumes=3)
    with rsc.LESSource(d, "flat") as src:
        I = src.info
        assert I.is_stretched == 0 and I.p_for_cn2 == 1 and I.p0 == 1.0 and I.tp == 60.0
        x, y, z = src.grid()
        assert I.rx == np.float32(np.float32(1.0e3) * np.float32(x.reshape(-1)[1] - x.reshape(-1)[0]))
        uvwt, cpxx, _ = src.read(2)
        np.testing.assert_allclose(uvwt[..., :3], vols[2].uvwt[..., :3], rtol=1e-6, atol=1e-4)
        np.testing.assert_allclose(cpxx[..., 0], vols[2].cpxx[..., 0], rtol=1e-6, atol=0)
        assert np.all(cpxx[..., 1:] == 0.0) and np.any(cpxx[..., 0] != 0.0)
        desc = src.descriptor()
        assert desc.view(np.uint32)[7] == 0   # uniform spacing


def test_twocell_scales(tmp_path):
    d, _, vols = small_folder(tmp_path, config="twocell", volumes=2)
    with rsc.LESSource(d, "twocell") as src:
        assert (src.info.v0, src.info.p0, src.info.tp, src.info.is_stretched) == (225.0, 225.0 ** 2, 5.0, 0)
        uvwt, cpxx, _ = src.read(1)
        np.testing.assert_allclose(uvwt[..., :3], vols[1].uvwt[..., :3], rtol=1e-6, atol=1e-4)
        np.testing.assert_allclose(cpxx[..., 1], vols[1].cpxx[..., 1], rtol=1e-6, atol=1e-4)


def test_errors(tmp_path):
    with pytest.raises(rsc.BackendError, match="fort.10_2"):
        rsc.LESSource(str(tmp_path / "nowhere"), "suctvort")
    d, cfg, vols = small_folder(tmp_path, volumes=13)
    with rsc.LESSource(d, "suctvort") as src:
        first = src.read(12)[0]
    with rsc.LESSource(d, "suctvort") as src:
        # frames = 2 files x 10: the second file holds 3, so frame 15 is past its end
        with pytest.raises(rsc.BackendError, match="beyond the end"):
            src.read(15)
        with pytest.raises(rsc.BackendError, match="outside"):
            src.read(20)
        with pytest.raises(rsc.BackendError, match="outside"):
            src.prefetch(99)
        uvwt, _, _ = src.read(12)   # still usable after the failures
        assert np.array_equal(uvwt, first)
    empty = tmp_path / "gridonly"
    empty.mkdir()
    os.rename(os.path.join(d, "fort.10_2"), str(empty / "fort.10_2"))
    with pytest.raises(rsc.BackendError, match="frame files"):
        rsc.LESSource(str(empty), "suctvort")
