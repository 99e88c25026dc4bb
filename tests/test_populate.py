"""RS_populate's initial state (rs.c:4568-4814): the backend's glibc rand()
against the C library's own, and the draws in RS_populate's order against a
restatement here using the C library's rand() itself.  CPU only (glibc)."""
import ctypes
import ctypes.util
import platform

import numpy as np
import pytest

from simradar_gb300 import rsc, synth

F = np.float32


def libc():
    if platform.system() != "Linux":
        pytest.skip("glibc needed")
    name = ctypes.util.find_library("c") or "libc.so.6"
    L = ctypes.CDLL(name)
    L.srand.argtypes = [ctypes.c_uint]
    L.rand.restype = ctypes.c_int
    return L


@pytest.mark.parametrize("seed", [19760520, 0, 1, 12345, 2**31 + 5, 2**32 - 1])
def test_rand_matches_glibc(backend, seed):
    L = libc()
    L.srand(seed)
    want = np.array([L.rand() for _ in range(5000)], dtype=np.int32)
    got = rsc.rand_sequence(seed, 5000)
    assert np.array_equal(got, want)


def reference_populate(L, seed, concept, origin, size, counts, dsd_r, dsd_cdf):
    """RS_populate's draw order with the C library's rand()."""
    n = sum(counts)
    pos = np.zeros((n, 4), np.float32)
    aux = np.zeros((n, 4), np.float32)
    rnd = np.zeros((n, 4), np.uint32)
    L.srand(seed)
    rmax = F(2147483647)

    def unit():
        return F(F(L.rand()) / rmax)
    i = 0
    for c in counts:
        for _ in range(c):
            pos[i, 0] = F(F(unit() * F(size[0])) + F(origin[0]))
            pos[i, 1] = F(F(unit() * F(size[1])) + F(origin[1]))
            pos[i, 2] = F(F(unit() * F(10.0)) + F(origin[2]))
            aux[i] = [0.0, unit(), 0.0, 1.0]
            rnd[i] = [L.rand() for _ in range(4)]
            i += 1
    L.srand((seed + seed) & 0xFFFFFFFF)
    nb = len(dsd_r)
    for i in range(counts[0]):
        a = unit()
        if concept & 0x10:
            b = int(F(a * F(nb)))
        else:
            b = 0
            for k in range(nb - 1, -1, -1):
                if a >= dsd_cdf[k]:
                    b = k
                    break
        pos[i, 3] = dsd_r[b]
        aux[i, 2] = F(F(F(b) + F(0.5)) / F(nb))
    return pos, aux, rnd


@pytest.mark.parametrize("concept", [synth.CONCEPT_DBU, synth.CONCEPT_DRAGGED])
def test_populate_matches_reference_order(backend, concept):
    L = libc()
    seed = 19760520
    origin, size = (-337.0, 1742.0, 0.0), (674.0, 678.0, 748.0)
    counts = [3000, 200, 100]
    r, pdf, cdf, nd = synth.marshall_palmer(np.arange(1, 11) * 0.5e-3)
    args = rsc.PopulateArgs.make(seed, concept, origin, size, counts, r, cdf)
    got, pop = rsc.populate_host(args, 3400)
    pos, aux, rnd = reference_populate(L, seed, concept, origin, size, counts, r, cdf)
    n = sum(counts)
    assert np.array_equal(got["pos"][:n].view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(got["aux"][:n].view(np.uint32), aux.view(np.uint32))
    assert np.array_equal(got["rnd"][:n], rnd)
    assert np.all(got["pos"][n:] == 0) and np.all(got["ori"][n:] == 0)
    assert np.all(got["ori"][:n] == [0.5, -0.5, -0.5, 0.5]) and np.all(got["tum"][:n] == [0, 0, 0, 1])
    assert np.all(got["rcs"][:n] == [1, 0, 1, 0]) and np.all(got["vel"] == 0)
    assert pop.sum() == counts[0]


def test_populate_rejects_fixed_positions(backend):
    args = rsc.PopulateArgs.make(1, synth.CONCEPT_FIXED_POS, (0, 0, 0), (1, 1, 1), [10])
    with pytest.raises(rsc.BackendError):
        rsc.populate_host(args, 10)
