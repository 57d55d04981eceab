"""The allocation-free DD(r) cross-correlation entry point (cf_gpu_countpairs_cross_noalloc),
called through the C ABI on device-resident catalogues, against countpairs() on the same
inputs.  Named so that it is collected last: it must pass on its own and after every other test
has used the library on this device."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_EDGES = 128
RTOL_AVG = 1e-6


def _noalloc(lib, torch, s1, s2, bins, periodic, boxsize, isa, weights, ravg=True):
    from corrfunc_gb300 import _capi as C
    dev = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda() for a in s1[:3] + s2[:3]]
    w = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda() for a in (s1[3], s2[3])] \
        if weights else [None, None]
    torch.cuda.synchronize()
    n = len(bins)
    edges = np.ascontiguousarray(bins, dtype=np.float64)
    npairs = np.zeros(n, dtype=np.uint64)
    avg = np.zeros(n)
    wavg = np.zeros(n)
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    rc = lib.cf_gpu_countpairs_cross_noalloc(
        len(s1[0]), p(dev[0]), p(dev[1]), p(dev[2]), p(w[0]),
        len(s2[0]), p(dev[3]), p(dev[4]), p(dev[5]), p(w[1]),
        n, edges.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(periodic),
        *(float(b) for b in np.broadcast_to(np.asarray(boxsize, dtype=float), (3,))), C.translate_isa(isa),
        npairs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
        avg.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if ravg else None,
        wavg.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    return rc, npairs, avg, wavg


def _catalogue(seed, n, boxsize):
    rng = np.random.default_rng(seed)
    x, y, z = (rng.random(n) * boxsize for _ in range(3))
    # a few exact duplicates across the two sets and points on the box faces
    x[:5] = 0.0
    w = rng.uniform(0.5, 1.5, n)
    return [x, y, z, w]


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import corrfunc_gb300
    return corrfunc_gb300.library(), torch


@pytest.mark.parametrize("periodic,isa,weights", [(True, "fallback", True), (False, "avx512f", False),
                                                  (True, "avx512f", True)])
def test_noalloc_matches_countpairs_twice_in_a_row(env, periodic, isa, weights):
    from corrfunc_gb300 import theory
    lib, torch = env
    L = 60.0
    s1 = _catalogue(11, 3000, L)
    s2 = _catalogue(12, 2500, L)
    s2[0][:50], s2[1][:50], s2[2][:50] = s1[0][:50], s1[1][:50], s1[2][:50]  # zero separations
    bins = np.array([0.0, 0.7, 1.5, 3.0, 6.0, 9.0, 12.5])
    kw = dict(X2=s2[0], Y2=s2[1], Z2=s2[2], periodic=periodic, boxsize=L, output_ravg=True, isa=isa)
    if weights:
        kw.update(weights1=s1[3], weights2=s2[3], weight_type="pair_product")
    want = theory.DD(0, 1, bins, s1[0], s1[1], s1[2], **kw)
    runs = []
    for _ in range(2):
        rc, npairs, avg, wavg = _noalloc(lib, torch, s1, s2, bins, periodic, L, isa, weights)
        runs.append((npairs, avg, wavg))
        assert rc == 0
        # the C arrays carry one entry per edge (entry 0 stays empty); the Python rows start at
        # the first [edges[0], edges[1]) bin
        assert npairs[0] == 0 and avg[0] == 0.0 and wavg[0] == 0.0
        assert np.array_equal(npairs[1:], want["npairs"])
        assert npairs.sum() > 0
        # countpairs() sums separations of its FP32 fast path: averages agree to 1e-6
        np.testing.assert_allclose(avg[1:], want["ravg"], rtol=RTOL_AVG, atol=1e-12)
        if weights:
            np.testing.assert_allclose(wavg[1:], want["weightavg"], rtol=RTOL_AVG, atol=1e-12)
        else:
            assert not wavg.any()
    # the two calls in a row agree with each other up to the order of the FP64 additions
    assert np.array_equal(runs[0][0], runs[1][0])
    np.testing.assert_allclose(runs[0][1], runs[1][1], rtol=1e-12, atol=0)
    np.testing.assert_allclose(runs[0][2], runs[1][2], rtol=1e-12, atol=0)


def test_noalloc_rejects_too_many_edges_and_bad_arguments(env):
    lib, torch = env
    s1 = _catalogue(3, 100, 50.0)
    s2 = _catalogue(4, 100, 50.0)
    bins = np.linspace(0.0, 5.0, MAX_EDGES + 1)
    rc, npairs, _, _ = _noalloc(lib, torch, s1, s2, bins, True, 50.0, "fallback", False)
    assert rc != 0 and not npairs.any()
    rc, _, _, _ = _noalloc(lib, torch, s1, s2, np.linspace(0.0, 5.0, MAX_EDGES), True, 50.0, "fallback", False)
    assert rc == 0
    # rmax too large for minimum-image wrapping
    rc, _, _, _ = _noalloc(lib, torch, s1, s2, np.array([0.0, 10.0, 24.6]), True, 50.0, "fallback", False)
    assert rc != 0
    # non-increasing edges
    rc, _, _, _ = _noalloc(lib, torch, s1, s2, np.array([0.0, 2.0, 2.0]), True, 50.0, "fallback", False)
    assert rc != 0
    # periodic wrapping needs a positive box size on every axis (no per-axis "no wrap" value)
    for box in ((50.0, -1.0, 50.0), (50.0, 50.0, 0.0)):
        rc, _, _, _ = _noalloc(lib, torch, s1, s2, np.array([0.0, 1.0, 2.0]), True, box, "fallback", False)
        assert rc != 0


def test_noalloc_empty_sets(env):
    lib, torch = env
    s1 = _catalogue(5, 64, 20.0)
    empty = [np.zeros(0) for _ in range(4)]
    rc, npairs, avg, _ = _noalloc(lib, torch, s1, empty, np.array([0.0, 1.0, 2.0]), False, 20.0, "fallback", False)
    assert rc == 0 and not npairs.any() and not avg.any()
