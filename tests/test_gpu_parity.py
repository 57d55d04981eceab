"""GPU parity: the CUDA path (through the C ABI) against the oracle, the committed golden
vectors and, where built, the reference libraries.  npairs must be bit-exact; averages within
1e-6 relative (double inputs) / 1e-4 (float inputs)."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402
from test_oracle import GOLDEN, _oracle_call, brute_numpy  # noqa: E402

pytestmark = pytest.mark.gpu

RTOL_AVG = 1e-6


@pytest.fixture(scope="module")
def gpu():
    import corrfunc_gb300
    lib = corrfunc_gb300.library()
    yield corrfunc_gb300
    lib.cf_gpu_set_precision(0)


@pytest.fixture(params=["fp32_refine", "fp64"])
def precision(request, gpu):
    gpu.set_precision(request.param)
    yield request.param
    gpu.set_precision("fp32_refine")


def _gpu_call(case, isa="fallback"):
    from corrfunc_gb300 import _capi as C
    args, kw = cases.make_inputs(case, isa=isa)
    return cases.runner(case["func"])(C.library(), *args, **kw)


def _check(func, got, want, rtol):
    assert np.array_equal(np.asarray(got["npairs"], dtype=np.uint64), np.asarray(want["npairs"], dtype=np.uint64)), \
        "npairs differ:\n%s\n%s" % (list(got["npairs"]), list(want["npairs"]))
    f = cases.AVG_FIELD[func]
    np.testing.assert_allclose(np.asarray(got[f], float), np.asarray(want[f], float), rtol=rtol, atol=1e-12)
    np.testing.assert_allclose(np.asarray(got["weightavg"], float), np.asarray(want["weightavg"], float), rtol=rtol,
                               atol=1e-12)


@pytest.mark.parametrize("isa", ["fallback", "avx512f"])
@pytest.mark.parametrize("case", cases.CASES, ids=[c["name"] for c in cases.CASES])
def test_gpu_matches_golden(gpu, precision, case, isa):
    """Every golden case in both formula families of the reference: the FALLBACK kernels' unfused
    sums and the AVX512F kernels' fused multiply-add chains (theory/DD/countpairs_kernels.c.src:
    188-190, theory/DDsmu/countpairs_s_mu_kernels.c.src:213-214)."""
    got = _gpu_call(case, isa)
    gold = GOLDEN["cases" if isa == "fallback" else "avx512f_cases"][case["name"]]
    assert [int(v) for v in got["npairs"]] == gold["npairs"]
    rtol = 1e-4 if case["dtype"] == "f4" else RTOL_AVG
    f = cases.AVG_FIELD[case["func"]]
    np.testing.assert_allclose(got[f], gold["avg"], rtol=rtol, atol=1e-12)
    np.testing.assert_allclose(got["weightavg"], gold["weightavg"], rtol=rtol, atol=1e-12)
    # wp and xi are derived from npairs x weightavg, so they inherit weightavg's relative tolerance
    # (times the (1 + xi) factor of the ratio and, for wp, the 2*pimax scale)
    if case["func"] == "wp":
        np.testing.assert_allclose(got["wp"], gold["wp"], rtol=rtol, atol=2 * case["pimax"] * rtol * 2)
    if case["func"] == "xi":
        np.testing.assert_allclose(got["xi"], gold["xi"], rtol=rtol, atol=rtol * 2)


@pytest.mark.parametrize("case", cases.CASES, ids=[c["name"] for c in cases.CASES])
def test_gpu_matches_oracle(gpu, orc, case):
    got = _gpu_call(case)
    want = _oracle_call(orc, case)
    rtol = 1e-4 if case["dtype"] == "f4" else RTOL_AVG
    _check(case["func"], got, want, rtol)


def test_gpu_dd_doctest(gpu, precision):
    from corrfunc_gb300 import theory
    d = GOLDEN["dd_doctest"]
    np.random.seed(d["seed"])
    X = np.random.uniform(0, d["boxsize"], d["N"])
    Y = np.random.uniform(0, d["boxsize"], d["N"])
    Z = np.random.uniform(0, d["boxsize"], d["N"])
    res = theory.DD(1, 4, d["edges"], X, Y, Z, weights1=np.ones_like(X), weight_type="pair_product",
                    output_ravg=True, boxsize=d["boxsize"], periodic=True)
    table = np.array(d["doctest_table"])
    assert list(res["npairs"]) == [int(v) for v in table[:, 3]]
    np.testing.assert_allclose(res["ravg"], table[:, 2], atol=5e-7)
    np.testing.assert_allclose(res["ravg"], d["reference"]["avg"], rtol=RTOL_AVG)


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("boxsize", [123.0, (51.0, 75.0, 123.0)], ids=["iso", "aniso"])
@pytest.mark.parametrize("func", ["DD", "DDrppi", "DDsmu"])
@pytest.mark.parametrize("autocorr", [0, 1])
def test_gpu_brute_clouds(gpu, func, boxsize, periodic, autocorr):
    """Port of Corrfunc/tests/test_theory.py:205-288 (two clouds, rmax up to 0.49 L)."""
    from corrfunc_gb300 import theory
    np.random.seed(1234)
    npts, eps = 100, 0.2
    box = np.array(boxsize)
    bins = np.linspace(0.01, 0.49 * box.min(), 20) if periodic else np.linspace(0.01, 2 * box.max(), 20)
    pimax = np.floor(0.49 * box.min())
    pos = np.random.uniform(low=-eps, high=eps, size=(npts, 3)) * box
    pos[npts // 2:] += box / 2.0
    pos %= box
    brute = brute_numpy(func, pos, box, periodic, bins, pimax=pimax, mu_max=0.5, nmu=10)
    p = pos.T
    kw = dict(periodic=periodic, boxsize=boxsize, X2=p[0], Y2=p[1], Z2=p[2])
    if func == "DD":
        got = theory.DD(autocorr, 1, bins, p[0], p[1], p[2], **kw)["npairs"]
    elif func == "DDrppi":
        got = theory.DDrppi(autocorr, 1, pimax, bins, p[0], p[1], p[2], **kw)["npairs"]
    else:
        got = theory.DDsmu(autocorr, 1, bins, 0.5, 10, p[0], p[1], p[2], **kw)["npairs"]
    assert np.array_equal(np.asarray(got, dtype=np.int64), brute.astype(np.int64))


@pytest.mark.parametrize("N", [1, 2])
def test_gpu_narrow_extent(gpu, N):
    from corrfunc_gb300 import theory
    pos = np.array([[0.0, 0.0], [0.0, 0.0], [0.0, 0.5]]) if N == 2 else np.array([[0.1], [0.2], [0.3]])
    res = theory.DD(1, 1, [0.2, 0.6, 1.0], pos[0], pos[1], pos[2], boxsize=(3.0, 3.0, 3.0), periodic=True)
    assert list(res["npairs"]) == ([2, 0] if N == 2 else [0, 0])


@pytest.mark.parametrize("autocorr", [0, 1])
def test_gpu_duplicate_cellpairs(gpu, autocorr):
    from corrfunc_gb300 import theory
    L = 432.0
    pos = np.array([[0.02, 0.98], [0.0, 0.0], [0.0, 0.0]]) * L
    r = theory.DD(autocorr, 1, np.array([0.01, 0.4]) * L, pos[0], pos[1], pos[2], X2=pos[0], Y2=pos[1], Z2=pos[2],
                  boxsize=L, periodic=True)
    assert list(r["npairs"]) == [2]
    pos = np.array([[0.0, 0.0], [0.0, 0.0], [0.0, 0.48]]) * L
    r = theory.DD(autocorr, 1, np.array([0.2, 0.3, 0.49]) * L, pos[0], pos[1], pos[2], X2=pos[0], Y2=pos[1],
                  Z2=pos[2], boxsize=L, periodic=True)
    assert list(r["npairs"]) == [0, 2]


def test_gpu_empty_inputs(gpu):
    from corrfunc_gb300 import theory
    e = np.zeros(0)
    r = theory.DD(1, 1, [1.0, 2.0, 3.0], e, e, e, boxsize=10.0, periodic=True)
    assert list(r["npairs"]) == [0, 0]
    x = np.array([1.0, 2.0])
    r = theory.DD(0, 1, [0.5, 2.0, 3.0], x, x, x, X2=e, Y2=e, Z2=e, boxsize=10.0, periodic=True)
    assert list(r["npairs"]) == [0, 0]


def test_gpu_pairs_on_bin_edges(gpu, orc, precision):
    """Pairs placed at separations equal to (or one ulp either side of) the bin edges: every such
    pair is inside the FP32 ambiguity band and must be decided by the FP64 re-evaluation."""
    from corrfunc_gb300 import theory
    edges = np.array([0.5, 1.0, 2.0, 3.0, 5.0])
    xs, ys, zs = [], [], []
    base = 10.0
    k = 0
    for e in edges:
        for d in (np.nextafter(e, 0), e, np.nextafter(e, 100)):
            x0 = base + 7.0 * k
            xs += [x0, x0 + d]
            ys += [5.0, 5.0]
            zs += [5.0, 5.0]
            k += 1
    # a 3-4-5 triangle lands exactly on r^2 = 25 in exact arithmetic
    xs += [200.0, 203.0]
    ys += [5.0, 9.0]
    zs += [5.0, 5.0]
    x, y, z = (np.array(a) for a in (xs, ys, zs))
    got = theory.DD(1, 1, edges, x, y, z, periodic=False, output_ravg=True)
    want = orc.DD(1, edges, x, y, z, periodic=False, output_ravg=True)
    assert np.array_equal(got["npairs"], want["npairs"])
    s = gpu.last_stats()
    assert s["pairs_refined"] > 0 or precision == "fp64"


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("func", ["DDrppi", "wp", "DDsmu"])
def test_gpu_2d_pairs_at_the_pruning_bounds(gpu, orc, func, periodic):
    """Pairs at |dz| = pimax, at rp (or s) equal to the top edge, and one ulp either side, in
    groups far apart and amid uniform points: the box pruning of the 2-D kernels (rp from the
    chunk box's xy rectangle, |dz| from its z range, s from the box) keeps every pair the oracle
    counts."""
    from corrfunc_gb300 import theory
    L, pimax = 100.0, 6.0
    edges = np.array([0.5, 1.0, 2.0, 4.0])
    top = edges[-1]
    xs, ys, zs = [], [], []
    k = 0
    for dxy in (np.nextafter(top, 0), top, np.nextafter(top, 100), 1.5):
        for dz in (np.nextafter(pimax, 0), pimax, np.nextafter(pimax, 100), 0.25):
            x0, y0 = 5.0 + 9.0 * (k % 10), 5.0 + 9.0 * (k // 10)
            xs += [x0, x0 + dxy]
            ys += [y0, y0]
            zs += [20.0, 20.0 + dz]
            k += 1
    rng = np.random.default_rng(31)
    xs += list(rng.random(3000) * L)
    ys += list(rng.random(3000) * L)
    zs += list(rng.random(3000) * L)
    x, y, z = (np.array(a) for a in (xs, ys, zs))
    if func == "DDrppi":
        got = theory.DDrppi(1, 1, pimax, edges, x, y, z, periodic=periodic, boxsize=L)
        want = orc.DDrppi(1, pimax, edges, x, y, z, periodic=periodic, boxsize=L)
    elif func == "wp":
        if not periodic:
            pytest.skip("wp is periodic only")
        got = theory.wp(L, pimax, 1, edges, x, y, z)
        want = orc.wp(L, pimax, edges, x, y, z)
    else:
        got = theory.DDsmu(1, 1, edges, 1.0, 5, x, y, z, periodic=periodic, boxsize=L)
        want = orc.DDsmu(1, edges, 1.0, 5, x, y, z, periodic=periodic, boxsize=L)
    assert np.array_equal(np.asarray(got["npairs"], np.uint64), np.asarray(want["npairs"], np.uint64))


@pytest.mark.parametrize("func", ["DD", "DDrppi", "DDsmu", "DDtheta"])
def test_gpu_fp32_refine_equals_fp64(gpu, func):
    """The FP32+FP64-refinement form and the plain FP64 form give identical counts."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks, theory
    outs = []
    for prec in ("fp32_refine", "fp64"):
        gpu.set_precision(prec)
        if func == "DDtheta":
            ra, dec = cat.sky_cap(20000, 5)
            r = mocks.DDtheta_mocks(1, 1, cat.log_bins(0.01, 5.0, 12), ra, dec, output_thetaavg=True)
            outs.append((r["npairs"].copy(), r["thetaavg"].copy()))
        else:
            x, y, z = cat.clustered_box(30000, 250.0, 9, sigma=2.0, mean_occupancy=60)
            bins = cat.log_bins(0.1, 20.0, 14)
            if func == "DD":
                r = theory.DD(1, 1, bins, x, y, z, boxsize=250.0, output_ravg=True)
                f = "ravg"
            elif func == "DDrppi":
                r = theory.DDrppi(1, 1, 20.0, bins, x, y, z, boxsize=250.0, output_rpavg=True)
                f = "rpavg"
            else:
                r = theory.DDsmu(1, 1, bins, 1.0, 10, x, y, z, boxsize=250.0, output_savg=True)
                f = "savg"
            outs.append((r["npairs"].copy(), r[f].copy()))
    gpu.set_precision("fp32_refine")
    assert np.array_equal(outs[0][0], outs[1][0])
    np.testing.assert_allclose(outs[0][1], outs[1][1], rtol=RTOL_AVG, atol=1e-12)


@pytest.mark.parametrize("func", ["DD", "DDrppi", "DDsmu", "wp", "xi", "DDtheta"])
def test_gpu_matches_reference_library_larger(gpu, reflibs, func):
    """Sizes the brute-force oracle would take long on, against the reference library itself."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks, theory
    lib = C.library()
    n, L = 200000, 300.0
    x, y, z = cat.clustered_box(n, L, 3, sigma=2.0, mean_occupancy=80)
    w = cat.weights(n, 4)
    bins = cat.log_bins(0.1, 25.0, 16)
    kw = dict(weights1=w, weight_type="pair_product", boxsize=L, isa="fallback")
    if func == "DD":
        a = theory.run_DD(lib, 1, 4, bins, x, y, z, output_ravg=True, **kw)
        b = theory.run_DD(reflibs["DD"], 1, 16, bins, x, y, z, output_ravg=True, **kw)
        f = "ravg"
    elif func == "DDrppi":
        a = theory.run_DDrppi(lib, 1, 4, 30.0, bins, x, y, z, output_rpavg=True, **kw)
        b = theory.run_DDrppi(reflibs["DDrppi"], 1, 16, 30.0, bins, x, y, z, output_rpavg=True, **kw)
        f = "rpavg"
    elif func == "DDsmu":
        a = theory.run_DDsmu(lib, 1, 4, bins, 1.0, 10, x, y, z, output_savg=True, **kw)
        b = theory.run_DDsmu(reflibs["DDsmu"], 1, 16, bins, 1.0, 10, x, y, z, output_savg=True, **kw)
        f = "savg"
    elif func == "wp":
        a = theory.run_wp(lib, L, 30.0, 4, bins, x, y, z, weights=w, weight_type="pair_product",
                          output_rpavg=True, isa="fallback")
        b = theory.run_wp(reflibs["wp"], L, 30.0, 16, bins, x, y, z, weights=w, weight_type="pair_product",
                          output_rpavg=True, isa="fallback")
        f = "rpavg"
    elif func == "xi":
        a = theory.run_xi(lib, L, 4, bins, x, y, z, output_ravg=True, isa="fallback")
        b = theory.run_xi(reflibs["xi"], L, 16, bins, x, y, z, output_ravg=True, isa="fallback")
        f = "ravg"
    else:
        ra, dec = cat.sky_cap(100000, 8)
        tb = cat.log_bins(0.01, 5.0, 12)
        a = mocks.run_DDtheta_mocks(lib, 1, 4, tb, ra.copy(), dec.copy(), output_thetaavg=True, isa="fallback")
        b = mocks.run_DDtheta_mocks(reflibs["DDtheta"], 1, 16, tb, ra.copy(), dec.copy(), output_thetaavg=True,
                                    isa="fallback")
        f = "thetaavg"
    assert np.array_equal(a["npairs"], b["npairs"])
    np.testing.assert_allclose(a[f], b[f], rtol=RTOL_AVG, atol=1e-12)


@pytest.mark.parametrize("func", ["DD", "DDrppi", "DDsmu"])
def test_gpu_zero_separation_pairs_with_rmin_zero(gpu, orc, func):
    """Duplicated points (separation exactly 0) count in the first bin when rmin = 0."""
    from corrfunc_gb300 import theory
    rng = np.random.default_rng(17)
    x, y, z = (rng.random(300) * 20.0 for _ in range(3))
    x2, y2, z2 = np.concatenate([x, x[:50]]), np.concatenate([y, y[:50]]), np.concatenate([z, z[:50]])
    bins = [0.0, 0.5, 1.0, 2.0]
    kw = dict(X2=x2, Y2=y2, Z2=z2, periodic=False)
    if func == "DD":
        got = theory.DD(0, 1, bins, x, y, z, **kw)
        want = orc.DD(0, bins, x, y, z, **kw)
    elif func == "DDrppi":
        got = theory.DDrppi(0, 1, 3.0, bins, x, y, z, **kw)
        want = orc.DDrppi(0, 3.0, bins, x, y, z, **kw)
    else:
        got = theory.DDsmu(0, 1, bins, 1.0, 4, x, y, z, **kw)
        want = orc.DDsmu(0, bins, 1.0, 4, x, y, z, **kw)
    assert np.array_equal(got["npairs"], want["npairs"])
    assert int(got["npairs"].sum()) > 0


@pytest.mark.parametrize("refine,max_cells", [((1, 1, 1), 100), ((3, 3, 2), 100), ((2, 2, 1), 5)],
                         ids=["refine111", "refine332", "maxcells5"])
def test_gpu_reference_lattice_variants(gpu, orc, refine, max_cells):
    """Custom refine factors and a small max_cells_per_dim change the reference lattice, hence
    which point of a wrapped pair is shifted: counts and averages still follow the oracle."""
    from corrfunc_gb300 import theory
    rng = np.random.default_rng(77)
    L = 60.0
    x, y, z = (rng.random(4000) * L for _ in range(3))
    w = rng.uniform(0.5, 1.5, 4000)
    bins = np.logspace(np.log10(0.2), np.log10(14.0), 12)
    kw = dict(weights1=w, weight_type="pair_product", periodic=True, boxsize=L, output_ravg=True,
              xbin_refine_factor=refine[0], ybin_refine_factor=refine[1], zbin_refine_factor=refine[2],
              max_cells_per_dim=max_cells)
    got = theory.DD(1, 1, bins, x, y, z, **kw)
    want = orc.DD(1, bins, x, y, z, weights1=w, weight_type="pair_product", periodic=True, boxsize=L,
                  output_ravg=True, refine=refine, custom_refine=refine != (2, 2, 1), max_cells_per_dim=max_cells)
    assert np.array_equal(got["npairs"], want["npairs"])
    np.testing.assert_allclose(got["ravg"], want["ravg"], rtol=RTOL_AVG, atol=1e-12)
    np.testing.assert_allclose(got["weightavg"], want["weightavg"], rtol=RTOL_AVG, atol=1e-12)


def test_gpu_many_bins_and_fine_2d_histograms(gpu, orc):
    """300 radial bins (shared histogram columns) and 2-D histograms with 120 pi / 90 mu bins."""
    from corrfunc_gb300 import theory
    rng = np.random.default_rng(78)
    L = 80.0
    x, y, z = (rng.random(5000) * L for _ in range(3))
    bins = np.linspace(0.05, 12.0, 301)
    got = theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=L, output_ravg=True)
    want = orc.DD(1, bins, x, y, z, periodic=True, boxsize=L, output_ravg=True)
    assert np.array_equal(got["npairs"], want["npairs"])
    np.testing.assert_allclose(got["ravg"], want["ravg"], rtol=RTOL_AVG, atol=1e-12)
    rp = np.logspace(np.log10(0.1), np.log10(10.0), 16)
    got = theory.DDrppi(1, 1, 24.0, rp, x, y, z, periodic=True, boxsize=L)
    want = orc.DDrppi(1, 24.0, rp, x, y, z, periodic=True, boxsize=L)
    assert np.array_equal(got["npairs"], want["npairs"])
    got = theory.DDsmu(1, 1, rp, 1.0, 90, x, y, z, periodic=True, boxsize=L)
    want = orc.DDsmu(1, rp, 1.0, 90, x, y, z, periodic=True, boxsize=L)
    assert np.array_equal(got["npairs"], want["npairs"])


COORD_RANGES = {
    # non-periodic clouds whose coordinates exercise the integer (fixed-point) lattice build:
    # far from the origin, negative, a tiny extent, one flat axis, values straddling +-0
    "far_offset": dict(lo=(1.0e6, -2.5e5, 3.0e7), span=(40.0, 40.0, 40.0), bins=(0.3, 12.0)),
    "negative": dict(lo=(-300.0, -280.0, -260.0), span=(30.0, 30.0, 30.0), bins=(0.2, 9.0)),
    "tiny_extent": dict(lo=(5.0, 5.0, 5.0), span=(2e-4, 2e-4, 2e-4), bins=(2e-6, 1.5e-4)),
    "flat_z": dict(lo=(0.0, 0.0, 7.25), span=(25.0, 25.0, 0.0), bins=(0.2, 8.0)),
    "around_zero": dict(lo=(-1e-3, -1e-3, -1e-3), span=(2e-3, 2e-3, 2e-3), bins=(1e-6, 1.2e-3)),
}


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("name", sorted(COORD_RANGES))
def test_gpu_coordinate_ranges(gpu, orc, precision, name, dtype):
    """Counts and averages follow the oracle for coordinate ranges that stress the fixed-point
    hi / lo split, the FP32 cell index and its margins, in both precisions."""
    from corrfunc_gb300 import theory
    c = COORD_RANGES[name]
    rng = np.random.default_rng(sum(ord(ch) for ch in name))
    n = 1500
    pos = [np.asarray(c["lo"][a] + rng.random(n) * c["span"][a], dtype=dtype) for a in range(3)]
    if name == "around_zero":
        pos[0][:20] = 0.0
        pos[1][:10] = -0.0
        pos[2][:5] = 0.0
    bins = np.logspace(np.log10(c["bins"][0]), np.log10(c["bins"][1]), 11)
    w = rng.uniform(0.5, 1.5, n).astype(dtype)
    kw = dict(weights1=w, weight_type="pair_product", periodic=False, output_ravg=True)
    got = theory.DD(1, 1, bins, *pos, **kw)
    want = orc.DD(1, bins, *(p.astype(np.float64) for p in pos), weights1=w.astype(np.float64),
                  weight_type="pair_product", periodic=False, output_ravg=True)
    assert np.array_equal(got["npairs"], want["npairs"])
    assert int(got["npairs"].sum()) > 0
    rtol = RTOL_AVG if dtype == np.float64 else 1e-4
    np.testing.assert_allclose(got["ravg"], want["ravg"], rtol=rtol, atol=1e-12)
    np.testing.assert_allclose(got["weightavg"], want["weightavg"], rtol=rtol, atol=1e-12)
    pimax = max(float(np.ceil(c["bins"][1])), 1.0)  # whole pi bins of 1
    got = theory.DDrppi(1, 1, pimax, bins, *pos, periodic=False)
    want = orc.DDrppi(1, pimax, bins, *(p.astype(np.float64) for p in pos), periodic=False)
    assert np.array_equal(got["npairs"], want["npairs"])


def test_gpu_work_list_resize(gpu, tmp_path):
    """A work list that outgrows its first buffer (forced by CF_TASK_CAPACITY=100 in a child
    process) is resized and the count rerun: the same counts and averages as the default path."""
    import subprocess
    from corrfunc_gb300 import theory
    rng = np.random.default_rng(91)
    x, y, z = (rng.random(20000) * 100.0 for _ in range(3))
    path = tmp_path / "pts.npy"
    np.save(str(path), np.stack([x, y, z]))
    bins = np.logspace(-1, np.log10(12.0), 10)
    want = theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=100.0, output_ravg=True)
    code = ("import sys, numpy as np; sys.path.insert(0, %r)\n"
            "from corrfunc_gb300 import theory\n"
            "import corrfunc_gb300\n"
            "x, y, z = np.load(%r)\n"
            "r = theory.DD(1, 1, np.logspace(-1, np.log10(12.0), 10), x, y, z, periodic=True, boxsize=100.0,"
            " output_ravg=True)\n"
            "print(' '.join(str(int(v)) for v in r['npairs']))\n"
            "print(' '.join(repr(float(v)) for v in r['ravg']))\n"
            "print(corrfunc_gb300.last_stats()['tasks'])\n") % (os.path.dirname(HERE), str(path))
    env = dict(os.environ, CF_TASK_CAPACITY="100")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.split("\n")
    assert [int(v) for v in lines[0].split()] == [int(v) for v in want["npairs"]]
    np.testing.assert_allclose([float(v) for v in lines[1].split()], want["ravg"], rtol=1e-12, atol=1e-15)
    assert int(lines[2]) > 100  # the list did outgrow the forced buffer


@pytest.mark.parametrize("func", ["wp", "xi"])
def test_gpu_points_outside_the_box_fail_loudly(gpu, capfd, func):
    """wp / xi lattice the periodic box [0, L): a point well outside it makes the call fail with
    a message (the reference's gridlink reports it out of bounds, utils/gridlink_impl.c.src:183;
    here the data span beyond the periodic length is reported first) instead of counting it."""
    from corrfunc_gb300 import theory
    rng = np.random.default_rng(5)
    L = 100.0
    x, y, z = (rng.random(2000) * L for _ in range(3))
    x[7] = 1.5 * L
    bins = np.logspace(-1, 1, 8)
    with pytest.raises(RuntimeError):
        if func == "wp":
            theory.wp(L, 10.0, 1, bins, x, y, z)
        else:
            theory.xi(L, 1, bins, x, y, z)
    err = capfd.readouterr().err
    assert "out of bounds" in err or "more than the periodic length" in err


def test_gpu_wp_cell_timer(gpu):
    """wp with c_cell_timer (theory/wp/countpairs_wp_impl.c.src:330-332, 433-463): one record per
    GPU work-list task; their pair counts (each task's window) bound the pairs evaluated (box
    pruning skips the j points out of the chunk's reach), the counts are unchanged."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    x, y, z = cat.clustered_box(30000, 150.0, 12)
    bins = cat.log_bins(0.2, 12.0, 9)
    plain = theory.wp(150.0, 15.0, 1, bins, x, y, z)
    res, api_time, cells = theory.wp(150.0, 15.0, 1, bins, x, y, z, c_api_timer=True, c_cell_timer=True)
    assert np.array_equal(res["npairs"], plain["npairs"])
    assert api_time > 0 and len(cells) == gpu.last_stats()["tasks"]
    window = int(np.sum(cells["N1"] * cells["N2"]))
    assert 0 < gpu.last_stats()["pairs_evaluated"] <= window
    assert (cells["time_in_ns"] > 0).all() and (cells["N1"] >= 1).all() and (cells["N1"] <= 32).all()
