"""The oracle (CPU restatement) pinned against the reference: committed golden vectors, the
reference's own known-answer tests, and the reference libraries built in oracle/_ref."""
import json
import os
import platform
import struct
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))
REF_ROOT = os.environ.get("CORRFUNC_REF_DIR", "/root/reference")


def _oracle_call(orc, case, isa="fallback"):
    args, kw = cases.make_inputs(case, isa=isa)
    f = case["func"]
    if f == "DD":
        auto, _nt, bins, x, y, z = args
        return orc.DD(auto, bins, x, y, z, **kw)
    if f == "DDrppi":
        auto, _nt, pimax, bins, x, y, z = args
        return orc.DDrppi(auto, pimax, bins, x, y, z, **kw)
    if f == "DDsmu":
        auto, _nt, bins, mu_max, nmu, x, y, z = args
        return orc.DDsmu(auto, bins, mu_max, nmu, x, y, z, **kw)
    if f == "wp":
        L, pimax, _nt, bins, x, y, z = args
        return orc.wp(L, pimax, bins, x, y, z, **kw)
    if f == "xi":
        L, _nt, bins, x, y, z = args
        return orc.xi(L, bins, x, y, z, **kw)
    auto, _nt, bins, ra, dec = args
    kw = dict(kw)
    return orc.DDtheta_mocks(auto, bins, ra, dec, **kw)


def check_result(func, res, gold, rtol=1e-9):
    assert [int(v) for v in res["npairs"]] == gold["npairs"]
    avg = np.asarray(res[cases.AVG_FIELD[func]], dtype=float)
    ga = np.asarray(gold["avg"])
    np.testing.assert_allclose(avg, ga, rtol=rtol, atol=1e-12)
    np.testing.assert_allclose(np.asarray(res["weightavg"], dtype=float), np.asarray(gold["weightavg"]), rtol=rtol,
                               atol=1e-12)
    if func == "wp":
        np.testing.assert_allclose(res["wp"], gold["wp"], rtol=rtol, atol=1e-9)
    if func == "xi":
        np.testing.assert_allclose(res["xi"], gold["xi"], rtol=rtol, atol=1e-9)


@pytest.mark.parametrize("case", cases.CASES, ids=[c["name"] for c in cases.CASES])
def test_oracle_matches_golden(orc, case):
    res = _oracle_call(orc, case)
    check_result(case["func"], res, GOLDEN["cases"][case["name"]])


@pytest.mark.parametrize("case", cases.CASES, ids=[c["name"] for c in cases.CASES])
def test_oracle_matches_golden_avx512f(orc, case):
    """The oracle's fused multiply-add formulas against the reference's AVX512F kernels."""
    res = _oracle_call(orc, case, isa="avx512f")
    check_result(case["func"], res, GOLDEN["avx512f_cases"][case["name"]])


def test_oracle_reproduces_dd_doctest(orc):
    d = GOLDEN["dd_doctest"]
    np.random.seed(d["seed"])
    X = np.random.uniform(0, d["boxsize"], d["N"])
    Y = np.random.uniform(0, d["boxsize"], d["N"])
    Z = np.random.uniform(0, d["boxsize"], d["N"])
    res = orc.DD(1, d["edges"], X, Y, Z, weights1=np.ones_like(X), weight_type="pair_product", output_ravg=True,
                 boxsize=d["boxsize"], periodic=True)
    table = np.array(d["doctest_table"])
    assert list(res["npairs"]) == [int(v) for v in table[:, 3]]
    np.testing.assert_allclose(res["ravg"], table[:, 2], atol=5e-7)
    np.testing.assert_allclose(res["weightavg"], table[:, 4], atol=5e-7)
    assert list(res["npairs"]) == d["reference"]["npairs"]
    np.testing.assert_allclose(res["ravg"], d["reference"]["avg"], rtol=1e-12)


ISAS = ["fallback"] + (["avx512f", "avx"] if platform.machine() in ("x86_64", "AMD64") else [])


@pytest.mark.parametrize("isa", ISAS)
@pytest.mark.parametrize("func", ["DD", "DDrppi", "DDsmu", "wp", "xi", "DDtheta"])
def test_oracle_matches_reference_library(orc, reflibs, func, isa):
    """Fresh seeded inputs (not in the golden file), both formula variants where the host has them."""
    from corrfunc_gb300 import mocks, theory
    rng = np.random.default_rng(hash((func, isa)) % 2**32)
    n, L = 2500, 60.0
    x, y, z = (rng.random(n) * L for _ in range(3))
    w = rng.uniform(0.5, 1.5, n)
    bins = np.logspace(np.log10(0.3), np.log10(12.0), 9)
    if func == "DD":
        r = theory.run_DD(reflibs["DD"], 1, 2, bins, x, y, z, weights1=w, weight_type="pair_product",
                          periodic=True, boxsize=L, output_ravg=True, isa=isa)
        o = orc.DD(1, bins, x, y, z, weights1=w, weight_type="pair_product", periodic=True, boxsize=L,
                   output_ravg=True, isa=isa)
        f = "ravg"
    elif func == "DDrppi":
        r = theory.run_DDrppi(reflibs["DDrppi"], 0, 2, 10.0, bins, x, y, z, X2=y, Y2=z, Z2=x, periodic=True,
                              boxsize=L, output_rpavg=True, isa=isa)
        o = orc.DDrppi(0, 10.0, bins, x, y, z, X2=y, Y2=z, Z2=x, periodic=True, boxsize=L, output_rpavg=True, isa=isa)
        f = "rpavg"
    elif func == "DDsmu":
        r = theory.run_DDsmu(reflibs["DDsmu"], 1, 2, bins, 0.8, 8, x, y, z, periodic=False, output_savg=True, isa=isa)
        o = orc.DDsmu(1, bins, 0.8, 8, x, y, z, periodic=False, output_savg=True, isa=isa)
        f = "savg"
    elif func == "wp":
        r = theory.run_wp(reflibs["wp"], L, 8.0, 2, bins, x, y, z, output_rpavg=True, isa=isa)
        o = orc.wp(L, 8.0, bins, x, y, z, output_rpavg=True, isa=isa)
        f = "rpavg"
    elif func == "xi":
        r = theory.run_xi(reflibs["xi"], L, 2, bins, x, y, z, weights=w, weight_type="pair_product",
                          output_ravg=True, isa=isa)
        o = orc.xi(L, bins, x, y, z, weights=w, weight_type="pair_product", output_ravg=True, isa=isa)
        f = "ravg"
    else:
        ra = rng.random(n) * 40.0
        dec = np.degrees(np.arcsin(rng.random(n) * 0.5))
        tb = np.logspace(-1.5, 0.8, 9)
        r = mocks.run_DDtheta_mocks(reflibs["DDtheta"], 1, 2, tb, ra.copy(), dec.copy(), output_thetaavg=True, isa=isa)
        o = orc.DDtheta_mocks(1, tb, ra, dec, output_thetaavg=True, isa=isa)
        f = "thetaavg"
    assert np.array_equal(r["npairs"], o["npairs"])
    np.testing.assert_allclose(o[f], r[f], rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("N", [1, 2])
def test_narrow_extent(orc, N):
    """Corrfunc/tests/test_theory.py:116-151: one or two points in a large box."""
    if N == 2:
        pos = np.array([[0.0, 0.0], [0.0, 0.0], [0.0, 0.5]])
    else:
        pos = np.array([[0.1], [0.2], [0.3]])
    res = orc.DD(1, [0.2, 0.6, 1.0], pos[0], pos[1], pos[2], boxsize=(3.0, 3.0, 3.0), periodic=True)
    assert list(res["npairs"]) == ([2, 0] if N == 2 else [0, 0])


@pytest.mark.parametrize("autocorr", [0, 1])
def test_duplicate_cellpairs(orc, autocorr):
    """Corrfunc/tests/test_theory.py:154-202: a pair straddling the wrap, rmax close to L/2."""
    L = 432.0
    pos = np.array([[0.02, 0.98], [0.0, 0.0], [0.0, 0.0]]) * L
    r = orc.DD(autocorr, np.array([0.01, 0.4]) * L, pos[0], pos[1], pos[2], X2=pos[0], Y2=pos[1], Z2=pos[2],
               boxsize=L, periodic=True)
    assert list(r["npairs"]) == [2]
    pos = np.array([[0.0, 0.0], [0.0, 0.0], [0.0, 0.48]]) * L
    r = orc.DD(autocorr, np.array([0.2, 0.3, 0.49]) * L, pos[0], pos[1], pos[2], X2=pos[0], Y2=pos[1],
               Z2=pos[2], boxsize=L, periodic=True)
    assert list(r["npairs"]) == [0, 2]


def brute_numpy(func, pos, boxsize, periodic, bins, pimax=None, mu_max=None, nmu=None):
    """Independent numpy brute force (Corrfunc/tests/test_theory.py:205-288)."""
    pdiff = np.abs(pos[:, np.newaxis] - pos)
    if periodic:
        pdiff -= (pdiff >= boxsize / 2) * boxsize
    if func == "DDrppi":
        sq = (pdiff[:, :, :2] ** 2).sum(-1).reshape(-1)
        pid = np.abs(pdiff[:, :, 2]).reshape(-1)
        return np.histogram2d(sq, pid, bins=(bins ** 2, np.linspace(0.0, pimax, int(pimax) + 1)))[0].reshape(-1)
    if func == "DDsmu":
        s = np.sqrt((pdiff ** 2).sum(-1).reshape(-1))
        s[s == 0.0] = np.inf
        mu = np.abs(pdiff[:, :, 2]).reshape(-1) / s
        return np.histogram2d(s, mu, bins=(bins, np.linspace(0, mu_max, nmu + 1)))[0].reshape(-1)
    return np.histogram((pdiff ** 2).sum(-1).reshape(-1), bins=bins ** 2)[0]


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("boxsize", [123.0, (51.0, 75.0, 123.0)], ids=["iso", "aniso"])
@pytest.mark.parametrize("func", ["DD", "DDrppi", "DDsmu"])
def test_brute_clouds(orc, func, boxsize, periodic):
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
        got = orc.DD(1, bins, p[0], p[1], p[2], **kw)["npairs"]
    elif func == "DDrppi":
        got = orc.DDrppi(1, pimax, bins, p[0], p[1], p[2], **kw)["npairs"]
    else:
        got = orc.DDsmu(1, bins, 0.5, 10, p[0], p[1], p[2], **kw)["npairs"]
    assert np.any(brute > 0)
    assert np.array_equal(np.asarray(got, dtype=np.int64), brute.astype(np.int64))


def _read_fastfood(path):
    data = open(path, "rb").read()
    off, recs = 0, []
    while off < len(data):
        n = struct.unpack("<i", data[off:off + 4])[0]
        recs.append(data[off + 4:off + 4 + n])
        off += n + 8
    return [np.frombuffer(r, dtype=np.float64) for r in recs if len(r) == len(recs[-1])]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "mocks", "tests")), reason="reference tree not present")
def test_oracle_reproduces_mr19_wtheta_golden(orc):
    """mocks/tests/Mr19_mock_wtheta.DD (Corrfunc/tests/test_mocks.py:62-80) on its own input."""
    ra, dec, _cz, w = _read_fastfood(os.path.join(REF_ROOT, "mocks", "tests", "data", "Mr19_mock_northonly.rdcz.ff"))
    res = orc.DDtheta_mocks(1, os.path.join(REF_ROOT, "mocks", "tests", "angular_bins"), ra.copy(), dec.copy(),
                            weights1=w, weight_type="pair_product", output_thetaavg=True)
    gold = np.loadtxt(os.path.join(REF_ROOT, "mocks", "tests", "Mr19_mock_wtheta.DD"))
    assert list(res["npairs"]) == [int(v) for v in gold[:, 0]]
    np.testing.assert_allclose(res["thetaavg"], gold[:, 1], rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(res["weightavg"], gold[:, 4], rtol=1e-6, atol=1e-9)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "mocks", "tests")), reason="reference tree not present")
def test_oracle_reproduces_mr19_rppi_mocks_golden(orc):
    """mocks/tests/Mr19_mock.DD (Corrfunc/tests/test_mocks.py:14-34) on its own input: cz -> comoving
    distance with cosmology 1, pimax 40, mocks/tests/bins, pair_product weights, rpavg."""
    ra, dec, cz, w = _read_fastfood(os.path.join(REF_ROOT, "mocks", "tests", "data", "Mr19_mock_northonly.rdcz.ff"))
    res = orc.DDrppi_mocks(1, 1, 40.0, os.path.join(REF_ROOT, "mocks", "tests", "bins"), ra.copy(), dec.copy(),
                           cz.copy(), weights1=w, weight_type="pair_product", output_rpavg=True)
    gold = np.loadtxt(os.path.join(REF_ROOT, "mocks", "tests", "Mr19_mock.DD"))
    assert list(res["npairs"]) == [int(v) for v in gold[:, 0]]
    np.testing.assert_allclose(res["rpavg"], gold[:, 1], rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(res["weightavg"], gold[:, 4], rtol=1e-6, atol=1e-9)


def test_oracle_mock_formula_families_agree_off_the_edges(orc):
    """The three double-precision formula families (fallback, AVX/SSE, AVX512F) of DDrppi_mocks and
    DDsmu_mocks differ only in rounding: on a small survey their counts agree except for pairs within
    a few ulps of an edge, i.e. in practice everywhere, and the rp-pi counts sum to the pairs a
    numpy restatement finds inside the (rp, pi) domain."""
    from corrfunc_gb300 import catalogs as cat
    ra, dec, cz = cat.survey(3000, 11)
    bins = cat.log_bins(0.5, 15.0, 8)
    outs = [orc.DDrppi_mocks(1, 1, 20.0, bins, ra.copy(), dec.copy(), cz.copy(), isa=isa)
            for isa in ("fallback", "avx", "avx512f")]
    for o in outs[1:]:
        assert np.array_equal(o["npairs"], outs[0]["npairs"])
    x, y, z = orc.mock_xyz(ra, dec, cz, False, 1, float(cz.max()) / orc.SPEED_OF_LIGHT + 0.01)
    P = np.stack([x, y, z], 1)
    s = P[None, :, :] - P[:, None, :]
    l = P[None, :, :] + P[:, None, :]
    pi2 = np.einsum("ijk,ijk->ij", s, l) ** 2 / np.einsum("ijk,ijk->ij", l, l)
    rp2 = np.einsum("ijk,ijk->ij", s, s) - pi2
    iu = np.triu_indices(len(x), 1)
    inside = (rp2[iu] >= bins[0] ** 2) & (rp2[iu] < bins[-1] ** 2) & (pi2[iu] < 20.0 ** 2)
    assert int(outs[0]["npairs"].sum()) == 2 * int(inside.sum())
    smu = [orc.DDsmu_mocks(1, 2, 1.0, 5, bins, ra.copy(), dec.copy(), cz.copy(), isa=isa)
           for isa in ("fallback", "avx", "avx512f")]
    for o in smu[1:]:
        assert np.array_equal(o["npairs"], smu[0]["npairs"])
    assert smu[0]["npairs"].sum() > 0


def test_oracle_mt19937_known_answers(orc):
    """MT19937 with seed 5489: first output 3499211612 and 10,000th output 4123659995 (the published
    known answers, the latter required of std::mt19937 by the C++ standard)."""
    u = orc.mt_uniforms(5489, 10000) * 4294967296.0
    assert int(u[0]) == 3499211612
    assert int(u[-1]) == 4123659995


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "mocks", "tests")), reason="reference tree not present")
def test_oracle_reproduces_mr19_vpf_mocks_golden(orc):
    """mocks/tests/Mr19_mock_vpf (Corrfunc/tests/test_mocks.py:83-113): 10,000 spheres of radius up to 10
    from the reference's centres file, 10 radii, p0..p5, cosmology 1 -- every count exact."""
    ra, dec, cz, _ = _read_fastfood(os.path.join(REF_ROOT, "mocks", "tests", "data", "Mr19_mock_northonly.rdcz.ff"))
    centers = os.path.join(REF_ROOT, "mocks", "tests", "data", "Mr19_centers_xyz_forVPF_rmax_10Mpc.txt")
    res, counts, cen = orc.vpf_mocks(10.0, 10, 10000, 6, 1, centers, 1, ra.copy(), dec.copy(), cz.copy(), ra.copy(),
                                     dec.copy(), cz.copy())
    gold = np.genfromtxt(os.path.join(REF_ROOT, "mocks", "tests", "Mr19_mock_vpf"))
    assert len(cen) == 10000
    assert np.array_equal(np.rint(gold[:, 1:] * 10000).astype(np.int64), counts.astype(np.int64))
    np.testing.assert_allclose(res["pN"], gold[:, 1:], rtol=1e-6, atol=1e-9)


def _gslshim():
    import ctypes
    path = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libcf_gslshim.so")
    if not os.path.exists(path):
        pytest.skip("GSL stand-in check library not built")
    lib = ctypes.CDLL(path)
    lib.cf_shim_mt_nth.restype = ctypes.c_uint32
    lib.cf_shim_mt_nth.argtypes = [ctypes.c_ulong, ctypes.c_int]
    lib.cf_shim_interp.restype = ctypes.c_double
    lib.cf_shim_interp.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                   ctypes.c_double]
    return lib


def test_gsl_stand_in_known_answers():
    """The test-only GSL stand-in the reference's survey and vpf sources are compiled against:
    MT19937's published known answers (seed 5489: first output 3499211612, 10,000th 4123659995),
    agreement with the oracle's own restatement of the generator for other seeds (seed 0 standing
    for GSL's default 4357), and the linear interpolant's formula."""
    import ctypes
    lib = _gslshim()
    assert lib.cf_shim_mt_nth(5489, 1) == 3499211612
    assert lib.cf_shim_mt_nth(5489, 10000) == 4123659995
    import oracle
    oracle.build()
    for seed in (0, 4357, 1, 2**31 + 5):
        u = oracle.mt_uniforms(seed, 700) * 4294967296.0
        assert [int(lib.cf_shim_mt_nth(seed, k)) for k in (1, 2, 624, 625, 700)] == \
            [int(u[k - 1]) for k in (1, 2, 624, 625, 700)]
    xa = np.array([0.0, 0.5, 1.25, 2.0, 4.0])
    ya = np.array([1.0, 3.0, 2.0, 7.5, -1.0])
    P = ctypes.POINTER(ctypes.c_double)
    for x in (0.0, 0.3, 0.5, 1.9999, 2.0, 3.3, 4.0):
        k = min(int(np.searchsorted(xa, x, side="right")) - 1, len(xa) - 2)
        want = ya[k] + (x - xa[k]) / (xa[k + 1] - xa[k]) * (ya[k + 1] - ya[k])
        assert lib.cf_shim_interp(xa.ctypes.data_as(P), ya.ctypes.data_as(P), len(xa), x) == want
    assert np.isnan(lib.cf_shim_interp(xa.ctypes.data_as(P), ya.ctypes.data_as(P), len(xa), 4.5))


SURVEY_ISAS = ["fallback"] + (["avx", "avx512f"] if platform.machine() in ("x86_64", "AMD64") else [])


@pytest.mark.parametrize("isa", SURVEY_ISAS)
@pytest.mark.parametrize("func", ["DDrppi_mocks", "DDsmu_mocks"])
def test_oracle_matches_reference_survey_counters(orc, reflibs_gsl, func, isa):
    """The oracle's survey counters against the reference's own DDrppi_mocks / DDsmu_mocks (compiled
    against the GSL stand-in): auto and cross, both cosmologies, weights, averages."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz = cat.survey(2500, 31, ra=(120.0, 170.0), dec=(0.0, 40.0), cz=(3000.0, 15000.0))
    ra2, dec2, cz2 = cat.survey(2000, 32, ra=(120.0, 170.0), dec=(0.0, 40.0), cz=(3000.0, 15000.0))
    w = cat.weights(2500, 33)
    w2 = cat.weights(2000, 34)
    bins = cat.log_bins(0.3, 18.0, 9)
    lib = reflibs_gsl[func]
    for auto, cosmo in ((1, 1), (0, 2)):
        kw = dict(weights1=w, weight_type="pair_product", isa=isa)
        okw = dict(weights1=w, weight_type="pair_product", isa=isa)
        if not auto:
            kw.update(RA2=ra2.copy(), DEC2=dec2.copy(), CZ2=cz2.copy(), weights2=w2)
            okw.update(RA2=ra2.copy(), DEC2=dec2.copy(), CZ2=cz2.copy(), weights2=w2)
        if func == "DDrppi_mocks":
            r = mocks.run_DDrppi_mocks(lib, auto, cosmo, 2, 25.0, bins, ra.copy(), dec.copy(), cz.copy(),
                                       output_rpavg=True, **kw)
            o = orc.DDrppi_mocks(auto, cosmo, 25.0, bins, ra.copy(), dec.copy(), cz.copy(), output_rpavg=True, **okw)
            f = "rpavg"
        else:
            r = mocks.run_DDsmu_mocks(lib, auto, cosmo, 2, 0.9, 6, bins, ra.copy(), dec.copy(), cz.copy(),
                                      output_savg=True, **kw)
            o = orc.DDsmu_mocks(auto, cosmo, 0.9, 6, bins, ra.copy(), dec.copy(), cz.copy(), output_savg=True, **okw)
            f = "savg"
        assert np.array_equal(r["npairs"], o["npairs"])
        assert int(np.sum(r["npairs"])) > 0
        np.testing.assert_allclose(o[f], r[f], rtol=1e-10, atol=1e-14)
        np.testing.assert_allclose(o["weightavg"], r["weightavg"], rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("periodic,refine,seed", [(True, (1, 1, 1), -1234), (True, (2, 2, 1), 7),
                                                  (False, (1, 1, 1), 11), (False, (2, 1, 3), 0)])
def test_oracle_matches_reference_vpf(orc, reflibs_gsl, periodic, refine, seed):
    """The oracle's counts in spheres against the reference's own theory vpf (its MT19937 centres
    from the GSL stand-in): every pN entry equal."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 120.0
    x, y, z = cat.clustered_box(20000, L, 21)
    kw = dict(periodic=periodic, boxsize=L)
    r = theory.run_vpf(reflibs_gsl["vpf"], 7.0, 7, 2000, 6, seed, x, y, z, xbin_refine_factor=refine[0],
                       ybin_refine_factor=refine[1], zbin_refine_factor=refine[2], **kw)
    o, counts = orc.vpf(7.0, 7, 2000, 6, seed, x, y, z, refine=refine, **kw)
    np.testing.assert_array_equal(r["rmax"], o["rmax"])
    assert np.array_equal(np.rint(r["pN"] * 2000).astype(np.int64), counts.astype(np.int64))
    assert counts[:, 1:].sum() > 0
