"""DDrppi_mocks / DDsmu_mocks (countpairs_mocks / countpairs_mocks_s_mu) on the GPU against the
oracle on seeded synthetic surveys: npairs bit-exact in every bin, separation and weight averages
within 1e-6 relative (float64 inputs; the oracle's formula is the reference's double-precision
one), for auto- and cross-correlations, the three formula families, cz and comoving-distance
inputs, both cosmologies, float32 inputs (against the double run on the upcast values) and the
in-place RA / DEC / redshift fix-ups."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_AVG = 1e-6


def _check(got, want, avg):
    assert np.array_equal(got["npairs"], want["npairs"])
    np.testing.assert_allclose(got[avg], want[avg], rtol=RTOL_AVG, atol=1e-9)
    np.testing.assert_allclose(got["weightavg"], want["weightavg"], rtol=RTOL_AVG, atol=1e-9)


def _survey(n, seed, dtype=np.float64, **kw):
    from corrfunc_gb300 import catalogs as cat
    ra, dec, cz = cat.survey(n, seed, **kw)
    w = cat.weights(n, seed + 50)
    return [a.astype(dtype) for a in (ra, dec, cz, w)]


def _copies(arrs):
    return [a.copy() for a in arrs]


@pytest.mark.parametrize("isa", ["fallback", "avx", "avx512f"])
@pytest.mark.parametrize("autocorr", [1, 0])
def test_rppi_mocks_matches_oracle(orc, isa, autocorr):
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    s1 = _survey(6000, 3)
    s2 = _survey(5000, 4)
    bins = cat.log_bins(0.3, 20.0, 10)
    kw = dict(weight_type="pair_product", output_rpavg=True, isa=isa)
    if autocorr:
        got = mocks.DDrppi_mocks(1, 1, 1, 25.0, bins, *_copies(s1[:3]), weights1=s1[3], **kw)
        want = orc.DDrppi_mocks(1, 1, 25.0, bins, *_copies(s1[:3]), weights1=s1[3], **kw)
    else:
        a, b = _copies(s1[:3]), _copies(s2[:3])
        got = mocks.DDrppi_mocks(0, 1, 1, 25.0, bins, *a, weights1=s1[3], RA2=b[0], DEC2=b[1], CZ2=b[2],
                                 weights2=s2[3], **kw)
        a, b = _copies(s1[:3]), _copies(s2[:3])
        want = orc.DDrppi_mocks(0, 1, 25.0, bins, *a, weights1=s1[3], RA2=b[0], DEC2=b[1], CZ2=b[2],
                                weights2=s2[3], **kw)
    assert got["npairs"].sum() > 0
    _check(got, want, "rpavg")


@pytest.mark.parametrize("isa", ["fallback", "avx", "avx512f"])
@pytest.mark.parametrize("autocorr", [1, 0])
def test_smu_mocks_matches_oracle(orc, isa, autocorr):
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    s1 = _survey(6000, 7)
    s2 = _survey(5000, 8)
    bins = cat.log_bins(0.5, 25.0, 12)
    kw = dict(weight_type="pair_product", output_savg=True, isa=isa)
    if autocorr:
        got = mocks.DDsmu_mocks(1, 2, 1, 1.0, 10, bins, *_copies(s1[:3]), weights1=s1[3], **kw)
        want = orc.DDsmu_mocks(1, 2, 1.0, 10, bins, *_copies(s1[:3]), weights1=s1[3], **kw)
    else:
        a, b = _copies(s1[:3]), _copies(s2[:3])
        got = mocks.DDsmu_mocks(0, 2, 1, 0.8, 8, bins, *a, weights1=s1[3], RA2=b[0], DEC2=b[1], CZ2=b[2],
                                weights2=s2[3], **kw)
        a, b = _copies(s1[:3]), _copies(s2[:3])
        want = orc.DDsmu_mocks(0, 2, 0.8, 8, bins, *a, weights1=s1[3], RA2=b[0], DEC2=b[1], CZ2=b[2],
                               weights2=s2[3], **kw)
    assert got["npairs"].sum() > 0
    _check(got, want, "savg")


def test_mocks_comoving_distance_input(orc):
    """is_comoving_dist: the third column is the distance itself (no cosmology table)."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz, w = _survey(8000, 12, cz=(60.0, 140.0))
    bins = cat.log_bins(0.2, 12.0, 9)
    got = mocks.DDrppi_mocks(1, 1, 1, 15.0, bins, ra.copy(), dec.copy(), cz.copy(), is_comoving_dist=True,
                             output_rpavg=True)
    want = orc.DDrppi_mocks(1, 1, 15.0, bins, ra.copy(), dec.copy(), cz.copy(), is_comoving_dist=True,
                            output_rpavg=True)
    _check(got, want, "rpavg")
    got = mocks.DDsmu_mocks(1, 1, 1, 0.5, 5, bins, ra.copy(), dec.copy(), cz.copy(), is_comoving_dist=True)
    want = orc.DDsmu_mocks(1, 1, 0.5, 5, bins, ra.copy(), dec.copy(), cz.copy(), is_comoving_dist=True)
    assert np.array_equal(got["npairs"], want["npairs"])


def test_mocks_float32_inputs_match_the_double_run(orc):
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz, w = _survey(6000, 21, dtype=np.float32)
    bins = cat.log_bins(0.3, 15.0, 8)
    got = mocks.DDrppi_mocks(1, 1, 1, 20.0, bins, ra.copy(), dec.copy(), cz.copy(), weights1=w,
                             weight_type="pair_product", output_rpavg=True)
    want = orc.DDrppi_mocks(1, 1, 20.0, bins, ra.astype(np.float64), dec.astype(np.float64),
                            cz.astype(np.float64), weights1=w.astype(np.float64), weight_type="pair_product",
                            output_rpavg=True)
    assert np.array_equal(got["npairs"], want["npairs"])
    np.testing.assert_allclose(got["rpavg"], want["rpavg"], rtol=1e-4, atol=1e-9)


def test_mocks_fix_ups_happen_in_place(orc):
    """RA in [-180, 180], DEC in [0, 180] and redshifts instead of cz are converted in place, as the
    reference does, and the counts equal those of the already-converted inputs."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz, _ = _survey(4000, 31)
    bins = cat.log_bins(0.5, 10.0, 6)
    want = mocks.DDrppi_mocks(1, 1, 1, 10.0, bins, ra.copy(), dec.copy(), cz.copy())
    ra2, dec2, z2 = ra - 180.0, dec + 90.0, cz / 299800.0
    got = mocks.DDrppi_mocks(1, 1, 1, 10.0, bins, ra2, dec2, z2)
    np.testing.assert_allclose(ra2, ra, rtol=0, atol=1e-9)
    np.testing.assert_allclose(dec2, dec, rtol=0, atol=1e-9)
    np.testing.assert_allclose(z2, cz, rtol=1e-12)
    orc_res = orc.DDrppi_mocks(1, 1, 10.0, bins, ra - 180.0, dec + 90.0, cz / 299800.0)
    assert np.array_equal(got["npairs"], orc_res["npairs"])
    assert want["npairs"].sum() > 0


def test_mocks_errors_raise():
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz, _ = _survey(500, 41)
    bins = cat.log_bins(0.5, 10.0, 4)
    with pytest.raises(RuntimeError):
        mocks.DDrppi_mocks(1, 3, 1, 10.0, bins, ra.copy(), dec.copy(), cz.copy())
    with pytest.raises(ValueError):
        mocks.DDsmu_mocks(1, 1, 1, 1.5, 5, bins, ra.copy(), dec.copy(), cz.copy())
    with pytest.raises(ValueError):
        mocks.DDrppi_mocks(0, 1, 1, 10.0, bins, ra.copy(), dec.copy(), cz.copy())


def test_mocks_near_the_observer_and_fine_bins(orc):
    """Galaxies from 1 to 40 Mpc/h: many pairs lie closer to the observer than twice the largest
    separation, where the FP32 line-of-sight bound does not hold and the pair goes to FP64; fine rp
    bins from 0.1 with weights and rpavg (every counted pair re-evaluated)."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz, w = _survey(9000, 61, cz=(100.0, 4000.0), ra=(0.0, 360.0), dec=(-60.0, 60.0))
    bins = cat.log_bins(0.1, 15.0, 14)
    kw = dict(weights1=w, weight_type="pair_product", output_rpavg=True)
    got = mocks.DDrppi_mocks(1, 1, 1, 20.0, bins, ra.copy(), dec.copy(), cz.copy(), **kw)
    want = orc.DDrppi_mocks(1, 1, 20.0, bins, ra.copy(), dec.copy(), cz.copy(), **kw)
    assert got["npairs"].sum() > 0
    _check(got, want, "rpavg")
    got = mocks.DDsmu_mocks(1, 1, 1, 0.7, 14, bins, ra.copy(), dec.copy(), cz.copy(), output_savg=True)
    want = orc.DDsmu_mocks(1, 1, 0.7, 14, bins, ra.copy(), dec.copy(), cz.copy(), output_savg=True)
    _check(got, want, "savg")


@pytest.mark.parametrize("precision", ["fp32_refine", "fp64"])
def test_mocks_mr19_sized_survey(orc, precision):
    """A survey of the reference test's size and footprint (40,000 galaxies of the 84,383, 14 rp bins
    0.1-25, pimax 40): both precisions give the oracle's counts."""
    import corrfunc_gb300 as cf
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz, w = _survey(40000, 71, ra=(110.0, 266.0), dec=(-4.0, 70.0), cz=(6000.0, 20000.0))
    bins = cat.log_bins(0.1, 25.0, 14)
    old = cf.get_precision()
    cf.set_precision(precision)
    try:
        got = mocks.DDrppi_mocks(1, 1, 1, 40.0, bins, ra.copy(), dec.copy(), cz.copy(), weights1=w,
                                 weight_type="pair_product")
    finally:
        cf.set_precision(old)
    want = orc.DDrppi_mocks(1, 1, 40.0, bins, ra.copy(), dec.copy(), cz.copy(), weights1=w, weight_type="pair_product")
    assert np.array_equal(got["npairs"], want["npairs"])
    np.testing.assert_allclose(got["weightavg"], want["weightavg"], rtol=RTOL_AVG, atol=1e-9)


@pytest.mark.parametrize("avg", [False, True])
def test_mocks_deep_survey(orc, avg):
    """cz from 100,000 to 250,000 km/s (comoving distances near 1,000-2,000 Mpc/h): the hi grid is
    coarse and |x| large; counts stay exact."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz, w = _survey(12000, 81, ra=(150.0, 160.0), dec=(0.0, 8.0), cz=(100000.0, 250000.0))
    bins = cat.log_bins(0.5, 30.0, 10)
    kw = dict(weights1=w, weight_type="pair_product", output_rpavg=avg)
    got = mocks.DDrppi_mocks(1, 2, 1, 30.0, bins, ra.copy(), dec.copy(), cz.copy(), **kw)
    want = orc.DDrppi_mocks(1, 2, 30.0, bins, ra.copy(), dec.copy(), cz.copy(), **kw)
    assert got["npairs"].sum() > 0
    _check(got, want, "rpavg")
    kw = dict(output_savg=avg)
    got = mocks.DDsmu_mocks(1, 2, 1, 1.0, 8, bins, ra.copy(), dec.copy(), cz.copy(), **kw)
    want = orc.DDsmu_mocks(1, 2, 1.0, 8, bins, ra.copy(), dec.copy(), cz.copy(), **kw)
    _check(got, want, "savg")


@pytest.mark.parametrize("func", ["DDrppi_mocks", "DDsmu_mocks"])
def test_mocks_match_reference_library(reflibs_gsl, func):
    """The GPU survey counters against the reference's own DDrppi_mocks / DDsmu_mocks (compiled
    against the test-only GSL stand-in) on a 20,000-galaxy survey, weighted, with averages."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz = cat.survey(20000, 41, ra=(110.0, 200.0), dec=(-4.0, 50.0), cz=(5000.0, 18000.0))
    w = cat.weights(20000, 42)
    bins = cat.log_bins(0.1, 25.0, 14)
    kw = dict(weights1=w, weight_type="pair_product", isa="fallback")
    if func == "DDrppi_mocks":
        a = mocks.run_DDrppi_mocks(C.library(), 1, 1, 1, 40.0, bins, ra.copy(), dec.copy(), cz.copy(),
                                   output_rpavg=True, **kw)
        b = mocks.run_DDrppi_mocks(reflibs_gsl[func], 1, 1, 16, 40.0, bins, ra.copy(), dec.copy(), cz.copy(),
                                   output_rpavg=True, **kw)
        f = "rpavg"
    else:
        a = mocks.run_DDsmu_mocks(C.library(), 1, 2, 1, 1.0, 10, bins, ra.copy(), dec.copy(), cz.copy(),
                                  output_savg=True, **kw)
        b = mocks.run_DDsmu_mocks(reflibs_gsl[func], 1, 2, 16, 1.0, 10, bins, ra.copy(), dec.copy(), cz.copy(),
                                  output_savg=True, **kw)
        f = "savg"
    assert np.array_equal(a["npairs"], b["npairs"])
    assert int(np.sum(a["npairs"])) > 0
    np.testing.assert_allclose(a[f], b[f], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(a["weightavg"], b["weightavg"], rtol=1e-6, atol=1e-12)
