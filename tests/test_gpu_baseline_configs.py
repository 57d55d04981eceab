"""GPU parity at the benchmark configurations' full sizes, against the reference's own pair
counters compiled into oracle/_ref (FALLBACK kernels on every host; the reference's
countpairs_impl.c.src:609-690 finalisation).  npairs bit-exact; averages within 1e-6 relative
for double inputs and 1e-4 for float inputs (float inputs are compared with the reference's
double-precision run on the same values upcast to double).

  * DD auto-correlation, 300,000 uniform points in a periodic L = 420 box, 20 log bins 0.1-25,
    ravg;
  * DD cross-correlation of two 2,000,000-point clustered catalogues (80 % in Gaussian blobs of
    sigma 2, Poisson occupancy 80), periodic L = 1000, pair_product weights U[0.5, 1.5], 25 log
    bins 0.1-50, float64 and float32 -- the benchmark's default workload, same seeds;
  * DDrppi, wp and DDsmu on 1,000,000 clustered points in L = 1000 (14 log rp bins 0.1-25,
    pimax 40; 20 log s bins 0.1-50, 10 mu bins);
  * DDtheta on the first 200,000 points of a 1,000,000-point cap (RA 0-90, sin DEC uniform up to
    60 deg), 20 log bins 0.01-10 deg, thetaavg, RA / DEC linking on.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def gpu():
    import corrfunc_gb300
    corrfunc_gb300.library()
    corrfunc_gb300.set_precision("fp32_refine")
    yield corrfunc_gb300
    corrfunc_gb300.set_precision("fp32_refine")


def _same(a, b, field, rtol):
    assert np.array_equal(np.asarray(a["npairs"], np.uint64), np.asarray(b["npairs"], np.uint64)), \
        "npairs differ:\n%s\n%s" % (list(a["npairs"]), list(b["npairs"]))
    for f in (field, "weightavg"):
        np.testing.assert_allclose(np.asarray(a[f], float), np.asarray(b[f], float), rtol=rtol, atol=1e-12)


def test_cfg_dd_auto_300k_uniform(gpu, reflibs):
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    x, y, z = cat.uniform_box(300_000, 420.0, 0)
    bins = cat.log_bins(0.1, 25.0, 20)
    kw = dict(periodic=True, boxsize=420.0, output_ravg=True, isa="fallback")
    got = theory.run_DD(C.library(), 1, 1, bins, x, y, z, **kw)
    want = theory.run_DD(reflibs["DD"], 1, NT, bins, x, y, z, **kw)
    _same(got, want, "ravg", 1e-6)
    assert int(got["npairs"].sum()) > 0


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_cfg_dd_cross_2M_clustered_weighted(gpu, reflibs, dtype):
    """The benchmark's default workload (same generator, seeds 1 / 2, weight seeds 101 / 102)."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 1000.0
    x1, y1, z1 = cat.clustered_box(2_000_000, L, 1, dtype=dtype)
    x2, y2, z2 = cat.clustered_box(2_000_000, L, 2, dtype=dtype)
    w1 = cat.weights(2_000_000, 101, dtype=dtype)
    w2 = cat.weights(2_000_000, 102, dtype=dtype)
    bins = cat.log_bins(0.1, 50.0, 25)
    got = theory.run_DD(C.library(), 0, 1, bins, x1, y1, z1, weights1=w1, X2=x2, Y2=y2, Z2=z2, weights2=w2,
                        weight_type="pair_product", periodic=True, boxsize=L, output_ravg=True, isa="fallback")
    up = (lambda a: a.astype(np.float64)) if dtype == np.float32 else (lambda a: a)
    want = theory.run_DD(reflibs["DD"], 0, NT, bins, up(x1), up(y1), up(z1), weights1=up(w1), X2=up(x2), Y2=up(y2),
                         Z2=up(z2), weights2=up(w2), weight_type="pair_product", periodic=True, boxsize=L,
                         output_ravg=True, isa="fallback")
    _same(got, want, "ravg", 1e-6 if dtype == np.float64 else 1e-4)
    assert int(got["npairs"].sum()) > 2_000_000_000


@pytest.fixture(scope="module")
def cfg3_points():
    from corrfunc_gb300 import catalogs as cat
    return cat.clustered_box(1_000_000, 1000.0, 3)


@pytest.mark.parametrize("func", ["DDrppi", "wp", "DDsmu"])
def test_cfg_2d_counters_1M_clustered(gpu, reflibs, cfg3_points, func):
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    x, y, z = cfg3_points
    L = 1000.0
    lib = C.library()
    if func == "DDrppi":
        rp = cat.log_bins(0.1, 25.0, 14)
        got = theory.run_DDrppi(lib, 1, 1, 40.0, rp, x, y, z, boxsize=L, output_rpavg=True, isa="fallback")
        want = theory.run_DDrppi(reflibs["DDrppi"], 1, NT, 40.0, rp, x, y, z, boxsize=L, output_rpavg=True,
                                 isa="fallback")
        field = "rpavg"
    elif func == "wp":
        rp = cat.log_bins(0.1, 25.0, 14)
        got = theory.run_wp(lib, L, 40.0, 1, rp, x, y, z, output_rpavg=True, isa="fallback")
        want = theory.run_wp(reflibs["wp"], L, 40.0, NT, rp, x, y, z, output_rpavg=True, isa="fallback")
        field = "rpavg"
        np.testing.assert_allclose(got["wp"], want["wp"], rtol=1e-6, atol=1e-9)
    else:
        sb = cat.log_bins(0.1, 50.0, 20)
        got = theory.run_DDsmu(lib, 1, 1, sb, 1.0, 10, x, y, z, boxsize=L, output_savg=True, isa="fallback")
        want = theory.run_DDsmu(reflibs["DDsmu"], 1, NT, sb, 1.0, 10, x, y, z, boxsize=L, output_savg=True,
                                isa="fallback")
        field = "savg"
    _same(got, want, field, 1e-6)
    assert int(np.sum(got["npairs"])) > 0


def test_cfg_ddtheta_cap_200k_of_1M(gpu, reflibs):
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec = cat.sky_cap(1_000_000, 4)
    n = 200_000
    tb = cat.log_bins(0.01, 10.0, 20)
    kw = dict(output_thetaavg=True, link_in_dec=True, link_in_ra=True, isa="fallback")
    got = mocks.run_DDtheta_mocks(C.library(), 1, 1, tb, ra[:n].copy(), dec[:n].copy(), **kw)
    want = mocks.run_DDtheta_mocks(reflibs["DDtheta"], 1, NT, tb, ra[:n].copy(), dec[:n].copy(), **kw)
    _same(got, want, "thetaavg", 1e-6)
    assert int(got["npairs"].sum()) > 0


def test_cfg_ddtheta_full_cap_fp32_equals_fp64(gpu):
    """The whole 1,000,000-point cap: the FP32 classification with FP64 re-evaluation gives the
    same counts as the form that evaluates every pair in FP64 (the reference's own run of this
    size takes minutes on the host)."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec = cat.sky_cap(1_000_000, 4)
    tb = cat.log_bins(0.01, 10.0, 20)
    out = []
    for prec in ("fp32_refine", "fp64"):
        gpu.set_precision(prec)
        r = mocks.DDtheta_mocks(1, 1, tb, ra.copy(), dec.copy(), output_thetaavg=False, isa="fallback")
        out.append(np.asarray(r["npairs"], np.uint64).copy())
    gpu.set_precision("fp32_refine")
    assert np.array_equal(out[0], out[1])
    assert int(out[0].sum()) > 0
