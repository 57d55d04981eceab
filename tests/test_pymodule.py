"""The CPython modules _countpairs / _countpairs_mocks (arguments of the reference's compiled
bindings): argument checking on the CPU, and on a GPU the same numbers as the ctypes front end."""
import numpy as np
import pytest


def _modules():
    try:
        from corrfunc_gb300 import _countpairs, _countpairs_mocks
    except ImportError as e:  # headers missing at build time
        pytest.skip("CPython modules not built: %s" % e)
    return _countpairs, _countpairs_mocks


def test_modules_export_the_reference_functions():
    cp, cpm = _modules()
    for name in ("countpairs", "countpairs_rp_pi", "countpairs_wp", "countpairs_xi", "countpairs_s_mu"):
        assert callable(getattr(cp, name))
    for name in ("countpairs_theta_mocks", "countpairs_rp_pi_mocks", "countpairs_s_mu_mocks"):
        assert callable(getattr(cpm, name))


def test_argument_errors_return_none(capfd):
    cp, cpm = _modules()
    x = np.random.default_rng(0).random(50)
    bins = "/nonexistent-bin-file"
    # unknown keyword, wrong positional type, 2-D positions, mixed dtypes, unknown weight type
    assert cp.countpairs(1, 1, bins, x, x, x, not_a_keyword=1) is None
    assert cp.countpairs(1, 1, bins, list(x), x, x) is None
    assert cp.countpairs(1, 1, bins, x.reshape(5, 10), x, x) is None
    assert cp.countpairs(1, 1, bins, x, x.astype(np.float32), x) is None
    assert cp.countpairs(1, 1, bins, x, x, x, weights1=np.ones((1, 50)), weight_type="inverse") is None
    # cross-correlation without the second set
    assert cp.countpairs(0, 1, bins, x, x, x) is None
    assert cpm.countpairs_theta_mocks(0, 1, bins, x, x) is None
    assert cpm.countpairs_rp_pi_mocks(0, 1, 1, 10.0, bins, x, x, x) is None
    assert cpm.countpairs_s_mu_mocks(1, 1, 1, 1.0, 5, bins, x, x, x.astype(np.float32)) is None
    assert "corrfunc_gb300" in capfd.readouterr().err


@pytest.mark.gpu
def test_modules_match_the_python_front_end():
    cp, cpm = _modules()
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks, theory
    L = 100.0
    x, y, z = cat.uniform_box(20000, L, 3)
    w = cat.weights(20000, 4)
    bins = cat.log_bins(0.5, 10.0, 8)
    with_w = dict(weights1=w.reshape(1, -1), weight_type="pair_product")

    got, t = cp.countpairs(1, 2, _binfile(bins), x, y, z, periodic=True, boxsize=(L, L, L), output_ravg=True,
                           c_api_timer=True, **with_w)
    want = theory.DD(1, 2, bins, x, y, z, weights1=w, weight_type="pair_product", periodic=True, boxsize=L,
                     output_ravg=True)
    assert [r[3] for r in got] == list(want["npairs"])
    np.testing.assert_allclose([r[2] for r in got], want["ravg"], rtol=1e-12)
    np.testing.assert_allclose([r[4] for r in got], want["weightavg"], rtol=1e-12)
    assert t > 0.0

    got, _ = cp.countpairs_rp_pi(1, 2, 20.0, _binfile(bins), x, y, z, periodic=True, boxsize=(L, L, L))
    want = theory.DDrppi(1, 2, 20.0, bins, x, y, z, periodic=True, boxsize=L)
    assert [r[4] for r in got] == list(want["npairs"])

    got, _ = cp.countpairs_s_mu(1, 2, _binfile(bins), 1.0, 5, x, y, z, periodic=True, boxsize=(L, L, L))
    want = theory.DDsmu(1, 2, bins, 1.0, 5, x, y, z, periodic=True, boxsize=L)
    assert [r[4] for r in got] == list(want["npairs"])

    got, _, cells = cp.countpairs_wp(L, 20.0, 2, _binfile(bins), x, y, z)
    want = theory.wp(L, 20.0, 2, bins, x, y, z)
    assert [r[4] for r in got] == list(want["npairs"])
    np.testing.assert_allclose([r[3] for r in got], want["wp"], rtol=1e-12)
    assert cells == []

    got, _ = cp.countpairs_xi(L, 2, _binfile(bins), x, y, z)
    want = theory.xi(L, 2, bins, x, y, z)
    assert [r[4] for r in got] == list(want["npairs"])

    ra, dec = cat.sky_cap(5000, 5)
    tb = cat.log_bins(0.05, 5.0, 8)
    got, _ = cpm.countpairs_theta_mocks(1, 2, _binfile(tb), ra.copy(), dec.copy(), output_thetaavg=True)
    want = mocks.DDtheta_mocks(1, 2, tb, ra.copy(), dec.copy(), output_thetaavg=True)
    assert [r[3] for r in got] == list(want["npairs"])
    np.testing.assert_allclose([r[2] for r in got], want["thetaavg"], rtol=1e-12)

    ra, dec, cz = cat.survey(4000, 6)
    mb = cat.log_bins(0.5, 10.0, 6)
    got, _ = cpm.countpairs_rp_pi_mocks(1, 1, 2, 12.0, _binfile(mb), ra.copy(), dec.copy(), cz.copy(),
                                        output_rpavg=True)
    want = mocks.DDrppi_mocks(1, 1, 2, 12.0, mb, ra.copy(), dec.copy(), cz.copy(), output_rpavg=True)
    assert [r[4] for r in got] == list(want["npairs"])
    assert [r[3] for r in got] == list(want["pimax"])
    got, _ = cpm.countpairs_s_mu_mocks(1, 2, 2, 0.9, 6, _binfile(mb), ra.copy(), dec.copy(), cz.copy())
    want = mocks.DDsmu_mocks(1, 2, 2, 0.9, 6, mb, ra.copy(), dec.copy(), cz.copy())
    assert [r[4] for r in got] == list(want["npairs"])


_FILES = []


def _binfile(edges):
    import tempfile
    f = tempfile.NamedTemporaryFile("w", suffix=".bins", delete=False)
    for lo, hi in zip(edges[:-1], edges[1:]):
        f.write("%.17g %.17g\n" % (lo, hi))
    f.close()
    _FILES.append(f.name)
    return f.name
