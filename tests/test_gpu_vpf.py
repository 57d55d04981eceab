"""Counts in spheres (countspheres / countspheres_mocks) on the GPU against the oracle: every pN
count exact, for periodic and non-periodic boxes, custom refine factors (including lattices so
coarse that the neighbour walk visits a cell twice, as the reference's does), float32 inputs,
survey catalogues with centres read from a file or drawn from randoms above a neighbour
threshold (the chosen centres are written to the file as the reference writes them)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _counts(res, norm):
    return np.rint(res["pN"] * norm).astype(np.int64)


@pytest.mark.parametrize("periodic,refine,seed", [(True, (1, 1, 1), -1234), (True, (2, 2, 1), 7),
                                                  (False, (1, 1, 1), 11), (False, (2, 1, 3), 0)])
def test_vpf_matches_oracle(orc, periodic, refine, seed):
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 200.0
    x, y, z = cat.clustered_box(60000, L, 5)
    kw = dict(periodic=periodic, boxsize=L)
    got = theory.vpf(9.0, 9, 5000, 7, seed, x, y, z, xbin_refine_factor=refine[0], ybin_refine_factor=refine[1],
                     zbin_refine_factor=refine[2], **kw)
    want, counts = orc.vpf(9.0, 9, 5000, 7, seed, x, y, z, refine=refine, **kw)
    np.testing.assert_array_equal(got["rmax"], want["rmax"])
    assert np.array_equal(_counts(got, 5000), counts.astype(np.int64))
    np.testing.assert_allclose(got["pN"], want["pN"], rtol=0, atol=1e-15)
    assert counts[:, 0].sum() > 0 and counts[:, 1:].sum() > 0


def test_vpf_coarse_lattice_revisits_cells(orc):
    """max_cells_per_dim = 3 with refine 2: the reference's neighbour walk wraps onto the same cells
    more than once (counting those points again); the GPU walk does the same."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 60.0
    x, y, z = cat.uniform_box(3000, L, 9)
    got = theory.vpf(8.0, 4, 2000, 30, 3, x, y, z, periodic=True, boxsize=L, xbin_refine_factor=2,
                     ybin_refine_factor=2, zbin_refine_factor=2, max_cells_per_dim=3)
    want, counts = orc.vpf(8.0, 4, 2000, 30, 3, x, y, z, periodic=True, boxsize=L, refine=(2, 2, 2),
                           max_cells_per_dim=3)
    assert np.array_equal(_counts(got, 2000), counts.astype(np.int64))


def test_vpf_float32_inputs(orc):
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 150.0
    x, y, z = (a.astype(np.float32) for a in cat.uniform_box(40000, L, 13))
    got = theory.vpf(6.0, 6, 3000, 5, 99, x, y, z, periodic=True, boxsize=L)
    want, counts = orc.vpf(6.0, 6, 3000, 5, 99, *(a.astype(np.float64) for a in (x, y, z)), periodic=True, boxsize=L)
    assert np.array_equal(_counts(got, 3000), counts.astype(np.int64))


def test_vpf_mocks_centres_from_randoms_and_file(orc, tmp_path):
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz = cat.survey(30000, 17)
    rra, rdec, rcz = cat.survey(60000, 18, frac_clustered=0.0)
    fn = str(tmp_path / "centres.txt")
    args = (ra.copy(), dec.copy(), cz.copy(), rra.copy(), rdec.copy(), rcz.copy())
    want, counts, cen = orc.vpf_mocks(5.0, 5, 4000, 6, 3, None, 1, *args)
    got = mocks.vpf_mocks(5.0, 5, 4000, 6, 3, fn, 1, *args)
    n = len(cen)
    assert n == 4000
    assert np.array_equal(_counts(got, n), counts.astype(np.int64))
    rows = [ln.split() for ln in open(fn).read().splitlines() if ln.strip()]
    assert len(rows) == n
    written = np.array([[float(v) for v in r[:3]] for r in rows])
    np.testing.assert_allclose(written, cen, rtol=0, atol=5e-7)
    assert all(float(r[3]) == 5.0 for r in rows)
    # a second call reads the centres back from the file (rounded to 6 decimals as written)
    again = mocks.vpf_mocks(5.0, 5, 4000, 6, 3, fn, 1, *args)
    want2, counts2, _ = orc.vpf_mocks(5.0, 5, 4000, 6, 3, fn, 1, *args)
    assert np.array_equal(_counts(again, 4000), counts2.astype(np.int64))


def test_vpf_pymodule_matches_front_end():
    try:
        from corrfunc_gb300 import _countpairs
    except ImportError as e:
        pytest.skip("CPython modules not built: %s" % e)
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 100.0
    x, y, z = cat.uniform_box(20000, L, 21)
    rows, t = _countpairs.countspheres_vpf(5.0, 5, 1000, 4, 42, x, y, z, boxsize=(L, L, L), c_api_timer=True)
    want = theory.vpf(5.0, 5, 1000, 4, 42, x, y, z, periodic=True, boxsize=L)
    assert [r[0] for r in rows] == list(want["rmax"])
    assert np.array_equal(np.array([r[1:] for r in rows]), want["pN"])
    assert t > 0.0


@pytest.mark.parametrize("periodic", [True, False])
def test_vpf_matches_reference_library(reflibs_gsl, periodic):
    """countspheres on the GPU against the reference's own theory vpf (its MT19937 sphere centres
    from the test-only GSL stand-in): 200,000 clustered points, 20,000 spheres, every pN count."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 300.0
    x, y, z = cat.clustered_box(200000, L, 23)
    got = theory.run_vpf(C.library(), 8.0, 8, 20000, 6, 77, x, y, z, periodic=periodic, boxsize=L)
    want = theory.run_vpf(reflibs_gsl["vpf"], 8.0, 8, 20000, 6, 77, x, y, z, periodic=periodic, boxsize=L)
    np.testing.assert_array_equal(got["rmax"], want["rmax"])
    assert np.array_equal(_counts(got, 20000), _counts(want, 20000))
    assert _counts(got, 20000)[:, 1:].sum() > 0
