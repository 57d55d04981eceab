"""Points just past the edge of the periodic box, against the reference's own pair counters
(oracle/_ref).

xi and wp lattice the box [0, L) and clamp a point up to one cell past its top edge into the edge
cell (utils/gridlink_impl.c.src:165-172; a point less than a cell below 0 truncates into cell 0).
Their cell-pair list links cells by index with the period as offset
(utils/gridlink_impl.c.src:494-521), so across the periodic boundary it leaves out some pairs in
range that the minimum image would count; the GPU path applies the same links (npairs bit-exact,
averages within 1e-6).  DD, DDrppi and DDsmu lattice the data extent and need no links.  The
catalogue crowds a slab around the x boundary and moves the points within 0.6 of it past one
edge.  Points spanning more than the period make the call fail: the reference's end cells then
overlap across the boundary and its pruning by cell bounds drops further pairs, which is not
reproduced."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L = 100.0
NT = min(os.cpu_count() or 1, 8)
BINS = np.logspace(-1, 1, 9)  # rmax = 10


@pytest.fixture(scope="module")
def gpu():
    import corrfunc_gb300
    corrfunc_gb300.library()
    corrfunc_gb300.set_precision("fp32_refine")
    return corrfunc_gb300


def _catalogue(side, seed=3, n=6000, delta=0.6):
    """side: "top" (points within delta above 0 moved past L), "bottom" (within delta below L moved
    below 0) or "both"."""
    rng = np.random.default_rng(seed)
    x, y, z = (rng.random(n) * L for _ in range(3))
    k = n // 3
    x[:k] = (rng.random(k) * 24.0 - 12.0) % L
    if side in ("top", "both"):
        x[x < delta] += L
    if side in ("bottom", "both"):
        m = (x > L - delta) & (x < L)
        x[m] -= L
    w = rng.uniform(0.5, 1.5, n)
    return x, y, z, w


def _run(lib, func, nthreads, x, y, z, w):
    from corrfunc_gb300 import theory
    if func == "DD":
        return theory.run_DD(lib, 1, nthreads, BINS, x, y, z, weights1=w, weight_type="pair_product", periodic=True,
                             boxsize=L, output_ravg=True, isa="fallback")
    if func == "DDcross":
        x2, y2, z2 = (np.roll(v, 17) for v in (x, y, z))
        return theory.run_DD(lib, 0, nthreads, BINS, x, y, z, X2=x2, Y2=(y2 + 0.25) % L, Z2=z2, periodic=True,
                             boxsize=L, output_ravg=True, isa="fallback")
    if func == "xi":
        return theory.run_xi(lib, L, nthreads, BINS, x, y, z, weights=w, weight_type="pair_product", output_ravg=True,
                             isa="fallback")
    if func == "wp":
        return theory.run_wp(lib, L, 10.0, nthreads, BINS, x, y, z, weights=w, weight_type="pair_product",
                             output_rpavg=True, isa="fallback")
    if func == "DDrppi":
        return theory.run_DDrppi(lib, 1, nthreads, 10.0, BINS, x, y, z, boxsize=L, output_rpavg=True, isa="fallback")
    return theory.run_DDsmu(lib, 1, nthreads, BINS, 1.0, 5, x, y, z, boxsize=L, output_savg=True, isa="fallback")


AVG = {"DD": "ravg", "DDcross": "ravg", "xi": "ravg", "wp": "rpavg", "DDrppi": "rpavg", "DDsmu": "savg"}


@pytest.mark.parametrize("side", ["top", "bottom"])
@pytest.mark.parametrize("func", ["DD", "DDcross", "xi", "wp", "DDrppi", "DDsmu"])
def test_points_past_the_box_edge_match_reference(gpu, reflibs, func, side):
    from corrfunc_gb300 import _capi as C
    x, y, z, w = _catalogue(side)
    got = _run(C.library(), func, 1, x, y, z, w)
    want = _run(reflibs["DD" if func == "DDcross" else func], func, NT, x, y, z, w)
    assert np.array_equal(np.asarray(got["npairs"], np.uint64), np.asarray(want["npairs"], np.uint64)), \
        "npairs differ:\n%s\n%s" % (list(got["npairs"]), list(want["npairs"]))
    assert int(np.sum(got["npairs"])) > 0
    for f in (AVG[func], "weightavg"):
        np.testing.assert_allclose(np.asarray(got[f], float), np.asarray(want[f], float), rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("func", ["wp", "xi"])
def test_links_leave_out_pairs_in_range(gpu, func):
    """The cases above are not vacuous: the links leave out pairs that the same catalogue wrapped
    into the box counts."""
    from corrfunc_gb300 import _capi as C
    x, y, z, w = _catalogue("bottom")
    past = _run(C.library(), func, 1, x, y, z, w)["npairs"]
    wrapped = _run(C.library(), func, 1, x % L, y, z, w)["npairs"]
    assert int(np.sum(wrapped)) > int(np.sum(past))


@pytest.mark.parametrize("func", ["DD", "xi", "wp", "DDrppi", "DDsmu"])
def test_points_spanning_more_than_the_period_fail_loudly(gpu, capfd, func):
    from corrfunc_gb300 import _capi as C
    x, y, z, w = _catalogue("both")
    with pytest.raises(RuntimeError):
        _run(C.library(), func, 1, x, y, z, w)
    assert "more than the periodic length" in capfd.readouterr().err
