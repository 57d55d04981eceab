"""Batched DD(r) cross-correlations (cf_gpu_batch_plan / cf_gpu_batch_run): every catalogue's
result equals countpairs() on the same arrays, across replays of the captured graph, with and
without the layout tuner, for float64 and float32 positions, weighted and not, in the merged form
(one lattice for all catalogues, chunk tasks) and the per-catalogue form."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_AVG = {np.float64: 1e-6, np.float32: 1e-4}


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return t


def _catalogues(dtype, sizes, n2, L, seed):
    from corrfunc_gb300 import catalogs as cat
    cats = []
    for k, n in enumerate(sizes):
        if n == 0:
            cats.append([np.zeros(0, dtype) for _ in range(4)])
            continue
        x, y, z = cat.clustered_box(n, L, seed + k) if k % 2 else cat.uniform_box(n, L, seed + k)
        w = np.random.default_rng(seed + 100 + k).uniform(0.5, 1.5, n)
        cats.append([a.astype(dtype) for a in (x, y, z, w)])
    x, y, z = cat.uniform_box(n2, L, seed + 999)
    w = np.random.default_rng(seed + 1999).uniform(0.5, 1.5, n2)
    second = [a.astype(dtype) for a in (x, y, z, w)]
    return cats, second


def _dev(torch, arrays):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


def _check(got, want, dtype):
    assert np.array_equal(got["npairs"], want["npairs"])
    np.testing.assert_allclose(got["ravg"], want["ravg"], rtol=RTOL_AVG[dtype], atol=1e-9)
    np.testing.assert_allclose(got["weightavg"], want["weightavg"], rtol=RTOL_AVG[dtype], atol=1e-9)


@pytest.mark.parametrize("dtype,weights,autotune", [(np.float64, True, True), (np.float32, True, False),
                                                    (np.float64, False, False)])
def test_batch_matches_countpairs(torch, dtype, weights, autotune):
    from corrfunc_gb300 import theory
    L = 200.0
    bins = np.logspace(np.log10(0.3), np.log10(15.0), 13)
    cats, second = _catalogues(dtype, [3000, 0, 12000, 700, 5000], 20000, L, 5)
    dev = [_dev(torch, c) for c in cats]
    dsec = _dev(torch, second)
    torch.cuda.synchronize()
    wt = "pair_product" if weights else None
    batch = theory.DDCrossBatch(bins, dev, dsec, periodic=True, boxsize=L, output_ravg=True, weight_type=wt,
                                autotune=autotune)
    try:
        for _ in range(2):
            got = batch.run()
            assert len(got) == len(cats)
            for c, g in zip(cats, got):
                kw = dict(X2=second[0], Y2=second[1], Z2=second[2], periodic=True, boxsize=L, output_ravg=True)
                if weights:
                    kw.update(weights1=c[3], weights2=second[3], weight_type="pair_product")
                if len(c[0]) == 0:
                    assert not g["npairs"].any()
                    continue
                want = theory.DD(0, 1, bins, c[0], c[1], c[2], **kw)
                _check(g, want, dtype)
        assert sum(int(g["npairs"].sum()) for g in got) > 0
    finally:
        batch.close()


@pytest.mark.parametrize("form", ["per_catalogue", "many_bins"])
def test_batch_other_forms_match_countpairs(torch, monkeypatch, form):
    """The per-catalogue form of a batch (one lattice and chunk range per catalogue on one work
    list): chosen with CF_BATCH_MERGED=0, and by itself for more bins than the byte table holds."""
    from corrfunc_gb300 import theory
    L = 200.0
    if form == "per_catalogue":
        monkeypatch.setenv("CF_BATCH_MERGED", "0")
        bins = np.logspace(np.log10(0.3), np.log10(15.0), 13)
    else:
        bins = np.logspace(np.log10(0.3), np.log10(15.0), 141)
    cats, second = _catalogues(np.float64, [3000, 9000, 700], 20000, L, 17)
    dev = [_dev(torch, c) for c in cats]
    dsec = _dev(torch, second)
    torch.cuda.synchronize()
    batch = theory.DDCrossBatch(bins, dev, dsec, periodic=True, boxsize=L, output_ravg=True,
                                weight_type="pair_product", autotune=False)
    try:
        got = batch.run()
    finally:
        batch.close()
    for c, g in zip(cats, got):
        want = theory.DD(0, 1, bins, c[0], c[1], c[2], weights1=c[3], X2=second[0], Y2=second[1], Z2=second[2],
                         weights2=second[3], weight_type="pair_product", periodic=True, boxsize=L, output_ravg=True)
        _check(g, want, np.float64)


def test_batch_replays_new_contents(torch):
    """The graph reads the arrays it was planned with: new contents of the same size give new counts."""
    from corrfunc_gb300 import theory
    L = 150.0
    bins = np.logspace(np.log10(0.5), np.log10(12.0), 9)
    cats, second = _catalogues(np.float64, [4000, 2500], 15000, L, 21)
    dev = [_dev(torch, c) for c in cats]
    dsec = _dev(torch, second)
    torch.cuda.synchronize()
    batch = theory.DDCrossBatch(bins, dev, dsec, periodic=True, boxsize=L, autotune=False)
    try:
        first = batch.run()
        from corrfunc_gb300 import catalogs as cat
        fresh = list(cat.clustered_box(2500, L, 4242))  # same generator as catalogue 1, new draw
        for k in range(3):
            dev[1][k].copy_(torch.from_numpy(fresh[k]))
        torch.cuda.synchronize()
        again = batch.run()
        assert np.array_equal(again[0]["npairs"], first[0]["npairs"])
        want = theory.DD(0, 1, bins, fresh[0], fresh[1], fresh[2], X2=second[0], Y2=second[1], Z2=second[2],
                         periodic=True, boxsize=L)
        assert np.array_equal(again[1]["npairs"], want["npairs"])
    finally:
        batch.close()


def test_batch_rejects_host_arrays_and_bad_weights(torch):
    from corrfunc_gb300 import theory
    x = np.zeros(10)
    with pytest.raises(TypeError):
        theory.DDCrossBatch([0.1, 1.0], [(x, x, x)], (x, x, x), periodic=False)
    d = torch.zeros(10, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        theory.DDCrossBatch([0.1, 1.0], [(d, d, d)], (d, d, d[:5]), periodic=False)


def test_batch_replay_outside_planned_box_fails_loudly(torch):
    """Non-periodic plans cover the planned extent only: a replay with a point beyond it is refused."""
    from corrfunc_gb300 import theory
    L = 100.0
    cats, second = _catalogues(np.float64, [2000], 8000, L, 31)
    dev = [_dev(torch, c) for c in cats]
    dsec = _dev(torch, second)
    torch.cuda.synchronize()
    batch = theory.DDCrossBatch(np.array([0.5, 2.0, 8.0]), dev, dsec, periodic=False, autotune=False)
    try:
        batch.run()
        dev[0][0][0] = 3.0 * L
        torch.cuda.synchronize()
        with pytest.raises(RuntimeError):
            batch.run()
    finally:
        batch.close()


def test_batch_matches_reference_library(torch, reflibs):
    """A few catalogues of a batch against the reference's own countpairs() (oracle/_ref) on the
    same float64 values: clustered catalogues against one uniform catalogue, pair_product weights,
    ravg -- npairs bit-exact, averages within 1e-6."""
    from corrfunc_gb300 import theory
    L = 300.0
    bins = np.logspace(np.log10(0.1), np.log10(25.0), 21)
    cats, second = _catalogues(np.float64, [40000, 9000, 25000], 60000, L, 31)
    dev = [_dev(torch, c) for c in cats]
    dsec = _dev(torch, second)
    torch.cuda.synchronize()
    batch = theory.DDCrossBatch(bins, dev, dsec, periodic=True, boxsize=L, output_ravg=True,
                                weight_type="pair_product", autotune=False)
    try:
        got = batch.run()
    finally:
        batch.close()
    for c, g in zip(cats, got):
        want = theory.run_DD(reflibs["DD"], 0, 8, bins, c[0], c[1], c[2], weights1=c[3], X2=second[0], Y2=second[1],
                             Z2=second[2], weights2=second[3], weight_type="pair_product", periodic=True, boxsize=L,
                             output_ravg=True, isa="fallback")
        assert np.array_equal(g["npairs"], want["npairs"])
        assert int(g["npairs"].sum()) > 0
        np.testing.assert_allclose(g["ravg"], want["ravg"], rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(g["weightavg"], want["weightavg"], rtol=1e-6, atol=1e-12)
