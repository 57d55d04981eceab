"""Split j columns: DD(r) and xi counted from a j lattice whose columns split every lattice column
2-4 ways per axis and whose slabs merge 1-8 lattice slabs (packed tasks over each chunk's
concatenated j ranges; CF_COLUMN_SPLIT=<split>,<merge> fixes the choice, which is read on every
call) give the counts of the unsplit work list bit for bit, and averages within the FP32 path's
tolerance: auto- and cross-correlations, periodic and not, anisotropic boxes, float32 inputs,
chunk lists longer than one packed task, and a work list that outgrows its first buffers."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SPLITS = ["2,1", "2,2", "3,4", "4,8"]


@pytest.fixture(scope="module")
def gpu():
    import corrfunc_gb300
    corrfunc_gb300.set_precision("fp32_refine")
    return corrfunc_gb300


def _count(gpu, monkeypatch, split, fn):
    monkeypatch.setenv("CF_COLUMN_SPLIT", split)
    res = fn()
    stats = gpu.last_stats()
    monkeypatch.delenv("CF_COLUMN_SPLIT")
    return res, stats


def _compare(got, want, rtol, fields=("ravg", "weightavg")):
    assert np.array_equal(np.asarray(got["npairs"], np.uint64), np.asarray(want["npairs"], np.uint64)), \
        "npairs differ:\n%s\n%s" % (list(got["npairs"]), list(want["npairs"]))
    for f in fields:
        if f in got.dtype.names:
            np.testing.assert_allclose(got[f], want[f], rtol=rtol, atol=1e-12)


def _uniform(n, box, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    return [(rng.random(n) * b).astype(dtype) for b in np.broadcast_to(np.asarray(box, float), (3,))]


CASES = {
    # periodic auto-correlation with separation averages
    "auto_periodic": dict(autocorr=1, n=30000, box=100.0, rmax=12.0, periodic=True),
    # anisotropic periodic box: the plane reach differs per axis
    "auto_aniso": dict(autocorr=1, n=30000, box=(50.0, 75.0, 120.0), rmax=10.0, periodic=True),
    # non-periodic, float32 positions
    "auto_open_f32": dict(autocorr=1, n=25000, box=80.0, rmax=9.0, periodic=False, dtype=np.float32),
    # weighted cross-correlation, different sizes
    "cross_weighted": dict(autocorr=0, n=20000, n2=15000, box=150.0, rmax=15.0, periodic=True, weights=True),
    # dense: a chunk's j list spans several packed tasks of 2048 positions
    "auto_dense": dict(autocorr=1, n=60000, box=50.0, rmax=8.0, periodic=True),
    # sparse, long reach: many short ranges per chunk, windows across the periodic boundary
    "cross_sparse": dict(autocorr=0, n=800, n2=1200, box=100.0, rmax=40.0, periodic=True),
}


def _run_case(name, c):
    from corrfunc_gb300 import theory
    dtype = c.get("dtype", np.float64)
    x, y, z = _uniform(c["n"], c["box"], 1, dtype)
    bins = np.logspace(-1, np.log10(c["rmax"]), 12)
    kw = dict(periodic=c["periodic"], output_ravg=True)
    if c["periodic"]:
        box = c["box"]
        kw["boxsize"] = tuple(box) if isinstance(box, tuple) else box
    if c["autocorr"]:
        if c.get("weights"):
            kw.update(weights1=np.ones_like(x), weight_type="pair_product")
        return lambda: theory.DD(1, 1, bins, x, y, z, **kw)
    x2, y2, z2 = _uniform(c["n2"], c["box"], 2, dtype)
    if c.get("weights"):
        rng = np.random.default_rng(3)
        kw.update(weights1=rng.uniform(0.5, 1.5, len(x)).astype(dtype),
                  weights2=rng.uniform(0.5, 1.5, len(x2)).astype(dtype), weight_type="pair_product")
    return lambda: theory.DD(0, 1, bins, x, y, z, X2=x2, Y2=y2, Z2=z2, **kw)


@pytest.mark.parametrize("split", SPLITS)
@pytest.mark.parametrize("name", sorted(CASES))
def test_split_matches_unsplit(gpu, monkeypatch, name, split):
    c = CASES[name]
    fn = _run_case(name, c)
    want, s1 = _count(gpu, monkeypatch, "1", fn)
    got, s2 = _count(gpu, monkeypatch, split, fn)
    assert s1["column_split"] == 1
    assert s2["column_split"] == int(split.split(",")[0])
    rtol = 1e-4 if c.get("dtype") == np.float32 else 1e-6
    _compare(got, want, rtol)


@pytest.mark.parametrize("split", ["3,4"])
def test_split_xi(gpu, monkeypatch, split):
    from corrfunc_gb300 import theory
    x, y, z = _uniform(30000, 100.0, 7)
    bins = np.logspace(-1, np.log10(15.0), 10)
    fn = lambda: theory.xi(100.0, 1, bins, x, y, z, output_ravg=True)  # noqa: E731
    want, _ = _count(gpu, monkeypatch, "1", fn)
    got, s = _count(gpu, monkeypatch, split, fn)
    assert s["column_split"] == 3
    _compare(got, want, 1e-6)
    np.testing.assert_allclose(got["xi"], want["xi"], rtol=1e-6, atol=1e-12)


def test_split_fp64_precision_stays_unsplit(gpu, monkeypatch):
    x, y, z = _uniform(5000, 60.0, 11)
    from corrfunc_gb300 import theory
    gpu.set_precision("fp64")
    try:
        _, s = _count(gpu, monkeypatch, "3,4",
                      lambda: theory.DD(1, 1, np.logspace(-1, 1, 8), x, y, z, periodic=True, boxsize=60.0))
    finally:
        gpu.set_precision("fp32_refine")
    assert s["column_split"] == 1


def test_split_work_list_resize(gpu, monkeypatch, tmp_path):
    """Packed tasks and range records that outgrow their first buffers (CF_TASK_CAPACITY=100 in a
    child process): both are resized and the count rerun, with the counts and averages of the
    in-process count."""
    from corrfunc_gb300 import theory
    x, y, z = _uniform(20000, 100.0, 91)
    path = tmp_path / "pts.npy"
    np.save(str(path), np.stack([x, y, z]))
    bins = np.logspace(-1, np.log10(12.0), 10)
    want, _ = _count(gpu, monkeypatch, "3,4", lambda: theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=100.0,
                                                                 output_ravg=True))
    code = ("import sys, numpy as np; sys.path.insert(0, %r)\n"
            "from corrfunc_gb300 import theory\n"
            "import corrfunc_gb300\n"
            "x, y, z = np.load(%r)\n"
            "r = theory.DD(1, 1, np.logspace(-1, np.log10(12.0), 10), x, y, z, periodic=True, boxsize=100.0,"
            " output_ravg=True)\n"
            "print(' '.join(str(int(v)) for v in r['npairs']))\n"
            "print(' '.join(repr(float(v)) for v in r['ravg']))\n"
            "s = corrfunc_gb300.last_stats()\n"
            "print(s['tasks'], s['column_split'])\n") % (os.path.dirname(HERE), str(path))
    env = dict(os.environ, CF_TASK_CAPACITY="100", CF_COLUMN_SPLIT="3,4")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.split("\n")
    assert [int(v) for v in lines[0].split()] == [int(v) for v in want["npairs"]]
    np.testing.assert_allclose([float(v) for v in lines[1].split()], want["ravg"], rtol=1e-12, atol=1e-15)
    tasks, split = (int(v) for v in lines[2].split())
    assert tasks > 100 and split == 3


def test_autotune_keeps_counts_and_reuses_its_choice(gpu):
    """The single-count autotuner: the first count of a shape times the splits and returns the
    same counts as an untuned count; the second count of that shape runs with the kept split."""
    from corrfunc_gb300 import theory
    x, y, z = _uniform(30000, 100.0, 21)
    bins = np.logspace(-1, np.log10(12.0), 12)
    gpu.set_autotune(False)
    want = theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=100.0, output_ravg=True)
    gpu.set_autotune(True)
    try:
        assert gpu.get_autotune()
        got1 = theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=100.0, output_ravg=True)
        s1 = gpu.last_stats()["column_split"]
        got2 = theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=100.0, output_ravg=True)
        s2 = gpu.last_stats()["column_split"]
    finally:
        gpu.set_autotune(False)
    assert 1 <= s1 <= 4 and s2 == s1
    _compare(got1, want, 1e-6)
    _compare(got2, got1, 0.0)


def test_find_fastest_wp_bin_refs(gpu):
    from corrfunc_gb300 import theory
    x, y, z = _uniform(5000, 100.0, 23)
    best, runtimes = theory.find_fastest_wp_bin_refs(100.0, 20.0, 1, np.logspace(-1, 1, 8), x, y, z, maxbinref=2,
                                                     nrepeats=1, return_runtimes=True)
    assert len(runtimes) == 8 and np.all(np.isfinite(runtimes["avg_time"]))
    assert all(1 <= v <= 2 for v in best)
    k = np.argmin(runtimes["avg_time"])
    assert best == (runtimes["nx"][k], runtimes["ny"][k], runtimes["nz"][k])


@pytest.mark.parametrize("name", ["auto_periodic", "auto_open_f32", "cross_weighted", "auto_dense"])
def test_chunk_walk_matches_work_list(gpu, monkeypatch, name):
    """CF_CHUNK_WALK=1: the pair kernel walks each chunk's neighbour columns itself (the own column's
    forward half first, in tiles that count only j > i) instead of taking a work list; the same
    counts and averages."""
    c = CASES[name]
    fn = _run_case(name, c)
    want = fn()
    monkeypatch.setenv("CF_CHUNK_WALK", "1")
    got = fn()
    stats = gpu.last_stats()
    monkeypatch.delenv("CF_CHUNK_WALK")
    assert stats["tasks"] == 0  # no work list
    rtol = 1e-4 if c.get("dtype") == np.float32 else 1e-6
    _compare(got, want, rtol)
