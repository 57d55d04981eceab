"""The reference's own Python wrappers (Corrfunc.theory.DD / DDrppi / DDsmu / wp / xi / vpf,
Corrfunc.mocks.DDtheta_mocks / DDrppi_mocks / DDsmu_mocks, unchanged) running on this project's
CPython modules: the drop-in at the Python layer (Corrfunc/theory/DD.py:205-284 calls
Corrfunc._countpairs.countpairs with its own format string and keywords).  Argument checks of
the wrappers run on the CPU; the counts are checked against the golden vectors on the GPU."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402
import ref_wrappers  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))
WRAPPER = {"DD": ("theory", "DD"), "DDrppi": ("theory", "DDrppi"), "DDsmu": ("theory", "DDsmu"),
           "wp": ("theory", "wp"), "xi": ("theory", "xi"), "DDtheta": ("mocks", "DDtheta_mocks")}


def test_reference_wrappers_import_and_check_arguments():
    """The unchanged wrappers import on top of the new modules and raise their own errors before
    any count (no GPU needed)."""
    Corrfunc = ref_wrappers.load()
    from Corrfunc.theory import DD, DDsmu
    x = np.random.default_rng(0).random(10)
    with pytest.raises(ValueError):
        DD(1, 1, [0.1, 0.2], x, x, x, periodic=True, boxsize=None)
    with pytest.raises(ValueError):
        DD(0, 1, [0.1, 0.2], x, x, x, periodic=False)  # cross-correlation without X2/Y2/Z2
    with pytest.raises(ValueError):
        DDsmu(1, 1, [0.1, 0.2], 1.5, 10, x, x, x, boxsize=1.0)  # mu_max beyond 1
    import corrfunc_gb300._countpairs as cp
    assert Corrfunc._countpairs is cp and DD.__module__ == "Corrfunc.theory.DD"


@pytest.mark.gpu
def test_reference_dd_wrapper_reproduces_its_doctest():
    """Corrfunc/theory/DD.py:166-202: N = 10,000 uniform points (numpy seed 42) in L = 420,
    theory/tests/bins, pair_product with unit weights, ravg -- the printed table."""
    Corrfunc = ref_wrappers.load()
    from Corrfunc.theory.DD import DD
    d = GOLDEN["dd_doctest"]
    np.random.seed(d["seed"])
    X = np.random.uniform(0, d["boxsize"], d["N"])
    Y = np.random.uniform(0, d["boxsize"], d["N"])
    Z = np.random.uniform(0, d["boxsize"], d["N"])
    res = DD(1, 4, np.array(d["edges"]), X, Y, Z, weights1=np.ones_like(X), weight_type="pair_product",
             output_ravg=True, boxsize=d["boxsize"], periodic=True)
    table = np.array(d["doctest_table"])
    assert list(res["npairs"]) == [int(v) for v in table[:, 3]]
    np.testing.assert_allclose(res["ravg"], table[:, 2], atol=5e-7)
    np.testing.assert_allclose(res["weightavg"], table[:, 4], atol=5e-7)
    np.testing.assert_allclose(res["ravg"], d["reference"]["avg"], rtol=1e-6)
    assert Corrfunc.__version__ == "2.5.3"


@pytest.mark.gpu
@pytest.mark.parametrize("case", cases.CASES, ids=[c["name"] for c in cases.CASES])
def test_reference_wrappers_match_golden(case):
    """Every golden case through the reference's own wrapper of its counter."""
    Corrfunc = ref_wrappers.load()
    mod, name = WRAPPER[case["func"]]
    fn = getattr(getattr(Corrfunc, mod), name)
    args, kw = cases.make_inputs(case)
    if case["func"] in ("DD", "DDrppi", "DDsmu") and not case["periodic"]:
        kw.pop("boxsize", None)
    res = fn(*args, **kw)
    if isinstance(res, tuple):
        res = res[0]
    gold = GOLDEN["cases"][case["name"]]
    assert [int(v) for v in res["npairs"]] == gold["npairs"]
    rtol = 1e-4 if case["dtype"] == "f4" else 1e-6
    np.testing.assert_allclose(res[cases.AVG_FIELD[case["func"]]], gold["avg"], rtol=rtol, atol=1e-12)
    np.testing.assert_allclose(res["weightavg"], gold["weightavg"], rtol=rtol, atol=1e-12)


@pytest.mark.gpu
def test_reference_wp_wrapper_returns_cell_timings():
    """Corrfunc/theory/wp.py:516-550: with c_cell_timer the wrapper converts the module's per-cell
    list into its structured array (N1, N2, time_in_ns, cellidx1, cellidx2, tid)."""
    ref_wrappers.load()
    from Corrfunc.theory.wp import wp
    from corrfunc_gb300 import catalogs as cat
    x, y, z = cat.uniform_box(20000, 100.0, 3)
    res, api_time, cells = wp(100.0, 10.0, 1, cat.log_bins(0.5, 10.0, 8), x, y, z, c_api_timer=True,
                              c_cell_timer=True)
    assert api_time > 0.0
    assert len(cells) > 0
    assert set(cells.dtype.names) == {"N1", "N2", "time_in_ns", "cellidx1", "cellidx2", "tid"}
    assert (cells["N1"] > 0).all() and (cells["N2"] > 0).all() and (cells["time_in_ns"] >= 0).all()
    # the per-task pair counts (each task's window) bound the pairs the GPU evaluated (box pruning
    # skips the j points out of a chunk's reach)
    import corrfunc_gb300
    window = int(np.sum(cells["N1"].astype(np.int64) * cells["N2"]))
    assert 0 < corrfunc_gb300.last_stats()["pairs_evaluated"] <= window
