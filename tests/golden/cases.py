"""Seeded parity cases shared by the golden-fixture generator and the tests.

Each case names a public function, its arguments and a seeded input recipe; ``make_inputs``
rebuilds the exact arrays on any machine (numpy PCG64 streams are stable across versions).
"""
import numpy as np

from corrfunc_gb300 import catalogs as cat


# shift of the "offset" kind: a uniform box far from the origin on every axis
OFFSET = (1.0e5, -3.0e4, 2.0e6)


def _box(kind, n, L, seed, dtype):
    if kind == "uniform":
        return cat.uniform_box(n, L, seed, dtype)
    if kind == "offset":
        x, y, z = cat.uniform_box(n, L, seed, np.float64)
        return tuple(np.asarray(a + o, dtype=dtype) for a, o in zip((x, y, z), OFFSET))
    return cat.clustered_box(n, L, seed, dtype=dtype, sigma=L / 200.0, mean_occupancy=40.0)


CASES = [
    dict(name="dd_auto_uniform_w", func="DD", autocorr=1, kind="uniform", n1=5000, L=100.0, seed=11,
         bins=("log", 0.5, 20.0, 10), periodic=True, weights=True, avg=True, dtype="f8"),
    dict(name="dd_cross_clustered_nonperiodic", func="DD", autocorr=0, kind="clustered", n1=3000, n2=4000,
         L=200.0, seed=12, bins=("log", 0.1, 25.0, 12), periodic=False, weights=True, avg=True, dtype="f8"),
    dict(name="dd_auto_float32", func="DD", autocorr=1, kind="uniform", n1=5000, L=100.0, seed=13,
         bins=("log", 0.5, 20.0, 10), periodic=True, weights=False, avg=True, dtype="f4"),
    dict(name="dd_cross_periodic_clustered", func="DD", autocorr=0, kind="clustered", n1=4000, n2=3000,
         L=150.0, seed=14, bins=("log", 0.1, 30.0, 15), periodic=True, weights=True, avg=False, dtype="f8"),
    dict(name="rppi_auto_clustered", func="DDrppi", autocorr=1, kind="clustered", n1=4000, L=150.0, seed=21,
         bins=("log", 0.2, 15.0, 8), pimax=12.0, periodic=True, weights=True, avg=True, dtype="f8"),
    dict(name="rppi_cross_nonperiodic", func="DDrppi", autocorr=0, kind="uniform", n1=3000, n2=3500, L=80.0,
         seed=22, bins=("log", 0.5, 10.0, 6), pimax=9.0, periodic=False, weights=False, avg=True, dtype="f8"),
    dict(name="smu_auto_periodic", func="DDsmu", autocorr=1, kind="clustered", n1=4000, L=120.0, seed=31,
         bins=("log", 0.5, 20.0, 8), mu_max=1.0, nmu=5, periodic=True, weights=True, avg=True, dtype="f8"),
    dict(name="smu_cross_mu05", func="DDsmu", autocorr=0, kind="uniform", n1=3000, n2=3000, L=80.0, seed=32,
         bins=("log", 0.5, 15.0, 6), mu_max=0.5, nmu=10, periodic=True, weights=False, avg=True, dtype="f8"),
    dict(name="wp_uniform", func="wp", autocorr=1, kind="uniform", n1=5000, L=100.0, seed=41,
         bins=("log", 0.3, 15.0, 8), pimax=10.0, periodic=True, weights=True, avg=True, dtype="f8"),
    dict(name="xi_clustered", func="xi", autocorr=1, kind="clustered", n1=5000, L=100.0, seed=51,
         bins=("log", 0.3, 20.0, 10), periodic=True, weights=False, avg=True, dtype="f8"),
    dict(name="theta_auto_cap", func="DDtheta", autocorr=1, kind="cap", n1=4000, seed=61,
         bins=("log", 0.01, 10.0, 10), weights=False, avg=True, dtype="f8"),
    dict(name="theta_cross_weighted", func="DDtheta", autocorr=0, kind="cap", n1=3000, n2=2500, seed=62,
         bins=("log", 0.05, 8.0, 8), weights=True, avg=True, dtype="f8"),
    # coordinates far from the origin (non-periodic), bins from zero (self pairs), float32 runs
    dict(name="dd_auto_far_offset", func="DD", autocorr=1, kind="offset", n1=4000, L=60.0, seed=15,
         bins=("log", 0.2, 9.0, 10), periodic=False, weights=True, avg=True, dtype="f8"),
    dict(name="dd_auto_rmin0", func="DD", autocorr=1, kind="clustered", n1=3000, L=50.0, seed=16,
         bins=("lin", 0.0, 6.0, 12), periodic=True, weights=True, avg=True, dtype="f8"),
    dict(name="rppi_cross_far_offset", func="DDrppi", autocorr=0, kind="offset", n1=2500, n2=3000, L=50.0,
         seed=23, bins=("log", 0.3, 8.0, 7), pimax=7.0, periodic=False, weights=True, avg=True, dtype="f8"),
    dict(name="smu_auto_float32", func="DDsmu", autocorr=1, kind="clustered", n1=4000, L=100.0, seed=33,
         bins=("log", 0.4, 15.0, 7), mu_max=0.8, nmu=8, periodic=True, weights=True, avg=True, dtype="f4"),
    dict(name="wp_float32_weighted", func="wp", autocorr=1, kind="clustered", n1=4000, L=100.0, seed=42,
         bins=("log", 0.3, 12.0, 8), pimax=15.0, periodic=True, weights=True, avg=True, dtype="f4"),
    dict(name="xi_uniform_rmin0", func="xi", autocorr=1, kind="uniform", n1=4000, L=80.0, seed=52,
         bins=("lin", 0.0, 10.0, 10), periodic=True, weights=True, avg=True, dtype="f8"),
    # weights over a wide range (1 % of the points weigh 100, the rest 0.005-0.015: products span
    # 1e8) and over a moderate one (0.06-1: products span about 300)
    dict(name="dd_auto_wide_weights", func="DD", autocorr=1, kind="uniform", n1=4000, L=80.0, seed=17,
         bins=("log", 0.3, 12.0, 10), periodic=True, weights=True, wkind="wide", avg=True, dtype="f8"),
    dict(name="dd_cross_moderate_weights", func="DD", autocorr=0, kind="clustered", n1=3000, n2=3500, L=120.0,
         seed=18, bins=("log", 0.2, 20.0, 12), periodic=True, weights=True, wkind="moderate", avg=True, dtype="f8"),
    dict(name="rppi_auto_wide_weights", func="DDrppi", autocorr=1, kind="clustered", n1=3000, L=100.0, seed=24,
         bins=("log", 0.2, 12.0, 8), pimax=10.0, periodic=True, weights=True, wkind="wide", avg=True, dtype="f8"),
    dict(name="theta_auto_wide_weights", func="DDtheta", autocorr=1, kind="cap", n1=3000, seed=63,
         bins=("log", 0.02, 8.0, 9), weights=True, wkind="wide", avg=True, dtype="f8"),
]


def case_weights(case, n, seed, dtype):
    """Per-point weights of a case: U[0.5, 1.5] by default; "wide": 1 % of the points weigh 100,
    the others U[0.005, 0.015]; "moderate": U[0.06, 1]."""
    kind = case.get("wkind", "default")
    if kind == "default":
        return cat.weights(n, seed, dtype=dtype)
    rng = np.random.default_rng(seed)
    if kind == "wide":
        w = rng.uniform(0.005, 0.015, n)
        w[rng.random(n) < 0.01] = 100.0
    else:
        w = rng.uniform(0.06, 1.0, n)
    return np.ascontiguousarray(w, dtype=dtype)


def bin_edges(spec):
    kind, lo, hi, n = spec
    if kind == "lin":
        return [float(v) for v in np.linspace(lo, hi, n + 1)]
    return list(cat.log_bins(lo, hi, n))


def make_inputs(case, isa="fallback"):
    """Returns (args, kwargs) for corrfunc_gb300.theory/mocks functions (without the library);
    `isa` selects the reference formula family ("fallback" or "avx512f")."""
    dt = np.float32 if case["dtype"] == "f4" else np.float64
    seed = case["seed"]
    func = case["func"]
    bins = bin_edges(case["bins"])
    auto = case["autocorr"]
    if func == "DDtheta":
        ra1, dec1 = cat.sky_cap(case["n1"], seed, dtype=dt)
        kw = dict(output_thetaavg=case["avg"], isa=isa)
        if case["weights"]:
            kw.update(weights1=case_weights(case, case["n1"], seed + 1000, dt), weight_type="pair_product")
        if not auto:
            ra2, dec2 = cat.sky_cap(case["n2"], seed + 1, dtype=dt)
            kw.update(RA2=ra2, DEC2=dec2)
            if case["weights"]:
                kw.update(weights2=case_weights(case, case["n2"], seed + 1001, dt))
        return [auto, 1, bins, ra1, dec1], kw
    L = case["L"]
    x1, y1, z1 = _box(case["kind"], case["n1"], L, seed, dt)
    kw = {}
    if case["weights"]:
        kw.update(weight_type="pair_product")
    if func in ("wp", "xi"):
        if case["weights"]:
            kw["weights"] = case_weights(case, case["n1"], seed + 1000, dt)
        kw["output_rpavg" if func == "wp" else "output_ravg"] = case["avg"]
        kw["isa"] = isa
        if func == "wp":
            return [L, case["pimax"], 1, bins, x1, y1, z1], kw
        return [L, 1, bins, x1, y1, z1], kw
    if case["weights"]:
        kw["weights1"] = case_weights(case, case["n1"], seed + 1000, dt)
    if not auto:
        x2, y2, z2 = _box(case["kind"], case["n2"], L, seed + 1, dt)
        kw.update(X2=x2, Y2=y2, Z2=z2)
        if case["weights"]:
            kw["weights2"] = case_weights(case, case["n2"], seed + 1001, dt)
    kw["periodic"] = case["periodic"]
    kw["boxsize"] = L if case["periodic"] else None
    kw["isa"] = "fallback"
    avg_key = {"DD": "output_ravg", "DDrppi": "output_rpavg", "DDsmu": "output_savg"}[func]
    kw[avg_key] = case["avg"]
    if func == "DD":
        return [auto, 1, bins, x1, y1, z1], kw
    if func == "DDrppi":
        return [auto, 1, case["pimax"], bins, x1, y1, z1], kw
    return [auto, 1, bins, case["mu_max"], case["nmu"], x1, y1, z1], kw


RUNNERS = {"DD": "run_DD", "DDrppi": "run_DDrppi", "DDsmu": "run_DDsmu", "wp": "run_wp", "xi": "run_xi",
           "DDtheta": "run_DDtheta_mocks"}
REF_MODULE = {"DD": "DD", "DDrppi": "DDrppi", "DDsmu": "DDsmu", "wp": "wp", "xi": "xi", "DDtheta": "DDtheta"}
AVG_FIELD = {"DD": "ravg", "DDrppi": "rpavg", "DDsmu": "savg", "wp": "rpavg", "xi": "ravg", "DDtheta": "thetaavg"}


def runner(func):
    from corrfunc_gb300 import mocks, theory
    mod = mocks if func == "DDtheta" else theory
    return getattr(mod, RUNNERS[func])
