#!/usr/bin/env python3
"""Generates tests/golden/golden.json from the reference's own pair counters.

Run in a container where the reference tree is available and oracle/_ref has been built
(`python oracle/build_ref.py all`):

    python tests/golden/make_golden.py [reference_root]

It records
  * for every seeded case in cases.py, the reference library's output (isa FALLBACK); for
    float32 inputs the reference's double-precision run on the upcast values (its float run,
    which accumulates in float, is stored beside it for information);
  * the same cases run with the reference's AVX512F kernels (fused multiply-add separations,
    theory/DD/countpairs_kernels.c.src:188-190 and siblings), in "avx512f_cases"; this needs an
    x86-64 host with AVX512F;
  * the DD(r) known answer of the reference's Python doctest (Corrfunc/theory/DD.py:166-202):
    its bin edges (theory/tests/bins) and the printed table, plus the reference library's
    full-precision output on the same seeded input.
Inputs themselves are not stored: cases.make_inputs() regenerates them from their seeds.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import cases  # noqa: E402
from corrfunc_gb300 import _capi as C  # noqa: E402
from corrfunc_gb300 import theory  # noqa: E402


def ref_lib(name):
    return C.bind(os.path.join(ROOT, "oracle", "_ref", "libcf_ref_%s.so" % name))


def result_dict(func, res):
    out = {"npairs": [int(v) for v in res["npairs"]], "avg": [float(v) for v in res[cases.AVG_FIELD[func]]]}
    out["weightavg"] = [float(v) for v in res["weightavg"]]
    if func == "wp":
        out["wp"] = [float(v) for v in res["wp"]]
    if func == "xi":
        out["xi"] = [float(v) for v in res["xi"]]
    return out


def doctest_case(refroot):
    src = open(os.path.join(refroot, "Corrfunc", "theory", "DD.py")).read()
    table = []
    for ln in src.splitlines():
        m = re.match(r"^\s+([0-9.]+)\s+([0-9.]+)\s+([0-9.]+)\s+(\d+)\s+([0-9.]+)\s*$", ln)
        if m:
            table.append([float(m.group(1)), float(m.group(2)), float(m.group(3)), int(m.group(4)),
                          float(m.group(5))])
    edges = []
    with open(os.path.join(refroot, "theory", "tests", "bins")) as f:
        rows = [ln.split() for ln in f if ln.strip() and not ln.strip().startswith("#")]
    edges = [float(rows[0][0])] + [float(r[1]) for r in rows]
    np.random.seed(42)
    N, L = 10000, 420.0
    X = np.random.uniform(0, L, N)
    Y = np.random.uniform(0, L, N)
    Z = np.random.uniform(0, L, N)
    w = np.ones_like(X)
    res = theory.run_DD(ref_lib("DD"), 1, 4, edges, X, Y, Z, weights1=w, weight_type="pair_product",
                        output_ravg=True, boxsize=L, periodic=True, isa="fallback")
    return {"N": N, "boxsize": L, "seed": 42, "edges": edges, "doctest_table": table,
            "reference": result_dict("DD", res)}


def run_case(case, isa):
    args, kw = cases.make_inputs(case, isa=isa)
    run = cases.runner(case["func"])
    lib = ref_lib(cases.REF_MODULE[case["func"]])
    res_f = None
    if case["dtype"] == "f4":
        # float inputs are pinned to the reference's double-precision run on the same values
        # upcast to double; the reference's own float run (float accumulators) is kept for
        # information only
        res_f = run(lib, *args, **kw)
        up = lambda a: a.astype(np.float64) if isinstance(a, np.ndarray) and a.dtype == np.float32 else a
        args = [up(a) for a in args]
        kw = {k: up(v) for k, v in kw.items()}
    out = result_dict(case["func"], run(lib, *args, **kw))
    if res_f is not None:
        out["reference_float_run_npairs"] = [int(v) for v in res_f["npairs"]]
    return out


def main():
    refroot = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = {"generator": "tests/golden/make_golden.py", "isa": "FALLBACK", "cases": {}, "avx512f_cases": {}}
    for case in cases.CASES:
        out["cases"][case["name"]] = run_case(case, "fallback")
        out["avx512f_cases"][case["name"]] = run_case(case, "avx512f")
        print("%-34s %12d pairs (fallback) %12d (avx512f)" % (case["name"], sum(out["cases"][case["name"]]["npairs"]),
                                                             sum(out["avx512f_cases"][case["name"]]["npairs"])))
    out["dd_doctest"] = doctest_case(refroot)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
