#!/usr/bin/env python3
"""Generates tests/golden/converters.json from the reference's Corrfunc/utils.py converters
(convert_3d_counts_to_cf, convert_rp_pi_counts_to_wp) on seeded synthetic pair counts.

    python tests/golden/make_converters.py [reference_root]

The reference module imports wurlitzer (not needed by the converters); a stand-in module is
registered so that the file imports without it."""
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference_utils(root):
    sys.modules.setdefault("wurlitzer", types.ModuleType("wurlitzer"))
    spec = importlib.util.spec_from_file_location("ref_corrfunc_utils", os.path.join(root, "Corrfunc", "utils.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def cases():
    rng = np.random.default_rng(2024)
    out = []
    for k, (nb, zero_rr) in enumerate([(10, False), (25, True), (1, False)]):
        rr = rng.integers(1000, 10 ** 7, nb)
        if zero_rr:
            rr[[0, 3]] = 0
        out.append(dict(name="cf_%d" % k, ND1=int(rng.integers(10 ** 3, 10 ** 6)), ND2=int(rng.integers(10 ** 3, 10 ** 6)),
                        NR1=int(rng.integers(10 ** 5, 10 ** 7)), NR2=int(rng.integers(10 ** 5, 10 ** 7)),
                        D1D2=rng.integers(0, 10 ** 6, nb).tolist(), D1R2=rng.integers(0, 10 ** 7, nb).tolist(),
                        D2R1=rng.integers(0, 10 ** 7, nb).tolist(), R1R2=rr.tolist()))
    nrp, npi = 7, 40
    n = nrp * npi
    out.append(dict(name="wp_0", ND1=200000, ND2=200000, NR1=600000, NR2=600000,
                    D1D2=rng.integers(10, 10 ** 5, n).tolist(), D1R2=rng.integers(10, 10 ** 6, n).tolist(),
                    D2R1=rng.integers(10, 10 ** 6, n).tolist(), R1R2=rng.integers(10 ** 3, 10 ** 7, n).tolist(),
                    nrpbins=nrp, pimax=40.0, dpi=1.0))
    return out


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    ref = load_reference_utils(root)
    res = []
    for c in cases():
        args = [c["ND1"], c["ND2"], c["NR1"], c["NR2"]] + [np.array(c[k]) for k in ("D1D2", "D1R2", "D2R1", "R1R2")]
        if c["name"].startswith("wp"):
            val = ref.convert_rp_pi_counts_to_wp(*args, c["nrpbins"], c["pimax"], dpi=c["dpi"])
        else:
            val = ref.convert_3d_counts_to_cf(*args)
        c = dict(c)
        c["result"] = [None if np.isnan(v) else float(v) for v in val]
        res.append(c)
    with open(os.path.join(HERE, "converters.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_converters.py", "cases": res}, f, indent=1)
    print("wrote", len(res), "cases")


if __name__ == "__main__":
    main()
