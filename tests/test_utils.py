"""Count -> correlation converters against the reference's Corrfunc/utils.py outputs
(tests/golden/converters.json, made by tests/golden/make_converters.py)."""
import json
import os

import numpy as np
import pytest

from corrfunc_gb300 import utils
from corrfunc_gb300.theory import DD_DTYPE

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "converters.json")))


@pytest.mark.parametrize("case", GOLD["cases"], ids=lambda c: c["name"])
def test_converters_match_reference(case):
    args = [case["ND1"], case["ND2"], case["NR1"], case["NR2"]] + [np.array(case[k])
                                                                 for k in ("D1D2", "D1R2", "D2R1", "R1R2")]
    if case["name"].startswith("wp"):
        got = utils.convert_rp_pi_counts_to_wp(*args, case["nrpbins"], case["pimax"], dpi=case["dpi"])
    else:
        got = utils.convert_3d_counts_to_cf(*args)
    want = np.array([np.nan if v is None else v for v in case["result"]])
    np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
    np.testing.assert_allclose(got[~np.isnan(got)], want[~np.isnan(want)], rtol=1e-14, atol=0)


def test_record_arrays_and_errors():
    rec = np.zeros(3, dtype=DD_DTYPE)
    rec["npairs"] = [10, 20, 30]
    cf = utils.convert_3d_counts_to_cf(10, 10, 20, 20, rec, rec, rec, rec)
    assert np.allclose(cf, (4 * np.array([10, 20, 30]) - 2 * 2 * np.array([10, 20, 30]) + [10, 20, 30]) / [10, 20, 30])
    with pytest.raises(ValueError):
        utils.convert_3d_counts_to_cf(1, 1, 1, 1, [1, 2], [1], [1, 2], [1, 2])
    with pytest.raises(ValueError):
        utils.convert_3d_counts_to_cf(1, 1, 1, 1, [1], [1], [1], [1], estimator="DP")
    with pytest.raises(ValueError):
        utils.convert_rp_pi_counts_to_wp(1, 1, 1, 1, [1] * 6, [1] * 6, [1] * 6, [1] * 6, 2, 3.0, dpi=0.0)
    with pytest.raises(ValueError):
        utils.convert_rp_pi_counts_to_wp(1, 1, 1, 1, [1] * 6, [1] * 6, [1] * 6, [1] * 6, 2, 4.0, dpi=1.0)


def test_ra_dec_fixups_follow_the_reference(capsys):
    """The survey front ends wrap RA by +180 when any RA < 0 and DEC by -90 when any DEC > 90,
    in place on the caller's arrays (Corrfunc/utils.py:421-461); other arrays are untouched."""
    from corrfunc_gb300 import mocks
    ra = np.array([-10.0, 20.0, 30.0])
    dec = np.array([10.0, 95.0, -5.0])
    r, d = mocks._fix_ra_dec(ra, dec)
    assert r is ra and d is dec
    assert list(ra) == [170.0, 200.0, 210.0]
    assert list(dec) == [-80.0, 5.0, -95.0]
    out = capsys.readouterr().out
    assert "negative RA" in out and "DEC values more than 90.0" in out
    ra2, dec2 = np.array([0.0, 359.0]), np.array([-90.0, 90.0])
    mocks._fix_ra_dec(ra2, dec2)
    assert list(ra2) == [0.0, 359.0] and list(dec2) == [-90.0, 90.0]
    with pytest.raises(TypeError):
        mocks._fix_ra_dec([1.0], np.array([1.0]))
