"""Pair counts -> correlation functions, with the arguments of Corrfunc.utils (Corrfunc/utils.py:27
convert_3d_counts_to_cf, :167 convert_rp_pi_counts_to_wp).  Host-side numpy, downstream of the
GPU pair counters: the Landy-Szalay estimator and its projection along the line of sight."""
import numpy as np

__all__ = ["convert_3d_counts_to_cf", "convert_rp_pi_counts_to_wp"]


def _counts(a):
    """npairs of a result record array, or the array itself."""
    try:
        return np.asarray(a["npairs"])
    except (IndexError, KeyError, ValueError, TypeError):
        return np.asarray(a)


def convert_3d_counts_to_cf(ND1, ND2, NR1, NR2, D1D2, D1R2, D2R1, R1R2, estimator="LS"):
    """Landy-Szalay correlation function from the four pair counts of two data sets (sizes ND1,
    ND2) and their randoms (NR1, NR2):

        xi = (f1 f2 D1D2 - f1 D1R2 - f2 D2R1 + R1R2) / R1R2,  f1 = NR1 / ND1,  f2 = NR2 / ND2,

    NaN where R1R2 is 0.  Counts are arrays or the record arrays the pair counters return."""
    dd, dr, rd, rr = (_counts(a) for a in (D1D2, D1R2, D2R1, R1R2))
    n = len(dd)
    if not (len(dr) == n and len(rd) == n and len(rr) == n):
        raise ValueError("Pair counts must have the same number of elements (same bins)")
    if not ("LS" in estimator or "Landy" in estimator):
        raise ValueError("Only the Landy-Szalay estimator is supported. Pass estimator='LS'. "
                         "(Got estimator = {0})".format(estimator))
    f1 = np.float64(NR1) / np.float64(ND1)
    f2 = np.float64(NR2) / np.float64(ND2)
    cf = np.full(n, np.nan)
    ok = rr > 0
    cf[ok] = (f1 * f2 * dd[ok] - f1 * dr[ok] - f2 * rd[ok] + rr[ok]) / rr[ok]
    return cf


def convert_rp_pi_counts_to_wp(ND1, ND2, NR1, NR2, D1D2, D1R2, D2R1, R1R2, nrpbins, pimax, dpi=1.0,
                               estimator="LS"):
    """Projected correlation function wp(rp) = 2 dpi sum over pi bins of xi(rp, pi), from DDrppi-
    style counts with nrpbins rp bins and pimax / dpi pi bins per rp bin (rp-major order)."""
    if dpi <= 0.0:
        raise ValueError("Binsize along the line of sight (dpi) = {0} must be positive".format(dpi))
    xi = convert_3d_counts_to_cf(ND1, ND2, NR1, NR2, D1D2, D1R2, D2R1, R1R2, estimator=estimator)
    npibins = len(xi) // nrpbins
    if npibins * nrpbins != len(xi):
        raise ValueError("Number of pi bins could not be calculated correctly: {0} bins is not a multiple of "
                         "{1} rp bins".format(len(xi), nrpbins))
    if dpi * npibins != pimax:
        raise ValueError("Pimax = {0} should be equal to the product of npibins = {1} and dpi = {2}. Check your "
                         "binning scheme.".format(pimax, npibins, dpi))
    wp = np.empty(nrpbins)
    for i in range(nrpbins):
        wp[i] = 2.0 * dpi * np.sum(xi[i * npibins:(i + 1) * npibins])
    return wp
