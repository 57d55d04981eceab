"""Python front ends for the survey-catalogue pair counters, mirroring Corrfunc.mocks:
DDtheta_mocks (Corrfunc/mocks/DDtheta_mocks.py:19-357), DDrppi_mocks
(Corrfunc/mocks/DDrppi_mocks.py:17-402), DDsmu_mocks (Corrfunc/mocks/DDsmu_mocks.py:17-352) and
vpf_mocks (Corrfunc/mocks/vpf_mocks.py:17-285)."""
import ctypes

import numpy as np

from . import _capi as C

DDTHETA_DTYPE = np.dtype([("thetamin", np.float64), ("thetamax", np.float64), ("thetaavg", np.float64),
                          ("npairs", np.uint64), ("weightavg", np.float64)])
DDRPPI_MOCKS_DTYPE = np.dtype([("rmin", np.float64), ("rmax", np.float64), ("rpavg", np.float64),
                               ("pimax", np.float64), ("npairs", np.uint64), ("weightavg", np.float64)])
DDSMU_MOCKS_DTYPE = np.dtype([("smin", np.float64), ("smax", np.float64), ("savg", np.float64),
                              ("mumax", np.float64), ("npairs", np.uint64), ("weightavg", np.float64)])


def _fix_ra_dec(ra, dec):
    """In-place wrap as Corrfunc/utils.py:421-461 does: RA += 180 when any RA < 0, DEC -= 90 when
    any DEC > 90 (the caller's arrays are modified, as with the reference)."""
    if not hasattr(ra, "dtype") or not hasattr(dec, "dtype"):
        raise TypeError("Input RA array must be a numpy array")
    if np.min(ra) < 0.0:  # numpy reductions: the builtins iterate element by element in Python
        print("Warning: found negative RA values, wrapping into [0.0, 360.0]  range")
        ra += 180.0
    if np.max(dec) > 90.0:
        print("Warning: found DEC values more than 90.0; wrapping into [-90.0, 90.0] range")
        dec -= 90.0
    return ra, dec


def run_DDtheta_mocks(lib, autocorr, nthreads, binfile, RA1, DEC1, weights1=None, RA2=None, DEC2=None,
                      weights2=None, link_in_dec=True, link_in_ra=True, verbose=False, output_thetaavg=False,
                      fast_acos=False, ra_refine_factor=2, dec_refine_factor=2, max_cells_per_dim=100,
                      copy_particles=True, enable_min_sep_opt=True, c_api_timer=False, isa="fastest",
                      weight_type=None):
    if not autocorr and (RA2 is None or DEC2 is None):
        raise ValueError("Must pass valid arrays for RA2/DEC2 for computing cross-correlation")
    RA1, DEC1 = _fix_ra_dec(RA1, DEC1)
    RA1 = C.as_positions(RA1)
    dt = RA1.dtype
    DEC1 = C.as_positions(DEC1, dt)
    if not autocorr:
        RA2, DEC2 = _fix_ra_dec(RA2, DEC2)
        RA2 = C.as_positions(RA2, dt)
        DEC2 = C.as_positions(DEC2, dt)
    else:
        RA2 = DEC2 = None
    w1, w2 = C.process_weights(weights1, weights2, RA1, RA2, weight_type, autocorr)
    if link_in_ra:
        link_in_dec = True
    o = C.get_config_options()
    o.verbose = 1 if verbose else 0
    o.instruction_set = C.translate_isa(isa) if isinstance(isa, str) else int(isa)
    o.link_in_dec = 1 if link_in_dec else 0
    o.link_in_ra = 1 if link_in_ra else 0
    o.need_avg_sep = 1 if output_thetaavg else 0
    o.fast_acos = 1 if fast_acos else 0
    o.max_cells_per_dim = int(max_cells_per_dim)
    o.copy_particles = 1 if copy_particles else 0
    o.enable_min_sep_opt = 1 if enable_min_sep_opt else 0
    o.c_api_timer = 1 if c_api_timer else 0
    o.autocorr = 1 if autocorr else 0
    o.periodic = 0
    o.float_type = dt.itemsize
    C.set_refine(o, (ra_refine_factor, dec_refine_factor, o.bin_refine_factors[2]))
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, w2, keep)
    res = C.ResultsTheta()
    if autocorr:
        # the CPython binding hands the first set over twice (mocks/python_bindings/_countpairs_mocks.c:1885)
        RA2p, DEC2p, n2 = RA1, DEC1, len(RA1)
    else:
        RA2p, DEC2p, n2 = RA2, DEC2, len(RA2)
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs_theta_mocks(len(RA1), C.ptr(RA1), C.ptr(DEC1), n2, C.ptr(RA2p), C.ptr(DEC2p),
                                        int(nthreads), int(autocorr), bf.encode(), ctypes.byref(res),
                                        ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    nb = res.nbin if bool(res.npairs) else 0
    npairs = C.carray(res.npairs, nb, np.uint64)
    tupp = C.carray(res.theta_upp, nb, np.float64)
    tavg = C.carray(res.theta_avg, nb, np.float64)
    wavg = C.carray(res.weightavg, nb, np.float64)
    lib.free_results_countpairs_theta(ctypes.byref(res))
    out = np.zeros(max(nb - 1, 0), dtype=DDTHETA_DTYPE)
    out["thetamin"] = tupp[:-1]
    out["thetamax"] = tupp[1:]
    out["thetaavg"] = tavg[1:]
    out["npairs"] = npairs[1:]
    out["weightavg"] = wavg[1:]
    return (out, o.c_api_time) if c_api_timer else out


def DDtheta_mocks(*args, **kwargs):
    """Angular pair counts DD(theta); see Corrfunc.mocks.DDtheta_mocks."""
    return run_DDtheta_mocks(C.library(), *args, **kwargs)


def _mock_inputs(autocorr, RA1, DEC1, CZ1, weights1, RA2, DEC2, CZ2, weights2, weight_type):
    if not autocorr and (RA2 is None or DEC2 is None or CZ2 is None):
        raise ValueError("Must pass valid arrays for RA2/DEC2/CZ2 for computing cross-correlation")
    RA1, DEC1 = _fix_ra_dec(RA1, DEC1)
    RA1 = C.as_positions(RA1)
    dt = RA1.dtype
    DEC1 = C.as_positions(DEC1, dt)
    CZ1 = C.as_positions(CZ1, dt)
    if not autocorr:
        RA2, DEC2 = _fix_ra_dec(RA2, DEC2)
        RA2, DEC2, CZ2 = (C.as_positions(a, dt) for a in (RA2, DEC2, CZ2))
    else:
        RA2 = DEC2 = CZ2 = None
    w1, w2 = C.process_weights(weights1, weights2, RA1, RA2, weight_type, autocorr)
    return RA1, DEC1, CZ1, RA2, DEC2, CZ2, w1, w2, dt


def _mock_options(dt, autocorr, is_comoving_dist, verbose, need_avg, fast_divide_and_NR_steps, refine,
                  max_cells_per_dim, copy_particles, enable_min_sep_opt, c_api_timer, isa):
    o = C.get_config_options()
    o.verbose = 1 if verbose else 0
    o.instruction_set = C.translate_isa(isa) if isinstance(isa, str) else int(isa)
    o.is_comoving_dist = 1 if is_comoving_dist else 0
    o.need_avg_sep = 1 if need_avg else 0
    o.fast_divide_and_NR_steps = int(fast_divide_and_NR_steps)
    o.max_cells_per_dim = int(max_cells_per_dim)
    o.copy_particles = 1 if copy_particles else 0
    o.enable_min_sep_opt = 1 if enable_min_sep_opt else 0
    o.c_api_timer = 1 if c_api_timer else 0
    o.autocorr = 1 if autocorr else 0
    o.periodic = 0
    o.float_type = dt.itemsize
    C.set_refine(o, refine)
    return o


def run_DDrppi_mocks(lib, autocorr, cosmology, nthreads, pimax, binfile, RA1, DEC1, CZ1, weights1=None, RA2=None,
                     DEC2=None, CZ2=None, weights2=None, is_comoving_dist=False, verbose=False, output_rpavg=False,
                     fast_divide_and_NR_steps=0, xbin_refine_factor=2, ybin_refine_factor=2, zbin_refine_factor=1,
                     max_cells_per_dim=100, copy_particles=True, enable_min_sep_opt=True, c_api_timer=False,
                     isa="fastest", weight_type=None):
    RA1, DEC1, CZ1, RA2, DEC2, CZ2, w1, w2, dt = _mock_inputs(autocorr, RA1, DEC1, CZ1, weights1, RA2, DEC2, CZ2,
                                                              weights2, weight_type)
    o = _mock_options(dt, autocorr, is_comoving_dist, verbose, output_rpavg, fast_divide_and_NR_steps,
                      (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                      copy_particles, enable_min_sep_opt, c_api_timer, isa)
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, w2, keep)
    res = C.ResultsRpPi()
    n2 = len(RA1) if autocorr else len(RA2)
    p2 = (RA1, DEC1, CZ1) if autocorr else (RA2, DEC2, CZ2)
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs_mocks(len(RA1), C.ptr(RA1), C.ptr(DEC1), C.ptr(CZ1), n2, C.ptr(p2[0]), C.ptr(p2[1]),
                                  C.ptr(p2[2]), int(nthreads), int(autocorr), bf.encode(), float(pimax),
                                  int(cosmology), ctypes.byref(res), ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    out = _rows_2d(lib.free_results_mocks, res, res.nbin, res.npibin, "rupp", "rpavg", float(pimax) / max(res.npibin, 1),
                   DDRPPI_MOCKS_DTYPE, ("rmin", "rmax", "rpavg", "pimax"))
    return (out, o.c_api_time) if c_api_timer else out


def run_DDsmu_mocks(lib, autocorr, cosmology, nthreads, mu_max, nmu_bins, binfile, RA1, DEC1, CZ1, weights1=None,
                    RA2=None, DEC2=None, CZ2=None, weights2=None, is_comoving_dist=False, verbose=False,
                    output_savg=False, fast_divide_and_NR_steps=0, xbin_refine_factor=2, ybin_refine_factor=2,
                    zbin_refine_factor=1, max_cells_per_dim=100, copy_particles=True, enable_min_sep_opt=True,
                    c_api_timer=False, isa="fastest", weight_type=None):
    if not np.isscalar(mu_max):
        raise TypeError("The parameter `mu_max` = {0}, has size = {1}. The code is expecting a scalar quantity"
                        .format(mu_max, np.size(mu_max)))
    if mu_max <= 0.0 or mu_max > 1.0:
        raise ValueError("The parameter `mu_max` = {0}, is the max. of cosine of an angle and should be within "
                         "(0.0, 1.0]".format(mu_max))
    RA1, DEC1, CZ1, RA2, DEC2, CZ2, w1, w2, dt = _mock_inputs(autocorr, RA1, DEC1, CZ1, weights1, RA2, DEC2, CZ2,
                                                              weights2, weight_type)
    o = _mock_options(dt, autocorr, is_comoving_dist, verbose, output_savg, fast_divide_and_NR_steps,
                      (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                      copy_particles, enable_min_sep_opt, c_api_timer, isa)
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, w2, keep)
    res = C.ResultsSMu()
    n2 = len(RA1) if autocorr else len(RA2)
    p2 = (RA1, DEC1, CZ1) if autocorr else (RA2, DEC2, CZ2)
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs_mocks_s_mu(len(RA1), C.ptr(RA1), C.ptr(DEC1), C.ptr(CZ1), n2, C.ptr(p2[0]),
                                       C.ptr(p2[1]), C.ptr(p2[2]), int(nthreads), int(autocorr), bf.encode(),
                                       float(mu_max), int(nmu_bins), int(cosmology), ctypes.byref(res),
                                       ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    out = _rows_2d(lib.free_results_mocks_s_mu, res, res.nsbin, res.nmu_bins, "supp", "savg",
                   float(mu_max) / max(res.nmu_bins, 1), DDSMU_MOCKS_DTYPE, ("smin", "smax", "savg", "mumax"))
    return (out, o.c_api_time) if c_api_timer else out


def _rows_2d(free, res, nbin, ninner, upp_name, avg_name, width, dtype, names):
    """Rows (low edge, high edge, avg, (j + 1) * width, npairs, weightavg) for bins 1..nbin-1 and inner
    bins 0..ninner-1, as the reference's bindings build them (mocks/python_bindings/_countpairs_mocks.c:1411-1425)."""
    if not bool(res.npairs):
        return np.zeros(0, dtype=dtype)
    tot = (nbin + 1) * (ninner + 1)
    npairs = C.carray(res.npairs, tot, np.uint64)
    upp = C.carray(getattr(res, upp_name), nbin, np.float64)
    avg = C.carray(getattr(res, avg_name), tot, np.float64)
    wavg = C.carray(res.weightavg, tot, np.float64)
    free(ctypes.byref(res))
    out = np.zeros((nbin - 1) * ninner, dtype=dtype)
    k = 0
    for i in range(1, nbin):
        for j in range(ninner):
            b = i * (ninner + 1) + j
            out[k] = (upp[i - 1], upp[i], avg[b], (j + 1) * width, npairs[b], wavg[b])
            k += 1
    return out


def DDrppi_mocks(*args, **kwargs):
    """DD(rp, pi) of survey catalogues; see Corrfunc.mocks.DDrppi_mocks."""
    return run_DDrppi_mocks(C.library(), *args, **kwargs)


def DDsmu_mocks(*args, **kwargs):
    """DD(s, mu) of survey catalogues; see Corrfunc.mocks.DDsmu_mocks."""
    return run_DDsmu_mocks(C.library(), *args, **kwargs)


def run_vpf_mocks(lib, rmax, nbins, nspheres, numpN, threshold_ngb, centers_file, cosmology, RA, DEC, CZ, RAND_RA,
                  RAND_DEC, RAND_CZ, verbose=False, is_comoving_dist=False, xbin_refine_factor=1, ybin_refine_factor=1,
                  zbin_refine_factor=1, max_cells_per_dim=100, copy_particles=True, c_api_timer=False, isa="fastest"):
    RA, DEC = _fix_ra_dec(RA, DEC)
    RAND_RA, RAND_DEC = _fix_ra_dec(RAND_RA, RAND_DEC)
    RA = C.as_positions(RA)
    dt = RA.dtype
    DEC, CZ, RAND_RA, RAND_DEC, RAND_CZ = (C.as_positions(a, dt) for a in (DEC, CZ, RAND_RA, RAND_DEC, RAND_CZ))
    o = _mock_options(dt, 1, is_comoving_dist, verbose, False, 0,
                      (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                      copy_particles, True, c_api_timer, isa)
    extra = C.get_extra_options()
    res = C.ResultsVpf()
    rc = lib.countspheres_mocks(len(RA), C.ptr(RA), C.ptr(DEC), C.ptr(CZ), len(RAND_RA), C.ptr(RAND_RA),
                                C.ptr(RAND_DEC), C.ptr(RAND_CZ), int(threshold_ngb), float(rmax), int(nbins),
                                int(nspheres), int(numpN), str(centers_file).encode(), int(cosmology),
                                ctypes.byref(res), ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    out = C.vpf_rows(res, int(numpN))
    lib.free_results_countspheres_mocks(ctypes.byref(res))
    return (out, o.c_api_time) if c_api_timer else out


def vpf_mocks(*args, **kwargs):
    """Counts in spheres of a survey catalogue; see Corrfunc.mocks.vpf_mocks."""
    return run_vpf_mocks(C.library(), *args, **kwargs)
