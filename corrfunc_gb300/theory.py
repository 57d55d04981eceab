"""Python front end for the theory pair counters, mirroring Corrfunc.theory.

``DD``, ``DDrppi``, ``DDsmu``, ``wp`` and ``xi`` take the same arguments and return the same
numpy structured arrays as Corrfunc 2.5.3 (Corrfunc/theory/DD.py:16-284 and siblings).  They
call the C ABI of libcorrfunc_gb300.so, whose counting runs on the GPU.  The ``run_*``
functions take the library handle explicitly; any library exporting the reference's C API
(theory/DD/countpairs.h and siblings) can be driven by them.
"""
import ctypes

import numpy as np

from . import _capi as C

DD_DTYPE = np.dtype([("rmin", np.float64), ("rmax", np.float64), ("ravg", np.float64),
                     ("npairs", np.uint64), ("weightavg", np.float64)])
DDRPPI_DTYPE = np.dtype([("rmin", np.float64), ("rmax", np.float64), ("rpavg", np.float64),
                         ("pimax", np.float64), ("npairs", np.uint64), ("weightavg", np.float64)])
DDSMU_DTYPE = np.dtype([("smin", np.float64), ("smax", np.float64), ("savg", np.float64),
                        ("mu_max", np.float64), ("npairs", np.uint64), ("weightavg", np.float64)])
WP_DTYPE = np.dtype([("rmin", np.float64), ("rmax", np.float64), ("rpavg", np.float64),
                     ("wp", np.float64), ("npairs", np.uint64), ("weightavg", np.float64)])
XI_DTYPE = np.dtype([("rmin", np.float64), ("rmax", np.float64), ("ravg", np.float64),
                     ("xi", np.float64), ("npairs", np.uint64), ("weightavg", np.float64)])


def _boxsize3(boxsize):
    b = np.atleast_1d(boxsize)
    if len(b) == 1:
        return (float(b[0]),) * 3
    return tuple(float(v) for v in b)


def _common_options(nthreads, periodic, boxsize, verbose, need_avg, refine, max_cells, copy_particles,
                    enable_min_sep_opt, c_api_timer, isa, dtype):
    o = C.get_config_options()
    o.verbose = 1 if verbose else 0
    o.periodic = 1 if periodic else 0
    o.need_avg_sep = 1 if need_avg else 0
    o.c_api_timer = 1 if c_api_timer else 0
    o.copy_particles = 1 if copy_particles else 0
    o.enable_min_sep_opt = 1 if enable_min_sep_opt else 0
    o.max_cells_per_dim = int(max_cells)
    o.instruction_set = C.translate_isa(isa) if isinstance(isa, str) else int(isa)
    o.float_type = np.dtype(dtype).itemsize
    if boxsize is not None:
        bx, by, bz = _boxsize3(boxsize)
        o.boxsize_x, o.boxsize_y, o.boxsize_z = bx, by, bz
    C.set_refine(o, refine)
    return o


def _pair_inputs(autocorr, X1, Y1, Z1, X2, Y2, Z2, weights1, weights2, weight_type):
    if not autocorr and (X2 is None or Y2 is None or Z2 is None):
        raise ValueError("Must pass valid arrays for X2/Y2/Z2 for computing cross-correlation")
    X1 = C.as_positions(X1)
    dt = X1.dtype
    Y1 = C.as_positions(Y1, dt)
    Z1 = C.as_positions(Z1, dt)
    if not autocorr:
        X2, Y2, Z2 = (C.as_positions(a, dt) for a in (X2, Y2, Z2))
    else:
        X2 = Y2 = Z2 = None
    w1, w2 = C.process_weights(weights1, weights2, X1, X2, weight_type, autocorr)
    return X1, Y1, Z1, X2, Y2, Z2, w1, w2


def run_DD(lib, autocorr, nthreads, binfile, X1, Y1, Z1, weights1=None, periodic=True, boxsize=None, X2=None,
           Y2=None, Z2=None, weights2=None, verbose=False, output_ravg=False, xbin_refine_factor=2,
           ybin_refine_factor=2, zbin_refine_factor=1, max_cells_per_dim=100, copy_particles=True,
           enable_min_sep_opt=True, c_api_timer=False, isa="fastest", weight_type=None):
    if periodic and boxsize is None:
        raise ValueError("Must specify a boxsize if periodic=True")
    X1, Y1, Z1, X2, Y2, Z2, w1, w2 = _pair_inputs(autocorr, X1, Y1, Z1, X2, Y2, Z2, weights1, weights2, weight_type)
    o = _common_options(nthreads, periodic, boxsize, verbose, output_ravg,
                        (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                        copy_particles, enable_min_sep_opt, c_api_timer, isa, X1.dtype)
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, w2, keep)
    res = C.ResultsDD()
    n2 = 0 if autocorr else len(X2)
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs(len(X1), C.ptr(X1), C.ptr(Y1), C.ptr(Z1), n2, C.ptr(X2), C.ptr(Y2), C.ptr(Z2),
                            int(nthreads), int(autocorr), bf.encode(), ctypes.byref(res), ctypes.byref(o),
                            ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    nb = res.nbin
    npairs = C.carray(res.npairs, nb, np.uint64)
    rupp = C.carray(res.rupp, nb, np.float64)
    ravg = C.carray(res.rpavg, nb, np.float64)
    wavg = C.carray(res.weightavg, nb, np.float64)
    lib.free_results(ctypes.byref(res))
    out = np.zeros(max(nb - 1, 0), dtype=DD_DTYPE)
    out["rmin"] = rupp[:-1]
    out["rmax"] = rupp[1:]
    out["ravg"] = ravg[1:]
    out["npairs"] = npairs[1:]
    out["weightavg"] = wavg[1:]
    return (out, o.c_api_time) if c_api_timer else out


def run_DDrppi(lib, autocorr, nthreads, pimax, binfile, X1, Y1, Z1, weights1=None, periodic=True, boxsize=None,
               X2=None, Y2=None, Z2=None, weights2=None, verbose=False, output_rpavg=False, xbin_refine_factor=2,
               ybin_refine_factor=2, zbin_refine_factor=1, max_cells_per_dim=100, copy_particles=True,
               enable_min_sep_opt=True, c_api_timer=False, isa="fastest", weight_type=None):
    if periodic and boxsize is None:
        raise ValueError("Must specify a boxsize if periodic=True")
    X1, Y1, Z1, X2, Y2, Z2, w1, w2 = _pair_inputs(autocorr, X1, Y1, Z1, X2, Y2, Z2, weights1, weights2, weight_type)
    o = _common_options(nthreads, periodic, boxsize, verbose, output_rpavg,
                        (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                        copy_particles, enable_min_sep_opt, c_api_timer, isa, X1.dtype)
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, w2, keep)
    res = C.ResultsRpPi()
    n2 = 0 if autocorr else len(X2)
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs_rp_pi(len(X1), C.ptr(X1), C.ptr(Y1), C.ptr(Z1), n2, C.ptr(X2), C.ptr(Y2), C.ptr(Z2),
                                  int(nthreads), int(autocorr), bf.encode(), float(pimax), ctypes.byref(res),
                                  ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    nb, npi = res.nbin, res.npibin
    tot = (nb + 1) * (npi + 1)
    npairs = C.carray(res.npairs, tot, np.uint64)
    rupp = C.carray(res.rupp, nb, np.float64)
    rpavg = C.carray(res.rpavg, tot, np.float64)
    wavg = C.carray(res.weightavg, tot, np.float64)
    lib.free_results_rp_pi(ctypes.byref(res))
    dpi = float(pimax) / npi
    rows = []
    for i in range(1, nb):
        for j in range(npi):
            idx = i * (npi + 1) + j
            rows.append((rupp[i - 1], rupp[i], rpavg[idx], (j + 1) * dpi, npairs[idx], wavg[idx]))
    out = np.array(rows, dtype=DDRPPI_DTYPE)
    return (out, o.c_api_time) if c_api_timer else out


def run_DDsmu(lib, autocorr, nthreads, binfile, mu_max, nmu_bins, X1, Y1, Z1, weights1=None, periodic=True,
              boxsize=None, X2=None, Y2=None, Z2=None, weights2=None, verbose=False, output_savg=False,
              fast_divide_and_NR_steps=0, xbin_refine_factor=2, ybin_refine_factor=2, zbin_refine_factor=1,
              max_cells_per_dim=100, copy_particles=True, enable_min_sep_opt=True, c_api_timer=False,
              isa="fastest", weight_type=None):
    if periodic and boxsize is None:
        raise ValueError("Must specify a boxsize if periodic=True")
    X1, Y1, Z1, X2, Y2, Z2, w1, w2 = _pair_inputs(autocorr, X1, Y1, Z1, X2, Y2, Z2, weights1, weights2, weight_type)
    o = _common_options(nthreads, periodic, boxsize, verbose, output_savg,
                        (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                        copy_particles, enable_min_sep_opt, c_api_timer, isa, X1.dtype)
    o.fast_divide_and_NR_steps = int(fast_divide_and_NR_steps)
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, w2, keep)
    res = C.ResultsSMu()
    n2 = 0 if autocorr else len(X2)
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs_s_mu(len(X1), C.ptr(X1), C.ptr(Y1), C.ptr(Z1), n2, C.ptr(X2), C.ptr(Y2), C.ptr(Z2),
                                 int(nthreads), int(autocorr), bf.encode(), float(mu_max), int(nmu_bins),
                                 ctypes.byref(res), ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    nb, nmu = res.nsbin, res.nmu_bins
    tot = (nb + 1) * (nmu + 1)
    npairs = C.carray(res.npairs, tot, np.uint64)
    supp = C.carray(res.supp, nb, np.float64)
    savg = C.carray(res.savg, tot, np.float64)
    wavg = C.carray(res.weightavg, tot, np.float64)
    lib.free_results_s_mu(ctypes.byref(res))
    dmu = float(mu_max) / nmu
    rows = []
    for i in range(1, nb):
        for j in range(nmu):
            idx = i * (nmu + 1) + j
            rows.append((supp[i - 1], supp[i], savg[idx], (j + 1) * dmu, npairs[idx], wavg[idx]))
    out = np.array(rows, dtype=DDSMU_DTYPE)
    return (out, o.c_api_time) if c_api_timer else out


def run_wp(lib, boxsize, pimax, nthreads, binfile, X, Y, Z, weights=None, weight_type=None, verbose=False,
           output_rpavg=False, xbin_refine_factor=2, ybin_refine_factor=2, zbin_refine_factor=1,
           max_cells_per_dim=100, copy_particles=True, enable_min_sep_opt=True, c_api_timer=False,
           c_cell_timer=False, isa="fastest"):
    X = C.as_positions(X)
    Y = C.as_positions(Y, X.dtype)
    Z = C.as_positions(Z, X.dtype)
    w1, _ = C.process_weights(weights, None, X, None, weight_type, True)
    o = _common_options(nthreads, True, boxsize, verbose, output_rpavg,
                        (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                        copy_particles, enable_min_sep_opt, c_api_timer, isa, X.dtype)
    o.c_cell_timer = 1 if c_cell_timer else 0
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, None, keep)
    res = C.ResultsWp()
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs_wp(len(X), C.ptr(X), C.ptr(Y), C.ptr(Z), float(_boxsize3(boxsize)[0]), int(nthreads),
                               bf.encode(), float(pimax), ctypes.byref(res), ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    nb = res.nbin
    npairs = C.carray(res.npairs, nb, np.uint64)
    rupp = C.carray(res.rupp, nb, np.float64)
    rpavg = C.carray(res.rpavg, nb, np.float64)
    wp_ = C.carray(res.wp, nb, np.float64)
    wavg = C.carray(res.weightavg, nb, np.float64)
    lib.free_results_wp(ctypes.byref(res))
    out = np.zeros(max(nb - 1, 0), dtype=WP_DTYPE)
    out["rmin"] = rupp[:-1]
    out["rmax"] = rupp[1:]
    out["rpavg"] = rpavg[1:]
    out["wp"] = wp_[1:]
    out["npairs"] = npairs[1:]
    out["weightavg"] = wavg[1:]
    if c_api_timer or c_cell_timer:
        ret = [out]
        if c_api_timer:
            ret.append(o.c_api_time)
        if c_cell_timer:
            ret.append(_cell_timings(o))
        return tuple(ret)
    return out


# field names of Corrfunc/theory/wp.py:271-276; aligned as the C struct api_cell_timings (40 bytes)
CELL_TIMER_DTYPE = np.dtype([("N1", np.int64), ("N2", np.int64), ("time_in_ns", np.int64), ("cellidx1", np.int32),
                             ("cellidx2", np.int32), ("tid", np.int32)], align=True)


def _cell_timings(o):
    """options->cell_timings as the structured array of Corrfunc/theory/wp.py:243-280 (one record
    per GPU work-list task: i-chunk size, j-range length, time, first indices, warp), then freed."""
    n = int(o.totncells_timings)
    if n <= 0 or not o.cell_timings:
        return np.zeros(0, dtype=CELL_TIMER_DTYPE)
    raw = np.ctypeslib.as_array(ctypes.cast(o.cell_timings, ctypes.POINTER(ctypes.c_uint8)),
                                shape=(n * CELL_TIMER_DTYPE.itemsize,))
    out = np.frombuffer(raw.tobytes(), dtype=CELL_TIMER_DTYPE).copy()
    libc = ctypes.CDLL(None)
    libc.free.argtypes = [ctypes.c_void_p]
    libc.free(ctypes.cast(o.cell_timings, ctypes.c_void_p))
    o.cell_timings = None
    o.totncells_timings = 0
    return out


def run_xi(lib, boxsize, nthreads, binfile, X, Y, Z, weights=None, weight_type=None, verbose=False,
           output_ravg=False, xbin_refine_factor=2, ybin_refine_factor=2, zbin_refine_factor=1,
           max_cells_per_dim=100, copy_particles=True, enable_min_sep_opt=True, c_api_timer=False,
           isa="fastest"):
    X = C.as_positions(X)
    Y = C.as_positions(Y, X.dtype)
    Z = C.as_positions(Z, X.dtype)
    w1, _ = C.process_weights(weights, None, X, None, weight_type, True)
    o = _common_options(nthreads, True, boxsize, verbose, output_ravg,
                        (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                        copy_particles, enable_min_sep_opt, c_api_timer, isa, X.dtype)
    extra = C.get_extra_options(C.weight_method_by_name(weight_type))
    keep = []
    C.fill_weights(extra, w1, None, keep)
    res = C.ResultsXi()
    with C.BinFile(binfile) as bf:
        rc = lib.countpairs_xi(len(X), C.ptr(X), C.ptr(Y), C.ptr(Z), float(_boxsize3(boxsize)[0]), int(nthreads),
                               bf.encode(), ctypes.byref(res), ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    nb = res.nbin
    npairs = C.carray(res.npairs, nb, np.uint64)
    rupp = C.carray(res.rupp, nb, np.float64)
    ravg = C.carray(res.ravg, nb, np.float64)
    xi_ = C.carray(res.xi, nb, np.float64)
    wavg = C.carray(res.weightavg, nb, np.float64)
    lib.free_results_xi(ctypes.byref(res))
    out = np.zeros(max(nb - 1, 0), dtype=XI_DTYPE)
    out["rmin"] = rupp[:-1]
    out["rmax"] = rupp[1:]
    out["ravg"] = ravg[1:]
    out["xi"] = xi_[1:]
    out["npairs"] = npairs[1:]
    out["weightavg"] = wavg[1:]
    return (out, o.c_api_time) if c_api_timer else out


def _device_array(a):
    """(device pointer, numpy dtype, length) of a CUDA array (``__cuda_array_interface__``, e.g. a
    torch tensor on the GPU)."""
    iface = getattr(a, "__cuda_array_interface__", None)
    if iface is None:
        raise TypeError("batched counts take device arrays (objects with __cuda_array_interface__)")
    if iface.get("strides") not in (None, (np.dtype(iface["typestr"]).itemsize,)):
        raise ValueError("device arrays must be contiguous")
    return int(iface["data"][0]), np.dtype(iface["typestr"]), int(iface["shape"][0])


class DDCrossBatch:
    """DD(r) cross-correlations of many catalogues against one catalogue, planned once and replayed
    as one CUDA graph (``cf_gpu_batch_plan`` / ``cf_gpu_batch_run``).  ``catalogues`` is a list of
    (X, Y, Z[, weights]) device arrays; ``second`` is (X2, Y2, Z2[, weights2]).  ``run()`` returns
    one record array per catalogue, each equal to
    ``DD(0, nthreads, binfile, X, Y, Z, X2=X2, Y2=Y2, Z2=Z2, ...)`` on the same arrays."""

    def __init__(self, binfile, catalogues, second, periodic=True, boxsize=None, output_ravg=False,
                 weight_type=None, autotune=True, isa="fastest", xbin_refine_factor=2, ybin_refine_factor=2,
                 zbin_refine_factor=1, max_cells_per_dim=100, lib=None):
        if periodic and boxsize is None:
            raise ValueError("Must specify a boxsize if periodic=True")
        self._lib = lib or C.library()
        need_w = weight_type is not None
        cols = [[_device_array(a) for a in cat[:4 if need_w else 3]] for cat in catalogues]
        sec = [_device_array(a) for a in second[:4 if need_w else 3]]
        dt = sec[0][1]
        if dt not in (np.dtype(np.float32), np.dtype(np.float64)):
            raise TypeError("positions must be float32 or float64")
        for cat in cols + [sec]:
            if any(c[1] != dt for c in cat) or any(c[2] != cat[0][2] for c in cat):
                raise ValueError("every array must have the dtype and length of the first")
        o = _common_options(1, periodic, boxsize, False, output_ravg,
                            (xbin_refine_factor, ybin_refine_factor, zbin_refine_factor), max_cells_per_dim,
                            True, True, False, isa, dt)
        nb = len(cols)
        P = ctypes.c_void_p * nb
        self._n1 = (ctypes.c_int64 * nb)(*[c[0][2] for c in cols])
        self._ptr = [P(*[c[k][0] for c in cols]) for k in range(3)]
        self._w = P(*[c[3][0] for c in cols]) if need_w else None
        method = C.weight_method_by_name(weight_type)
        plan = ctypes.c_void_p()
        with C.BinFile(binfile) as bf:
            rc = self._lib.cf_gpu_batch_plan(nb, self._n1, self._ptr[0], self._ptr[1], self._ptr[2], self._w,
                                             sec[0][2], sec[0][0], sec[1][0], sec[2][0],
                                             sec[3][0] if need_w else None, bf.encode(), ctypes.byref(o),
                                             int(method), 1 if autotune else 0, ctypes.byref(plan))
        if rc != 0:
            raise RuntimeError("RuntimeError occurred")
        self._plan = plan
        self.nbatch = nb

    def run(self):
        res = (C.ResultsDD * self.nbatch)()
        if self._lib.cf_gpu_batch_run(self._plan, res) != 0:
            raise RuntimeError("RuntimeError occurred")
        outs = []
        for r in res:
            nb = r.nbin
            out = np.zeros(max(nb - 1, 0), dtype=DD_DTYPE)
            rupp = C.carray(r.rupp, nb, np.float64)
            out["rmin"] = rupp[:-1]
            out["rmax"] = rupp[1:]
            out["ravg"] = C.carray(r.rpavg, nb, np.float64)[1:]
            out["npairs"] = C.carray(r.npairs, nb, np.uint64)[1:]
            out["weightavg"] = C.carray(r.weightavg, nb, np.float64)[1:]
            self._lib.free_results(ctypes.byref(r))
            outs.append(out)
        return outs

    def close(self):
        if getattr(self, "_plan", None):
            self._lib.cf_gpu_batch_free(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_vpf(lib, rmax, nbins, nspheres, numpN, seed, X, Y, Z, verbose=False, periodic=True, boxsize=None,
            xbin_refine_factor=1, ybin_refine_factor=1, zbin_refine_factor=1, max_cells_per_dim=100,
            copy_particles=True, c_api_timer=False, isa="fastest"):
    """Counts in spheres: Corrfunc/theory/vpf.py:17-262 (countspheres)."""
    X = C.as_positions(X)
    dt = X.dtype
    Y = C.as_positions(Y, dt)
    Z = C.as_positions(Z, dt)
    o = _common_options(1, periodic, boxsize, verbose, False, (xbin_refine_factor, ybin_refine_factor,
                                                               zbin_refine_factor),
                        max_cells_per_dim, copy_particles, True, c_api_timer, isa, dt)
    extra = C.get_extra_options()
    res = C.ResultsVpf()
    rc = lib.countspheres(len(X), C.ptr(X), C.ptr(Y), C.ptr(Z), float(rmax), int(nbins), int(nspheres), int(numpN),
                          int(seed) & 0xffffffffffffffff, ctypes.byref(res), ctypes.byref(o), ctypes.byref(extra))
    if rc != 0:
        raise RuntimeError("RuntimeError occurred")
    out = C.vpf_rows(res, int(numpN))
    lib.free_results_countspheres(ctypes.byref(res))
    return (out, o.c_api_time) if c_api_timer else out


def vpf(*args, **kwargs):
    """Counts in spheres pN(r); see Corrfunc.theory.vpf."""
    return run_vpf(C.library(), *args, **kwargs)


def DD(*args, **kwargs):
    """3-D pair counts DD(r); see Corrfunc.theory.DD (Corrfunc/theory/DD.py:16)."""
    return run_DD(C.library(), *args, **kwargs)


def DDrppi(*args, **kwargs):
    """Pair counts in (rp, pi); see Corrfunc.theory.DDrppi."""
    return run_DDrppi(C.library(), *args, **kwargs)


def DDsmu(*args, **kwargs):
    """Pair counts in (s, mu); see Corrfunc.theory.DDsmu."""
    return run_DDsmu(C.library(), *args, **kwargs)


def wp(*args, **kwargs):
    """Projected correlation function w_p(rp) in a periodic box; see Corrfunc.theory.wp."""
    return run_wp(C.library(), *args, **kwargs)


def find_fastest_wp_bin_refs(boxsize, pimax, nthreads, binfile, X, Y, Z, verbose=False, output_rpavg=False,
                             max_cells_per_dim=100, isa="fastest", maxbinref=3, nrepeats=3, return_runtimes=False):
    """The combination of bin refine factors (1 .. maxbinref per axis) with the shortest mean wp
    runtime over nrepeats calls, as Corrfunc/theory/wp.py:17-216 finds it: returns (nx, ny, nz),
    and with return_runtimes also the structured array of every combination's nx, ny, nz,
    avg_time and sigma_time (seconds of the call).  Here the refine factors only define the
    reference lattice whose cell pairs the counts follow, not the GPU's own lattice, so the
    runtimes come out close to one another; ``corrfunc_gb300.set_autotune`` tunes the GPU's
    lattice instead (DD and xi)."""
    import itertools
    import time
    refs = range(1, int(maxbinref) + 1)
    dtype = np.dtype([("nx", np.int64), ("ny", np.int64), ("nz", np.int64), ("avg_time", np.float64),
                      ("sigma_time", np.float64)])
    runtimes = np.zeros(int(maxbinref) ** 3, dtype=dtype)
    runtimes["avg_time"] = runtimes["sigma_time"] = np.inf
    for k, (nx, ny, nz) in enumerate(itertools.product(refs, refs, refs)):
        total = total_sq = 0.0
        for _ in range(int(nrepeats)):
            t0 = time.time()
            wp(boxsize, pimax, nthreads, binfile, X, Y, Z, verbose=verbose, output_rpavg=output_rpavg,
               xbin_refine_factor=nx, ybin_refine_factor=ny, zbin_refine_factor=nz,
               max_cells_per_dim=max_cells_per_dim, isa=isa)
            dt = time.time() - t0
            total += dt
            total_sq += dt * dt
        avg = total / nrepeats
        sigma = np.sqrt(max(total_sq / nrepeats - avg * avg, 0.0))
        runtimes[k] = (nx, ny, nz, avg, sigma)
        if verbose:
            print("nx = {0} ny = {1} nz = {2} avg time = {3:0.3g} sec".format(nx, ny, nz, avg))
    best = runtimes[np.argmin(runtimes["avg_time"])]
    best = (int(best["nx"]), int(best["ny"]), int(best["nz"]))
    if return_runtimes:
        return best, runtimes
    return best


def xi(*args, **kwargs):
    """3-D correlation function xi(r) in a periodic box; see Corrfunc.theory.xi."""
    return run_xi(C.library(), *args, **kwargs)
