"""ctypes view of the C ABI in include/corrfunc_gb300.h.

The struct layouts are byte-identical to Corrfunc 2.5.3's utils/defs.h and the per-module
result structs, so the same declarations drive libcorrfunc_gb300.so and any other library that
exports the reference's C API.
"""
import ctypes
import os
from ctypes import (POINTER, Structure, c_char, c_double, c_int, c_int8, c_int32, c_int64,
                    c_size_t, c_uint8, c_uint16, c_uint32, c_uint64, c_void_p)

import numpy as np

API_VERSION = b'"2.5.3"'  # quotes included, as the reference's STR(VERSION) produces
BOXSIZE_NOTGIVEN = -2.0
NLATMAX = 100
MAX_NUM_WEIGHTS = 10
WEIGHT_NONE = -42
WEIGHT_PAIR_PRODUCT = 0
BINNING_CUST = 0x1
PRECISION_FP32_REFINE = 0
PRECISION_FP64 = 1

ISA_ENUMS = {"FASTEST": -1, "FALLBACK": 0, "SSE": 1, "SSE2": 2, "SSE3": 3, "SSSE3": 4, "SSE4": 5,
             "SSE42": 6, "AVX": 7, "AVX2": 8, "AVX512F": 9}
VALID_ISA = ["FALLBACK", "AVX512F", "AVX2", "AVX", "SSE42", "FASTEST"]


class ApiCellTimings(Structure):
    _fields_ = [("N1", c_int64), ("N2", c_int64), ("time_in_ns", c_int64),
                ("first_cellindex", c_int), ("second_cellindex", c_int), ("tid", c_int)]


_RESERVED = 1024 - 33 - 8 - 11 * 8 - 3 * 4 - 2 - 16 - 8 - 8


class ConfigOptions(Structure):
    _fields_ = [("boxsize_x", c_double), ("boxsize_y", c_double), ("boxsize_z", c_double),
                ("OMEGA_M", c_double), ("OMEGA_B", c_double), ("OMEGA_L", c_double),
                ("HUBBLE", c_double), ("LITTLE_H", c_double), ("SIGMA_8", c_double), ("NS", c_double),
                ("c_api_time", c_double),
                ("cell_timings", POINTER(ApiCellTimings)), ("totncells_timings", c_int64),
                ("float_type", c_size_t), ("instruction_set", c_int32), ("version", c_char * 32),
                ("verbose", c_uint8), ("c_api_timer", c_uint8), ("c_cell_timer", c_uint8),
                ("need_avg_sep", c_uint8), ("autocorr", c_uint8), ("periodic", c_uint8),
                ("sort_on_z", c_uint8), ("is_comoving_dist", c_uint8), ("link_in_dec", c_uint8),
                ("link_in_ra", c_uint8), ("fast_divide_and_NR_steps", c_uint8), ("fast_acos", c_uint8),
                ("enable_min_sep_opt", c_uint8), ("bin_refine_factors", c_int8 * 3),
                ("max_cells_per_dim", c_uint16), ("copy_particles", c_uint8), ("use_heap_sort", c_uint8),
                ("binning_flags", c_uint32), ("reserved", c_uint8 * _RESERVED)]


class WeightStruct(Structure):
    _fields_ = [("weights", c_void_p * MAX_NUM_WEIGHTS), ("num_weights", c_int64)]


class ExtraOptions(Structure):
    _fields_ = [("weights0", WeightStruct), ("weights1", WeightStruct), ("weight_method", c_int),
                ("reserved", c_uint8 * (1024 - 2 * ctypes.sizeof(WeightStruct) - 4))]


class ResultsDD(Structure):
    _fields_ = [("npairs", POINTER(c_uint64)), ("rupp", POINTER(c_double)), ("rpavg", POINTER(c_double)),
                ("weightavg", POINTER(c_double)), ("nbin", c_int)]


class ResultsRpPi(Structure):
    _fields_ = [("npairs", POINTER(c_uint64)), ("rupp", POINTER(c_double)), ("rpavg", POINTER(c_double)),
                ("weightavg", POINTER(c_double)), ("pimax", c_double), ("nbin", c_int), ("npibin", c_int)]


class ResultsSMu(Structure):
    _fields_ = [("npairs", POINTER(c_uint64)), ("supp", POINTER(c_double)), ("savg", POINTER(c_double)),
                ("mu_max", c_double), ("mu_min", c_double), ("weightavg", POINTER(c_double)),
                ("nsbin", c_int), ("nmu_bins", c_int)]


class ResultsWp(Structure):
    _fields_ = [("npairs", POINTER(c_uint64)), ("wp", POINTER(c_double)), ("rupp", POINTER(c_double)),
                ("rpavg", POINTER(c_double)), ("weightavg", POINTER(c_double)), ("pimax", c_double),
                ("nbin", c_int)]


class ResultsXi(Structure):
    _fields_ = [("npairs", POINTER(c_uint64)), ("xi", POINTER(c_double)), ("rupp", POINTER(c_double)),
                ("ravg", POINTER(c_double)), ("weightavg", POINTER(c_double)), ("nbin", c_int)]


class ResultsVpf(Structure):
    """results_countspheres / results_countspheres_mocks (pN is an array of nbin rows)."""
    _fields_ = [("pN", POINTER(POINTER(c_double))), ("rmax", c_double), ("nbin", c_int), ("nc", c_int),
                ("num_pN", c_int)]


class ResultsTheta(Structure):
    _fields_ = [("npairs", POINTER(c_uint64)), ("theta_upp", POINTER(c_double)),
                ("theta_avg", POINTER(c_double)), ("weightavg", POINTER(c_double)), ("nbin", c_int)]


assert ctypes.sizeof(ConfigOptions) == 1024
assert ctypes.sizeof(ExtraOptions) == 1024

# exported symbol -> (argtypes, restype)
_PROTOS = {
    "countpairs": ([c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int, c_int,
                    ctypes.c_char_p, POINTER(ResultsDD), POINTER(ConfigOptions), POINTER(ExtraOptions)], c_int),
    "free_results": ([POINTER(ResultsDD)], None),
    "countpairs_rp_pi": ([c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                          c_int, ctypes.c_char_p, c_double, POINTER(ResultsRpPi), POINTER(ConfigOptions),
                          POINTER(ExtraOptions)], c_int),
    "free_results_rp_pi": ([POINTER(ResultsRpPi)], None),
    "countpairs_s_mu": ([c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                         c_int, ctypes.c_char_p, c_double, c_int, POINTER(ResultsSMu), POINTER(ConfigOptions),
                         POINTER(ExtraOptions)], c_int),
    "free_results_s_mu": ([POINTER(ResultsSMu)], None),
    "countpairs_wp": ([c_int64, c_void_p, c_void_p, c_void_p, c_double, c_int, ctypes.c_char_p, c_double,
                       POINTER(ResultsWp), POINTER(ConfigOptions), POINTER(ExtraOptions)], c_int),
    "free_results_wp": ([POINTER(ResultsWp)], None),
    "countpairs_xi": ([c_int64, c_void_p, c_void_p, c_void_p, c_double, c_int, ctypes.c_char_p,
                       POINTER(ResultsXi), POINTER(ConfigOptions), POINTER(ExtraOptions)], c_int),
    "free_results_xi": ([POINTER(ResultsXi)], None),
    "countpairs_theta_mocks": ([c_int64, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int, c_int,
                                ctypes.c_char_p, POINTER(ResultsTheta), POINTER(ConfigOptions),
                                POINTER(ExtraOptions)], c_int),
    "free_results_countpairs_theta": ([POINTER(ResultsTheta)], None),
    # the mocks result structs have the layouts of the theory rp-pi / s-mu ones
    "countpairs_mocks": ([c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                          c_int, ctypes.c_char_p, c_double, c_int, POINTER(ResultsRpPi), POINTER(ConfigOptions),
                          POINTER(ExtraOptions)], c_int),
    "free_results_mocks": ([POINTER(ResultsRpPi)], None),
    "countpairs_mocks_s_mu": ([c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                               c_int, ctypes.c_char_p, c_double, c_int, c_int, POINTER(ResultsSMu),
                               POINTER(ConfigOptions), POINTER(ExtraOptions)], c_int),
    "free_results_mocks_s_mu": ([POINTER(ResultsSMu)], None),
    "countspheres": ([c_int64, c_void_p, c_void_p, c_void_p, c_double, c_int, c_int, c_int, ctypes.c_ulong,
                      POINTER(ResultsVpf), POINTER(ConfigOptions), POINTER(ExtraOptions)], c_int),
    "free_results_countspheres": ([POINTER(ResultsVpf)], None),
    "countspheres_mocks": ([c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                            c_double, c_int, c_int, c_int, ctypes.c_char_p, c_int, POINTER(ResultsVpf),
                            POINTER(ConfigOptions), POINTER(ExtraOptions)], c_int),
    "free_results_countspheres_mocks": ([POINTER(ResultsVpf)], None),
}

_GPU_PROTOS = {
    "cf_gpu_set_precision": ([c_int], c_int),
    "cf_gpu_get_precision": ([], c_int),
    "cf_gpu_set_autotune": ([c_int], c_int),
    "cf_gpu_get_autotune": ([], c_int),
}


class GpuStats(Structure):
    _fields_ = [("pair_kernel_ms", c_double), ("gridlink_ms", c_double), ("total_gpu_ms", c_double),
                ("pairs_evaluated", c_uint64), ("pairs_refined", c_uint64), ("tasks", c_uint64),
                ("kernel_launches", c_int), ("num_cells", c_int), ("blocks_per_sm", c_int),
                ("warps_per_block", c_int), ("lane_stride", c_int), ("column_split", c_int), ("pairs_slow", c_uint64)]


_GPU_PROTOS["cf_gpu_last_stats"] = ([POINTER(GpuStats)], c_int)
_GPU_PROTOS["cf_gpu_batch_plan"] = (
    [c_int, POINTER(c_int64), POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p), c_int64,
     c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_char_p, POINTER(ConfigOptions), c_int, c_int,
     POINTER(c_void_p)], c_int)
_GPU_PROTOS["cf_gpu_batch_run"] = ([c_void_p, POINTER(ResultsDD)], c_int)
_GPU_PROTOS["cf_gpu_batch_free"] = ([c_void_p], None)
_GPU_PROTOS["cf_gpu_countpairs_cross_noalloc"] = (
    [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
     POINTER(c_double), c_int, c_double, c_double, c_double, c_int, POINTER(c_uint64), POINTER(c_double),
     POINTER(c_double), c_void_p], c_int)

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PACKAGE_DIR, "libcorrfunc_gb300.so")
# the benchmark's work unit (cf_reference_candidate_pairs) without the CUDA engine
WORKUNIT_LIB_PATH = os.path.join(PACKAGE_DIR, "libcf_workunit.so")
_WORKUNIT_PROTO = ([c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                    ctypes.c_char_p, POINTER(ConfigOptions), POINTER(c_uint64)], c_int)


def bind(path, gpu=False):
    """Load a shared library that exports the reference's pair-counting C API."""
    lib = ctypes.CDLL(path)
    for name, (argt, rest) in _PROTOS.items():
        if not hasattr(lib, name):
            continue
        f = getattr(lib, name)
        f.argtypes = argt
        f.restype = rest
    if gpu:
        for name, (argt, rest) in _GPU_PROTOS.items():
            f = getattr(lib, name)
            f.argtypes = argt
            f.restype = rest
    return lib


_LIB = None


def library():
    """The GB300 library.  Raises if it has not been built (there is no fallback)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcorrfunc_gb300.so is not built (run `python -m corrfunc_gb300.build`); "
                              "corrfunc_gb300 has no CPU fallback")
        _LIB = bind(LIB_PATH, gpu=True)
    return _LIB


_WORKUNIT = None


def workunit_library():
    """Host-only library exporting cf_reference_candidate_pairs (loads no GPU code)."""
    global _WORKUNIT
    if _WORKUNIT is None:
        if not os.path.exists(WORKUNIT_LIB_PATH):
            raise ImportError("libcf_workunit.so is not built (run `python -m corrfunc_gb300.build`)")
        lib = ctypes.CDLL(WORKUNIT_LIB_PATH)
        lib.cf_reference_candidate_pairs.argtypes, lib.cf_reference_candidate_pairs.restype = _WORKUNIT_PROTO
        _WORKUNIT = lib
    return _WORKUNIT


def reference_candidate_pairs(set1, set2, binfile, options, autocorr):
    """The reference lattice's candidate pairs of a countpairs() call (the benchmark work unit)."""
    lib = workunit_library()
    out = c_uint64()
    rc = lib.cf_reference_candidate_pairs(len(set1[0]), *(ptr(a) for a in set1[:3]), len(set2[0]),
                                          *(ptr(a) for a in set2[:3]), int(autocorr), binfile.encode(),
                                          ctypes.byref(options), ctypes.byref(out))
    if rc != 0:
        raise RuntimeError("cf_reference_candidate_pairs failed")
    return int(out.value)


def get_config_options():
    """Python restatement of get_config_options() as the reference's CPython binding
    initialises it (theory/python_bindings/_countpairs.c:1152-1160)."""
    o = ConfigOptions()
    ctypes.memset(ctypes.byref(o), 0, ctypes.sizeof(o))
    o.version = API_VERSION
    o.boxsize_x = o.boxsize_y = o.boxsize_z = BOXSIZE_NOTGIVEN
    o.float_type = 8
    o.instruction_set = -1
    o.periodic = 1
    o.link_in_dec = 1
    o.link_in_ra = 1
    o.enable_min_sep_opt = 1
    o.copy_particles = 1
    o.max_cells_per_dim = NLATMAX
    o.bin_refine_factors[0] = 2
    o.bin_refine_factors[1] = 2
    o.bin_refine_factors[2] = 1
    o.binning_flags = 0
    return o


def get_extra_options(weight_method=WEIGHT_NONE):
    e = ExtraOptions()
    ctypes.memset(ctypes.byref(e), 0, ctypes.sizeof(e))
    e.weight_method = weight_method
    nw = 1 if weight_method == WEIGHT_PAIR_PRODUCT else 0
    e.weights0.num_weights = nw
    e.weights1.num_weights = nw
    return e


def host_highest_isa():
    """The highest instruction set of this host, as the reference's CPython binding resolves
    isa = -1 before calling the C library (theory/python_bindings/_countpairs.c:1239-1241)."""
    try:
        flags = open("/proc/cpuinfo").read()
    except OSError:
        return ISA_ENUMS["FALLBACK"]
    for name, flag in (("AVX512F", " avx512f"), ("AVX2", " avx2"), ("AVX", " avx "), ("SSE42", " sse4_2")):
        if flag in flags:
            return ISA_ENUMS[name]
    return ISA_ENUMS["FALLBACK"]


def translate_isa(isa):
    """isa string -> enum (Corrfunc/utils.py:464-518); "fastest" resolves to the host's highest."""
    if not isinstance(isa, str):
        raise TypeError("isa must be a string")
    up = isa.upper()
    if up not in VALID_ISA:
        raise ValueError("Desired instruction set = {0} is not in the list of valid instruction sets = {1}"
                         .format(isa, VALID_ISA))
    v = ISA_ENUMS[up]
    return host_highest_isa() if v == -1 else v


def set_refine(o, refine):
    """Custom refine factors switch the binning scheme to BINNING_CUST
    (theory/python_bindings/_countpairs.c:1243-1250)."""
    if tuple(refine) != (o.bin_refine_factors[0], o.bin_refine_factors[1], o.bin_refine_factors[2]):
        for k in range(3):
            o.bin_refine_factors[k] = int(refine[k])
        o.binning_flags = (o.binning_flags & ~0xF) | BINNING_CUST


def weight_method_by_name(name):
    if name is None or name == "":
        return WEIGHT_NONE
    if name in ("pair_product", "p"):
        return WEIGHT_PAIR_PRODUCT
    raise ValueError('unknown weight_type "%s"!' % name)


class BinFile:
    """Context manager: a bin-file path, or a temporary file written from an array of edges
    (Corrfunc/utils.py:324-381)."""

    def __init__(self, binfile):
        self.binfile = binfile
        self.path = None
        self.tmp = False

    def __enter__(self):
        b = self.binfile
        if isinstance(b, (str, bytes, os.PathLike)):
            p = os.fspath(b)
            if isinstance(p, bytes):
                p = p.decode()
            if not os.path.isfile(p):
                raise IOError("Could not find file = `{0}` containing the bins".format(p))
            self.path = p
            return p
        edges = list(b)
        if len(edges) < 1:
            raise TypeError("Input `binfile` was not a valid array (>= 1 element).Num elements = 0")
        import tempfile
        edges = sorted(edges)
        with tempfile.NamedTemporaryFile(delete=False, mode="w", suffix=".bins") as f:
            for i in range(len(edges) - 1):
                f.write("{0} {1}\n".format(edges[i], edges[i + 1]))
            self.path = f.name
        self.tmp = True
        return self.path

    def __exit__(self, *exc):
        if self.tmp and self.path and os.path.exists(self.path):
            os.remove(self.path)
        return False


def as_positions(arr, dtype=None):
    a = np.asarray(arr)
    if dtype is None:
        dtype = a.dtype if a.dtype in (np.float32, np.float64) else np.float64
    return np.ascontiguousarray(a, dtype=dtype)


def prep_weights(w, x):
    """Scalar / 1-D / 2-D weights -> (nweights, n) (Corrfunc/utils.py:967-1027)."""
    if w is None:
        return None
    if isinstance(w, float):
        w = np.array(w, dtype=x.dtype)
    w = np.atleast_1d(w)
    if w.shape[-1] == 1:
        w = np.tile(w, len(x))
    w = np.atleast_2d(w)
    return np.ascontiguousarray(w, dtype=x.dtype)


def process_weights(weights1, weights2, X1, X2, weight_type, autocorr):
    if weight_type is None:
        return None, None
    weights1 = prep_weights(weights1, X1)
    if not autocorr:
        weights2 = prep_weights(weights2, X2)
        if (weights1 is None) != (weights2 is None) and weight_type != "pair_product":
            raise ValueError("If using a weight_type other than 'pair_product', you must provide both weight arrays.")
        if weights1 is None and weights2 is not None:
            weights1 = np.ones((len(weights2), len(X1)), dtype=X1.dtype)
        if weights2 is None and weights1 is not None:
            weights2 = np.ones((len(weights1), len(X2)), dtype=X2.dtype)
    else:
        weights2 = None
    return weights1, weights2


def fill_weights(extra, weights1, weights2, keep):
    if weights1 is not None:
        for k in range(weights1.shape[0]):
            row = np.ascontiguousarray(weights1[k])
            keep.append(row)
            extra.weights0.weights[k] = row.ctypes.data
        extra.weights0.num_weights = weights1.shape[0]
    if weights2 is not None:
        for k in range(weights2.shape[0]):
            row = np.ascontiguousarray(weights2[k])
            keep.append(row)
            extra.weights1.weights[k] = row.ctypes.data
        extra.weights1.num_weights = weights2.shape[0]


def ptr(a):
    return None if a is None else c_void_p(a.ctypes.data)


def carray(p, n, dtype):
    """Copy n elements from a C pointer into a numpy array."""
    if n <= 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(p, shape=(n,)).astype(dtype, copy=True)


def vpf_rows(res, num_pN):
    """(rmax_k, pN[k][0..num_pN-1]) rows as the reference's bindings build them
    (theory/python_bindings/_countpairs.c:2674-2690): rmax_k = (k + 1) * rmax / nbin."""
    dt = np.dtype([("rmax", np.float64), ("pN", (np.float64, num_pN))])
    out = np.zeros(res.nbin, dtype=dt)
    rstep = res.rmax / float(res.nbin) if res.nbin else 0.0
    for k in range(res.nbin):
        out["rmax"][k] = (k + 1) * rstep
        out["pN"][k] = [res.pN[k][i] for i in range(num_pN)]
    return out
