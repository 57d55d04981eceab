"""C ABI checks that need no GPU: exported symbols, struct layouts against the reference's
headers, bin parsing, reference-geometry resolution, and the error paths (same return codes as
the reference library for the same invalid inputs)."""
import ctypes
import os
import re
import subprocess
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "corrfunc_gb300.h")
STAGED_UTILS = os.path.join(ROOT, "oracle", "_ref", "src", "utils")


@pytest.fixture(scope="module")
def lib():
    from corrfunc_gb300 import _capi as C
    if not os.path.exists(C.LIB_PATH):
        from corrfunc_gb300 import build
        build.build()
    return C.bind(C.LIB_PATH, gpu=True)


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = []
    for m in re.finditer(r"^(?!static)(?:int|void)\s+([a-z_0-9]+)\s*\(", src, flags=re.M):
        names.append(m.group(1))
    return names


def test_library_exports_every_declared_symbol(lib):
    names = header_functions()
    assert "countpairs" in names and "countpairs_theta_mocks" in names and len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_ctypes_struct_sizes():
    from corrfunc_gb300 import _capi as C
    assert ctypes.sizeof(C.ConfigOptions) == 1024
    assert ctypes.sizeof(C.ExtraOptions) == 1024


FIELDS = ["boxsize", "boxsize_y", "boxsize_z", "OMEGA_M", "NS", "c_api_time", "cell_timings", "totncells_timings",
          "float_type", "instruction_set", "version", "verbose", "c_api_timer", "c_cell_timer", "need_avg_sep",
          "autocorr", "periodic", "sort_on_z", "is_comoving_dist", "link_in_dec", "link_in_ra",
          "fast_divide_and_NR_steps", "fast_acos", "enable_min_sep_opt", "bin_refine_factors", "max_cells_per_dim",
          "copy_particles", "use_heap_sort", "binning_flags", "reserved"]


def _offsets_program(include):
    lines = ['#include <stdio.h>', '#include <stddef.h>', include, 'int main(void){']
    lines.append('printf("%zu %zu\\n", sizeof(struct config_options), sizeof(struct extra_options));')
    for f in FIELDS:
        lines.append('printf("%zu\\n", offsetof(struct config_options, ' + f + '));')
    for f in ["weights0", "weights1", "weight_method", "reserved"]:
        lines.append('printf("%zu\\n", offsetof(struct extra_options, ' + f + '));')
    lines.append('return 0;}')
    return "\n".join(lines)


def _run_c(src, incdirs):
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-std=gnu11", "-w", c, "-o", exe] + ["-I" + i for i in incdirs])
        return subprocess.check_output([exe]).decode()


def test_header_compiles_and_matches_its_own_layout():
    out = _run_c(_offsets_program('#include "corrfunc_gb300.h"'), [os.path.join(ROOT, "include")])
    assert out.splitlines()[0] == "1024 1024"


@pytest.mark.skipif(not os.path.isdir(STAGED_UTILS), reason="staged reference headers not available")
def test_struct_layout_identical_to_reference_defs_h():
    mine = _run_c(_offsets_program('#include "corrfunc_gb300.h"'), [os.path.join(ROOT, "include")])
    ref = _run_c(_offsets_program('#define VERSION "2.5.3"\n#include "defs.h"'), [STAGED_UTILS])
    assert mine == ref


def test_version_string_matches_reference_convention(lib):
    from corrfunc_gb300 import _capi as C
    assert C.API_VERSION == b'"2.5.3"'


def _bins_file(text):
    f = tempfile.NamedTemporaryFile("w", delete=False, suffix=".bins")
    f.write(text)
    f.close()
    return f.name


def test_setup_bins_matches_oracle(lib, orc):
    lib.cf_setup_bins.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
    lib.cf_setup_bins.restype = ctypes.c_int
    text = "# comment line\n  0.1 0.2\n\n0.2   0.5 trailing\n   # indented comment\n0.5 1.25\n"
    p = _bins_file(text)
    try:
        rmin, rmax, nb = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        arr = ctypes.POINTER(ctypes.c_double)()
        assert lib.cf_setup_bins(p.encode(), ctypes.byref(rmin), ctypes.byref(rmax), ctypes.byref(nb),
                                 ctypes.byref(arr)) == 0
        got = np.array([arr[i] for i in range(nb.value)])
        want = orc.read_bins(p)
        assert np.array_equal(got, want)
        assert rmin.value == 0.1 and rmax.value == 1.25
    finally:
        os.remove(p)


class RefRule(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("periodic", ctypes.c_int), ("boxsize", ctypes.c_double * 3),
                ("max_size", ctypes.c_double * 3), ("refine", ctypes.c_int * 3), ("custom_refine", ctypes.c_int),
                ("max_cells", ctypes.c_int), ("dfl_kind", ctypes.c_int), ("boost_kind", ctypes.c_int),
                ("np1", ctypes.c_int64)]


class Geometry(ctypes.Structure):
    _fields_ = [("periodic", ctypes.c_int * 3), ("wrap", ctypes.c_double * 3), ("ref_min", ctypes.c_double * 3),
                ("ref_inv", ctypes.c_double * 3), ("ref_nmesh", ctypes.c_int * 3), ("refine_used", ctypes.c_int * 3)]


@pytest.mark.parametrize("seed", range(40))
def test_reference_geometry_matches_oracle(lib, orc, seed):
    rng = np.random.default_rng(seed)
    kind = ["extent", "box"][seed % 2]
    dfl = ["per_axis", "xi", "wp", "none"][(seed // 2) % 4] if kind == "box" else ["per_axis", "none"][seed % 3 == 0]
    if kind == "box" and dfl in ("per_axis", "none"):
        dfl = "xi"
    L = float(rng.uniform(50, 2000))
    rmax = float(rng.uniform(0.5, 0.45 * L))
    zsize = float(rng.uniform(0.5, 0.45 * L))
    lo = list(rng.uniform(0, 0.1 * L, 3))
    hi = [lo[a] + float(rng.uniform(0.3, 0.9)) * L for a in range(3)]
    refine = [int(v) for v in rng.integers(1, 4, 3)]
    custom = bool(rng.integers(0, 2))
    np1 = int(rng.integers(1, 10 ** 6))
    max_cells = int(rng.integers(2, 120))
    box = (L, L, L) if (kind == "box" or seed % 5) else (L, -1.0, 0.0)
    R = RefRule()
    R.kind = 1 if kind == "extent" else 2
    R.periodic = 1
    for a in range(3):
        R.boxsize[a] = box[a]
        R.max_size[a] = (rmax, rmax, zsize)[a]
        R.refine[a] = refine[a]
    R.custom_refine = int(custom)
    R.max_cells = max_cells
    R.dfl_kind = {"per_axis": 0, "xi": 1, "wp": 2, "none": 3}[dfl]
    R.boost_kind = 1 if dfl == "none" else 0
    R.np1 = np1
    G = Geometry()
    lib.cf_resolve_geometry.argtypes = [ctypes.POINTER(RefRule), ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(Geometry)]
    lib.cf_resolve_geometry.restype = ctypes.c_int
    lo_c = (ctypes.c_double * 3)(*lo)
    hi_c = (ctypes.c_double * 3)(*hi)
    try:
        want = orc.reference_lattice(kind, lo, hi, box, True, (rmax, rmax, zsize), refine, custom, max_cells,
                                     np1, dfl)
    except RuntimeError:
        assert lib.cf_resolve_geometry(ctypes.byref(R), lo_c, hi_c, ctypes.byref(G)) != 0
        return
    assert lib.cf_resolve_geometry(ctypes.byref(R), lo_c, hi_c, ctypes.byref(G)) == 0
    lat_min, lat_inv, nmesh, wrap, per = want
    assert list(G.ref_nmesh) == list(nmesh)
    assert list(G.ref_min) == list(lat_min)
    assert list(G.ref_inv) == list(lat_inv)
    assert list(G.wrap) == list(wrap)
    assert list(G.periodic) == list(per)


def _call_dd(lib, **over):
    """countpairs() with one field of the options / arguments made invalid."""
    from corrfunc_gb300 import _capi as C
    x = np.linspace(1.0, 9.0, 50)
    o = C.get_config_options()
    o.verbose = 0
    o.boxsize_x = o.boxsize_y = o.boxsize_z = 10.0
    for k, v in over.get("opt", {}).items():
        setattr(o, k, v)
    e = C.get_extra_options()
    res = C.ResultsDD()
    bins = over.get("bins", [0.5, 1.0, 2.0])
    with C.BinFile(bins) as bf:
        return lib.countpairs(len(x), C.ptr(x), C.ptr(x), C.ptr(x), 0, None, None, None, 1,
                              over.get("autocorr", 1), bf.encode(), ctypes.byref(res), ctypes.byref(o), ctypes.byref(e))


ERROR_CASES = {
    "bad_version": dict(opt=dict(version=b"2.4.0")),
    "bad_float_type": dict(opt=dict(float_type=3)),
    "boxsize_not_given": dict(opt=dict(boxsize_x=-2.0)),
    "rmin_ge_rmax": dict(bins=[2.0, 2.0]),
    "bad_autocorr": dict(autocorr=2),
    "rmax_ge_half_box": dict(bins=[0.5, 6.0]),
}


@pytest.mark.parametrize("name", sorted(ERROR_CASES))
def test_error_paths_fail_like_the_reference(lib, name):
    """Invalid inputs return EXIT_FAILURE from the GPU library; where the reference library is
    built, it returns the same code for the same input."""
    rc = _call_dd(lib, **ERROR_CASES[name])
    assert rc == 1
    refp = os.path.join(ROOT, "oracle", "_ref", "libcf_ref_DD.so")
    if os.path.exists(refp) and name != "bad_autocorr":
        from corrfunc_gb300 import _capi as C
        assert _call_dd(C.bind(refp), **ERROR_CASES[name]) == 1


def test_theta_rejects_declination_above_180(lib):
    from corrfunc_gb300 import _capi as C
    ra = np.array([10.0, 20.0])
    dec = np.array([10.0, 190.0])
    o = C.get_config_options()
    e = C.get_extra_options()
    res = C.ResultsTheta()
    with C.BinFile([0.1, 1.0]) as bf:
        rc = lib.countpairs_theta_mocks(2, C.ptr(ra), C.ptr(dec), 2, C.ptr(ra), C.ptr(dec), 1, 1, bf.encode(),
                                        ctypes.byref(res), ctypes.byref(o), ctypes.byref(e))
    assert rc == 1


def test_smu_rejects_bad_mu(lib):
    from corrfunc_gb300 import _capi as C
    x = np.linspace(1.0, 9.0, 20)
    for mu_max, nmu in [(1.5, 5), (0.0, 5), (0.5, 0)]:
        o = C.get_config_options()
        o.boxsize_x = o.boxsize_y = o.boxsize_z = 10.0
        e = C.get_extra_options()
        res = C.ResultsSMu()
        with C.BinFile([0.5, 1.0, 2.0]) as bf:
            rc = lib.countpairs_s_mu(len(x), C.ptr(x), C.ptr(x), C.ptr(x), 0, None, None, None, 1, 1, bf.encode(),
                                     mu_max, nmu, ctypes.byref(res), ctypes.byref(o), ctypes.byref(e))
        assert rc == 1


def _call_mocks(lib, smu=False, cosmology=1, dec_value=10.0, mu_max=1.0, nmu=5, bins=(0.5, 1.0, 2.0), pimax=10.0):
    from corrfunc_gb300 import _capi as C
    ra = np.array([150.0, 150.1, 150.2])
    dec = np.array([10.0, 10.1, dec_value])
    cz = np.array([8000.0, 8010.0, 8020.0])
    o = C.get_config_options()
    e = C.get_extra_options()
    with C.BinFile(list(bins)) as bf:
        if smu:
            res = C.ResultsSMu()
            return lib.countpairs_mocks_s_mu(3, C.ptr(ra), C.ptr(dec), C.ptr(cz), 3, C.ptr(ra), C.ptr(dec), C.ptr(cz), 1,
                                             1, bf.encode(), mu_max, nmu, cosmology, ctypes.byref(res),
                                             ctypes.byref(o), ctypes.byref(e))
        res = C.ResultsRpPi()
        return lib.countpairs_mocks(3, C.ptr(ra), C.ptr(dec), C.ptr(cz), 3, C.ptr(ra), C.ptr(dec), C.ptr(cz), 1, 1,
                                    bf.encode(), pimax, cosmology, ctypes.byref(res), ctypes.byref(o),
                                    ctypes.byref(e))


@pytest.mark.parametrize("smu", [False, True])
def test_mocks_reject_bad_inputs(lib, smu):
    """Unknown cosmology, DEC above 180 and a zero lower separation edge fail as in
    mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:62-66,283-298 (and the DDsmu_mocks copies);
    mu_max outside (0, 1] and nmu_bins < 1 fail for DDsmu_mocks."""
    assert _call_mocks(lib, smu, cosmology=3) == 1
    assert _call_mocks(lib, smu, dec_value=190.0) == 1
    assert _call_mocks(lib, smu, bins=(0.0, 1.0, 2.0)) == 1
    if smu:
        assert _call_mocks(lib, True, mu_max=1.5) == 1
        assert _call_mocks(lib, True, mu_max=0.0) == 1
        assert _call_mocks(lib, True, nmu=0) == 1
    else:
        assert _call_mocks(lib, False, pimax=0.5) == 1


def test_vpf_rejects_bad_inputs(lib, tmp_path):
    """countspheres / countspheres_mocks input checks (theory/vpf/countspheres_impl.c.src:162-167,
    mocks/vpf_mocks/countspheres_mocks_impl.c.src:219-222, unknown cosmology)."""
    from corrfunc_gb300 import _capi as C
    x = np.linspace(1.0, 9.0, 30)
    for rmax, nbin, nc, npn in [(0.0, 5, 10, 3), (1.0, 0, 10, 3), (1.0, 5, 0, 3), (1.0, 5, 10, 0)]:
        o = C.get_config_options()
        o.boxsize_x = o.boxsize_y = o.boxsize_z = 10.0
        res = C.ResultsVpf()
        assert lib.countspheres(len(x), C.ptr(x), C.ptr(x), C.ptr(x), rmax, nbin, nc, npn, 1, ctypes.byref(res),
                                ctypes.byref(o), None) == 1
    ra, dec, cz = np.full(5, 150.0), np.full(5, 10.0), np.full(5, 8000.0)
    o = C.get_config_options()
    res = C.ResultsVpf()
    f = str(tmp_path / "centres.txt").encode()
    assert lib.countspheres_mocks(5, C.ptr(ra), C.ptr(dec), C.ptr(cz), 5, C.ptr(ra), C.ptr(dec), C.ptr(cz), 1, 5.0, 5, 10,
                                  3, f, 3, ctypes.byref(res), ctypes.byref(o), None) == 1


def test_no_gpu_fails_loudly_not_silently(lib):
    """Without a usable GPU the library reports failure; it never falls back to the CPU."""
    import corrfunc_gb300
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    from corrfunc_gb300 import theory
    x = np.linspace(1.0, 9.0, 50)
    with pytest.raises(RuntimeError):
        theory.DD(1, 1, [0.5, 1.0, 2.0], x, x, x, boxsize=10.0)


COMPAT_PROGRAM = r"""
/* a program written against the reference's per-module headers and libraries */
#include <stdio.h>
#include <stdlib.h>
#include "countpairs.h"
#include "countpairs_rp_pi_mocks.h"
#include "io.h"

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    double *x = NULL, *y = NULL, *z = NULL;
    const int64_t n = read_positions(argv[1], "a", sizeof(double), 3, &x, &y, &z);
    if (n <= 0) return 3;
    struct config_options options = get_config_options();
    options.boxsize = 100.0;
    results_countpairs res;
    if (countpairs(n, x, y, z, n, x, y, z, 4, 1, argv[2], &res, &options, NULL) != EXIT_SUCCESS) return 1;
    for (int i = 1; i < res.nbin; i++) printf("%llu\n", (unsigned long long)res.npairs[i]);
    free_results(&res);
    free(x); free(y); free(z);
    return 0;
}
"""


def _build_compat(tmp_path):
    import shutil
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "prog.c"
    src.write_text(COMPAT_PROGRAM)
    exe = tmp_path / "prog"
    libdir = os.path.join(ROOT, "corrfunc_gb300")
    r = subprocess.run(["gcc", "-std=c99", str(src), "-o", str(exe), "-I", os.path.join(ROOT, "include", "compat"),
                        "-L" + libdir, "-lcountpairs", "-lcountpairs_rp_pi_mocks", "-lcorrfunc_gpu", "-Wl,-rpath," + libdir, "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def test_reference_header_and_library_names_build(tmp_path, lib):
    """-I include/compat and -l<module> (the reference's per-module header and library names) build a
    reference program unchanged; without a GPU it fails loudly with the library's message."""
    exe = _build_compat(tmp_path)
    pts = tmp_path / "pts.txt"
    rng = np.random.default_rng(1)
    np.savetxt(str(pts), rng.uniform(0, 100.0, (500, 3)))
    bins = tmp_path / "bins"
    bins.write_text("0.5 1.0\n1.0 5.0\n5.0 10.0\n")
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    r = subprocess.run([exe, str(pts), str(bins)], capture_output=True, text=True, timeout=300)
    if has_gpu:
        assert r.returncode == 0, r.stderr
        from corrfunc_gb300 import theory
        x, y, z = np.loadtxt(str(pts)).T
        want = theory.DD(1, 4, [0.5, 1.0, 5.0, 10.0], x, y, z, periodic=True, boxsize=100.0)
        assert [int(v) for v in r.stdout.split()] == list(want["npairs"])
    else:
        assert r.returncode == 1
        assert "no CUDA device" in r.stderr or "corrfunc_gb300" in r.stderr


def test_autotune_switch_needs_no_gpu():
    """The single-count autotuner's switch is host state: set, read back and cleared without a
    GPU."""
    import corrfunc_gb300
    lib = corrfunc_gb300.library()
    assert lib.cf_gpu_get_autotune() == 0
    assert lib.cf_gpu_set_autotune(1) == 0 and lib.cf_gpu_get_autotune() == 1
    assert lib.cf_gpu_set_autotune(0) == 0 and lib.cf_gpu_get_autotune() == 0

