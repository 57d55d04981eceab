#!/usr/bin/env python3
"""Build recipe for the *reference* Corrfunc 2.5.3 pair counters (test infrastructure only).

This compiles the reference's own C sources for the six pair-counting modules, the survey
counters (DDrppi_mocks, DDsmu_mocks), the counts-in-spheres modules (vpf, vpf_mocks) and its
particle-file readers (``io/io.c``) into per-module shared libraries under ``oracle/_ref/`` so
that the tests and the CPU baseline leg of ``bench.py`` can call the reference through its public
C API (``theory/DD/countpairs.h:28-35`` and siblings).  Nothing in the product links it.  The
survey and vpf sources include GSL headers; GSL is not installed here, so they are compiled
against the test-only stand-in in ``oracle/gsl_shim`` (linear interpolation and MT19937 restated
from their published descriptions).

The reference generates ``X_double.c`` / ``X_float.c`` from ``X.c.src`` by a sed
substitution of the token ``DOUBLE`` (``rules.mk:26-52``).  This recipe performs the same
substitution itself (it does not run the reference's own make system) and writes every
output -- the expanded sources, a verbatim staging copy of the few plain ``.c``/``.h`` files
the modules need, the object files and the ``.so`` files -- into ``oracle/_ref/`` only.
``oracle/_ref/`` is git-ignored, so none of it enters the history.

Two phases:

* ``stage``  (needs the reference tree; default ``/root/reference`` or ``$CORRFUNC_REF_DIR``):
  expand and copy the module sources into ``oracle/_ref/src``.
* ``compile`` (needs only ``oracle/_ref/src``): gcc -O3 -fopenmp each module into
  ``oracle/_ref/libcf_ref_<module>.so``.  This phase also runs on a machine that has the
  staged tree but not the reference checkout (the staged tree travels with the repo copy).

Usage:  python oracle/build_ref.py [stage|compile|all]   (default: all)
"""
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(REF_OUT, "src")
REF_DIR = os.environ.get("CORRFUNC_REF_DIR", "/root/reference")
VERSION = "2.5.3"

UTILS_PLAIN = ["utils.c", "progressbar.c", "cpu_features.c"]
IO_FILES = ["io.c", "io.h", "ftread.c", "ftread.h"]
UTILS_HEADERS = ["defs.h", "macros.h", "utils.h", "progressbar.h", "cpu_features.h",
                 "function_precision.h", "sglib.h", "avx512_calls.h", "avx2_calls.h",
                 "avx_calls.h", "sse_calls.h", "fast_acos.h", "set_cosmo_dist.h", "cosmology_params.h"]
# plain sources of the survey modules (cz -> comoving distance), compiled only into those
UTILS_COSMO = ["set_cosmo_dist.c", "cosmology_params.c"]
# test-only stand-in for the GSL headers the survey counters and theory vpf include (GSL is not
# installed here): oracle/gsl_shim/gsl/*.h
GSL_SHIM = os.path.join(HERE, "gsl_shim")
UTILS_SRC_TEMPLATES = ["gridlink_impl", "gridlink_utils", "gridlink_mocks_impl"]
UTILS_HDR_TEMPLATES = ["gridlink_impl", "gridlink_utils", "gridlink_mocks_impl", "cellarray",
                       "cellarray_mocks", "cell_pair", "weight_defs", "weight_functions"]

# module name -> (directory, public .c, impl template stem, kernel template stem, utils templates)
MODULES = {
    "DD": ("theory/DD", "countpairs.c", "countpairs_impl", "countpairs_kernels",
           ["gridlink_impl", "gridlink_utils"]),
    "DDrppi": ("theory/DDrppi", "countpairs_rp_pi.c", "countpairs_rp_pi_impl",
               "countpairs_rp_pi_kernels", ["gridlink_impl", "gridlink_utils"]),
    "DDsmu": ("theory/DDsmu", "countpairs_s_mu.c", "countpairs_s_mu_impl",
              "countpairs_s_mu_kernels", ["gridlink_impl", "gridlink_utils"]),
    "wp": ("theory/wp", "countpairs_wp.c", "countpairs_wp_impl", "wp_kernels",
           ["gridlink_impl", "gridlink_utils"]),
    "xi": ("theory/xi", "countpairs_xi.c", "countpairs_xi_impl", "xi_kernels",
           ["gridlink_impl", "gridlink_utils"]),
    "DDtheta": ("mocks/DDtheta_mocks", "countpairs_theta_mocks.c", "countpairs_theta_mocks_impl",
                "countpairs_theta_mocks_kernels", ["gridlink_mocks_impl", "gridlink_utils"]),
    # these include GSL headers: compiled against the test-only stand-in in oracle/gsl_shim
    "DDrppi_mocks": ("mocks/DDrppi_mocks", "countpairs_rp_pi_mocks.c", "countpairs_rp_pi_mocks_impl",
                     "countpairs_rp_pi_mocks_kernels", ["gridlink_mocks_impl", "gridlink_utils"]),
    "DDsmu_mocks": ("mocks/DDsmu_mocks", "countpairs_s_mu_mocks.c", "countpairs_s_mu_mocks_impl",
                    "countpairs_s_mu_mocks_kernels", ["gridlink_mocks_impl", "gridlink_utils"]),
    "vpf": ("theory/vpf", "countspheres.c", "countspheres_impl", "vpf_kernels", ["gridlink_impl", "gridlink_utils"]),
    "vpf_mocks": ("mocks/vpf_mocks", "countspheres_mocks.c", "countspheres_mocks_impl", "vpf_mocks_kernels",
                  ["gridlink_impl", "gridlink_utils"]),
}
# modules whose sources need the GSL stand-in and, for the survey ones, the cosmology sources
GSL_MODULES = {"DDrppi_mocks": True, "DDsmu_mocks": True, "vpf": False, "vpf_mocks": True}


def _expand(src, dst, prec):
    """Same token substitution as the reference's %_double.c / %_float.c rules."""
    with open(src) as f:
        lines = f.readlines()
    if prec == "double":
        head = ["#ifndef DOUBLE_PREC\n", "#define DOUBLE_PREC\n", "#endif\n"]
    else:
        head = ["#ifdef DOUBLE_PREC\n", "#undef DOUBLE_PREC\n", "#endif\n"]
    out = ["/* expanded from %s for the oracle build */\n" % os.path.basename(src)] + head
    for ln in lines:
        out.append(ln if "DOUBLE_PREC" in ln else ln.replace("DOUBLE", prec))
    with open(dst, "w") as f:
        f.writelines(out)


def stage():
    if not os.path.isdir(REF_DIR):
        print("build_ref: reference tree %s not present; skipping stage" % REF_DIR)
        return False
    if os.path.isdir(SRC_OUT):
        shutil.rmtree(SRC_OUT)
    udst = os.path.join(SRC_OUT, "utils")
    os.makedirs(udst)
    usrc = os.path.join(REF_DIR, "utils")
    for fn in UTILS_PLAIN + UTILS_HEADERS + UTILS_COSMO:
        shutil.copy(os.path.join(usrc, fn), udst)
    for stem in UTILS_SRC_TEMPLATES:
        for prec in ("double", "float"):
            _expand(os.path.join(usrc, stem + ".c.src"), os.path.join(udst, "%s_%s.c" % (stem, prec)), prec)
    for stem in UTILS_HDR_TEMPLATES:
        for prec in ("double", "float"):
            _expand(os.path.join(usrc, stem + ".h.src"), os.path.join(udst, "%s_%s.h" % (stem, prec)), prec)
    for name, (mdir, pub, impl, kern, _u) in MODULES.items():
        msrc = os.path.join(REF_DIR, mdir)
        mdst = os.path.join(SRC_OUT, name)
        os.makedirs(mdst)
        shutil.copy(os.path.join(msrc, pub), mdst)
        shutil.copy(os.path.join(msrc, pub[:-2] + ".h"), mdst)
        for prec in ("double", "float"):
            _expand(os.path.join(msrc, impl + ".c.src"), os.path.join(mdst, "%s_%s.c" % (impl, prec)), prec)
            _expand(os.path.join(msrc, impl + ".h.src"), os.path.join(mdst, "%s_%s.h" % (impl, prec)), prec)
            _expand(os.path.join(msrc, kern + ".c.src"), os.path.join(mdst, "%s_%s.c" % (kern, prec)), prec)
    # the reference's Python wrappers (Corrfunc/*.py, theory/*.py, mocks/*.py), unchanged, so
    # that tests can run them on this project's CPython extension modules
    pdst = os.path.join(SRC_OUT, "py", "Corrfunc")
    for sub in ("", "theory", "mocks"):
        d = os.path.join(REF_DIR, "Corrfunc", sub)
        os.makedirs(os.path.join(pdst, sub), exist_ok=True)
        for fn in sorted(os.listdir(d)):
            if fn.endswith(".py"):
                shutil.copy(os.path.join(d, fn), os.path.join(pdst, sub, fn))
    # the particle-file readers (io/io.c, io/ftread.c), for the reader tests
    idst = os.path.join(SRC_OUT, "io")
    os.makedirs(idst)
    for fn in IO_FILES:
        shutil.copy(os.path.join(REF_DIR, "io", fn), idst)
    print("build_ref: staged reference sources into %s" % SRC_OUT)
    return True


def _cflags():
    arch = platform.machine()
    flags = ["-std=c99", "-O3", "-fPIC", "-fopenmp", "-w",
             '-DVERSION="%s"' % VERSION, "-DUSE_OMP", "-D_POSIX_SOURCE=200809L", "-D_GNU_SOURCE",
             "-DENABLE_MIN_SEP_OPT", "-DCOPY_PARTICLES"]
    # The reference builds with -march=native; keep the host's fastest ISA (that is the
    # reference's own behaviour), aarch64 gcc spells it -mcpu=native.
    flags.append("-march=native" if arch in ("x86_64", "AMD64") else "-mcpu=native")
    return flags


def _compile_module(name):
    mdir, pub, impl, kern, utems = MODULES[name]
    mdst = os.path.join(SRC_OUT, name)
    udst = os.path.join(SRC_OUT, "utils")
    objdir = os.path.join(REF_OUT, "obj", name)
    os.makedirs(objdir, exist_ok=True)
    srcs = [os.path.join(mdst, pub)]
    srcs += [os.path.join(mdst, "%s_%s.c" % (impl, p)) for p in ("double", "float")]
    srcs += [os.path.join(udst, "%s_%s.c" % (u, p)) for u in utems for p in ("double", "float")]
    srcs += [os.path.join(udst, fn) for fn in UTILS_PLAIN]
    inc = ["-I" + mdst, "-I" + udst]
    if name in GSL_MODULES:
        inc.append("-I" + GSL_SHIM)
        if GSL_MODULES[name]:
            srcs += [os.path.join(udst, fn) for fn in UTILS_COSMO]
    objs = []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s)[:-2] + ".o")
        cmd = ["gcc"] + _cflags() + inc + ["-c", s, "-o", o]
        subprocess.check_call(cmd)
        objs.append(o)
    so = os.path.join(REF_OUT, "libcf_ref_%s.so" % name)
    subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", so] + objs + ["-lm"])
    return so


def _compile_io():
    idst = os.path.join(SRC_OUT, "io")
    udst = os.path.join(SRC_OUT, "utils")
    if not os.path.isdir(idst):
        return None
    objdir = os.path.join(REF_OUT, "obj", "io")
    os.makedirs(objdir, exist_ok=True)
    objs = []
    for s in [os.path.join(idst, "io.c"), os.path.join(idst, "ftread.c")] + [os.path.join(udst, fn) for fn in UTILS_PLAIN]:
        o = os.path.join(objdir, os.path.basename(s)[:-2] + ".o")
        subprocess.check_call(["gcc"] + _cflags() + ["-I" + idst, "-I" + udst, "-c", s, "-o", o])
        objs.append(o)
    so = os.path.join(REF_OUT, "libcf_ref_io.so")
    subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", so] + objs + ["-lm"])
    return so


def _compile_shim_check():
    """libcf_gslshim.so: the GSL stand-in's generator and interpolant, for their known-answer tests."""
    so = os.path.join(REF_OUT, "libcf_gslshim.so")
    subprocess.check_call(["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-I" + GSL_SHIM,
                           os.path.join(GSL_SHIM, "shim_check.c"), "-o", so, "-lm"])
    return so


def compile_all():
    if not os.path.isdir(SRC_OUT):
        print("build_ref: no staged sources in %s; reference libraries not built" % SRC_OUT)
        return []
    mods = [m for m in MODULES if os.path.isdir(os.path.join(SRC_OUT, m))]
    with ThreadPoolExecutor(max_workers=min(11, os.cpu_count() or 1)) as ex:
        sos = list(ex.map(_compile_module, mods))
        io = ex.submit(_compile_io).result()
        sos.append(ex.submit(_compile_shim_check).result())
    if io:
        sos.append(io)
    print("build_ref: built %d reference libraries" % len(sos))
    return sos


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("stage", "all"):
        stage()
    if what in ("compile", "all"):
        compile_all()
