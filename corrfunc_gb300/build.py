"""In-tree build of libcorrfunc_gb300.so (C host layer + sm_103a CUDA engine).

    python -m corrfunc_gb300.build          # or corrfunc_gb300.build.build()

The host C files are compiled with gcc (-ffp-contract=off keeps the double-precision
finalisation free of contractions), the CUDA engine with nvcc for sm_103a only, and both are
linked into corrfunc_gb300/libcorrfunc_gb300.so.  Translation units compile in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcorrfunc_gb300.so")
WORKUNIT_LIB = os.path.join(HERE, "libcf_workunit.so")
HOST_SOURCES = ("cf_api.c", "cf_common.c", "cf_io.c", "cf_workunit.c")

NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build corrfunc_gb300")
    return cand


def _cuda_root(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build(verbose=False, extra_nvcc=()):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cuda = _cuda_root(nvcc)
    inc = ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    jobs = []
    for c in HOST_SOURCES:
        obj = os.path.join(BUILD, c[:-2] + ".o")
        jobs.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wno-unused-function"]
                    + inc + ["-c", os.path.join(CSRC, c), "-o", obj])
    cu_objs = []
    for cu in ("cf_engine.cu", "cf_noalloc.cu"):
        obj = os.path.join(BUILD, cu[:-3] + ".o")
        cu_objs.append(obj)
        jobs.append([nvcc] + NVCC_ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                          "-Xcompiler", "-ffp-contract=off"] + list(extra_nvcc) + inc
                    + ["-c", os.path.join(CSRC, cu), "-o", obj])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
    objs = [os.path.join(BUILD, c[:-2] + ".o") for c in HOST_SOURCES] + cu_objs
    tmp = LIB + ".tmp"
    _run([nvcc] + NVCC_ARCH + ["-shared", "-o", tmp] + objs
         + ["-L" + os.path.join(cuda, "lib64"), "-lcudart_static", "-lpthread", "-ldl", "-lrt", "-lm", "-Xcompiler", "-fopenmp"])
    os.replace(tmp, LIB)
    # the work unit alone, without the CUDA engine (CPU-only measurements load this one)
    tmp = WORKUNIT_LIB + ".tmp"
    _run(["gcc", "-shared", "-o", tmp, os.path.join(BUILD, "cf_workunit.o"), os.path.join(BUILD, "cf_common.o"), "-lm"])
    os.replace(tmp, WORKUNIT_LIB)
    link_module_names()
    build_python_modules(verbose)
    build_cli()
    return LIB


# the reference's per-module library names (theory/*/Makefile, mocks/*/Makefile: LIBNAME)
# per-module library names of the reference's makefiles, and the generic GPU link name
MODULE_LIBS = ("countpairs", "countpairs_rp_pi", "countpairs_s_mu", "countpairs_wp", "countpairs_xi", "countspheres",
               "countpairs_theta_mocks", "countpairs_rp_pi_mocks", "countpairs_s_mu_mocks", "countspheres_mocks",
               "corrfunc_gpu")


def link_module_names():
    """lib<module>.so links to libcorrfunc_gb300.so, so that -l<module> link lines of programs built
    against the reference's per-module libraries resolve to this library."""
    for name in MODULE_LIBS:
        link = os.path.join(HERE, "lib%s.so" % name)
        if os.path.lexists(link):
            os.remove(link)
        os.symlink(os.path.basename(LIB), link)


CLI_COMMANDS = ("DD", "DDrppi", "DDsmu", "wp", "xi", "vpf", "DDtheta_mocks", "DDrppi_mocks", "DDsmu_mocks", "vpf_mocks")


def build_cli():
    """The reference's command-line programs as one binary (csrc/cf_cli.c) in bin/, linked against
    libcorrfunc_gb300.so, with one link per command name."""
    bindir = os.path.join(HERE, "bin")
    os.makedirs(bindir, exist_ok=True)
    exe = os.path.join(bindir, "corrfunc_gb300_cli")
    _run(["gcc", "-std=gnu11", "-O2", "-Wall", "-Wno-unused-function", "-I" + INCLUDE, os.path.join(CSRC, "cf_cli.c"),
          "-o", exe + ".tmp", "-L" + HERE, "-lcorrfunc_gb300", "-lm", "-Wl,-rpath,$ORIGIN/.."])
    os.replace(exe + ".tmp", exe)
    for name in CLI_COMMANDS:
        link = os.path.join(bindir, name)
        if os.path.lexists(link):
            os.remove(link)
        os.symlink("corrfunc_gb300_cli", link)
    return exe


def python_module_paths():
    import sysconfig
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return [os.path.join(HERE, name + suffix) for name in ("_countpairs", "_countpairs_mocks")]


def build_python_modules(verbose=False):
    """CPython extension modules _countpairs / _countpairs_mocks (csrc/cf_pymodule.c), linked
    against libcorrfunc_gb300.so in this directory.  Skipped with a note when the Python or numpy
    headers are missing."""
    import sysconfig
    pyinc = sysconfig.get_paths().get("include", "")
    try:
        import numpy
        npinc = numpy.get_include()
    except Exception:
        npinc = ""
    if not (os.path.exists(os.path.join(pyinc, "Python.h")) and
            os.path.exists(os.path.join(npinc, "numpy", "arrayobject.h"))):
        print("corrfunc_gb300: Python or numpy headers not found; _countpairs modules not built")
        return []
    src = os.path.join(CSRC, "cf_pymodule.c")
    obj = os.path.join(BUILD, "cf_pymodule.o")
    _run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-Wall", "-Wno-unused-function", "-Wno-missing-field-initializers",
          "-I" + INCLUDE, "-I" + pyinc, "-I" + npinc, "-c", src, "-o", obj])
    out = []
    for path in python_module_paths():
        tmp = path + ".tmp"
        _run(["gcc", "-shared", "-o", tmp, obj, "-L" + HERE, "-lcorrfunc_gb300", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, path)
        out.append(path)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
