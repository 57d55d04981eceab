"""Particle-file readers (read_positions / read_columns_into_array) and the command-line programs.

CPU: the readers against the reference's own io/io.c (built from its sources in oracle/_ref) on
fast-food files in both precisions and on ASCII / CSV files with comments and unparsable lines,
the .gz fallback, and the programs' argument errors.  GPU: every program's stdout table equals the
Python front end's results on the same files, and cf_gpu_read_positions_device feeds
cf_gpu_countpairs_device."""
import ctypes
import gzip
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "corrfunc_gb300", "bin")
REF_IO = os.path.join(ROOT, "oracle", "_ref", "libcf_ref_io.so")


def _read_fn(path):
    lib = ctypes.CDLL(path)
    f = lib.read_columns_into_array
    f.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    f.restype = ctypes.c_int64
    return f


def _read(fn, path, fmt, size, nf):
    ptrs = (ctypes.c_void_p * nf)()
    n = fn(path.encode(), fmt.encode(), size, nf, ptrs)
    if n < 0:
        return None
    ct = ctypes.c_float if size == 4 else ctypes.c_double
    dt = np.float32 if size == 4 else np.float64
    out = [np.ctypeslib.as_array(ctypes.cast(ptrs[k], ctypes.POINTER(ct)), shape=(n,)).astype(dt, copy=True)
           if n > 0 else np.zeros(0, dt) for k in range(nf)]
    libc = ctypes.CDLL(None)
    for k in range(nf):
        libc.free(ctypes.c_void_p(ptrs[k]))
    return out


def write_fastfood(path, cols, dtype):
    """Fast-food file: records (5 ints), (9 floats), (1 float), then one record per column."""
    def rec(arr):
        b = np.ascontiguousarray(arr).tobytes()
        return np.uint32(len(b)).tobytes() + b + np.uint32(len(b)).tobytes()
    n = len(cols[0])
    with open(path, "wb") as f:
        f.write(rec(np.array([0, n, 0, 0, 0], dtype=np.int32)))
        f.write(rec(np.zeros(9, dtype=np.float32)))
        f.write(rec(np.zeros(1, dtype=np.float32)))
        for c in cols:
            f.write(rec(np.asarray(c, dtype=dtype)))


def write_ascii(path, cols, sep=" ", junk=True):
    rows = np.stack(cols, 1)
    with open(path, "w") as f:
        for i, r in enumerate(rows):
            f.write(sep.join("%.17g" % v for v in r) + "\n")
            if junk and i == 3:
                f.write("not a number here\n")


@pytest.fixture(scope="module")
def ours():
    from corrfunc_gb300 import _capi as C
    if not os.path.exists(C.LIB_PATH):
        from corrfunc_gb300 import build
        build.build()
    return _read_fn(C.LIB_PATH)


@pytest.mark.parametrize("fmt,fdtype", [("f", np.float64), ("f", np.float32), ("a", None), ("c", None)])
@pytest.mark.parametrize("size", [4, 8])
def test_readers_match_the_reference(ours, tmp_path, fmt, fdtype, size):
    rng = np.random.default_rng(3)
    cols = [rng.uniform(-50, 500, 1234) for _ in range(3)]
    path = str(tmp_path / "pts.dat")
    if fmt == "f":
        write_fastfood(path, cols, fdtype)
    else:
        write_ascii(path, cols, sep="," if fmt == "c" else "\t ")
    got = _read(ours, path, fmt, size, 3)
    assert got is not None and len(got[0]) == 1234
    src = [np.asarray(c, dtype=fdtype) if fdtype is not None else np.asarray(c) for c in cols]
    for g, c in zip(got, src):
        assert np.array_equal(g, c.astype(np.float32 if size == 4 else np.float64))
    if os.path.exists(REF_IO):
        want = _read(_read_fn(REF_IO), path, fmt, size, 3)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)


def test_reader_gz_fallback_and_errors(ours, tmp_path):
    cols = [np.arange(10.0), np.arange(10.0) * 2, np.arange(10.0) * 3]
    plain = tmp_path / "g.txt"
    write_ascii(str(plain), cols, junk=False)
    with open(str(plain), "rb") as f, gzip.open(str(plain) + ".gz", "wb") as g:
        g.write(f.read())
    os.remove(str(plain))
    got = _read(ours, str(plain), "a", 8, 3)
    assert got is not None and np.array_equal(got[2], cols[2])
    assert os.path.exists(str(plain))
    assert _read(ours, str(tmp_path / "missing.txt"), "a", 8, 3) is None
    assert _read(ours, str(plain), "x", 8, 3) is None
    assert _read(ours, str(plain), "a", 2, 3) is None


def _run(cmd, args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([os.path.join(BIN, cmd)] + [str(a) for a in args], capture_output=True, text=True, env=e,
                          timeout=600)


def _have_cli():
    if not os.path.exists(os.path.join(BIN, "DD")):
        pytest.skip("command-line programs not built")


def test_cli_argument_errors(tmp_path):
    _have_cli()
    assert _run("DD", ["a", "b"]).returncode == 1
    assert "Missing required parameters" in _run("DD", ["a", "b"]).stderr
    r = _run("DD", ["f1", "a", "f1", "a", "bins", "100", "1", "pair_product"])
    assert r.returncode == 1 and "optional arguments" in r.stderr
    r = _run("DDrppi_mocks", ["f1", "a", "f1", "a", "bins", "40", "1", "0"])
    assert r.returncode == 1 and "Nthreads must be at least 1" in r.stderr
    assert _run("vpf", ["1"]).returncode == 1
    r = subprocess.run([os.path.join(BIN, "corrfunc_gb300_cli")], capture_output=True, text=True)
    assert r.returncode == 1


# ------------------------------------------------------------------------------ GPU

def _bins(tmp_path, edges, name="bins"):
    p = tmp_path / name
    with open(str(p), "w") as f:
        for lo, hi in zip(edges[:-1], edges[1:]):
            f.write("%.17g %.17g\n" % (lo, hi))
    return str(p)


def _table(out):
    return np.array([[float(v) for v in ln.split()] for ln in out.strip().splitlines()])


@pytest.mark.gpu
def test_cli_theory_programs_match_the_front_end(tmp_path):
    _have_cli()
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    L = 150.0
    x, y, z = cat.clustered_box(20000, L, 4)
    w = cat.weights(20000, 5)
    f = str(tmp_path / "pts.txt")
    write_ascii(f, [x, y, z], junk=False)
    fw = str(tmp_path / "w.txt")
    write_ascii(fw, [w], junk=False)
    ff = str(tmp_path / "pts.ff")
    write_fastfood(ff, [x, y, z], np.float64)
    bins = cat.log_bins(0.5, 12.0, 8)
    bf = _bins(tmp_path, bins)
    x4, y4, z4 = (a.astype(np.float32) for a in (x, y, z))
    # DD, default build: single precision inputs, periodic, weights from a file
    r = _run("DD", [f, "a", f, "a", bf, L, 4, "pair_product", fw, "a"])
    assert r.returncode == 0, r.stderr
    t = _table(r.stdout)
    want = theory.DD(1, 4, bins, x4, y4, z4, weights1=w.astype(np.float32), weight_type="pair_product", periodic=True,
                     boxsize=L)
    assert [int(v) for v in t[:, 3]] == list(want["npairs"])
    np.testing.assert_allclose(t[:, 4], want["weightavg"], rtol=1e-5)
    # double precision inputs from a fast-food file
    r = _run("DD", [ff, "f", ff, "f", bf, L, 4], env={"CF_CLI_DOUBLE": "1"})
    t = _table(r.stdout)
    want = theory.DD(1, 4, bins, x, y, z, periodic=True, boxsize=L)
    assert [int(v) for v in t[:, 3]] == list(want["npairs"])
    # DDrppi, DDsmu, wp, xi
    r = _run("DDrppi", [f, "a", f, "a", bf, 20, L, 2])
    want = theory.DDrppi(1, 2, 20.0, bins, x4, y4, z4, periodic=True, boxsize=L)
    assert [int(v) for v in _table(r.stdout)[:, 3]] == list(want["npairs"])
    r = _run("DDsmu", [f, "a", f, "a", bf, 1.0, 5, L, 2])
    want = theory.DDsmu(1, 2, bins, 1.0, 5, x4, y4, z4, periodic=True, boxsize=L)
    assert [int(v) for v in _table(r.stdout)[:, 3]] == list(want["npairs"])
    r = _run("wp", [L, f, "a", bf, 20, 2])
    t = _table(r.stdout)
    want = theory.wp(L, 20.0, 2, bins, x4, y4, z4)
    assert [int(v) for v in t[:, 3]] == list(want["npairs"])
    np.testing.assert_allclose(t[:, 4], want["wp"], rtol=1e-5, atol=1e-6)
    r = _run("xi", [L, f, "a", bf, 2])
    t = _table(r.stdout)
    want = theory.xi(L, 2, bins, x4, y4, z4)
    assert [int(v) for v in t[:, 3]] == list(want["npairs"])
    # vpf (default refine factors 2, 2, 1 of get_config_options)
    r = _run("vpf", [6.0, 6, 2000, 4, f, "a", 77, L])
    assert r.returncode == 0, r.stderr
    t = _table(r.stdout)
    want = theory.vpf(6.0, 6, 2000, 4, 77, x4, y4, z4, periodic=True, boxsize=L, xbin_refine_factor=2,
                      ybin_refine_factor=2, zbin_refine_factor=1)
    np.testing.assert_allclose(t[:, 1:], want["pN"], rtol=1e-3, atol=1e-9)


@pytest.mark.gpu
def test_cli_mocks_programs_match_the_front_end(tmp_path):
    _have_cli()
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks
    ra, dec, cz = cat.survey(8000, 8)
    f = str(tmp_path / "gal.ff")
    write_fastfood(f, [ra, dec, cz], np.float64)
    bins = cat.log_bins(0.5, 10.0, 6)
    bf = _bins(tmp_path, bins)
    r = _run("DDrppi_mocks", [f, "f", f, "f", bf, 10, 1, 2])
    assert r.returncode == 0, r.stderr
    t = _table(r.stdout)
    want = mocks.DDrppi_mocks(1, 1, 2, 10.0, bins, ra.copy(), dec.copy(), cz.copy(), output_rpavg=True)
    assert [int(v) for v in t[:, 0]] == list(want["npairs"])
    np.testing.assert_allclose(t[:, 1], want["rpavg"], rtol=0, atol=2e-8)
    r = _run("DDsmu_mocks", [f, "f", f, "f", bf, 1.0, 4, 2, 2])
    want = mocks.DDsmu_mocks(1, 2, 2, 1.0, 4, bins, ra.copy(), dec.copy(), cz.copy(), output_savg=True)
    assert [int(v) for v in _table(r.stdout)[:, 0]] == list(want["npairs"])
    tf = str(tmp_path / "sky.ff")
    write_fastfood(tf, [ra, dec], np.float64)
    tb = _bins(tmp_path, cat.log_bins(0.05, 3.0, 6), "tbins")
    r = _run("DDtheta_mocks", [tf, "f", tf, "f", tb, 2])
    t = _table(r.stdout)
    want = mocks.DDtheta_mocks(1, 2, cat.log_bins(0.05, 3.0, 6), ra.copy(), dec.copy(), output_thetaavg=True)
    assert [int(v) for v in t[:, 3]] == list(want["npairs"])
    # vpf_mocks: randoms with the volume-based threshold, centres written to the file
    rra, rdec, rcz = cat.survey(20000, 9, frac_clustered=0.0)
    rf = str(tmp_path / "ran.ff")
    write_fastfood(rf, [rra, rdec, rcz], np.float64)
    cen = str(tmp_path / "centres.txt")
    r = _run("vpf_mocks", [4.0, 4, 500, 3, 1.0e7, f, "f", rf, "f", cen, 1])
    assert r.returncode == 0, r.stderr
    assert os.path.exists(cen)
    t = _table(r.stdout)
    assert t.shape == (4, 4)


@pytest.mark.gpu
def test_read_positions_device_feeds_countpairs_device(tmp_path):
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    lib = C.bind(C.LIB_PATH, gpu=True)
    L = 100.0
    x, y, z = cat.uniform_box(30000, L, 12)
    ff = str(tmp_path / "p.ff")
    write_fastfood(ff, [x, y, z], np.float64)
    f = lib.cf_gpu_read_positions_device
    f.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    f.restype = ctypes.c_int64
    dev = (ctypes.c_void_p * 3)()
    n = f(ff.encode(), b"f", 8, 3, dev)
    assert n == 30000
    lib.cf_gpu_countpairs_device.argtypes = lib.countpairs.argtypes
    lib.cf_gpu_countpairs_device.restype = ctypes.c_int
    o = C.get_config_options()
    o.boxsize_x = o.boxsize_y = o.boxsize_z = L
    e = C.get_extra_options()
    res = C.ResultsDD()
    bins = cat.log_bins(0.5, 8.0, 6)
    with C.BinFile(bins) as bf:
        rc = lib.cf_gpu_countpairs_device(n, dev[0], dev[1], dev[2], n, dev[0], dev[1], dev[2], 1, 1, bf.encode(),
                                          ctypes.byref(res), ctypes.byref(o), ctypes.byref(e))
    assert rc == 0
    got = [res.npairs[i] for i in range(1, res.nbin)]
    lib.free_results(ctypes.byref(res))
    lib.cf_gpu_free_device.argtypes = [ctypes.c_void_p]
    for k in range(3):
        lib.cf_gpu_free_device(dev[k])
    want = theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=L)
    assert got == list(want["npairs"])
