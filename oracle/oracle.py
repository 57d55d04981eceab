"""ORACLE (test infrastructure only): CPU restatement of Corrfunc 2.5.3's six pair counters.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module, and
only as the checker.  The pair loop is the brute-force C restatement in cf_oracle.c (exact
double-precision per-pair arithmetic of the reference kernels); this file restates the
surrounding driver logic:

  * bin files: utils/utils.c:62-106 (nbin = lines + 1, rupp[0] = first low edge);
  * the reference lattice that decides which point of a wrapped auto pair is shifted:
    utils/gridlink_utils.c.src:31-49 (get_binsize), theory/DD/countpairs_impl.c.src:231-332
    (wrap values, default refine rule, boost), theory/xi/countpairs_xi_impl.c.src:211-262 and
    theory/wp/countpairs_wp_impl.c.src:236-290 (box lattice for xi / wp);
  * finalisation: x2 for auto-correlations and self pairs (theory/DD/countpairs_impl.c.src:609-664,
    with the weight of self pairs added to flat bin 1 in every module, e.g.
    theory/DDrppi/countpairs_rp_pi_impl.c.src:618-642), averages, xi and wp from the analytic
    random counts (theory/xi/countpairs_xi_impl.c.src:581-626, theory/wp/countpairs_wp_impl.c.src:615-660);
  * angular inputs: unit vectors from RA/DEC with libm
    (mocks/DDtheta_mocks/countpairs_theta_mocks_impl.c.src:569-608);
  * survey inputs of DDrppi_mocks / DDsmu_mocks: the in-place RA/DEC/cz fix-ups
    (mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:43-112), cosmology 1 / 2
    (utils/cosmology_params.c:28-55) and the comoving positions (cfo_mock_xyz in cf_oracle.c).

Results are returned in the same structured-array layout as corrfunc_gb300.theory / .mocks.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "liboracle.so")

R3, RPPI, WP, SMU, THETA, RPPI_MOCK, SMU_MOCK = 0, 1, 2, 3, 4, 5, 6
SPEED_OF_LIGHT = 299800.0
OMEGA_M = {1: 0.25, 2: 0.302}
PI_OVER_180 = 0.017453292519943295769236907684886127134428718885417254560971


class _Params(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("autocorr", ctypes.c_int32), ("fma_formula", ctypes.c_int32),
                ("chord_formula", ctypes.c_int32), ("periodic", ctypes.c_int32 * 3), ("nmesh", ctypes.c_int32 * 3),
                ("wrap", ctypes.c_double * 3), ("lat_min", ctypes.c_double * 3), ("lat_inv", ctypes.c_double * 3),
                ("nedges", ctypes.c_int32), ("npibin", ctypes.c_int32), ("pimax", ctypes.c_double),
                ("edges", ctypes.POINTER(ctypes.c_double)), ("need_avg", ctypes.c_int32),
                ("need_weight", ctypes.c_int32), ("fast_acos", ctypes.c_int32), ("pad", ctypes.c_int32)]


def build(force=False):
    src = os.path.join(HERE, "cf_oracle.c")
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               src, "-o", SO, "-lm"])
    return SO


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        build()
        _LIB = ctypes.CDLL(SO)
        _LIB.cfo_count.restype = ctypes.c_int
    return _LIB


def read_bins(binfile):
    """utils/utils.c:62-106 restated."""
    if not isinstance(binfile, (str, bytes, os.PathLike)):
        e = sorted(float(v) for v in binfile)
        lines = ["{0} {1}".format(e[i], e[i + 1]) for i in range(len(e) - 1)]
    else:
        with open(binfile) as f:
            lines = f.read().splitlines()
    data = [ln for ln in lines if ln.strip() and not ln.strip().startswith("#")]
    nbin = len(data) + 1
    rupp = [0.0] * (nbin + 1)
    idx = 1
    for ln in lines:
        parts = ln.split()
        try:
            lo, hi = float(parts[0]), float(parts[1])
        except (IndexError, ValueError):
            continue
        if idx == 1:
            rupp[0] = lo
        rupp[idx] = hi
        idx += 1
    rmax = rupp[idx - 1]
    rupp[nbin] = rmax
    rupp[nbin - 1] = rmax
    return np.array(rupp[:nbin], dtype=np.float64)


def _binsize(xdiff, xwrap, rmax, refine, max_cells):
    n = int(refine * xdiff / rmax)
    n = max(n, 1)
    if xwrap > 0 and rmax >= xwrap / 2:
        raise RuntimeError("rmax must be less than half of the periodic box")
    n = min(n, max_cells)
    n = max(n, 2)
    return xdiff / n, n


def reference_lattice(kind, lo, hi, boxsize, periodic, max_size, refine, custom, max_cells, np1, dfl):
    """(lat_min, lat_inv, nmesh, wrap, periodic_axes) of the reference lattice."""
    refine = list(refine)
    if kind == "box":
        lo = [0.0] * 3
        hi = [boxsize[0]] * 3
        wrap = [boxsize[0]] * 3
        per = [1, 1, 1]
    else:
        per = [1 if (periodic and boxsize[a] >= 0) else 0 for a in range(3)]
        wrap = [(boxsize[a] if boxsize[a] > 0 else hi[a] - lo[a]) if per[a] else 0.0 for a in range(3)]
    if not custom:
        if dfl == "per_axis":
            for a in range(3):
                if max_size[a] < 0.05 * wrap[a]:
                    refine[a] = 1
        elif dfl == "xi":
            if max_size[0] < 0.05 * boxsize[0]:
                refine = [1, 1, 1]
        elif dfl == "wp":
            if max_size[0] < 0.05 * boxsize[0]:
                refine[0] = refine[1] = 1
            if max_size[2] < 0.05 * boxsize[0]:
                refine[2] = 1

    def grid(ref):
        out = [_binsize(hi[a] - lo[a], wrap[a], max_size[a], ref[a], max_cells) for a in range(3)]
        return [o[0] for o in out], [o[1] for o in out]

    bs, nm = grid(refine)
    if dfl != "none":
        avg_np = float(np1) / (nm[0] * nm[1] * nm[2])
        mx = max(nm)
        if (mx <= 10 or avg_np >= 250) and mx < max_cells and not custom:
            refine[0] += 1
            refine[1] += 1
            bs, nm = grid(refine)
    inv = [1.0 / b if b > 0 else 0.0 for b in bs]
    return lo, inv, nm, wrap, per


def _count(mode, autocorr, pos1, w1, pos2, w2, edges, lattice, fma, chord, npibin=0, pimax=0.0,
           need_avg=True, need_w=False, nthreads=0):
    lib = _lib()
    p = _Params()
    p.mode, p.autocorr, p.fma_formula, p.chord_formula = mode, int(autocorr), int(fma), int(chord)
    lat_min, lat_inv, nmesh, wrap, per = lattice
    for a in range(3):
        p.periodic[a] = int(per[a])
        p.nmesh[a] = int(nmesh[a])
        p.wrap[a] = float(wrap[a])
        p.lat_min[a] = float(lat_min[a])
        p.lat_inv[a] = float(lat_inv[a])
    e = np.ascontiguousarray(edges, dtype=np.float64)
    p.nedges = len(e)
    p.edges = e.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    p.npibin = int(npibin)
    p.pimax = float(pimax)
    p.need_avg = int(bool(need_avg))
    p.need_weight = int(bool(need_w))
    nb = len(e) * (npibin + 1) if mode in (RPPI, SMU, RPPI_MOCK, SMU_MOCK) else len(e)
    npairs = np.zeros(nb, dtype=np.uint64)
    avg = np.zeros(nb)
    ws = np.zeros(nb)
    x1, y1, z1 = (np.ascontiguousarray(a, dtype=np.float64) for a in pos1)
    if autocorr:
        x2, y2, z2 = x1, y1, z1
        w2 = w1
    else:
        x2, y2, z2 = (np.ascontiguousarray(a, dtype=np.float64) for a in pos2)
    w1 = None if w1 is None else np.ascontiguousarray(w1, dtype=np.float64)
    w2 = None if w2 is None else np.ascontiguousarray(w2, dtype=np.float64)

    def P(a):
        return None if a is None else a.ctypes.data_as(ctypes.c_void_p)

    lib.cfo_count(ctypes.byref(p), ctypes.c_int64(len(x1)), P(x1), P(y1), P(z1), P(w1),
                  ctypes.c_int64(len(x2)), P(x2), P(y2), P(z2), P(w2),
                  npairs.ctypes.data_as(ctypes.c_void_p), avg.ctypes.data_as(ctypes.c_void_p),
                  ws.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(nthreads))
    return npairs, avg, ws


def _finalize(npairs, avg, ws, autocorr, first_zero, self_idx, n1, self_w, need_avg, need_w, div_start=0):
    npairs = npairs.copy()
    avg = avg.copy()
    ws = ws.copy()
    if autocorr:
        npairs *= 2
        avg *= 2.0
        ws *= 2.0
        if first_zero:
            npairs[self_idx] += n1
            if need_w:
                ws[1] += self_w
    for i in range(div_start, len(npairs)):
        if npairs[i] > 0:
            if need_avg:
                avg[i] /= float(npairs[i])
            if need_w:
                ws[i] /= float(npairs[i])
    if not need_avg:
        avg[:] = 0.0
    if not need_w:
        ws[:] = 0.0
    return npairs, avg, ws


def _formula(isa):
    """fused-multiply-add chain for AVX512F, chord form for the SIMD angular kernels."""
    up = isa.upper() if isinstance(isa, str) else isa
    return (up == "AVX512F"), (up in ("AVX512F", "AVX2", "AVX", "SSE42"))


def _weights(w, n):
    if w is None:
        return None
    w = np.atleast_2d(np.asarray(w, dtype=np.float64))
    return np.ascontiguousarray(w[0])


def _extent(*arrs):
    lo = [min(float(np.min(a[k])) for a in arrs) for k in range(3)]
    hi = [max(float(np.max(a[k])) for a in arrs) for k in range(3)]
    return lo, hi


def _box3(boxsize):
    if boxsize is None:
        return (-2.0, -2.0, -2.0)
    b = np.atleast_1d(boxsize).astype(float)
    return (b[0], b[0], b[0]) if len(b) == 1 else tuple(b)


def DD(autocorr, binfile, X1, Y1, Z1, weights1=None, periodic=True, boxsize=None, X2=None, Y2=None, Z2=None,
       weights2=None, output_ravg=False, refine=(2, 2, 1), custom_refine=False, max_cells_per_dim=100,
       isa="fallback", weight_type=None, nthreads=0):
    from corrfunc_gb300.theory import DD_DTYPE
    rupp = read_bins(binfile)
    rmax = rupp[-1]
    pos1 = (X1, Y1, Z1)
    pos2 = pos1 if autocorr else (X2, Y2, Z2)
    lo, hi = _extent(pos1) if autocorr else _extent(pos1, pos2)
    lat = reference_lattice("extent", lo, hi, _box3(boxsize), periodic, (rmax, rmax, rmax), refine, custom_refine,
                            max_cells_per_dim, len(X1), "per_axis")
    need_w = weight_type is not None
    w1 = _weights(weights1, len(X1)) if need_w else None
    w2 = (w1 if autocorr else _weights(weights2, len(X2))) if need_w else None
    if need_w and not autocorr:
        if w1 is None:
            w1 = np.ones(len(X1))
        if w2 is None:
            w2 = np.ones(len(X2))
    fma, chord = _formula(isa)
    c, a, w = _count(R3, autocorr, pos1, w1, pos2, w2, rupp * rupp, lat, fma, chord, need_avg=output_ravg,
                     need_w=need_w, nthreads=nthreads)
    self_w = float(np.sum(w1 * w1)) if (autocorr and need_w and rupp[0] <= 0) else 0.0
    c, a, w = _finalize(c, a, w, autocorr, rupp[0] <= 0, 1, len(X1), self_w, output_ravg, need_w)
    out = np.zeros(len(rupp) - 1, dtype=DD_DTYPE)
    out["rmin"], out["rmax"] = rupp[:-1], rupp[1:]
    out["ravg"], out["npairs"], out["weightavg"] = a[1:], c[1:], w[1:]
    return out


def _twod(mode, autocorr, binfile, zsize, npibin, pimax_or_mu, X1, Y1, Z1, weights1, periodic, boxsize, X2, Y2,
          Z2, weights2, output_avg, refine, custom_refine, max_cells, isa, weight_type, dfl, nthreads):
    rupp = read_bins(binfile)
    rmax = rupp[-1]
    pos1 = (X1, Y1, Z1)
    pos2 = pos1 if autocorr else (X2, Y2, Z2)
    lo, hi = _extent(pos1) if autocorr else _extent(pos1, pos2)
    lat = reference_lattice("extent", lo, hi, _box3(boxsize), periodic, (rmax, rmax, zsize), refine, custom_refine,
                            max_cells, len(X1), dfl)
    need_w = weight_type is not None
    w1 = _weights(weights1, len(X1)) if need_w else None
    w2 = (w1 if autocorr else _weights(weights2, len(X2))) if need_w else None
    if need_w and not autocorr:
        w1 = np.ones(len(X1)) if w1 is None else w1
        w2 = np.ones(len(X2)) if w2 is None else w2
    fma, chord = _formula(isa)
    c, a, w = _count(mode, autocorr, pos1, w1, pos2, w2, rupp * rupp, lat, fma, chord, npibin=npibin,
                     pimax=pimax_or_mu, need_avg=output_avg, need_w=need_w, nthreads=nthreads)
    self_w = float(np.sum(w1 * w1)) if (autocorr and need_w and rupp[0] <= 0) else 0.0
    c, a, w = _finalize(c, a, w, autocorr, rupp[0] <= 0, npibin + 1, len(X1), self_w, output_avg, need_w)
    return rupp, c, a, w


def DDrppi(autocorr, pimax, binfile, X1, Y1, Z1, weights1=None, periodic=True, boxsize=None, X2=None, Y2=None,
           Z2=None, weights2=None, output_rpavg=False, refine=(2, 2, 1), custom_refine=False, max_cells_per_dim=100,
           isa="fallback", weight_type=None, nthreads=0):
    from corrfunc_gb300.theory import DDRPPI_DTYPE
    npibin = int(pimax)
    rupp, c, a, w = _twod(RPPI, autocorr, binfile, pimax, npibin, pimax, X1, Y1, Z1, weights1, periodic, boxsize,
                          X2, Y2, Z2, weights2, output_rpavg, refine, custom_refine, max_cells_per_dim, isa,
                          weight_type, "per_axis", nthreads)
    dpi = pimax / npibin
    rows = []
    for i in range(1, len(rupp)):
        for j in range(npibin):
            k = i * (npibin + 1) + j
            rows.append((rupp[i - 1], rupp[i], a[k], (j + 1) * dpi, c[k], w[k]))
    return np.array(rows, dtype=DDRPPI_DTYPE)


def DDsmu(autocorr, binfile, mu_max, nmu_bins, X1, Y1, Z1, weights1=None, periodic=True, boxsize=None, X2=None,
          Y2=None, Z2=None, weights2=None, output_savg=False, refine=(2, 2, 1), custom_refine=False,
          max_cells_per_dim=100, isa="fallback", weight_type=None, nthreads=0):
    from corrfunc_gb300.theory import DDSMU_DTYPE
    rupp0 = read_bins(binfile)
    smax = rupp0[-1]
    rupp, c, a, w = _twod(SMU, autocorr, binfile, smax * mu_max, nmu_bins, mu_max, X1, Y1, Z1, weights1, periodic,
                          boxsize, X2, Y2, Z2, weights2, output_savg, refine, custom_refine, max_cells_per_dim, isa,
                          weight_type, "none", nthreads)
    dmu = mu_max / nmu_bins
    rows = []
    for i in range(1, len(rupp)):
        for j in range(nmu_bins):
            k = i * (nmu_bins + 1) + j
            rows.append((rupp[i - 1], rupp[i], a[k], (j + 1) * dmu, c[k], w[k]))
    return np.array(rows, dtype=DDSMU_DTYPE)


def _box_counts(mode, boxsize, binfile, zsize, pimax, X, Y, Z, weights, output_avg, refine, custom_refine,
                max_cells, isa, weight_type, dfl, nthreads):
    rupp = read_bins(binfile)
    rmax = rupp[-1]
    L = float(np.atleast_1d(boxsize)[0])
    lat = reference_lattice("box", None, None, (L, L, L), True, (rmax, rmax, zsize), refine, custom_refine,
                            max_cells, len(X), dfl)
    need_w = weight_type is not None
    w1 = _weights(weights, len(X)) if need_w else None
    fma, chord = _formula(isa)
    c, a, w = _count(mode, True, (X, Y, Z), w1, None, None, rupp * rupp, lat, fma, chord, npibin=1, pimax=pimax,
                     need_avg=output_avg, need_w=need_w, nthreads=nthreads)
    self_w = float(np.sum(w1 * w1)) if (need_w and rupp[0] <= 0) else 0.0
    c, a, w = _finalize(c, a, w, True, rupp[0] <= 0, 1, len(X), self_w, output_avg, need_w)
    N = len(X)
    wsum, wsq = float(N), float(N)
    if need_w:
        wsum = 0.0
        acc = 0.0
        for v in w1:
            wsum += v
            acc += v * v
        wsq = N + acc
    return rupp, c, a, w, L, wsum, wsq


def xi(boxsize, binfile, X, Y, Z, weights=None, weight_type=None, output_ravg=False, refine=(2, 2, 1),
       custom_refine=False, max_cells_per_dim=100, isa="fallback", nthreads=0):
    from corrfunc_gb300.theory import XI_DTYPE
    rmax = read_bins(binfile)[-1]
    rupp, c, a, w, L, wsum, wsq = _box_counts(R3, boxsize, binfile, rmax, 0.0, X, Y, Z, weights, output_ravg, refine,
                                              custom_refine, max_cells_per_dim, isa, weight_type, "xi", nthreads)
    N = len(X)
    prefac = wsum * (wsum - wsum / N) / (L * L * L)
    out = np.zeros(len(rupp) - 1, dtype=XI_DTYPE)
    rlow = 0.0
    xis = np.zeros(len(rupp))
    for i in range(len(rupp)):
        weight0 = float(c[i]) * (w[i] if weight_type is not None else 1.0)
        vol = 4.0 / 3.0 * math.pi * (rupp[i] * rupp[i] * rupp[i] - rlow * rlow * rlow)
        if vol > 0.0:
            wr = prefac * vol
            if rlow <= 0.0:
                wr += wsq
            xis[i] = weight0 / wr - 1.0
        else:
            xis[i] = -2.0
        rlow = rupp[i]
    out["rmin"], out["rmax"], out["ravg"] = rupp[:-1], rupp[1:], a[1:]
    out["xi"], out["npairs"], out["weightavg"] = xis[1:], c[1:], w[1:]
    return out


def wp(boxsize, pimax, binfile, X, Y, Z, weights=None, weight_type=None, output_rpavg=False, refine=(2, 2, 1),
       custom_refine=False, max_cells_per_dim=100, isa="fallback", nthreads=0):
    from corrfunc_gb300.theory import WP_DTYPE
    rupp, c, a, w, L, wsum, wsq = _box_counts(WP, boxsize, binfile, pimax, pimax, X, Y, Z, weights, output_rpavg,
                                              refine, custom_refine, max_cells_per_dim, isa, weight_type, "wp",
                                              nthreads)
    N = len(X)
    prefac = wsum * (wsum - wsum / N) / (L * L * L)
    twice = 2.0 * pimax
    wps = np.zeros(len(rupp))
    rlow = 0.0
    for i in range(len(rupp)):
        weight0 = float(c[i]) * (w[i] if weight_type is not None else 1.0)
        vol = math.pi * (rupp[i] * rupp[i] - rlow * rlow) * twice
        if vol > 0.0:
            wr = prefac * vol
            if rlow <= 0.0:
                wr += wsq
            wps[i] = (weight0 / wr - 1) * twice
        else:
            wps[i] = -2.0 * twice
        rlow = rupp[i]
    out = np.zeros(len(rupp) - 1, dtype=WP_DTYPE)
    out["rmin"], out["rmax"], out["rpavg"] = rupp[:-1], rupp[1:], a[1:]
    out["wp"], out["npairs"], out["weightavg"] = wps[1:], c[1:], w[1:]
    return out


def unit_vectors(ra, dec):
    ra = np.asarray(ra, dtype=np.float64)
    dec = np.asarray(dec, dtype=np.float64)
    cd = np.cos(dec * PI_OVER_180)
    return cd * np.cos(ra * PI_OVER_180), cd * np.sin(ra * PI_OVER_180), np.sin(dec * PI_OVER_180)


def DDtheta_mocks(autocorr, binfile, RA1, DEC1, weights1=None, RA2=None, DEC2=None, weights2=None,
                  output_thetaavg=False, isa="fallback", weight_type=None, nthreads=0):
    from corrfunc_gb300.mocks import DDTHETA_DTYPE
    tupp = read_bins(binfile)
    cos_upp = np.cos(tupp * PI_OVER_180)
    pos1 = unit_vectors(RA1, DEC1)
    pos2 = pos1 if autocorr else unit_vectors(RA2, DEC2)
    need_w = weight_type is not None
    w1 = _weights(weights1, len(RA1)) if need_w else None
    w2 = (w1 if autocorr else _weights(weights2, len(RA2))) if need_w else None
    if need_w and not autocorr:
        w1 = np.ones(len(RA1)) if w1 is None else w1
        w2 = np.ones(len(RA2)) if w2 is None else w2
    fma, chord = _formula(isa)
    lat = ([0.0] * 3, [0.0] * 3, [1, 1, 1], [0.0] * 3, [0, 0, 0])
    c, a, w = _count(THETA, autocorr, pos1, w1, pos2, w2, cos_upp, lat, fma, chord, need_avg=output_thetaavg,
                     need_w=need_w, nthreads=nthreads)
    self_w = float(np.sum(w1 * w1)) if (autocorr and need_w and tupp[0] <= 0) else 0.0
    c, a, w = _finalize(c, a, w, autocorr, tupp[0] <= 0, 1, len(RA1), self_w, output_thetaavg, need_w, div_start=1)
    out = np.zeros(len(tupp) - 1, dtype=DDTHETA_DTYPE)
    out["thetamin"], out["thetamax"] = tupp[:-1], tupp[1:]
    out["thetaavg"], out["npairs"], out["weightavg"] = a[1:], c[1:], w[1:]
    return out


def fix_ra_dec_cz(ra, dec, cz, is_comoving_dist):
    """In-place fix-ups of mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:43-112."""
    if np.any(dec > 180):
        raise RuntimeError("DEC above 180 degrees")
    if np.any(ra < 0.0):
        ra += 180.0
    if np.any(dec > 90.0):
        dec -= 90.0
    if max(0.0, float(np.max(cz))) < 10.0 and not is_comoving_dist:
        cz *= SPEED_OF_LIGHT


def mock_xyz(ra, dec, cz, is_comoving_dist, cosmology, zmax, with_dist=False):
    lib = _lib()
    ra, dec, cz = (np.ascontiguousarray(a, dtype=np.float64) for a in (ra, dec, cz))
    n = len(ra)
    x, y, z = np.zeros(n), np.zeros(n), np.zeros(n)

    def P(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    d = np.zeros(n)
    lib.cfo_mock_xyz.restype = ctypes.c_int
    rc = lib.cfo_mock_xyz(ctypes.c_int64(n), P(ra), P(dec), P(cz), ctypes.c_int(int(bool(is_comoving_dist))),
                          ctypes.c_double(OMEGA_M.get(cosmology, 0.25)), ctypes.c_double(zmax), P(x), P(y), P(z),
                          P(d))
    if rc != 0:
        raise RuntimeError("redshift outside the comoving-distance table")
    if with_dist:
        return x, y, z, d
    return x, y, z


def _mock_counts(mode, autocorr, cosmology, binfile, npibin, pimax_or_mu, RA1, DEC1, CZ1, weights1, RA2, DEC2, CZ2,
                 weights2, is_comoving_dist, output_avg, isa, weight_type, nthreads):
    if cosmology not in OMEGA_M:
        raise RuntimeError("Cosmology=%d not implemented" % cosmology)
    rupp = read_bins(binfile)
    sets = [(RA1, DEC1, CZ1)] + ([] if autocorr else [(RA2, DEC2, CZ2)])
    for ra, dec, cz in sets:
        fix_ra_dec_cz(ra, dec, cz, is_comoving_dist)
    czmax = 0.0
    for _, _, cz in sets:
        czmax = max(czmax, float(np.max(cz)))
    zmax = czmax * (1.0 / SPEED_OF_LIGHT) + 0.01
    pos1 = mock_xyz(RA1, DEC1, CZ1, is_comoving_dist, cosmology, zmax)
    pos2 = pos1 if autocorr else mock_xyz(RA2, DEC2, CZ2, is_comoving_dist, cosmology, zmax)
    need_w = weight_type is not None
    w1 = _weights(weights1, len(RA1)) if need_w else None
    w2 = (w1 if autocorr else _weights(weights2, len(RA2))) if need_w else None
    if need_w and not autocorr:
        w1 = np.ones(len(RA1)) if w1 is None else w1
        w2 = np.ones(len(RA2)) if w2 is None else w2
    fma, simd = _formula(isa)
    lat = ([0.0] * 3, [0.0] * 3, [1, 1, 1], [0.0] * 3, [0, 0, 0])
    c, a, w = _count(mode, autocorr, pos1, w1, pos2, w2, rupp * rupp, lat, fma, simd, npibin=npibin,
                     pimax=pimax_or_mu, need_avg=output_avg, need_w=need_w, nthreads=nthreads)
    c, a, w = _finalize(c, a, w, autocorr, False, npibin + 1, len(RA1), 0.0, output_avg, need_w)
    return rupp, c, a, w


def DDrppi_mocks(autocorr, cosmology, pimax, binfile, RA1, DEC1, CZ1, weights1=None, RA2=None, DEC2=None, CZ2=None,
                 weights2=None, is_comoving_dist=False, output_rpavg=False, isa="fallback", weight_type=None,
                 nthreads=0):
    from corrfunc_gb300.mocks import DDRPPI_MOCKS_DTYPE
    npibin = int(pimax)
    rupp, c, a, w = _mock_counts(RPPI_MOCK, autocorr, cosmology, binfile, npibin, pimax, RA1, DEC1, CZ1, weights1,
                                 RA2, DEC2, CZ2, weights2, is_comoving_dist, output_rpavg, isa, weight_type, nthreads)
    dpi = pimax / npibin
    rows = []
    for i in range(1, len(rupp)):
        for j in range(npibin):
            k = i * (npibin + 1) + j
            rows.append((rupp[i - 1], rupp[i], a[k], (j + 1) * dpi, c[k], w[k]))
    return np.array(rows, dtype=DDRPPI_MOCKS_DTYPE)


def DDsmu_mocks(autocorr, cosmology, mu_max, nmu_bins, binfile, RA1, DEC1, CZ1, weights1=None, RA2=None, DEC2=None,
                CZ2=None, weights2=None, is_comoving_dist=False, output_savg=False, isa="fallback", weight_type=None,
                nthreads=0):
    from corrfunc_gb300.mocks import DDSMU_MOCKS_DTYPE
    rupp, c, a, w = _mock_counts(SMU_MOCK, autocorr, cosmology, binfile, nmu_bins, mu_max, RA1, DEC1, CZ1, weights1,
                                 RA2, DEC2, CZ2, weights2, is_comoving_dist, output_savg, isa, weight_type, nthreads)
    dmu = mu_max / nmu_bins
    rows = []
    for i in range(1, len(rupp)):
        for j in range(nmu_bins):
            k = i * (nmu_bins + 1) + j
            rows.append((rupp[i - 1], rupp[i], a[k], (j + 1) * dmu, c[k], w[k]))
    return np.array(rows, dtype=DDSMU_MOCKS_DTYPE)


# ---- counts in spheres ----

VPF_DTYPE_CACHE = {}


def vpf_dtype(num_pN):
    return np.dtype([("rmax", np.float64), ("pN", (np.float64, num_pN))])


def mt_uniforms(seed, n):
    """n uniforms of MT19937 seeded as GSL's gsl_rng_mt19937 (cfo_mt_uniforms)."""
    lib = _lib()
    out = np.zeros(n)
    lib.cfo_mt_uniforms(ctypes.c_ulong(seed & 0xffffffffffffffff), ctypes.c_int64(n),
                        out.ctypes.data_as(ctypes.c_void_p))
    return out


def get_binsize(xdiff, xwrap, rmax, refine, max_cells):
    """utils/gridlink_utils.c.src:31-49."""
    n = int(refine * xdiff / rmax)
    n = max(n, 1)
    if xwrap > 0 and rmax >= xwrap / 2:
        raise RuntimeError("rmax must be less than half of the periodic box")
    n = min(n, max_cells)
    n = max(n, 2)
    return xdiff / n, n


def _vpf_counts(pts, lat_min, lat_inv, nmesh, refine, periodic, wrap, cen, cell, rmax, nbin, num_pN, within=False):
    lib = _lib()
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in pts)
    cen = np.ascontiguousarray(cen, dtype=np.float64).reshape(-1)
    cell = np.ascontiguousarray(cell, dtype=np.int32).reshape(-1)
    ncen = len(cen) // 3

    def P(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    arr_i = lambda v: (ctypes.c_int * 3)(*[int(t) for t in v])  # noqa: E731
    arr_d = lambda v: (ctypes.c_double * 3)(*[float(t) for t in v])  # noqa: E731
    pN = np.zeros(nbin * num_pN, dtype=np.uint64)
    ngb = np.zeros(max(ncen, 1), dtype=np.uint32)
    lib.cfo_vpf.restype = ctypes.c_int
    rc = lib.cfo_vpf(ctypes.c_int64(len(x)), P(x), P(y), P(z), arr_i(nmesh), arr_d(lat_min), arr_d(lat_inv),
                     arr_i(refine), ctypes.c_int(int(periodic)), arr_d(wrap), ctypes.c_int64(ncen), P(cen), P(cell),
                     ctypes.c_double(rmax), ctypes.c_int(nbin), ctypes.c_int(num_pN),
                     None if within else P(pN), P(ngb) if within else None)
    if rc != 0:
        raise RuntimeError("points outside the lattice")
    return ngb[:ncen] if within else pN.reshape(nbin, num_pN)


def _vpf_rows(pn, rmax, nbin, num_pN, norm):
    out = np.zeros(nbin, dtype=vpf_dtype(num_pN))
    rstep = rmax / float(nbin)
    for b in range(nbin):
        out["rmax"][b] = (b + 1) * rstep
        out["pN"][b] = [float(v) * (1.0 / float(norm)) for v in pn[b]]
    return out


def vpf(rmax, nbins, nspheres, numpN, seed, X, Y, Z, periodic=True, boxsize=None, refine=(1, 1, 1),
        max_cells_per_dim=100):
    """theory/vpf/countspheres_impl.c.src:136-479 restated; returns (results, counts)."""
    pts = [np.ascontiguousarray(a, dtype=np.float64) for a in (X, Y, Z)]
    lo = [float(np.min(a)) for a in pts]
    hi = [float(np.max(a)) for a in pts]
    b3 = _box3(boxsize)
    wrap = [(b3[a] if (periodic and b3[a] > 0) else hi[a] - lo[a]) for a in range(3)]
    nmesh, inv = [], []
    for a in range(3):
        bs, n = get_binsize(hi[a] - lo[a], wrap[a], rmax, refine[a], max_cells_per_dim)
        nmesh.append(n)
        inv.append(1.0 / bs if bs > 0 else 0.0)
    inv_wrap = [1.0 / w for w in wrap]
    need = 3 * nspheres * 4 + 64
    while True:
        u = mt_uniforms(seed, need)
        cen, cell, k = [], [], 0
        while len(cen) < nspheres and k + 3 <= need:
            c = [wrap[a] * u[k + a] + lo[a] for a in range(3)]
            k += 3
            if not periodic and any((c[a] - lo[a]) < rmax or (hi[a] - c[a]) < rmax for a in range(3)):
                continue
            idx = []
            for a in range(3):
                t = int(nmesh[a] * (c[a] - lo[a]) * inv_wrap[a])
                if t > nmesh[a] - 1:
                    t -= 1
                idx.append(t)
            cen.append(c)
            cell.append(idx)
        if len(cen) == nspheres:
            break
        need *= 4
    pn = _vpf_counts(pts, lo, inv, nmesh, refine, periodic, wrap, cen, cell, rmax, nbins, numpN)
    return _vpf_rows(pn, rmax, nbins, numpN, nspheres), pn


def vpf_mocks(rmax, nbins, nspheres, numpN, threshold_ngb, centers_file, cosmology, RA, DEC, CZ, RAND_RA, RAND_DEC,
              RAND_CZ, is_comoving_dist=False, refine=(1, 1, 1), max_cells_per_dim=100):
    """mocks/vpf_mocks/countspheres_mocks_impl.c.src:208-638 restated (the centres file is read,
    never written); returns (results, counts, centres)."""
    need_randoms = True
    file_rows = None
    if centers_file is not None and os.path.exists(centers_file):
        rows = [ln for ln in open(centers_file).read().splitlines() if ln.strip() and not ln.strip().startswith("#")]
        if rows and float(rows[0].split()[3]) >= rmax and len(rows) >= nspheres:
            need_randoms = False
            file_rows = rows
    czs = [np.asarray(CZ, dtype=np.float64)] + ([np.asarray(RAND_CZ, dtype=np.float64)] if need_randoms else [])
    zmax = max(0.0, max(float(np.max(c)) for c in czs)) * (1.0 / SPEED_OF_LIGHT) + 0.01
    gx, gy, gz, gd = mock_xyz(RA, DEC, CZ, is_comoving_dist, cosmology, zmax, with_dist=True)
    rcube = 0.0
    for v in gd:
        if v > rcube:
            rcube = float(v)
    if need_randoms:
        rx, ry, rz, rd = mock_xyz(RAND_RA, RAND_DEC, RAND_CZ, is_comoving_dist, cosmology, zmax, with_dist=True)
        for v in rd:
            if v > rcube:
                rcube = float(v)
    rcube = rcube + 1.0
    G = [gx + rcube, gy + rcube, gz + rcube]
    rcube = 2.0 * rcube
    inv_rcube = 1.0 / rcube
    nmesh, inv = [], []
    for a in range(3):
        bs, n = get_binsize(rcube, 0.0, rmax, refine[a], max_cells_per_dim)
        nmesh.append(n)
        inv.append(1.0 / bs if bs > 0 else 0.0)

    def cell_of(c):
        idx = []
        for a in range(3):
            t = int(nmesh[a] * (c[a] - 0.0) * inv_rcube)
            if t > nmesh[a] - 1:
                t -= 1
            idx.append(t)
        return idx

    nran = len(RAND_RA)
    if need_randoms:
        R = [rx + rcube / 2.0, ry + rcube / 2.0, rz + rcube / 2.0]
        cand = [[R[0][t], R[1][t], R[2][t]] for t in range(nran)]
        cells = [cell_of(c) for c in cand]
        ngb = _vpf_counts(R, [0.0] * 3, inv, nmesh, refine, False, [0.0] * 3, cand, cells, rmax, 1, 1, within=True)
        cen, cell = [], []
        for t in range(nran):
            if len(cen) >= nspheres:
                break
            if int(ngb[t]) > threshold_ngb:
                cen.append(cand[t])
                cell.append(cells[t])
    else:
        cen = []
        for ln in file_rows[:min(nspheres, nran)]:
            v = [float(t) for t in ln.split()[:4]]
            cen.append(v[:3])
        cell = [cell_of(c) for c in cen]
    pn = _vpf_counts(G, [0.0] * 3, inv, nmesh, refine, False, [0.0] * 3, cen, cell, rmax, nbins, numpN)
    return _vpf_rows(pn, rmax, nbins, numpN, len(cen)), pn, np.array(cen)
