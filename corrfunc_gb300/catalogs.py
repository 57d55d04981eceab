"""Seeded synthetic catalogues (numpy PCG64) with the shapes and distributions of the
benchmark workloads: uniform periodic boxes, a clustered box (Gaussian blobs plus a uniform
component) and a spherical-cap sky patch.  Used by bench.py and the tests; no dataset is read.
"""
import numpy as np


def uniform_box(n, boxsize, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    x = rng.random(n) * boxsize
    y = rng.random(n) * boxsize
    z = rng.random(n) * boxsize
    return x.astype(dtype), y.astype(dtype), z.astype(dtype)


def clustered_box(n, boxsize, seed, nblobs=None, sigma=2.0, mean_occupancy=80.0, frac_clustered=0.8,
                  dtype=np.float64):
    """80% of the points in isotropic Gaussian blobs (centres uniform, occupancy Poisson), 20%
    uniform, wrapped into [0, boxsize) and shuffled."""
    rng = np.random.default_rng(seed)
    n_cl = int(round(frac_clustered * n))
    if nblobs is None:
        nblobs = max(1, int(round(n_cl / mean_occupancy)))
    centres = rng.random((nblobs, 3)) * boxsize
    occ = rng.poisson(mean_occupancy, nblobs)
    total = int(occ.sum())
    # trim or top up the blob members to exactly n_cl
    if total > n_cl:
        cut = np.cumsum(occ)
        keep = np.searchsorted(cut, n_cl)
        occ = occ[:keep + 1].copy()
        occ[-1] -= int(occ.sum()) - n_cl
        centres = centres[:keep + 1]
    elif total < n_cl:
        extra = rng.integers(0, nblobs, n_cl - total)
        occ = occ + np.bincount(extra, minlength=nblobs)
    owner = np.repeat(np.arange(len(occ)), occ)
    pts = centres[owner] + rng.normal(0.0, sigma, (len(owner), 3))
    uni = rng.random((n - n_cl, 3)) * boxsize
    pts = np.concatenate([pts, uni]) % boxsize
    rng.shuffle(pts)
    pts = pts.astype(dtype)
    return np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1]), np.ascontiguousarray(pts[:, 2])


def sky_cap(n, seed, ra_max=90.0, dec_max=60.0, dtype=np.float64):
    """RA uniform in [0, ra_max) deg, DEC with sin(DEC) uniform in [0, sin(dec_max)]."""
    rng = np.random.default_rng(seed)
    ra = rng.random(n) * ra_max
    dec = np.degrees(np.arcsin(rng.random(n) * np.sin(np.radians(dec_max))))
    return ra.astype(dtype), dec.astype(dtype)


def survey(n, seed, ra=(150.0, 180.0), dec=(0.0, 30.0), cz=(6000.0, 12000.0), frac_clustered=0.6, dtype=np.float64):
    """(RA, DEC, cz) of a synthetic redshift survey: a fraction of the galaxies in compact groups
    (0.2 deg, 200 km/s scatter), the rest uniform on the sky patch (sin DEC uniform) and in cz."""
    rng = np.random.default_rng(seed)
    sd = np.sin(np.radians(dec))
    nc = int(n * frac_clustered)
    nu = n - nc
    r = rng.uniform(ra[0], ra[1], nu)
    d = np.degrees(np.arcsin(rng.uniform(sd[0], sd[1], nu)))
    c = rng.uniform(cz[0], cz[1], nu)
    if nc:
        ng = max(1, nc // 25)
        g = rng.integers(0, ng, nc)
        gr = rng.uniform(ra[0], ra[1], ng)
        gd = np.degrees(np.arcsin(rng.uniform(sd[0], sd[1], ng)))
        gc = rng.uniform(cz[0], cz[1], ng)
        r = np.concatenate([r, np.clip(gr[g] + rng.normal(0.0, 0.2, nc), ra[0], ra[1])])
        d = np.concatenate([d, np.clip(gd[g] + rng.normal(0.0, 0.2, nc), dec[0], dec[1])])
        c = np.concatenate([c, np.clip(gc[g] + rng.normal(0.0, 200.0, nc), cz[0], cz[1])])
    perm = rng.permutation(n)
    return r[perm].astype(dtype), d[perm].astype(dtype), c[perm].astype(dtype)


def weights(n, seed, lo=0.5, hi=1.5, dtype=np.float64):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, n).astype(dtype)


def log_bins(rmin, rmax, nbins):
    return np.logspace(np.log10(rmin), np.log10(rmax), nbins + 1)
