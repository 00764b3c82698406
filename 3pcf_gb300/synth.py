"""Seeded synthetic catalogs with the shapes of the benchmark workloads.

The reference ships real MICE catalogs only up to 50k points (its 100k/500k files
are absent), so every benchmark workload is generated here from numpy's PCG64
with a recorded seed.  Coordinates are float32; the text writers print them with
``%.9g`` so that ``fscanf("%f")`` in the reference programs reads back exactly the
same floats.

Workloads (sizes and distributions):
  * clustered blobs: 20 Gaussian blobs (sigma 5) with centres uniform in a 100^3
    cube; each point picks a blob uniformly.
  * uniform randoms in a cube.
  * light-cone slab: flat-sky angles uniform in [-10, 10] degrees, comoving
    distance uniform in [500, 1500] (number density falling as r^-2 in a cone),
    x = r*theta_x, y = r*theta_y, z = r; optionally clustered around 2000 blob
    centres drawn from the same law.
  * lattice stress: uniform in a 500^3 box with 30 % of points snapped to the
    integer lattice, so many sides fall exactly on integer bin edges.
"""
import numpy as np


def blobs(n, n_blobs=20, sigma=5.0, box=100.0, seed=1):
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(0.0, box, size=(n_blobs, 3))
    which = rng.integers(0, n_blobs, size=n)
    pts = centres[which] + rng.normal(0.0, sigma, size=(n, 3))
    return pts.astype(np.float32)


def uniform(n, box=100.0, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(0.0, box, size=(n, 3)).astype(np.float32)


def lightcone(n, clustered=False, n_blobs=2000, sigma=5.0, seed=0, half_angle_deg=10.0,
              r_min=500.0, r_max=1500.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    a = np.deg2rad(half_angle_deg)

    def draw(m):
        tx = rng.uniform(-a, a, size=m)
        ty = rng.uniform(-a, a, size=m)
        r = rng.uniform(r_min, r_max, size=m)
        return np.stack([r * tx, r * ty, r], axis=1)

    if not clustered:
        return draw(n).astype(np.float32)
    centres = draw(n_blobs)
    which = rng.integers(0, n_blobs, size=n)
    pts = centres[which] + rng.normal(0.0, sigma, size=(n, 3))
    return pts.astype(np.float32)


def lattice_mix(n, box=500.0, frac=0.3, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = rng.uniform(0.0, box, size=(n, 3))
    snap = rng.random(n) < frac
    pts[snap] = np.round(pts[snap])
    return pts.astype(np.float32)


def write_header_catalog(path, xyz):
    """Header-count format read by src/3pcf_C_version.cc:311-332: N, then x y z."""
    xyz = np.asarray(xyz, dtype=np.float32)
    with open(path, "w") as f:
        f.write("%d\n" % len(xyz))
        for p in xyz:
            f.write("%.9g %.9g %.9g\n" % (float(p[0]), float(p[1]), float(p[2])))


def write_7col_catalog(path, xyz):
    """Seven-column format read by src/3pcf_C_version_triangle_parametrization.cc:377
    and src/2pcf_C_version.cc:248: id ra dec z x y z (only x y z are used)."""
    xyz = np.asarray(xyz, dtype=np.float32)
    with open(path, "w") as f:
        for i, p in enumerate(xyz):
            f.write("%d 0 0 0 %.9g %.9g %.9g\n" % (i, float(p[0]), float(p[1]), float(p[2])))
