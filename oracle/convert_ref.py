"""Test infrastructure (the oracle): numpy float64 restatement of the catalog
conversion of sample_data/gen_flat_MICE_data.py:53-99 (quadratic
redshift-distance fit, then ra/dec/distance -> x, y, z)."""
import math

import numpy as np

MICE_FIT = (-1.07199554e+00, 3.01313296e+03, -6.38827998e+02)  # :83


def radecz_to_xyz(ra, dec, redshift, poly=MICE_FIT):
    p0, p1, p2 = poly
    ra, dec, z = (np.asarray(v, dtype=np.float64) for v in (ra, dec, redshift))
    r = p0 + p1 * z + p2 * z * z                 # :55-56
    rad = math.pi / 180.0                         # :63
    x = r * np.sin(rad * (90 - dec)) * np.sin(rad * ra)   # :71-73
    y = r * np.sin(rad * (90 - dec)) * np.cos(rad * ra)
    zc = r * np.cos(rad * (90 - dec))
    return np.stack([x, y, zc], axis=1)
