"""Test infrastructure (the oracle): a Python 3 restatement of the
reference's examples/sum_voxels.py (:1-56), which adds triangle-histogram files
of voxel jobs: header values of the last file, counts summed as floats, the
file's printf layout, and the newline its print statement appends."""
import numpy as np


def sum_voxels(paths):
    tot = None
    for path in paths:
        with open(path) as f:
            vals = f.read().split()
        ngals = [int(v) for v in vals[0:3]]          # :33
        nbins = [int(v) for v in vals[3:6]]          # :34
        hv = [[float(v) for v in vals[6 + 3 * i:9 + 3 * i]] for i in range(3)]  # :35-36
        pts = np.array([float(v) for v in vals[15:]])  # :38
        tot = pts.copy() if tot is None else tot + pts  # :40-43
    tot = tot.reshape(nbins)
    out = "".join("%d\n" % n for n in ngals)
    out += "%d %d %d\n" % tuple(nbins)
    out += "".join("%-6.3f %-6.3f %-6.3f\n" % tuple(h) for h in hv)
    for i in range(nbins[0]):
        for j in range(nbins[1]):
            out += "".join("%d " % int(v) for v in tot[i][j]) + "\n"
    return out + "\n"
