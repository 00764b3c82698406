#!/usr/bin/env python3
"""Golden vectors for the estimators (test infrastructure only): the
reference's own post-processing scripts executed on committed histogram files.

examples/plot_MICE_2pcf.py and examples/plot_MICE_3pcf.py are Python 2 scripts
that read histogram files, compute xi (2pcf) and the Szapudi-Szalay zeta and
the reduced zeta (3pcf), and plot them.  This script runs each of them
unmodified apart from two mechanical Python 2 -> 3 rewrites (a ``print``
statement becomes ``pass``; ``xrange`` becomes ``range``), with matplotlib
replaced by a recorder that keeps the y values of every ``plot`` call, on:

* the compiled-reference pair files tests/golden/ref/2pcf_<variant>_{DD,DR,RR}
  -> ``tpcf`` (xi) and the table the script writes, master_2pcf_reference.dat;
* the compiled-reference triangle files tests/golden/ref/tp_<variant>_{DDD,DDR,DRR,RRR}
  -> ``tpcf`` (zeta, S x Q x T);
* the reference's own LRG golden files (tests/golden/sandbox/*_Debbie_LRG_*)
  -> zeta and, for s bin SBIN and q bins QBINS, the reduced zeta the script
  plots (it reads master_2pcf_reference.dat, here the table made in the step
  before from 2pcf_default).  The script takes the theta bin width from the
  file's header, printed with three decimals, and builds its theta axis with
  np.arange: with 16 or 32 theta bins (width 0.062 or 0.031 as printed) the
  axis has one value too many and the reduced-zeta line fails, so the
  reduced zeta is pinned on the 25-bin LRG files only (width 0.040).

Output: tests/golden/estimator_pins.npz.  Needs the reference checkout
(TPCF_REFERENCE_DIR or the first argument).
"""
import gzip
import os
import re
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("TPCF_REFERENCE_DIR") or (sys.argv[1] if len(sys.argv) > 1 else None)
SBIN, QBINS = 3, [0, 2, 5]
PAIR_VARIANTS = ["2pcf_default", "2pcf_s40_1_21"]
TP_VARIANTS = ["tp_s8_q8_t16", "tp_default"]
LRG = "Debbie_LRG_CPU_10degx10deg_LRG_binning_SLAC_1k.dat"


class Recorder:
    """Stands in for matplotlib: every attribute is a callable returning a
    recorder; plot(x, y, ...) keeps y."""

    def __init__(self, log):
        self._log = log

    def __getattr__(self, name):
        def call(*a, **k):
            if name == "plot" and len(a) >= 2:
                self._log.append(np.array(a[1], dtype=np.float64, copy=True))
            return Recorder(self._log)
        return call


def py3(source):
    out = []
    for line in source.splitlines():
        m = re.match(r"^(\s*)print\b(?!\s*\()", line)
        out.append(m.group(1) + "pass" if m else line.replace("xrange(", "range("))
    return "\n".join(out) + "\n"


def run_script(name, argv, cwd):
    with open(os.path.join(REFERENCE, "examples", name)) as f:
        code = compile(py3(f.read()), name, "exec")
    log = []
    mpl = types.ModuleType("matplotlib")
    pylab = Recorder(log)
    mpl.pylab = pylab
    saved = (dict(sys.modules), list(sys.argv), os.getcwd())
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pylab"] = pylab
    sys.argv = [name] + argv
    os.chdir(cwd)
    ns = {"__name__": "__main__"}
    err = None
    try:
        exec(code, ns)
    except ValueError as e:  # see the note on the theta axis above
        err = e
    finally:
        sys.modules.clear()
        sys.modules.update(saved[0])
        sys.argv = saved[1]
        os.chdir(saved[2])
    return ns, log, err


def write_fixture(src_gz, dst):
    with gzip.open(src_gz, "rb") as f, open(dst, "wb") as g:
        g.write(f.read())


def main():
    if not REFERENCE or not os.path.isdir(REFERENCE):
        print("make_estimator_pins: give the reference checkout (TPCF_REFERENCE_DIR or the first argument)")
        return 1
    pins = {}
    with tempfile.TemporaryDirectory() as tmp:
        for var in PAIR_VARIANTS:
            for h in ("DD", "DR", "RR"):
                write_fixture(os.path.join(HERE, "ref", "%s_%s.dat.gz" % (var, h)), os.path.join(tmp, "p_%s.dat" % h))
            ns, _, err = run_script("plot_MICE_2pcf.py", ["p_DD.dat"], tmp)
            assert err is None, err
            pins["xi_" + var] = np.asarray(ns["tpcf"], dtype=np.float64)
            with open(os.path.join(tmp, "master_2pcf_reference.dat")) as f:
                pins["table_" + var] = np.array(f.read())
        # the 3pcf script reads the table of the default pair binning
        with open(os.path.join(tmp, "master_2pcf_reference.dat"), "w") as f:
            f.write(str(pins["table_2pcf_default"]))
        for var in TP_VARIANTS:
            for h in ("DDD", "DDR", "DRR", "RRR"):
                write_fixture(os.path.join(HERE, "ref", "%s_%s.dat.gz" % (var, h)), os.path.join(tmp, "t_%s.dat" % h))
            ns, _, _ = run_script("plot_MICE_3pcf.py", ["t_DDD.dat", str(SBIN)] + [str(q) for q in QBINS], tmp)
            pins["zeta_" + var] = np.asarray(ns["tpcf"], dtype=np.float64)
        for h in ("DDD", "DDR", "DRR", "RRR"):
            write_fixture(os.path.join(HERE, "sandbox", "%s_%s.gz" % (h, LRG)), os.path.join(tmp, "l_%s.dat" % h))
        ns, log, err = run_script("plot_MICE_3pcf.py", ["l_DDD.dat", str(SBIN)] + [str(q) for q in QBINS], tmp)
        assert err is None, err
        pins["zeta_lrg"] = np.asarray(ns["tpcf"], dtype=np.float64)
        # per q bin the script plots: ddd, ddr, drr, rrr, ddd again, zeta,
        # reduced zeta (in that order)
        per_q = len(log) // len(QBINS)
        pins["reduced_lrg"] = np.stack([log[i * per_q + per_q - 1] for i in range(len(QBINS))])
    pins["sbin"] = np.array(SBIN)
    pins["qbins"] = np.array(QBINS)
    np.savez_compressed(os.path.join(HERE, "estimator_pins.npz"), **pins)
    print("written", os.path.join(HERE, "estimator_pins.npz"), sorted(pins))
    return 0


if __name__ == "__main__":
    sys.exit(main())
