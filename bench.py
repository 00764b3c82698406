#!/usr/bin/env python3
"""Benchmark of the triplet-counting hot path.

Default workload (one "step"): the full triangle-parametrization DDD, DDR, DRR
and RRR histograms of a 10,000-point clustered catalog (20 Gaussian blobs,
sigma 5, centres uniform in a 100^3 cube) against 10,000 uniform randoms in a
200^3 cube, binned s: 8 bins on [2,10), q: 8 bins on [1,3), theta: 16 bins on
[0, pi) (theta/3.14159 on [0,1) as the reference computes it), counted in one
batched launch with bit-exact histograms.  The unit is the triangle as the
reference's loop nest visits it (its numcalc counter): 1.334e12 per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timing: device time of the engine's kernels from CUDA events on the engine's
stream, summed over K steps after W warm-up steps; L2 is flushed before every
step (256 MiB write).  e2e repeats the step through the C ABI from host
buffers: catalog upload, count, histogram download, catalog release.
Under torchrun every rank counts its own replica of the workload (different
seeds, no collective on the data path: weak scaling) and the slowest rank's
time is reported.
"""
import argparse
import json
import os
import platform
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "3pcf_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for _p in (PKG, ORACLE):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

W_TP = 58  # issue slots per triangle of the triangle-parametrization path (fixed constant)
SPEC_AXES = [(8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)]
N_D, N_R = 10000, 10000
METRIC = "triangles/s (bit-exact histos), guarded-FP32 batched vs plain FP64; p50/p99 ms"


def workload(rank):
    import synth
    d = synth.blobs(N_D, n_blobs=20, sigma=5.0, box=100.0, seed=1 + 1000 * rank)
    r = synth.uniform(N_R, box=200.0, seed=0 + 1000 * rank)
    return d, r


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"sm_max_mhz": 2070.0}, "fallback"


def issue_peak(device=0):
    """SM issue rate in T lane-instructions/s (SMs x 128 lanes x max SM clock)
    and a note on where the numbers come from."""
    peaks, kind = measured_peaks()
    try:
        import torch
        nsm = torch.cuda.get_device_properties(device).multi_processor_count
    except Exception:
        nsm = 152
    return (nsm * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12,
            "%d SMs x 128 lanes x sm_max_mhz (%s MEASURED_PEAKS)" % (nsm, kind))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms, each sample
    stamped with the host time it arrived (summary() keeps those inside a
    window, e.g. the timed region)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, window=None):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            if window is not None and not (window[0] <= t <= window[1]):
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(world, local):
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class L2Flush:
    def __init__(self, device):
        self.buf = None
        try:
            import torch
            if torch.cuda.is_available():
                self.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda:%d" % device)
                self.torch = torch
        except Exception:
            self.buf = None

    def __call__(self):
        if self.buf is not None:
            self.buf.zero_()
            self.torch.cuda.synchronize()


def reference_binary():
    import ref_build
    if not ref_build.binary("tp_s8_q8_t16"):
        try:
            ref_build.write_configured()
            ref_build.compile_all()
        except Exception:
            pass
    return ref_build.binary("tp_s8_q8_t16")


_JOB_ID = [0]
_JOB_LOCK = threading.Lock()


def run_reference_job(exe, cats, flags, workdir):
    with _JOB_LOCK:
        _JOB_ID[0] += 1
        out = os.path.join(workdir, "out_%d.dat" % _JOB_ID[0])
    t0 = time.perf_counter()
    r = subprocess.run([exe] + cats + flags + ["-o", out],
                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, cwd=workdir)
    dt = time.perf_counter() - t0
    n = 0
    for line in r.stdout.splitlines()[::-1]:
        if line.startswith("numcalc:"):
            n = int(line.split()[1])
            break
    return n, dt, r.returncode


def cpu_baseline_single(d):
    """The reference program itself, single-threaded as it runs, on a bounded
    sample: DDD of the first 1000 points of the clustered catalog."""
    import synth
    exe = reference_binary()
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "D1000.dat")
        synth.write_7col_catalog(path, d[:1000])
        if exe:
            n, dt, rc = run_reference_job(exe, [path, path, path], [], tmp)
            if rc == 0 and n > 0:
                return {"value": n / dt, "unit": "triangles/s", "cores": 1, "kind": "reference",
                        "sample": "reference TP program (s8 q8 t16 build), DDD on the first 1000 points of the "
                                  "clustered catalog, %d triangles in %.1f s, 1 process" % (n, dt)}
    import oracle
    t0 = time.perf_counter()
    _, n = oracle.triangle([d[:1000]] * 3, 0, SPEC_AXES, nthreads=1)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "triangles/s", "cores": 1, "kind": "port",
            "sample": "oracle restatement, DDD on the first 1000 points, %d triangles, 1 thread" % n}


def impl_reference(args):
    """The reference's own CPU program on every host core: job-level
    parallelism with its -X/-x index chunks (one process per core), which is
    how the reference spreads work (examples/run_CPU_calculation_each_voxels.csh)."""
    world, rank, local = dist_env()
    if rank != 0:
        return 0
    import synth
    exe = reference_binary()
    try:
        cores = len(os.sched_getaffinity(0))
    except Exception:
        cores = os.cpu_count() or 1
    if not exe:
        print(json.dumps({"impl": "reference", "unavailable": "reference TP program could not be built here"}))
        return 0
    d, r = workload(0)
    div = 16
    with tempfile.TemporaryDirectory() as tmp:
        dp, rp = os.path.join(tmp, "D.dat"), os.path.join(tmp, "R.dat")
        synth.write_7col_catalog(dp, d)
        synth.write_7col_catalog(rp, r)
        combos = [[dp, dp, dp], [dp, dp, rp], [dp, rp, rp], [rp, rp, rp]]
        step_id = [0]

        def step():
            jobs = []
            for p in range(cores):
                s = step_id[0] * cores + p
                cats = combos[s % 4]
                a, b, c = (s // 4) % div, (s // 64) % div, (s // 7) % div
                jobs.append((cats, ["-X", str(div), "-x", "%03d%03d%03d" % (a, b, c)]))
            step_id[0] += 1
            t0 = time.perf_counter()
            import concurrent.futures
            with concurrent.futures.ThreadPoolExecutor(max_workers=cores) as ex:
                res = list(ex.map(lambda j: run_reference_job(exe, j[0], j[1], tmp), jobs))
            dt = time.perf_counter() - t0
            return sum(n for n, _, _ in res), dt

        for _ in range(args.warmup):
            step()
        tot_n, tot_t, per = 0, 0.0, []
        for _ in range(args.steps):
            n, dt = step()
            tot_n += n
            tot_t += dt
            per.append(dt * 1e3)
    value = tot_n / tot_t
    sample = ("reference TP program (s8 q8 t16 build), %d concurrent processes per step, each one -X %d index-chunk "
              "job of the DDD/DDR/DRR/RRR workload (~%.2e triangles per step)" % (cores, div, tot_n / args.steps))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "triangles/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_t * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "triangle parametrization DDD+DDR+DRR+RRR, 10k clustered + 10k uniform, "
                                   "s8[2,10) q8[1,3) theta16[0,1)", "l2": "inputs resident in host memory"},
            "p50_ms": statistics.median(per), "p99_ms": float(np.percentile(per, 99)),
            "cpu_baseline": {"value": value, "unit": "triangles/s", "cores": cores, "kind": "reference",
                             "sample": sample},
            "e2e": {"value": value, "unit": "triangles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def kernel_counters():
    """ncu counters of one fast-kernel launch of this workload (committed
    summary in profiles/): name -> value."""
    p = os.path.join(ROOT, "profiles", "triangle_fast_kernel_tp10k_counters.txt")
    out = {}
    if os.path.exists(p):
        with open(p) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 2 and not line.startswith("#"):
                    out[parts[0]] = float(parts[1])
    return out


def traffic_per_launch():
    """DRAM bytes (read + write) of one fast-kernel launch, from ncu."""
    c = kernel_counters()
    if "dram__bytes_read.sum" not in c:
        return None
    return int(c["dram__bytes_read.sum"] + c.get("dram__bytes_write.sum", 0))


def impl_ours(args):
    world, rank, local = dist_env()
    dist = init_dist(world, local)
    import tpcf
    d, r = workload(rank)
    nan = tpcf.NAN_ZERO if platform.machine() == "aarch64" else tpcf.NAN_INT_MIN
    eng = tpcf.Engine(local)
    loops = [tpcf.LOOP_SAME, tpcf.LOOP_ONE, tpcf.LOOP_ONE, tpcf.LOOP_SAME]

    def specs(precision):
        return [tpcf.make_spec(tpcf.TRIANGLE, lp, SPEC_AXES, precision=precision, nan_policy=nan) for lp in loops]

    hd, hr = eng.catalog(d), eng.catalog(r)
    jobs = [eng.job([hd, hd, hd]), eng.job([hd, hd, hr]), eng.job([hd, hr, hr]), eng.job([hr, hr, hr])]
    sp32 = specs(tpcf.GUARDED_FP32)
    flush = L2Flush(local)
    dev_ms, main_ms, wall_ms = [], [], []
    launches = 0
    units = evaluated = recheck = binned = 0
    ref_hists = None
    with ClockSampler(local) as clocks:  # running during the warm-up already
        for _ in range(args.warmup):
            eng.count_batch(sp32, jobs)
        eng.stats()
        barrier(dist)
        t_timed = time.time()
        for _ in range(args.steps):
            flush()
            t0 = time.perf_counter()
            hists = eng.count_batch(sp32, jobs)
            wall_ms.append((time.perf_counter() - t0) * 1e3)
            st = eng.stats()
            dev_ms.append(st["kernel_ms"])
            main_ms.append(st["main_kernel_ms"])
            launches += st["kernel_launches"]
            units, evaluated, recheck = st["loop_units"], st["evaluated_units"], st["recheck_units"]
            binned = st["binned_units"]
            if ref_hists is None:
                ref_hists = hists
            elif any(not np.array_equal(a, b) for a, b in zip(hists, ref_hists)):
                raise RuntimeError("histograms differ between steps")
        barrier(dist)
        t_timed_end = time.time()
    total_s = max_over_ranks(dist, sum(dev_ms) / 1e3)
    all_units = sum_over_ranks(dist, units * args.steps)
    value = all_units / total_s
    ms_per_step = total_s * 1e3 / args.steps

    # e2e through the C ABI from host buffers (upload, count, download, release)
    e2e_ms, e2e_parts = [], []
    h2d = d2h = 0
    barrier(dist)
    for _ in range(max(3, min(args.steps, 10))):
        flush()
        eng.stats()
        t0 = time.perf_counter()
        a, b = eng.catalog(d), eng.catalog(r)
        t1 = time.perf_counter()
        js = [eng.job([a, a, a]), eng.job([a, a, b]), eng.job([a, b, b]), eng.job([b, b, b])]
        hs = eng.count_batch(sp32, js)
        st = eng.stats()
        eng.release(a)
        eng.release(b)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_parts.append(((t1 - t0) * 1e3, st["plan_ms"], st["kernel_ms"], st["total_ms"]))
        h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
        if any(not np.array_equal(x, y) for x, y in zip(hs, ref_hists)):
            raise RuntimeError("e2e histograms differ")
    barrier(dist)
    e2e_s = max_over_ranks(dist, statistics.mean(e2e_ms) / 1e3)
    e2e_value = sum_over_ranks(dist, units) / e2e_s

    # the same step's jobs counted one at a time (device time of the counting
    # kernel per histogram; the batched step runs them in one launch)
    per_job = {}
    for name, sp, jb in zip(("DDD", "DDR", "DRR", "RRR"), sp32, jobs):
        t = []
        for _ in range(3):
            eng.count(sp, jb)
            t.append(eng.stats()["main_kernel_ms"])
        per_job[name] = {"ms": statistics.median(t), "binned": eng.stats()["binned_units"],
                         "loop_triangles": eng.stats()["loop_units"]}

    # plain FP64 kernel on the same jobs (one step; the >=3x comparison)
    fp64 = None
    if not args.no_fp64:
        h64 = eng.count_batch(specs(tpcf.PLAIN_FP64), jobs)
        st = eng.stats()
        if any(not np.array_equal(x, y) for x, y in zip(h64, ref_hists)):
            raise RuntimeError("plain FP64 histograms differ from the guarded FP32 ones")
        fp64 = {"value": units / (st["kernel_ms"] / 1e3), "unit": "triangles/s", "ms_per_step": st["kernel_ms"],
                "guarded_over_fp64": (units / (statistics.mean(dev_ms) / 1e3)) / (units / (st["kernel_ms"] / 1e3))}

    # Szapudi-Szalay zeta from the bit-exact counts, and its error against
    # zeta from FP64-geometry counts (one step of the FP64-geometry kernel)
    zeta = None
    if not args.no_fp64:
        import estimators
        hg = eng.count_batch(specs(tpcf.GEOMETRY_FP64), jobs)
        geo_ms = eng.stats()["kernel_ms"]
        nd, nr = len(d), len(r)
        ns = [(nd, nd, nd), (nd, nd, nr), (nd, nr, nr), (nr, nr, nr)]
        z = estimators.zeta(*ref_hists, *ns)
        zg = estimators.zeta(*hg, *ns)
        err = estimators.zeta_error(z, zg, ref_hists[3])
        pop = ref_hists[3] > 0
        zeta = {"estimator": "Szapudi-Szalay (DDD - 3DDR + 3DRR - RRR)/RRR", "fp64_oracle": "same formulas in double "
                "from the float coordinates (TPCF_GEOMETRY_FP64 kernel)", "fp64_ms": geo_ms,
                "populated_bins": err["bins"], "mean": float(np.mean(z[pop])) if pop.any() else 0.0,
                "max_abs_err": err["max_abs"], "rms_err": err["rms"], "max_rel_err": err["max_rel"],
                "counts_moved": int(sum(np.abs(a.astype(np.int64) - b.astype(np.int64)).sum()
                                        for a, b in zip(ref_hists, hg)))}

    if rank != 0:
        eng.close()
        return 0
    peaks, peak_kind = measured_peaks()
    try:
        import torch
        nsm = torch.cuda.get_device_properties(local).multi_processor_count
    except Exception:
        nsm = 152
    peak = nsm * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    achieved = W_TP * binned / (statistics.mean(main_ms) / 1e3) / 1e12
    # all lane instructions the kernel issues (ncu count of one launch) over
    # this run's kernel time: how busy the issue slots are, useful or not
    kc = kernel_counters()
    issue_frac = None
    if "smsp__inst_executed.sum" in kc:
        lane_inst = kc["smsp__inst_executed.sum"] * kc.get("smsp__thread_inst_executed_per_inst_executed.ratio", 32.0)
        issue_frac = lane_inst / (statistics.mean(main_ms) / 1e3) / 1e12 / peak
    cpu = None if args.no_cpu_baseline else cpu_baseline_single(d)
    csum = clocks.summary(window=(t_timed, t_timed_end))
    line = {
        "metric": METRIC, "value": value, "unit": "triangles/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "triangle parametrization DDD+DDR+DRR+RRR, 10k clustered (20 blobs, sigma 5, 100^3) "
                               "+ 10k uniform (200^3), s8[2,10) q8[1,3) theta16[0,1), guarded FP32, one batched launch",
                   "triangles_per_step": units, "evaluated_triangles_per_step": evaluated,
                   "binned_triangles_per_step": binned,
                   "rechecked_triangles_per_step": recheck, "l2": "flushed before every step (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "p50_ms": statistics.median(dev_ms), "p99_ms": float(np.percentile(dev_ms, 99)),
        "wall_ms_per_step": statistics.mean(wall_ms),
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": "triangles/s", "ms_per_step": e2e_s * 1e3, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "breakdown_ms": {k: statistics.median(p[i] for p in e2e_parts) for i, k in
                                 enumerate(("catalogs", "views_and_planning", "kernels", "count_call"))}},
        "per_job": per_job,
        "plain_fp64": fp64,
        "zeta": zeta,
        "roofline": {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Tinst/s",
                     "frac": achieved / peak, "traffic": traffic_per_launch(), "issue_frac": issue_frac,
                     "kernel": "triangle_fast_kernel", "per_unit": "%d lane-instructions per binned triangle (one that reaches the s/q/theta arithmetic)" % W_TP,
                     "peak_source": "%d SMs x 128 lanes x sm_max_mhz (%s MEASURED_PEAKS)" % (nsm, peak_kind)},
        "cpu_baseline": cpu,
        "clocks": csum,
    }
    print(json.dumps(line))
    eng.close()
    return 0


# ---------------------------------------------------------------------------
# Other workloads (python bench.py --config NAME); the default is the 10k + 10k
# triangle-parametrization workload above.

def _line(metric, value, unit, args, config, **kw):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
         "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
         "config": config}
    d.update(kw)
    print(json.dumps(d))


def run_pairs(args):
    """2pcf pair counts DD + DR + RR of 50k clustered (100 blobs, sigma 5) + 50k
    uniform points in a 100^3 cube, 700 bins on [0,70), one batched launch;
    FP32 path vs all-FP64 kernel, counts identical."""
    import tpcf
    import synth
    d = synth.blobs(50000, n_blobs=100, sigma=5.0, box=100.0, seed=1)
    r = synth.uniform(50000, box=100.0, seed=2)
    eng = tpcf.Engine(0)
    hd, hr = eng.catalog(d), eng.catalog(r)
    loops = [tpcf.LOOP_SAME, tpcf.LOOP_ONE, tpcf.LOOP_SAME]
    sp = [tpcf.make_spec(tpcf.PAIR, lp, [(700, 0.0, 70.0)]) for lp in loops]
    s64 = [tpcf.make_spec(tpcf.PAIR, lp, [(700, 0.0, 70.0)], precision=tpcf.PLAIN_FP64) for lp in loops]
    jobs = [eng.job([hd, hd]), eng.job([hd, hr]), eng.job([hr, hr])]
    for _ in range(args.warmup):
        eng.count_batch(sp, jobs)
    ms = []
    for _ in range(args.steps):
        h32 = eng.count_batch(sp, jobs)
        st = eng.stats()
        ms.append(st["kernel_ms"])
    h64 = eng.count_batch(s64, jobs)
    fp64_ms = eng.stats()["kernel_ms"]
    mean = statistics.mean(ms) / 1e3
    _line("pairs/s (bit-exact histos)", st["loop_units"] / mean, "pairs/s", args,
          {"workload": "2pcf DD+DR+RR, 50k clustered (100 blobs, sigma 5) + 50k uniform in 100^3, 700 bins on [0,70)",
           "pairs_per_step": st["loop_units"], "evaluated_pairs_per_step": st["evaluated_units"],
           "counted": [int(h.sum()) for h in h32]},
          ms_per_step=mean * 1e3, p50_ms=statistics.median(ms), p99_ms=float(np.percentile(ms, 99)),
          roofline=_issue_roofline(8 * st["evaluated_units"] / mean / 1e12, "pair_kernel",
                                   "8 lane-instructions per evaluated pair (pairs of tiles within reach)"),
          plain_fp64={"ms_per_step": fp64_ms, "identical": all(np.array_equal(a, b) for a, b in zip(h32, h64))})
    eng.close()
    return 0


JBJ_AXES = [(8, 2.0, 10.0), (8, 0.2, 1.0), (10, 0.0, 1.0)]


def run_jbj(args):
    """JBJ shape parametrization (s, s/m, (l - m)/s) DDD+DDR+DRR+RRR on the
    default catalogs (10k clustered + 10k uniform): s 8 bins on [2,10), s/m 8
    on [0.2,1), (l - m)/s 10 on [0,1), the reference's two extra bin-0 counts
    per visited triangle (compat).  The FP32 fast kernel (exact: the
    reference's float operations, no guard band) against the per-triangle
    kernel that visits every triangle of its tasks."""
    import tpcf
    d, r = workload(0)
    eng = tpcf.Engine(0)
    hd, hr = eng.catalog(d), eng.catalog(r)
    loops = [tpcf.LOOP_SAME, tpcf.LOOP_ONE, tpcf.LOOP_ONE, tpcf.LOOP_SAME]
    jobs = [eng.job([hd, hd, hd]), eng.job([hd, hd, hr]), eng.job([hd, hr, hr]), eng.job([hr, hr, hr])]
    sp = [tpcf.make_spec(tpcf.TRIANGLE_JBJ, lp, JBJ_AXES) for lp in loops]
    flush = L2Flush(0)
    for _ in range(args.warmup):
        eng.count_batch(sp, jobs)
    ms, ref = [], None
    for _ in range(args.steps):
        flush()
        h = eng.count_batch(sp, jobs)
        st = eng.stats()
        ms.append(st["kernel_ms"])
        if ref is None:
            ref = h
        elif any(not np.array_equal(a, b) for a, b in zip(h, ref)):
            raise RuntimeError("histograms differ between steps")
    units = st["loop_units"]
    mean = statistics.mean(ms) / 1e3
    exact = None
    if not args.no_fp64:
        h64 = eng.count_batch([tpcf.make_spec(tpcf.TRIANGLE_JBJ, lp, JBJ_AXES, precision=tpcf.PLAIN_FP64)
                               for lp in loops], jobs)
        st64 = eng.stats()
        exact = {"ms_per_step": st64["kernel_ms"], "identical": all(np.array_equal(a, b) for a, b in zip(h64, ref)),
                 "fast_over_exhaustive": st64["kernel_ms"] / (mean * 1e3)}
    _line("triangles/s (bit-exact histos)", units / mean, "triangles/s", args,
          {"workload": "JBJ (s, s/m, (l-m)/s) DDD+DDR+DRR+RRR, 10k clustered + 10k uniform, s8[2,10) q8[0.2,1) "
                       "t10[0,1), compat bin-0 counts", "triangles_per_step": units,
           "evaluated_triangles_per_step": st["evaluated_units"], "binned_triangles_per_step": st["binned_units"]},
          ms_per_step=mean * 1e3, p50_ms=statistics.median(ms), exhaustive_kernel=exact)
    eng.close()
    if exact is not None and not exact["identical"]:
        return 1
    return 0


def run_three_side(args):
    """Three-side DDD + RRR, 1000 clustered + 1000 uniform points in a
    100^3 cube, 16 bins on [0,40) (reference overflow aliasing), 2e9 triangles."""
    import tpcf
    import synth
    d = synth.blobs(1000, n_blobs=20, sigma=5.0, box=100.0, seed=1)
    r = synth.uniform(1000, box=100.0, seed=0)
    eng = tpcf.Engine(0)
    hd, hr = eng.catalog(d), eng.catalog(r)
    sp = [tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [(16, 0.0, 40.0)])] * 2
    jobs = [eng.job([hd, hd, hd]), eng.job([hr, hr, hr])]
    for _ in range(args.warmup):
        eng.count_batch(sp, jobs)
    ms = []
    for _ in range(args.steps):
        eng.count_batch(sp, jobs)
        ms.append(eng.stats()["kernel_ms"])
    units = eng.stats()["loop_units"]
    multisets = sum(n * (n + 1) * (n + 2) // 6 for n in (len(d), len(r)))
    h64 = eng.count_batch([tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [(16, 0.0, 40.0)],
                                          precision=tpcf.PLAIN_FP64)] * 2, jobs)
    fp64_ms = eng.stats()["kernel_ms"]
    h32 = eng.count_batch(sp, jobs)
    same = all(np.array_equal(a, b) for a, b in zip(h32, h64))
    cpu = None
    import ref_build
    exe = ref_build.binary("3side_n16_0_40")
    if exe and not args.no_cpu_baseline:
        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, "D400.dat")
            synth.write_header_catalog(path, d[:400])
            t0 = time.perf_counter()
            subprocess.run([exe, path, path, path, "-o", os.path.join(tmp, "o.dat")], stdout=subprocess.DEVNULL,
                           check=True)
            dt = time.perf_counter() - t0
            cpu = {"value": 400 ** 3 / dt, "unit": "triangles/s", "cores": 1, "kind": "reference",
                   "sample": "reference three-side program (16 bins on [0,40)), DDD of 400 clustered points, "
                             "6.4e7 triangles in %.1f s, as built (lock diagnostic included)" % dt}
    mean = statistics.mean(ms) / 1e3
    _line("triangles/s (bit-exact histos)", units / mean, "triangles/s", args,
          {"workload": "three-side DDD+RRR, 1000 clustered + 1000 uniform, 16 bins on [0,40)",
           "triangles_per_step": units},
          ms_per_step=mean * 1e3, p50_ms=statistics.median(ms), p99_ms=float(np.percentile(ms, 99)),
          plain_fp64={"value": units / (fp64_ms / 1e3), "ms_per_step": fp64_ms, "identical": same},
          roofline=_issue_roofline(10 * multisets / mean / 1e12, "three_side_kernel",
                                   "10 lane-instructions per multiset of three points (the kernel visits each "
                                   "multiset {i <= j <= k} once and counts all its orderings; %d multisets for "
                                   "the %d ordered triples)" % (multisets, units)),
          cpu_baseline=cpu)
    eng.close()
    return 0


def _issue_roofline(achieved, kernel, per_unit):
    peak, source = issue_peak()
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Tinst/s", "frac": achieved / peak,
            "kernel": kernel, "per_unit": per_unit, "peak_source": source}


def _jackknife_region(xyz):
    """4 x 4 cells of the flat-sky angles (x/z, y/z) over [-10, 10] degrees."""
    a = np.deg2rad(10.0)
    tx = np.clip(((xyz[:, 0] / xyz[:, 2] + a) / (2 * a) * 4).astype(int), 0, 3)
    ty = np.clip(((xyz[:, 1] / xyz[:, 2] + a) / (2 * a) * 4).astype(int), 0, 3)
    return tx * 4 + ty


def run_voxel(args):
    """100k clustered + 100k uniform points in a 20x20 degree
    light-cone slab (depth 500-1500, density falling as r^-2).  The common
    bounding box is cut into 10x10x10 voxels (~53x54x103, each edge above the
    longest counted side, 40); the catalogs are ordered by voxel.  One step is
    ONE launch of: the four full histograms (DDD, DDR, DRR, RRR), every
    canonical neighbour-voxel job of each (summed on the device into one
    histogram per kind, which must equal the full one exactly), and the jobs
    of the 16 jackknife subsamples (one 4x4 angular cell left out) x 4
    histograms: DDR subsamples as jobs of their own (its loop compares data
    and random indices, so removing points changes that comparison), the
    DDD, DRR and RRR subsamples from one decomposition of the region-ordered
    catalogs into jobs grouped by the regions they touch (summed on the
    device per group; a subsample is the full count minus the groups that
    touch its region).  The first call also counts those subsamples directly
    and checks that they are identical."""
    import tpcf
    import synth
    import voxels
    d = synth.lightcone(100000, clustered=True, seed=11)
    r = synth.lightcone(100000, seed=12)
    lo = np.minimum(d.min(0), r.min(0)).astype(np.float64)
    hi = np.maximum(d.max(0), r.max(0)).astype(np.float64)
    hi = hi + 1e-6 * (hi - lo)
    grid = (10, 10, 10)
    od, sd, ed = voxels.voxel_order(d, lo, hi, grid)
    orr, sr, er = voxels.voxel_order(r, lo, hi, grid)
    d, r = d[od], r[orr]
    rd, rr = _jackknife_region(d), _jackknife_region(r)
    nan = tpcf.NAN_ZERO if platform.machine() == "aarch64" else tpcf.NAN_INT_MIN
    eng = tpcf.Engine(0)
    kinds = (("DDD", tpcf.LOOP_SAME), ("DDR", tpcf.LOOP_ONE), ("DRR", tpcf.LOOP_ONE), ("RRR", tpcf.LOOP_SAME))
    loops = {"same": tpcf.LOOP_SAME, "one": tpcf.LOOP_ONE, "all": tpcf.LOOP_ALL}
    spec = {lp: tpcf.make_spec(tpcf.TRIANGLE, lp, SPEC_AXES, nan_policy=nan) for lp in loops.values()}
    hd, hr = eng.catalog(d), eng.catalog(r)
    cat = {"D": hd, "R": hr}
    specs, jobs, outs = [], [], []

    def add(sp, jb, out):
        specs.append(sp)
        jobs.append(jb)
        outs.append(out)

    roles = {"DDD": "DDD", "DDR": "DDR", "DRR": "DRR", "RRR": "RRR"}
    for o, (k, lp) in enumerate(kinds):  # outputs 0-3: full histograms
        add(spec[lp], eng.job([cat[x] for x in roles[k]]), o)
    nvox = 0
    for o, (k, lp) in enumerate(kinds):  # outputs 4-7: voxel sums
        for rl, rg, loop, glob in voxels.spatial_jobs(k, (sd, ed), (sr, er), grid):
            add(spec[loops[loop]], eng.job([cat[x] for x in rl], rg, global_index=glob), 4 + o)
            nvox += 1
    sub = []
    for reg in range(16):  # outputs 8-23: DDR jackknife subsamples
        jd, jr = eng.catalog(d[rd != reg]), eng.catalog(r[rr != reg])
        sub.append({"D": jd, "R": jr})
        add(spec[tpcf.LOOP_ONE], eng.job([sub[reg][x] for x in "DDR"]), 8 + reg)
    # DDD, DRR, RRR subsamples from one decomposition of the region-ordered catalogs
    gd, gr = np.argsort(rd, kind="stable"), np.argsort(rr, kind="stable")
    dg, rg_, rdg, rrg = d[gd], r[gr], rd[gd], rr[gr]
    cd = np.searchsorted(rdg, np.arange(16), "left"), np.searchsorted(rdg, np.arange(16), "right")
    cr = np.searchsorted(rrg, np.arange(16), "left"), np.searchsorted(rrg, np.arange(16), "right")
    blo, bhi = voxels.cell_boxes([dg, rg_], [cd[0], cr[0]], [cd[1], cr[1]], 16)
    neighbours, near = voxels.box_near(blo, bhi, 40.0 * 1.001)  # longest counted side < 40
    hdg, hrg = eng.catalog(dg), eng.catalog(rg_)
    gcat = {"D": hdg, "R": hrg}
    group_base, n_out = {}, 24
    for k, lp in kinds:
        if k == "DDR":
            continue
        cj, gid, groups = voxels.jackknife_groups(k, cd, cr, neighbours, near)
        for j, g in zip(cj, gid):
            add(spec[loops[j[2]]], eng.job([gcat[x] for x in j[0]], j[1], global_index=j[3]), n_out + g)
        group_base[k] = (n_out, groups)
        n_out += len(groups)

    def jackknife(hs):
        """16 x 4 subsample histograms (region-major, DDD DDR DRR RRR)."""
        out = {}
        for k, (base, groups) in group_base.items():
            out[k] = voxels.jackknife_from_groups(hs[base:base + len(groups)], groups, 16)[1]
        out["DDR"] = [hs[8 + reg] for reg in range(16)]
        return [out[k][reg] for reg in range(16) for k, _ in kinds]

    batch = eng.prepare(specs, jobs, outs, n_out)
    t0 = time.perf_counter()
    hs = eng.count_prepared(batch)
    first_s = time.perf_counter() - t0  # includes views and planning of every job
    # the subsamples counted as jobs of their own, once, for the identity check
    direct = eng.count_batch([spec[lp] for reg in range(16) for k, lp in kinds],
                             [eng.job([sub[reg][x] for x in roles[k]]) for reg in range(16) for k, _ in kinds])
    jk_exact = all(np.array_equal(a, b) for a, b in zip(jackknife(hs), direct))
    # the reference-loop triangles of the histograms a step delivers: the full
    # and voxel jobs, and every subsample as its own loop (the region
    # decomposition jobs are the means, not outputs)
    n_region = len(jobs) - 4 - nvox - 16
    units = (sum(eng.loop_units(sp, jb) for sp, jb in zip(specs[:4 + nvox + 16], jobs[:4 + nvox + 16]))
             + sum(eng.loop_units(spec[lp], eng.job([sub[reg][x] for x in roles[k]]))
                   for reg in range(16) for k, lp in kinds if k != "DDR"))
    for _ in range(max(0, args.warmup - 1)):
        eng.count_prepared(batch)
    ms, wall, st = [], [], None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        hs = eng.count_prepared(batch)
        jk = jackknife(hs)
        wall.append((time.perf_counter() - t0) * 1e3)
        st = eng.stats()
        ms.append(st["kernel_ms"])
    exact = [bool(np.array_equal(hs[o], hs[4 + o])) for o in range(4)]
    # zeta of the full light cone with its jackknife error bars (16 subsamples)
    import estimators
    zj = estimators.zeta_jackknife(tuple(hs[:4]), [tuple(jk[4 * reg:4 * reg + 4]) for reg in range(16)],
                                   (len(d), len(r)),
                                   [(int((rd != reg).sum()), int((rr != reg).sum())) for reg in range(16)])
    pop = np.nonzero(hs[3] > 0)[0]
    top = pop[np.argsort(hs[3][pop])[::-1][:5]]
    zeta_jk = {"estimator": "Szapudi-Szalay zeta of the full sample; jackknife covariance (N-1)/N sum_r "
                            "(zeta_r - mean)(zeta_r - mean)^T over the 16 subsamples",
               "populated_bins": int(len(pop)),
               "median_sigma": float(np.median(zj["sigma"][pop])) if len(pop) else 0.0,
               "median_abs_zeta_over_sigma": float(np.median(np.abs(zj["zeta"][pop]) /
                                                             np.maximum(zj["sigma"][pop], 1e-300)))
               if len(pop) else 0.0,
               "most_populated": [{"bin": int(b), "zeta": float(zj["zeta"][b]), "sigma": float(zj["sigma"][b])}
                                  for b in top]}
    mean = statistics.mean(ms) / 1e3
    _line("triangles/s (bit-exact histos)", units / mean, "triangles/s", args,
          {"workload": "light cone 100k clustered + 100k uniform, TP s8 q8 t16; one launch of 4 full histograms "
                       "+ %d canonical neighbour-voxel jobs (10x10x10 voxels, summed per kind on the device) "
                       "+ 16 jackknife subsamples x 4 histograms (DDR: 16 jobs; DDD, DRR, RRR: %d jobs of the "
                       "region decomposition in %d groups)" % (nvox, n_region, n_out - 24),
           "jobs": len(jobs), "jackknife_equals_subsample_counts": jk_exact,
           "voxel_jobs": nvox, "occupied_voxels": [int((ed > sd).sum()), int((er > sr).sum())],
           "voxel_sum_equals_full": exact, "counted_full": [int(hs[o].sum()) for o in range(4)],
           "triangles_per_step": units, "launched_loop_triangles_per_step": st["loop_units"],
           "evaluated_triangles_per_step": st["evaluated_units"],
           "binned_triangles_per_step": st["binned_units"], "tasks": st["tasks"],
           "first_call_s": first_s, "launch_shape": {"hist_copies": st["hist_copies"], "ctas_per_sm": st["ctas_per_sm"]}},
          ms_per_step=mean * 1e3, wall_ms_per_step=statistics.mean(wall), p50_ms=statistics.median(ms),
          p99_ms=float(np.percentile(ms, 99)), gpu_launches=st["kernel_launches"] * args.steps,
          graph_replays=st["graph_replays"], zeta_jackknife=zeta_jk,
          roofline={"bound": "issue", "achieved": W_TP * st["binned_units"] / (st["main_kernel_ms"] / 1e3) / 1e12,
                    "unit": "Tinst/s", "per_unit": "58 lane-instructions per binned triangle"})
    eng.close()
    if not all(exact) or not jk_exact:
        print("voxel sums or jackknife subsamples differ", exact, jk_exact, file=sys.stderr)
        return 1
    return 0


def run_lattice(args):
    """500k points uniform in a 500^3 box with 30 % on the integer
    lattice; three-side 32 bins on [0,32) restricted to triples whose sides are
    all below 32; FP32 path vs all-FP64 kernel, counts identical."""
    import tpcf
    import synth
    npts = args.lattice_points  # 500k; fewer at the same density for profiling
    pts = synth.lattice_mix(npts, box=500.0 * (npts / 500000.0) ** (1.0 / 3.0), frac=0.3, seed=3)
    eng = tpcf.Engine(0)
    h = eng.catalog(pts)
    job = eng.job([h, h, h])
    s32 = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [(32, 0.0, 32.0)], overflow=tpcf.OVERFLOW_CLEAN)
    s64 = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [(32, 0.0, 32.0)], overflow=tpcf.OVERFLOW_CLEAN,
                         precision=tpcf.PLAIN_FP64)
    for _ in range(args.warmup):
        eng.count(s32, job)
    ms = []
    for _ in range(args.steps):
        h32 = eng.count(s32, job)
        st = eng.stats()
        ms.append(st["kernel_ms"])
    # FP64 comparison on every point (or, with --fp64-slab, the slab x < 100)
    full = not args.fp64_slab
    sub = pts if full else pts[pts[:, 0] < 100.0]
    hs = h if full else eng.catalog(sub)
    js = eng.job([hs, hs, hs])
    h64 = eng.count(s64, js)
    st64 = eng.stats()
    h32s = h32 if full else eng.count(s32, js)
    mean = statistics.mean(ms) / 1e3
    _line("triangles/s (bit-exact histos)", st["loop_units"] / mean, "triangles/s", args,
          {"workload": "%dk points, %.4g^3 box, 30 %% on the integer lattice, three-side 32 bins on [0,32), "
                       "sides < 32 only" % (npts // 1000, 500.0 * (npts / 500000.0) ** (1.0 / 3.0)),
           "triangles_per_step": st["loop_units"],
           "evaluated_triangles_per_step": st["evaluated_units"], "tasks": st["tasks"],
           "counted": int(h32.sum())},
          ms_per_step=mean * 1e3, wall_ms_per_step=st["total_ms"],
          roofline=_issue_roofline(10 * int(h32.sum()) / 6 / mean / 1e12, "three_side_grouped_kernel",
                                   "10 lane-instructions per counted multiset of three points (all sides < 32; the "
                                   "kernel counts each multiset once for all its orderings: counted triples / 6)"),
          plain_fp64={"ms_per_step": st64["kernel_ms"], "points": int(len(sub)),
                      "sample": "all points" if full else "slab x < 100",
                      "identical": bool(np.array_equal(h32s, h64))})
    eng.close()
    return 0


def run_serving(args):
    """Serving: 2000 jobs with Poisson arrivals (rate --rate per second, seed
    2) on resident catalogs whose sizes are log-uniform in [500, 50000], drawn
    from the clustered-cube and light-cone generators;
    70 % triangle jobs (DDD/DDR/DRR/RRR), 30 % pair jobs (DD/DR/RR, 700 bins on
    [0,70)); p50/p99 latency from arrival to histogram and throughput."""
    import tpcf
    import synth
    rng = np.random.Generator(np.random.PCG64(2))
    nan = tpcf.NAN_ZERO if platform.machine() == "aarch64" else tpcf.NAN_INT_MIN
    eng = tpcf.Engine(0)
    pool = {"cube": [], "cone": []}
    sizes = np.exp(rng.uniform(np.log(500), np.log(50000), size=24)).astype(int)
    for i, n in enumerate(sizes):
        fam = "cube" if i % 2 == 0 else "cone"
        if fam == "cube":
            # 500 points per blob, as in the 10k-point cube workload
            dd = synth.blobs(n, n_blobs=max(1, n // 500), seed=1000 + i)
            rr = synth.uniform(n, box=100.0, seed=2000 + i)
        else:
            dd, rr = synth.lightcone(n, clustered=True, seed=3000 + i), synth.lightcone(n, seed=4000 + i)
        pool[fam].append((eng.catalog(dd), eng.catalog(rr), n))
    tp = lambda loop: tpcf.make_spec(tpcf.TRIANGLE, loop, SPEC_AXES, nan_policy=nan)
    pr = lambda loop: tpcf.make_spec(tpcf.PAIR, loop, [(700, 0.0, 70.0)])
    jobs, sizes_of, kinds, cube_jobs = [], [], [], set()
    for k in range(args.jobs):
        fam = "cube" if rng.random() < 0.5 else "cone"
        if fam == "cube":
            cube_jobs.add(k)
        a = pool[fam][int(rng.integers(len(pool[fam])))]
        b = pool[fam][int(rng.integers(len(pool[fam])))]
        hd, hr = a[0], b[1]
        if rng.random() < 0.7:
            kind = int(rng.integers(4))
            hs, loop = [([hd, hd, hd], tpcf.LOOP_SAME), ([hd, hd, hr], tpcf.LOOP_ONE),
                        ([hd, hr, hr], tpcf.LOOP_ONE), ([hr, hr, hr], tpcf.LOOP_SAME)][kind]
            jobs.append((tp(loop), eng.job(hs)))
            sizes_of.append((a[2], b[2]))
            kinds.append(["DDD", "DDR", "DRR", "RRR"][kind])
        else:
            kind = int(rng.integers(3))
            hs, loop = [([hd, hd], tpcf.LOOP_SAME), ([hd, hr], tpcf.LOOP_ONE), ([hr, hr], tpcf.LOOP_SAME)][kind]
            jobs.append((pr(loop), eng.job(hs)))
            sizes_of.append((a[2], b[2]))
            kinds.append(["DD", "DR", "RR"][kind])
    units = sum(eng.loop_units(s, j) for s, j in jobs)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=len(jobs)))
    for s, j in jobs[:20]:  # warm the kernels and the acos table
        eng.count(s, j)
    tickets = [None] * len(jobs)
    t0 = time.perf_counter()

    def submitter():
        for i, (s, j) in enumerate(jobs):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets[i] = eng.submit(s, j)

    th = threading.Thread(target=submitter)
    th.start()
    lat, run, kept = [], [], {}
    job_points = [[int(v) for v in sizes_of[i]] for i in range(len(jobs))]  # (data, random) catalog sizes
    for i, (s, j) in enumerate(jobs):
        while tickets[i] is None:
            time.sleep(0.0005)
        h, l_ms, r_ms = eng.wait_timed(tickets[i], s)
        if i % 40 == 0:
            kept[i] = h
        lat.append(l_ms)
        run.append(r_ms)
    makespan = time.perf_counter() - t0
    th.join()
    # every 40th job counted again on its own: the same histogram as in the mix
    alone_equal = all(np.array_equal(eng.count(*jobs[i]), h) for i, h in kept.items())
    _line("jobs/s with p50/p99 latency (bit-exact histos)", len(jobs) / makespan, "jobs/s", args,
          {"workload": "%d Poisson-arrival jobs at %.0f/s, catalogs 500-50000 points (log-uniform), 70 %% triangle "
                       "(s8 q8 t16) / 30 %% pair (700 bins) jobs, resident catalogs" % (len(jobs), args.rate),
           "jobs": len(jobs), "triangles_and_pairs": units,
           "alone_equals_mix": {"jobs_checked": len(kept), "identical": alone_equal}},
          p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
          mean_batch_ms=float(np.mean(run)), makespan_s=makespan, units_per_s=units / makespan,
          # a job's latency cannot be below the run time of the batch it ran in:
          # the share of jobs whose own batch ran longer than 100 ms bounds p99
          batch_ms_p99=float(np.percentile(run, 99)), jobs_in_batches_over_100ms=int(np.sum(np.array(run) > 100.0)),
          wait_ms_p99=float(np.percentile(np.array(lat) - np.array(run), 99)),
          slowest_jobs=[{"latency_ms": lat[i], "batch_ms": run[i], "kind": kinds[i], "catalog_points": job_points[i],
                         "family": "cube" if i in cube_jobs else "cone"}
                        for i in np.argsort(lat)[::-1][:int(0.01 * len(lat)) + 1]])
    eng.close()
    return 0 if alone_equal else 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--config", default="tp10k", choices=["tp10k", "three1k", "voxel100k", "lattice500k", "serving",
                                                              "pairs50k", "jbj10k"])
    ap.add_argument("--jobs", type=int, default=2000, help="serving: number of jobs")
    ap.add_argument("--rate", type=float, default=25.0, help="serving: Poisson arrival rate (jobs/s)")
    ap.add_argument("--fp64-slab", action="store_true", help="lattice500k: FP64 comparison on the slab x < 100 only")
    ap.add_argument("--lattice-points", type=int, default=500000,
                    help="lattice500k: number of points (same density; smaller cases for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return impl_reference(args)
    if args.config != "tp10k":
        return {"three1k": run_three_side, "voxel100k": run_voxel, "lattice500k": run_lattice,
                "serving": run_serving, "pairs50k": run_pairs, "jbj10k": run_jbj}[args.config](args)
    return impl_ours(args)


if __name__ == "__main__":
    sys.exit(main())
