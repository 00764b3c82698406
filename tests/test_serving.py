"""Serving loop (tpcf_submit / tpcf_wait): jobs of mixed kinds and sizes
submitted while others run must give exactly the histograms they give alone;
cancellation, timeouts and admission by device-memory budget."""
import os
import threading

import numpy as np
import pytest

import synth
import tpcf

pytestmark = pytest.mark.gpu

TP = [(8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)]
PAIR = [(700, 0.0, 70.0)]


def _catalogs():
    return [synth.blobs(n, n_blobs=max(1, n // 400), sigma=5.0, box=60.0, seed=100 + n) for n in (300, 900, 2000)] + \
           [synth.lightcone(n, seed=200 + n) for n in (500, 1500, 4000)]


def _jobs(eng, handles):
    jobs = []
    rng = np.random.default_rng(7)
    for t in range(24):
        a, b = (int(x) for x in rng.integers(0, len(handles), size=2))
        ha, hb = handles[a], handles[b]
        kind = t % 5
        if kind == 0:
            jobs.append((tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_SAME, TP), eng.job([ha, ha, ha])))
        elif kind == 1:
            jobs.append((tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_ONE, TP), eng.job([ha, ha, hb])))
        elif kind == 2:
            jobs.append((tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_ONE, TP), eng.job([ha, hb, hb])))
        elif kind == 3:
            jobs.append((tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, PAIR), eng.job([ha, ha])))
        else:
            jobs.append((tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_ONE, PAIR), eng.job([ha, hb])))
    return jobs


def test_results_identical_alone_and_in_the_mix():
    with tpcf.Engine(0) as eng:
        handles = [eng.catalog(c) for c in _catalogs()]
        jobs = _jobs(eng, handles)
        alone = [eng.count(s, j) for s, j in jobs]
        # submitted from two threads while earlier jobs are already running
        tickets = [None] * len(jobs)

        def submit(idx):
            for i in idx:
                tickets[i] = eng.submit(*jobs[i])

        th = [threading.Thread(target=submit, args=(range(k, len(jobs), 2),)) for k in (0, 1)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for (spec, _), t, want in zip(jobs, tickets, alone):
            got, latency, run = eng.wait_timed(t, spec)
            assert np.array_equal(got, want)
            assert latency >= run >= 0
        assert sum(int(a.sum()) for a in alone) > 0


@pytest.mark.parametrize("slice_heavy", ["1", "0"])
def test_heavy_jobs_in_slices_identical(monkeypatch, slice_heavy):
    """Every job counted as heavy (TPCF_HEAVY_COST=1): heavy serving batches
    run alone on the first lane, in slices of their task list, while light
    lanes (none here) could run between the slices; each result equals its
    count alone."""
    monkeypatch.setenv("TPCF_HEAVY_COST", "1")
    monkeypatch.setenv("TPCF_SLICE_HEAVY", slice_heavy)
    monkeypatch.setenv("TPCF_SLICE_TASKS", "7")  # many slices even for these small jobs
    with tpcf.Engine(0) as eng:
        handles = [eng.catalog(c) for c in _catalogs()]
        jobs = _jobs(eng, handles)
        alone = [eng.count(s, j) for s, j in jobs]
        tickets = [eng.submit(s, j) for s, j in jobs]
        for (spec, _), t, want in zip(jobs, tickets, alone):
            assert np.array_equal(eng.wait(t, spec), want)


def test_cancel_and_timeout():
    with tpcf.Engine(0) as eng:
        h = eng.catalog(synth.blobs(6000, n_blobs=6, sigma=5.0, box=60.0, seed=3))
        spec = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_SAME, TP)
        ts = [eng.submit(spec, eng.job([h, h, h])) for _ in range(6)]
        st = eng.cancel(ts[-1])
        if st == 0:
            with pytest.raises(tpcf.EngineError) as e:
                eng.wait(ts[-1], spec)
            assert e.value.status == -7  # TPCF_ERR_CANCELLED
        else:
            eng.wait(ts[-1], spec)  # it had already started: it completes normally
        first = None
        try:
            eng.wait(ts[0], spec, timeout_ms=0)
        except tpcf.EngineError as err:
            assert err.status == -5  # TPCF_ERR_TIMEOUT; the job keeps running
        for t in ts[:-1]:
            got = eng.wait(t, spec)
            if first is None:
                first = got
            assert np.array_equal(got, first)
        with pytest.raises(tpcf.EngineError) as e:
            eng.wait(123456789, spec)
        assert e.value.status == -6  # TPCF_ERR_NOT_FOUND


def test_admission_budget_serialises_but_stays_exact(monkeypatch):
    monkeypatch.setenv("TPCF_ADMIT_BYTES", "1")  # every batch exceeds it: one batch in flight at a time
    with tpcf.Engine(0) as eng:
        handles = [eng.catalog(c) for c in _catalogs()]
        jobs = _jobs(eng, handles)[:10]
        alone = [eng.count(s, j) for s, j in jobs]
        tickets = [eng.submit(s, j) for s, j in jobs]
        for (spec, _), t, want in zip(jobs, tickets, alone):
            assert np.array_equal(eng.wait(t, spec), want)


@pytest.mark.parametrize("heavy_cost,lanes", [("1", "2"), ("1e9", "3")])
def test_heavy_jobs_run_alone_and_stay_exact(monkeypatch, heavy_cost, lanes):
    """Scheduling by job size: heavy jobs alone on the first worker, light
    jobs batched on the others; every histogram as when counted alone."""
    monkeypatch.setenv("TPCF_HEAVY_COST", heavy_cost)
    monkeypatch.setenv("TPCF_SERVING_LANES", lanes)
    with tpcf.Engine(0) as eng:
        handles = [eng.catalog(c) for c in _catalogs()]
        jobs = _jobs(eng, handles)
        alone = [eng.count(s, j) for s, j in jobs]
        tickets = [eng.submit(s, j) for s, j in jobs]
        for (spec, _), t, want in zip(jobs, tickets, alone):
            assert np.array_equal(eng.wait(t, spec), want)
