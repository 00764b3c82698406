"""Repeated batches replay a captured CUDA graph of the whole step (zero,
count, recheck, copy back); the counts are the same as with graphs off, and a
changed batch is captured anew."""
import numpy as np
import pytest

import synth
import tpcf

pytestmark = pytest.mark.gpu

TP = [(8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)]


def _batch(eng, hd, hr):
    loops = [tpcf.LOOP_SAME, tpcf.LOOP_ONE, tpcf.LOOP_ONE, tpcf.LOOP_SAME]
    specs = [tpcf.make_spec(tpcf.TRIANGLE, lp, TP) for lp in loops]
    jobs = [eng.job([hd, hd, hd]), eng.job([hd, hd, hr]), eng.job([hd, hr, hr]), eng.job([hr, hr, hr])]
    return specs, jobs


def test_graph_replay_matches_direct_launches(monkeypatch):
    monkeypatch.setenv("TPCF_AUTOTUNE", "0")  # the autotuner times shapes without graphs
    d = synth.blobs(1500, n_blobs=4, sigma=5.0, box=60.0, seed=31)
    r = synth.uniform(1400, box=60.0, seed=32)
    with tpcf.Engine(0) as eng:
        hd, hr = eng.catalog(d), eng.catalog(r)
        specs, jobs = _batch(eng, hd, hr)
        first = eng.count_batch(specs, jobs)
        # the first count of a newly planned batch of several fast-kernel jobs
        # is pipelined (the later jobs are planned while the first counts) and
        # launched directly; the repeated batch replays a graph of both parts
        assert eng.stats()["graph_replays"] == 0
        again = eng.count_batch(specs, jobs)
        assert eng.stats()["graph_replays"] == 1
        for a, b in zip(first, again):
            assert np.array_equal(a, b)
        # another batch on the same lane: captured anew, still exact
        pair = eng.count(tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [(700, 0.0, 70.0)]), eng.job([hd, hd]))
        back = eng.count_batch(specs, jobs)
        for a, b in zip(first, back):
            assert np.array_equal(a, b)
        monkeypatch.setenv("TPCF_GRAPHS", "0")
        direct = eng.count_batch(specs, jobs)
        assert eng.stats()["graph_replays"] == 0
        for a, b in zip(first, direct):
            assert np.array_equal(a, b)
        # one launch over all the batch's tasks (no pipelining): the same counts
        monkeypatch.setenv("TPCF_PIPELINE", "0")
        monkeypatch.setenv("TPCF_GRAPHS", "1")
        e1 = tpcf.Engine(0)
        try:
            ha, hb = e1.catalog(d), e1.catalog(r)
            s1, j1 = _batch(e1, ha, hb)
            single = e1.count_batch(s1, j1)
            assert e1.stats()["graph_replays"] == 1
        finally:
            e1.close()
        for a, b in zip(first, single):
            assert np.array_equal(a, b)
        assert np.array_equal(pair, eng.count(tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [(700, 0.0, 70.0)]),
                                              eng.job([hd, hd])))
        assert sum(int(a.sum()) for a in first) > 0


@pytest.mark.parametrize("kind", ["triangle", "three_side", "pair"])
def test_autotuner_times_every_shape_once_and_stays_exact(kind):
    """A batch seen for the second time is counted once per candidate launch
    shape (every count exact); later calls use the fastest shape."""
    d = synth.blobs(1200, n_blobs=4, sigma=5.0, box=60.0, seed=41)
    with tpcf.Engine(0) as eng:
        h = eng.catalog(d)
        if kind == "triangle":
            spec, job = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_SAME, TP), eng.job([h, h, h])
        elif kind == "three_side":
            spec, job = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [(16, 0.0, 40.0)]), eng.job([h, h, h])
        else:
            spec, job = tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [(700, 0.0, 70.0)]), eng.job([h, h])
        first = eng.count(spec, job)
        assert eng.stats()["tuned_shapes"] == 0
        second = eng.count(spec, job)
        n_shapes = eng.stats()["tuned_shapes"]
        assert n_shapes >= 2
        third = eng.count(spec, job)
        st = eng.stats()
        assert st["tuned_shapes"] == 0
        assert st["ctas_per_sm"] >= 1
        assert np.array_equal(first, second) and np.array_equal(first, third)
        assert first.sum() > 0
