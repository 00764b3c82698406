"""Job sharding across ranks: assignment, and the gather of histograms over a
world_size-2 gloo group on CPU (histograms from the oracle)."""
import os
import socket

import numpy as np
import pytest

import sharding


def test_assign_covers_every_job_once_and_balances():
    costs = [50, 1, 1, 30, 20, 20, 7, 7, 3, 0]
    parts = sharding.assign(costs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert sharding.assign(costs, 3) == parts  # deterministic
    assert sharding.assign([], 2) == [[], []]
    assert sharding.assign(costs, 1) == [list(range(len(costs)))]


def test_sum_voxels():
    a = np.array([1, 2, 3], dtype=np.uint64)
    b = np.array([0, 5, 1], dtype=np.uint64)
    assert np.array_equal(sharding.sum_voxels([a, b]), [1, 7, 4])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cases():
    import synth
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    d = synth.blobs(90, n_blobs=2, sigma=3.0, box=20.0, seed=4)
    r = synth.uniform(80, box=20.0, seed=5)
    # voxel chunks of D and R (index ranges, 3 chunks each) as separate jobs
    jobs = []
    for a in range(3):
        for b in range(3):
            jobs.append(([d[30 * a:30 * a + 30], d[30 * b:30 * b + 30], r], 1))
    jobs.append(([d, d, d], 0))
    jobs.append(([r, r, r], 0))
    return spec, jobs


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec, jobs = _cases()
    costs = [len(c[0]) * len(c[1]) * len(c[2]) for c, _ in jobs]
    mine = sharding.assign(costs, world)[rank]
    hists = [oracle.triangle(jobs[j][0], jobs[j][1], spec, nthreads=1)[0] for j in mine]
    got = sharding.gather(dist, mine, hists, len(jobs), 1024, rank, world)
    if rank == 0:
        np.save(out, got)
    dist.barrier()
    dist.destroy_process_group()


def test_gather_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    import oracle
    out = str(tmp_path / "h.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    got = np.load(out)
    spec, jobs = _cases()
    want = np.stack([oracle.triangle(c, w, spec, nthreads=1)[0] for c, w in jobs])
    assert np.array_equal(got, want)
    assert want.sum() > 0


def test_voxel_chunks_match_reference_helpers():
    import refformat as rf
    import voxels
    for div, n in ((2, 1000), (10, 100000), (7, 53), (3, 3)):
        for idx in range(div):
            assert voxels.vox2gal(div, idx, n) == rf.vox2gal(div, idx, n)
    with pytest.raises(ValueError):
        voxels.vox2gal(10, 0, 5)
    for v in (0, 1, 1000, 1001001, 9009009, 123456789):
        assert voxels.decode(v) == rf.voxel_indices(v, 3)
        assert voxels.decode(v, 2) == rf.voxel_indices(v, 2)
    cr = voxels.chunk_ranges(10, [100, 100, 93])
    assert len(cr) == 1000 and cr[0][0] == (0, 0, 0) and cr[-1][1][2] == (81, 93)
    assert len(voxels.chunk_ranges(3, [9, 9])) == 9
