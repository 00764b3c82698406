"""Jobs across ranks, one process per GPU.

The reference splits a large count into independent voxel jobs
(examples/build_voxel_submission_scripts.py: one batch job per `-x iiijjjkkk`
index triple) and adds the resulting files (examples/sum_voxels.py).  Here the
same independence is used across GPUs: each rank counts its share of the jobs
in one batched launch and the histograms meet on rank 0.  There is no exchange
on the data path; the only collective is the final gather of histograms.
"""
import heapq

import numpy as np


def assign(costs, world):
    """Longest-processing-time-first assignment of jobs to ranks: returns, per
    rank, the sorted job indices.  Deterministic (ties by job index, then rank)."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(x) for x in out]


def gather(dist, my_jobs, my_hists, njobs, hist_len, rank, world):
    """Histograms of all jobs on rank 0 (None elsewhere).  my_hists[i] belongs
    to job my_jobs[i]; every job is owned by exactly one rank."""
    import torch
    local = torch.zeros((njobs, hist_len), dtype=torch.int64)
    for j, h in zip(my_jobs, my_hists):
        local[j] = torch.from_numpy(np.asarray(h, dtype=np.uint64).astype(np.int64))
    if world == 1:
        return local.numpy().astype(np.uint64)
    # every job has one owner, so the sum over ranks is a gather
    dist.reduce(local, dst=0, op=dist.ReduceOp.SUM)
    return local.numpy().astype(np.uint64) if rank == 0 else None


def sum_voxels(hists):
    """The sum of voxel-job histograms (examples/sum_voxels.py adds the count
    arrays of the files element-wise)."""
    hs = [np.asarray(h, dtype=np.uint64) for h in hists]
    out = np.zeros_like(hs[0])
    for h in hs:
        out += h
    return out
