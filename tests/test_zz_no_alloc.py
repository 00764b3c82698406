"""The pair-count entry point that allocates no device memory
(tpcf_pair_count_noalloc), for callers that must not allocate: code running
inside a framework whose memory pool owns the device, or a plugin that may not
grow its host application's device footprint.  The caller owns every buffer it
passes (here: torch tensors); the entry point's own working buffers are a fixed
per-device array inside the library.

Checked through the C ABI against the allocating entry point (tpcf_count with
a pair spec) and against the oracle's pair loop (src/2pcf_C_version.cc:358-387
restated) on two calls in a row; integer counts must be identical.  This file
is collected last so that a run stopping at its first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest

import oracle
import synth
import tpcf

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 18


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def _noalloc(xyz0, xyz1, loop, axis, same):
    import torch
    c0 = [_dev(xyz0[:, k]) for k in range(3)]
    c1 = c0 if same else [_dev(xyz1[:, k]) for k in range(3)]
    hist = torch.full((axis[0],), 123456789, dtype=torch.int64, device="cuda")  # stale values must be cleared
    torch.cuda.synchronize()
    st = tpcf.lib().tpcf_pair_count_noalloc(c0[0].data_ptr(), c0[1].data_ptr(), c0[2].data_ptr(), len(xyz0),
                                            c1[0].data_ptr(), c1[1].data_ptr(), c1[2].data_ptr(),
                                            len(xyz0) if same else len(xyz1), loop, np.float32(axis[1]),
                                            np.float32(axis[2]), axis[0], hist.data_ptr(), None)
    torch.cuda.synchronize()
    assert st == 0, tpcf.status_string(st)
    return hist.cpu().numpy().astype(np.uint64)


def _allocating(xyz0, xyz1, loop, axis, same):
    with tpcf.Engine(0) as eng:
        h0 = eng.catalog(xyz0)
        h1 = h0 if same else eng.catalog(xyz1)
        return eng.count(tpcf.make_spec(tpcf.PAIR, loop, [axis]), eng.job([h0, h1]))


@pytest.mark.parametrize("axis", [(700, 0.0, 70.0), (40, 1.0, 21.0)])
def test_noalloc_matches_allocating_entry_point(axis):
    pytest.importorskip("torch")
    d = synth.blobs(3000, n_blobs=10, sigma=5.0, box=100.0, seed=71)
    r = synth.uniform(2600, box=100.0, seed=72)
    for xyz0, xyz1, loop, same in ((d, d, tpcf.LOOP_SAME, True), (d, r, tpcf.LOOP_ONE, False),
                                   (r, d, tpcf.LOOP_SAME, False)):
        want = _allocating(xyz0, xyz1, loop, axis, same)
        ref, _ = oracle.pair([xyz0, xyz1], 1 if loop == tpcf.LOOP_ONE else 0, axis[1], axis[2], axis[0])
        first = _noalloc(xyz0, xyz1, loop, axis, same)
        second = _noalloc(xyz0, xyz1, loop, axis, same)  # the shared array keeps the first call's contents
        assert want.sum() > 0
        assert np.array_equal(want, ref)
        assert np.array_equal(first, want)
        assert np.array_equal(second, want)


def test_noalloc_rejects_sizes_beyond_its_array():
    torch = pytest.importorskip("torch")
    x = torch.zeros(MAX_POINTS + 1, dtype=torch.float32, device="cuda")
    hist = torch.zeros(10, dtype=torch.int64, device="cuda")
    p = x.data_ptr()
    st = tpcf.lib().tpcf_pair_count_noalloc(p, p, p, MAX_POINTS + 1, p, p, p, 10, tpcf.LOOP_ONE,
                                            np.float32(0), np.float32(1), 10, hist.data_ptr(), None)
    assert st == -1  # TPCF_ERR_INVALID
