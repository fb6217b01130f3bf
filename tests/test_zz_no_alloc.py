"""ecmg_knn_noalloc, the kNN entry point that allocates nothing (its scratch
is a fixed device array): for callers that may not allocate device memory
while they run the query, e.g. a real-time frame loop or a plug-in whose host
application owns the allocator.  Two calls in a row must give what ecmg_knn
gives with caller-provided scratch, so the shared array's leftover contents
from one call cannot leak into the next.  This file is collected last."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_knn_noalloc_matches_knn_twice(lib):
    """two calls in a row with different sizes, boxes and cells: the second,
    smaller call lays its grid out differently, so leftovers of the first in
    the shared array would show up as differences"""
    import torch

    dev = torch.device("cuda:0")
    rng = np.random.default_rng(4)
    calls = [dict(n=20000, k=16, r=3.0, box=(0.0, 0.0, 60.0, 60.0), cell=1.0, frac=0.9),
             dict(n=7000, k=10, r=2.5, box=(-10.0, -5.0, 30.0, 40.0), cell=1.7, frac=0.6)]
    for c in calls:
        n, k, r, box, cell = c["n"], c["k"], c["r"], c["box"], c["cell"]
        need = lib.ecmg_knn_scratch_bytes(n, *box, cell)
        assert 0 < need <= 16 * 1024 * 1024
        scratch = torch.empty(need, dtype=torch.uint8, device=dev)
        # a few agents outside the box (the overflow bucket every query scans)
        xy = np.stack([rng.uniform(box[0] - 2, box[2] + 2, n), rng.uniform(box[1] - 2, box[3] + 2, n)], 1)
        pos = torch.from_numpy(xy.astype(np.float32)).to(dev)
        act = torch.from_numpy((rng.uniform(0, 1, n) < c["frac"]).astype(np.uint8)).to(dev)
        ref_ids = torch.full((n, k), -5, dtype=torch.int32, device=dev)
        ref_cnt = torch.zeros(n, dtype=torch.int32, device=dev)
        assert lib.ecmg_knn(pos.data_ptr(), act.data_ptr(), n, k, r, *box, cell, ref_ids.data_ptr(),
                            ref_cnt.data_ptr(), scratch.data_ptr(), need, None) == 0
        ids = torch.full((n, k), -9, dtype=torch.int32, device=dev)
        cnt = torch.full((n,), -9, dtype=torch.int32, device=dev)
        assert lib.ecmg_knn_noalloc(pos.data_ptr(), act.data_ptr(), n, k, r, *box, cell, ids.data_ptr(),
                                    cnt.data_ptr(), None) == 0
        torch.cuda.synchronize()
        live = act.cpu().numpy() == 1
        assert np.array_equal(cnt.cpu().numpy(), ref_cnt.cpu().numpy())
        assert np.array_equal(ids.cpu().numpy()[live], ref_ids.cpu().numpy()[live])
        assert ref_cnt.cpu().numpy()[live].mean() > 1.0


def test_knn_noalloc_rejects_oversize(lib):
    import torch

    dev = torch.device("cuda:0")
    n = 4_000_000  # needs more than the 16 MiB array
    pos = torch.zeros((16, 2), dtype=torch.float32, device=dev)
    act = torch.zeros(16, dtype=torch.uint8, device=dev)
    out = torch.zeros(16, dtype=torch.int32, device=dev)
    assert lib.ecmg_knn_scratch_bytes(n, 0.0, 0.0, 100.0, 100.0, 1.0) > 16 * 1024 * 1024
    rc = lib.ecmg_knn_noalloc(pos.data_ptr(), act.data_ptr(), n, 4, 1.0, 0.0, 0.0, 100.0, 100.0, 1.0,
                              out.data_ptr(), out.data_ptr(), None)
    assert rc == 3  # ECMG_ERR_BOUND, before any device work


def test_knn_noalloc_captured_in_a_cuda_graph(lib):
    """after a first call outside capture (which resolves the array's device
    address), a call captured into a CUDA graph replays correctly: the query
    makes no host-to-device copy and no allocation, so the graph holds only
    its memsets and kernels and recomputes from the current positions"""
    import torch

    dev = torch.device("cuda:0")
    rng = np.random.default_rng(9)
    n, k, r, box, cell = 12000, 12, 2.5, (0.0, 0.0, 50.0, 50.0), 1.2

    def fresh():
        return torch.from_numpy(rng.uniform(-1.0, 51.0, (n, 2)).astype(np.float32)).to(dev)

    pos = fresh()
    act = torch.from_numpy((rng.uniform(0, 1, n) < 0.8).astype(np.uint8)).to(dev)
    ids = torch.full((n, k), -9, dtype=torch.int32, device=dev)
    cnt = torch.full((n,), -9, dtype=torch.int32, device=dev)
    s = torch.cuda.Stream()
    args = lambda: (pos.data_ptr(), act.data_ptr(), n, k, r, *box, cell, ids.data_ptr(), cnt.data_ptr(),  # noqa: E731
                    s.cuda_stream)
    assert lib.ecmg_knn_noalloc(*args()) == 0
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        rc = lib.ecmg_knn_noalloc(*args())
    assert rc == 0
    need = lib.ecmg_knn_scratch_bytes(n, *box, cell)
    scratch = torch.empty(need, dtype=torch.uint8, device=dev)
    for _ in range(2):
        pos.copy_(fresh())
        ids.fill_(-9)
        cnt.fill_(-9)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        ref_ids = torch.full((n, k), -5, dtype=torch.int32, device=dev)
        ref_cnt = torch.zeros(n, dtype=torch.int32, device=dev)
        assert lib.ecmg_knn(pos.data_ptr(), act.data_ptr(), n, k, r, *box, cell, ref_ids.data_ptr(),
                            ref_cnt.data_ptr(), scratch.data_ptr(), need, None) == 0
        torch.cuda.synchronize()
        live = act.cpu().numpy() == 1
        assert np.array_equal(cnt.cpu().numpy(), ref_cnt.cpu().numpy())
        assert np.array_equal(ids.cpu().numpy()[live], ref_ids.cpu().numpy()[live])
        assert ref_cnt.cpu().numpy()[live].mean() > 1.0
