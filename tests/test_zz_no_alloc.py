"""The allocation-free kNN entry point, sg_knn_noalloc.

It exists for callers that cannot allocate device memory for scratch (an
application whose device memory is owned by its own pool, or a caller that
cannot afford cudaMalloc's device-wide synchronisation).  Its scratch is a
fixed array inside the library, so this test checks, through the C ABI, that
two calls in a row give exactly the graph of the allocating sg_knn and of the
oracle (and the same count of exact FP64 rescans), that the second call is
not disturbed by what the first left in the shared array, that the largest
accepted problem (16,384 points, 32 dimensions, k = 100, candidate lists
clamped to 128) runs, and that a problem above the fixed limits is refused
without touching outputs.  The file name makes pytest collect it after every
other test file.
"""
import numpy as np
import pytest

from oracle import knn as oknn


def _call(fn_name, X, k, margin=16):
    import torch
    from snapatac2_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda")
    Xt = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).to(dev)
    n, d = X.shape
    nbr = torch.full((n, k), -7, dtype=torch.int64, device=dev)
    dist = torch.full((n, k), -7.0, dtype=torch.float64, device=dev)
    nfb = torch.full((1,), -7, dtype=torch.int32, device=dev)
    sh = torch.cuda.current_stream().cuda_stream
    if fn_name == "sg_knn":
        nbytes = int(L.sg_knn_scratch_bytes(n, d, k, margin))
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        st = L.sg_knn(Xt.data_ptr(), n, d, k, margin, nbr.data_ptr(), dist.data_ptr(), scratch.data_ptr(), nbytes,
                      nfb.data_ptr(), sh)
    else:
        st = L.sg_knn_noalloc(Xt.data_ptr(), n, d, k, margin, nbr.data_ptr(), dist.data_ptr(), nfb.data_ptr(), sh)
    torch.cuda.synchronize()
    return st, nbr.cpu().numpy(), dist.cpu().numpy(), int(nfb.cpu()[0])


def _check_against_both(X, k, margin=16):
    st_a, nbr_a, dist_a, nfb_a = _call("sg_knn", X, k, margin)
    st_b, nbr_b, dist_b, nfb_b = _call("sg_knn_noalloc", X, k, margin)
    assert st_a == 0 and st_b == 0
    assert np.array_equal(nbr_b, nbr_a)
    assert np.array_equal(dist_b, dist_a)
    assert nfb_b == nfb_a and nfb_b >= 0
    # the oracle's graph: rows sorted by column index, sqrt distances
    o_nbr, o_dist = oknn.knn_arrays(X, k)
    assert np.array_equal(nbr_b, o_nbr)
    assert np.array_equal(dist_b, o_dist)


@pytest.mark.gpu
def test_noalloc_knn_matches_allocating_entry_point_twice():
    rng = np.random.default_rng(42)
    # first call: a larger clustered problem; second: smaller, different k
    # and dimension, so stale scratch from call one would show up
    centers = rng.standard_normal((6, 30))
    X1 = centers[rng.integers(0, 6, 12000)] + 0.05 * rng.standard_normal((12000, 30))
    X2 = rng.standard_normal((3000, 12))
    for X, k in ((X1, 50), (X2, 15)):
        _check_against_both(X, k)


@pytest.mark.gpu
def test_noalloc_knn_at_its_largest_problem():
    # exactly the limits: 16,384 points, 32 dimensions, k = 100, and a
    # margin that takes k + margin past the 128-entry candidate lists (the
    # entry point clamps it), twice in a row
    rng = np.random.default_rng(7)
    centers = rng.standard_normal((10, 32))
    X = centers[rng.integers(0, 10, 16384)] + 0.1 * rng.standard_normal((16384, 32))
    for _ in range(2):
        _check_against_both(X, 100, margin=40)


@pytest.mark.gpu
def test_noalloc_knn_refuses_problems_above_its_limits():
    rng = np.random.default_rng(0)
    for X, k in ((rng.standard_normal((16385, 8)), 10),   # too many points
                 (rng.standard_normal((500, 33)), 10),     # too many dimensions
                 (rng.standard_normal((500, 8)), 101)):    # too many neighbours
        st, nbr, dist, nfb = _call("sg_knn_noalloc", X, k)
        assert st == 3  # SG_ERR_CAP
        assert np.all(nbr == -7) and np.all(dist == -7.0) and nfb == -7
