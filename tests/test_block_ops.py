"""The block Gram-Schmidt kernels of the Krylov solver through the C ABI:
sg_block_proj (C = Q[:, :ncols]ᵀ W) and sg_block_update (W -= Q[:, :ncols] C)
against FP64 NumPy, for every block width, FP32 and FP64, ragged row counts
and column counts, with NaN planted in the basis columns past ncols (which
neither kernel may read).  An odd leading dimension takes the untiled FP32
kernels, an aligned one the tiled kernels; both are checked.  Tolerance: FP32
accumulation over at most 640 terms, 4e-5 of Σ|q||w| per entry (FP64: 1e-13)."""
import numpy as np
import pytest

SHAPES = [(1, 1), (37, 5), (1000, 37), (20011, 200), (100003, 333), (4099, 608)]


def _case(n, ncols, B, ldq, dtype, seed):
    import torch
    rng = np.random.default_rng(seed)
    Q = rng.standard_normal((n, ldq))
    Q[:, ncols:] = np.nan
    W = rng.standard_normal((n, B))
    C = rng.standard_normal((ncols, B))
    td = torch.float32 if dtype == 0 else torch.float64
    Qn = Q.astype(np.float32 if dtype == 0 else np.float64)
    Wn = W.astype(Qn.dtype)
    dev = torch.device("cuda")
    return (torch.from_numpy(Qn).to(dev), torch.from_numpy(Wn).to(dev), torch.from_numpy(C).to(dev),
            Qn[:, :ncols].astype(np.float64), Wn.astype(np.float64), C, td)


@pytest.mark.gpu
@pytest.mark.parametrize("B", [4, 8, 16, 32])
@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("aligned", [True, False])
def test_proj_and_update_match_fp64(B, dtype, aligned):
    import torch
    from snapatac2_gb300 import _lib
    L = _lib.lib()
    sh = torch.cuda.current_stream().cuda_stream
    nparts = int(L.sg_proj_parts())
    tol = 4e-5 if dtype == 0 else 1e-13
    for i, (n, ncols) in enumerate(SHAPES):
        if ncols + B > 640:
            continue
        ldq = (ncols + B + 3) // 4 * 4 if aligned else ncols + B + 1
        if not aligned and ldq % 4 == 0:
            ldq += 1
        Qt, Wt, Ct, Q, W, C, td = _case(n, ncols, B, ldq, dtype, 100 * B + i)
        part = torch.empty(nparts * ncols * B, dtype=torch.float64, device="cuda")
        out = torch.empty(ncols, B, dtype=torch.float64, device="cuda")
        _lib.check(L.sg_block_proj(dtype, B, n, Qt.data_ptr(), ldq, ncols, Wt.data_ptr(), part.data_ptr(), nparts,
                                   out.data_ptr(), sh), "proj")
        ref = Q.T @ W
        bound = np.abs(Q).T @ np.abs(W)
        err = np.abs(out.cpu().numpy() - ref)
        assert np.all(err <= tol * bound + 1e-30), (n, ncols, float((err / bound).max()))
        _lib.check(L.sg_block_update(dtype, B, n, Qt.data_ptr(), ldq, ncols, Ct.data_ptr(), Wt.data_ptr(), sh),
                   "update")
        ref = W - Q @ C
        bound = np.abs(Q) @ np.abs(C) + np.abs(W)
        got = Wt.cpu().numpy().astype(np.float64)
        err = np.abs(got - ref)
        assert np.all(np.isfinite(got))
        assert np.all(err <= tol * bound + 1e-30), (n, ncols, float((err / bound).max()))


@pytest.mark.gpu
def test_tiled_kernels_are_deterministic():
    import torch
    from snapatac2_gb300 import _lib
    L = _lib.lib()
    sh = torch.cuda.current_stream().cuda_stream
    nparts = int(L.sg_proj_parts())
    n, ncols, B = 50021, 317, 16
    Qt, Wt, Ct, *_ = _case(n, ncols, B, 336, 0, 7)
    outs, ws = [], []
    for _ in range(2):
        part = torch.empty(nparts * ncols * B, dtype=torch.float64, device="cuda")
        out = torch.empty(ncols, B, dtype=torch.float64, device="cuda")
        W = Wt.clone()
        _lib.check(L.sg_block_proj(0, B, n, Qt.data_ptr(), 336, ncols, W.data_ptr(), part.data_ptr(), nparts,
                                   out.data_ptr(), sh), "proj")
        _lib.check(L.sg_block_update(0, B, n, Qt.data_ptr(), 336, ncols, Ct.data_ptr(), W.data_ptr(), sh), "update")
        outs.append(out.cpu().numpy())
        ws.append(W.cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(ws[0], ws[1])
