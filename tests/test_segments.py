"""Row, segment and chunk entry points (csrc/segments.cu) against NumPy /
SciPy restatements on seeded inputs: the Nyström per-chunk rescaling (the
oracle's ``rescale_chunk``), CSR row selection, the byte gather of barcodes
and the gene-level maximum.  All GPU."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import nystrom as ony


def _rescale_ref(q, v, chunk):
    return np.vstack([ony.rescale_chunk(q[r0:r0 + chunk], v) for r0 in range(0, q.shape[0], chunk)])


@pytest.mark.gpu
@pytest.mark.parametrize("n,k,chunk", [(3001, 12, 700), (500, 1, 20000), (2048, 40, 256), (77, 256, 10)])
def test_gpu_nystrom_rescale(n, k, chunk):
    import torch
    from snapatac2_gb300._nystrom import rescale_chunks
    rng = np.random.default_rng(n + k)
    q = rng.standard_normal((n, k)) + 0.3
    v = rng.uniform(0.1, 1.0, k)
    if k > 1:
        v[-1] = -0.5          # some d <= 0: the chunk minimum replaces them
    ref = _rescale_ref(q, v, chunk)
    g = torch.from_numpy(q).cuda()
    rescale_chunks(g, torch.from_numpy(v).cuda(), chunk)
    np.testing.assert_allclose(g.cpu().numpy(), ref, rtol=1e-12, atol=1e-14)


@pytest.mark.gpu
def test_gpu_nystrom_rescale_no_positive_degree_raises():
    import torch
    from snapatac2_gb300._nystrom import rescale_chunks
    q = np.abs(np.random.default_rng(1).standard_normal((300, 1))) + 0.1
    v = np.array([-1.0])        # d = -q * Σq < 0 for every row
    with pytest.raises(ValueError):
        ony.rescale_chunk(q, v)
    with pytest.raises(ValueError, match="no positive"):
        rescale_chunks(torch.from_numpy(q).cuda(), torch.from_numpy(v).cuda(), 1000)


@pytest.mark.gpu
@pytest.mark.parametrize("valued", [False, True])
def test_gpu_select_rows(valued):
    import torch
    from snapatac2_gb300._binning import DeviceCSR
    from snapatac2_gb300._nystrom import select_rows
    rng = np.random.default_rng(7)
    X = sp.random(2000, 3000, density=0.01, format="csr", random_state=3, dtype=np.float32)
    X = sp.vstack([X, sp.csr_matrix((50, 3000), dtype=np.float32)]).tocsr()
    rows = np.concatenate([rng.choice(X.shape[0], 700, replace=False), [2010, 5, 5]])
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()
    csr = DeviceCSR(d(X.indptr, np.int64), d(X.indices, np.int32), d(X.data, np.float32) if valued else None,
                    X.shape)
    out = select_rows(csr, d(rows, np.int64))
    ref = X[rows]
    np.testing.assert_array_equal(out.indptr.cpu().numpy(), ref.indptr)
    np.testing.assert_array_equal(out.indices.cpu().numpy(), ref.indices)
    if valued:
        np.testing.assert_array_equal(out.data.cpu().numpy(), ref.data)
    else:
        assert out.data is None
    empty = select_rows(csr, d(np.zeros(0), np.int64))
    assert empty.shape == (0, 3000) and empty.indptr.cpu().tolist() == [0] and empty.indices.numel() == 0


@pytest.mark.gpu
def test_gpu_gather_bytes():
    import torch
    from snapatac2_gb300._import import _gather_barcodes
    rng = np.random.default_rng(2)
    text = rng.integers(0, 256, 100_000, dtype=np.uint8)
    offs = rng.integers(0, 99_000, 3000).astype(np.int64)
    lens = rng.integers(0, 60, 3000).astype(np.int64)
    lens[::7] = 0
    got = _gather_barcodes(torch.from_numpy(text).cuda(), offs, lens)
    ref = b"".join(text[o:o + n].tobytes() for o, n in zip(offs, lens))
    assert got == ref
    assert _gather_barcodes(torch.from_numpy(text).cuda(), offs[:0], lens[:0]) == b""


def _gene_max_ref(indptr, region, counts, region_gene):
    ptr, idx, val = [0], [], []
    for r in range(len(indptr) - 1):
        best: dict = {}
        for e in range(indptr[r], indptr[r + 1]):
            g = int(region_gene[region[e]])
            best[g] = max(best.get(g, 0), int(counts[e]))
        for g in sorted(best):
            idx.append(g)
            val.append(best[g])
        ptr.append(len(idx))
    return np.array(ptr), np.array(idx, dtype=np.int64), np.array(val, dtype=np.int64)


@pytest.mark.gpu
@pytest.mark.parametrize("n,regions,genes", [(300, 5000, 700), (40, 20, 3), (5, 10, 10)])
def test_gpu_gene_max(n, regions, genes):
    import torch
    from snapatac2_gb300._genes import gene_max
    rng = np.random.default_rng(n)
    lens = np.minimum(rng.integers(0, 60, n), regions)
    lens[::5] = 0
    indptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    region = np.concatenate([np.sort(rng.choice(regions, l, replace=False)) for l in lens]).astype(np.int32)
    counts = rng.integers(1, 2**31 - 1, region.size).astype(np.int32)
    counts[::3] = 1
    region_gene = rng.integers(0, genes, regions).astype(np.int32)
    d = lambda a: torch.from_numpy(a).cuda()
    ip, ix, dv = gene_max(d(indptr), d(region), d(counts), d(region_gene))
    rp, ri, rv = _gene_max_ref(indptr, region, counts, region_gene)
    np.testing.assert_array_equal(ip.cpu().numpy(), rp)
    np.testing.assert_array_equal(ix.cpu().numpy(), ri)
    np.testing.assert_array_equal(dv.cpu().numpy(), rv)
    ip, ix, dv = gene_max(d(np.zeros(n + 1, np.int64)), d(region[:0]), d(counts[:0]), d(region_gene))
    assert ip.cpu().tolist() == [0] * (n + 1) and ix.numel() == 0
