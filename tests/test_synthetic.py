"""The seeded generators that stand in for real data (CPU): genome shape,
per-cell fragment counts ~ LogNormal(ln 1e4, 0.6), lengths ~ Geometric
(mean 200 bp), fragments inside their chromosome, rows sorted by
(start, length), the binary matrices' row density and index layout, and
determinism per seed."""
import numpy as np

from snapatac2_gb300 import synthetic as S


def test_genome_shape():
    g = S.make_genome()
    names = [c for c, _ in g]
    sizes = np.array([s for _, s in g])
    assert names == [f"chr{i}" for i in range(1, 23)] + ["chrX", "chrY"]
    assert sizes.sum() == 3_100_000_000 and np.all(sizes > 0)
    assert 6.1e6 < np.sum(-(-sizes // 500)) < 6.3e6          # about 6.2M tiles of 500 bp


def test_fragment_distributions_and_layout():
    g = S.make_genome()
    fr = S.make_fragments(400, g, seed=3)
    counts = np.diff(fr.indptr)
    lc = np.log(counts)
    assert abs(np.exp(np.median(lc)) / 1e4 - 1) < 0.1         # median 1e4
    assert abs(lc.std() - 0.6) < 0.06                          # sigma 0.6
    ln = fr.length.astype(np.int64)
    assert ln.min() >= 1 and abs(ln.mean() - 200) < 3          # geometric, mean 200 bp
    sizes = np.array([s for _, s in g], dtype=np.int64)
    end = np.cumsum(sizes)
    pos = fr.pos.astype(np.int64)
    chrom = np.searchsorted(end, pos, side="right")
    assert np.all(chrom < len(g))
    assert np.all(pos + ln <= end[chrom])                      # never past the chromosome end
    assert fr.pos.dtype == np.uint64 and fr.length.dtype == np.uint32 and fr.indptr.dtype == np.int64
    for r in range(0, 400, 37):                                # rows sorted by (start, length)
        p, L = pos[fr.indptr[r]:fr.indptr[r + 1]], ln[fr.indptr[r]:fr.indptr[r + 1]]
        assert np.all((np.diff(p) > 0) | ((np.diff(p) == 0) & (np.diff(L) >= 0)))
    assert set(np.unique(fr.clusters)) <= set(range(8))
    again = S.make_fragments(400, g, seed=3)
    assert np.array_equal(again.pos, fr.pos) and np.array_equal(again.length, fr.length)
    assert not np.array_equal(S.make_fragments(400, g, seed=4).indptr, fr.indptr)


def test_binary_csr_density_and_layout():
    B = S.binary_csr(1000, 500_000, nnz_per_cell=4000, seed=2)
    assert B.shape == (1000, 500_000)
    assert B.indptr.dtype == np.int64 and B.indices.dtype == np.int32
    d = np.diff(B.indptr)
    assert abs(np.median(d) / 4000 - 1) < 0.03                 # ~4k distinct features in the median row
    assert abs(d.mean() / (4000 * np.exp(0.3 ** 2 / 2)) - 1) < 0.03   # lognormal targets: mean x exp(s²/2)
    assert B.indices.min() >= 0 and B.indices.max() < 500_000
    for r in range(0, 1000, 53):                               # sorted, unique within each row
        assert np.all(np.diff(B.indices[B.indptr[r]:B.indptr[r + 1]]) > 0)
    again = S.binary_csr(1000, 500_000, nnz_per_cell=4000, seed=2)
    assert np.array_equal(again.indices, B.indices) and np.array_equal(again.indptr, B.indptr)
