"""Tile binning: oracle pinned to goldens and properties (CPU), GPU path
bit-exact against the oracle (GPU).

Reference: gen_mat_pair / gen_mat_single
(snapatac2-core/src/feature_count/data_iter.rs:313-415), properties from
snapatac2-python/tests/test_tools.py:144-162 (insertion totals do not depend
on the bin size) and tests/test_pipeline.py:10-31 (excluding chromosomes
equals importing without them).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import binning as ob
from snapatac2_gb300 import synthetic as syn

FIX = np.load(os.path.join(GOLDEN, "tile_bin.npz"))
GENOME = [(str(n), int(s)) for n, s in zip(FIX["chrom_names"], FIX["chrom_sizes"])]
CASES = sorted({k.split("_")[0] for k in FIX.files if k.startswith("case")})


def _case(c):
    kw = json.loads(str(FIX[f"{c}_spec"]))
    want = (FIX[f"{c}_indptr"], FIX[f"{c}_idx"], FIX[f"{c}_cnt"], int(FIX[f"{c}_ncols"]))
    return kw, want


def _eq(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a[:3], b[:3])) and a[3] == b[3]


# ----------------------------------------------------------------- CPU -----
@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_golden(case):
    kw, want = _case(case)
    got = ob.tile_bin(FIX["indptr"], FIX["pos"], FIX["length"], GENOME, **kw)
    assert _eq(got, want)
    got_np = ob.tile_bin_numpy(FIX["indptr"], FIX["pos"], FIX["length"], GENOME, **kw)
    assert _eq(got_np, want)


def test_oracle_golden_semantics():
    # hand-checked rows: PIC counts one hit when both ends share a tile
    genome = [("a", 1000), ("b", 300)]
    # cell 0: [a:0-100) -> both ends in tile 0; [a:450-560) spans tiles 0,1
    # cell 1: b:[0,300) ends at 299 in tile 2 (first tile of b)
    indptr = np.array([0, 2, 3])
    pos = np.array([0, 450, 1000], dtype=np.uint64)
    ln = np.array([100, 110, 300], dtype=np.uint32)
    ip, ix, ct, nc = ob.tile_bin(indptr, pos, ln, genome, bin_size=500, exclude_chroms=[])
    assert nc == 3
    assert ip.tolist() == [0, 2, 3] and ix.tolist() == [0, 1, 2] and ct.tolist() == [2, 1, 1]
    ip, ix, ct, _ = ob.tile_bin(indptr, pos, ln, genome, bin_size=500, exclude_chroms=[],
                                counting_strategy="insertion")
    assert ix.tolist() == [0, 1, 2] and ct.tolist() == [3, 1, 2]
    ip, ix, ct, _ = ob.tile_bin(indptr, pos, ln, genome, bin_size=500, exclude_chroms=[],
                                counting_strategy="fragment")
    assert ix.tolist() == [0, 1, 2] and ct.tolist() == [2, 1, 1]


def test_oracle_errors():
    genome = [("a", 1000), ("b", 300)]
    indptr = np.array([0, 2])
    # fragment running past the end of chromosome a: the reference panics
    with pytest.raises(ob.OracleError) as e:
        ob.tile_bin(indptr, np.array([10, 950], dtype=np.uint64), np.array([5, 60], dtype=np.uint32),
                    genome, exclude_chroms=[])
    assert e.value.entry == 1
    # same fragment on an excluded chromosome is skipped without error
    ob.tile_bin(indptr, np.array([10, 950], dtype=np.uint64), np.array([5, 60], dtype=np.uint32),
                genome, exclude_chroms=["a"])
    # start past the genome end
    with pytest.raises(ob.OracleError):
        ob.tile_bin(np.array([0, 1]), np.array([1300], dtype=np.uint64), np.array([1], dtype=np.uint32),
                    genome, exclude_chroms=[])


def _small_frags(seed=3, n=40):
    g = syn.make_genome(total=30_000_000, n_chrom=6)
    fm = syn.make_fragments(n, g, enriched_bins=3000, median_frags=1500, seed=seed)
    return g, fm


def test_insertion_totals_do_not_depend_on_bin_size():
    g, fm = _small_frags()
    tot = None
    for b in (500, 1000, 5000, 10000):
        ip, ix, ct, _ = ob.tile_bin(fm.indptr, fm.pos, fm.length, g, bin_size=b, exclude_chroms=[],
                                    counting_strategy="insertion")
        s = ct.astype(np.int64).sum()
        tot = s if tot is None else tot
        assert s == tot == 2 * fm.n_fragments


def _drop_chroms(g, fm, drop):
    """Re-encode fragments on the genome without the dropped chromosomes."""
    sizes = np.array([s for _, s in g], dtype=np.int64)
    ends = np.cumsum(sizes)
    starts = ends - sizes
    chrom = np.searchsorted(ends, fm.pos.astype(np.int64), side="right")
    keep_c = np.array([n not in drop for n, _ in g])
    new_start = np.cumsum(np.where(keep_c, sizes, 0)) - np.where(keep_c, sizes, 0)
    keep = keep_c[chrom]
    pos = (fm.pos.astype(np.int64) - starts[chrom] + new_start[chrom])[keep]
    cell = np.repeat(np.arange(fm.n_cells), np.diff(fm.indptr))[keep]
    indptr = np.zeros(fm.n_cells + 1, dtype=np.int64)
    np.cumsum(np.bincount(cell, minlength=fm.n_cells), out=indptr[1:])
    g2 = [(n, s) for n, s in g if n not in drop]
    return g2, indptr, pos.astype(np.uint64), fm.length[keep]


def test_exclude_equals_dropping_chromosomes():
    g, fm = _small_frags(seed=5)
    drop = [g[0][0], g[3][0]]
    a = ob.tile_bin(fm.indptr, fm.pos, fm.length, g, exclude_chroms=drop)
    g2, ip2, pos2, len2 = _drop_chroms(g, fm, drop)
    b = ob.tile_bin(ip2, pos2, len2, g2, exclude_chroms=[])
    assert _eq(a, b)


# ----------------------------------------------------------------- GPU -----
def _gpu(indptr, pos, length, genome, **kw):
    import torch
    from snapatac2_gb300 import _binning
    from snapatac2_gb300.genome import ChromSizes
    layout = _binning.tile_layout(ChromSizes(genome), kw.get("bin_size", 500),
                                  kw.get("exclude_chroms", ["chrM", "chrY", "M", "Y"]))
    dev = torch.device("cuda")
    st = kw.get("counting_strategy", "paired-insertion")
    r = _binning.tile_matrix(torch.from_numpy(np.asarray(indptr, dtype=np.int64)).to(dev),
                             torch.from_numpy(np.asarray(pos, dtype=np.uint64).view(np.int64)).to(dev),
                             torch.from_numpy(np.asarray(length, dtype=np.uint32).view(np.int32)).to(dev),
                             layout, bin_size=kw.get("bin_size", 500), strategy=st,
                             min_frag_size=kw.get("min_frag_size"), max_frag_size=kw.get("max_frag_size"))
    return (r.indptr.cpu().numpy(), r.indices.cpu().numpy(), r.data.cpu().numpy().view(np.uint32),
            r.shape[1])


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_matches_golden(case):
    kw, want = _case(case)
    got = _gpu(FIX["indptr"], FIX["pos"], FIX["length"], GENOME, **kw)
    assert _eq(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("strategy", ["paired-insertion", "insertion", "fragment", "single"])
def test_gpu_matches_oracle_large_cells(strategy):
    # median 20k fragments: many cells exceed the shared-memory key capacity
    # and take the global-scratch sort path
    g = syn.make_genome()
    fm = syn.make_fragments(64, g, median_frags=20000, sigma=0.8, seed=21)
    kw = dict(bin_size=500, exclude_chroms=["chrY"], counting_strategy=strategy)
    want = ob.tile_bin(fm.indptr, fm.pos, fm.length, g, **kw)
    got = _gpu(fm.indptr, fm.pos, fm.length, g, **kw)
    assert _eq(got, want)


@pytest.mark.gpu
def test_gpu_edge_cases():
    g = [("a", 1000), ("b", 300), ("c", 7)]
    # empty cells, zero-length fragment (end = start - 1), fragment ending on
    # the last base, fragments on an excluded chromosome, size filters
    indptr = np.array([0, 0, 3, 3, 6, 6])
    pos = np.array([500, 999, 1000, 1001, 1299, 1300], dtype=np.uint64)
    ln = np.array([0, 1, 300, 10, 1, 7], dtype=np.uint32)
    for kw in [dict(exclude_chroms=[]), dict(exclude_chroms=["b"]), dict(exclude_chroms=[], bin_size=1),
               dict(exclude_chroms=[], min_frag_size=2, max_frag_size=200),
               dict(exclude_chroms=[], counting_strategy="fragment", bin_size=3),
               dict(exclude_chroms=[], counting_strategy="insertion", bin_size=7)]:
        want = ob.tile_bin(indptr, pos, ln, g, **kw)
        got = _gpu(indptr, pos, ln, g, **kw)
        assert _eq(got, want), kw
    # no cells at all
    got = _gpu(np.array([0]), np.zeros(0, np.uint64), np.zeros(0, np.uint32), g, exclude_chroms=[])
    assert got[0].tolist() == [0] and got[1].size == 0


@pytest.mark.gpu
def test_gpu_range_errors_match_oracle():
    from snapatac2_gb300._lib import SnapGB300Error
    g = [("a", 1000), ("b", 300)]
    indptr = np.array([0, 2, 4])
    pos = np.array([10, 20, 950, 1100], dtype=np.uint64)
    ln = np.array([5, 5, 60, 10], dtype=np.uint32)
    with pytest.raises(ob.OracleError) as eo:
        ob.tile_bin(indptr, pos, ln, g, exclude_chroms=[])
    with pytest.raises(SnapGB300Error) as eg:
        _gpu(indptr, pos, ln, g, exclude_chroms=[])
    assert eg.value.code == 2 and eg.value.bad_index == eo.value.entry == 2
    # past the genome end
    with pytest.raises(SnapGB300Error):
        _gpu(np.array([0, 1]), np.array([1300], dtype=np.uint64), np.array([1], dtype=np.uint32), g,
             exclude_chroms=[])
    # excluded chromosome: no error, same as the oracle
    want = ob.tile_bin(indptr, pos, ln, g, exclude_chroms=["a"])
    assert _eq(_gpu(indptr, pos, ln, g, exclude_chroms=["a"]), want)


@pytest.mark.gpu
def test_gpu_insertion_totals_do_not_depend_on_bin_size():
    g = syn.make_genome()
    fm = syn.make_fragments(200, g, seed=9)
    for b in (500, 1000, 5000, 10000):
        ip, ix, ct, _ = _gpu(fm.indptr, fm.pos, fm.length, g, bin_size=b, exclude_chroms=[],
                             counting_strategy="insertion")
        assert ct.astype(np.int64).sum() == 2 * fm.n_fragments


@pytest.mark.gpu
def test_add_tile_matrix_api():
    import snapatac2_gb300 as snap
    g = syn.make_genome(total=50_000_000, n_chrom=6)
    fm = syn.make_fragments(30, g, enriched_bins=4000, median_frags=2000, seed=4)
    adata = snap.pp.fragments_to_anndata(fm.indptr, fm.pos, fm.length, g)
    snap.pp.add_tile_matrix(adata, bin_size=500)
    want = ob.tile_bin(fm.indptr, fm.pos, fm.length, g, bin_size=500)
    assert adata.X.dtype == np.uint32 and adata.shape == (30, want[3])
    assert _eq((adata.X.indptr, adata.X.indices, adata.X.data, adata.X.shape[1]), want)
    assert adata.var_names[0] == "chr1:0-500"
    out = snap.pp.add_tile_matrix(adata, bin_size=1000, inplace=False, exclude_chroms="chrX")
    w2 = ob.tile_bin(fm.indptr, fm.pos, fm.length, g, bin_size=1000, exclude_chroms=["chrX"])
    assert _eq((out.X.indptr, out.X.indices, out.X.data, out.X.shape[1]), w2)
    assert adata.X.shape[1] == want[3]  # the input is untouched
