"""snap.pp.make_peak_matrix: the oracle on hand-made rows and its C
restatement against its Python one (CPU), the GPU
region counter against the oracle (GPU), and a property that ties it to the
tile matrix: with every genome tile given as a peak, the peak matrix is the
tile matrix."""
import gzip

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import regions as org

NAMES = ["chr1", "chr2"]
SIZES = [1000, 500]


def test_oracle_strategies():
    # one paired fragment chr1:[100, 300): insertions at 100 and 299
    ptr, pos, ln = [0, 1], [100], [200]
    peaks = ["chr1:50-150", "chr1:250-400", "chr1:0-1000", "chr1:150-250", "chr2:0-10", "chr1:50-150"]
    ip, ix, dv, names = org.region_counts(ptr, pos, ln, NAMES, SIZES, peaks, strategy="insertion")
    assert names == ["chr1:50-150", "chr1:250-400", "chr1:0-1000", "chr1:150-250", "chr2:0-10"]  # repeat dropped
    assert dict(zip(ix.tolist(), dv.tolist())) == {0: 1, 1: 1, 2: 2}     # both insertions in 0-1000
    _, ix, dv, _ = org.region_counts(ptr, pos, ln, NAMES, SIZES, peaks, strategy="paired-insertion")
    assert dict(zip(ix.tolist(), dv.tolist())) == {0: 1, 1: 1, 2: 1}
    _, ix, dv, _ = org.region_counts(ptr, pos, ln, NAMES, SIZES, peaks, strategy="fragment")
    assert dict(zip(ix.tolist(), dv.tolist())) == {0: 1, 1: 1, 2: 1, 3: 1}
    _, ix, dv, _ = org.region_counts(ptr, pos, ln, NAMES, SIZES, peaks, strategy="fragment", max_frag_size=150)
    assert ix.size == 0
    # single-end: the stored position only (1000 + 5 is chr2:5)
    _, ix, dv, _ = org.region_counts([0, 2], [100, 1005], [10, -3], NAMES, SIZES, peaks, paired=False)
    assert dict(zip(ix.tolist(), dv.tolist())) == {0: 1, 2: 1, 4: 1}


def test_c_oracle_hand_made_rows():
    ptr, pos, ln = [0, 1], [100], [200]
    peaks = ["chr1:50-150", "chr1:250-400", "chr1:0-1000", "chr1:150-250", "chr2:0-10", "chr1:50-150"]
    for strategy, kw in [("insertion", {}), ("paired-insertion", {}), ("fragment", {}),
                         ("fragment", dict(max_frag_size=150))]:
        got = org.region_counts_c(ptr, pos, ln, NAMES, SIZES, peaks, strategy=strategy, **kw)
        ref = org.region_counts(ptr, pos, ln, NAMES, SIZES, peaks, strategy=strategy, **kw)
        for g, r in zip(got[:3], ref[:3]):
            np.testing.assert_array_equal(g, r)
        assert got[3] == ref[3]
    got = org.region_counts_c([0, 2], [100, 1005], [10, 3], NAMES, SIZES, peaks, paired=False)
    assert dict(zip(got[1].tolist(), got[2].tolist())) == {0: 1, 2: 1, 4: 1}
    with pytest.raises(ValueError, match="outside the genome"):
        org.region_counts_c([0, 2], [100, 1500], [10, 3], NAMES, SIZES, peaks)
    with pytest.raises(ValueError, match="outside the genome"):
        org.region_counts([0, 2], [100, 1500], [10, 3], NAMES, SIZES, peaks)


def _data(n_cells=30, seed=0):
    from snapatac2_gb300 import synthetic as S
    g = S.make_genome(total=8_000_000, n_chrom=6)
    fr = S.make_fragments(n_cells, g, median_frags=400, enriched_bins=500, seed=seed)
    rng = np.random.default_rng(seed)
    peaks = []
    for c, size in g:
        starts = np.sort(rng.integers(0, size - 2000, 300))
        widths = rng.choice([1, 200, 500, 5000], 300)
        peaks += [f"{c}:{s}-{min(s + w, size + 50)}" for s, w in zip(starts.tolist(), widths.tolist())]
    peaks += peaks[:7] + ["chrUn:0-100", f"{g[0][0]}:10-10", f"{g[1][0]}:0-{g[1][1]}"]
    rng.shuffle(peaks)
    return g, fr, peaks


@pytest.mark.parametrize("strategy,kw", [("insertion", {}), ("paired-insertion", {}), ("fragment", {}),
                                         ("paired-insertion", dict(min_frag_size=50, max_frag_size=300)),
                                         ("single", {})])
def test_c_oracle_matches_python_oracle(strategy, kw):
    """The C restatement (OpenMP over cells) gives the Python restatement's
    matrix bit for bit, whatever the thread count."""
    g, fr, peaks = _data(seed=21 + len(kw))
    names, sizes = [c for c, _ in g], [s for _, s in g]
    paired = strategy != "single"
    ref = org.region_counts(fr.indptr, fr.pos, fr.length, names, sizes, peaks, strategy=strategy, paired=paired,
                            **kw)
    for threads in (1, 4):
        got = org.region_counts_c(fr.indptr, fr.pos, fr.length, names, sizes, peaks, strategy=strategy,
                                  paired=paired, n_threads=threads, **kw)
        for a, b in zip(got[:3], ref[:3]):
            np.testing.assert_array_equal(a, b)
        assert got[3] == ref[3]


@pytest.mark.gpu
@pytest.mark.parametrize("strategy,kw", [("insertion", {}), ("paired-insertion", {}), ("fragment", {}),
                                         ("paired-insertion", dict(min_frag_size=50, max_frag_size=300)),
                                         ("single", {})])
def test_gpu_region_counts_match_oracle(strategy, kw):
    import torch
    from snapatac2_gb300 import _regions
    from snapatac2_gb300.genome import ChromSizes
    seed = {"insertion": 1, "paired-insertion": 2, "fragment": 3, "single": 4}[strategy] + 10 * len(kw)
    g, fr, peaks = _data(seed=seed)
    names, sizes = [c for c, _ in g], [s for _, s in g]
    paired = strategy != "single"
    length = fr.length.astype(np.int64) if paired else np.where(np.arange(fr.n_fragments) % 2, 1, -1) * 7
    ref = org.region_counts(fr.indptr, fr.pos, length, names, sizes, peaks, strategy=strategy, paired=paired, **kw)
    dev = torch.device("cuda")
    regs = _regions.build_regions(peaks, names, dev)
    t_len = torch.from_numpy(length.astype(np.int32)).to(dev)
    res = _regions.region_matrix(torch.from_numpy(fr.indptr).to(dev), torch.from_numpy(fr.pos.view(np.int64)).to(dev),
                                 t_len, ChromSizes(g), regs, strategy=strategy, **kw)
    assert regs.names == ref[3]
    np.testing.assert_array_equal(res.indptr.cpu().numpy(), ref[0])
    np.testing.assert_array_equal(res.indices.cpu().numpy(), ref[1])
    np.testing.assert_array_equal(res.data.cpu().numpy().view(np.uint32), ref[2])


@pytest.mark.gpu
def test_gpu_peaks_as_tiles_equal_tile_matrix():
    import snapatac2_gb300 as snap
    from snapatac2_gb300 import synthetic as S
    g = S.make_genome(total=4_000_000, n_chrom=4)
    fr = S.make_fragments(20, g, median_frags=300, enriched_bins=300, seed=3)
    for strategy in ("insertion", "paired-insertion", "fragment"):
        ad = snap.pp.fragments_to_anndata(fr.indptr, fr.pos, fr.length, g)
        snap.pp.add_tile_matrix(ad, bin_size=500, exclude_chroms=None, counting_strategy=strategy)
        peaks = list(ad.var_names)
        pm = snap.pp.make_peak_matrix(ad, use_rep=peaks, counting_strategy=strategy)
        assert list(pm.var_names) == peaks
        assert (pm.X != ad.X).nnz == 0
        assert pm.X.dtype == np.uint32


@pytest.mark.gpu
def test_gpu_make_peak_matrix_api(tmp_path):
    import snapatac2_gb300 as snap
    g, fr, peaks = _data(n_cells=12, seed=9)
    ad = snap.pp.fragments_to_anndata(fr.indptr, fr.pos, fr.length, g, obs_names=[f"c{i}" for i in range(12)])
    p = tmp_path / "peaks.txt.gz"
    with gzip.open(p, "wt") as fh:
        fh.write("\n".join(peaks) + "\n")
    a = snap.pp.make_peak_matrix(ad, peak_file=str(p))
    ad.uns["peaks"] = {"Peaks": np.array(peaks, dtype=object)}
    b = snap.pp.make_peak_matrix(ad)
    assert list(a.obs_names) == [f"c{i}" for i in range(12)]
    assert (a.X != b.X).nnz == 0 and list(a.var_names) == list(b.var_names)
    with pytest.raises(RuntimeError):
        snap.pp.make_peak_matrix(ad, peak_file=str(p), use_rep="peaks")
    assert snap.pp.make_peak_matrix(ad, inplace=True) is None
    assert (ad.X != b.X).nnz == 0


def test_c_oracle_random_small_cases():
    """Both restatements on 60 random tiny genomes: nested, touching and
    zero-width peaks, repeats, fragments at chromosome edges, zero-length
    fragments, random size filters, every strategy."""
    rng = np.random.default_rng(123)
    strategies = ["insertion", "fragment", "paired-insertion", "single"]
    for trial in range(60):
        sizes = [int(x) for x in rng.integers(50, 400, 3)]
        names = ["chrA", "chrB", "chrC"]
        peaks = []
        for _ in range(int(rng.integers(1, 30))):
            c = int(rng.integers(0, 4))
            s = int(rng.integers(0, 420))
            peaks.append(f"{(names + ['chrZ'])[c]}:{s}-{s + int(rng.integers(0, 120))}")
        peaks += peaks[:3]
        n_cells = int(rng.integers(1, 8))
        counts = rng.integers(0, 25, n_cells)
        indptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        F = int(indptr[-1])
        chrom = rng.integers(0, 3, F)
        csz = np.asarray(sizes)[chrom]
        length = rng.integers(0, 150, F)
        length = np.minimum(length, csz)
        start = (rng.random(F) * (csz - length + 1)).astype(np.int64)
        base = np.concatenate([[0], np.cumsum(sizes)[:-1]])
        pos = (base[chrom] + start).astype(np.uint64)
        strategy = strategies[trial % 4]
        kw = {}
        if trial % 3 == 0:
            kw = dict(min_frag_size=int(rng.integers(0, 60)), max_frag_size=int(rng.integers(60, 160)))
        paired = strategy != "single"
        if not paired:
            kw = {}
        ref = org.region_counts(indptr, pos, length, names, sizes, peaks, strategy=strategy, paired=paired, **kw)
        got = org.region_counts_c(indptr, pos, length, names, sizes, peaks, strategy=strategy, paired=paired, **kw)
        for a, b in zip(got[:3], ref[:3]):
            np.testing.assert_array_equal(a, b, err_msg=f"trial {trial}")
        assert got[3] == ref[3]


def test_oracle_aggregate_x_hand_made():
    var = ["chr1:0-100", "chr1:100-200", "chr2:0-50", "chr9:0-10"]
    X = np.array([[1, 2, 0, 5], [0, 0, 3, 0]], dtype=np.float64)
    peaks = ["chr1:50-150", "chr1:150-160", "chr2:10-20", "chr1:0-1000"]
    ip, ix, dv, names = org.aggregate_x(X, var, ["chr1", "chr2"], peaks)
    assert names == peaks
    assert ip.tolist() == [0, 3, 4]
    assert dict(zip(ix[:3].tolist(), dv[:3].tolist())) == {0: 3.0, 1: 2.0, 3: 3.0}
    assert ix[3:].tolist() == [2] and dv[3:].tolist() == [3.0]


def test_oracle_aggregate_x_of_tiles_is_the_insertion_peak_matrix():
    """Peaks made of whole 500 bp tiles: aggregating the insertion-count tile
    matrix (use_x) gives the insertion-strategy peak matrix of the fragments,
    since every insertion lies in exactly one tile."""
    from oracle import binning as ob
    g, fr, _ = _data(n_cells=12, seed=31)
    names, sizes = [c for c, _ in g], [s for _, s in g]
    ip, ix, dv, ncol = ob.tile_bin(fr.indptr, fr.pos, fr.length, g, bin_size=500,
                                   counting_strategy="insertion", exclude_chroms=[])[:4]
    tiles = [f"{c}:{s}-{min(s + 500, size)}" for c, size in g for s in range(0, size, 500)]
    assert len(tiles) == ncol
    rng = np.random.default_rng(2)
    peaks = []
    for c, size in g:
        for s in np.sort(rng.choice(size // 500 - 4, 40, replace=False)).tolist():
            peaks.append(f"{c}:{s * 500}-{(s + int(rng.integers(1, 4))) * 500}")
    X = sp.csr_matrix((dv.astype(np.float64), ix, ip), shape=(fr.n_cells, ncol))
    agg = org.aggregate_x(X, tiles, names, peaks)
    ref = org.region_counts(fr.indptr, fr.pos, fr.length, names, sizes, peaks, strategy="insertion")
    np.testing.assert_array_equal(agg[0], ref[0])
    np.testing.assert_array_equal(agg[1], ref[1])
    np.testing.assert_array_equal(agg[2], ref[2].astype(np.float64))


# ------------------------------------------------------------ use_x -----
def test_overlap_map_matches_brute_force_and_tile_layout():
    """The host feature -> region map of use_x: every overlapping region of
    every feature (half-open intervals), from parsed names and from a tile
    matrix's layout alike."""
    from snapatac2_gb300._regions import overlap_map
    from snapatac2_gb300.genome import GenomeIndex, TileNames
    rng = np.random.default_rng(0)
    var = [f"chr{c}:{s}-{s + rng.integers(50, 800)}" for c in (1, 2) for s in rng.integers(0, 20000, 200)]
    peaks = ([f"chr{c}:{s}-{s + rng.integers(10, 3000)}" for c in (1, 2, 3) for s in rng.integers(0, 20000, 100)]
             + ["chr1:5-10", "chr1:5-10"])
    fptr, freg, names = overlap_map(var, peaks)
    regs = org.unique_regions(peaks)
    assert names == [f"{c}:{s}-{e}" for c, s, e in regs]
    for j, v in enumerate(var):
        c, s, e = org.parse_region(v)
        want = sorted(k for k, (rc, rs, re_) in enumerate(regs) if rc == c and rs < e and re_ > s)
        assert freg[fptr[j]:fptr[j + 1]].tolist() == want
    g = [("chr1", 12345), ("chr2", 7000), ("chrX", 999)]
    tiles = TileNames(GenomeIndex(g, 500))
    a = overlap_map(tiles, peaks)
    b = overlap_map([tiles[i] for i in range(len(tiles))], peaks)
    for x, y in zip(a[:2], b[:2]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("integer", [True, False])
def test_gpu_use_x_peak_matrix_matches_oracle(integer):
    """make_peak_matrix(use_x=True) on a tile matrix: the aggregation by
    peaks equals the oracle's restatement entry for entry (uint32 sums of
    integer counts, FP64 sums of real values) and, for insertion counts
    over whole-tile peaks, the insertion peak matrix of the fragments."""
    import snapatac2_gb300 as snap
    from oracle import binning as ob
    g, fr, _ = _data(n_cells=40, seed=37)
    names, sizes = [c for c, _ in g], [s for _, s in g]
    ip, ix, dv, ncol = ob.tile_bin(fr.indptr, fr.pos, fr.length, g, bin_size=500,
                                   counting_strategy="insertion", exclude_chroms=[])[:4]
    tiles = [f"{c}:{s}-{min(s + 500, size)}" for c, size in g for s in range(0, size, 500)]
    rng = np.random.default_rng(5)
    peaks = []
    for c, size in g:
        for s in np.sort(rng.choice(size // 500 - 4, 60, replace=False)).tolist():
            peaks.append(f"{c}:{s * 500}-{(s + int(rng.integers(1, 4))) * 500}")
        peaks.append(f"{c}:{int(rng.integers(0, size // 2))}-{size // 2 + 777}")  # long, unaligned
    vals = dv.astype(np.uint32) if integer else dv.astype(np.float64) * rng.uniform(0.5, 2.0, dv.size)
    X = sp.csr_matrix((vals, ix, ip), shape=(fr.n_cells, ncol))
    ad = snap.AnnData(X, var_names=tiles)
    out = snap.pp.make_peak_matrix(ad, use_rep=peaks, use_x=True)
    ref = org.aggregate_x(X, tiles, names, peaks)
    Y = out.X
    np.testing.assert_array_equal(Y.indptr, ref[0])
    np.testing.assert_array_equal(Y.indices, ref[1])
    if integer:
        assert Y.dtype == np.uint32
        np.testing.assert_array_equal(Y.data.astype(np.float64), ref[2])
        aligned = [p for p in peaks if int(p.split(":")[1].split("-")[0]) % 500 == 0
                   and int(p.split("-")[1]) % 500 == 0]
        ins = org.region_counts(fr.indptr, fr.pos, fr.length, names, sizes, aligned, strategy="insertion")
        sub = snap.pp.make_peak_matrix(ad, use_rep=aligned, use_x=True).X
        np.testing.assert_array_equal(sub.indptr, ins[0])
        np.testing.assert_array_equal(sub.data, ins[2])
    else:
        assert Y.dtype == np.float64
        np.testing.assert_allclose(Y.data, ref[2], rtol=1e-15, atol=0)
    assert list(out.var_names) == ref[3]
