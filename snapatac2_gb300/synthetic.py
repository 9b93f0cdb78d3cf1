"""Seeded synthetic inputs for the cell-embedding path.

No public dataset ships with the reference (its fixtures are git-LFS stubs and
``snap.datasets`` downloads over HTTP), so these generators stand in for real
scATAC-seq data with the shapes and value distributions of the workloads:

* a 3.1 Gb genome in 24 chromosomes (``chr1`` .. ``chr22``, ``chrX``, ``chrY``);
* per-cell fragment counts ~ LogNormal(ln median, sigma);
* cells drawn from ``n_clusters`` clusters, each with its own enriched set of
  500 bp genome tiles weighted by Zipf(a); a fragment lands in the cluster's
  enriched set with probability ``p_enriched`` and uniformly elsewhere;
* fragment lengths ~ Geometric with mean 200 bp, clipped so that a fragment
  never runs past the end of its chromosome (the reference panics otherwise,
  ``snapatac2-core/src/genome.rs:397-399``).

The fragment output uses the reference's ``obsm['fragment_paired']`` encoding
(``snapatac2-core/src/preprocessing/import.rs:22-30,161-210``): one row per
cell, column = global 0-based base index of the fragment start, value =
fragment length; each row sorted by (start, length).

``binary_csr`` draws the cell-by-feature matrices of the large workloads
directly: binary CSR over ``n_features`` columns with the same cluster/Zipf
model, int64 ``indptr`` and int32 sorted, de-duplicated column indices.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def make_genome(total: int = 3_100_000_000, n_chrom: int = 24) -> list[tuple[str, int]]:
    """Chromosome names and sizes summing to ``total``.

    Sizes decrease linearly from chr1 to chrX; chrY is a quarter of chr1.
    """
    names = [f"chr{i}" for i in range(1, n_chrom - 1)] + ["chrX", "chrY"][: max(0, min(2, n_chrom))]
    names = names[:n_chrom]
    w = np.array([1.0 - 0.035 * i for i in range(n_chrom)], dtype=np.float64)
    if n_chrom >= 2:
        w[-1] = 0.25
    sizes = np.floor(w / w.sum() * total).astype(np.int64)
    sizes[0] += total - int(sizes.sum())
    return [(n, int(s)) for n, s in zip(names, sizes)]


@dataclass
class FragmentMatrix:
    """Paired-end fragments in the ``fragment_paired`` encoding."""

    indptr: np.ndarray   # int64 [n_cells + 1]
    pos: np.ndarray      # uint64 [F]  global 0-based base index of the start
    length: np.ndarray   # uint32 [F]  fragment length in bp
    clusters: np.ndarray  # int32 [n_cells] generating cluster of each cell

    @property
    def n_cells(self) -> int:
        return int(self.indptr.shape[0] - 1)

    @property
    def n_fragments(self) -> int:
        return int(self.pos.shape[0])


def _zipf_cdf(n: int, a: float) -> np.ndarray:
    w = np.arange(1, n + 1, dtype=np.float64) ** (-a)
    c = np.cumsum(w)
    return c / c[-1]


def make_fragments(
    n_cells: int,
    genome: list[tuple[str, int]] | None = None,
    *,
    n_clusters: int = 8,
    enriched_bins: int = 50_000,
    zipf_a: float = 1.1,
    p_enriched: float = 0.7,
    median_frags: float = 10_000.0,
    sigma: float = 0.6,
    mean_len: float = 200.0,
    bin_size: int = 500,
    seed: int = 0,
) -> FragmentMatrix:
    """Draw ``n_cells`` cells of paired-end fragments (see module docstring)."""
    if genome is None:
        genome = make_genome()
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.array([s for _, s in genome], dtype=np.int64)
    base_end = np.cumsum(sizes)
    base_start = base_end - sizes
    gsize = int(base_end[-1])
    nb = -(-sizes // bin_size)
    bin_end = np.cumsum(nb)
    bin_start = bin_end - nb
    total_bins = int(bin_end[-1])
    n_enr = min(enriched_bins, total_bins)

    counts = np.maximum(1, np.rint(rng.lognormal(np.log(median_frags), sigma, n_cells))).astype(np.int64)
    clusters = rng.integers(0, n_clusters, n_cells).astype(np.int32)
    enr = np.stack([rng.choice(total_bins, n_enr, replace=False) for _ in range(n_clusters)])
    cdf = _zipf_cdf(n_enr, zipf_a)

    F = int(counts.sum())
    cell = np.repeat(np.arange(n_cells, dtype=np.int64), counts)
    length = rng.geometric(1.0 / mean_len, F).astype(np.int64)
    is_enr = rng.random(F) < p_enriched
    gpos = np.empty(F, dtype=np.int64)
    # enriched draws: a Zipf-ranked tile of the cell's cluster, uniform inside it
    ne = int(is_enr.sum())
    rank = np.searchsorted(cdf, rng.random(ne), side="right").clip(0, n_enr - 1)
    gbin = enr[clusters[cell[is_enr]], rank]
    chrom = np.searchsorted(bin_end, gbin, side="right")
    off = (gbin - bin_start[chrom]) * bin_size + rng.integers(0, bin_size, ne)
    off = np.minimum(off, sizes[chrom] - 1)
    gpos[is_enr] = base_start[chrom] + off
    # background draws: uniform over the genome
    nbk = F - ne
    gpos[~is_enr] = rng.integers(0, gsize, nbk)
    # clip so that start + length <= chromosome length
    chrom = np.searchsorted(base_end, gpos, side="right")
    off = gpos - base_start[chrom]
    csz = sizes[chrom]
    length = np.minimum(length, csz)
    off = np.minimum(off, csz - length)
    gpos = base_start[chrom] + off

    # sort each row by (start, length)
    order = np.argsort(length, kind="stable")
    key = (cell[order] << np.int64(34)) | gpos[order]
    order = order[np.argsort(key, kind="stable")]
    indptr = np.zeros(n_cells + 1, dtype=np.int64)
    np.cumsum(counts, out=indptr[1:])
    return FragmentMatrix(
        indptr=indptr,
        pos=gpos[order].astype(np.uint64),
        length=length[order].astype(np.uint32),
        clusters=clusters,
    )


@dataclass
class BinaryCSR:
    """Binary (implicit 1.0) cell-by-feature CSR matrix."""

    indptr: np.ndarray   # int64 [n + 1]
    indices: np.ndarray  # int32 [nnz], sorted and unique within each row
    n_cols: int
    clusters: np.ndarray  # int32 [n]

    @property
    def shape(self) -> tuple[int, int]:
        return (int(self.indptr.shape[0] - 1), int(self.n_cols))

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])


def _oversample_factor(n_features, nnz_per_cell, n_enr, cdf, p_enriched, rng) -> float:
    """Draws per wanted unique feature, from a 200-row pilot (collisions of
    the Zipf-weighted enriched draws make unique < draws)."""
    factor = 1.0
    enr = rng.choice(n_features, n_enr, replace=False)
    for _ in range(3):
        d = int(round(nnz_per_cell * factor))
        uniq = []
        for _r in range(200):
            is_e = rng.random(d) < p_enriched
            col = rng.integers(0, n_features, d)
            ne = int(is_e.sum())
            col[is_e] = enr[np.searchsorted(cdf, rng.random(ne), side="right").clip(0, n_enr - 1)]
            uniq.append(np.unique(col).size)
        factor *= nnz_per_cell / max(float(np.mean(uniq)), 1.0)
    return factor


def binary_csr(
    n_cells: int,
    n_features: int = 500_000,
    *,
    nnz_per_cell: float = 4_000.0,
    sigma: float = 0.3,
    n_clusters: int = 8,
    enriched: int = 50_000,
    zipf_a: float = 1.1,
    p_enriched: float = 0.7,
    seed: int = 0,
    chunk_cells: int = 20_000,
) -> BinaryCSR:
    """Binary CSR with ~``nnz_per_cell`` distinct features in the median row
    (the row targets are lognormal, so the mean row holds about
    exp(sigma² / 2) times as many: ~4,140 at 4,000 and sigma 0.3).

    Per row, the target ``t`` ~ LogNormal(ln(nnz_per_cell), sigma); ``t * f``
    features are drawn (``p_enriched`` of them Zipf-ranked from the cluster's
    enriched set, the rest uniform) and de-duplicated, with the oversampling
    factor ``f`` set from a pilot (at the median target) so that a row of
    target ``nnz_per_cell`` holds about that many distinct features.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    n_enr = min(enriched, n_features)
    cdf = _zipf_cdf(n_enr, zipf_a)
    factor = _oversample_factor(n_features, nnz_per_cell, n_enr, cdf, p_enriched,
                                np.random.Generator(np.random.PCG64(seed + 1)))
    draws = np.maximum(1, np.rint(factor * rng.lognormal(np.log(nnz_per_cell), sigma, n_cells))).astype(np.int64)
    draws = np.minimum(draws, 4 * n_features)
    clusters = rng.integers(0, n_clusters, n_cells).astype(np.int32)
    enr = np.stack([rng.choice(n_features, n_enr, replace=False) for _ in range(n_clusters)]).astype(np.int64)
    rows_idx = []
    row_nnz = np.zeros(n_cells, dtype=np.int64)
    for c0 in range(0, n_cells, chunk_cells):
        c1 = min(n_cells, c0 + chunk_cells)
        d = draws[c0:c1]
        D = int(d.sum())
        cell = np.repeat(np.arange(c0, c1, dtype=np.int64), d)
        is_enr = rng.random(D) < p_enriched
        col = rng.integers(0, n_features, D)
        ne = int(is_enr.sum())
        rank = np.searchsorted(cdf, rng.random(ne), side="right").clip(0, n_enr - 1)
        col[is_enr] = enr[clusters[cell[is_enr]], rank]
        key = np.unique((cell << np.int64(32)) | col)
        r = key >> np.int64(32)
        rows_idx.append((key & np.int64(0xFFFFFFFF)).astype(np.int32))
        row_nnz[c0:c1] = np.bincount(r - c0, minlength=c1 - c0)
    indptr = np.zeros(n_cells + 1, dtype=np.int64)
    np.cumsum(row_nnz, out=indptr[1:])
    return BinaryCSR(indptr=indptr, indices=np.concatenate(rows_idx), n_cols=n_features, clusters=clusters)


def binary_csr_device(
    n_cells: int,
    n_features: int = 500_000,
    *,
    nnz_per_cell: float = 4_000.0,
    sigma: float = 0.3,
    n_clusters: int = 8,
    enriched: int = 50_000,
    zipf_a: float = 1.1,
    p_enriched: float = 0.7,
    seed: int = 0,
    device=None,
    chunk_cells: int = 25_000,
):
    """Same model as ``binary_csr``, drawn on the GPU with torch (fast input
    generation for the large workloads; a different random stream than the
    NumPy generator).  Returns (indptr int64, indices int32) CUDA tensors.
    """
    import torch
    dev = torch.device(device) if device is not None else torch.device("cuda")
    rng = np.random.Generator(np.random.PCG64(seed))
    n_enr = min(enriched, n_features)
    cdf_np = _zipf_cdf(n_enr, zipf_a)
    factor = _oversample_factor(n_features, nnz_per_cell, n_enr, cdf_np, p_enriched,
                                np.random.Generator(np.random.PCG64(seed + 1)))
    draws = np.maximum(1, np.rint(factor * rng.lognormal(np.log(nnz_per_cell), sigma, n_cells))).astype(np.int64)
    draws = np.minimum(draws, 4 * n_features)
    clusters = rng.integers(0, n_clusters, n_cells).astype(np.int64)
    enr = np.stack([rng.choice(n_features, n_enr, replace=False) for _ in range(n_clusters)]).astype(np.int64)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    cdf = torch.from_numpy(cdf_np).to(dev)
    enr_t = torch.from_numpy(enr).to(dev)
    cl_t = torch.from_numpy(clusters).to(dev)
    row_nnz = torch.zeros(n_cells, dtype=torch.int64, device=dev)
    parts = []
    for c0 in range(0, n_cells, chunk_cells):
        c1 = min(n_cells, c0 + chunk_cells)
        d = torch.from_numpy(draws[c0:c1]).to(dev)
        D = int(draws[c0:c1].sum())
        cell = torch.repeat_interleave(torch.arange(c0, c1, device=dev), d)
        is_enr = torch.rand(D, generator=g, device=dev) < p_enriched
        col = torch.randint(0, n_features, (D,), generator=g, device=dev)
        u = torch.rand(D, generator=g, device=dev, dtype=torch.float64)
        rank = torch.searchsorted(cdf, u, right=True).clamp_(0, n_enr - 1)
        ecol = enr_t[cl_t[cell], rank]
        col = torch.where(is_enr, ecol, col)
        key = torch.unique(cell * n_features + col)  # sorted, de-duplicated
        r = key // n_features
        parts.append((key - r * n_features).to(torch.int32))
        row_nnz[c0:c1] = torch.bincount(r - c0, minlength=c1 - c0)
        del cell, is_enr, col, u, rank, ecol, key, r
    indptr = torch.zeros(n_cells + 1, dtype=torch.int64, device=dev)
    torch.cumsum(row_nnz, 0, out=indptr[1:])
    return indptr, torch.cat(parts), clusters


# ---- fragment files ----------------------------------------------------------

MITO_NAME, MITO_SIZE = "chrM", 16_569


def cell_barcodes(n_cells: int, seed: int = 0) -> list[str]:
    """Distinct 10x-style barcodes: 16 random bases + "-1"."""
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    out: list[str] = []
    seen: set = set()
    while len(out) < n_cells:
        for row in rng.integers(0, 4, (n_cells - len(out), 16)):
            b = "".join("ACGT"[i] for i in row) + "-1"
            if b not in seen:
                seen.add(b)
                out.append(b)
    return out


def fragment_text(frags: FragmentMatrix, genome: list[tuple[str, int]], *, seed: int = 0,
                  order: str = "position", dup_frac: float = 0.15, mito_frac: float = 0.02,
                  single_end: bool = False, header: bool = True, device=None):
    """A fragment file (uint8 torch tensor of its text) for ``frags``.

    Lines ``chrom\\tstart\\tend\\tbarcode\\tcount[\\tstrand]\\n`` in the format
    of ``snapatac2-core/src/preprocessing/qc.rs:303-348``; chromosome-local
    0-based starts, ``end = start + length``.  ``count`` is 1, or 2..5 for a
    ``dup_frac`` share of the lines (PCR duplicates); about ``mito_frac`` of
    each cell's lines are added on ``chrM`` (16,569 bp).  ``order``:
    "position" (chromosome, start: how 10x pipelines write them),
    "barcode" (barcode bytes, then position) or "shuffle".  Built with torch
    on ``device`` (fixed-width rows, then the padding dropped), so that large
    files can be drawn on the GPU.
    """
    import torch
    dev = torch.device(device) if device is not None else torch.device("cpu")
    g = torch.Generator(device="cpu").manual_seed(seed + 104729)
    names = [n for n, _ in genome] + [MITO_NAME]
    sizes = np.array([s for _, s in genome] + [MITO_SIZE], dtype=np.int64)
    base_end = np.cumsum(sizes[:-1])
    n = frags.n_cells
    counts = np.diff(frags.indptr)
    cell = torch.repeat_interleave(torch.arange(n), torch.from_numpy(counts)).to(dev)
    gpos = torch.from_numpy(frags.pos.astype(np.int64)).to(dev)
    length = torch.from_numpy(frags.length.astype(np.int64)).to(dev)
    bend = torch.from_numpy(base_end).to(dev)
    chrom = torch.searchsorted(bend, gpos, right=True)
    start = gpos - torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), bend])[chrom]
    # mitochondrial fragments
    n_m = np.random.Generator(np.random.PCG64(seed + 31)).poisson(mito_frac * np.maximum(counts, 1))
    if n_m.sum():
        mcell = torch.repeat_interleave(torch.arange(n), torch.from_numpy(n_m)).to(dev)
        mlen = torch.randint(50, 500, (int(n_m.sum()),), generator=g).to(dev)
        mstart = (torch.rand(int(n_m.sum()), generator=g).to(dev) * (MITO_SIZE - mlen)).long()
        cell = torch.cat([cell, mcell])
        chrom = torch.cat([chrom, torch.full_like(mcell, len(names) - 1)])
        start = torch.cat([start, mstart])
        length = torch.cat([length, mlen])
    F = int(cell.numel())
    cnt = torch.ones(F, dtype=torch.int64, device=dev)
    dup = torch.rand(F, generator=g).to(dev) < dup_frac
    cnt[dup] = torch.randint(2, 6, (int(dup.sum()),), generator=g).to(dev)
    strand = (torch.rand(F, generator=g).to(dev) < 0.5) if single_end else None
    bcs = cell_barcodes(n, seed)
    if order == "position":
        key = (chrom << 40) | (start << 8) | torch.clamp(length, max=255)
        perm = torch.sort(key, stable=True).indices
    elif order == "barcode":
        rank = np.empty(n, dtype=np.int64)
        rank[np.argsort(np.array([b.encode() for b in bcs], dtype=object), kind="stable")] = np.arange(n)
        r = torch.from_numpy(rank).to(dev)[cell]
        key = (chrom << 40) | (start << 8) | torch.clamp(length, max=255)
        perm = torch.sort(key, stable=True).indices
        perm = perm[torch.sort(r[perm], stable=True).indices]
    elif order == "shuffle":
        perm = torch.randperm(F, generator=g).to(dev)
    else:
        raise ValueError(order)
    cell, chrom, start, length, cnt = cell[perm], chrom[perm], start[perm], length[perm], cnt[perm]
    end = start + length
    if strand is not None:
        strand = strand[perm]

    def table(strings):
        w = max(len(s) for s in strings)
        t = np.zeros((len(strings), w), dtype=np.uint8)
        ln = np.zeros(len(strings), dtype=np.int64)
        for i, s in enumerate(strings):
            b = s.encode()
            t[i, :len(b)] = np.frombuffer(b, dtype=np.uint8)
            ln[i] = len(b)
        return torch.from_numpy(t).to(dev), torch.from_numpy(ln).to(dev)

    def digits(v, w=20):
        nd = torch.ones_like(v)
        p = torch.full_like(v, 10)
        for _ in range(w - 1):
            nd += (v >= p).long()
            p = p * 10
        d = torch.zeros((v.numel(), w), dtype=torch.uint8, device=dev)
        x = v.clone()
        for k in range(w - 1, -1, -1):
            d[:, k] = (x % 10 + 48).to(torch.uint8)
            x = x // 10
        col = torch.arange(w, device=dev)
        return d, col.unsqueeze(0) >= (w - nd).unsqueeze(1)

    ct, cl = table(names)
    bt, bl = table(bcs)
    parts, masks = [], []
    tab = torch.full((F, 1), 9, dtype=torch.uint8, device=dev)
    ones = torch.ones((F, 1), dtype=torch.bool, device=dev)
    parts.append(ct[chrom]); masks.append(torch.arange(ct.shape[1], device=dev).unsqueeze(0) < cl[chrom].unsqueeze(1))
    for v, w in ((start, 11), (end, 11)):
        parts += [tab]; masks += [ones]
        d, m = digits(v, w)
        parts.append(d); masks.append(m)
    parts += [tab]; masks += [ones]
    parts.append(bt[cell]); masks.append(torch.arange(bt.shape[1], device=dev).unsqueeze(0) < bl[cell].unsqueeze(1))
    parts += [tab]; masks += [ones]
    d, m = digits(cnt, 2)
    parts.append(d); masks.append(m)
    if strand is not None:
        parts += [tab]; masks += [ones]
        parts.append(torch.where(strand, 45, 43).to(torch.uint8).unsqueeze(1)); masks.append(ones)
    parts.append(torch.full((F, 1), 10, dtype=torch.uint8, device=dev)); masks.append(ones)
    body = torch.cat(parts, 1)[torch.cat(masks, 1)]
    if header:
        h = torch.from_numpy(np.frombuffer(b"# synthetic fragments\n# columns: chrom start end barcode count\n",
                                           dtype=np.uint8).copy()).to(dev)
        body = torch.cat([h, body])
    return body


def fragment_genome(genome: list[tuple[str, int]]) -> dict:
    """chrom_sizes for importing ``fragment_text`` output (with chrM)."""
    d = dict(genome)
    d[MITO_NAME] = MITO_SIZE
    return d
