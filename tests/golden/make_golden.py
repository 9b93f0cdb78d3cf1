"""Generate the committed golden fixtures of ``tests/golden``.

Run from the repository root:  python tests/golden/make_golden.py

* ``genome_index.json``  known-answer vectors of the reference's
  ``GenomeBaseIndex`` tests, parsed from the reference source
  (``snapatac2-core/src/genome.rs:496-597``, ``test_index1``/``test_index2``).
* ``tile_bin.npz``        a small synthetic fragment set and the oracle's tile
  matrices (``gen_mat_pair`` restated in ``oracle/tile_bin.c``, cross-checked
  against the NumPy restatement) for every counting strategy.
* ``spectral.npz``        a small binary cell x feature matrix and the output of
  the reference's spectral arithmetic (IDF, L2 row norm, degree, SciPy ARPACK
  ``eigsh``) as restated in ``oracle/spectral.py``.
* ``knn.npz``             a small embedding and its exact kNN graph
  (``oracle/knn.c``).
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

# root of the SnapATAC2 source tree the fixtures are cut from: the first
# command-line argument, else $SNAPATAC2_REFERENCE
REFERENCE_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SNAPATAC2_REFERENCE", "")
if not REFERENCE_ROOT:
    sys.exit("usage: python " + os.path.basename(__file__) + " <SnapATAC2 source root> (or set SNAPATAC2_REFERENCE)")

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.join(ROOT, "tests", "golden")
REF_GENOME_RS = os.path.join(REFERENCE_ROOT, "snapatac2-core/src/genome.rs")


def genome_goldens() -> dict:
    src = open(REF_GENOME_RS).read()
    t1 = src[src.index("fn test_index1()"):src.index("fn test_index2()")]
    t2 = src[src.index("fn test_index2()"):src.index("fn test_read_transcript()")]
    chrom = [(n, int(s)) for n, s in re.findall(r'\("(\w+)"\.to_owned\(\),\s*(\d+)\)', t1)]
    ranges = [(c, int(a), int(b)) for c, a, b in re.findall(r'get_range\("(\w+)"\)\.unwrap\(\),\s*(\d+)\.\.(\d+)', t1)]
    # blocks of (index, "chr:start-end") checked after with_step(s)
    blocks = re.split(r"index = index\.with_step\((\d+)\);", t1)
    region = []
    steps = [1] + [int(x) for x in blocks[1::2]]
    for step, body in zip(steps, blocks[0::2]):
        for i, c, s, e in re.findall(r'\((\d+),\s*"(\w+):(\d+)-(\d+)"\)', body):
            region.append({"step": step, "index": int(i), "chrom": c, "start": int(s), "end": int(e)})
    coarse = []
    parts = t2.split("let index2 = index.with_step(2);")
    for i, j in re.findall(r"\((\d+),\s*(\d+)\)", parts[0]):
        coarse.append({"step": 1, "base": int(i), "index": int(j)})
    for i, j in re.findall(r"\((\d+),\s*(\d+)\)", parts[1]):
        coarse.append({"step": 2, "base": int(i), "index": int(j)})
    return {"source": "snapatac2-core/src/genome.rs:496-597", "chrom_sizes": chrom, "ranges": ranges,
            "regions": region, "coarsed": coarse}


def tile_fixture():
    from oracle import binning
    from snapatac2_gb300 import synthetic as syn
    genome = syn.make_genome(total=20_000_000, n_chrom=5)  # chr1..chr3, chrX, chrY
    fm = syn.make_fragments(24, genome, enriched_bins=2000, median_frags=800, sigma=0.6, seed=7)
    out = {"chrom_names": np.array([n for n, _ in genome]), "chrom_sizes": np.array([s for _, s in genome]),
           "indptr": fm.indptr, "pos": fm.pos, "length": fm.length}
    cases = [("paired-insertion", 500, ["chrY"], None, None), ("insertion", 500, ["chrY"], None, None),
             ("fragment", 500, ["chrY"], None, None), ("single", 500, [], None, None),
             ("paired-insertion", 1000, ["chr2", "chrY"], 50, 400), ("insertion", 137, [], 1, 10_000)]
    for i, (st, b, ex, mn, mx) in enumerate(cases):
        kw = dict(bin_size=b, exclude_chroms=ex, counting_strategy=st, min_frag_size=mn, max_frag_size=mx)
        a = binning.tile_bin(fm.indptr, fm.pos, fm.length, genome, **kw)
        c = binning.tile_bin_numpy(fm.indptr, fm.pos, fm.length, genome, **kw)
        assert all(np.array_equal(x, y) for x, y in zip(a[:3], c[:3])) and a[3] == c[3]
        out[f"case{i}_spec"] = np.array(json.dumps(kw))
        out[f"case{i}_indptr"], out[f"case{i}_idx"], out[f"case{i}_cnt"] = a[0], a[1], a[2]
        out[f"case{i}_ncols"] = np.array(a[3])
    np.savez_compressed(os.path.join(OUT, "tile_bin.npz"), **out)


def spectral_fixture():
    import scipy.sparse as sp
    from oracle import spectral as osp
    from snapatac2_gb300 import synthetic as syn
    B = syn.binary_csr(400, 3000, nnz_per_cell=150, n_clusters=4, enriched=600, seed=11)
    X = sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape)
    evals, evecs = osp.spectral(X, n_comps=30, random_state=0)
    raw_evals, raw_evecs = osp.eigen(*osp.operator(X), 30, 0)
    np.savez_compressed(os.path.join(OUT, "spectral.npz"), indptr=B.indptr, indices=B.indices,
                        shape=np.array(B.shape), evals=evals, evecs=evecs, raw_evals=raw_evals,
                        raw_evecs=raw_evecs)


def knn_fixture():
    from oracle import knn as oknn
    rng = np.random.default_rng(5)
    X = rng.standard_normal((300, 12))
    X[7] = X[3]  # an exact duplicate point: distance 0 to another index
    nbr, dist = oknn.knn_arrays(X, 10)
    np.savez_compressed(os.path.join(OUT, "knn.npz"), X=X, k=np.array(10), nbr=nbr, dist=dist)


if __name__ == "__main__":
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(OUT, "genome_index.json"), "w") as f:
        json.dump(genome_goldens(), f, indent=1)
    tile_fixture()
    spectral_fixture()
    knn_fixture()
    print("wrote", sorted(os.listdir(OUT)))
