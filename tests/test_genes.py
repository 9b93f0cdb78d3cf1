"""snap.pp.make_gene_matrix: the oracle's annotation reading and promoter
regions on a hand-made file (CPU), and the GPU gene / transcript matrices
against the oracle on a synthetic annotation (GPU)."""
import numpy as np
import pytest

from oracle import genes as ogn

GTF = """#!genome-build test
chr1\tsrc\tgene\t101\t500\t.\t+\t.\tgene_id "G1"; gene_name "A";
chr1\tsrc\ttranscript\t101\t500\t.\t+\t.\tgene_id "G1"; transcript_id "T1"; gene_name "A"; transcript_name "A-1";
chr1\tsrc\ttranscript\t3001\t3500\t.\t-\t.\tgene_id "G2"; transcript_id "T2"; gene_name "B";
chr1\tsrc\texon\t3001\t3100\t.\t-\t.\tgene_id "G2"; transcript_id "T2"; gene_name "B";
"""


def test_oracle_transcripts_and_promoters(tmp_path):
    p = tmp_path / "a.gtf"
    p.write_text(GTF)
    ts = ogn.read_transcripts(p)
    assert [t["transcript_id"] for t in ts] == ["T1", "T2"]
    assert ts[0]["transcript_name"] == "A-1" and ts[1]["transcript_name"] is None
    # "+": [left0 - 2000 (saturating), right0); "-": [left0, right0 + 2000)
    assert ogn.promoter_regions(ts) == [("chr1", 0, 499), ("chr1", 3000, 5499)]
    assert ogn.promoter_regions(ts, 10, 5, False) == [("chr1", 90, 105), ("chr1", 3494, 3509)]
    g = tmp_path / "a.gff3.gz"
    import gzip
    with gzip.open(g, "wt") as fh:
        fh.write("##gff-version 3\nchr1\tsrc\ttranscript\t11\t20\t.\t-\t.\t"
                 "ID=T9;transcript_id=T9;gene_name=C%3BD;gene_id=G9\n")
    t = ogn.read_transcripts(g)[0]
    assert t["gene_name"] == "C;D" and t["strand"] == "-"


def _annotation(g, rng, n_genes=150):
    lines = []
    for i in range(n_genes):
        c, size = g[rng.integers(0, len(g))]
        for j in range(int(rng.integers(1, 4))):
            left = int(rng.integers(1, size - 60_000))
            right = left + int(rng.integers(200, 50_000))
            strand = "+" if rng.random() < 0.5 else "-"
            lines.append(f'{c}\tsim\ttranscript\t{left}\t{right}\t.\t{strand}\t.\t'
                         f'gene_id "G{i}"; transcript_id "T{i}.{j}"; gene_name "N{i % 120}";')
    lines.append(lines[5].replace('transcript_id "', 'transcript_id "dup'))   # same promoter region twice
    lines.append('chrUn\tsim\ttranscript\t10\t900\t.\t+\t.\tgene_id "Gu"; transcript_id "Tu"; gene_name "U";')
    return "\n".join(lines) + "\n"


@pytest.mark.gpu
@pytest.mark.parametrize("id_type,kw", [("gene", {}), ("transcript", {}),
                                        ("gene", dict(upstream=1000, downstream=1000, include_gene_body=False)),
                                        ("gene", dict(counting_strategy="fragment")),
                                        ("gene", dict(counting_strategy="insertion", max_frag_size=250))])
def test_gpu_gene_matrix_matches_oracle(tmp_path, id_type, kw):
    import snapatac2_gb300 as snap
    from snapatac2_gb300 import synthetic as S
    g = S.make_genome(total=20_000_000, n_chrom=6)
    fr = S.make_fragments(25, g, median_frags=500, enriched_bins=800, seed=4)
    rng = np.random.default_rng(len(kw) + (id_type == "gene"))
    p = tmp_path / "anno.gtf"
    p.write_text(_annotation(g, rng))
    ad = snap.pp.fragments_to_anndata(fr.indptr, fr.pos, fr.length, g)
    got = snap.pp.make_gene_matrix(ad, str(p), id_type=id_type, **kw)
    okw = dict(kw)
    strategy = okw.pop("counting_strategy", "paired-insertion")
    ref = ogn.gene_matrix(fr.indptr, fr.pos, fr.length, [c for c, _ in g], [s for _, s in g],
                          ogn.read_transcripts(p), id_type=id_type, strategy=strategy, **okw)
    assert list(got.var_names) == ref[3]
    X = got.X.tocsr()
    np.testing.assert_array_equal(X.indptr, ref[0])
    np.testing.assert_array_equal(X.indices, ref[1])
    np.testing.assert_array_equal(X.data, ref[2])
    assert X.dtype == np.uint32


@pytest.mark.gpu
@pytest.mark.parametrize("id_type", ["gene", "transcript"])
def test_gpu_use_x_gene_matrix_matches_oracle(tmp_path, id_type):
    """make_gene_matrix(use_x=True): the tile matrix aggregated by the
    transcripts' promoter regions (transcript level) and its maximum over
    each gene's transcripts (gene level), against the oracle."""
    import snapatac2_gb300 as snap
    from oracle import binning as ob
    from snapatac2_gb300 import synthetic as S
    g = S.make_genome(total=20_000_000, n_chrom=6)
    fr = S.make_fragments(25, g, median_frags=500, enriched_bins=800, seed=8)
    p = tmp_path / "anno.gtf"
    p.write_text(_annotation(g, np.random.default_rng(3)))
    ad = snap.pp.fragments_to_anndata(fr.indptr, fr.pos, fr.length, g)
    snap.pp.add_tile_matrix(ad, exclude_chroms=None)
    got = snap.pp.make_gene_matrix(ad, str(p), id_type=id_type, use_x=True)
    tiles = [ad.var_names[i] for i in range(ad.n_vars)]
    ref = ogn.gene_matrix_from_x(ad.X, tiles, [c for c, _ in g], ogn.read_transcripts(p), id_type=id_type)
    assert list(got.var_names) == ref[3]
    X = got.X.tocsr()
    np.testing.assert_array_equal(X.indptr, ref[0])
    np.testing.assert_array_equal(X.indices, ref[1])
    np.testing.assert_array_equal(X.data, ref[2].astype(np.uint32))
