"""Host-side logic of the gene / peak matrices and the import (CPU): the
product's annotation reader and promoter regions against the oracle's, region
strings, the per-chromosome region index handed to the region counter, the
genome order of the import, and the column index check of input matrices."""
import gzip

import numpy as np
import pytest
import torch

from oracle import genes as ogn

GTF = """#!genome-build test
chr1\tsrc\tgene\t101\t500\t.\t+\t.\tgene_id "G1"; gene_name "A";
chr1\tsrc\ttranscript\t101\t500\t.\t+\t.\tgene_id "G1"; transcript_id "T1"; gene_name "A"; transcript_name "A-1";
chr2\tsrc\ttranscript\t3001\t3500\t.\t-\t.\tgene_id "G2"; transcript_id "T2"; gene_name "B";
chr2\tsrc\ttranscript\t1\t40\t.\t+\t.\tgene_id "G3"; transcript_id "T3"; gene_name "C"; gene_name "dup";
chr1\tsrc\texon\t3001\t3100\t.\t-\t.\tgene_id "G2"; transcript_id "T2"; gene_name "B";
"""

GFF = ("##gff-version 3\n"
       "chr1\tsrc\ttranscript\t11\t20\t.\t-\t.\tID=T9;transcript_id=T9;gene_name=C%3BD;gene_id=G9\n"
       "chr3\tsrc\ttranscript\t500\t900\t.\t+\t.\ttranscript_id=T8;gene_name=E;gene_id=G8;transcript_name=E-1\n")


def _files(tmp_path):
    a = tmp_path / "a.gtf"
    a.write_text(GTF)
    b = tmp_path / "b.gff3.gz"
    with gzip.open(b, "wt") as fh:
        fh.write(GFF)
    c = tmp_path / "c.annotation"          # no known extension: decided by the first record
    c.write_text(GFF)
    return [a, b, c]


def test_read_transcripts_matches_oracle(tmp_path):
    from snapatac2_gb300._genes import read_transcripts
    for p in _files(tmp_path):
        got, ref = read_transcripts(p), ogn.read_transcripts(p)
        assert len(got) == len(ref) > 0
        for g, r in zip(got, ref):
            for key in ("chrom", "left", "right", "strand", "transcript_id", "gene_name", "gene_id",
                        "transcript_name"):
                assert g[key] == r[key], (p, key)
    t = read_transcripts(_files(tmp_path)[1])
    assert t[0]["gene_name"] == "C;D" and t[1]["transcript_name"] == "E-1"
    assert read_transcripts(tmp_path / "a.gtf")[2]["gene_name"] == "C"   # first occurrence of a repeated key


def test_read_transcripts_errors(tmp_path):
    from snapatac2_gb300._genes import read_transcripts
    p = tmp_path / "bad.gtf"
    p.write_text('chr1\tsrc\ttranscript\t1\t5\t.\t+\t.\tgene_id "G"; gene_name "A";\n')
    with pytest.raises(ValueError, match="transcript_id"):
        read_transcripts(p)
    p.write_text("chr1\tsrc\ttranscript\t1\t5\n")
    with pytest.raises(ValueError, match="parse"):
        read_transcripts(p)


@pytest.mark.parametrize("up,down,body", [(2000, 0, True), (10, 5, False), (0, 0, True), (5000, 300, False)])
def test_promoter_regions_match_oracle(tmp_path, up, down, body):
    from snapatac2_gb300._genes import promoter_regions, read_transcripts
    ts = read_transcripts(_files(tmp_path)[0]) + read_transcripts(_files(tmp_path)[1])
    assert promoter_regions(ts, up, down, body) == ogn.promoter_regions(ts, up, down, body)
    with pytest.raises(ValueError, match="strand"):
        promoter_regions([dict(ts[0], strand=".")], up, down, body)


def test_parse_region():
    from snapatac2_gb300._regions import parse_region
    assert parse_region("chr1:100-200") == ("chr1", 100, 200)
    assert parse_region(" chrUn:KI270:5-9\n") == ("chrUn:KI270", 5, 9)
    assert parse_region("HLA-A:0-10") == ("HLA-A", 0, 10)
    with pytest.raises(ValueError):
        parse_region("chr1-100-200")


def test_build_regions_index():
    """Repeats dropped (first kept), regions grouped by chromosome in genome
    order and sorted by start, running maximum of the ends, feature ids; a
    region on a chromosome outside the genome stays a feature with no entry."""
    from snapatac2_gb300._regions import build_regions
    peaks = ["chr2:50-90", "chr1:300-400", "chr1:10-1000", "chr1:300-400", ("chr1", 20, 30), "chrZ:1-5",
             "chr2:5-10", "chr1:500-600"]
    rs = build_regions(peaks, ["chr1", "chr2", "chr3"], torch.device("cpu"))
    assert rs.names == ["chr2:50-90", "chr1:300-400", "chr1:10-1000", "chr1:20-30", "chrZ:1-5", "chr2:5-10",
                        "chr1:500-600"]
    assert rs.ptr.tolist() == [0, 4, 6, 6]
    assert rs.start.tolist() == [10, 20, 300, 500, 5, 50]
    assert rs.end.tolist() == [1000, 30, 400, 600, 10, 90]
    assert rs.maxend.tolist() == [1000, 1000, 1000, 1000, 10, 90]
    assert rs.rid.tolist() == [2, 3, 1, 6, 5, 0]
    assert rs.rid.dtype == torch.int32 and rs.start.dtype == torch.int64
    empty = build_regions([], ["chr1"], torch.device("cpu"))
    assert empty.names == [] and empty.ptr.tolist() == [0, 0] and empty.start.numel() == 0


def test_sorted_chrom_sizes_byte_order():
    from snapatac2_gb300._import import sorted_chrom_sizes
    from snapatac2_gb300.genome import ChromSizes
    d = {"chrX": 5, "chr10": 3, "chr2": 4, "chrM": 1, "chr1": 9, "Chr3": 2}
    want = ["Chr3", "chr1", "chr10", "chr2", "chrM", "chrX"]
    assert sorted_chrom_sizes(d).names == want
    assert sorted_chrom_sizes(list(d.items())).names == want
    cs = sorted_chrom_sizes(type("G", (), {"chrom_sizes": d})())
    assert cs.names == want and cs.sizes == [d[k] for k in want]
    with pytest.raises(ValueError):
        ChromSizes([("a", 1), ("a", 2)])
    assert np.asarray(sorted_chrom_sizes(d).sizes).sum() == sum(d.values())


def test_column_index_check():
    """Matrices with a column index outside [0, m) are refused before any
    kernel looks the column up (SciPy does not check bounds by default)."""
    from snapatac2_gb300._binning import DeviceCSR
    from snapatac2_gb300._eigen import check_column_indices
    ptr = torch.tensor([0, 2, 3], dtype=torch.int64)
    check_column_indices(DeviceCSR(ptr, torch.tensor([0, 4, 1], dtype=torch.int32), None, (2, 5)))
    check_column_indices(DeviceCSR(torch.zeros(2, dtype=torch.int64), torch.zeros(0, dtype=torch.int32), None,
                                   (1, 5)))
    for bad in ([0, 5, 1], [0, -1, 1]):
        with pytest.raises(ValueError, match="column indices"):
            check_column_indices(DeviceCSR(ptr, torch.tensor(bad, dtype=torch.int32), None, (2, 5)))


def test_read_transcripts_reference_known_answer(tmp_path):
    """The reference's test_read_transcript (genome.rs:599-643, via
    tests/golden/transcripts.json): the same transcript from its GFF3 and GTF
    text, and a GTF line whose quoted value holds ';' parses."""
    import json
    import os
    from snapatac2_gb300._genes import read_transcripts
    with open(os.path.join(os.path.dirname(__file__), "golden", "transcripts.json")) as fh:
        g = json.load(fh)
    (tmp_path / "a.gff3").write_text(g["gff"] + "\n")
    (tmp_path / "a.gtf").write_text(g["gtf"] + "\n")
    (tmp_path / "w.gtf").write_text(g["worked"] + "\n")
    for reader in (read_transcripts, ogn.read_transcripts):
        for name in ("a.gff3", "a.gtf"):
            t = reader(tmp_path / name)[0]
            assert {k: t[k] for k in g["expected"]} == g["expected"], (reader, name)
        w = reader(tmp_path / "w.gtf")
        assert len(w) == 1 and w[0]["transcript_id"] == "XM_5" and w[0]["gene_name"] == "RGD"
    (tmp_path / "q.gtf").write_text('chr1\tG\ttranscript\t5\t9\t.\t-\t.\tgene_id "G"; transcript_id "T;1"; '
                                    'gene_name "A;B"; level 2\n')
    for reader in (read_transcripts, ogn.read_transcripts):
        t = reader(tmp_path / "q.gtf")[0]
        assert (t["transcript_id"], t["gene_name"], t["gene_id"]) == ("T;1", "A;B", "G")


def test_import_result_to_anndata_slots(caplog):
    """The import's AnnData layout (import.rs:161-210, genome.rs:247-251):
    obsm['fragment_paired'] (uint32 sizes, genome-wide columns), obs QC
    columns, uns['reference_sequences'], and the reference's warning with
    no cells (import.rs:112)."""
    import logging
    from snapatac2_gb300._import import FRAGMENT_PAIRED, ImportResult, to_anndata
    from snapatac2_gb300.genome import ChromSizes
    cs = ChromSizes([("chr1", 100), ("chr2", 50)])
    r = ImportResult(key=FRAGMENT_PAIRED, obs_names=["A", "B"], indptr=np.array([0, 1, 3]),
                     indices=np.array([5, 10, 120]), data=np.array([20, 30, 10], dtype=np.uint32),
                     n_fragment=np.array([1, 2], dtype=np.uint64), frac_dup=np.array([0.0, 0.5]),
                     frac_mito=np.array([0.0, 0.0]), chrom_sizes=cs, info={})
    ad = to_anndata(r)
    m = ad.obsm[FRAGMENT_PAIRED]
    assert m.shape == (2, 150) and m.dtype == np.uint32 and m.indices.tolist() == [5, 10, 120]
    assert list(ad.obs_names) == ["A", "B"] and ad.n_obs == 2
    assert set(ad.obs.keys()) == {"n_fragment", "frac_dup", "frac_mito"}
    ref = ad.uns["reference_sequences"]
    assert list(ref["reference_seq_name"]) == ["chr1", "chr2"] and list(ref["reference_seq_length"]) == [100, 50]
    with caplog.at_level(logging.WARNING):
        empty = to_anndata(ImportResult(None, [], None, None, None, None, None, None, cs, {}))
    assert empty.n_obs == 0 and "No barcodes passed the QC filter. No data is imported." in caplog.text
