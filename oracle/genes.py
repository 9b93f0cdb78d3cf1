"""ORACLE (test infrastructure only): the gene activity matrix restated in Python.

Restates ``snap.pp.make_gene_matrix`` over fragments:

* transcripts: the "transcript" records of a GTF or GFF3 file
  (``read_transcripts_from_gtf`` / ``_from_gff``, snapatac2-core/src/genome.rs:45-190;
  file type by extension, snapatac2-python/src/utils.rs:376-399), 1-based
  closed coordinates, the attributes named by the ``*_key`` options
  (``from_gtf`` / ``from_gff``, genome.rs:76-145).  The line formats are
  those of the third-party noodles GTF / GFF3 readers (not in the reference
  tree): nine tab-separated columns, GTF attributes ``key "value";``,
  GFF3 attributes ``key=value;`` with %XX escapes;
* promoter regions (``Promoters::new``, genome.rs:198-232): with
  ``left``/``right`` the 0-based first and last base, "+" strand gives
  [left - upstream (saturating), downstream + (right if gene body else
  left)), "-" strand [(left if gene body else right) - downstream
  (saturating), right + upstream);
* counting: the regions as an index set (repeats dropped) counted by
  ``RegionCounter`` (oracle ``regions.region_counts``); "transcript" columns
  are region indices under the transcript ids, "gene" columns take, per
  gene name, the maximum over the regions whose index, read as a transcript
  index, names that gene (``GeneCount::get_values``, counter.rs:270-283),
  genes numbered by first appearance.
"""
from __future__ import annotations

import gzip
from urllib.parse import unquote

import numpy as np

from . import regions as org


def _open(path):
    return gzip.open(path, "rt") if str(path).endswith(".gz") else open(path, "rt")


def _attrs_gtf(s: str) -> dict:
    """GTF attributes ``key value; key "value"; ...``: a quoted value may hold
    ';' (the noodles GTF reader's entry format); the first of repeated keys
    is kept."""
    out: dict = {}
    i, n = 0, len(s)
    while i < n:
        while i < n and s[i] in " \t;":
            i += 1
        if i >= n:
            break
        j = i
        while j < n and s[j] not in " \t;":
            j += 1
        key = s[i:j]
        while j < n and s[j] in " \t":
            j += 1
        if j < n and s[j] == '"':
            k = s.find('"', j + 1)
            k = n if k < 0 else k
            val, j = s[j + 1:k], k + 1
        else:
            k = s.find(";", j)
            k = n if k < 0 else k
            val, j = s[j:k].strip(), k
        out.setdefault(key, val)
        i = j
    return out


def _attrs_gff(s: str) -> dict:
    out = {}
    for part in s.strip().split(";"):
        if not part:
            continue
        k, _, v = part.partition("=")
        out.setdefault(unquote(k.strip()), unquote(v.strip()))
    return out


def read_transcripts(path, *, transcript_name_key="transcript_name", transcript_id_key="transcript_id",
                     gene_name_key="gene_name", gene_id_key="gene_id") -> list[dict]:
    p = str(path)
    stem = p[:-3] if p.endswith(".gz") else p
    if stem.endswith(".gff") or stem.endswith(".gtf"):
        gff = stem.endswith(".gff")
    else:  # utils.rs:390-397: GFF first, GTF when that fails (decided on the first record)
        gff = False
        with _open(path) as fh:
            for line in fh:
                f = line.rstrip("\n").split("\t")
                if len(f) >= 9 and not line.startswith("#"):
                    gff = "=" in f[8] and '"' not in f[8]
                    break
    out = []
    with _open(path) as fh:
        for line in fh:
            line = line.rstrip("\n")
            if not line or line.startswith("#"):
                continue
            f = line.split("\t")
            if len(f) < 9:
                raise ValueError(f"failed to parse {'GFF' if gff else 'GTF'} line: {line}")
            if f[2] != "transcript":
                continue
            a = _attrs_gff(f[8]) if gff else _attrs_gtf(f[8])
            for key in (transcript_id_key, gene_name_key, gene_id_key):
                if key not in a:
                    raise ValueError(f"failed to find '{key}' in record: {line}")
            out.append({"chrom": f[0], "left": int(f[3]), "right": int(f[4]), "strand": f[6],
                        "transcript_id": a[transcript_id_key], "gene_name": a[gene_name_key],
                        "gene_id": a[gene_id_key], "transcript_name": a.get(transcript_name_key)})
    return out


def promoter_regions(transcripts, upstream=2000, downstream=0, include_gene_body=True):
    regs = []
    for t in transcripts:
        left, right = t["left"] - 1, t["right"] - 1
        if t["strand"] == "+":
            s, e = max(left - upstream, 0), downstream + (right if include_gene_body else left)
        elif t["strand"] == "-":
            s, e = max((left if include_gene_body else right) - downstream, 0), right + upstream
        else:
            raise ValueError(f"Miss strand information for {t['transcript_id']}")
        regs.append((t["chrom"], s, e))
    return regs


def gene_matrix(indptr, pos, length, chrom_names, chrom_sizes, transcripts, *, id_type="gene", upstream=2000,
                downstream=0, include_gene_body=True, strategy="paired-insertion", paired=True,
                min_frag_size=None, max_frag_size=None):
    """(indptr, indices, data, var_names) of the gene (or transcript) matrix."""
    regs = promoter_regions(transcripts, upstream, downstream, include_gene_body)
    ip, ix, dv, _ = org.region_counts(indptr, pos, length, chrom_names, chrom_sizes, regs, strategy=strategy,
                                      paired=paired, min_frag_size=min_frag_size, max_frag_size=max_frag_size)
    return _by_id(ip, ix, dv, transcripts, id_type)


def gene_matrix_from_x(X, var_names, chrom_names, transcripts, *, id_type="gene", upstream=2000, downstream=0,
                       include_gene_body=True):
    """``use_x=True`` of ``create_gene_matrix`` (snapatac2-core/src/feature_count/matrix.rs:211-218): X
    aggregated by the transcripts' promoter regions (``regions.aggregate_x``), then the same transcript /
    gene levels as the fragment path."""
    regs = promoter_regions(transcripts, upstream, downstream, include_gene_body)
    ip, ix, dv, _ = org.aggregate_x(X, var_names, chrom_names, regs)
    return _by_id(ip, ix, dv, transcripts, id_type)


def _by_id(ip, ix, dv, transcripts, id_type):
    """Region k read as transcript k; the gene level keeps each row's maximum over a gene's transcripts."""
    if id_type == "transcript":
        return ip, ix, dv, [t["transcript_id"] for t in transcripts]
    gidx: dict = {}
    for t in transcripts:
        gidx.setdefault(t["gene_name"], len(gidx))
    out_ptr, out_idx, out_val = [0], [], []
    for r in range(ip.size - 1):
        row: dict = {}
        for k, v in zip(ix[ip[r]:ip[r + 1]].tolist(), dv[ip[r]:ip[r + 1]].tolist()):
            g = gidx[transcripts[k]["gene_name"]]
            row[g] = max(row.get(g, v), v)
        for g in sorted(row):
            out_idx.append(g)
            out_val.append(row[g])
        out_ptr.append(len(out_idx))
    return (np.array(out_ptr, dtype=np.int64), np.array(out_idx, dtype=np.int64),
            np.array(out_val).astype(np.uint32), list(gidx))
