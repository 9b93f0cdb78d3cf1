"""``snap.pp.make_gene_matrix`` on the GPU: cell-by-gene activity.

Drop-in counterpart of ``snapatac2-python/python/snapatac2/preprocessing/_basic.py:707-800``
over the PyO3 ``mk_gene_matrix`` (``snapatac2-python/src/preprocessing.rs:432-500``)
and ``create_gene_matrix`` (``snapatac2-core/src/feature_count/matrix.rs:175-273``).
The annotation is read on the host (GTF / GFF3 "transcript" records,
``snapatac2-core/src/genome.rs:45-190``); the promoter regions
(``Promoters::new``, ``genome.rs:198-232``) are counted by the GPU region
counter (``sg_region_plan`` / ``sg_region_run``), and the gene level keeps,
per gene, the maximum over its regions (``GeneCount::get_values``,
``snapatac2-core/src/feature_count/counter.rs:270-283``) on the device
(``sg_gene_max``: radix sort of (cell, gene) keys, segment maximum).
"""
from __future__ import annotations

import ctypes
import gzip
from urllib.parse import unquote

import numpy as np
import scipy.sparse as sp
import torch

from ._anndata import AnnData
from ._regions import build_regions, region_matrix


def _open(path):
    return gzip.open(path, "rt") if str(path).endswith(".gz") else open(path, "rt")


def _attrs(s: str, gff: bool) -> dict:
    if not gff:
        return _attrs_gtf(s)
    out: dict = {}
    for part in s.strip().split(";"):
        part = part.strip()
        if part:
            k, _, v = part.partition("=")
            out.setdefault(unquote(k.strip()), unquote(v.strip()))
    return out


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


def read_transcripts(path, *, transcript_name_key="transcript_name", transcript_id_key="transcript_id",
                     gene_name_key="gene_name", gene_id_key="gene_id") -> list[dict]:
    """"transcript" records of a GTF or GFF3 file (plain or gzip): chrom,
    1-based closed left/right, strand, ids and names (``from_gtf`` /
    ``from_gff``, genome.rs:76-145).  The file type follows the extension;
    otherwise GFF3 when the attributes use key=value."""
    p = str(path)
    stem = p[:-3] if p.endswith(".gz") else p
    gff = stem.endswith(".gff")
    if not (stem.endswith(".gff") or stem.endswith(".gtf")):
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
            a = _attrs(f[8], gff)
            for key in (transcript_id_key, gene_name_key, gene_id_key):
                if key not in a:
                    raise ValueError(f"failed to find '{key}' in record: {line}")
            out.append({"chrom": f[0], "left": int(f[3]), "right": int(f[4]), "strand": f[6],
                        "transcript_id": a[transcript_id_key], "gene_name": a[gene_name_key],
                        "gene_id": a[gene_id_key], "transcript_name": a.get(transcript_name_key)})
    return out


def promoter_regions(transcripts, upstream: int, downstream: int, include_gene_body: bool):
    """``Promoters::new`` (genome.rs:198-232) for each transcript."""
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


def gene_max(indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor, region_gene: torch.Tensor):
    """Per row, the maximum count over the regions of each gene
    (``sg_gene_max``: (row, gene) keys radix-sorted with their counts, runs
    reduced by maximum).  Returns (indptr int64, gene int32, count int32)."""
    from . import _lib
    L = _lib.lib()
    dev = indptr.device
    n = indptr.numel() - 1
    nnz = int(indices.numel())
    sh = torch.cuda.current_stream(dev).cuda_stream
    nbytes = int(L.sg_gene_max_scratch_bytes(nnz))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
    out_ptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    out_idx = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    out_val = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    n_out = ctypes.c_int64(0)
    idx, val, rg = indices.contiguous(), data.contiguous(), region_gene.contiguous()
    if idx.dtype != torch.int32 or val.element_size() != 4 or rg.dtype != torch.int32:
        raise ValueError("gene_max: int32 region indices and region_gene, 32-bit counts expected")
    _lib.check(L.sg_gene_max(n, indptr.data_ptr(), idx.data_ptr() if nnz else None,
                             val.data_ptr() if nnz else None, rg.data_ptr() if rg.numel() else None, nnz,
                             scratch.data_ptr(), nbytes, out_ptr.data_ptr(), out_idx.data_ptr(), out_val.data_ptr(),
                             ctypes.byref(n_out), sh), "sg_gene_max")
    u = int(n_out.value)
    return out_ptr, out_idx[:u], out_val[:u]


def make_gene_matrix(adata, gene_anno, *, inplace: bool = False, file=None, backend="hdf5", chunk_size: int = 500,
                     use_x: bool = False, id_type: str = "gene", upstream: int = 2000, downstream: int = 0,
                     include_gene_body: bool = True, transcript_name_key: str = "transcript_name",
                     transcript_id_key: str = "transcript_id", gene_name_key: str = "gene_name",
                     gene_id_key: str = "gene_id", min_frag_size: int | None = None,
                     max_frag_size: int | None = None, counting_strategy: str = "paired-insertion", device=None):
    """Cell-by-gene activity matrix (``_basic.py:707-800``).

    ``gene_anno``: a GTF / GFF3 file (or an object with ``.annotation``).
    Same keywords and outputs as the reference.  ``use_x=True`` aggregates
    the existing X by the transcripts' regions instead of counting fragments
    (``_basic.py:715,823``), integer X only at the gene level (maximum over
    a gene's transcripts).  Backed ``file=`` output is not supported.
    """
    from .preprocessing import _device, _fragment_arrays, read_chrom_sizes
    if id_type not in ("gene", "transcript"):
        raise ValueError("id_type must be 'transcript' or 'gene'")
    if counting_strategy not in ("fragment", "insertion", "paired-insertion"):
        raise ValueError("Counting strategy must be one of 'insertion', 'fragment', or 'paired-insertion'")
    if file is not None:
        raise NotImplementedError("backed (file=...) output is not supported; use file=None")
    if hasattr(gene_anno, "annotation"):
        gene_anno = gene_anno.annotation
    transcripts = read_transcripts(gene_anno, transcript_name_key=transcript_name_key,
                                   transcript_id_key=transcript_id_key, gene_name_key=gene_name_key,
                                   gene_id_key=gene_id_key)
    regs = promoter_regions(transcripts, upstream, downstream, include_gene_body)
    dev = _device(device)
    if use_x:
        from ._binning import DeviceCSR
        from ._regions import aggregate_x
        Y, rnames = aggregate_x(adata.X, adata.var_names, regs, dev)
        if id_type == "gene" and Y.dtype != np.uint32:
            raise NotImplementedError("use_x=True with id_type='gene' needs an integer X")
        data = Y.data.view(np.int32) if Y.dtype == np.uint32 else Y.data
        res = DeviceCSR(torch.from_numpy(Y.indptr.astype(np.int64)).to(dev),
                        torch.from_numpy(Y.indices.astype(np.int32)).to(dev), torch.from_numpy(data).to(dev),
                        Y.shape)
        rs_names = rnames
    else:
        cs = read_chrom_sizes(adata)
        paired, indptr, pos, length = _fragment_arrays(adata)
        rs = build_regions(regs, cs.names, dev)
        rs_names = rs.names
        t_len = torch.from_numpy(np.ascontiguousarray(length).view(np.int32)).to(dev) if paired else None
        res = region_matrix(torch.from_numpy(indptr).to(dev), torch.from_numpy(pos).to(dev), t_len, cs, rs,
                            strategy=counting_strategy if paired else "single",
                            min_frag_size=min_frag_size if paired else None,
                            max_frag_size=max_frag_size if paired else None)
    if id_type == "transcript":
        names = [t["transcript_id"] for t in transcripts]
        ip, ix, dv = res.indptr, res.indices, res.data
        var = {"gene_name": np.array([t["gene_name"] for t in transcripts], dtype=object)}
    else:
        gidx: dict = {}
        for t in transcripts:
            gidx.setdefault(t["gene_name"], len(gidx))
        names = list(gidx)
        # region k is read as transcript k (the reference's indexing; regions repeat-free)
        region_gene = torch.tensor([gidx[transcripts[k]["gene_name"]] for k in range(len(rs_names))],
                                   dtype=torch.int32, device=dev)
        ip, ix, dv = gene_max(res.indptr, res.indices, res.data, region_gene)
        var = None
    dvh = dv.cpu().numpy()
    X = sp.csr_matrix((dvh.view(np.uint32) if dvh.dtype == np.int32 else dvh, ix.cpu().numpy(), ip.cpu().numpy()),
                      shape=(res.shape[0], len(names)))
    if inplace:
        if hasattr(adata, "set_n_vars"):
            adata.set_n_vars(X.shape[1])
        adata.X = X
        adata.var_names = names
        if var is not None and hasattr(adata, "var"):
            for k, v in var.items():
                adata.var[k] = v
        return None
    return AnnData(X, obs=dict(getattr(adata, "obs", {}) or {}), var=var, obs_names=adata.obs_names,
                   var_names=names)
