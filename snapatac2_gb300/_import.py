"""``snap.pp.import_fragments`` on the GPU.

Drop-in counterpart of ``snapatac2-python/python/snapatac2/preprocessing/_basic.py:156-340``
(``import_fragments``) over the PyO3 entry
``snapatac2-python/src/preprocessing.rs:87-172`` and
``snapatac2-core/src/preprocessing/import.rs:31-210``.  The host reads the
file (plain or gzip) and uploads its bytes; parsing, grouping by barcode, QC,
filtering and the per-cell sort run as CUDA kernels behind the C ABI
(``sg_frag_*`` in ``include/snapgb300.h``).
"""
from __future__ import annotations

import ctypes
import gzip
import logging
import os
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from ._anndata import AnnData
from .genome import ChromSizes

FRAGMENT_SINGLE = "fragment_single"
FRAGMENT_PAIRED = "fragment_paired"
HASH_SEED = 0x5EED_F4A6_0001


@dataclass
class ImportResult:
    """Arrays of one import (host copies)."""
    key: str | None            # FRAGMENT_PAIRED / FRAGMENT_SINGLE, None when no cell passed
    obs_names: list
    indptr: np.ndarray | None
    indices: np.ndarray | None
    data: np.ndarray | None
    n_fragment: np.ndarray | None
    frac_dup: np.ndarray | None
    frac_mito: np.ndarray | None
    chrom_sizes: ChromSizes    # sorted by name, as the reference's BTreeMap
    info: dict


def read_fragment_file(path) -> torch.Tensor:
    """The decompressed bytes of a fragment file (gzip, zstd or plain text)
    in a pinned host buffer (uint8 tensor), ready for an asynchronous copy."""
    with open(path, "rb") as fh:
        head = fh.read(4)
    if head[:2] == b"\x1f\x8b":
        with gzip.open(path, "rb") as fh:
            data = fh.read()
    elif head == b"\x28\xb5\x2f\xfd":
        try:
            import zstandard
        except ImportError as e:  # pragma: no cover - depends on the environment
            raise NotImplementedError("zstd-compressed fragment files need the 'zstandard' module") from e
        with open(path, "rb") as fh:
            data = zstandard.ZstdDecompressor().decompress(fh.read())
    else:  # plain text: read straight into the pinned buffer
        n = os.path.getsize(path)
        out = torch.empty(max(n, 1), dtype=torch.uint8, pin_memory=True)
        with open(path, "rb") as fh:
            got = fh.readinto(memoryview(out.numpy())[:n]) if n else 0
        return out[:got]
    out = torch.empty(max(len(data), 1), dtype=torch.uint8, pin_memory=True)
    out.numpy()[:len(data)] = np.frombuffer(data, dtype=np.uint8)
    return out[:len(data)]


def sorted_chrom_sizes(chrom_sizes) -> ChromSizes:
    """The genome table in the reference's order: ``chrom_size`` arrives as a
    ``BTreeMap<String, u64>`` (preprocessing.rs:95), i.e. sorted by bytes."""
    if hasattr(chrom_sizes, "chrom_sizes"):
        chrom_sizes = chrom_sizes.chrom_sizes
    items = chrom_sizes.items() if isinstance(chrom_sizes, dict) else list(chrom_sizes)
    items = sorted(((str(k), int(v)) for k, v in items), key=lambda kv: kv[0].encode())
    return ChromSizes(items)


def _blob(strings: list[bytes]):
    off = np.zeros(len(strings) + 1, dtype=np.int64)
    if strings:
        off[1:] = np.cumsum([len(s) for s in strings])
    blob = np.frombuffer(b"".join(strings) or b"\0", dtype=np.uint8)
    return blob, off


@dataclass
class DeviceImport:
    """Results of one import, on the device (see ``sg_frag_emit``)."""
    key: str | None
    indptr: torch.Tensor | None      # int64 [cells + 1]
    indices: torch.Tensor | None     # int64 [entries]
    data: torch.Tensor | None        # int32 [entries] (uint32 bits for paired data)
    bc_loc: torch.Tensor | None      # int64 [cells]: byte offset << 16 | length in the text
    n_fragment: torch.Tensor | None  # int64 [cells] (uint64 values)
    frac_dup: torch.Tensor | None
    frac_mito: torch.Tensor | None
    chrom_sizes: ChromSizes
    info: dict


def upload_text(text, device) -> torch.Tensor:
    """Host bytes -> uint8 device tensor through a pinned staging buffer."""
    buf = np.frombuffer(text, dtype=np.uint8) if not isinstance(text, np.ndarray) else text.view(np.uint8)
    pinned = torch.empty(max(buf.size, 1), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:buf.size] = buf
    return pinned[:buf.size].to(device, non_blocking=True)


def import_device(d_text: torch.Tensor, chrom_sizes, *, min_num_fragments: int = 200,
                  sorted_by_barcode: bool = True, whitelist=None, chrM=("chrM", "M"), shift_left: int = 0,
                  shift_right: int = 0) -> DeviceImport:
    """The import of fragment-file text already in device memory (uint8)."""
    if d_text.dtype != torch.uint8 or not d_text.is_cuda:
        raise ValueError("d_text must be a uint8 CUDA tensor")
    dev = d_text.device
    L = _lib.lib()
    cs = sorted_chrom_sizes(chrom_sizes)
    if len(cs) == 0:
        raise ValueError("chrom_size cannot be empty")
    if d_text.numel() and d_text.data_ptr() % 16:
        d_text = d_text.clone()  # the line index reads 16-byte vectors
    nbytes = int(d_text.numel())
    sh = torch.cuda.current_stream(dev).cuda_stream
    base = d_text.data_ptr() if nbytes else None

    scr = torch.empty(max(int(L.sg_frag_line_scratch_bytes(nbytes)), 8), dtype=torch.uint8, device=dev)
    nl = ctypes.c_int64()
    _lib.check(L.sg_frag_count_lines(base, nbytes, scr.data_ptr(), ctypes.byref(nl), sh), "sg_frag_count_lines")
    n_lines = int(nl.value)
    line_start = torch.empty(n_lines + 1, dtype=torch.int64, device=dev)
    _lib.check(L.sg_frag_index_lines(base, nbytes, scr.data_ptr(), n_lines, line_start.data_ptr(), sh),
               "sg_frag_index_lines")
    del scr

    names = [n.encode() for n in cs.names]
    cblob, coff = _blob(names)
    sizes = np.asarray(cs.sizes, dtype=np.uint64)
    cbase = np.zeros(len(sizes), dtype=np.uint64)
    if len(sizes) > 1:
        cbase[1:] = np.cumsum(sizes[:-1], dtype=np.uint64)
    mito = {c.encode() if isinstance(c, str) else bytes(c) for c in (chrM or [])}
    cmito = np.array([n in mito for n in names], dtype=np.uint8)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_cblob, d_coff, d_size, d_base, d_mito = t(cblob), t(coff), t(sizes.view(np.int64)), t(cbase.view(np.int64)), t(cmito)

    has_wl = whitelist is not None
    wl = sorted({w.encode() if isinstance(w, str) else bytes(w) for w in whitelist}) if has_wl else []
    wblob, woff = _blob(wl)
    d_wblob, d_woff = t(wblob), t(woff)

    ws_bytes = int(L.sg_frag_workspace_bytes(n_lines, len(wl)))
    ws = torch.empty(max(ws_bytes, 256), dtype=torch.uint8, device=dev)
    info = (ctypes.c_int64 * 10)()
    code = L.sg_frag_import(base, nbytes, line_start.data_ptr(), n_lines, d_cblob.data_ptr(), d_coff.data_ptr(),
                            d_size.data_ptr(), d_base.data_ptr(), d_mito.data_ptr(), len(names),
                            int(sizes.sum(dtype=np.uint64)), d_wblob.data_ptr(), d_woff.data_ptr(), len(wl),
                            int(has_wl), int(max(min_num_fragments, 0)), int(bool(sorted_by_barcode)),
                            int(shift_left), int(shift_right), HASH_SEED, ws.data_ptr(), ws_bytes, info, sh)
    inf = [int(v) for v in info]
    if code != _lib.SG_OK:
        line = inf[3]
        where = f" (line {line + 1})" if line >= 0 else ""
        if code == _lib.SG_ERR_UNSORTED:
            raise ValueError("Please sort fragment file by barcodes")
        if code in (_lib.SG_ERR_PARSE, _lib.SG_ERR_RANGE, _lib.SG_ERR_CONVERT):
            raise ValueError(f"import_fragments: {_lib.status_string(code)}{where}")
        _lib.check(code, "sg_frag_import")
    K, nnz, paired = inf[0], inf[1], inf[2]
    meta = {"cells": K, "entries": nnz, "paired": paired, "records": inf[4], "barcodes": inf[5],
            "rehash": inf[6], "sort_path": inf[7], "kernels": inf[8] + (5 if nbytes else 0), "lines": n_lines,
            "bytes": nbytes}
    if K == 0:
        return DeviceImport(None, None, None, None, None, None, None, None, cs, meta)
    e = lambda n, dt=torch.int64: torch.empty(max(n, 1), dtype=dt, device=dev)  # noqa: E731
    indptr, indices, data = e(K + 1), e(nnz), e(nnz, torch.int32)
    bc, nf, fd, fm = e(K), e(K), e(K, torch.float64), e(K, torch.float64)
    _lib.check(L.sg_frag_emit(ws.data_ptr(), n_lines, len(wl), info, indptr.data_ptr(), indices.data_ptr(),
                              data.data_ptr(), bc.data_ptr(), nf.data_ptr(), fd.data_ptr(), fm.data_ptr(), sh),
               "sg_frag_emit")
    return DeviceImport(FRAGMENT_PAIRED if paired == 1 else FRAGMENT_SINGLE, indptr[:K + 1], indices[:nnz],
                        data[:nnz], bc[:K], nf[:K], fd[:K], fm[:K], cs, meta)


def to_host(r: DeviceImport, d_text: torch.Tensor, host_text=None) -> ImportResult:
    """Host copies of a DeviceImport, with the barcodes as strings.  The
    barcode bytes come from ``host_text`` when given, else from the device."""
    if r.key is None:
        return ImportResult(None, [], None, None, None, None, None, None, r.chrom_sizes, r.info)
    # device -> pinned host buffers, one asynchronous copy each, one synchronisation
    outs = (r.indptr, r.indices, r.data, r.bc_loc, r.n_fragment, r.frac_dup, r.frac_mito)
    host = [torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in outs]
    for h, t in zip(host, outs):
        h.copy_(t, non_blocking=True)
    torch.cuda.current_stream(r.indptr.device).synchronize()
    indptr, indices, data, bc_loc, n_fragment, frac_dup, frac_mito = (h.numpy() for h in host)
    bc_h = bc_loc.view(np.uint64)
    offs, lens = (bc_h >> np.uint64(16)).astype(np.int64), (bc_h & np.uint64(0xFFFF)).astype(np.int64)
    if host_text is None:
        host_text = _gather_barcodes(d_text, offs, lens)
        offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    mv = memoryview(host_text)
    obs_names = [bytes(mv[o:o + n]).decode() for o, n in zip(offs.tolist(), lens.tolist())]
    paired = r.key == FRAGMENT_PAIRED
    return ImportResult(
        key=r.key, obs_names=obs_names, indptr=indptr, indices=indices,
        data=data.view(np.uint32) if paired else data, n_fragment=n_fragment.view(np.uint64),
        frac_dup=frac_dup, frac_mito=frac_mito, chrom_sizes=r.chrom_sizes, info=r.info)


def import_text(text: bytes | np.ndarray | torch.Tensor, chrom_sizes, *, min_num_fragments: int = 200,
                sorted_by_barcode: bool = True, whitelist=None, chrM=("chrM", "M"), shift_left: int = 0,
                shift_right: int = 0, device=None, host_text=None) -> ImportResult:
    """Import fragment-file text (bytes on the host, or a uint8 tensor) and
    return host arrays.  ``host_text`` (the same bytes on the host) saves
    reading the kept cells' barcodes back from the device."""
    from .tools import _UPLOADS, release_uploads
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    borrowed: list = []
    if isinstance(text, torch.Tensor):
        if text.dtype != torch.uint8:
            raise ValueError("text must be uint8")
        if text.is_cuda:
            d_text = text.to(dev)
        else:  # host text: into a pooled device buffer (no first-touch cost on reuse)
            buf = _UPLOADS.take(dev, torch.uint8, text.numel())
            borrowed.append(buf)
            d_text = buf[:text.numel()]
            d_text.copy_(text, non_blocking=text.is_pinned())
    else:
        if host_text is None and isinstance(text, (bytes, bytearray)):
            host_text = text
        d_text = upload_text(text, dev)
    try:
        r = import_device(d_text, chrom_sizes, min_num_fragments=min_num_fragments,
                          sorted_by_barcode=sorted_by_barcode, whitelist=whitelist, chrM=chrM,
                          shift_left=shift_left, shift_right=shift_right)
        return to_host(r, d_text, host_text)
    finally:
        del d_text
        release_uploads(borrowed)


def _gather_barcodes(d_text: torch.Tensor, offs: np.ndarray, lens: np.ndarray) -> bytes:
    """The kept cells' barcode bytes, concatenated, read from the device
    (``sg_gather_bytes`` into one buffer, one copy back)."""
    if offs.size == 0:
        return b""
    L = _lib.lib()
    dev = d_text.device
    dst = np.zeros(offs.size, dtype=np.int64)
    np.cumsum(lens[:-1], out=dst[1:])
    total = int(lens.sum())
    meta = torch.from_numpy(np.concatenate([offs.astype(np.int64), dst])).to(dev)
    ln = torch.from_numpy(lens.astype(np.int32)).to(dev)
    out = torch.empty(max(total, 1), dtype=torch.uint8, device=dev)
    sh = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(L.sg_gather_bytes(offs.size, meta.data_ptr(), ln.data_ptr(), meta.data_ptr() + 8 * offs.size,
                                 d_text.data_ptr(), out.data_ptr(), sh), "sg_gather_bytes")
    return out[:total].cpu().numpy().tobytes()


def to_anndata(res: ImportResult, adata=None):
    """Write an ImportResult into an AnnData (in memory) like the reference:
    ``obsm[fragment_paired | fragment_single]``, ``obs`` n_fragment /
    frac_dup / frac_mito, obs_names, ``uns['reference_sequences']``."""
    if res.key is None:
        logging.getLogger(__name__).warning("No barcodes passed the QC filter. No data is imported.")
        return adata if adata is not None else AnnData()
    K = len(res.obs_names)
    m = sp.csr_matrix((res.data, res.indices, res.indptr), shape=(K, res.chrom_sizes.total_size()))
    uns = {"reference_sequences": {"reference_seq_name": np.array(res.chrom_sizes.names, dtype=object),
                                   "reference_seq_length": np.array(res.chrom_sizes.sizes, dtype=np.uint64)}}
    obs = {"n_fragment": res.n_fragment, "frac_dup": res.frac_dup, "frac_mito": res.frac_mito}
    return AnnData(obsm={res.key: m}, obs=obs, uns=uns, n_obs=K, obs_names=list(res.obs_names))


def import_fragments(fragment_file, chrom_sizes, *, file=None, min_num_fragments: int = 200,
                     sorted_by_barcode: bool = True, whitelist=None, chrM=["chrM", "M"], shift_left: int = 0,
                     shift_right: int = 0, chunk_size: int = 2000, tempdir=None, backend="hdf5", n_jobs: int = 8,
                     device=None):
    """Import fragment files and compute the basic QC metrics (``_basic.py:156-340``).

    Same keywords and outputs as the reference: ``obsm['fragment_paired']``
    (or ``'fragment_single'``), ``obs`` columns ``n_fragment``, ``frac_dup``,
    ``frac_mito``, ``uns['reference_sequences']``.  ``file`` (backed output)
    is not supported; ``chunk_size``, ``tempdir`` and ``n_jobs`` are accepted
    for compatibility (the whole file is processed in device memory).
    """
    cs = chrom_sizes.chrom_sizes if hasattr(chrom_sizes, "chrom_sizes") else chrom_sizes
    if len(cs) == 0:
        raise ValueError("chrom_size cannot be empty")
    if file is not None:
        raise NotImplementedError("backed (file=...) output is not supported; use file=None")
    if whitelist is not None:
        if isinstance(whitelist, (str, os.PathLike)):
            with open(whitelist, "r") as fl:
                whitelist = set(line.strip() for line in fl)
        else:
            whitelist = set(whitelist)
    if isinstance(fragment_file, list):
        return [import_fragments(f, chrom_sizes, min_num_fragments=min_num_fragments,
                                 sorted_by_barcode=sorted_by_barcode, whitelist=whitelist, chrM=chrM,
                                 shift_left=shift_left, shift_right=shift_right, device=device)
                for f in fragment_file]
    text = read_fragment_file(fragment_file)
    res = import_text(text, cs, min_num_fragments=min_num_fragments, sorted_by_barcode=sorted_by_barcode,
                      whitelist=whitelist, chrM=chrM, shift_left=shift_left, shift_right=shift_right,
                      device=device, host_text=text.numpy())
    return to_anndata(res)
