"""ORACLE (test infrastructure only): fragment-file import restated in Python.

Restates ``snap.pp.import_fragments`` for small inputs, loop for loop:

* record parsing: ``Fragment::from_str``
  (snapatac2-core/src/preprocessing/qc.rs:303-348): tab-separated chrom,
  start, end (unsigned decimal), barcode ("." = none), optional count
  (missing or "." = 1) and optional strand ("+", "-", "." = none); further
  fields are ignored.  Lines come from the bed-utils 0.7.1 reader with
  comment prefix "#" (snapatac2-python/src/preprocessing.rs:125-129): the
  newline, and a carriage return before it, are dropped, and lines starting
  with "#" are skipped;
* ``shift_fragment`` (preprocessing.rs:174-184): saturating unsigned shifts;
* the minimum-count whitelist of unsorted input (preprocessing.rs:106-122)
  and the sort by barcode (preprocessing.rs:136-152);
* ``import_fragments`` / ``make_arraydata`` / ``count_fragments``
  (snapatac2-core/src/preprocessing/import.rs:31-210): records with
  end != start grouped in runs of equal barcode, the whitelist, the
  "Please sort fragment file by barcodes" check, per-cell QC
  (``FragmentQCBuilder``, qc.rs:445-465), the minimum-fragment filter and
  each cell's (position, signed size) pairs sorted;
* chromosome order: the reference receives ``chrom_sizes`` as a
  ``BTreeMap`` (preprocessing.rs:95), so the genome index follows the names'
  byte order (genome.rs:296-312, 387-406).

The reference is a release build, so ``end - start`` of a fragment with
end < start wraps instead of failing (the record stays; the conversion of its
signed size then decides); this restatement follows that.
"""
from __future__ import annotations

import numpy as np

U64_MAX = (1 << 64) - 1


class ImportError_(ValueError):
    """The reference panics or returns an error for this input."""


def _parse_uint(s: bytes, bits: int, what: str, lineno: int) -> int:
    if not s or not s.isdigit():
        raise ImportError_(f"line {lineno}: invalid {what} {s!r}")
    v = int(s)
    if v >> bits:
        raise ImportError_(f"line {lineno}: {what} {s!r} out of range")
    return v


def parse_record(line: bytes, lineno: int) -> dict:
    """qc.rs:303-348."""
    fields = line.split(b"\t")
    chrom = fields[0]
    if len(fields) < 2:
        raise ImportError_(f"line {lineno}: missing start position")
    start = _parse_uint(fields[1], 64, "start position", lineno)
    if len(fields) < 3:
        raise ImportError_(f"line {lineno}: missing end position")
    end = _parse_uint(fields[2], 64, "end position", lineno)
    if len(fields) < 4:
        raise ImportError_(f"line {lineno}: missing name")
    barcode = None if fields[3] == b"." else fields[3]
    count = 1
    if len(fields) >= 5 and fields[4] != b".":
        count = _parse_uint(fields[4], 32, "count", lineno)
    strand = None
    if len(fields) >= 6 and fields[5] != b".":
        if fields[5] == b"+":
            strand = "+"
        elif fields[5] == b"-":
            strand = "-"
        else:
            raise ImportError_(f"line {lineno}: invalid strand {fields[5]!r}")
    return {"chrom": chrom, "start": start, "end": end, "barcode": barcode, "count": count,
            "strand": strand, "line": lineno}


def read_records(text: bytes) -> list[dict]:
    lines = text.split(b"\n")
    if lines and lines[-1] == b"":
        lines.pop()          # text ended with a newline
        terminated = len(lines)
    else:
        terminated = len(lines) - 1
    out = []
    for i, ln in enumerate(lines):
        if i < terminated and ln.endswith(b"\r"):
            ln = ln[:-1]
        if ln.startswith(b"#"):
            continue
        out.append(parse_record(ln, i))
    return out


def _sat_add(x: int, s: int) -> int:
    return min(max(x + s, 0), U64_MAX)


def shift_fragment(f: dict, shift_left: int, shift_right: int) -> None:
    """preprocessing.rs:174-184."""
    if shift_left != 0:
        f["start"] = _sat_add(f["start"], shift_left)
        if f["strand"] is not None:
            f["end"] = _sat_add(f["end"], shift_left)
    if shift_right != 0 and f["strand"] is None:
        f["end"] = _sat_add(f["end"], shift_right)


def _wrap_i64(x: int) -> int:
    x &= U64_MAX
    return x - (1 << 64) if x >> 63 else x


def import_fragments(text: bytes, chrom_sizes: dict, *, min_num_fragments: int = 200,
                     sorted_by_barcode: bool = True, whitelist=None, chrM=("chrM", "M"),
                     shift_left: int = 0, shift_right: int = 0) -> dict:
    """The AnnData content the reference writes, as plain arrays.

    Returns a dict with ``key`` ("fragment_paired" / "fragment_single" or None
    when no cell passed), ``obs_names``, ``indptr``, ``indices`` (global base
    index of the fragment start, or of its last base for reverse-strand
    reads), ``data`` (uint32 fragment size, or int32 signed size),
    ``n_fragment``, ``frac_dup``, ``frac_mito``, ``chrom_names`` and
    ``chrom_sizes`` (the reference_sequences table).
    """
    if len(chrom_sizes) == 0:
        raise ValueError("chrom_size cannot be empty")
    names = sorted(chrom_sizes, key=lambda s: s.encode())
    sizes = [int(chrom_sizes[n]) for n in names]
    offset, acc = {}, 0
    for n, s in zip(names, sizes):
        offset[n.encode()] = (acc, s)
        acc += s
    genome_size = acc
    mito = {c.encode() for c in chrM}
    wl = None if whitelist is None else {w.encode() if isinstance(w, str) else bytes(w) for w in whitelist}

    recs = read_records(text)
    for f in recs:
        shift_fragment(f, shift_left, shift_right)
    paired = bool(recs) and recs[0]["strand"] is None

    if not sorted_by_barcode and min_num_fragments > 0:
        counts: dict = {}
        for f in recs:
            if f["barcode"] is None:
                raise ImportError_(f"line {f['line']}: fragment without a barcode")
            counts[f["barcode"]] = counts.get(f["barcode"], 0) + 1
        lst = {k for k, v in counts.items() if v >= min_num_fragments}
        wl = lst if wl is None else lst & wl
    if not sorted_by_barcode:
        recs = sorted(recs, key=lambda f: (f["barcode"] is not None, f["barcode"] or b""))

    # runs of equal barcode over the records with end - start != 0 (import.rs:68-70)
    groups: list[tuple[bytes, list]] = []
    for f in recs:
        if (f["end"] - f["start"]) & U64_MAX == 0:
            continue
        if f["barcode"] is None:
            raise ImportError_(f"line {f['line']}: fragment without a barcode")
        if groups and groups[-1][0] == f["barcode"]:
            groups[-1][1].append(f)
        else:
            groups.append((f["barcode"], [f]))

    scanned: set = set()
    obs_names, rows, qc = [], [], []
    for bc, frags in groups:
        if wl is not None and bc not in wl:
            continue
        unique = total = nmito = 0
        values = []
        for f in frags:                                   # count_fragments, import.rs:161-210
            ch = f["chrom"]
            if ch not in offset:
                continue
            total += f["count"]
            if ch in mito:
                nmito += 1
            else:
                unique += 1
            start, end = _wrap_i64(f["start"]), _wrap_i64(f["end"])
            size = _wrap_i64(end - start)
            base, csize = offset[ch]
            if f["strand"] == "-":
                p, shift = (end - 1) & U64_MAX, -size
            else:
                p, shift = f["start"], size
            if p >= csize:
                raise ImportError_(f"line {f['line']}: position {p} out of range for {ch.decode()}")
            if paired and not 0 <= shift < (1 << 32):
                raise ImportError_(f"line {f['line']}: cannot convert size {shift} to u32")
            if not paired and not -(1 << 31) <= shift < (1 << 31):
                raise ImportError_(f"line {f['line']}: cannot convert size {shift} to i32")
            values.append((base + p, shift))
        values.sort()
        if bc in scanned:                                 # import.rs:145-147
            raise ImportError_("Please sort fragment file by barcodes")
        scanned.add(bc)
        if unique < min_num_fragments:
            continue
        obs_names.append(bc.decode())
        rows.append(values)
        with np.errstate(divide="ignore", invalid="ignore"):
            tot = np.float64(total)
            um = np.float64(unique + nmito)
            qc.append((unique, np.float64(1.0) - um / tot, np.float64(nmito) / um))

    out = {"key": None, "obs_names": obs_names, "chrom_names": names, "chrom_sizes": sizes,
           "genome_size": genome_size, "paired": paired}
    if not rows:
        return out
    indptr = np.zeros(len(rows) + 1, dtype=np.int64)
    indptr[1:] = np.cumsum([len(r) for r in rows])
    flat = [v for r in rows for v in r]
    out.update(
        key="fragment_paired" if paired else "fragment_single",
        indptr=indptr,
        indices=np.array([v[0] for v in flat], dtype=np.int64),
        data=np.array([v[1] for v in flat], dtype=np.uint32 if paired else np.int32),
        n_fragment=np.array([q[0] for q in qc], dtype=np.uint64),
        frac_dup=np.array([q[1] for q in qc], dtype=np.float64),
        frac_mito=np.array([q[2] for q in qc], dtype=np.float64),
    )
    return out


# ---- the same import in C (oracle/fragments.c), for a CPU baseline of realistic speed ----

def import_fragments_c(text: bytes, chrom_sizes: dict, *, min_num_fragments: int = 200,
                       sorted_by_barcode: bool = True, whitelist=None, chrM=("chrM", "M"),
                       shift_left: int = 0, shift_right: int = 0) -> dict:
    """``import_fragments`` through oracle/fragments.c; same result dict."""
    import ctypes
    from ._build import load_lib

    class Out(ctypes.Structure):
        _fields_ = [("n_cells", ctypes.c_int64), ("nnz", ctypes.c_int64), ("paired", ctypes.c_int64),
                    ("bad_line", ctypes.c_int64), ("error", ctypes.c_int64)] + \
                   [(k, ctypes.c_void_p) for k in ("indptr", "indices", "data", "bc_off", "bc_len", "n_fragment",
                                                     "frac_dup", "frac_mito")]

    if len(chrom_sizes) == 0:
        raise ValueError("chrom_size cannot be empty")
    lib = load_lib("fragments")
    f = lib.oracle_import
    P, I64 = ctypes.c_void_p, ctypes.c_int64
    f.restype = I64
    f.argtypes = [ctypes.c_char_p, I64, ctypes.c_char_p, P, P, P, P, ctypes.c_int, ctypes.c_char_p, P, I64,
                  ctypes.c_int, ctypes.c_uint64, ctypes.c_int, I64, I64, ctypes.POINTER(Out)]
    lib.oracle_import_free.argtypes = [ctypes.POINTER(Out)]
    names = sorted(chrom_sizes, key=lambda s: s.encode())
    nb = [n.encode() for n in names]
    coff = np.concatenate([[0], np.cumsum([len(b) for b in nb])]).astype(np.int64)
    csize = np.array([int(chrom_sizes[n]) for n in names], dtype=np.uint64)
    cbase = np.concatenate([[0], np.cumsum(csize)[:-1]]).astype(np.uint64)
    mito = {c.encode() for c in chrM}
    cmito = np.array([b in mito for b in nb], dtype=np.uint8)
    wl = sorted({w.encode() if isinstance(w, str) else bytes(w) for w in whitelist}) if whitelist is not None else []
    woff = np.concatenate([[0], np.cumsum([len(w) for w in wl])]).astype(np.int64)
    o = Out()
    err = f(text, len(text), b"".join(nb), coff.ctypes.data, csize.ctypes.data, cbase.ctypes.data, cmito.ctypes.data,
            len(nb), b"".join(wl), woff.ctypes.data, len(wl), int(whitelist is not None),
            int(max(min_num_fragments, 0)), int(bool(sorted_by_barcode)), int(shift_left), int(shift_right),
            ctypes.byref(o))
    if err:
        raise ImportError_(f"line {o.bad_line}: import error {err}")
    paired = bool(o.paired == 1)
    out = {"key": None, "obs_names": [], "chrom_names": names, "chrom_sizes": [int(x) for x in csize],
           "genome_size": int(csize.sum()), "paired": paired}
    try:
        K, nnz = int(o.n_cells), int(o.nnz)
        if K == 0:
            return out
        arr = lambda ptr, n, dt: np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(dt)), shape=(n,)).copy()  # noqa: E731
        offs = arr(o.bc_off, K, ctypes.c_int64)
        lens = arr(o.bc_len, K, ctypes.c_int32)
        data = arr(o.data, nnz, ctypes.c_int64) if nnz else np.zeros(0, np.int64)
        out.update(
            key="fragment_paired" if paired else "fragment_single",
            obs_names=[text[a:a + b].decode() for a, b in zip(offs.tolist(), lens.tolist())],
            indptr=arr(o.indptr, K + 1, ctypes.c_int64),
            indices=arr(o.indices, nnz, ctypes.c_int64) if nnz else np.zeros(0, np.int64),
            data=data.astype(np.uint32 if paired else np.int32),
            n_fragment=arr(o.n_fragment, K, ctypes.c_uint64),
            frac_dup=arr(o.frac_dup, K, ctypes.c_double),
            frac_mito=arr(o.frac_mito, K, ctypes.c_double))
        return out
    finally:
        lib.oracle_import_free(ctypes.byref(o))
