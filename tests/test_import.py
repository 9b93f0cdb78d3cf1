"""snap.pp.import_fragments: the oracle on hand-made files (CPU), the GPU
import against the oracle on synthetic files (GPU), and the reference's own
import properties (``snapatac2-python/tests/test_tools.py:127-141``: export
after import gives back the input records; ``test_pipeline.py:10-31``:
chromosomes dropped at import equal chromosomes excluded at binning)."""
import numpy as np
import pytest

from oracle import fragments as ofr

GENOME = {"chr2": 5000, "chr1": 10000, "chr10": 3000, "chrM": 500}


def _text(lines, nl="\n", trailing=True):
    s = nl.join(lines) + (nl if trailing else "")
    return s.encode()


# ---- oracle (CPU) --------------------------------------------------------------

def test_oracle_chrom_order_and_positions():
    t = _text(["chr2\t10\t20\tA\t1", "chr1\t5\t9\tA\t1", "chr10\t0\t4\tA\t1"])
    r = ofr.import_fragments(t, GENOME, min_num_fragments=0)
    assert r["chrom_names"] == ["chr1", "chr10", "chr2", "chrM"]   # byte order (BTreeMap)
    # chr1 at 0, chr10 at 10000, chr2 at 13000
    assert r["indices"].tolist() == [5, 10000, 13010]
    assert r["data"].tolist() == [4, 4, 10] and r["data"].dtype == np.uint32
    assert r["key"] == "fragment_paired"


def test_oracle_qc_and_filters():
    lines = ["# header", "chr1\t1\t5\tB\t3", "chr1\t2\t9\tB\t.", "chrM\t1\t3\tB\t2", "chrUn\t1\t3\tB\t9",
             "chr1\t4\t4\tB\t1",                                   # zero length: dropped before grouping
             "chr2\t1\t2\tA\t1"]
    r = ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0)
    assert r["obs_names"] == ["B", "A"]                           # first-appearance order (sorted input)
    assert r["n_fragment"].tolist() == [2, 1]
    # B: unique 2, mito 1, total count 3 + 1 + 2 = 6 (chrUn is outside the genome)
    assert r["frac_dup"][0] == 1.0 - 3.0 / 6.0
    assert r["frac_mito"][0] == 1.0 / 3.0
    assert r["indptr"].tolist() == [0, 3, 4]
    r2 = ofr.import_fragments(_text(lines), GENOME, min_num_fragments=2)
    assert r2["obs_names"] == ["B"]
    r3 = ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0, whitelist=["A"])
    assert r3["obs_names"] == ["A"]


def test_oracle_unsorted_input():
    lines = ["chr1\t1\t5\tB\t1", "chr1\t1\t5\tA\t1", "chr1\t2\t5\tB\t1"]
    with pytest.raises(ValueError, match="Please sort"):
        ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0)
    r = ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0, sorted_by_barcode=False)
    assert r["obs_names"] == ["A", "B"]
    # a non-whitelisted barcode may repeat
    r = ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0, whitelist=["A"])
    assert r["obs_names"] == ["A"]


def test_oracle_single_end_and_shifts():
    lines = ["chr1\t10\t20\tA\t1\t+", "chr1\t10\t20\tA\t1\t-", "chr1\t30\t40\tA\t1\t."]
    r = ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0)
    assert r["key"] == "fragment_single" and r["data"].dtype == np.int32
    # "-": position of the last base (19), value -size; "." on a single-end file: +size
    assert list(zip(r["indices"].tolist(), r["data"].tolist())) == [(10, 10), (19, -10), (30, 10)]
    r = ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0, shift_left=4, shift_right=-3)
    # stranded: start and end both + shift_left; unstranded: start + 4, end - 3
    assert list(zip(r["indices"].tolist(), r["data"].tolist())) == [(14, 10), (23, -10), (34, 3)]


def test_oracle_line_endings_and_errors():
    crlf = _text(["chr1\t1\t5\tA\t1", "chr1\t2\t6\tA\t1"], nl="\r\n", trailing=False)
    r = ofr.import_fragments(crlf, GENOME, min_num_fragments=0)
    assert r["indices"].tolist() == [1, 2]
    for bad in (["chr1\t1"], ["chr1\tx\t5\tA"], ["chr1\t1\t5\tA\t1\t*"], [""], ["chr1\t1\t5\t.\t1"]):
        with pytest.raises(ValueError):
            ofr.import_fragments(_text(bad), GENOME, min_num_fragments=0)
    with pytest.raises(ValueError, match="out of range"):
        ofr.import_fragments(_text(["chr10\t3000\t3005\tA\t1"]), GENOME, min_num_fragments=0)
    with pytest.raises(ValueError, match="u32"):
        ofr.import_fragments(_text(["chr1\t9\t5\tA\t1"]), GENOME, min_num_fragments=0)
    # errors in records that are never processed do not count
    r = ofr.import_fragments(_text(["chr1\t9\t5\tA\t1", "chr1\t1\t5\tB\t1"]), GENOME, min_num_fragments=0,
                             whitelist=["B"])
    assert r["obs_names"] == ["B"]


# ---- GPU against the oracle ---------------------------------------------------------

def _check_same(res, ref):
    assert res.key == ref["key"]
    assert res.obs_names == ref["obs_names"]
    if ref["key"] is None:
        return
    np.testing.assert_array_equal(res.indptr, ref["indptr"])
    np.testing.assert_array_equal(res.indices, ref["indices"])
    assert res.data.dtype == ref["data"].dtype
    np.testing.assert_array_equal(res.data, ref["data"])
    np.testing.assert_array_equal(res.n_fragment, ref["n_fragment"])
    np.testing.assert_array_equal(res.frac_dup, ref["frac_dup"])      # bit for bit (NaN == NaN)
    np.testing.assert_array_equal(res.frac_mito, ref["frac_mito"])
    assert res.chrom_sizes.names == ref["chrom_names"]


def _synthetic(n_cells=40, median=300, order="position", single_end=False, seed=3):
    from snapatac2_gb300 import synthetic as S
    g = S.make_genome(total=20_000_000, n_chrom=24)
    fr = S.make_fragments(n_cells, g, median_frags=median, seed=seed, enriched_bins=2000)
    t = S.fragment_text(fr, g, order=order, single_end=single_end, seed=seed)
    return bytes(t.numpy()), S.fragment_genome(g)


CASES = [
    dict(order="position", kw=dict(sorted_by_barcode=False, min_num_fragments=100)),
    dict(order="position", kw=dict(sorted_by_barcode=False, min_num_fragments=0)),
    dict(order="barcode", kw=dict(sorted_by_barcode=True, min_num_fragments=200)),
    dict(order="barcode", kw=dict(sorted_by_barcode=True, min_num_fragments=0, shift_left=-4, shift_right=5)),
    dict(order="shuffle", kw=dict(sorted_by_barcode=False, min_num_fragments=150, chrM=["chrM", "M"])),
    dict(order="barcode", single_end=True, kw=dict(sorted_by_barcode=True, min_num_fragments=10, shift_left=3)),
    dict(order="position", single_end=True, kw=dict(sorted_by_barcode=False, min_num_fragments=0)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(CASES)))
def test_gpu_import_matches_oracle(case):
    from snapatac2_gb300 import _import
    c = CASES[case]
    text, genome = _synthetic(order=c["order"], single_end=c.get("single_end", False), seed=case)
    ref = ofr.import_fragments(text, genome, **c["kw"])
    res = _import.import_text(text, genome, **c["kw"])
    assert res.info["rehash"] == 0
    _check_same(res, ref)


@pytest.mark.gpu
def test_gpu_import_whitelist_and_edge_files():
    from snapatac2_gb300 import _import
    text, genome = _synthetic(order="barcode", seed=11)
    names = ofr.import_fragments(text, genome, min_num_fragments=0)["obs_names"]
    wl = names[::3] + ["NOT-A-BARCODE", names[1][:-1]]
    for kw in (dict(whitelist=wl, min_num_fragments=0), dict(whitelist=wl, min_num_fragments=250),
               dict(whitelist=[], min_num_fragments=0)):
        _check_same(_import.import_text(text, genome, **kw), ofr.import_fragments(text, genome, **kw))
    small = [
        _text(["chr1\t1\t5\tA\t1", "chr1\t2\t6\tA\t1"], nl="\r\n", trailing=False),
        _text(["# only a comment"]),
        b"",
        _text(["chr1\t1\t5\tA\t1", "chr1\t4\t4\tB\t1", "chrUn\t1\t5\tC\t1"]),
        _text(["chr1\t1\t5\tA\t1\t.\textra\tfields", "chr2\t1\t2\tA"]),
        _text(["chr1\t1\t5\tB\t0", "chrM\t1\t2\tA\t0"]),                    # total count 0: NaN / inf
        _text(["chr1\t9\t5\tA\t1\t-", "chr2\t0\t7\tA\t1\t+"]),             # end < start on a single-end file
    ]
    for t in small:
        kw = dict(min_num_fragments=0)
        _check_same(_import.import_text(t, GENOME, **kw), ofr.import_fragments(t, GENOME, **kw))


@pytest.mark.gpu
def test_gpu_import_errors():
    from snapatac2_gb300 import _import
    cases = [
        (["chr1\t1\t5\tB\t1", "chr1\t1\t5\tA\t1", "chr1\t2\t5\tB\t1"], "Please sort"),
        (["chr1\t1\t5\tA\t1", "chr1\tx\t5\tA"], "malformed.*line 2"),
        (["chr1\t1\t5\tA\t1", "chr1\t1\t5\t.\t1"], "malformed.*line 2"),
        (["chr10\t3000\t3005\tA\t1"], "out of range"),
        (["chr1\t9\t5\tA\t1"], "value type"),
        (["chr1\t10\t13\tA\t1"], "value type", dict(shift_left=4, shift_right=-5)),  # shifts invert it
    ]
    for lines, msg, *kw in cases:
        kw = kw[0] if kw else {}
        with pytest.raises(ValueError):
            ofr.import_fragments(_text(lines), GENOME, min_num_fragments=0, **kw)
        with pytest.raises(ValueError, match=msg):
            _import.import_text(_text(lines), GENOME, min_num_fragments=0, **kw)


def test_c_oracle_roundtrip():
    """test_tools.py:127-141 on the oracle (CPU): the imported fragments,
    exported back to records, are the file's records."""
    text, genome = _synthetic(n_cells=30, order="position", seed=21)
    res = ofr.import_fragments_c(text, genome, min_num_fragments=0, sorted_by_barcode=False)
    names, sizes = res["chrom_names"], res["chrom_sizes"]
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    got = []
    for r, bc in enumerate(res["obs_names"]):
        lo, hi = res["indptr"][r], res["indptr"][r + 1]
        for p, v in zip(res["indices"][lo:hi], res["data"][lo:hi]):
            c = int(np.searchsorted(starts, p, side="right") - 1)
            got.append((names[c], int(p - starts[c]), int(p - starts[c] + v), bc))
    want = [tuple(f[:1]) + (int(f[1]), int(f[2]), f[3]) for f in
            (ln.split("\t") for ln in text.decode().splitlines() if not ln.startswith("#"))]
    assert len(got) > 1000 and sorted(got) == sorted(want)


@pytest.mark.gpu
def test_gpu_import_roundtrip_and_exclude():
    """test_tools.py:127-141 and test_pipeline.py:10-31 on a synthetic file."""
    import snapatac2_gb300 as snap
    from snapatac2_gb300 import _import
    text, genome = _synthetic(n_cells=30, order="position", seed=21)
    res = _import.import_text(text, genome, min_num_fragments=0, sorted_by_barcode=False)
    names = res.chrom_sizes.names
    starts = np.concatenate([[0], np.cumsum(res.chrom_sizes.sizes)[:-1]])
    got = []
    for r, bc in enumerate(res.obs_names):
        for p, v in zip(res.indices[res.indptr[r]:res.indptr[r + 1]], res.data[res.indptr[r]:res.indptr[r + 1]]):
            c = int(np.searchsorted(starts, p, side="right") - 1)
            got.append((names[c], int(p - starts[c]), int(p - starts[c] + v), bc))
    want = []
    for ln in text.decode().splitlines():
        if ln.startswith("#"):
            continue
        f = ln.split("\t")
        want.append((f[0], int(f[1]), int(f[2]), f[3]))
    assert sorted(got) == sorted(want)

    sub = {k: v for k, v in genome.items() if k not in ("chr1", "chr10")}
    a1 = _import.to_anndata(_import.import_text(text, sub, min_num_fragments=0, sorted_by_barcode=False))
    a2 = _import.to_anndata(_import.import_text(text, genome, min_num_fragments=0, sorted_by_barcode=False))
    snap.pp.add_tile_matrix(a1, exclude_chroms=None)
    snap.pp.add_tile_matrix(a2, exclude_chroms=["chr1", "chr10"])
    np.testing.assert_array_equal(a1.X.data, a2.X.data)
    assert list(a1.obs_names) == list(a2.obs_names)
    assert list(a1.var_names) == list(a2.var_names)


@pytest.mark.gpu
def test_gpu_import_file_api(tmp_path):
    import gzip
    import snapatac2_gb300 as snap
    text, genome = _synthetic(n_cells=25, order="position", seed=5)
    p = tmp_path / "frags.tsv.gz"
    with gzip.open(p, "wb") as fh:
        fh.write(text)
    ad = snap.pp.import_fragments(str(p), genome, sorted_by_barcode=False, min_num_fragments=50)
    ref = ofr.import_fragments(text, genome, sorted_by_barcode=False, min_num_fragments=50)
    assert list(ad.obs_names) == ref["obs_names"]
    m = ad.obsm["fragment_paired"]
    np.testing.assert_array_equal(m.indices, ref["indices"])
    np.testing.assert_array_equal(ad.obs["frac_dup"], ref["frac_dup"])
    assert list(ad.uns["reference_sequences"]["reference_seq_name"]) == ref["chrom_names"]


@pytest.mark.gpu
def test_gpu_import_device_text_and_plain_file(tmp_path):
    """Text already on the device (barcodes read back from it) and a plain,
    uncompressed file read straight into pinned memory."""
    import torch
    import snapatac2_gb300 as snap
    from snapatac2_gb300 import _import
    text, genome = _synthetic(n_cells=15, order="shuffle", seed=8)
    kw = dict(sorted_by_barcode=False, min_num_fragments=20)
    ref = ofr.import_fragments(text, genome, **kw)
    d = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda()
    _check_same(_import.import_text(d, genome, **kw), ref)
    p = tmp_path / "frags.tsv"
    p.write_bytes(text)
    ad = snap.pp.import_fragments(str(p), genome, **kw)
    assert list(ad.obs_names) == ref["obs_names"]
    np.testing.assert_array_equal(ad.obsm["fragment_paired"].data, ref["data"])


@pytest.mark.gpu
@pytest.mark.parametrize("n,bits", [(1, 64), (1000, 64), (5000, 13), (70000, 40), (300001, 64)])
def test_gpu_radix_sort_stable(n, bits):
    import ctypes
    import torch
    from snapatac2_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2 ** 63, n, dtype=np.int64).view(np.uint64)
    if n > 10:
        keys[: n // 3] = keys[0]  # many equal keys: stability matters
    vals = np.arange(n, dtype=np.uint64)
    dev = torch.device("cuda")
    k = torch.from_numpy(keys.view(np.int64)).to(dev)
    v = torch.from_numpy(vals.view(np.int64)).to(dev)
    ka, va = torch.empty_like(k), torch.empty_like(v)
    scr = torch.empty(int(L.sg_radix_scratch_bytes(n)), dtype=torch.uint8, device=dev)
    alt = ctypes.c_int(0)
    _lib.check(L.sg_radix_sort_u64(n, k.data_ptr(), v.data_ptr(), ka.data_ptr(), va.data_ptr(), 0, bits,
                                   scr.data_ptr(), ctypes.byref(alt), torch.cuda.current_stream().cuda_stream),
               "sg_radix_sort_u64")
    rk, rv = (ka, va) if alt.value else (k, v)
    masked = keys & np.uint64((1 << bits) - 1 if bits < 64 else 2 ** 64 - 1)
    order = np.argsort(masked, kind="stable")
    np.testing.assert_array_equal(rv.cpu().numpy().view(np.uint64), order.astype(np.uint64))
    np.testing.assert_array_equal(rk.cpu().numpy().view(np.uint64), keys[order])


# ---- the two oracle restatements (Python, C) agree (CPU) ---------------------------

def _same_oracle(a, b):
    assert a["key"] == b["key"] and a["obs_names"] == b["obs_names"] and a["paired"] == b["paired"]
    if a["key"] is None:
        return
    for k in ("indptr", "indices", "data", "n_fragment", "frac_dup", "frac_mito"):
        assert a[k].dtype == b[k].dtype, k
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_c_oracle_matches_python_oracle(case):
    c = CASES[case]
    text, genome = _synthetic(n_cells=25, order=c["order"], single_end=c.get("single_end", False), seed=case + 40)
    try:
        ref = ofr.import_fragments(text, genome, **c["kw"])
    except ValueError:  # the data make the reference panic (e.g. a shift past a chromosome end): so must C
        with pytest.raises(ValueError):
            ofr.import_fragments_c(text, genome, **c["kw"])
        return
    _same_oracle(ref, ofr.import_fragments_c(text, genome, **c["kw"]))


def test_c_oracle_edge_files_and_errors():
    small = [
        _text(["chr1\t1\t5\tA\t1", "chr1\t2\t6\tA\t1"], nl="\r\n", trailing=False),
        _text(["# only a comment"]), b"",
        _text(["chr1\t1\t5\tA\t1", "chr1\t4\t4\tB\t1", "chrUn\t1\t5\tC\t1"]),
        _text(["chr1\t1\t5\tA\t1\t.\textra\tfields", "chr2\t1\t2\tA"]),
        _text(["chr1\t1\t5\tB\t0", "chrM\t1\t2\tA\t0"]),
        _text(["chr1\t9\t5\tA\t1\t-", "chr2\t0\t7\tA\t1\t+"]),
    ]
    for t in small:
        for kw in (dict(min_num_fragments=0), dict(min_num_fragments=1, sorted_by_barcode=False),
                   dict(min_num_fragments=0, whitelist=["A"])):
            _same_oracle(ofr.import_fragments(t, GENOME, **kw), ofr.import_fragments_c(t, GENOME, **kw))
    for lines in (["chr1\t1\t5\tB\t1", "chr1\t1\t5\tA\t1", "chr1\t2\t5\tB\t1"], ["chr1\tx\t5\tA"],
                  ["chr1\t1\t5\t.\t1"], ["chr10\t3000\t3005\tA\t1"], ["chr1\t9\t5\tA\t1"]):
        with pytest.raises(ValueError):
            ofr.import_fragments_c(_text(lines), GENOME, min_num_fragments=0)
