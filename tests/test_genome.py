"""GenomeIndex against the reference's known-answer vectors
(snapatac2-core/src/genome.rs:496-597, parsed into golden/genome_index.json)."""
import json
import os

import numpy as np

from snapatac2_gb300.genome import GenomeIndex, TileNames
from conftest import GOLDEN

G = json.load(open(os.path.join(GOLDEN, "genome_index.json")))


def test_ranges_and_sizes():
    idx = GenomeIndex([tuple(x) for x in G["chrom_sizes"]])
    for c, a, b in G["ranges"]:
        assert idx.get_range(c) == range(a, b)
    assert [s for _, s in idx.chrom_sizes] == [s for _, s in G["chrom_sizes"]]


def test_regions_and_reverse():
    base = GenomeIndex([tuple(x) for x in G["chrom_sizes"]])
    assert len(G["regions"]) == 14
    for r in G["regions"]:
        idx = base.with_step(r["step"])
        assert idx.get_region(r["index"]) == (r["chrom"], r["start"], r["end"])
        assert idx.get_position_rev(r["chrom"], r["start"]) == r["index"]


def test_coarsed_positions():
    base = GenomeIndex([tuple(x) for x in G["chrom_sizes"]])
    assert len(G["coarsed"]) == 20
    for r in G["coarsed"]:
        idx = base.with_step(r["step"])
        assert idx.get_coarsed_position(r["base"]) == r["index"]
        if r["step"] == 2:
            c, s, _ = base.get_region(r["base"])
            assert idx.get_position_rev(c, s) == r["index"]


def test_position_rev_out_of_range():
    idx = GenomeIndex([("1", 13), ("2", 71)])
    try:
        idx.get_position_rev("1", 13)
    except IndexError:
        pass
    else:
        raise AssertionError("expected IndexError (the reference panics)")


def test_tile_names():
    idx = GenomeIndex([("chr1", 1200), ("chr2", 500)], 500)
    names = TileNames(idx)
    assert len(names) == 4
    assert list(names) == ["chr1:0-500", "chr1:500-1000", "chr1:1000-1200", "chr2:0-500"]
    assert names[-1] == "chr2:0-500"
    assert names[np.array([True, False, False, True])] == ["chr1:0-500", "chr2:0-500"]
