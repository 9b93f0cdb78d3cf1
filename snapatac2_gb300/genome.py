"""Genome coordinate <-> tile index arithmetic (host side).

Mirrors the reference's ``GenomeBaseIndex`` (``snapatac2-core/src/genome.rs:288-484``):
a list of chromosomes with cumulative base lengths and, for a tile size
``step``, cumulative tile counts ``ceil(len / step)``.  The same tables are
uploaded to the GPU binning kernel (``binned_offsets``), so the host methods
here and the kernel agree by construction.
"""
from __future__ import annotations

from typing import Iterable, Sequence

import numpy as np


class ChromSizes:
    """Ordered (name, length) pairs; ``snapatac2-core/src/genome.rs`` ``ChromSizes``."""

    def __init__(self, items: Iterable[tuple[str, int]] | dict):
        if isinstance(items, dict):
            items = items.items()
        self.names: list[str] = []
        self.sizes: list[int] = []
        for n, s in items:
            self.names.append(str(n))
            self.sizes.append(int(s))
        if len(set(self.names)) != len(self.names):
            raise ValueError("duplicate chromosome names")

    def __len__(self) -> int:
        return len(self.names)

    def __iter__(self):
        return iter(zip(self.names, self.sizes))

    def total_size(self) -> int:
        return int(sum(self.sizes))

    def to_dict(self) -> dict:
        return dict(zip(self.names, self.sizes))


class GenomeIndex:
    """0-based index mapping genomic loci to integers (``genome.rs:288-293``).

    ``base_accum`` holds cumulative chromosome lengths, ``binned_accum`` the
    cumulative number of tiles of size ``step`` (``with_step``,
    ``genome.rs:365-384``).
    """

    def __init__(self, chrom_sizes: ChromSizes | Sequence[tuple[str, int]] | dict, step: int = 1):
        if not isinstance(chrom_sizes, ChromSizes):
            chrom_sizes = ChromSizes(chrom_sizes)
        self.chrom_sizes = chrom_sizes
        self.names = list(chrom_sizes.names)
        self._pos = {n: i for i, n in enumerate(self.names)}
        sizes = np.asarray(chrom_sizes.sizes, dtype=np.uint64)
        self.sizes = sizes
        self.base_accum = np.cumsum(sizes, dtype=np.uint64)
        self.step = int(step)
        nb = (sizes + np.uint64(step - 1)) // np.uint64(step)
        self.binned_accum = np.cumsum(nb, dtype=np.uint64)

    def with_step(self, s: int) -> "GenomeIndex":
        return GenomeIndex(self.chrom_sizes, s)

    def __len__(self) -> int:
        return int(self.binned_accum[-1]) if len(self.binned_accum) else 0

    def contain_chrom(self, chrom: str) -> bool:
        return chrom in self._pos

    def get_range(self, chrom: str) -> range | None:
        """Tile index range of a chromosome (``genome.rs:315-324``)."""
        i = self._pos.get(chrom)
        if i is None:
            return None
        start = int(self.binned_accum[i - 1]) if i else 0
        return range(start, int(self.binned_accum[i]))

    def get_position_rev(self, chrom: str, pos: int) -> int:
        """(chrom, 0-based position) -> tile index (``genome.rs:387-406``)."""
        i = self._pos.get(chrom)
        if i is None:
            raise KeyError(f"Chromosome {chrom} not found")
        if pos >= int(self.sizes[i]) or pos < 0:
            raise IndexError(f"Position {pos} is out of range for chromosome {chrom}")
        base = int(self.binned_accum[i - 1]) if i else 0
        return base + pos // self.step

    def _locate(self, idx: int) -> tuple[int, int]:
        # first chromosome whose cumulative tile count exceeds idx (genome.rs:419-434)
        j = int(np.searchsorted(self.binned_accum, np.uint64(idx), side="right"))
        if j >= len(self.names):
            raise IndexError(f"index {idx} is past the end of the genome")
        prev = int(self.binned_accum[j - 1]) if j else 0
        return j, idx - prev

    def get_position(self, idx: int) -> tuple[str, int]:
        """Tile index -> (chrom, start position of the tile)."""
        j, r = self._locate(idx)
        return self.names[j], r * self.step

    def get_region(self, idx: int) -> tuple[str, int, int]:
        """Tile index -> (chrom, start, end); the last tile is truncated (``genome.rs:437-466``)."""
        j, r = self._locate(idx)
        start = r * self.step
        end = min(start + self.step, int(self.sizes[j]))
        return self.names[j], start, end

    def get_coarsed_position(self, pos: int) -> int:
        """Base index -> tile index (``genome.rs:469-484``)."""
        if self.step <= 1:
            return int(pos)
        j = int(np.searchsorted(self.base_accum, np.uint64(pos), side="right"))
        acc = int(self.base_accum[j - 1]) if j else 0
        acc_low = int(self.binned_accum[j - 1]) if j else 0
        return acc_low + (int(pos) - acc) // self.step

    def binned_offsets(self) -> np.ndarray:
        """First tile index of every chromosome (uint64)."""
        out = np.zeros(len(self.names), dtype=np.uint64)
        out[1:] = self.binned_accum[:-1]
        return out


class TileNames(Sequence):
    """Lazy ``var_names`` of a tile matrix: ``chrom:start-end`` per tile.

    The reference builds an interval index (``GenomeBaseIndex::to_index``,
    ``genome.rs:326-338``); its names are ``chr1:0-500``, ``chr1:500-1000`` ...
    with the last tile of a chromosome ending at the chromosome length.
    Names are produced on demand instead of materialising ~6M strings.
    """

    def __init__(self, index: GenomeIndex):
        self._index = index

    def __len__(self) -> int:
        return len(self._index)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[j] for j in range(*i.indices(len(self)))]
        if isinstance(i, (np.ndarray, list)):
            a = np.asarray(i)
            if a.dtype == bool:
                a = np.flatnonzero(a)
            return [self[int(j)] for j in a]
        n = len(self)
        i = int(i)
        if i < 0:
            i += n
        if not 0 <= i < n:
            raise IndexError(i)
        c, s, e = self._index.get_region(i)
        return f"{c}:{s}-{e}"

    def to_numpy(self) -> np.ndarray:
        return np.array([self[i] for i in range(len(self))], dtype=object)


def parse_region(txt: str) -> tuple[str, int, int]:
    """Parse ``chrom:start-end``."""
    chrom, rng = txt.rsplit(":", 1)
    s, e = rng.split("-")
    return chrom, int(s), int(e)
