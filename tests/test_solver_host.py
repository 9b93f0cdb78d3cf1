"""Host-side arithmetic of the eigensolver's library calls (CPU: these entry
points touch no device): the Python driver's default basis and thick-restart
size agree with the library's own defaults (the workspace it sizes for
basis 0 equals the one for the Python values), the Rayleigh-Ritz limit caps
the basis, and the row order of the longest-first schedule has the size
sg_row_order writes."""
import pytest

from snapatac2_gb300 import _eigen, _lib


@pytest.mark.parametrize("k", [5, 10, 30, 50])
@pytest.mark.parametrize("block", [4, 8, 16, 32])
@pytest.mark.parametrize("n", [20_000, 100_000, 1_000_000])
def test_default_basis_matches_library(k, block, n):
    L = _lib.load()
    m = 500_000
    M, keep = _eigen._default_basis(k, block, n)
    assert M % block == 0 and keep >= k + 2 * block and M + block <= _eigen.RITZ_MAX
    want = int(L.sg_lanczos_work_bytes(0, block, k, n, m, M, keep))
    assert want > 0
    assert int(L.sg_lanczos_work_bytes(0, block, k, n, m, 0, 0)) == want


def test_default_basis_values():
    assert _eigen._default_basis(30, 16, 100_000) == (384, 96)
    assert _eigen._default_basis(30, 32, 100_000) == (608, 96)  # capped by the 640 limit
    assert _eigen._default_basis(30, 8, 100_000)[1] == 96


def test_row_order_positions():
    L = _lib.load()
    for rows, want in [(0, 0), (1, 4), (4, 4), (5, 8), (500_000, 500_000), (500_001, 500_004)]:
        assert int(L.sg_row_order_positions(rows)) == want
    assert int(L.sg_row_order_positions(-1)) == -1
    assert int(L.sg_row_order_scratch_bytes(500_000)) > 4 * 8 * 500_000
