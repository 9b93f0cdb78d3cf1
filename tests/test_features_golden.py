"""select_features ranking against golden vectors of the reference's own
``_find_most_accessible_features`` (``_basic.py:952-967``, run on seeded
counts by ``tests/golden/make_feature_golden.py``), for the oracle's
restatement and for the package's host ranking (CPU).

NumPy's default argsort orders ties in an implementation-defined way that
can differ between NumPy builds for different CPUs; the vectors were made
on x86-64, where the selected indices must match exactly.  Elsewhere the
sequence of selected counts (independent of the tie order) must match."""
import os
import platform

import numpy as np
import pytest

from oracle import features as ofe

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "features.npz"))
N_CASES = sum(1 for k in GOLDEN.files if k.startswith("count"))


def _check(sel, i):
    count, want = GOLDEN[f"count{i}"], GOLDEN[f"selected{i}"]
    sel = np.asarray(sel)
    if platform.machine() in ("x86_64", "AMD64"):
        np.testing.assert_array_equal(sel, want)
    else:
        np.testing.assert_array_equal(count[sel], count[want])


@pytest.mark.parametrize("i", range(N_CASES))
def test_oracle_ranking_matches_reference(i):
    lo, up, tot = GOLDEN[f"params{i}"]
    _check(ofe.most_accessible(GOLDEN[f"count{i}"], lo, up, int(tot)), i)


@pytest.mark.parametrize("i", range(N_CASES))
def test_package_ranking_matches_reference(i):
    from snapatac2_gb300.preprocessing import _find_most_accessible_features
    lo, up, tot = GOLDEN[f"params{i}"]
    _check(_find_most_accessible_features(GOLDEN[f"count{i}"], lo, up, int(tot)), i)
