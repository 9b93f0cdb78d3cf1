"""Argument errors of the drop-in API (CPU): raised before any device work,
with the reference's exception types and messages (``_basic.py:307``,
``_embedding.py:238,243``, ``_knn.py:83``, ``preprocessing.rs:352,361``,
``matrix.rs:270``); options the reference has but this build does not
support raise NotImplementedError instead of differing silently."""
import numpy as np
import pytest
import scipy.sparse as sp

import snapatac2_gb300 as snap


def _adata():
    X = sp.random(50, 40, density=0.2, format="csr", random_state=0, dtype=np.float32)
    return snap.AnnData(X)


@pytest.mark.parametrize("kw,exc,msg", [
    (dict(counting_strategy="bogus"), ValueError, "Counting strategy must be one of"),
    (dict(value_type="bogus"), ValueError, "Value type must be one of 'target', 'total', or 'fraction'"),
    (dict(summary_type="bogus"), ValueError, "Summary type must be one of 'sum', 'mean', or 'count'"),
    (dict(file="out.h5ad"), NotImplementedError, "backed"),
])
def test_add_tile_matrix_arguments(kw, exc, msg):
    with pytest.raises(exc, match=msg):
        snap.pp.add_tile_matrix(_adata(), **kw)


@pytest.mark.parametrize("kw,exc,msg", [
    (dict(sample_size=1), ValueError, "when sample_size is an integer, it should be > 1"),
    (dict(sample_size=1.5), ValueError, "when sample_size is a float, it should be > 0 and <= 1"),
    (dict(sample_size=0.0), ValueError, "when sample_size is a float"),
    (dict(distance_metric="jaccard"), NotImplementedError, "cosine"),
])
def test_spectral_arguments(kw, exc, msg):
    with pytest.raises(exc, match=msg):
        snap.tl.spectral(_adata(), features=None, **kw)


def test_knn_arguments():
    ad = _adata()
    ad.obsm["X_spectral"] = np.random.default_rng(0).standard_normal((50, 5))
    with pytest.raises(ValueError, match="method must be one of 'hora', 'pynndescent', 'kdtree'"):
        snap.pp.knn(ad, method="bogus")
    with pytest.raises(NotImplementedError, match="approximate"):
        snap.pp.knn(ad, method="hora")


def test_select_features_unsupported_options():
    with pytest.raises(NotImplementedError, match="whitelist/blacklist"):
        snap.pp.select_features(_adata(), whitelist="peaks.bed")
    with pytest.raises(NotImplementedError, match="max_iter"):
        snap.pp.select_features(_adata(), max_iter=2)


def test_peak_and_gene_matrix_arguments(tmp_path):
    ad = _adata()
    with pytest.raises(ValueError, match="Counting strategy must be one of"):
        snap.pp.make_peak_matrix(ad, use_rep=["chr1:0-10"], counting_strategy="bogus")
    with pytest.raises(ValueError, match="id_type must be 'transcript' or 'gene'"):
        snap.pp.make_gene_matrix(ad, str(tmp_path / "a.gtf"), id_type="bogus")
    with pytest.raises(NotImplementedError, match="backed"):
        snap.pp.make_peak_matrix(ad, use_rep=["chr1:0-10"], use_x=True, file="out.h5ad")


def test_import_fragments_arguments(tmp_path):
    p = tmp_path / "f.tsv"
    p.write_text("chr1\t10\t50\tAAAC\t1\n")
    with pytest.raises(ValueError, match="chrom_size cannot be empty"):
        snap.pp.import_fragments(str(p), {})
    with pytest.raises(NotImplementedError, match="backed"):
        snap.pp.import_fragments(str(p), {"chr1": 1000}, file=str(tmp_path / "o.h5ad"))


def test_spectral_nystrom_ignores_feature_weights_like_the_reference(monkeypatch):
    """_embedding.py:264 calls the Nystrom path without feature_weights: the
    weights are dropped (with a warning) and IDF is used."""
    from snapatac2_gb300 import _nystrom
    seen = {}

    def fake(X, features, n_comps, sample_size, **kw):
        seen.update(kw)
        return np.array([0.5]), np.zeros((X.shape[0], 1))

    monkeypatch.setattr(_nystrom, "spectral_nystrom", fake)
    ad = _adata()
    with pytest.warns(UserWarning, match="feature_weights are not used"):
        snap.tl.spectral(ad, features=None, sample_size=10, feature_weights=np.ones(40))
    assert seen["feature_weights"] is None and seen["random_state"] == 0


def test_spectral_needs_selected_features():
    with pytest.raises(NameError, match="Please call `select_features` first"):
        snap.tl.spectral(_adata())
