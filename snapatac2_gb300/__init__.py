"""GB300-native implementation of SnapATAC2's cell-embedding path.

Drop-in API (same names, keywords, defaults and output slots as
``snapatac2.pp`` / ``snapatac2.tl``):

* ``pp.import_fragments`` -- fragment file -> per-cell fragment matrix + QC
                             (parse, group by barcode, sort: GPU)
* ``pp.add_tile_matrix``  -- fragments -> cell x 500 bp tile counts (GPU)
* ``pp.make_peak_matrix`` -- fragments -> cell x peak counts (GPU)
* ``pp.make_gene_matrix`` -- fragments -> cell x gene activity (GPU counting)
* ``pp.select_features``  -- most accessible tiles (column counts on the GPU,
                             ranking on the host with NumPy's tie order)
* ``tl.spectral``         -- matrix-free cosine spectral embedding (GPU)
* ``pp.knn``              -- exact Euclidean kNN graph (GPU)

Beyond the reference:

* ``spectral_batched``    -- many datasets embedded in one stacked solve
* ``topk_eigenvalue_sum`` -- sum of the top-k eigenvalues as a differentiable
                             function of the feature weights (torch.autograd)

All compute goes through ``libsnapgb300.so`` (C ABI in ``include/snapgb300.h``).
"""
from . import genome  # noqa: F401
from ._anndata import AnnData, is_anndata  # noqa: F401


class _Namespace:
    def __init__(self, **kw):
        self.__dict__.update(kw)


def __getattr__(name):
    # lazy namespaces so that importing the package needs neither a GPU nor torch.cuda
    if name == "pp":
        from . import preprocessing as _p
        from . import _knn_api as _k
        from . import _import as _i
        from . import _regions as _r
        from . import _genes as _g
        ns = _Namespace(import_fragments=_i.import_fragments, add_tile_matrix=_p.add_tile_matrix,
                        make_peak_matrix=_r.make_peak_matrix, make_gene_matrix=_g.make_gene_matrix,
                        select_features=_p.select_features, knn=_k.knn,
                        fragments_to_anndata=_p.fragments_to_anndata)
        globals()["pp"] = ns
        return ns
    if name == "tl":
        from . import tools as _t
        ns = _Namespace(spectral=_t.spectral)
        globals()["tl"] = ns
        return ns
    if name == "spectral_batched":
        from ._batched import spectral_batched
        return spectral_batched
    if name == "topk_eigenvalue_sum":
        from ._adjoint import topk_eigenvalue_sum
        return topk_eigenvalue_sum
    raise AttributeError(name)


__version__ = "0.1.0"
