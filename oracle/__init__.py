"""ORACLE -- test infrastructure only.

CPU restatements of the reference's arithmetic on the cell-embedding path,
used for comparison by ``tests/``, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py``.  Nothing in the ``snapatac2_gb300``
package imports this package.

* ``binning``  -- tile binning (``gen_mat_pair`` / ``gen_mat_single``), C + NumPy
* ``spectral`` -- IDF weights, row normalisation, degree, ARPACK ``eigsh``
* ``knn``      -- exact kNN graph, C (OpenMP) brute force in FP64
* ``features`` -- ``select_features`` ranking
* ``fragments`` -- ``import_fragments``, Python + C
* ``regions``  -- cell-by-region counts (peak matrix), Python + C (OpenMP)
* ``genes``    -- annotation reading, promoter regions, gene-level maximum
* ``nystrom``  -- Nyström extension and ``orthogonalize``
"""
from ._build import build_oracle, load_lib  # noqa: F401
