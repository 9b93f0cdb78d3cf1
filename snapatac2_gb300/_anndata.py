"""A minimal in-memory AnnData stand-in.

The reference operates on ``anndata.AnnData`` or its own Rust-backed
``AnnData`` (``snapatac2-python/src/utils/anndata.rs:175-236``).  Neither
``anndata`` nor ``pandas`` is available here, so this class provides the
slots the cell-embedding path reads and writes, with the same names:

``X`` (scipy CSR), ``obs`` / ``var`` (dicts of columns), ``obs_names``,
``var_names``, ``obsm``, ``obsp``, ``uns``, ``n_obs``, ``n_vars``, ``shape``.

Any object exposing those attributes (for example a real ``anndata.AnnData``)
is accepted by the functions of this package.
"""
from __future__ import annotations

from typing import Any

import numpy as np


class _Columns(dict):
    """dict of equal-length columns with ``in`` and ``[]`` like a DataFrame."""

    def __init__(self, n: int, data: dict | None = None):
        super().__init__()
        self._n = n
        for k, v in (data or {}).items():
            self[k] = v

    def __setitem__(self, k, v):
        v = np.asarray(v)
        if v.ndim == 0:
            v = np.full(self._n, v)
        if v.shape[0] != self._n:
            raise ValueError(f"column {k!r} has length {v.shape[0]}, expected {self._n}")
        super().__setitem__(k, v)

    def to_numpy(self) -> dict:
        return dict(self)


class AnnData:
    def __init__(self, X=None, *, obs: dict | None = None, var: dict | None = None,
                 obsm: dict | None = None, obsp: dict | None = None, uns: dict | None = None,
                 obs_names=None, var_names=None, n_obs: int | None = None, n_vars: int | None = None):
        if X is not None:
            n_obs, n_vars = X.shape
        if n_obs is None:
            if obs_names is not None:
                n_obs = len(obs_names)
            elif obsm:
                n_obs = next(iter(obsm.values())).shape[0]
            else:
                n_obs = 0
        self._n_obs = int(n_obs)
        self._n_vars = int(n_vars or 0)
        self.X = X
        self.obs = _Columns(self._n_obs, obs)
        self.var = _Columns(self._n_vars, var)
        self.obsm: dict[str, Any] = dict(obsm or {})
        self.obsp: dict[str, Any] = dict(obsp or {})
        self.uns: dict[str, Any] = dict(uns or {})
        self.obs_names = obs_names if obs_names is not None else [str(i) for i in range(self._n_obs)]
        self._var_names = var_names
        self.isbacked = False

    # -- shape ------------------------------------------------------------
    @property
    def n_obs(self) -> int:
        return self._n_obs

    @property
    def n_vars(self) -> int:
        return self._n_vars

    @property
    def shape(self) -> tuple[int, int]:
        return (self._n_obs, self._n_vars)

    @property
    def var_names(self):
        if self._var_names is None:
            return [str(i) for i in range(self._n_vars)]
        return self._var_names

    @var_names.setter
    def var_names(self, v):
        self._var_names = v

    def set_n_vars(self, n: int) -> None:
        """Resize the var axis (drops var columns), as the reference does when X is replaced."""
        self._n_vars = int(n)
        self.var = _Columns(self._n_vars)

    def __repr__(self) -> str:
        parts = [f"AnnData object with n_obs × n_vars = {self.n_obs} × {self.n_vars}"]
        for name in ("obs", "var", "uns", "obsm", "obsp"):
            keys = list(getattr(self, name).keys())
            if keys:
                parts.append(f"    {name}: " + ", ".join(repr(k) for k in keys))
        return "\n".join(parts)


def is_anndata(x) -> bool:
    """Duck-typed check (``snapatac2-python/python/snapatac2/_utils.py:7-8``)."""
    return hasattr(x, "obsm") and hasattr(x, "n_obs") and hasattr(x, "uns")
