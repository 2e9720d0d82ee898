"""Run the reference's own gen_FFT_PowerSpectra (simulations/Utilities/glow_up.py:632-847)
on frame files, in this container, to make the power-spectrum golden fixture.

FIXTURE GENERATION ONLY (called by gen_golden.py --spectrum); tests read the
.npz it produces and never import this file.

glow_up.py imports packages this container does not have.  They are replaced
here by stand-ins in sys.modules before the import:
  pandas   a minimal DataFrame/Series with exactly the operations
           gen_FFT_PowerSpectra uses (read_csv of a frame file, column access,
           insert, filter(like=), replace, mean(axis=1) skipping NaN); columns
           of unequal length are aligned on the row index and padded with NaN,
           as pandas does
  skimage  an empty skimage.metrics (imported at module level, unused here)
Everything else glow_up.py imports (numpy, scipy, scikit-learn, joblib,
regex, psutil, its own slick.py) is the real package.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np


# ------------------------------------------------------------ pandas stand-in
class Series:
    def __init__(self, data=None, dtype=None):
        self.values = np.zeros(0) if data is None else np.asarray(data, dtype=np.float64 if dtype is None else dtype)

    def __len__(self):
        return len(self.values)

    def replace(self, a, b):
        v = self.values.astype(np.float64).copy()
        v[v == a] = b
        return Series(v)

    def dropna(self):
        return Series(self.values[~np.isnan(self.values)])

    def to_numpy(self, dtype=None):
        return self.values.astype(dtype) if dtype is not None else self.values


class DataFrame:
    def __init__(self, data=None, columns=None):
        self._cols: dict[str, Series] = {}
        if isinstance(data, dict):
            for k, v in data.items():
                self._cols[k] = v if isinstance(v, Series) else Series(v)
        for c in columns or []:
            self._cols.setdefault(c, Series())

    @property
    def columns(self):
        return list(self._cols.keys())

    @columns.setter
    def columns(self, names):
        self._cols = dict(zip(names, self._cols.values()))

    def _nrows(self):
        return max((len(s) for s in self._cols.values()), default=0)

    def _padded(self, s, n):
        v = np.full(n, np.nan)
        v[:len(s)] = s.values
        return v

    def __getitem__(self, key):
        if isinstance(key, list):
            return DataFrame({k: self._cols[k] for k in key})
        return self._cols[key]

    def __setitem__(self, key, val):
        self._cols[key] = val if isinstance(val, Series) else Series(val)

    def insert(self, loc, name, val):
        items = list(self._cols.items())
        items.insert(loc, (name, val if isinstance(val, Series) else Series(val)))
        self._cols = dict(items)

    def filter(self, like):
        return DataFrame({k: v for k, v in self._cols.items() if like in k})

    def replace(self, a, b):
        return DataFrame({k: v.replace(a, b) for k, v in self._cols.items()})

    def mean(self, axis=0):
        assert axis == 1
        n = self._nrows()
        if not self._cols:
            return Series(np.full(n, np.nan))
        m = np.stack([self._padded(s, n) for s in self._cols.values()], axis=1)
        with np.errstate(invalid="ignore"):
            cnt = np.sum(~np.isnan(m), axis=1)
            tot = np.nansum(m, axis=1)
            return Series(np.where(cnt > 0, tot / np.maximum(cnt, 1), np.nan))

    def column_array(self, key):
        return self._padded(self._cols[key], self._nrows())


def read_csv(path, header=0, **_kw):
    with open(path) as f:
        names = f.readline().rstrip("\n").split(",")
        rows = [ln.rstrip("\n").split(",") for ln in f if ln.strip()]
    cols = list(zip(*rows)) if rows else [[] for _ in names]
    if len(names) > len(cols):      # a trailing separator in the header
        names = names[:len(cols)]
    return DataFrame({n: Series(np.array([float(x) for x in c])) for n, c in zip(names, cols)})


def _install_stand_ins():
    pd = types.ModuleType("pandas")
    pd.DataFrame, pd.Series, pd.read_csv = DataFrame, Series, read_csv
    pd.read_table = read_csv
    sys.modules["pandas"] = pd
    sk = types.ModuleType("skimage")
    skm = types.ModuleType("skimage.metrics")
    skm.structural_similarity = None
    sk.metrics = skm
    sys.modules["skimage"] = sk
    sys.modules["skimage.metrics"] = skm


def load_glow_up(ref_root, home):
    """Import the reference's glow_up module with the stand-ins above.  glow_up
    makes a cache folder under ~ at import; `home` (a scratch folder the caller
    removes) stands in for ~ so nothing is written outside it."""
    _install_stand_ins()
    os.environ["HOME"] = home
    sys.dont_write_bytecode = True
    util = os.path.join(ref_root, "simulations", "Utilities")
    sys.path.insert(0, util)
    import glow_up  # noqa: E402  (the reference's module, unmodified)
    return glow_up


def spectrum_of_frame(glow_up, path, binwidth=0.5):
    """gen_FFT_PowerSpectra on one frame file; returns (k, power) of its single
    field column (the reference marks empty bins NaN)."""
    df = glow_up.gen_FFT_PowerSpectra([path], pathtodir=os.path.dirname(path), ext="csv", binwidth=binwidth)
    kcol = [c for c in df.columns if c.startswith("k_R_")][0]
    pcol = [c for c in df.columns if c.startswith("POWER[") and "_R_" in c and "MEAN" not in c][0]
    return df.column_array(kcol), df.column_array(pcol)
