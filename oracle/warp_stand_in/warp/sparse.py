"""ORACLE test infrastructure: the warp.sparse functions warp_cfd calls, restated for
1x1 blocks (CSR) from Warp's documentation, on the numpy Warp stand-in.

* bsr_from_triplets: a matrix from (row, column, value) triplets, entries sorted by
  row then column, duplicates summed (call sites: FV/terms/equation.py:53-57);
* BsrMatrix.uncompress_rows, bsr_get_diag (equation.py:80-83), bsr_mv (FV/model.py:287);
* _bsr_block_index(row, col, offsets, columns): the entry index of (row, col) or -1
  (FV/kernels/equation_kernels.py:7,114,183).
"""
from __future__ import annotations

import numpy as np

from . import array, int32


class BsrMatrix:
    def __init__(self, nrow, ncol, offsets, columns, values):
        self.nrow = int(nrow)
        self.ncol = int(ncol)
        self.offsets = array(data=offsets, dtype=int32)
        self.columns = array(data=columns, dtype=int32)
        self.values = values
        self.block_shape = (1, 1)

    @property
    def nnz(self):
        return int(self.offsets._data[-1])

    @property
    def shape(self):
        return (self.nrow, self.ncol)

    @property
    def scalar_type(self):
        return self.values.dtype

    def uncompress_rows(self, out=None):
        rows = np.repeat(np.arange(self.nrow, dtype=np.int32), np.diff(self.offsets._data))
        return array(data=rows, dtype=int32)

    def _scipy(self):
        import scipy.sparse as sp

        return sp.csr_matrix((self.values._data, self.columns._data, self.offsets._data), shape=self.shape)


def bsr_from_triplets(rows_of_blocks, cols_of_blocks, rows, columns, values, prune_numerical_zeros=True,
                      masked=False, **kw):
    r = np.asarray(rows._data if isinstance(rows, array) else rows, dtype=np.int64)
    c = np.asarray(columns._data if isinstance(columns, array) else columns, dtype=np.int64)
    v = values._data if isinstance(values, array) else np.asarray(values)
    keep = np.ones(r.shape[0], dtype=bool)
    if prune_numerical_zeros:
        keep &= v != 0
    r, c, v = r[keep], c[keep], v[keep]
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    # duplicates summed, in triplet order
    key = r * int(cols_of_blocks) + c
    uniq, first = np.unique(key, return_index=True)
    summed = np.add.reduceat(v, first) if v.shape[0] else v
    ur, uc = uniq // int(cols_of_blocks), uniq % int(cols_of_blocks)
    offsets = np.zeros(int(rows_of_blocks) + 1, dtype=np.int64)
    np.add.at(offsets, ur + 1, 1)
    offsets = np.cumsum(offsets)
    vals = array(data=summed.astype(v.dtype), dtype=values.dtype if isinstance(values, array) else v.dtype.type)
    return BsrMatrix(rows_of_blocks, cols_of_blocks, offsets.astype(np.int32), uc.astype(np.int32), vals)


def bsr_get_diag(A, out=None):
    d = np.zeros(A.nrow, dtype=A.values._data.dtype)
    rows = A.uncompress_rows()._data
    cols = A.columns._data
    hit = rows == cols
    d[rows[hit]] = A.values._data[hit]
    if out is None:
        return array(data=d, dtype=A.values.dtype)
    out._data[...] = d
    return out


def bsr_mv(A, x, y=None, alpha=1.0, beta=0.0, **kw):
    xv = x._data.reshape(-1)
    res = A._scipy() @ xv
    if y is None:
        return array(data=(alpha * res).astype(xv.dtype), dtype=x.dtype if not hasattr(x.dtype, "_inner_shape")
                     else x.dtype)
    y._data.reshape(-1)[...] = alpha * res + beta * y._data.reshape(-1)
    return y


def _bsr_block_index(row, col, bsr_offsets, bsr_columns):
    lo, hi = int(bsr_offsets[row]), int(bsr_offsets[row + 1])
    cols = bsr_columns._data[lo:hi]
    j = int(np.searchsorted(cols, col))
    if j < cols.shape[0] and int(cols[j]) == int(col):
        return lo + j
    return -1


def bsr_zeros(rows_of_blocks, cols_of_blocks, block_type, device=None):
    return BsrMatrix(rows_of_blocks, cols_of_blocks, np.zeros(rows_of_blocks + 1, np.int32), np.zeros(0, np.int32),
                     array(shape=0, dtype=block_type))
