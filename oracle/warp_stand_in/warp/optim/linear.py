"""ORACLE test infrastructure: warp.optim.linear (cg, bicgstab, preconditioner) restated
from Warp's published documentation on the numpy Warp stand-in; warp_cfd calls them at
FV/terms/equation.py:195-200 (bicgstab for momentum, cg for pressure, Jacobi
preconditioner).

* ``preconditioner(A, ptype="diag")``: the Jacobi operator x -> x / diag(A) (a zero
  diagonal entry leaves its component unscaled);
* ``cg`` / ``bicgstab(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None,
  check_every=10, ...)``: solve in place in x; stop when ||r||_2 <= max(atol, tol ||b||_2)
  (a tolerance not given takes the other's value), checked before the first iteration
  and then every ``check_every`` iterations (0: every iteration); ``maxiter`` 0 = the
  system size.  Return (iterations, final ||r||_2, the absolute tolerance used).
  Preconditioned CG; right-preconditioned BiCGSTAB.
Arithmetic in the arrays' own precision with float64 reductions.
"""
from __future__ import annotations

import numpy as np

from .. import array


class _Diag:
    def __init__(self, A):
        d = np.zeros(A.nrow, dtype=A.values._data.dtype)
        rows = A.uncompress_rows()._data
        hit = rows == A.columns._data
        d[rows[hit]] = A.values._data[hit]
        inv = np.ones_like(d)
        nz = d != 0
        inv[nz] = (d.dtype.type(1.0) / d[nz]).astype(d.dtype)
        self.inv = inv

    def apply(self, v):
        return (v * self.inv).astype(v.dtype)


def preconditioner(A, ptype="diag"):
    if ptype not in ("diag", "diag_abs"):
        raise ValueError(f"unsupported preconditioner {ptype!r}")
    return _Diag(A)


def _threshold(b, tol, atol):
    if tol is None and atol is None:
        tol = atol = 0.0
    elif tol is None:
        tol = atol
    elif atol is None:
        atol = tol
    return max(float(atol), float(tol) * float(np.linalg.norm(b.astype(np.float64))))


def _dot(a, b):
    return float(np.dot(a.astype(np.float64), b.astype(np.float64)))


def cg(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10, use_cuda_graph=True):
    S = A._scipy()
    bv = b._data.reshape(-1)
    xv = x._data.reshape(-1)
    T = xv.dtype.type
    maxiter = int(maxiter) or A.nrow
    thr = _threshold(bv, tol, atol)
    Minv = M.apply if M is not None else (lambda v: v.copy())
    r = (bv - S @ xv).astype(T)
    z = Minv(r)
    p = z.copy()
    rz = _dot(r, z)
    rr = _dot(r, r)
    k = 0
    if np.sqrt(rr) <= thr:
        return 0, float(np.sqrt(rr)), thr
    while k < maxiter:
        Ap = (S @ p).astype(T)
        pAp = _dot(p, Ap)
        if pAp == 0.0:
            break
        alpha = rz / pAp
        xv += T(alpha) * p
        r -= T(alpha) * Ap
        z = Minv(r)
        rz_new = _dot(r, z)
        beta = rz_new / rz if rz != 0.0 else 0.0
        rz = rz_new
        p = (z + T(beta) * p).astype(T)
        k += 1
        rr = _dot(r, r)
        if (check_every <= 0 or k % check_every == 0) and np.sqrt(rr) <= thr:
            break
    return k, float(np.sqrt(rr)), thr


def bicgstab(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10, use_cuda_graph=True,
             is_left_preconditioner=False):
    S = A._scipy()
    bv = b._data.reshape(-1)
    xv = x._data.reshape(-1)
    T = xv.dtype.type
    maxiter = int(maxiter) or A.nrow
    thr = _threshold(bv, tol, atol)
    Minv = M.apply if M is not None else (lambda v: v.copy())
    r = (bv - S @ xv).astype(T)
    r0 = r.copy()
    rho = _dot(r0, r)
    p = r.copy()
    rr = _dot(r, r)
    k = 0
    if np.sqrt(rr) <= thr:
        return 0, float(np.sqrt(rr)), thr
    while k < maxiter:
        y = Minv(p)
        v = (S @ y).astype(T)
        r0v = _dot(r0, v)
        if r0v == 0.0:
            break
        alpha = rho / r0v
        s = (r - T(alpha) * v).astype(T)
        xv += T(alpha) * y
        z = Minv(s)
        t = (S @ z).astype(T)
        tt = _dot(t, t)
        omega = _dot(t, s) / tt if tt != 0.0 else 0.0
        xv += T(omega) * z
        r = (s - T(omega) * t).astype(T)
        rho_new = _dot(r0, r)
        k += 1
        rr = _dot(r, r)
        if (check_every <= 0 or k % check_every == 0) and np.sqrt(rr) <= thr:
            break
        if omega == 0.0 or rho == 0.0:
            break
        beta = (rho_new / rho) * (alpha / omega)
        rho = rho_new
        p = (r + T(beta) * (p - T(omega) * v)).astype(T)
    return k, float(np.sqrt(rr)), thr
