"""Band structure from scattering matrices on the GPU (khepri/eigentricks.py:5-55).

Same functions and return conventions as the reference: ``scattering_splitlr``,
``scattering_det``, ``scattering_eigenvalues(S, dos=False)``, ``on_shell`` and
``band_structure``.  S is the reference's dense [4 ng, 4 ng] matrix (blocks p = 0:2ng,
m = 2ng:4ng); a stack of them [B, 4 ng, 4 ng] is solved in one call; a Crystal S-matrix
[2, 2, n, n] is accepted too and read as [[S11, S12], [S21, S22]].  The pencil (Sl, Sr) is
solved as the eigenproblem of Sr^-1 Sl (khp_scattering_eig: one inverse of S22, three products,
one batched eigensolve) instead of scipy's QZ; results are returned as numpy arrays.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi, engine


def as_dense(S):
    """[2, 2, n, n] -> [2n, 2n] (blocks [[S11, S12], [S21, S22]]); dense input unchanged."""
    if isinstance(S, torch.Tensor):
        S = S.detach().cpu().numpy()
    S = np.asarray(S)
    if S.ndim == 4 and S.shape[:2] == (2, 2):
        n = S.shape[2]
        return S.transpose(0, 2, 1, 3).reshape(2 * n, 2 * n)
    return S


def scattering_splitlr(S):
    """Sl, Sr of the pencil (eigentricks.py:5-23), on the host like the reference."""
    S = as_dense(S)
    ng = S.shape[0] // 4
    p = np.s_[0:2 * ng]
    m = np.s_[2 * ng:4 * ng]
    Sl = np.zeros_like(S)
    Sl[p, p] = S[p, p]
    Sl[m, p] = S[m, p]
    Sl[m, m] = -np.eye(2 * ng, dtype=Sl.dtype)
    Sr = np.zeros_like(S)
    Sr[p, p] = np.eye(2 * ng, dtype=Sr.dtype)
    Sr[p, m] = -S[p, m]
    Sr[m, m] = -S[m, m]
    return Sl, Sr


def _solve(S, vectors=True, det=False, device="cuda"):
    """Batched eigenpairs (and determinants) of Sr^-1 Sl on the GPU: w [B, N], v [B, N, N] or
    None, d [B] or None, status [B]."""
    _capi.require_cuda()
    lib = _capi.load()
    dev = torch.device(device)
    St = torch.as_tensor(np.ascontiguousarray(S), dtype=torch.complex128).to(dev)
    B, N = St.shape[0], St.shape[1]
    if N % 4 or St.shape[2] != N:
        raise ValueError("S must be [4 ng, 4 ng] (or a batch of them)")
    ng = N // 4
    w = torch.empty((B, N), dtype=torch.complex128, device=dev)
    v = torch.empty((B, N, N), dtype=torch.complex128, device=dev) if vectors else None
    d = torch.empty((B,), dtype=torch.complex128, device=dev) if det else None
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    ws = engine.workspace(lib.khp_scattering_eig_workspace(B, ng), dev)
    with engine._stage("khp_scattering_eig"):
        code = lib.khp_scattering_eig(B, ng, _capi.ptr(St), N * N, _capi.ptr(w), _capi.ptr(v), _capi.ptr(d),
                                      _capi.ptr(status), _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
    _capi.check(code, "khp_scattering_eig")
    out = (w.cpu().numpy(), None if v is None else v.cpu().numpy(), None if d is None else d.cpu().numpy(),
           status.cpu().numpy())
    return out


def scattering_det(S):
    """det(S11 - S12 S22^-1 S21) det(S22) (eigentricks.py:25-29); a batch gives an array."""
    S = as_dense(S)
    single = S.ndim == 2
    _, _, d, _ = _solve(S[None] if single else S, vectors=False, det=True)
    return d[0] if single else d


def scattering_eigenvalues(S, dos=False):
    """(w, v) or (w, v, det) of the pencil (Sl, Sr) (eigentricks.py:30-39); None when S holds a
    NaN, as in the reference.  For a batch [B, N, N], arrays over the batch (rows of problems
    with a NaN are NaN).  A singular S22 (infinite pencil eigenvalue) raises KhpError."""
    S = as_dense(S)
    single = S.ndim == 2
    Sb = S[None] if single else S
    nan = np.isnan(Sb).reshape(Sb.shape[0], -1).any(axis=1)
    if single and nan[0]:
        return None
    # problems holding a NaN are solved as the identity and reported as NaN
    eye = np.eye(Sb.shape[1], dtype=complex)[None]
    w, v, d, st = _solve(np.where(nan[:, None, None], eye, Sb), vectors=True, det=dos)
    bad = (st != 0) & ~nan
    if bad.any():
        i = int(np.flatnonzero(bad)[0])
        raise _capi.KhpError(f"problem {i}: {_capi.decode_status(int(st[i]))}")
    if nan.any():
        w[nan] = np.nan
        v[nan] = np.nan
        if d is not None:
            d[nan] = np.nan
    if single:
        return (w[0], v[0], d[0]) if dos else (w[0], v[0])
    return (w, v, d) if dos else (w, v)


def on_shell(eigenvalues, tol=1e-10):
    """|w| == 1 within tol (eigentricks.py:41-42)."""
    return np.isclose(np.abs(eigenvalues), 1.0, rtol=0.0, atol=tol)


def _filter(w):
    w = w.real
    w = w[w > 0]
    w = w[w < 1]
    return w[on_shell(w)]


def band_structure(S):
    """Real parts in (0, 1) of the on-shell pencil eigenvalues (eigentricks.py:46-55); None
    when S holds a NaN.  A batch gives a list of arrays."""
    S = as_dense(S)
    res = scattering_eigenvalues(S)
    if res is None:
        return None
    w, _ = res
    if w.ndim == 1:
        return _filter(w)
    return [None if np.isnan(wi).any() else _filter(wi) for wi in w]
