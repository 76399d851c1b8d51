"""Batched RCWA solves: many (wavelength, k-point, polarisation) problems of one structure per launch.

``solve_rt`` is the batched counterpart of the reference's one-problem-per-call loop
(README.md:52-58: set_source -> solve -> poynting_flux_end).  Problems are processed in chunks;
inside a chunk every kernel launch covers all problems.  The star-product chain is streamed
left to right (only the running S-matrix and one layer S-matrix are live), and patterned layers
that share a pixmap share one eigensolve per problem.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi, engine
from .engine import LayerSpec


def _specs(layers, epsi, epse):
    specs = {name: LayerSpec(kind, eps, depth) for name, (kind, eps, depth) in layers.items()}
    specs["__inc__"] = LayerSpec("inc", epsi, 0.0)
    specs["__trn__"] = LayerSpec("trn", epse, 0.0)
    return specs


def global_smatrix(struct, specs, stack, prob, status):
    """Global S-matrix of every problem of the chunk, streamed left to right."""
    modes = {}
    Stot, _, _, _ = engine.closed_form(struct, "inc", specs["__inc__"].eps, 0.0, prob, status)
    for name in list(stack) + ["__trn__"]:
        sp = specs[name]
        if sp.kind == "pixmap":
            entry = struct.prepare_map(sp.eps)
            if entry["key"] not in modes:
                modes[entry["key"]] = engine.layer_modes(struct, entry, prob, status)
            W, V, lam = modes[entry["key"]]
            S = engine.layer_smatrix(struct, W, V, lam, sp.depth, prob, status)
        else:
            S, _, _, _ = engine.closed_form(struct, sp.kind, sp.eps, sp.depth, prob, status)
        Stot = engine.star(Stot, S, status)
        del S
    return Stot


def solve_chunk(struct, specs, stack, prob, status, orders=False, epsi=1.0, epse=1.0):
    """R, T (and per-order powers) of one chunk of problems on the device."""
    Stot = global_smatrix(struct, specs, stack, prob, status)
    return engine.flux(struct, Stot, prob, epsi, epse, orders=orders)


def solve_chunk_both_pols(struct, specs, stack, prob, status, epsi=1.0, epse=1.0):
    """R, T for (te, tm) = (1, 0) and (0, 1) from one S-matrix per problem: each [B, 2]."""
    Stot = global_smatrix(struct, specs, stack, prob, status)
    one, zero = torch.ones_like(prob.te), torch.zeros_like(prob.te)
    out = []
    for te, tm in ((one, zero), (zero, one)):
        p = engine.Problems(prob.k0, prob.kp, te, tm)
        r, t, _, _ = engine.flux(struct, Stot, p, epsi, epse)
        out.append((r, t))
    return torch.stack([out[0][0], out[1][0]], 1), torch.stack([out[0][1], out[1][1]], 1)


class StackPlan:
    """Host description of a layer stack for khp_solve_batched, with the stacked per-pixmap
    device matrices (C, Hx, Hy) it reads."""

    def __init__(self, struct, specs, stack):
        kinds, maps, eps, depth = [], [], [], []
        keys, entries = [], []
        for name in stack:
            sp = specs[name]
            if sp.kind == "pixmap":
                e = struct.prepare_map(sp.eps)
                if e["key"] not in keys:
                    keys.append(e["key"])
                    entries.append(e)
                kinds.append(1)
                maps.append(keys.index(e["key"]))
                eps.append(0j)
            else:
                kinds.append(0)
                maps.append(0)
                eps.append(complex(sp.eps))
            depth.append(float(sp.depth))
        self.kinds = np.asarray(kinds, dtype=np.int32)
        self.maps = np.asarray(maps, dtype=np.int32)
        self.eps = np.asarray(eps, dtype=np.complex128)
        self.depth = np.asarray(depth, dtype=np.float64)
        self.nmaps = len(entries)
        if entries:
            self.conv = torch.cat([e["conv"] for e in entries]).contiguous()
            self.hx = torch.cat([e["hx"] for e in entries]).contiguous()
            self.hy = torch.cat([e["hy"] for e in entries]).contiguous()
        else:
            self.conv = self.hx = self.hy = None


def _host(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def solve_chunk_gamma(struct, plan, prob, status, epsi=1.0, epse=1.0, te=None, tm=None, precision="fp64",
                      refine=2):
    """R, T of one chunk by the reflection-matrix recursion (khp_solve_batched).

    te, tm: optional [B, npol] complex device tensors (default: prob.te, prob.tm as one
    polarisation); the recursion runs once and every polarisation is read from it.
    Returns R, T of shape [B] (one polarisation) or [B, npol].
    """
    B = prob.batch
    dev = struct.device
    one_pol = te is None
    if one_pol:
        te, tm = prob.te.reshape(B, 1), prob.tm.reshape(B, 1)
    te, tm = te.contiguous(), tm.contiguous()
    npol = te.shape[1]
    R = torch.empty((B, npol), dtype=torch.float64, device=dev)
    T = torch.empty((B, npol), dtype=torch.float64, device=dev)
    lib = _capi.load()
    L = len(plan.kinds)
    epsi, epse = complex(epsi), complex(epse)
    common = (B, struct.pw[0], struct.pw[1], L, _host(plan.kinds), _host(plan.maps), _host(plan.eps),
              _host(plan.depth), plan.nmaps, _capi.ptr(plan.conv), _capi.ptr(plan.hx), _capi.ptr(plan.hy),
              _capi.ptr(struct.gx), _capi.ptr(struct.gy), epsi.real, epsi.imag, epse.real, epse.imag,
              _capi.ptr(prob.kp), _capi.ptr(prob.k0), npol, _capi.ptr(te), _capi.ptr(tm))
    if precision == "mixed":
        ws = engine.workspace(lib.khp_solve_batched_mixed_workspace(B, struct.nh, L, _host(plan.kinds),
                                                                     _host(plan.maps)), dev)
        with engine._stage("khp_solve_batched_mixed"):
            code = lib.khp_solve_batched_mixed(*common, int(refine), _capi.ptr(R), _capi.ptr(T), _capi.ptr(status),
                                               _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
        _capi.check(code, "khp_solve_batched_mixed")
    else:
        ws = engine.workspace(lib.khp_solve_batched_workspace(B, struct.nh, L, _host(plan.kinds), _host(plan.maps)),
                              dev)
        with engine._stage("khp_solve_batched"):
            code = lib.khp_solve_batched(*common, _capi.ptr(R), _capi.ptr(T), _capi.ptr(status), _capi.ptr(ws),
                                         ws.numel(), _capi.stream_ptr())
        _capi.check(code, "khp_solve_batched")
    if one_pol:
        return R[:, 0], T[:, 0]
    return R, T


def both_pol_weights(B, device):
    """te, tm [B, 2] for the polarisations (te, tm) = (1, 0) and (0, 1)."""
    te = torch.zeros((B, 2), dtype=torch.complex128, device=device)
    tm = torch.zeros((B, 2), dtype=torch.complex128, device=device)
    te[:, 0] = 1.0
    tm[:, 1] = 1.0
    return te, tm


def solve_chunk_gamma_both_pols(struct, plan, prob, status, epsi=1.0, epse=1.0, precision="fp64", refine=2):
    """R, T [B, 2] for (te, tm) = (1, 0) and (0, 1) from one recursion per problem."""
    te, tm = both_pol_weights(prob.batch, struct.device)
    return solve_chunk_gamma(struct, plan, prob, status, epsi, epse, te, tm, precision, refine)


def solve_rt(pw, layers, stack, wavelengths, kp, te=1.0, tm=0.0, lattice="square", epsi=1.0, epse=1.0,
             chunk=256, orders=False, device="cuda", struct=None, strict=True, both_pols=False, method="gamma",
             refine=2):
    """R and T of every problem (host numpy arrays); problems share ``layers``/``stack``.

    layers: name -> ("pixmap", eps_map, depth) | ("uniform", eps, depth); stack: layer names
    from the incidence side.  wavelengths [P], kp [P, 2] (absolute, complex allowed), te/tm
    scalars or [P].  Returns (R, T, status) or (R, T, r_orders, t_orders, status) with
    ``orders=True``.  ``both_pols=True`` returns R, T of shape [P, 2] for (te, tm) = (1, 0)
    and (0, 1).  ``method``: "gamma" (reflection-matrix recursion in FP64, khp_solve_batched),
    "mixed" (the same recursion in FP32 with FP64 eigen-refinement and ``refine`` rounds of FP64
    iterative refinement, khp_solve_batched_mixed) or "chain" (layer S-matrices and the
    star-product chain, as the reference; needed for per-order powers).  With ``strict`` a
    non-zero per-problem status raises KhpError.
    """
    if orders:
        method = "chain"
    _capi.require_cuda()
    wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
    P = wl.shape[0]
    kpa = np.asarray(kp, dtype=complex).reshape(P, 2)
    te = np.broadcast_to(np.asarray(te, dtype=complex), (P,))
    tm = np.broadcast_to(np.asarray(tm, dtype=complex), (P,))
    if struct is None:
        struct = engine.StructureGPU(pw, engine.lattice_vectors(lattice), device)
    specs = _specs(layers, epsi, epse)
    plan = StackPlan(struct, specs, stack) if method in ("gamma", "mixed") else None
    prec = "mixed" if method == "mixed" else "fp64"
    R = np.empty((P, 2) if both_pols else P)
    T = np.empty((P, 2) if both_pols else P)
    ro = np.empty((P, struct.nh)) if orders else None
    to = np.empty((P, struct.nh)) if orders else None
    st = np.zeros(P, dtype=np.int32)
    for s in range(0, P, chunk):
        e = min(P, s + chunk)
        prob = engine.Problems.make(wl[s:e], kpa[s:e], te[s:e], tm[s:e], struct.device)
        status = torch.zeros(e - s, dtype=torch.int32, device=struct.device)
        if method in ("gamma", "mixed"):
            r_o = t_o = None
            if both_pols:
                r, t = solve_chunk_gamma_both_pols(struct, plan, prob, status, epsi, epse, prec, refine)
            else:
                r, t = solve_chunk_gamma(struct, plan, prob, status, epsi, epse, precision=prec, refine=refine)
        elif both_pols:
            r, t = solve_chunk_both_pols(struct, specs, stack, prob, status, epsi, epse)
            r_o = t_o = None
        else:
            r, t, r_o, t_o = solve_chunk(struct, specs, stack, prob, status, orders, epsi, epse)
        R[s:e] = r.cpu().numpy()
        T[s:e] = t.cpu().numpy()
        if orders:
            ro[s:e] = r_o.cpu().numpy()
            to[s:e] = t_o.cpu().numpy()
        st[s:e] = status.cpu().numpy()
    if strict and st.any():
        bad = int(np.flatnonzero(st)[0])
        raise _capi.KhpError(f"problem {bad}: {_capi.decode_status(int(st[bad]))}")
    if orders:
        return R, T, ro, to, st
    return R, T, st
