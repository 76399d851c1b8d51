"""Batched RCWA solves: many (wavelength, k-point, polarisation) problems of one structure per launch.

``solve_rt`` is the batched counterpart of the reference's one-problem-per-call loop
(README.md:52-58: set_source -> solve -> poynting_flux_end).  Problems are processed in chunks;
inside a chunk every kernel launch covers all problems.  The star-product chain is streamed
left to right (only the running S-matrix and one layer S-matrix are live), and patterned layers
that share a pixmap share one eigensolve per problem.
"""
from __future__ import annotations

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


def solve_rt(pw, layers, stack, wavelengths, kp, te=1.0, tm=0.0, lattice="square", epsi=1.0, epse=1.0,
             chunk=256, orders=False, device="cuda", struct=None, strict=True, both_pols=False):
    """R and T of every problem (host numpy arrays); problems share ``layers``/``stack``.

    layers: name -> ("pixmap", eps_map, depth) | ("uniform", eps, depth); stack: layer names
    from the incidence side.  wavelengths [P], kp [P, 2] (absolute, complex allowed), te/tm
    scalars or [P].  Returns (R, T, status) or (R, T, r_orders, t_orders, status) with
    ``orders=True``.  ``both_pols=True`` solves each S-matrix once and returns R, T of shape
    [P, 2] for (te, tm) = (1, 0) and (0, 1).  With ``strict`` a non-zero per-problem status
    raises KhpError.
    """
    _capi.require_cuda()
    wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
    P = wl.shape[0]
    kpa = np.asarray(kp, dtype=complex).reshape(P, 2)
    te = np.broadcast_to(np.asarray(te, dtype=complex), (P,))
    tm = np.broadcast_to(np.asarray(tm, dtype=complex), (P,))
    if struct is None:
        struct = engine.StructureGPU(pw, engine.lattice_vectors(lattice), device)
    specs = _specs(layers, epsi, epse)
    R = np.empty((P, 2) if both_pols else P)
    T = np.empty((P, 2) if both_pols else P)
    ro = np.empty((P, struct.nh)) if orders else None
    to = np.empty((P, struct.nh)) if orders else None
    st = np.zeros(P, dtype=np.int32)
    for s in range(0, P, chunk):
        e = min(P, s + chunk)
        prob = engine.Problems.make(wl[s:e], kpa[s:e], te[s:e], tm[s:e], struct.device)
        status = torch.zeros(e - s, dtype=torch.int32, device=struct.device)
        if both_pols:
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
