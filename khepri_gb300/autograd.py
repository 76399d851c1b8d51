"""Differentiable R, T and per-order powers with respect to the permittivity maps.

``solve_rt`` is a ``torch.autograd.Function`` over the hand-written adjoint of the batched
mixed-precision solve (khp_solve_batched_mixed_grad + khp_convmat_bwd).  The reference has no
gradient: its users difference whole solves (two solves per pixel, khepri/crystal.py:180-206 and
363-396 for every perturbed map); here one backward call gives dL/d(eps) for every pixel of every
map.

Memory: nothing of the forward solve is kept for the backward pass but its inputs.  The backward
call solves the stack again and runs the adjoint in the same launch sequence (modes, recursion
factors, refinement and the transposed sweep all recomputed), so the device holds one chunk of
problems at a time in either pass, whatever the batch and layer count: this is the per-layer
checkpointing with eigenvector recomputation of the design, taken to its limit.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi, batch


def _structures_with_maps(structures, maps):
    """The structures with every ("pixmap", k, depth) layer given map k (host array)."""
    out = []
    for pw, layers, stack in structures:
        lay = {}
        for name, (kind, e, d) in layers.items():
            lay[name] = (kind, maps[int(e)], d) if kind == "pixmap" else (kind, e, d)
        out.append((pw, lay, stack))
    return out


def _map_layers(structures):
    """For every structure, one layer name per distinct map index it uses: {map index: name}."""
    out = []
    for _, layers, stack in structures:
        first = {}
        for name in stack:
            kind, e, _ = layers[name]
            if kind == "pixmap":
                first.setdefault(int(e), name)
        out.append(first)
    return out


def _check_distinct(structures, maps):
    # the batched solver merges maps of identical content within a structure; distinct map
    # indices with identical values would then share one gradient
    for s, first in enumerate(_map_layers(structures)):
        ks = sorted(first)
        for a in range(len(ks)):
            for b in range(a + 1, len(ks)):
                if np.array_equal(maps[ks[a]], maps[ks[b]]):
                    raise ValueError(f"structure {s}: maps {ks[a]} and {ks[b]} are identical; use one map index "
                                     "for layers that share a permittivity")


def _solve(call, maps, device, dR=None, dT=None):
    ents = _structures_with_maps(call["structures"], maps)
    return batch.solve_structures_grad(ents, call["wavelengths"], call["kp"], which=call["which"], dR=dR, dT=dT,
                                       te=call["te"], tm=call["tm"], lattice=call["lattice"], epsi=call["epsi"],
                                       epse=call["epse"], chunk=call["chunk"], refine=call["refine"],
                                       strict=call["strict"], device=device)


class _SolveRT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps_maps, call):
        maps = eps_maps.detach().cpu().numpy()
        _check_distinct(call["structures"], maps)
        dev = eps_maps.device
        R, T, Ro, To, _, st = _solve(call, maps, dev if eps_maps.is_cuda else "cuda")
        ctx.call = call
        ctx.save_for_backward(eps_maps)
        f64 = torch.float64
        status = torch.as_tensor(st, dtype=torch.int32, device=dev)
        ctx.mark_non_differentiable(status)
        return (torch.as_tensor(R, dtype=f64, device=dev), torch.as_tensor(T, dtype=f64, device=dev),
                torch.as_tensor(Ro, dtype=f64, device=dev), torch.as_tensor(To, dtype=f64, device=dev), status)

    @staticmethod
    def backward(ctx, gR, gT, gRo, gTo, _gst):
        (eps_maps,) = ctx.saved_tensors
        call = ctx.call
        pw = call["structures"][0][0]
        shape = (len(call["wavelengths"]), pw[0] * pw[1])

        def weights(g_tot, g_ord):
            # R = sum of the per-order powers, so dL/dR adds to every order's weight
            if g_tot is None and g_ord is None:
                return None
            w = np.zeros(shape)
            if g_ord is not None:
                w += g_ord.detach().double().cpu().numpy()
            if g_tot is not None:
                w += g_tot.detach().double().cpu().numpy()[:, None]
            return w

        maps = eps_maps.detach().cpu().numpy()
        _, _, _, _, grads, _ = _solve(call, maps, eps_maps.device if eps_maps.is_cuda else "cuda",
                                      dR=weights(gR, gRo), dT=weights(gT, gTo))
        g = np.zeros(maps.shape, dtype=np.complex128)
        for s, first in enumerate(_map_layers(call["structures"])):
            for k, name in first.items():
                if name in grads[s]:
                    g[k] += grads[s][name]
        # dL = Re sum(g d eps): a real map's gradient is Re g; for a complex map torch expects the
        # conjugate (the direction of steepest ascent in the complex plane)
        if eps_maps.is_complex():
            out = torch.as_tensor(np.conj(g), device=eps_maps.device).to(eps_maps.dtype)
        else:
            out = torch.as_tensor(g.real, device=eps_maps.device).to(eps_maps.dtype)
        return out, None


def solve_rt(eps_maps, structures, wavelengths, kp, which=None, te=1.0, tm=0.0, lattice="square", epsi=1.0,
             epse=1.0, chunk=256, refine=2, strict=True):
    """R, T [P], per-order powers R_orders, T_orders [P, nh] and status [P], differentiable with
    respect to ``eps_maps``.

    eps_maps: torch tensor [M, nx, ny] (real or complex; axis 1 = x), the permittivity maps;
    structures: list of (pw, layers, stack) as in batch.solve_structures, where a patterned layer
    is ("pixmap", k, depth) with k an index into eps_maps (layers that share a permittivity use one
    index); which: [P] structure of every problem (default: problem i uses structure i); every
    structure has the same harmonic count.  A backward pass through any function of R, T and the
    per-order powers returns dL/d(eps_maps) from the hand-written adjoint.  Problems whose
    mixed-precision solve was flagged (status bits 8, 32) keep their flag and are not re-solved
    (there is no FP64 gradient path); with ``strict`` they raise KhpError.
    """
    if not torch.is_tensor(eps_maps) or eps_maps.dim() != 3:
        raise ValueError("eps_maps must be a torch tensor [M, nx, ny]")
    _capi.require_cuda()
    wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
    call = {"structures": structures, "wavelengths": wl, "kp": np.asarray(kp), "which": which, "te": te, "tm": tm,
            "lattice": lattice, "epsi": epsi, "epse": epse, "chunk": chunk, "refine": refine, "strict": strict}
    return _SolveRT.apply(eps_maps, call)
