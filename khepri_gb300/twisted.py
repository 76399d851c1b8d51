"""Twisted bilayers on the GPU: an extended crystal over the product expansion e1 + e2, e2 being
e1 rotated by a twist angle (khepri/expansion.py:52-73; khepri/extension.py:10-126; the
construction of examples/crystal_api/twisted_phc.py:35-57).

Layers on e1 (the incidence half-space and ``lower``) and on e2 (``upper`` and the emergence
half-space) are solved at base size for every shift by a harmonic of the other expansion, as
ExtendedLayer.solve does (extension.py:82-111), here in one batched launch per layer for all
problems and shifts.  Uniform layers of the product expansion (``gap``) are diagonal per harmonic
and are solved on e1 with the shifts.  The chains of each side stay at base size; only the final
combination is dense (khp_twisted_rt).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _capi, engine
from .engine import LayerSpec


def rotation_matrix(angle_rad):
    """tools.py:23-24."""
    c, s = math.cos(angle_rad), math.sin(angle_rad)
    return np.array([[c, -s], [s, c]])


def product_g_vectors(g1, g2):
    """Minkowski sum (expansion.py:60-74): index p * N + q, g = g1[p] + g2[q]."""
    return (g1[:, :, None] + g2[:, None, :]).reshape(2, -1)


class TwistedBilayer:
    """A twisted stack: incidence half-space (eps ``epsi``) and ``lower`` layers on e1, uniform
    ``gap`` layers of the product expansion, ``upper`` layers and the emergence half-space
    (``epse``) on e2 = e1 rotated by ``angle_rad``.  Layers: ("pixmap", eps_map, depth) |
    ("uniform", eps, depth); gap layers must be uniform."""

    def __init__(self, pw, lattice, angle_rad, lower, gap, upper, epsi=1.0, epse=1.0, device="cuda"):
        _capi.require_cuda()
        self.pw = (int(pw[0]), int(pw[1]))
        self.N = self.pw[0] * self.pw[1]
        lat = engine.lattice_vectors(lattice) if isinstance(lattice, str) else np.asarray(lattice, dtype=float)
        self.g1 = engine.g_vectors(self.pw, lat)
        self.g2 = rotation_matrix(angle_rad) @ self.g1
        self.gsum = product_g_vectors(self.g1, self.g2)
        self.device = torch.device(device)
        self.s1 = engine.StructureGPU(self.pw, lat, device)
        self.s2 = engine.StructureGPU(self.pw, lat, device)
        self.s2.gx = torch.tensor(self.g2[0], dtype=torch.float64, device=self.device)
        self.s2.gy = torch.tensor(self.g2[1], dtype=torch.float64, device=self.device)
        self.gx_ext = torch.tensor(self.gsum[0], dtype=torch.float64, device=self.device)
        self.gy_ext = torch.tensor(self.gsum[1], dtype=torch.float64, device=self.device)
        for kind, _, _ in gap:
            if kind != "uniform":
                raise ValueError("gap layers of the product expansion must be uniform")
        self.lower, self.gap, self.upper = list(lower), list(gap), list(upper)
        self.epsi, self.epse = complex(epsi), complex(epse)

    def _chain(self, struct, layers, prob, status, first=None, last=None):
        """first * layers[0] * ... * last at base size for every (problem, shift)."""
        S = None
        specs = []
        if first is not None:
            specs.append(first)
        specs += [LayerSpec(k, e, d) for k, e, d in layers]
        if last is not None:
            specs.append(last)
        modes = {}
        for sp in specs:
            if sp.kind == "pixmap":
                entry = struct.prepare_map(sp.eps)
                if entry["key"] not in modes:
                    modes[entry["key"]] = engine.layer_modes(struct, entry, prob, status)
                W, V, lam = modes[entry["key"]]
                L = engine.layer_smatrix(struct, W, V, lam, sp.depth, prob, status)
            else:
                L, _, _, _ = engine.closed_form(struct, sp.kind, sp.eps, sp.depth, prob, status)
            S = L if S is None else engine.star(S, L, status)
        return S

    def solve_rt(self, wavelengths, kp, te=1.0, tm=1.0, both_pols=False, chunk=32, strict=True):
        """R, T of every problem (host arrays; [P] or [P, 2] with ``both_pols`` for (te, tm) =
        (1, 0) and (0, 1)) and the status words."""
        wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
        P = wl.shape[0]
        kpa = np.asarray(kp, dtype=complex).reshape(P, 2)
        te = np.broadcast_to(np.asarray(te, dtype=complex), (P,))
        tm = np.broadcast_to(np.asarray(tm, dtype=complex), (P,))
        N = self.N
        npol = 2 if both_pols else 1
        R = np.empty((P, npol))
        T = np.empty((P, npol))
        st = np.zeros(P, dtype=np.int32)
        lib = _capi.load()
        dev = self.device
        for s0 in range(0, P, chunk):
            idx = np.arange(s0, min(P, s0 + chunk))
            B = len(idx)
            # base problems: b * N + m at kp_b + g_other[m]
            kp_left = (kpa[idx][:, None, :] + self.g2.T[None, :, :]).reshape(B * N, 2)
            kp_right = (kpa[idx][:, None, :] + self.g1.T[None, :, :]).reshape(B * N, 2)
            wl_rep = np.repeat(wl[idx], N)
            pl = engine.Problems.make(wl_rep, kp_left, 1.0, 0.0, dev)
            pr = engine.Problems.make(wl_rep, kp_right, 1.0, 0.0, dev)
            st_l = torch.zeros(B * N, dtype=torch.int32, device=dev)
            st_r = torch.zeros(B * N, dtype=torch.int32, device=dev)
            SL = self._chain(self.s1, self.lower + self.gap, pl, st_l, first=LayerSpec("inc", self.epsi, 0.0))
            SR = self._chain(self.s2, self.upper, pr, st_r, last=LayerSpec("trn", self.epse, 0.0))
            prob = engine.Problems.make(wl[idx], kpa[idx], te[idx], tm[idx], dev)
            if both_pols:
                tt = torch.zeros((B, 2), dtype=torch.complex128, device=dev)
                tmm = torch.zeros((B, 2), dtype=torch.complex128, device=dev)
                tt[:, 0] = 1.0
                tmm[:, 1] = 1.0
            else:
                tt, tmm = prob.te.reshape(B, 1).contiguous(), prob.tm.reshape(B, 1).contiguous()
            r = torch.empty((B, npol), dtype=torch.float64, device=dev)
            t = torch.empty((B, npol), dtype=torch.float64, device=dev)
            status = torch.zeros(B, dtype=torch.int32, device=dev)
            ws = engine.workspace(lib.khp_twisted_rt_workspace(B, N), dev)
            SL, SR = SL.contiguous(), SR.contiguous()  # held until the launches are enqueued
            with engine._stage("khp_twisted_rt"):
                code = lib.khp_twisted_rt(B, N, _capi.ptr(SL), _capi.ptr(SR),
                                          _capi.ptr(self.gx_ext), _capi.ptr(self.gy_ext), _capi.ptr(prob.kp),
                                          _capi.ptr(prob.k0), npol, _capi.ptr(tt), _capi.ptr(tmm), self.epsi.real,
                                          self.epsi.imag, self.epse.real, self.epse.imag, _capi.ptr(r), _capi.ptr(t),
                                          None, None, _capi.ptr(status), _capi.ptr(ws), ws.numel(),
                                          _capi.stream_ptr())
            _capi.check(code, "khp_twisted_rt")
            R[idx] = r.cpu().numpy()
            T[idx] = t.cpu().numpy()
            base = (st_l | st_r).reshape(B, N).cpu().numpy()
            st[idx] = status.cpu().numpy() | np.bitwise_or.reduce(base, axis=1)
        if strict and st.any():
            bad = int(np.flatnonzero(st)[0])
            raise _capi.KhpError(f"problem {bad}: {_capi.decode_status(int(st[bad]))}")
        if not both_pols:
            return R[:, 0], T[:, 0], st
        return R, T, st
