"""Differentiable complex128 restatement of the reference's solve — TEST INFRASTRUCTURE ONLY.

The same algorithm as ``oracle/khepri_oracle.py`` (which restates the reference, Kaeryv/Khepri),
written in torch complex128 so that autograd differentiates it: the convolution matrix from the
pixmap's FFT (khepri/tools.py:33-56), the patterned-layer modes by ``torch.linalg.eig`` of P Q
(khepri/alternative.py:158-178), build_scatmat (alternative.py:181-195), the half-spaces and
homogeneous layers (alternative.py:32-156), the forward star-product chain (alternative.py:19-30,
khepri/layer.py:35-60) and the per-order powers of poynting_flux_end (khepri/crystal.py:363-396,
alternative.py:235-245).  It is the autograd reference for the hand-written adjoint: checked
against the numpy oracle first (tests/test_torch_oracle.py), then used for gradients.

Who may use it: ``tests/`` only.  The product package never imports it.  torch's eig backward
divides by eigenvalue differences, so it needs a spectrum without exact degeneracies (random
density maps have none; symmetric pixmaps at normal incidence do).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import khepri_oracle as ko

C128 = torch.complex128


def _t(a):
    return torch.as_tensor(np.asarray(a), dtype=C128)


def convolution_matrix(eps_map, pw):
    """tools.py:33-56: C[r, c] = fftshift(fft2(eps))/(nx ny) at (g0 + p_r - p_c, g0 + q_r - q_c)."""
    eps_map = eps_map.to(C128)
    nx, ny = eps_map.shape
    coefs = torch.fft.fftshift(torch.fft.fft2(eps_map)) / (nx * ny)
    px, py = pw
    r = np.arange(px * py)
    p, q = r % px, r // px
    ix = torch.as_tensor(nx // 2 + p[:, None] - p[None, :])
    iy = torch.as_tensor(ny // 2 + q[:, None] - q[None, :])
    return coefs[ix, iy]


def _block_diag4(a, b, c, d):
    return torch.cat([torch.cat([torch.diag(a), torch.diag(b)], 1), torch.cat([torch.diag(c), torch.diag(d)], 1)], 0)


def solve_structured_layer(kx, ky, conv):
    """alternative.py:158-178: (lambda^2, W) = eig(P Q), lambda = principal sqrt, V = Q W / lambda."""
    nh = kx.shape[0]
    eye = torch.eye(nh, dtype=C128)
    dkx, dky = torch.diag(kx), torch.diag(ky)
    ic_kx = torch.linalg.solve(conv, dkx)
    ic_ky = torch.linalg.solve(conv, dky)
    p = torch.cat([torch.cat([dkx @ ic_ky, eye - dkx @ ic_kx], 1), torch.cat([dky @ ic_ky - eye, -dky @ ic_kx], 1)], 0)
    q = torch.cat([torch.cat([dkx @ dky, conv - dkx @ dkx], 1), torch.cat([dky @ dky - conv, -dky @ dkx], 1)], 0)
    lam2, w = torch.linalg.eig(p @ q)
    lam = torch.sqrt(lam2)
    v = (q @ w) / lam[None, :]
    return w, v, lam


def _branch_kz(arg):
    """alternative.py:92-96, 145-149: Re(arg) < 0 -> -i sqrt(-arg), else sqrt(arg)."""
    neg = arg.real < 0
    return torch.where(neg, -1j * torch.sqrt(-arg), torch.sqrt(arg))


def solve_uniform_layer(kx, ky, eps):
    """alternative.py:130-156: W = I, lambda = i kz, V = Q / lambda."""
    nh = kx.shape[0]
    eps = torch.as_tensor(eps, dtype=C128)
    q = _block_diag4(kx * ky, eps - kx ** 2, ky ** 2 - eps, -ky * kx)
    kz = _branch_kz(eps - kx ** 2 - ky ** 2)
    lam = torch.cat([1j * kz, 1j * kz])
    return torch.eye(2 * nh, dtype=C128), q / lam[None, :], lam


def free_space_eigenmodes(kx, ky):
    """alternative.py:84-99."""
    w, v, _ = solve_uniform_layer(kx, ky, 1.0)
    return w, v


def build_scatmat(w, v, w0, v0, lam, depth, k0):
    """alternative.py:181-195 (symmetric layer)."""
    t1 = torch.linalg.solve(w, w0)
    t2 = torch.linalg.solve(v, v0)
    a, b = t1 + t2, t1 - t2
    x = torch.diag(torch.exp(-lam * depth * k0))
    ainv_x = torch.linalg.solve(a, x)
    t = a - x @ b @ ainv_x @ b
    s11 = torch.linalg.solve(t, x @ b @ ainv_x @ a - b)
    s12 = torch.linalg.solve(t, x @ (a - b @ torch.linalg.solve(a, b)))
    return (s11, s12, s12, s11)


def redheffer_product(sa, sb):
    """alternative.py:19-30 (four separate solves)."""
    n = sa[0].shape[-1]
    eye = torch.eye(n, dtype=C128)
    d = eye - sb[0] @ sa[3]
    f = eye - sa[3] @ sb[0]
    s11 = sa[0] + sa[1] @ torch.linalg.solve(d, sb[0]) @ sa[2]
    s12 = sa[1] @ torch.linalg.solve(d, sb[1])
    s21 = sb[2] @ torch.linalg.solve(f, sa[2])
    s22 = sb[3] + sb[2] @ torch.linalg.solve(f, sa[3]) @ sb[1]
    return (s11, s12, s21, s22)


def _half_spaces(kx, ky, w0, v0, eps, which):
    """alternative.py:32-82 (incidence: which = 0, emergence: which = 1), constants here."""
    s, _, _, _ = (ko.scattering_reflection if which == 0 else ko.scattering_transmission)(
        kx.numpy(), ky.numpy(), w0.numpy(), v0.numpy(), eps)
    return tuple(_t(s[i, j]) for i in range(2) for j in range(2))


def solve_orders(pw, layers, stack, wavelength, te=1.0, tm=0.0, kp=(0.0, 0.0), lattice="square", epsi=1.0,
                 epse=1.0):
    """R, T and the per-order powers r, t [Nh] of one problem (crystal.py:180-206, 363-396).

    layers: name -> ("pixmap", eps map as a torch tensor [nx, ny] (autograd flows through it),
    depth) | ("uniform", eps, depth); stack: names from the incidence side.
    """
    lat = ko.lattice_vectors(lattice)
    gvec = ko.g_vectors(pw, lat)
    k0 = 2.0 * math.pi / wavelength
    kx_n, ky_n, _ = ko.k_vectors(gvec, kp, wavelength)
    kx, ky = _t(kx_n), _t(ky_n)
    w0, v0 = free_space_eigenmodes(kx, ky)
    cache = {}
    smats = [_half_spaces(kx, ky, w0, v0, epsi, 0)]
    for name in stack:
        if name not in cache:
            kind, eps, depth = layers[name]
            if kind == "pixmap":
                w, v, lam = solve_structured_layer(kx, ky, convolution_matrix(eps, pw))
            else:
                w, v, lam = solve_uniform_layer(kx, ky, eps)
            cache[name] = build_scatmat(w, v, w0, v0, lam, depth, k0)
        smats.append(cache[name])
    smats.append(_half_spaces(kx, ky, w0, v0, epse, 1))
    n = 2 * kx.shape[0]
    zero, eye = torch.zeros((n, n), dtype=C128), torch.eye(n, dtype=C128)
    stot = (zero, eye, eye, zero)
    for s in smats:
        stot = redheffer_product(stot, s)
    kzi = np.conj(np.sqrt(complex(k0 ** 2 * epsi - kp[0] ** 2 - kp[1] ** 2)))
    c1p = _t(ko.incident(pw, te, tm, (kp[0], kp[1], kzi)))

    def fluxes(c_out, eps_medium):
        kxm, kym, kzm = (_t(a) for a in ko.k_vectors(gvec, kp, wavelength, eps_medium))
        nh = kx.shape[0]
        sx, sy = c_out[:nh], c_out[nh:]
        sz = -(kxm * sx + kym * sy) / kzm
        per = kzm.real / np.real(kzi / k0) * (sx.abs() ** 2 + sy.abs() ** 2 + sz.abs() ** 2)
        return per.sum(), per

    t, t_orders = fluxes(stot[2] @ c1p, epse)
    r, r_orders = fluxes(stot[0] @ c1p, epsi)
    return r, t, r_orders, t_orders
