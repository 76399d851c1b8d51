"""The tmat formulation on the GPU (khepri/tmat: lattice.py, tools.py, matrices.py,
scattering.py), SI units.

The host side mirrors the reference's lattice bookkeeping (g vectors, kz, the polarisation
bases eta / mu, the dense U, Vi, Ve, the Fourier coefficients eps_g): O(number of harmonics)
arithmetic.  The O(n^3) work runs in libkhp: the layer's field matrix A, its exponential,
U E Vi, matrix_s and the slice-squaring star products (khp_tmat_layer_smatrix, batched over
wavelengths and kp), and multS / matrix_s on their own (khp_tmat_multS, khp_tmat_matrix_s).
Scattering matrices are dense [4 ng, 4 ng] in the reference's [p; m] layout; numpy in, numpy out
(torch CUDA tensors in, torch out).
"""
from __future__ import annotations

import cmath
import math
from math import prod

import numpy as np
import torch

from . import _capi, engine

C0 = 299792458.0
MU0 = 4 * math.pi * 1e-7
MU0C = MU0 * C0  # constants.py:3-5
TWOPI = 2 * math.pi


def nanometers(x):
    return x * 1e-9


def grid_center(shape):
    """tools.py:14-22."""
    assert shape[0] % 2 == shape[1] % 2, "Grid dimensions should have same parity."
    if shape[0] % 2 == 0:
        return shape[0] // 2, shape[1] // 2
    return (shape[0] - 1) // 2, (shape[1] - 1) // 2


def grid_size(pw):
    """tools.py:24-37: ((nx, ny), q)."""
    assert pw[0] % 2 == pw[1] % 2, "Plane waves should have same parity."
    if pw[0] % 2 == 0:
        nx, ny = pw[0] // 2, pw[1] // 2
        return (nx, ny), (4 * nx, 4 * ny)
    nx, ny = (pw[0] - 1) // 2, (pw[1] - 1) // 2
    return (nx, ny), (4 * nx + 1, 4 * ny + 1)


def gvectors(b1, b2, shape, dtype=np.float32):
    """lattice.py:32-38."""
    cx, cy = grid_center(shape)
    m1 = np.arange(shape[0], dtype=dtype) - cx
    m2 = np.arange(shape[1], dtype=dtype) - cy
    return np.add.outer(b1[0] * m1, b2[0] * m2), np.add.outer(b1[1] * m1, b2[1] * m2)


def compute_kz(gx, gy, epsilon, wavelength, kp=(0.0, 0.0), dtype=np.complex128):
    """tools.py:39-47."""
    u2 = np.abs(kp[0] + gx) ** 2 + np.abs(kp[1] + gy) ** 2
    kz = np.emath.sqrt(epsilon * (TWOPI / wavelength) ** 2 - u2).astype(dtype)
    flip = (kz.imag < 0.0) | (np.isclose(kz.imag, 0.0) & (kz.real < 0.0))
    return np.where(flip, -kz, kz)


def _unit_planar(gx, gy, kp):
    ux = (kp[0] + gx).astype(complex)
    uy = (kp[1] + gy).astype(complex)
    nrm = np.sqrt(np.abs(ux) ** 2 + np.abs(uy) ** 2)
    small = nrm ** 2 < np.finfo(float).eps
    safe = np.where(small, 1.0, nrm)
    return np.where(small, 1.0, ux / safe), np.where(small, 0.0, uy / safe)


def compute_eta(gx, gy, kp=(0.0, 0.0)):
    """tools.py:49-59."""
    ux, uy = _unit_planar(gx, gy, kp)
    return uy, -ux


def compute_mu(gx, gy, kzg, epsilon, wavelength, kp=(0.0, 0.0)):
    """tools.py:62-71."""
    ux, uy = _unit_planar(gx, gy, kp)
    f = kzg / (cmath.sqrt(epsilon) * TWOPI / wavelength)
    return f * ux, f * uy


def coords_from_index(p, n, g):
    """tools.py:73-75."""
    return np.subtract(np.unravel_index(g, p, order="F"), n)


def epsilon_g(q, islands_data, eps_host, inverse=False):
    """tools.py:76-86."""
    f = (lambda v: 1 / v) if inverse else (lambda v: v)
    out = np.zeros(q, dtype=complex)
    out[q[0] // 2, q[1] // 2] = f(eps_host)
    for bf, e in islands_data:
        out += (f(e) - f(eps_host)) * bf
    return out


def _fexpz(z):
    z = np.asarray(z, dtype=complex)
    out = np.empty_like(z)
    big = np.abs(z) > 1e-2
    out[big] = (np.exp(z[big]) - 1.0) / z[big]
    w = z[~big]
    out[~big] = 1 + w / 2.0 * (1 + w / 3.0 * (1 + w / 4.0 * (1 + w / 5.0 * (1 + w / 6.0 * (1 + w / 7)))))
    return out


def transform(shape, params, Gx, Gy, sigma):
    """fourier.py:20-63 for the island shapes of the tmat path: disc, rectangle, uniform."""
    if shape == "disc":
        from scipy import special
        c0, c1, r = params
        norm = np.sqrt(Gx * Gx + Gy * Gy) * r
        at0 = np.isclose(Gx, 0.0) & np.isclose(Gy, 0.0)
        out = np.zeros_like(Gx, dtype=complex)
        nz = ~at0
        out[nz] = (np.pi * r ** 2 / sigma * 2 * np.exp(-1j * (c0 * Gx[nz] + c1 * Gy[nz])) * special.jv(1.0, norm[nz])
                   / norm[nz])
        out[at0] = np.pi * r ** 2 / sigma
        return out
    if shape == "rectangle":
        ll0, ll1, ur0, ur1 = params
        a, b = ur0 - ll0, ur1 - ll1
        return a * b / sigma * _fexpz(-1j * Gx * a) * _fexpz(-1j * Gy * b) * np.exp(-1j * (ll0 * Gx + ll1 * Gy))
    if shape == "uniform":
        return np.zeros_like(Gx)
    raise ValueError(f"unknown island shape {shape!r}")


def _u_blocks(kz, eta, mu, eps, wavelength):
    """matrix_u (matrices.py:9-42) as its 16 blocks of diagonals [16, ng] (block (a, c) at a*4+c)."""
    hU = MU0C / cmath.sqrt(eps)
    mgx, mgy = mu[0].T.ravel(), mu[1].T.ravel()
    egx, egy = eta[0].T.ravel(), eta[1].T.ravel()
    dg = cmath.sqrt(eps) * math.pi / wavelength / kz.T.ravel()
    B = np.zeros((16, mgx.size), dtype=complex)
    for (a, c), d in {(0, 0): dg * mgy, (2, 0): dg * mgy, (0, 1): -dg * mgx, (2, 1): -dg * mgx,
                      (1, 0): dg * egy, (3, 0): -dg * egy, (1, 1): -dg * egx, (3, 1): dg * egx,
                      (0, 2): -hU * dg * egy, (2, 2): hU * dg * egy, (1, 2): hU * dg * mgy, (3, 2): hU * dg * mgy,
                      (1, 3): -hU * dg * mgx, (3, 3): -hU * dg * mgx, (2, 3): -hU * dg * egx,
                      (0, 3): hU * dg * egx}.items():
        B[a * 4 + c] = d
    return B


def _v_blocks(eta, mu, eps):
    """matrix_v (matrices.py:44-74) as its 16 blocks of diagonals."""
    hV = np.sqrt(eps) / MU0C
    mgx, mgy = mu[0].T.ravel(), mu[1].T.ravel()
    egx, egy = eta[0].T.ravel(), eta[1].T.ravel()
    B = np.zeros((16, mgx.size), dtype=complex)
    for (a, c), d in {(0, 0): egx, (1, 0): egy, (2, 0): hV * mgx, (3, 0): hV * mgy,
                      (0, 1): -mgx, (1, 1): -mgy, (2, 1): hV * egx, (3, 1): hV * egy,
                      (0, 2): egx, (1, 2): egy, (2, 2): -hV * mgx, (3, 2): -hV * mgy,
                      (0, 3): mgx, (1, 3): mgy, (2, 3): hV * egx, (3, 3): hV * egy}.items():
        B[a * 4 + c] = d
    return B


def _dense(blocks):
    ng = blocks.shape[1]
    M = np.zeros((4 * ng, 4 * ng), dtype=complex)
    for k in range(16):
        a, c = divmod(k, 4)
        M[a * ng:(a + 1) * ng, c * ng:(c + 1) * ng] += np.diag(blocks[k])
    return M


class CartesianLattice:
    """lattice.py:40-211: reciprocal lattice, incidence / emergence media, polarisation bases."""

    def __init__(self, pw, a1, a2, eps_incid=1.0, eps_emerg=1.0, dtype=np.float32):
        coef = TWOPI / (a1[0] * a2[1] - a1[1] * a2[0])
        self.a1, self.a2 = a1, a2
        self.b1 = (a2[1] * coef, -a2[0] * coef)
        self.b2 = (-a1[1] * coef, a1[0] * coef)
        self.n, self.q = grid_size(pw)
        self.Gx, self.Gy = gvectors(self.b1, self.b2, self.q, dtype=dtype)
        self.area = abs(a1[0] * a2[1] - a1[1] * a2[0])
        self.eps_incid, self.eps_emerg = eps_incid, eps_emerg
        self.dtype = dtype
        self.pw = tuple(pw)
        self.eta_ = None

    @property
    def nx(self):
        """lattice.py:61-63."""
        return (self.q[0] // 4, (self.q[0] - 1) // 4)[self.q[0] % 2]

    @property
    def ny(self):
        """lattice.py:65-67."""
        return (self.q[1] // 4, (self.q[1] - 1) // 4)[self.q[1] % 2]

    @property
    def gx(self):
        """lattice.py:69-75."""
        return self.Gx[self.nx:self.q[0] - self.nx, self.ny:self.q[0] - self.ny]

    @property
    def gy(self):
        """lattice.py:81-86."""
        return self.Gy[self.nx:self.q[0] - self.nx, self.ny:self.q[0] - self.ny]

    @property
    def eta_normal(self):
        """lattice.py:92-98 (cached)."""
        if self.eta_ is None:
            self.eta_ = compute_eta(self.gx, self.gy)
        return self.eta_

    def eta(self, wavelength, kp):
        """lattice.py:100-105."""
        return compute_eta(self.gx, self.gy, kp=kp)

    def kp_angle(self, wavelength, theta_deg, phi_deg):
        """lattice.py:107-111."""
        return engine.compute_kplanar(self.eps_incid, wavelength, theta_deg, phi_deg)

    def kzi(self, wavelength, kp):
        """lattice.py:113-117."""
        return compute_kz(self.gx, self.gy, self.eps_incid, wavelength, kp)

    def kze(self, wavelength, kp):
        """lattice.py:119-123."""
        return compute_kz(self.gx, self.gy, self.eps_emerg, wavelength, kp)

    def mugi(self, wavelength, kp):
        """lattice.py:125-126."""
        return compute_mu(self.gx, self.gy, self.kzi(wavelength, kp), self.eps_incid, wavelength, kp)

    def muge(self, wavelength, kp):
        """lattice.py:128-129."""
        return compute_mu(self.gx, self.gy, self.kze(wavelength, kp), self.eps_emerg, wavelength, kp)

    def u_blocks(self, wavelength, kp):
        """the 4x4 blocks of diagonals of U (lattice.py:131-139), as the GPU kernels take them."""
        return _u_blocks(self.kzi(wavelength, kp), self.eta(wavelength, kp), self.mugi(wavelength, kp),
                         self.eps_incid, wavelength)

    def vi_blocks(self, wavelength, kp):
        """the 4x4 blocks of diagonals of Vi (lattice.py:141-149)."""
        return _v_blocks(self.eta(wavelength, kp), self.mugi(wavelength, kp), self.eps_incid)

    def ve_blocks(self, wavelength, kp):
        """the 4x4 blocks of diagonals of Ve (lattice.py:151-159)."""
        return _v_blocks(self.eta(wavelength, kp), self.muge(wavelength, kp), self.eps_emerg)

    def U(self, wavelength, kp):
        """lattice.py:131-139 (dense)."""
        return _dense(self.u_blocks(wavelength, kp))

    def Vi(self, wavelength, kp):
        """lattice.py:141-149 (dense)."""
        return _dense(self.vi_blocks(wavelength, kp))

    def Ve(self, wavelength, kp):
        """lattice.py:151-159 (dense)."""
        return _dense(self.ve_blocks(wavelength, kp))

    def bz_path(self, k_points, resolutions=(), a=1.0):
        """lattice.py:161-178."""
        main = {"G": (0, 0), "X": (0, 0.99 * np.pi / a), "M": (0.99 * np.pi / a, 0.99 * np.pi / a)}
        assert len(k_points) > 1, "Give at least two k-points"
        res = list(resolutions)
        if len(res) == 0:
            res = [10] * (len(k_points) - 1)
        elif len(res) == 1:
            res = [res[0]] * (len(k_points) - 1)
        assert len(res) == len(k_points) - 1, "Give resolution for each interval between k-points"
        traj = []
        for i, r in enumerate(res):
            s0, s1 = main[k_points[i]], main[k_points[i + 1]]
            for j in range(r):
                traj.append(np.array([s0[0] + (s1[0] - s0[0]) * j / r, s0[1] + (s1[1] - s0[1]) * j / r]))
        return traj

    def g_vectors(self):
        """lattice.py:180-183."""
        g = np.stack((self.gx.real.flat, self.gy.real.flat), axis=0).T
        yield from g

    def G_vectors(self):
        """lattice.py:185-188."""
        g = np.stack((self.Gx.real.flat, self.Gy.real.flat), axis=0).T
        yield from g

    def restrict_radius_mask(self, radius):
        """lattice.py:212-213."""
        return np.linalg.norm(np.array(list(self.g_vectors())), axis=-1) < radius


# ------------------------------------------------------------------------------------------
# device calls
# ------------------------------------------------------------------------------------------
def _to_dev(M, dev):
    if isinstance(M, torch.Tensor):
        return M.to(device=dev, dtype=torch.complex128).contiguous(), True
    return torch.as_tensor(np.ascontiguousarray(M), dtype=torch.complex128).to(dev), False


def _check_status(status, what):
    st = status.cpu().numpy()
    if st.any():
        i = int(np.flatnonzero(st)[0])
        raise _capi.KhpError(f"{what}: problem {i}: {_capi.decode_status(int(st[i]))}")


def multS(S1, S2, device="cuda"):
    """matrices.py:194-212 on the GPU; S1, S2 [4 ng, 4 ng] or batches [B, 4 ng, 4 ng]."""
    _capi.require_cuda()
    lib = _capi.load()
    dev = torch.device(device)
    a, was_t = _to_dev(S1, dev)
    b, _ = _to_dev(S2, dev)
    single = a.dim() == 2
    if single:
        a, b = a[None], b[None]
    B, N = a.shape[0], a.shape[1]
    ng = N // 4
    out = torch.empty_like(a)
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    ws = engine.workspace(lib.khp_tmat_multS_workspace(B, ng), dev)
    with engine._stage("khp_tmat_multS"):
        code = lib.khp_tmat_multS(B, ng, _capi.ptr(a), N * N, _capi.ptr(b), N * N, _capi.ptr(out),
                                  _capi.ptr(status), _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
    _capi.check(code, "khp_tmat_multS")
    _check_status(status, "multS")
    out = out[0] if single else out
    return out if was_t else out.cpu().numpy()


def matrix_s(T, device="cuda"):
    """matrices.py:171-180 on the GPU."""
    _capi.require_cuda()
    lib = _capi.load()
    dev = torch.device(device)
    t, was_t = _to_dev(T, dev)
    single = t.dim() == 2
    if single:
        t = t[None]
    B, N = t.shape[0], t.shape[1]
    ng = N // 4
    out = torch.empty_like(t)
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    ws = engine.workspace(lib.khp_tmat_multS_workspace(B, ng), dev)
    code = lib.khp_tmat_matrix_s(B, ng, _capi.ptr(t), _capi.ptr(out), _capi.ptr(status), _capi.ptr(ws), ws.numel(),
                                 _capi.stream_ptr())
    _capi.check(code, "khp_tmat_matrix_s")
    _check_status(status, "matrix_s")
    out = out[0] if single else out
    return out if was_t else out.cpu().numpy()


class LayerMatrix:
    """scattering.py:9-23: a layer's scattering matrix; ``@`` with another LayerMatrix is multS."""

    def __init__(self, S, keep_metadata=False):
        self.S = S

    def numpy(self):
        """scattering.py:13-14: the S-matrix as a numpy array."""
        return self.S.cpu().numpy() if isinstance(self.S, torch.Tensor) else self.S

    def copy(self):
        """scattering.py:16-17: an independent copy."""
        return LayerMatrix(self.S.clone() if isinstance(self.S, torch.Tensor) else self.S.copy())

    def __matmul__(self, rhs):
        if isinstance(rhs, LayerMatrix):
            return LayerMatrix(multS(self.S, rhs.S))
        return self.S @ rhs


def scattering_matrices(pw, lattice, islands_data, eps_host, wavelengths, kps, depth=100e-9, slicing_pow=3,
                        intermediates=False, device="cuda"):
    """Layer S-matrices of one island layout for a batch of (wavelength, kp) problems in one
    launch (the batched form of scattering_matrix_islands).  islands_data: [(Fourier transform on
    lattice.Gx/Gy, eps)].  Returns a torch CUDA tensor [B, 4 ng, 4 ng], and with
    ``intermediates`` also A, E = expm(-A d / 2^p) and T = U E Vi."""
    _capi.require_cuda()
    lib = _capi.load()
    dev = torch.device(device)
    wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
    kp = np.asarray(kps, dtype=float).reshape(-1, 2)
    B = wl.size
    assert kp.shape[0] == B
    _, q = grid_size(pw)
    epsg = epsilon_g(q, islands_data, eps_host)
    iepsg = epsilon_g(q, islands_data, eps_host, inverse=True)
    px, py = lattice.gx.shape
    ng = px * py
    u = np.stack([lattice.u_blocks(wl[b], tuple(kp[b])) for b in range(B)])
    v = np.stack([lattice.vi_blocks(wl[b], tuple(kp[b])) for b in range(B)])
    t = lambda a, dt=torch.complex128: torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(dev)  # noqa: E731
    eg, ieg = t(epsg), t(iepsg)
    gx = t(lattice.gx.T.ravel().real, torch.float64)
    gy = t(lattice.gy.T.ravel().real, torch.float64)
    kpt, wlt, ut, vt = t(kp, torch.float64), t(wl, torch.float64), t(u), t(v)
    N = 4 * ng
    S = torch.empty((B, N, N), dtype=torch.complex128, device=dev)
    extra = [torch.empty_like(S) for _ in range(3)] if intermediates else [None, None, None]
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    ws = engine.workspace(lib.khp_tmat_layer_workspace(B, ng), dev)
    with engine._stage("khp_tmat_layer_smatrix"):
        code = lib.khp_tmat_layer_smatrix(B, px, py, q[0], q[1], _capi.ptr(eg), _capi.ptr(ieg), _capi.ptr(gx),
                                          _capi.ptr(gy), _capi.ptr(kpt), _capi.ptr(wlt), _capi.ptr(ut), _capi.ptr(vt),
                                          float(depth), int(slicing_pow), _capi.ptr(S), _capi.ptr(extra[0]),
                                          _capi.ptr(extra[1]), _capi.ptr(extra[2]), _capi.ptr(status), _capi.ptr(ws),
                                          ws.numel(), _capi.stream_ptr())
    _capi.check(code, "khp_tmat_layer_smatrix")
    _check_status(status, "tmat layer")
    return (S, *extra) if intermediates else S


def scattering_matrix(pw, lattice, island_type, params, island_eps, eps_host, wavelength, kp, depth=100e-9,
                      slicing_pow=3):
    """scattering.py:25-51."""
    bf = transform(island_type, params, lattice.Gx, lattice.Gy, lattice.area)
    S = scattering_matrices(pw, lattice, [(bf, island_eps)], eps_host, [wavelength], [kp], depth, slicing_pow)
    return LayerMatrix(S[0].cpu().numpy())


def scattering_matrix_islands(pw, lattice, islands_description, eps_host, wavelength, kp, depth=100e-9,
                              slicing_pow=3):
    """scattering.py:54-80: islands_description = [{"shape", "params", "epsilon"}]."""
    data = [(transform(i["shape"], i["params"], lattice.Gx, lattice.Gy, lattice.area), i["epsilon"])
            for i in islands_description]
    S = scattering_matrices(pw, lattice, data, eps_host, [wavelength], [kp], depth, slicing_pow)
    return LayerMatrix(S[0].cpu().numpy())


def scattering_air_tmp(pw, lattice, wavelength, depth):
    """scattering.py:83-91: free-space propagation exp(i kz d) on the diagonal."""
    ng = prod(pw)
    kzs = compute_kz(lattice.gx, lattice.gy, 1.0, wavelength)
    S = np.zeros((4 * ng, 4 * ng), dtype=complex)
    d = np.exp(1j * kzs.ravel() * depth)
    for j in range(4):
        S[np.arange(ng) + j * ng, np.arange(ng) + j * ng] = d
    return LayerMatrix(S)


def scattering_identity(pw):
    """scattering.py:121-127."""
    I = np.eye(2 * prod(pw))
    return np.vstack([np.hstack([np.zeros_like(I), I]), np.hstack([I, np.zeros_like(I)])])


def scattering_interface(lattice, wavelength, kp=(0, 0)):
    """scattering.py:129-134: matrix_s(U Ve) on the GPU."""
    return LayerMatrix(matrix_s(lattice.U(wavelength, kp) @ lattice.Ve(wavelength, kp)))
