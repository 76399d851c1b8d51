"""CPU oracle for the Crystal RCWA solve path — TEST INFRASTRUCTURE ONLY.

This module restates, in plain numpy complex128 with LAPACK-backed dense solves and
``numpy.linalg.eig``, the algorithm the reference (Kaeryv/Khepri) runs for
``Crystal.solve`` + ``poynting_flux_end`` + ``fields_volume``.  Every function names the
reference lines it follows (paths relative to the reference project root).

Who may use it: ``tests/``, ``__graft_entry__.smoke()`` (to check the GPU result) and ``bench.py``
(its ``cpu_baseline`` leg and ``--impl reference`` arm).  The product package
``khepri_gb300`` never imports it.

Parity pinning: the oracle is checked (tests/test_oracle_golden.py) against golden vectors
produced by running the reference itself on the same inputs (tests/golden/make_golden.py),
and against the reference's own known-answer test, the thin-film Fresnel check of
test/integration/test_complex_eps.py:13-42.

The arithmetic underneath lives in numpy/LAPACK (zgesv, zgeev, zgemm) and numpy's FFT
(pocketfft), exactly as in the reference; numpy versions there are unpinned
(requirements.txt:1-5).
"""
from __future__ import annotations

import cmath
import math
from types import SimpleNamespace

import numpy as np

TWOPI = 2.0 * math.pi


# ---------------------------------------------------------------------------------------
# Basis: harmonic indices, reciprocal lattice, k-vectors
# ---------------------------------------------------------------------------------------
def expansion_indices(pw):
    """Integer harmonic pairs (m, n), m varying fastest: flat index k = j*Px + i.

    Follows khepri/expansion.py:4-16 (odd pw asserted; meshgrid(m, n) flattened).
    """
    px, py = pw
    if px % 2 != 1 or py % 2 != 1:
        raise AssertionError("harmonic counts must be odd")
    m = np.arange(-(px - 1) // 2, (px - 1) // 2 + 1)
    n = np.arange(-(py - 1) // 2, (py - 1) // 2 + 1)
    mm, nn = np.meshgrid(m, n)
    return np.vstack([mm.ravel(), nn.ravel()])


def reciprocal_basis(lattice):
    """(b1, b2) with b_i . a_j = 2*pi*delta_ij; khepri/tools.py:64-69."""
    a1, a2 = np.asarray(lattice[0], dtype=float), np.asarray(lattice[1], dtype=float)
    det = a1[0] * a2[1] - a1[1] * a2[0]
    s = TWOPI / det
    b1 = np.array([a2[1] * s, -a2[0] * s])
    b2 = np.array([-a1[1] * s, a1[0] * s])
    return np.stack([b1, b2])


def lattice_vectors(lattice="square", pitch=1.0):
    """khepri/crystal.py:60-74."""
    if isinstance(lattice, str):
        if lattice == "square":
            return pitch * np.asarray([[1.0, 0.0], [0.0, 1.0]])
        if lattice == "hexagonal":
            return pitch * np.asarray([[math.sqrt(3) / 2, 0.5], [math.sqrt(3) / 2, -0.5]])
        raise NotImplementedError(f"This {lattice} magic-string is not emplemented.")
    return np.asarray(lattice)


def g_vectors(pw, lattice):
    """G = m*b1 + n*b2 for every harmonic, shape [2, Nh]; khepri/expansion.py:37-40."""
    rec = reciprocal_basis(lattice)
    idx = expansion_indices(pw)
    return rec[0][:, None] * idx[0][None, :] + rec[1][:, None] * idx[1][None, :]


def k_vectors(gvec, kp, wavelength, eps=1.0):
    """Normalised (Kx, Ky, Kz) = (kp + G, kz)/k0; kz = conj(sqrt(k0^2 conj(eps) - kx^2 - ky^2)).

    Follows khepri/expansion.py:43-50 and kz_from_kplanar expansion.py:19-26.
    """
    k0 = TWOPI / wavelength
    kx = np.asarray(kp[0], dtype=complex) + gvec[0]
    ky = np.asarray(kp[1], dtype=complex) + gvec[1]
    kz = np.conj(np.sqrt((k0 ** 2 * np.conj(eps) - kx ** 2 - ky ** 2).astype(complex)))
    return kx / k0, ky / k0, kz / k0


def compute_kplanar(eps_inc, wavelength, theta_deg=0.0, phi_deg=0.0):
    """In-plane wavevector of the incident plane wave; khepri/tools.py:17-21."""
    phi, theta = np.deg2rad(phi_deg), np.deg2rad(theta_deg)
    direction = np.array([np.cos(phi), np.sin(phi)], dtype=complex)
    return direction * cmath.sqrt(eps_inc) * TWOPI / wavelength * np.sin(theta)


# ---------------------------------------------------------------------------------------
# Convolution (Toeplitz) matrix
# ---------------------------------------------------------------------------------------
def fourier_coefficients(eps_map):
    """fftshift(fft2(eps)) / (Nx*Ny); khepri/tools.py:33-35."""
    eps_map = np.asarray(eps_map)
    return np.fft.fftshift(np.fft.fft2(eps_map)) / eps_map.size


def convolution_matrix_fourier(coefs, pw):
    """C[r, c] = coefs[g0x + p_r - p_c, g0y + q_r - q_c] with r = q*Px + p.

    Vectorised form of the double loop in khepri/tools.py:38-56 (g0 = floor(N/2)).
    """
    px, py = pw
    nx, ny = coefs.shape
    r = np.arange(px * py)
    p, q = r % px, r // px
    ix = nx // 2 + p[:, None] - p[None, :]
    iy = ny // 2 + q[:, None] - q[None, :]
    return coefs[ix, iy].astype(complex)


def convolution_matrix(eps_map, pw):
    """khepri/tools.py:33-35."""
    return convolution_matrix_fourier(fourier_coefficients(eps_map), pw)


# ---------------------------------------------------------------------------------------
# Per-layer eigenmodes and S-matrices (khepri/alternative.py)
# ---------------------------------------------------------------------------------------
def _branch_kz(arg):
    """kz with the uniform/free-space branch: Re(arg) < 0 -> -i*sqrt(-arg), else sqrt(arg).

    alternative.py:92-96 and 145-149.
    """
    arg = np.asarray(arg, dtype=complex).copy()
    neg = arg.real < 0
    out = np.empty_like(arg)
    out[neg] = -1j * np.sqrt(-arg[neg])
    out[~neg] = np.sqrt(arg[~neg])
    return out


def _block_diag4(a, b, c, d):
    """[[diag(a), diag(b)], [diag(c), diag(d)]] as a dense 2N x 2N matrix."""
    return np.block([[np.diag(a), np.diag(b)], [np.diag(c), np.diag(d)]])


def free_space_eigenmodes(kx, ky):
    """Gap medium (eps = 1): W0 = I, V0 = Q0 / (i kz0) column-wise; alternative.py:84-99."""
    nh = len(kx)
    q0 = _block_diag4(kx * ky, 1 - kx ** 2, ky ** 2 - 1, -ky * kx)
    kz = _branch_kz(1 - kx ** 2 - ky ** 2)
    lam = np.concatenate([1j * kz, 1j * kz])
    return np.eye(2 * nh, dtype=complex), q0 / lam[None, :]


def solve_uniform_layer(kx, ky, eps):
    """Analytic modes of a homogeneous layer: W = I, lambda = i kz, V = Q / lambda.

    alternative.py:130-156 (mu_r = 1).
    """
    nh = len(kx)
    q = _block_diag4(kx * ky, eps - kx ** 2, ky ** 2 - eps, -ky * kx)
    kz = _branch_kz(eps - kx ** 2 - ky ** 2)
    lam = np.concatenate([1j * kz, 1j * kz])
    return np.eye(2 * nh, dtype=complex), q / lam[None, :], lam


def solve_structured_layer(kx, ky, conv):
    """Modes of a patterned layer: eig(P Q), lambda = principal sqrt, V = Q W / lambda.

    alternative.py:158-178.  P uses C^-1 K products (solve(C, K)), Q uses C.
    """
    nh = len(kx)
    eye = np.eye(nh, dtype=complex)
    ic_kx = np.linalg.solve(conv, np.diag(kx))
    ic_ky = np.linalg.solve(conv, np.diag(ky))
    dkx, dky = np.diag(kx), np.diag(ky)
    p = np.block([[dkx @ ic_ky, eye - dkx @ ic_kx], [dky @ ic_ky - eye, -dky @ ic_kx]])
    q = np.block([[dkx @ dky, conv - dkx @ dkx], [dky @ dky - conv, -dky @ dkx]])
    lam2, w = np.linalg.eig(p @ q)
    lam = np.sqrt(lam2 + 0j)
    v = (q @ w) / lam[None, :]
    return w, v, lam


def build_scatmat(w, v, w0, v0, lam, depth, k0):
    """Symmetric-layer S-matrix with propagator X = diag(exp(-lambda k0 d)).

    alternative.py:181-195: A = W^-1 W0 + V^-1 V0, B = W^-1 W0 - V^-1 V0,
    T = A - X B A^-1 X B, S11 = S22 = T^-1 (X B A^-1 X A - B), S12 = S21 = T^-1 X (A - B A^-1 B).
    """
    t1 = np.linalg.solve(w, w0)
    t2 = np.linalg.solve(v, v0)
    a, b = t1 + t2, t1 - t2
    x = np.diag(np.exp(-lam * depth * k0))
    ainv_x = np.linalg.solve(a, x)
    t = a - x @ b @ ainv_x @ b
    s11 = np.linalg.solve(t, x @ b @ ainv_x @ a - b)
    s12 = np.linalg.solve(t, x @ (a - b @ np.linalg.solve(a, b)))
    return np.array([[s11, s12], [s12, s11]])


def _half_space_blocks(kx, ky, w0, v0, eps):
    """Shared part of the two half-space S-matrices; alternative.py:32-56, 59-82."""
    q = _block_diag4(kx * ky, eps - kx ** 2, ky ** 2 - eps, -ky * kx)
    kz = np.conj(np.sqrt((eps - kx ** 2 - ky ** 2).astype(complex)))
    lam = np.concatenate([1j * kz, 1j * kz])
    w = np.eye(2 * len(kx), dtype=complex)
    v = q / lam[None, :]
    a = np.linalg.solve(w0, w) + np.linalg.solve(v0, v)
    b = np.linalg.solve(w0, w) - np.linalg.solve(v0, v)
    return a, b, w, v, lam


def scattering_reflection(kx, ky, w0, v0, eps):
    """Incidence half-space: S11 = -A^-1 B, S12 = 2A^-1, S21 = (A - B A^-1 B)/2, S22 = B A^-1.

    alternative.py:32-56.
    """
    a, b, w, v, lam = _half_space_blocks(kx, ky, w0, v0, eps)
    ainv = np.linalg.inv(a)
    s = np.array([[-np.linalg.solve(a, b), 2 * ainv],
                  [0.5 * (a - b @ np.linalg.solve(a, b)), b @ ainv]])
    return s, w, v, lam


def scattering_transmission(kx, ky, w0, v0, eps):
    """Emergence half-space: S11 = B A^-1, S12 = (A - B A^-1 B)/2, S21 = 2A^-1, S22 = -A^-1 B.

    alternative.py:59-82.
    """
    a, b, w, v, lam = _half_space_blocks(kx, ky, w0, v0, eps)
    ainv = np.linalg.inv(a)
    s = np.array([[b @ ainv, 0.5 * (a - b @ np.linalg.solve(a, b))],
                  [2 * ainv, -np.linalg.solve(a, b)]])
    return s, w, v, lam


def scattering_identity(n):
    """[[0, I], [I, 0]]; alternative.py:220-232 (block form)."""
    eye = np.eye(n, dtype=complex)
    zero = np.zeros((n, n), dtype=complex)
    return np.array([[zero, eye], [eye, zero]])


def redheffer_product(sa, sb):
    """Star product SA * SB with four separate solves; alternative.py:19-30."""
    eye = np.eye(sa.shape[-1], dtype=complex)
    d = eye - sb[0, 0] @ sa[1, 1]
    f = eye - sa[1, 1] @ sb[0, 0]
    s11 = sa[0, 0] + sa[0, 1] @ np.linalg.solve(d, sb[0, 0]) @ sa[1, 0]
    s12 = sa[0, 1] @ np.linalg.solve(d, sb[0, 1])
    s21 = sb[1, 0] @ np.linalg.solve(f, sa[1, 0])
    s22 = sb[1, 1] + sb[1, 0] @ np.linalg.solve(f, sa[1, 1]) @ sb[0, 1]
    return np.array([[s11, s12], [s21, s22]])


def stack_layers(smats, mask):
    """Forward chain I*S_0*...*S_L (copies where mask) and the reverse chain; layer.py:35-60."""
    n = smats[0].shape[-1]
    stot = scattering_identity(n)
    forward = []
    for s, keep in zip(smats, mask):
        stot = redheffer_product(stot, s)
        forward.append(stot.copy() if keep else None)
    srev = scattering_identity(n)
    rmask = list(reversed(mask[1:]))
    reverse = []
    for i, s in enumerate(reversed(smats[1:])):
        reverse.append(srev.copy() if rmask[i] else None)
        srev = redheffer_product(s.copy(), srev)
    reverse.append(srev.copy())
    return forward, list(reversed(reverse)), stot


# ---------------------------------------------------------------------------------------
# Source and fluxes
# ---------------------------------------------------------------------------------------
def incident(pw, te, tm, k_vector):
    """Plane-wave source vector [ex, ey] with a delta at harmonic (Nh-1)//2.

    alternative.py:101-128: (te, tm) normalised; aTE = -(z_dev x kbar)/|.|, aTM = aTE x kbar/|.|,
    with z_dev = (0, 0, -1); at normal incidence aTE = x, aTM = y.
    """
    norm = math.hypot(abs(te), abs(tm))
    te, tm = te / norm, tm / norm
    kvec = np.asarray(k_vector, dtype=complex)
    kp_norm = np.linalg.norm(kvec[:2])
    kbar = kvec / np.linalg.norm(kvec)
    if abs(kp_norm) < 1e-8:
        a_te = np.array([1.0, 0.0, 0.0], dtype=complex)
        a_tm = np.array([0.0, 1.0, 0.0], dtype=complex)
    else:
        z_dev = np.array([0.0, 0.0, -1.0], dtype=complex)
        a_te = -np.cross(z_dev, kbar)
        a_te = a_te / np.linalg.norm(a_te)
        a_tm = np.cross(a_te, kbar)
        a_tm = a_tm / np.linalg.norm(a_tm)
    nh = pw[0] * pw[1]
    pol = te * a_te + tm * a_tm
    out = np.zeros(2 * nh, dtype=complex)
    out[(nh - 1) // 2] = pol[0]
    out[nh + (nh - 1) // 2] = pol[1]
    return out


def poynting_fluxes(gvec, c_out, kp, wavelength, epsi, eps_medium):
    """Per-order power t_g = Re(kz_g)/Re(kzi) (|sx|^2+|sy|^2+|sz|^2), sz = -(kx sx + ky sy)/kz.

    alternative.py:235-245 (kz in the exit medium, kzi in the incidence medium).
    """
    k0 = TWOPI / wavelength
    kzi = np.conj(cmath.sqrt(k0 ** 2 * epsi - kp[0] ** 2 - kp[1] ** 2)) / k0
    nh = len(c_out) // 2
    sx, sy = c_out[:nh], c_out[nh:]
    kx, ky, kz = k_vectors(gvec, kp, wavelength, eps_medium)
    sz = -(kx * sx + ky * sy) / kz
    t = kz.real / np.real(kzi) * (np.abs(sx) ** 2 + np.abs(sy) ** 2 + np.abs(sz) ** 2)
    return np.sum(t), t


# ---------------------------------------------------------------------------------------
# Fields (khepri/fields.py, khepri/fourier.py:136-142)
# ---------------------------------------------------------------------------------------
def eigenbasis_matrix(w, v):
    """[[W, W], [-V, V]]; fields.py:46-51."""
    return np.block([[w, w], [-v, v]])


def translate_mode_amplitudes(sl, sr, c1p):
    """c+ = (I - Sl22 Sr11)^-1 Sl21 c1p, c- = Sr11 c+; fields.py:18-27."""
    f = np.eye(len(c1p)) - sl[1, 1] @ sr[0, 0]
    cp = np.linalg.solve(f, sl[1, 0] @ c1p)
    return cp, sr[0, 0] @ cp


def fourier_fields(ri, lam, r0, amps, zbar):
    """RI (L o RI^-1 R0 c) with L = [exp(lam zbar), exp(-lam zbar)] clamped at |L| <= 1e14.

    fields.py:53-62.
    """
    prop = np.concatenate([np.exp(lam * zbar), np.exp(-lam * zbar)])
    big = np.abs(prop) > 1e14
    prop[big] = prop[big] / (np.abs(prop[big]) / 1e14)
    out = ri @ (prop * np.linalg.solve(ri, r0 @ np.concatenate(amps)))
    return np.split(out, 4)


def longitudinal_fields(sx, sy, ux, uy, kx, ky, ic):
    """uz = -i(kx sy - ky sx); sz = -i IC (kx uy - ky ux); fields.py:68-76."""
    uz = -1j * (kx * sy - ky * sx)
    if np.ndim(ic) == 0:
        sz = -1j * ic * (kx * uy - ky * ux)
    else:
        sz = -1j * ic @ (kx * uy - ky * ux)
    return sz, uz


def idft(coefs, kx, ky, x, y):
    """sum_g c_g exp(i (kx_g x + ky_g y)) on the points (x, y); fourier.py:136-142."""
    phase = np.exp(1j * (kx[:, None] * x.ravel()[None, :] + ky[:, None] * y.ravel()[None, :]))
    return (coefs[:, None] * phase).sum(axis=0).reshape(x.shape)


# ---------------------------------------------------------------------------------------
# Crystal restatement (khepri/crystal.py)
# ---------------------------------------------------------------------------------------
class OracleCrystal:
    """Stateful solver with the reference's Crystal method names and semantics.

    khepri/crystal.py:42-400 (square / hexagonal / explicit lattices; uniform and pixmap layers;
    half-space media epsi/epse).  Layers are solved once per unique name (crystal.py:183-186).
    """

    def __init__(self, pw, lattice="square", lattice_pitch=1, void=False, epsi=1, epse=1):
        self.pw = tuple(pw)
        self.lattice = lattice_vectors(lattice, lattice_pitch)
        self.gvec = g_vectors(self.pw, self.lattice)
        self.nh = self.pw[0] * self.pw[1]
        self.void = void
        self.epsi, self.epse = epsi, epse
        self.layers = {}
        self.source = None
        self.S = None

    def add_layer_uniform(self, name, epsilon, depth):
        """crystal.py:97-103."""
        self.layers[name] = SimpleNamespace(kind="uniform", eps=epsilon, depth=depth, fields=False)

    def add_layer_pixmap(self, name, epsilon, depth):
        """crystal.py:113-117 (the array is kept by reference, layer.py:108)."""
        self.layers[name] = SimpleNamespace(kind="pixmap", eps=epsilon, depth=depth, fields=False)

    def add_layer_analytical(self, name, epsilon, epsilon_host, depth):
        """crystal.py:119-123: islands description (Drawing.islands()) and host permittivity."""
        self.layers[name] = SimpleNamespace(kind="analytical", eps=epsilon, eps_host=epsilon_host, depth=depth,
                                            fields=False)

    def set_device(self, layers_stack, fields_mask=False):
        """crystal.py:131-164."""
        self.device_stack = list(layers_stack)
        self.global_stacking = ([] if self.void else ["Sref"]) + list(layers_stack) + ([] if self.void else ["Strans"])
        if not self.void:
            self.layers.setdefault("Sref", SimpleNamespace(kind="inc", eps=self.epsi, depth=0, fields=True))
            self.layers.setdefault("Strans", SimpleNamespace(kind="trn", eps=self.epse, depth=0, fields=True))
        if isinstance(fields_mask, bool):
            fields_mask = [fields_mask] * len(layers_stack)
        self.stack_retain_mask = [True] + list(fields_mask) + [True]
        for name, keep in zip(self.global_stacking, self.stack_retain_mask):
            self.layers[name].fields |= keep

    @property
    def depth(self):
        """crystal.py:166-178."""
        return sum(self.layers[n].depth for n in self.device_stack)

    def set_source(self, wavelength, te=1.0, tm=1.0, theta=0.0, phi=0.0, kp=None):
        """crystal.py:345-360."""
        self.source = SimpleNamespace(te=te, tm=tm, theta=theta, phi=phi, wavelength=wavelength)
        if kp is not None:
            self.kp = (kp[0], kp[1])
        else:
            self.kp = tuple(compute_kplanar(self.epsi, wavelength, theta, phi))
        self.k0 = TWOPI / wavelength
        self.kzi = np.conj(cmath.sqrt(self.k0 ** 2 * self.epsi - self.kp[0] ** 2 - self.kp[1] ** 2))

    def _solve_layer(self, layer, kx, ky, w0, v0, k0):
        """layer.py:145-194."""
        if layer.kind in ("pixmap", "analytical"):
            conv = (convolution_matrix(layer.eps, self.pw) if layer.kind == "pixmap" else
                    analytical_convolution_matrix(layer.eps, layer.eps_host, self.pw, self.lattice))
            layer.IC = np.linalg.inv(conv)
            layer.W, layer.V, layer.L = solve_structured_layer(kx, ky, conv)
            layer.S = build_scatmat(layer.W, layer.V, w0, v0, layer.L, layer.depth, k0)
        elif layer.kind == "uniform":
            layer.W, layer.V, layer.L = solve_uniform_layer(kx, ky, layer.eps)
            layer.S = build_scatmat(layer.W, layer.V, w0, v0, layer.L, layer.depth, k0)
            layer.IC = 1 / layer.eps
        elif layer.kind == "inc":
            layer.S, layer.W, layer.V, layer.L = scattering_reflection(kx, ky, w0, v0, layer.eps)
            layer.IC = 1 / layer.eps
        else:
            layer.S, layer.W, layer.V, layer.L = scattering_transmission(kx, ky, w0, v0, layer.eps)
            layer.IC = 1 / layer.eps

    def solve(self):
        """crystal.py:180-206."""
        assert self.source is not None, "Call set_source before solving."
        wl = self.source.wavelength
        kx, ky, _ = k_vectors(self.gvec, self.kp, wl)
        w0, v0 = free_space_eigenmodes(kx, ky)
        for name in set(self.global_stacking):
            self._solve_layer(self.layers[name], kx, ky, w0, v0, TWOPI / wl)
        stacked = [self.layers[n] for n in self.global_stacking]
        pos = list(np.cumsum([l.depth for l in stacked]))
        pos[-1] = np.inf
        if not self.void:
            pos.insert(0, -np.inf)
        self.stack_positions = pos
        self.stacking_matrices, self.stacking_reverse_matrices, self.Stot = stack_layers(
            [l.S for l in stacked], self.stack_retain_mask)
        self.S = self.Stot

    def poynting_flux_end(self, only_total=True):
        """crystal.py:363-396 (W_ref = I, so c1p = inc)."""
        assert self.S is not None, "Call solve first"
        wl = self.source.wavelength
        inc = incident(self.pw, self.source.te, self.source.tm, (self.kp[0], self.kp[1], self.kzi))
        w_ref, w_trn = self.layers["Sref"].W, self.layers["Strans"].W
        c1p = np.linalg.inv(w_ref) @ inc
        t = poynting_fluxes(self.gvec, w_trn @ self.Stot[1, 0] @ c1p, self.kp, wl, self.epsi, self.epse)
        r = poynting_fluxes(self.gvec, w_ref @ self.Stot[0, 0] @ c1p, self.kp, wl, self.epsi, self.epsi)
        if only_total:
            return r[0].real, t[0].real
        return r, t

    # -- fields -------------------------------------------------------------------------
    def _locate(self, z):
        """crystal.py:208-232."""
        idx = int(np.searchsorted(self.stack_positions, z)) - 1
        zr = z if z <= 0 else z - self.stack_positions[idx]
        return self.layers[self.global_stacking[idx]], idx, zr

    def _fourier_fields(self, z, inc_fields):
        """crystal.py:234-279."""
        layer, idx, zr = self._locate(z)
        assert layer.fields, f"Layer at {z} did not store eigenspace."
        wl = self.source.wavelength
        k0 = TWOPI / wl
        kx, ky, _ = k_vectors(self.gvec, self.kp, wl)
        w0, v0 = free_space_eigenmodes(kx, ky)
        ri = eigenbasis_matrix(layer.W, layer.V)
        r0 = eigenbasis_matrix(w0, v0)
        rref = eigenbasis_matrix(self.layers["Sref"].W, self.layers["Sref"].V)
        n = 2 * self.nh
        c1p = np.linalg.solve(rref, inc_fields)[:n]
        cp, cm = translate_mode_amplitudes(self.stacking_matrices[idx], self.stacking_reverse_matrices[idx], c1p)
        sx, sy, ux, uy = fourier_fields(ri, layer.L, r0, (cp, cm), k0 * (layer.depth - zr))
        sz, uz = longitudinal_fields(sx, sy, ux, uy, kx, ky, layer.IC)
        return sx, sy, sz, ux, uy, uz

    def source_fields(self):
        """crystal.py:281-295: (E, H) source vectors with H = 0."""
        e = incident(self.pw, self.source.te, self.source.tm, (self.kp[0], self.kp[1], self.kzi))
        return e, np.zeros_like(e)

    def fields_coords_xy(self, x, y, z, incident_fields=None):
        """crystal.py:297-333."""
        x, y = np.asarray(x), np.asarray(y)
        assert x.shape == y.shape and x.ndim == 2, "x and y must be 2D meshgrids"
        assert self.S is not None, "Call solve first."
        if incident_fields is None:
            incident_fields = np.concatenate(self.source_fields())
        elif isinstance(incident_fields, tuple):
            incident_fields = np.concatenate(incident_fields)
        wl = self.source.wavelength
        k0 = TWOPI / wl
        kx, ky, _ = k_vectors(self.gvec, self.kp, wl)
        ff = self._fourier_fields(z, incident_fields)
        out = np.asarray([idft(s, k0 * kx, k0 * ky, x, y) for s in ff])
        return out[:3], out[3:]

    def fields_volume(self, x, y, z, incident_fields=None):
        """crystal.py:335-343: E, H of shape [Nz, 3, X, Y]."""
        if incident_fields is None:
            incident_fields = self.source_fields()
        inc = np.concatenate(incident_fields)
        res = [self.fields_coords_xy(x, y, zi, inc) for zi in z]
        return np.asarray([r[0] for r in res]), np.asarray([r[1] for r in res])


def solve_rt(pw, layers, stack, wavelength, te=1.0, tm=1.0, theta=0.0, phi=0.0, kp=None,
             lattice="square", epsi=1, epse=1, only_total=True):
    """Convenience wrapper: build a Crystal, solve once, return poynting_flux_end() (the user
    loop of README.md:52-58 over crystal.py:180-206 and 363-396)."""
    cl = OracleCrystal(pw, lattice=lattice, epsi=epsi, epse=epse)
    for name, (kind, eps, depth) in layers.items():
        if kind == "uniform":
            cl.add_layer_uniform(name, eps, depth)
        else:
            cl.add_layer_pixmap(name, eps, depth)
    cl.set_device(stack, False)
    cl.set_source(wavelength, te, tm, theta, phi, kp)
    cl.solve()
    return cl.poynting_flux_end(only_total)


# ---------------------------------------------------------------------------------------
# Twisted bilayers: product expansions and extended layers (khepri/expansion.py:52-73,
# khepri/extension.py:10-126)
# ---------------------------------------------------------------------------------------
def rotation_matrix(angle_rad):
    """tools.py:23-24."""
    c, s = math.cos(angle_rad), math.sin(angle_rad)
    return np.array([[c, -s], [s, c]])


def twisted_g_vectors(g1, g2):
    """Minkowski sum of two expansions, expansion.py:60-74: index i = i1 * N2 + i2 with g = g1[i1] +
    g2[i2] (the left operand's vectors vary slowest)."""
    return (g1[:, :, None] + g2[:, None, :]).reshape(2, -1)


def joint_subspace(mats, kind):
    """Scatter N matrices of size 2N (one per shift m) into the 2N^2 space; extension.py:10-49.

    Within each polarisation quadrant, kind 0 puts element (a, b) of matrix m at
    (m N + a, m N + b) and kind 1 at (a N + m, b N + m)."""
    n_base = mats[0].shape[0] // 2
    N = n_base
    out = np.zeros((2 * N * N, 2 * N * N), dtype=mats[0].dtype)
    a = np.arange(N)
    for m, mat in enumerate(mats):
        idx = m * N + a if kind == 0 else a * N + m
        for bi in range(2):
            for bj in range(2):
                out[np.ix_(bi * N * N + idx, bj * N * N + idx)] = mat[bi * N:(bi + 1) * N, bj * N:(bj + 1) * N]
    return out


def joint_subspace_s(smats, kind):
    """The four blocks of extended S-matrices; extension.py:52-62."""
    return np.array([[joint_subspace([s[i, j] for s in smats], kind) for j in range(2)] for i in range(2)])


def _base_layer_s(layer, pw, gvec, kp, wavelength):
    """S of one base-expansion layer at in-plane k (layer.py:145-194)."""
    kx, ky, _ = k_vectors(gvec, kp, wavelength)
    w0, v0 = free_space_eigenmodes(kx, ky)
    k0 = TWOPI / wavelength
    kind, eps, depth = layer
    if kind == "pixmap":
        w, v, lam = solve_structured_layer(kx, ky, convolution_matrix(eps, pw))
        return build_scatmat(w, v, w0, v0, lam, depth, k0)
    if kind == "uniform":
        w, v, lam = solve_uniform_layer(kx, ky, eps)
        return build_scatmat(w, v, w0, v0, lam, depth, k0)
    if kind == "inc":
        return scattering_reflection(kx, ky, w0, v0, eps)[0]
    return scattering_transmission(kx, ky, w0, v0, eps)[0]


def twisted_solve_rt(pw, lattice, angle_rad, lower, gap, upper, wavelength, te=1.0, tm=1.0, kp=(0.0, 0.0),
                     epsi=1.0, epse=1.0):
    """R, T of a twisted bilayer as the reference's extended crystal computes them
    (examples/crystal_api/twisted_phc.py:35-57 with crystal.py:180-206, 363-396):
    the incidence half-space and ``lower`` layers use the base expansion e1 (lattice), the
    ``upper`` layers and the emergence half-space use e2 = e1 rotated by ``angle_rad``; every such
    layer's extended S-matrix is the joint subspace of its base solves at kp + g for every g of
    the other expansion (extension.py:82-111); ``gap`` layers are uniform layers of the product
    expansion.  Layers: ("pixmap", eps_map, depth) | ("uniform", eps, depth)."""
    lat = lattice_vectors(lattice) if isinstance(lattice, str) else np.asarray(lattice)
    g1 = g_vectors(pw, lat)
    g2 = rotation_matrix(angle_rad) @ g1
    gsum = twisted_g_vectors(g1, g2)
    N = pw[0] * pw[1]
    kp = np.asarray(kp, dtype=complex)

    def extended(layer, on_e1):
        # base over e1: shifts from e2, kind 1; base over e2: shifts from e1, kind 0
        gb, gs, kind = (g1, g2, 1) if on_e1 else (g2, g1, 0)
        return joint_subspace_s([_base_layer_s(layer, pw, gb, kp + gs[:, m], wavelength) for m in range(N)], kind)

    smats = [extended(("inc", epsi, 0.0), True)]
    smats += [extended(l, True) for l in lower]
    kx, ky, _ = k_vectors(gsum, kp, wavelength)
    w0, v0 = free_space_eigenmodes(kx, ky)
    k0 = TWOPI / wavelength
    for kind, eps, depth in gap:
        w, v, lam = solve_uniform_layer(kx, ky, eps)
        smats.append(build_scatmat(w, v, w0, v0, lam, depth, k0))
    smats += [extended(l, False) for l in upper]
    smats.append(extended(("trn", epse, 0.0), False))
    _, _, stot = stack_layers(smats, [False] * len(smats))
    kzi = np.conj(cmath.sqrt(k0 ** 2 * epsi - kp[0] ** 2 - kp[1] ** 2))
    inc = incident((N, N), te, tm, (kp[0], kp[1], kzi))
    t = poynting_fluxes(gsum, stot[1, 0] @ inc, kp, wavelength, epsi, epse)
    r = poynting_fluxes(gsum, stot[0, 0] @ inc, kp, wavelength, epsi, epsi)
    return r[0].real, t[0].real, stot


# ---------------------------------------------------------------------------------------
# Analytical layers: closed-form Fourier coefficients of islands (khepri/layer.py:161-168,
# khepri/fourier.py:7-68, 145-159)
# ---------------------------------------------------------------------------------------
def _fexpz(z):
    """(exp(z) - 1) / z with the reference's series below |z| = 1e-2; fourier.py:7-20."""
    z = np.asarray(z, dtype=complex)
    out = np.empty_like(z)
    big = np.abs(z) > 1e-2
    out[big] = (np.exp(z[big]) - 1.0) / z[big]
    s = z[~big]
    out[~big] = 1 + s / 2.0 * (1 + s / 3.0 * (1 + s / 4.0 * (1 + s / 5.0 * (1 + s / 6.0 * (1 + s / 7)))))
    return out


def island_transform(island, gx, gy, sigma):
    """2-D Fourier transform of one island at (gx, gy); fourier.py:23-58 (rectangle, disc)."""
    kind, p = island["type"], island["params"]
    if kind == "rectangle":
        ll0, ll1, ur0, ur1 = p
        a, b = ur0 - ll0, ur1 - ll1
        return a * b / sigma * _fexpz(-1j * gx * a) * _fexpz(-1j * gy * b) * np.exp(-1j * (ll0 * gx + ll1 * gy))
    if kind == "disc":
        from scipy import special
        c0, c1, r = p
        norm = np.sqrt(gx * gx + gy * gy) * r
        at0 = np.isclose(gx, 0.0) & np.isclose(gy, 0.0)
        out = np.zeros_like(gx, dtype=complex)
        nz = ~at0
        out[nz] = np.pi * r ** 2 / sigma * 2 * np.exp(-1j * (c0 * gx[nz] + c1 * gy[nz])) * special.jv(1.0, norm[nz]) / norm[nz]
        out[at0] = np.pi * r ** 2 / sigma
        return out
    raise NotImplementedError(kind)


def analytical_convolution_matrix(islands, eps_host, pw, lattice="square"):
    """C of an analytical layer: island transforms on the expanded grid (3 Px x 3 Py harmonics,
    expansion.py:86-92), combined with the host (fourier.py:145-159), the flat array reshaped to
    that grid as the reference does, then the Toeplitz rule (tools.py:38-56); layer.py:161-168."""
    lat = lattice_vectors(lattice) if isinstance(lattice, str) else np.asarray(lattice, dtype=float)
    recip = reciprocal_basis(lat)
    sigma = abs(lat[0, 0] * lat[1, 1] - lat[0, 1] * lat[1, 0])
    epw = tuple(e * 3 if e > 1 else 1 for e in pw)
    idx = expansion_indices(epw)
    g = np.sum(recip[:, :, None] * idx[:, None], axis=0)
    gx, gy = g[0], g[1]
    length = gx.shape[0]
    eps_g = np.zeros(length, dtype=complex)
    eps_g[(length - 1) // 2] = eps_host
    for isl in islands:
        eps_g += (isl["epsilon"] - eps_host) * island_transform(isl, gx, gy, sigma)
    return convolution_matrix_fourier(eps_g.reshape(epw), pw)


# ------------------------------------------------------------------------------------------
# Band structure from S (khepri/eigentricks.py:5-55)
# ------------------------------------------------------------------------------------------
def scattering_splitlr(S):
    """eigentricks.py:5-23: the pencil (Sl, Sr) of a dense [4 ng, 4 ng] S."""
    ng = S.shape[0] // 4
    p = np.s_[0:2 * ng]
    m = np.s_[2 * ng:4 * ng]
    Sl = np.zeros_like(S)
    Sl[p, p] = S[p, p]
    Sl[m, p] = S[m, p]
    Sl[m, m] = -np.eye(2 * ng, dtype=S.dtype)
    Sr = np.zeros_like(S)
    Sr[p, p] = np.eye(2 * ng, dtype=S.dtype)
    Sr[p, m] = -S[p, m]
    Sr[m, m] = -S[m, m]
    return Sl, Sr


def scattering_det(S):
    """eigentricks.py:25-29."""
    ng = S.shape[0] // 4
    p = np.s_[0:2 * ng]
    m = np.s_[2 * ng:4 * ng]
    return np.linalg.det(S[p, p] - S[p, m] @ np.linalg.inv(S[m, m]) @ S[m, p]) * np.linalg.det(S[m, m])


def scattering_eigenvalues(S, dos=False):
    """eigentricks.py:30-39: generalized eigenpairs of (Sl, Sr) by QZ (scipy.linalg.eig)."""
    from scipy.linalg import eig
    Sl, Sr = scattering_splitlr(S)
    if np.any(np.isnan(Sr)) or np.any(np.isnan(Sl)):
        return None
    w, v = eig(Sl, Sr)
    return (w, v, scattering_det(S)) if dos else (w, v)


def band_structure(S):
    """eigentricks.py:46-55."""
    res = scattering_eigenvalues(S)
    if res is None:
        return None
    w = res[0].real
    w = w[w > 0]
    w = w[w < 1]
    return w[np.isclose(np.abs(w), 1.0, rtol=0.0, atol=1e-10)]


def match_eigenvalues(a, b):
    """Largest relative distance from each finite value of b to its nearest value in a (a test
    helper for eigenvalue sets whose order is arbitrary)."""
    a = np.asarray(a)
    b = np.asarray(b)
    b = b[np.isfinite(b)]
    if b.size == 0:
        return 0.0
    d = np.abs(b[:, None] - a[None, :]).min(axis=1)
    return float((d / np.maximum(1.0, np.abs(b))).max())


# ------------------------------------------------------------------------------------------
# Brillouin-zone-integrated beams (khepri/beams.py:164-207)
# ------------------------------------------------------------------------------------------
def amplitudes_from_fields(fields, g, kp, x, y, bzs):
    """beams.py:164-190 with fourier.slow_dft (fourier.py:94-104): fields [X, Y, 2, 3] divided by
    exp(i kp.r), cut into bzs[0] x bzs[1] cells of ns x ns samples, the cells' direct DFTs at the
    g vectors [2, ng] summed, over (cells * ns).  The reference's cut pairs the samples of cell i
    ((c1 ns + ix, c0 ns + iy), c0 = i // bzs[1], c1 = i % bzs[1]) with the coordinates of
    ((d1 ns + ix, d0 ns + iy), d1 = i // bzs[0], d0 = i % bzs[0]); restated by these index maps."""
    b0, b1 = bzs
    X, Y = x.shape
    ns = X // b1
    F = fields / np.exp(1j * (kp[0] * x + kp[1] * y))[..., None, None]
    F = F[..., :2].reshape(X, Y, 4)  # (Ex, Ey, Hx, Hy)
    cells = b0 * b1
    i = np.arange(cells)[:, None, None]
    ix = np.arange(ns)[None, :, None]
    iy = np.arange(ns)[None, None, :]
    fr, fc = (i % b1) * ns + ix, (i // b1) * ns + iy
    cr, cc = (i // b0) * ns + ix, (i % b0) * ns + iy
    vals = F[fr, fc].reshape(-1, 4)
    xs = x[cr, cc].reshape(-1)
    ys = y[cr, cc].reshape(-1)
    ph = np.exp(-1j * (np.outer(xs, g[0]) + np.outer(ys, g[1])))  # [points, ng]
    return (vals.T @ ph) / (cells * ns)


def gen_bzi_grid(shape, a=1, reciproc=None):
    """beams.py:193-207."""
    if reciproc is None:
        b1, b2 = [2 * np.pi / a, 0], [0, 2 * np.pi / a]
    else:
        b1, b2 = reciproc
    si, sj = 1 / shape[0], 1 / shape[1]
    i, j = np.meshgrid(np.arange(-0.5 + si / 2, 0.5, si), np.arange(-0.5 + sj / 2, 0.5, sj), indexing="ij")
    return np.stack([b1[0] * i + b2[0] * j, b1[1] * i + b2[1] * j])


# ------------------------------------------------------------------------------------------
# tmat formulation (khepri/tmat/lattice.py, tools.py, matrices.py, scattering.py): SI units,
# the layer's transfer matrix from expm of the 4 ng x 4 ng field matrix, sliced and squared by
# star products in the dense [p; m] layout.
# ------------------------------------------------------------------------------------------
MU0C = 4 * math.pi * 1e-7 * 299792458.0  # constants.py:3-5


def tmat_grid_size(pw):
    """tools.py:27-37: (nx, ny) and the q grid of the Fourier coefficients."""
    if pw[0] % 2 == 0:
        nx, ny = pw[0] // 2, pw[1] // 2
        return (nx, ny), (4 * nx, 4 * ny)
    nx, ny = (pw[0] - 1) // 2, (pw[1] - 1) // 2
    return (nx, ny), (4 * nx + 1, 4 * ny + 1)


def tmat_lattice(pw, a1, a2):
    """lattice.py:32-87: reciprocal basis, the q-grid G vectors and the pw sub-grid g vectors
    (cut with q[0] on both axes, as lattice.py:77-84)."""
    coef = TWOPI / (a1[0] * a2[1] - a1[1] * a2[0])
    b1 = (a2[1] * coef, -a2[0] * coef)
    b2 = (-a1[1] * coef, a1[0] * coef)
    _, q = tmat_grid_size(pw)
    cx = q[0] // 2 if q[0] % 2 == 0 else (q[0] - 1) // 2
    cy = q[1] // 2 if q[1] % 2 == 0 else (q[1] - 1) // 2
    m1 = np.arange(q[0]) - cx
    m2 = np.arange(q[1]) - cy
    Gx = np.add.outer(b1[0] * m1, b2[0] * m2)
    Gy = np.add.outer(b1[1] * m1, b2[1] * m2)
    nx = q[0] // 4 if q[0] % 2 == 0 else (q[0] - 1) // 4
    ny = q[1] // 4 if q[1] % 2 == 0 else (q[1] - 1) // 4
    cut = np.s_[nx:q[0] - nx, ny:q[0] - ny]
    return SimpleNamespace(pw=tuple(pw), b1=b1, b2=b2, q=q, Gx=Gx, Gy=Gy, gx=Gx[cut], gy=Gy[cut],
                           area=abs(a1[0] * a2[1] - a1[1] * a2[0]))


def tmat_kz(gx, gy, eps, wavelength, kp):
    """tools.py:39-47: kz with Im >= 0 (and Re >= 0 when Im == 0)."""
    u2 = np.abs(kp[0] + gx) ** 2 + np.abs(kp[1] + gy) ** 2
    kz = np.emath.sqrt(eps * (TWOPI / wavelength) ** 2 - u2).astype(complex)
    flip = (kz.imag < 0.0) | (np.isclose(kz.imag, 0.0) & (kz.real < 0.0))
    return np.where(flip, -kz, kz)


def _unit_planar(gx, gy, kp):
    ux = (kp[0] + gx).astype(complex)
    uy = (kp[1] + gy).astype(complex)
    nrm = np.sqrt(np.abs(ux) ** 2 + np.abs(uy) ** 2)
    small = nrm ** 2 < np.finfo(float).eps
    safe = np.where(small, 1.0, nrm)
    return np.where(small, 1.0, ux / safe), np.where(small, 0.0, uy / safe)


def tmat_eta(gx, gy, kp):
    """tools.py:49-59: eta = (u_y, -u_x) of the unit planar wavevector ((0, -1) at u = 0)."""
    ux, uy = _unit_planar(gx, gy, kp)
    return uy, -ux


def tmat_mu(gx, gy, kz, eps, wavelength, kp):
    """tools.py:62-71: mu = kz / (sqrt(eps) k0) u."""
    ux, uy = _unit_planar(gx, gy, kp)
    f = kz / (cmath.sqrt(eps) * TWOPI / wavelength)
    return f * ux, f * uy


def _blocks_to_dense(blocks, ng):
    M = np.zeros((4 * ng, 4 * ng), dtype=complex)
    for (i, j), d in blocks.items():
        M[i * ng:(i + 1) * ng, j * ng:(j + 1) * ng] += np.diag(d)
    return M


def tmat_u_blocks(kz, eta, mu, eps, wavelength):
    """matrices.py:9-42 (matrix_u) as its 4 x 4 blocks of diagonals, harmonics in .T order."""
    hU = MU0C / cmath.sqrt(eps)
    mgx, mgy = mu[0].T.ravel(), mu[1].T.ravel()
    egx, egy = eta[0].T.ravel(), eta[1].T.ravel()
    dg = cmath.sqrt(eps) * math.pi / wavelength / kz.T.ravel()
    return {(0, 0): dg * mgy, (2, 0): dg * mgy, (0, 1): -dg * mgx, (2, 1): -dg * mgx,
            (1, 0): dg * egy, (3, 0): -dg * egy, (1, 1): -dg * egx, (3, 1): dg * egx,
            (0, 2): -hU * dg * egy, (2, 2): hU * dg * egy, (1, 2): hU * dg * mgy, (3, 2): hU * dg * mgy,
            (1, 3): -hU * dg * mgx, (3, 3): -hU * dg * mgx, (2, 3): -hU * dg * egx, (0, 3): hU * dg * egx}


def tmat_v_blocks(eta, mu, eps):
    """matrices.py:44-74 (matrix_v) as its 4 x 4 blocks of diagonals."""
    hV = np.sqrt(eps) / MU0C
    mgx, mgy = mu[0].T.ravel(), mu[1].T.ravel()
    egx, egy = eta[0].T.ravel(), eta[1].T.ravel()
    return {(0, 0): egx, (1, 0): egy, (2, 0): hV * mgx, (3, 0): hV * mgy,
            (0, 1): -mgx, (1, 1): -mgy, (2, 1): hV * egx, (3, 1): hV * egy,
            (0, 2): egx, (1, 2): egy, (2, 2): -hV * mgx, (3, 2): -hV * mgy,
            (0, 3): mgx, (1, 3): mgy, (2, 3): hV * egx, (3, 3): hV * egy}


def tmat_uv(lat, wavelength, kp, eps_incid, eps_emerg):
    """lattice.py:138-171: U (incidence), Vi (incidence), Ve (emergence), dense."""
    ng = lat.gx.size
    kzi = tmat_kz(lat.gx, lat.gy, eps_incid, wavelength, kp)
    kze = tmat_kz(lat.gx, lat.gy, eps_emerg, wavelength, kp)
    eta = tmat_eta(lat.gx, lat.gy, kp)
    mui = tmat_mu(lat.gx, lat.gy, kzi, eps_incid, wavelength, kp)
    mue = tmat_mu(lat.gx, lat.gy, kze, eps_emerg, wavelength, kp)
    return (_blocks_to_dense(tmat_u_blocks(kzi, eta, mui, eps_incid, wavelength), ng),
            _blocks_to_dense(tmat_v_blocks(eta, mui, eps_incid), ng),
            _blocks_to_dense(tmat_v_blocks(eta, mue, eps_emerg), ng))


def tmat_epsilon_g(q, islands_data, eps_host, inverse=False):
    """tools.py:76-86."""
    f = (lambda v: 1 / v) if inverse else (lambda v: v)
    out = np.zeros(q, dtype=complex)
    out[q[0] // 2, q[1] // 2] = f(eps_host)
    for bf, e in islands_data:
        out += (f(e) - f(eps_host)) * bf
    return out


def tmat_indices(pw, nxy):
    """tools.py:73-75 (coords_from_index, Fortran order) for every harmonic."""
    g = np.arange(pw[0] * pw[1])
    return np.stack([g % pw[0] - nxy[0], g // pw[0] - nxy[1]], axis=1)


def tmat_matrix_a(pw, gx, gy, eps_g, epsinv_g, wavelength, kp):
    """matrices.py:126-169 (matrix_a): 4 x 4 blocks of ng x ng, vectorised."""
    nx, ny = gx.shape[0] // 2, gx.shape[1] // 2
    ind = tmat_indices(pw, (nx, ny))
    c1 = TWOPI / wavelength
    ieo, iseo, imo, ismo = 1j / MU0C * c1, 1j * MU0C / c1, 1j * MU0C * c1, 1j / MU0C / c1
    ng = gx.size
    ux = kp[0] + gx.T.ravel()
    uy = kp[1] + gy.T.ravel()
    d1 = ind[:, 0][:, None] - ind[:, 0][None, :] + 2 * nx
    d2 = ind[:, 1][:, None] - ind[:, 1][None, :] + 2 * ny
    E = eps_g[d1, d2]
    Ei = epsinv_g[d1, d2]
    I = np.eye(ng)
    A = np.zeros((4 * ng, 4 * ng), dtype=complex)

    def put(i, j, M):
        A[i * ng:(i + 1) * ng, j * ng:(j + 1) * ng] = M

    put(2, 0, -ismo * np.diag(ux * uy))
    put(3, 0, -ismo * np.diag(uy ** 2) + ieo * E)
    put(2, 1, ismo * np.diag(ux ** 2) - ieo * E)
    put(3, 1, ismo * np.diag(ux * uy))
    put(1, 2, -imo * I + iseo * uy[:, None] * Ei * uy[None, :])
    put(0, 3, imo * I - iseo * ux[:, None] * Ei * ux[None, :])
    put(0, 2, iseo * ux[:, None] * Ei * uy[None, :])
    put(1, 3, -iseo * uy[:, None] * Ei * ux[None, :])
    return A


def tmat_matrix_s(T):
    """matrices.py:171-180."""
    h = T.shape[0] // 2
    p, m = np.s_[0:h], np.s_[h:2 * h]
    S = np.zeros_like(T)
    S[p, p] = np.linalg.inv(T[p, p])
    S[p, m] = -S[p, p] @ T[p, m]
    S[m, p] = T[m, p] @ S[p, p]
    S[m, m] = T[m, m] + T[m, p] @ S[p, m]
    return S


def tmat_multS(S1, S2):
    """matrices.py:194-212: star product in the dense [p; m] layout."""
    h = S1.shape[0] // 2
    p, m = np.s_[0:h], np.s_[h:2 * h]
    I0 = np.eye(h, dtype=S1.dtype)
    I = I0 - S1[p, m] @ S2[m, p]
    G1 = np.linalg.solve(I, S1[p, p])
    G2 = np.linalg.solve(I, S1[p, m])
    S = np.empty_like(S1)
    S[p, p] = S2[p, p] @ G1
    S[m, p] = S1[m, p] + S1[m, m] @ S2[m, p] @ G1
    S[p, m] = S2[p, m] + S2[p, p] @ G2 @ S2[m, m]
    S[m, m] = S1[m, m] @ (I0 + S2[m, p] @ G2) @ S2[m, m]
    return S


def tmat_layer_smatrix(A, U, Vi, depth, slicing_pow):
    """scattering.py:25-51: T = U expm(-A d / 2^p) Vi, S = matrix_s(T), squared p times."""
    from scipy.linalg import expm
    E = expm(-A * (depth / 2 ** slicing_pow))
    S = tmat_matrix_s(U @ E @ Vi)
    for _ in range(slicing_pow):
        S = tmat_multS(S, S)
    return S, E
