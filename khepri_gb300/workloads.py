"""Seeded synthetic inputs for the RCWA solve workloads.

No public dataset is involved in the reference's benchmarks; these generators produce the
structures the sweeps are quoted on, deterministically from ``numpy.random.default_rng(seed)``:

* ``disc_canvas`` — a disc on a pixmap with the reference Drawing conventions
  (khepri/draw.py:20-44: axis 0 is x, grid ``linspace(-0.5, 0.5, N)`` including both ends,
  points strictly inside the radius take the disc permittivity).
* ``plain_sweep`` — 5x5 harmonics, [patterned, uniform, patterned], 151 frequencies
  (examples/crystal_api/test_crystal.py:23-43 at a 128x128 pixmap).
* ``batched_sweep`` — 11x11 harmonics, union of 1-4 periodic discs (eps 12 in eps 1) on a
  256x256 map, 3 patterned + 2 uniform layers, 64 frequencies x a 32x32 Bloch grid x 2
  polarisations.
* ``uneven_batch`` — structures with odd harmonic counts 3..17, 1-8 lossy smoothed layers.
* ``inverse_design`` — sigmoid densities on 64x64 maps, 9x9 harmonics.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

TWOPI = 2.0 * math.pi


def disc_canvas(n, radius, eps_disc, eps_background, center=(0.0, 0.0), shape=None):
    """Pixmap eps[x, y] with one disc, Drawing semantics (khepri/draw.py:30-44)."""
    nx, ny = (n, n) if shape is None else shape
    xs = np.linspace(-0.5, 0.5, nx)
    ys = np.linspace(-0.5, 0.5, ny)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    canvas = np.full((nx, ny), float(eps_background))
    canvas[np.sqrt((X - center[0]) ** 2 + (Y - center[1]) ** 2) < radius] = eps_disc
    return canvas


def bzi_grid(shape, a=1.0):
    """Cell-centred first-Brillouin-zone grid of a square lattice, shape [2, s0, s1].

    Same point set as khepri/beams.py:193-207 (gen_bzi_grid).
    """
    b = TWOPI / a
    si, sj = 1.0 / shape[0], 1.0 / shape[1]
    i, j = np.meshgrid(np.arange(-0.5 + si / 2, 0.5, si), np.arange(-0.5 + sj / 2, 0.5, sj), indexing="ij")
    return np.stack([b * i, b * j])


def periodic_gaussian_blur(img, sigma_px):
    """Periodic Gaussian smoothing by multiplication in Fourier space."""
    nx, ny = img.shape
    fx = np.fft.fftfreq(nx)[:, None]
    fy = np.fft.fftfreq(ny)[None, :]
    kernel = np.exp(-2.0 * math.pi ** 2 * sigma_px ** 2 * (fx ** 2 + fy ** 2))
    return np.fft.ifft2(np.fft.fft2(img) * kernel).real


def multi_disc_map(rng, n=256, eps_in=12.0, eps_out=1.0, max_discs=4):
    """Union of U{1..max_discs} discs, centres U(0,1)^2, radii U(0.1,0.3), minimum-image distance.

    Pixel i sits at x = i/n (axis 0 = x).
    """
    k = int(rng.integers(1, max_discs + 1))
    centres = rng.uniform(0.0, 1.0, size=(k, 2))
    radii = rng.uniform(0.1, 0.3, size=k)
    xs = np.arange(n) / n
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    inside = np.zeros((n, n), dtype=bool)
    for (cx, cy), r in zip(centres, radii):
        dx = X - cx
        dy = Y - cy
        dx -= np.round(dx)
        dy -= np.round(dy)
        inside |= dx * dx + dy * dy < r * r
    return np.where(inside, eps_in, eps_out).astype(float)


@dataclass
class Structure:
    """One layer stack: ``layers`` maps a name to ('pixmap', eps_map, depth) or ('uniform', eps, depth)."""

    pw: tuple
    layers: dict
    stack: list
    epsi: complex = 1.0
    epse: complex = 1.0
    lattice: str = "square"


@dataclass
class Sweep:
    """A structure and the (wavelength, kp, te, tm) problems solved on it."""

    structure: Structure
    wavelengths: np.ndarray
    kp: np.ndarray  # [P, 2] absolute in-plane wavevector per problem
    te: np.ndarray = field(default_factory=lambda: np.array([1.0]))
    tm: np.ndarray = field(default_factory=lambda: np.array([0.0]))


def plain_sweep(pw=(5, 5), n_pix=128, nfreq=151):
    """5x5, 128x128 map eps 12 with an eps-1 disc r=0.4, [P(0.55), U(1, 1.1), P(0.55)], normal incidence."""
    canvas = disc_canvas(n_pix, 0.4, 1.0, 12.0)
    st = Structure(pw=tuple(pw), layers={"S1": ("uniform", 1.0, 1.1), "Scyl": ("pixmap", canvas, 0.55)},
                   stack=["Scyl", "S1", "Scyl"])
    f = np.linspace(0.49, 0.60, nfreq)
    return Sweep(st, 1.0 / f, np.zeros((nfreq, 2)), np.array([1.0]), np.array([0.0]))


def batched_structure(seed, pw=(11, 11), n_pix=256):
    """One seed of the 11x11 batched sweep: [P1, U1, P2, U2, P3] sharing one multi-disc map."""
    rng = np.random.default_rng(seed)
    emap = multi_disc_map(rng, n_pix)
    d = rng.uniform(0.2, 1.0, size=5)
    eu = rng.uniform(1.0, 4.0, size=2)
    layers = {
        "P1": ("pixmap", emap, d[0]), "U1": ("uniform", eu[0], d[1]),
        "P2": ("pixmap", emap, d[2]), "U2": ("uniform", eu[1], d[3]),
        "P3": ("pixmap", emap, d[4]),
    }
    return Structure(pw=tuple(pw), layers=layers, stack=["P1", "U1", "P2", "U2", "P3"])


def batched_problems(nfreq=64, nk=32):
    """(wavelength, kp) pairs of the sweep: frequencies 0.3-0.7 c/a x an nk x nk cell-centred BZ grid.

    Problem index = f_index * nk*nk + k_index (frequency slowest).
    """
    f = np.linspace(0.3, 0.7, nfreq)
    kg = bzi_grid((nk, nk)).reshape(2, -1).T  # [nk*nk, 2]
    wl = np.repeat(1.0 / f, kg.shape[0])
    kp = np.tile(kg, (nfreq, 1))
    return wl, kp


def uneven_structures(count, seed=0, n_pix=128, max_pw=17, max_layers=8):
    """Structures with odd harmonic counts 3..max_pw and 1..max_layers lossy smoothed layers.

    Re eps = blur(U(1,12)), Im eps = -blur(U(0,0.1)) (negative imaginary part = loss in the
    reference's convention), sigma = 4 px; depths U(0.2,1.0); one frequency U(0.3,0.8) and a
    k-point uniform in the part of the first zone inside the light cone (|kp| < k0), where the
    incident wave propagates and R, T are defined.  Returns a list of (Structure, wavelength, kp).
    """
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        p = int(rng.choice(np.arange(3, max_pw + 1, 2)))
        nl = int(rng.integers(1, max_layers + 1))
        layers, stack = {}, []
        for li in range(nl):
            re = periodic_gaussian_blur(rng.uniform(1.0, 12.0, size=(n_pix, n_pix)), 4.0)
            im = -periodic_gaussian_blur(rng.uniform(0.0, 0.1, size=(n_pix, n_pix)), 4.0)
            layers[f"L{li}"] = ("pixmap", re + 1j * im, float(rng.uniform(0.2, 1.0)))
            stack.append(f"L{li}")
        f = float(rng.uniform(0.3, 0.8))
        while True:
            kp = (rng.uniform(0.0, 1.0, size=2) - 0.5) * TWOPI
            if math.hypot(kp[0], kp[1]) < 0.98 * TWOPI * f:
                break
        out.append((Structure(pw=(p, p), layers=layers, stack=stack), 1.0 / f, kp))
    return out


def inverse_design(count, seed=0, n_pix=64, pw=(9, 9)):
    """Designs theta ~ N(0,1), rho = sigmoid(theta), eps = 1 + 11 rho; stack [P(0.3), P(0.3), U(2.1, 1.0)]."""
    rng = np.random.default_rng(seed)
    thetas = rng.standard_normal(size=(count, n_pix, n_pix))
    structs = []
    for th in thetas:
        eps = 1.0 + 11.0 / (1.0 + np.exp(-th))
        layers = {"D1": ("pixmap", eps, 0.3), "D2": ("pixmap", eps, 0.3), "Sub": ("uniform", 2.1, 1.0)}
        structs.append(Structure(pw=tuple(pw), layers=layers, stack=["D1", "D2", "Sub"]))
    return thetas, structs, np.linspace(0.4, 0.6, 16)
