"""Plane-wave expansion (khepri/expansion.py:4-73): harmonic indices, g vectors, rotation and
the Minkowski sum used by twisted bilayers.  Host-side bookkeeping, O(number of harmonics)."""
from __future__ import annotations

import numpy as np

from . import engine


def generate_expansion_indices(pw):
    """expansion.py:4-16: [2, px * py] integer indices, the first varying fastest."""
    return engine.expansion_indices(pw)


def kz_from_kplanar(kx, ky, k0, epsilon):
    """expansion.py:19-26: kz = conj(sqrt(k0^2 conj(eps) - kx^2 - ky^2))."""
    arg = k0 ** 2 * np.conj(epsilon) - kx ** 2 - ky ** 2
    return np.conj(np.sqrt(np.asarray(arg, dtype=complex)))


class Expansion:
    """expansion.py:28-84 (the plotting helper is left out)."""

    def __init__(self, pw, lattice=None):
        self.pw = tuple(pw)
        if lattice is None:
            lattice = np.asarray([[1.0, 0.0], [0.0, 1.0]])
        lattice = np.asarray(lattice, dtype=float)
        self.a = float(np.linalg.norm(lattice[0]))
        self.reciprocal = np.asarray(engine.reciprocal_basis(lattice))
        self.expansion_indices = generate_expansion_indices(self.pw)
        self._g_vectors = np.sum(self.reciprocal[:, :, None] * self.expansion_indices[:, None], axis=0)
        self.sigma = abs(lattice[0][0] * lattice[1][1] - lattice[0][1] * lattice[1][0])

    @property
    def g_vectors(self):
        """expansion.py:76-84 (a copy of the [2][Nh] G vectors)."""
        return self._g_vectors.copy()

    def rotate(self, angle_rad):
        """expansion.py:52-53: rotates the G vectors in place."""
        c, s = np.cos(angle_rad), np.sin(angle_rad)
        self._g_vectors = np.array([[c, -s], [s, c]]) @ self._g_vectors

    def __add__(self, rhs):
        """Minkowski sum: index (self index) * N_rhs + (rhs index)."""
        g = (self.g_vectors[:, :, None] + rhs.g_vectors[:, None, :]).reshape(2, -1)
        e = Expansion((self.pw[0] ** 2, self.pw[1] ** 2))
        e._g_vectors = g
        e._base_g_vectors = np.stack((self.g_vectors, rhs.g_vectors))
        e.expansion_lhs = self
        e.expansion_rhs = rhs
        return e

    def g_vectors_expanded(self, mul):
        """expansion.py:86-93: G vectors of a grid ``mul`` times finer (used by analytical layers)."""
        epw = [p * mul if p > 1 else 1 for p in self.pw]
        idx = engine.expansion_indices(epw)
        g = np.sum(self.reciprocal[:, :, None] * idx[:, None], axis=0)
        return g[0], g[1], epw

    def k_vectors(self, k_parallel, wavelength, epsilon=1):
        """expansion.py:95-97 with _compute_k_vector (43-50): K = (k_par + G) and Kz."""
        k0 = 2 * np.pi / wavelength
        k = np.zeros((3, self._g_vectors.shape[1]), dtype=np.complex128)
        k[0:2] = np.asarray(k_parallel)[:, None] + self._g_vectors
        k[2] = kz_from_kplanar(k[0], k[1], k0, epsilon)
        return k / k0
