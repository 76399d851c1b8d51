"""The team-generic dense kernels (Hessenberg reduction, windowed QR, eigenvectors, LU) compiled
for the host and run by a team of one thread: the same source as the GPU kernels, checked here
against numpy on every CPU run (tests/host/team_dense_host.cpp)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("needs g++")
    out = tmp_path_factory.mktemp("teamhost") / "libteamhost.so"
    src = os.path.join(ROOT, "tests", "host", "team_dense_host.cpp")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "khepri_gb300", "csrc"), src, "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    P, I = ctypes.c_void_p, ctypes.c_int
    L.host_gehrd.argtypes = [I, P, P, I]
    L.host_geev.argtypes = [I, P, P, P]
    L.host_geev_f32.argtypes = [I, P, P, P]
    L.host_gesv.argtypes = [I, I, P, P]
    L.host_geev_log.argtypes = [I, P, P, P, I]
    L.host_geev_unwindowed.argtypes = [I, P, P, P]
    L.host_geev_unwindowed_f32.argtypes = [I, P, P, P]
    L.host_geev_log_f32.argtypes = [I, P, P, P, I]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _rand(n, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(dtype)


@pytest.mark.parametrize("n", [8, 64, 97, 131])
def test_hessenberg_blocked_matches_unblocked(lib, n):
    A = _rand(n, n)
    out = {}
    for blocked in (0, 1):
        H = A.copy()
        Z = np.zeros_like(A)
        lib.host_gehrd(n, _p(H), _p(Z), blocked)
        assert np.abs(np.tril(H, -2)).max() == 0.0
        assert np.abs(Z.conj().T @ Z - np.eye(n)).max() < 1e-13
        assert np.abs(Z @ H @ Z.conj().T - A).max() / np.abs(A).max() < 1e-13
        out[blocked] = (H, Z)
    # the same reflectors, applied in another order: the same H and Q up to rounding
    assert np.abs(out[0][0] - out[1][0]).max() < 1e-10
    assert np.abs(out[0][1] - out[1][1]).max() < 1e-11


def _match(lam, ref):
    """max |lam_i - ref_j| over a greedy nearest matching."""
    ref = list(ref)
    worst = 0.0
    for v in lam:
        k = int(np.argmin(np.abs(np.asarray(ref) - v)))
        worst = max(worst, abs(ref[k] - v))
        ref.pop(k)
    return worst


@pytest.mark.parametrize("n", [1, 2, 33, 70, 150])
def test_geev_fp64(lib, n):
    A = _rand(n, 100 + n)
    W = np.zeros_like(A)
    lam = np.zeros(n, np.complex128)
    assert lib.host_geev(n, _p(A.copy()), _p(W), _p(lam)) == 0
    scale = np.abs(A).max() * n
    assert np.abs(A @ W - W * lam).max() / (scale * np.abs(W).max()) < 1e-13
    assert _match(lam, np.linalg.eigvals(A)) / scale < 1e-12


def test_geev_fp32(lib):
    n = 80
    A = _rand(n, 5, np.complex64)
    W = np.zeros_like(A)
    lam = np.zeros(n, np.complex64)
    assert lib.host_geev_f32(n, _p(A.copy()), _p(W), _p(lam)) == 0
    A64, W64 = A.astype(np.complex128), W.astype(np.complex128)
    assert np.abs(A64 @ W64 - W64 * lam).max() / (np.abs(A).max() * n * np.abs(W).max()) < 1e-5


@pytest.mark.parametrize("n", [2, 3, 5, 33, 34, 70, 150])
def test_windowed_qr_matches_unwindowed(lib, n):
    # the windowed sweep (bulge chased inside a shared-memory window, the rows and columns outside
    # it updated afterwards) applies the same rotations in the same order to every element as the
    # one-rotation-at-a-time sweep: identical results
    for dtype, fn, fn_ref in ((np.complex128, lib.host_geev, lib.host_geev_unwindowed),
                              (np.complex64, lib.host_geev_f32, lib.host_geev_unwindowed_f32)):
        A = _rand(n, 500 + n, dtype)
        W0, lam0 = np.zeros_like(A), np.zeros(n, dtype)
        W, lam = np.zeros_like(A), np.zeros(n, dtype)
        assert fn_ref(n, _p(A.copy()), _p(W0), _p(lam0)) == 0
        assert fn(n, _p(A.copy()), _p(W), _p(lam)) == 0
        assert np.array_equal(lam, lam0), (dtype, np.abs(lam - lam0).max())
        assert np.array_equal(W, W0), (dtype, np.abs(W - W0).max())


@pytest.mark.parametrize("n", [5, 33, 70, 150])
def test_geev_rotation_log_is_exact(lib, n):
    # Z updated through the rotation log (deferred, and flushed by the team whenever the log is
    # full) receives the same rotations in the same order as the eager update: identical results
    for dtype, fn, fn_log in ((np.complex128, lib.host_geev, lib.host_geev_log),
                              (np.complex64, lib.host_geev_f32, lib.host_geev_log_f32)):
        A = _rand(n, 300 + n, dtype)
        W0, lam0 = np.zeros_like(A), np.zeros(n, dtype)
        assert fn(n, _p(A.copy()), _p(W0), _p(lam0)) == 0
        # room for every sweep; room for about three sweeps (many flushes); room for one sweep
        for cap in (100 * n * n, 3 * n, max(n - 1, 1)):
            W, lam = np.zeros_like(A), np.zeros(n, dtype)
            assert fn_log(n, _p(A.copy()), _p(W), _p(lam), cap) == 0
            assert np.array_equal(lam, lam0), (dtype, cap)
            assert np.array_equal(W, W0), (dtype, cap, np.abs(W - W0).max())


def test_geev_repeated_and_real_spectrum(lib):
    # a defect-free matrix with a double eigenvalue and a real one
    n = 12
    rng = np.random.default_rng(9)
    X = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    d = np.array([2.0, 2.0] + list(rng.standard_normal(n - 2)), dtype=np.complex128)
    A = X @ np.diag(d) @ np.linalg.inv(X)
    W = np.zeros_like(A)
    lam = np.zeros(n, np.complex128)
    assert lib.host_geev(n, _p(A.copy()), _p(W), _p(lam)) == 0
    assert _match(lam, d) < 1e-8


@pytest.mark.parametrize("n,m", [(5, 1), (40, 3), (100, 7)])
def test_lu_solve(lib, n, m):
    A = _rand(n, 200 + n)
    rng = np.random.default_rng(n)
    B = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
    X = B.copy()
    assert lib.host_gesv(n, m, _p(A.copy()), _p(X)) == 0
    ref = np.linalg.solve(A, B)
    assert np.abs(X - ref).max() / np.abs(ref).max() < 1e-11


def _sweep_pq(i):
    """P Q of the 11x11 sweep structure's patterned layer at sweep problem i (the eigenproblem of
    alternative.py:158-178), built by the oracle's formulas."""
    import sys
    sys.path.insert(0, ROOT)
    from khepri_gb300 import workloads
    from oracle import khepri_oracle as ko

    st = workloads.batched_structure(0)
    wl, kp = workloads.batched_problems()
    eps = [v for v in st.layers.values() if v[0] == "pixmap"][0][1]
    conv = ko.convolution_matrix(eps, st.pw)
    kx, ky, _ = ko.k_vectors(ko.g_vectors(st.pw, ko.lattice_vectors("square")), kp[i], wl[i])
    eye = np.eye(len(kx))
    ic_kx, ic_ky = np.linalg.solve(conv, np.diag(kx)), np.linalg.solve(conv, np.diag(ky))
    dkx, dky = np.diag(kx), np.diag(ky)
    p = np.block([[dkx @ ic_ky, eye - dkx @ ic_kx], [dky @ ic_ky - eye, -dky @ ic_kx]])
    q = np.block([[dkx @ dky, conv - dkx @ dkx], [dky @ dky - conv, -dky @ dkx]])
    return p @ q


@pytest.mark.parametrize("i", [0, 2])
def test_windowed_qr_matches_unwindowed_sweep_matrices(lib, i):
    # the sweep's 242 x 242 P Q matrices split in the middle during the FP32 QR (the active block's
    # first row moves, and with it every later window), which random matrices rarely do: the
    # windowed sweep must stay identical to the unwindowed one there too
    M = _sweep_pq(i)
    n = M.shape[0]
    for dtype, fn, fn_ref in ((np.complex64, lib.host_geev_f32, lib.host_geev_unwindowed_f32),
                              (np.complex128, lib.host_geev, lib.host_geev_unwindowed)):
        A = M.astype(dtype)
        W0, lam0 = np.zeros_like(A), np.zeros(n, dtype)
        W, lam = np.zeros_like(A), np.zeros(n, dtype)
        assert fn_ref(n, _p(A.copy()), _p(W0), _p(lam0)) == 0
        assert fn(n, _p(A.copy()), _p(W), _p(lam)) == 0
        assert np.array_equal(lam, lam0), (dtype, np.abs(lam - lam0).max())
        assert np.array_equal(W, W0), (dtype, np.abs(W - W0).max())
