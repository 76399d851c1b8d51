"""Solve + gradient (khp_solve_batched_mixed_grad, khp_convmat_bwd) against central finite
differences of the FP64 star-product path, on the inverse-design stack (normal incidence, where
every eigenvalue of P Q is doubly degenerate) and on an oblique, lossy, two-map stack."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# |g_adjoint - g_fd| <= GRAD_RTOL * max|g_fd| + GRAD_ATOL (FP32 O(n^3) work in the gradient,
# FD of the FP64 path with step 1e-5)
GRAD_RTOL = 1e-4
GRAD_ATOL = 1e-7


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def _design_layers(eps):
    return {"D1": ("pixmap", eps, 0.3), "D2": ("pixmap", eps, 0.3), "Sub": ("uniform", 2.1, 1.0)}


def test_grad_inverse_design_fd(khp):
    from khepri_gb300 import batch
    rng = np.random.default_rng(3)
    pw = (5, 5)
    nh = pw[0] * pw[1]
    c = (nh - 1) // 2
    theta = rng.standard_normal((16, 16))
    freqs = np.array([0.42, 0.5, 0.58])
    stack = ["D1", "D2", "Sub"]

    def eps_of(th):
        return 1.0 + 11.0 * _sigmoid(th)

    def loss_fd(th):
        _, _, _, to, _ = batch.solve_rt(pw, _design_layers(eps_of(th)), stack, 1.0 / freqs, np.zeros((3, 2)), 1.0,
                                        0.0, orders=True)
        return to[:, c].mean()

    structs = [(pw, _design_layers(eps_of(theta)), stack)]
    dT = np.zeros((3, nh))
    dT[:, c] = 1.0 / 3.0
    R, T, Ro, To, grads, st = batch.solve_structures_grad(structs, 1.0 / freqs, np.zeros((3, 2)), which=[0, 0, 0],
                                                          dT=dT)
    assert not st.any()
    # forward parity of the per-order powers against the FP64 chain
    _, _, ro64, to64, _ = batch.solve_rt(pw, structs[0][1], stack, 1.0 / freqs, np.zeros((3, 2)), 1.0, 0.0,
                                         orders=True)
    np.testing.assert_allclose(To, to64, atol=1e-8)
    np.testing.assert_allclose(Ro, ro64, atol=1e-8)
    g_eps = grads[0]["D1"]
    np.testing.assert_array_equal(g_eps, grads[0]["D2"])
    s = _sigmoid(theta)
    g_theta = g_eps.real * 11.0 * s * (1.0 - s)
    h = 1e-5
    pix = [(0, 0), (3, 7), (8, 8), (15, 2), (11, 13), (5, 10)]
    g_fd = []
    for (x, y) in pix:
        tp, tm_ = theta.copy(), theta.copy()
        tp[x, y] += h
        tm_[x, y] -= h
        g_fd.append((loss_fd(tp) - loss_fd(tm_)) / (2 * h))
    g_fd = np.array(g_fd)
    g_ad = np.array([g_theta[x, y] for (x, y) in pix])
    print("adjoint", g_ad, "\nfd     ", g_fd)
    assert np.abs(g_ad - g_fd).max() <= GRAD_RTOL * np.abs(g_fd).max() + GRAD_ATOL


def test_grad_oblique_lossy_two_maps_fd(khp):
    from khepri_gb300 import batch
    rng = np.random.default_rng(5)
    pw = (3, 5)
    nh = pw[0] * pw[1]
    m1 = 1.5 + 8.0 * rng.random((12, 14)) - 0.05j * rng.random((12, 14))
    m2 = 2.0 + 5.0 * rng.random((12, 14)) - 0.02j * rng.random((12, 14))
    stack = ["A", "U", "B"]

    def layers_of(a, b):
        return {"A": ("pixmap", a, 0.45), "U": ("uniform", 2.5 - 0.01j, 0.2), "B": ("pixmap", b, 0.35)}

    wl = np.array([1.0 / 0.47, 1.0 / 0.53])
    kp = np.array([[0.3, -0.2], [0.5, 0.4]]) * 2 * np.pi * 0.4
    te, tm = 0.6, 0.8j
    wR = rng.random((2, nh))
    wT = rng.random((2, nh))

    def loss_fd(a, b):
        _, _, ro, to, _ = batch.solve_rt(pw, layers_of(a, b), stack, wl, kp, te, tm, orders=True)
        return float((wR * ro).sum() + (wT * to).sum())

    R, T, Ro, To, grads, st = batch.solve_structures_grad([(pw, layers_of(m1, m2), stack)], wl, kp, which=[0, 0],
                                                          dR=wR, dT=wT, te=te, tm=tm)
    assert not st.any()
    h = 1e-5
    checks = []
    for name, mp in (("A", 0), ("B", 1)):
        g = grads[0][name]
        for (x, y) in [(1, 2), (7, 9), (11, 0)]:
            for part, unit in (("re", 1.0), ("im", 1j)):
                a, b = m1.copy(), m2.copy()
                tgt = a if mp == 0 else b
                tgt[x, y] += h * unit
                lp = loss_fd(a, b)
                tgt[x, y] -= 2 * h * unit
                lm = loss_fd(a, b)
                fd = (lp - lm) / (2 * h)
                ad = (g[x, y] * unit).real
                checks.append((ad, fd))
    ad, fd = np.array(checks).T
    print("adjoint", ad, "\nfd     ", fd)
    assert np.abs(ad - fd).max() <= GRAD_RTOL * np.abs(fd).max() + GRAD_ATOL
