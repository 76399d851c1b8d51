"""The complex128 torch restatement of the solve (oracle/torch_c128.py, the autograd reference for
the gradients) against the numpy oracle, which is pinned to the reference's golden vectors: R, T
and every per-order power to 1e-12.  Its autograd gradient is checked here against central finite
differences of the numpy oracle (CPU only)."""
import numpy as np
import pytest
import torch

from khepri_gb300 import workloads
from oracle import khepri_oracle as ko
from oracle import torch_c128 as tc


def _numpy_orders(pw, layers, stack, wl, te, tm, kp=(0.0, 0.0), epsi=1.0, epse=1.0):
    (r, ro), (t, to) = ko.solve_rt(pw, layers, stack, wl, te, tm, kp=kp, epsi=epsi, epse=epse, only_total=False)
    return r, t, ro, to


@pytest.mark.parametrize("case", ["design", "oblique_lossy"])
def test_torch_oracle_matches_numpy_oracle(case):
    if case == "design":
        thetas, structs, freqs = workloads.inverse_design(1, seed=3, n_pix=32, pw=(5, 5))
        st, wl, kp, te, tm, epsi, epse = structs[0], 1.0 / freqs[5], (0.0, 0.0), 1.0, 0.0, 1.0, 1.0
    else:
        rng = np.random.default_rng(7)
        emap = 2.0 + 8.0 * rng.random((24, 20)) - 0.2j * rng.random((24, 20))
        layers = {"P": ("pixmap", emap, 0.4), "U": ("uniform", 2.25 - 0.05j, 0.3)}
        st = workloads.Structure(pw=(3, 5), layers=layers, stack=["P", "U", "P"])
        wl, te, tm, epsi, epse = 1.7, 0.6, 0.8j, 1.5, 2.0
        kp = tuple(ko.compute_kplanar(epsi, wl, 20.0, 35.0).real)
    ref = _numpy_orders(st.pw, st.layers, st.stack, wl, te, tm, kp, epsi, epse)
    tl = {k: (kind, torch.as_tensor(np.asarray(e)) if kind == "pixmap" else e, d)
          for k, (kind, e, d) in st.layers.items()}
    out = tc.solve_orders(st.pw, tl, st.stack, wl, te, tm, kp=kp, epsi=epsi, epse=epse)
    for a, b in zip(out, ref):
        np.testing.assert_allclose(np.asarray(a.detach()), np.asarray(b), rtol=0, atol=1e-12)


def test_torch_oracle_gradient_matches_finite_differences():
    """d(zeroth-order T)/d(theta) of a 5x5 design by autograd of the torch restatement against
    central differences (h = 1e-6) of the numpy oracle on 6 pixels: per element 1e-4 relative
    (+1e-10).  At h = 1e-6 the differences carry ~1e-9 of rounding (the solve's own ~1e-15 / h);
    at h = 1e-4 they agree with autograd to ~1e-8 relative."""
    thetas, structs, freqs = workloads.inverse_design(1, seed=11, n_pix=16, pw=(5, 5))
    st, wl = structs[0], 1.0 / freqs[3]
    th = torch.tensor(thetas[0], dtype=torch.float64, requires_grad=True)

    def layers_of(eps):
        return {"D1": ("pixmap", eps, 0.3), "D2": ("pixmap", eps, 0.3), "Sub": ("uniform", 2.1, 1.0)}

    eps = 1.0 + 11.0 * torch.sigmoid(th)
    _, _, _, to = tc.solve_orders(st.pw, layers_of(eps), st.stack, wl)
    to[(to.shape[0] - 1) // 2].backward()
    g = th.grad.numpy()

    def t0(theta):
        e = 1.0 + 11.0 / (1.0 + np.exp(-theta))
        _, _, _, t_orders = _numpy_orders(st.pw, layers_of(e), st.stack, wl, 1.0, 0.0)
        return t_orders[(len(t_orders) - 1) // 2]

    rng = np.random.default_rng(0)
    h = 1e-6
    for idx in rng.choice(thetas[0].size, 6, replace=False):
        i, j = np.unravel_index(idx, thetas[0].shape)
        tp, tm_ = thetas[0].copy(), thetas[0].copy()
        tp[i, j] += h
        tm_[i, j] -= h
        fd = (t0(tp) - t0(tm_)) / (2 * h)
        assert abs(g[i, j] - fd) <= 1e-4 * abs(fd) + 1e-10, (i, j, g[i, j], fd)
