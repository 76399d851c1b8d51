"""The inverse-design gradient (9x9 harmonics, 64x64 densities theta, eps = 1 + 11 sigmoid(theta),
stack [P(0.3), P(0.3), U(2.1, 1.0)], normal incidence, loss = mean over frequencies of the
zeroth-order T) through khepri_gb300.autograd.solve_rt, the torch.autograd.Function over the
hand-written adjoint, against two references on the CPU:

* autograd of the complex128 torch restatement of the reference's solve (oracle/torch_c128.py),
  on every pixel;
* central finite differences of the numpy oracle, on 32 random pixels per design, at h = 1e-6
  (floor 1e-8 for its rounding) and at h = 1e-4.

Tolerance, per element: |g - g_ref| <= 1e-4 |g_ref| + 1e-5 max|g_ref|.  The second term is the
floor of the mixed-precision adjoint: its FP32 products err by ~2e-6 of the largest component on
every pixel, so the per-element 1e-4 bar holds alone for every pixel whose gradient is at least
~2 % of the largest, and pixels with smaller gradients meet the floor.  The errors measured are
printed: per element over the pixels with |g_ref| >= 1e-2 max|g_ref|, and relative to max|g_ref|.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F_IDX = [0, 5, 10, 15]  # of the 16 frequencies 0.4-0.6
REL = 1e-4
FLOOR = 1e-5  # of the largest gradient component


def _setup(designs):
    from khepri_gb300 import workloads
    thetas, structs, freqs = workloads.inverse_design(designs, seed=0)
    return thetas, freqs[F_IDX]


def _structures(designs):
    stack = ["D1", "D2", "Sub"]
    return [((9, 9), {"D1": ("pixmap", d, 0.3), "D2": ("pixmap", d, 0.3), "Sub": ("uniform", 2.1, 1.0)}, stack)
            for d in range(designs)]


def _check(g, ref, what, gmax, floor=0.0):
    err = np.abs(g - ref)
    big = np.abs(ref) >= 1e-2 * gmax
    rel = err[big] / np.abs(ref[big]) if big.any() else np.zeros(1)
    print(f"{what}: max per-element relative error {rel.max():.2e} (median {np.median(rel):.2e}) over the "
          f"{big.sum()} of {ref.size} pixels with |g| >= 1e-2 max|g|; max abs error / max|g| {err.max() / gmax:.2e}")
    bad = err > REL * np.abs(ref) + max(FLOOR * gmax, floor)
    assert not bad.any(), (what, np.argwhere(bad)[:5], g[bad][:5], ref[bad][:5])


def test_autograd_inverse_design_9x9(khp):
    import torch
    from khepri_gb300 import autograd
    from oracle import khepri_oracle as ko
    from oracle import torch_c128 as tc
    D = 2
    thetas, f = _setup(D)
    F = len(f)
    nh = 81
    c = (nh - 1) // 2
    th = torch.tensor(thetas, dtype=torch.float64, device="cuda", requires_grad=True)
    eps = 1.0 + 11.0 * torch.sigmoid(th)
    which = np.repeat(np.arange(D), F)
    wl = np.tile(1.0 / f, D)
    R, T, Ro, To, st = autograd.solve_rt(eps, _structures(D), wl, np.zeros((D * F, 2)), which=which)
    assert not st.any()
    loss = To[:, c].reshape(D, F).mean(1)
    loss.sum().backward()
    g = th.grad.cpu().numpy()
    for d in range(D):
        # autograd of the complex128 restatement
        tt = torch.tensor(thetas[d], dtype=torch.float64, requires_grad=True)
        e = 1.0 + 11.0 * torch.sigmoid(tt)
        lay = {"D1": ("pixmap", e, 0.3), "D2": ("pixmap", e, 0.3), "Sub": ("uniform", 2.1, 1.0)}
        t0 = [tc.solve_orders((9, 9), lay, ["D1", "D2", "Sub"], 1.0 / fk)[3][c] for fk in f]
        ref_loss = torch.stack(t0).mean()
        ref_loss.backward()
        assert abs(ref_loss.item() - loss[d].item()) < 1e-6
        g_ref = tt.grad.numpy()
        gmax = np.abs(g_ref).max()
        _check(g[d], g_ref, f"design {d} vs complex128 autograd", gmax)
        # central differences of the numpy oracle
        rng = np.random.default_rng(100 + d)
        pix = rng.choice(thetas[d].size, 32, replace=False)

        def loss_np(theta):
            en = 1.0 + 11.0 / (1.0 + np.exp(-theta))
            lay_np = {"D1": ("pixmap", en, 0.3), "D2": ("pixmap", en, 0.3), "Sub": ("uniform", 2.1, 1.0)}
            return np.mean([ko.solve_rt((9, 9), lay_np, ["D1", "D2", "Sub"], 1.0 / fk, 1.0, 0.0,
                                        only_total=False)[1][1][c] for fk in f])

        def central(h):
            out = []
            for p in pix:
                i, j = np.unravel_index(p, thetas[d].shape)
                tp, tm = thetas[d].copy(), thetas[d].copy()
                tp[i, j] += h
                tm[i, j] -= h
                out.append((loss_np(tp) - loss_np(tm)) / (2 * h))
            return np.array(out)

        gi = g[d].reshape(-1)[pix]
        # h = 1e-6 (the step the inverse-design spec names): its difference carries the complex128
        # solve's rounding, ~1e-14 / h = 1e-8 absolute, which is 1e-3 of these ~1e-5 gradients;
        # h = 1e-4: truncation ~h^2 = 1e-8 relative.
        for h, floor in ((1e-6, 1e-8), (1e-4, 0.0)):
            _check(gi, central(h), f"design {d} vs central differences h={h:g} (32 pixels)", gmax, floor)
