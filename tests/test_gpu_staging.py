"""Problem inputs reach the device intact when their copies queue behind other work.

engine.Problems.make stages host inputs through pinned memory and queues the copies on the
current stream without waiting; a staging buffer released before its copy ran could be taken by
the next staging and overwritten.  Here the stream is kept busy (torch's own bounded sleep
kernel) while several problem sets of equal sizes are staged.  The inputs must also arrive
row-major whatever their host memory order (a column-major kp once scrambled the twisted path's
k-vectors)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_problem_inputs_survive_a_busy_stream(khp):
    import torch
    from khepri_gb300 import engine
    rng = np.random.default_rng(0)
    want, got = [], []
    torch.cuda._sleep(200_000_000)  # ~0.1 s of device time ahead of the copies
    for _ in range(6):
        wl = rng.uniform(1.0, 3.0, 9)
        kp = rng.standard_normal((9, 2)) + 1j * rng.standard_normal((9, 2))
        te = rng.standard_normal(9) + 1j * rng.standard_normal(9)
        tm = rng.standard_normal(9) + 1j * rng.standard_normal(9)
        want.append((2 * np.pi / wl, kp, te, tm))
        got.append(engine.Problems.make(wl, kp, te, tm, "cuda"))
    torch.cuda.synchronize()
    for (k0, kp, te, tm), p in zip(want, got):
        np.testing.assert_array_equal(p.k0.cpu().numpy(), k0)
        np.testing.assert_array_equal(p.kp.cpu().numpy(), kp)
        np.testing.assert_array_equal(p.te.cpu().numpy(), te)
        np.testing.assert_array_equal(p.tm.cpu().numpy(), tm)


def test_problem_inputs_are_row_major(khp):
    """A column-major kp (as broadcasting against a transposed array builds it) arrives row-major:
    the kernels read kp as [B][2]."""
    import torch
    from khepri_gb300 import engine
    g = np.random.default_rng(1).standard_normal((2, 9))
    kp = (np.array([[0.3, 0.1]], dtype=complex)[:, None, :] + g.T[None, :, :]).reshape(9, 2)
    assert kp.flags["F_CONTIGUOUS"] and not kp.flags["C_CONTIGUOUS"]
    p = engine.Problems.make(np.ones(9), kp, 1.0, 0.0, "cuda")
    torch.cuda.synchronize()
    assert p.kp.is_contiguous()
    np.testing.assert_array_equal(p.kp.cpu().numpy(), kp)
