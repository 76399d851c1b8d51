"""Checks of large matrices against fixtures that hold seeded samples and matrix-vector checksums
instead of every entry (tests/golden/make_golden.py, _pin)."""
import numpy as np


def check_pinned(g, name, M, seed, rtol, atol=0.0):
    """M's sampled entries within atol + rtol |ref|; M r and l M within (atol + rtol max|M|)
    times the checksum vectors' 1-norms, for the seeded vectors the fixture was made with."""
    M = np.asarray(M)
    rng = np.random.default_rng(seed)
    idx = rng.choice(M.size, size=min(M.size, 6000), replace=False)
    r = rng.standard_normal(M.shape[1]) + 1j * rng.standard_normal(M.shape[1])
    l = rng.standard_normal(M.shape[0]) + 1j * rng.standard_normal(M.shape[0])
    assert np.array_equal(idx, g[f"{name}_idx"]), f"{name}: sample positions differ (seed {seed})"
    ref = g[f"{name}_val"]
    got = M.flat[idx]
    err = np.abs(got - ref)
    assert np.all(err <= atol + rtol * np.abs(ref)), f"{name}: entry error {err.max():.3e}"
    tol = atol + rtol * np.abs(M).max()
    e1 = np.abs(M @ r - g[f"{name}_Mr"]).max()
    e2 = np.abs(l @ M - g[f"{name}_lM"]).max()
    assert e1 <= tol * np.abs(r).sum() and e2 <= tol * np.abs(l).sum(), f"{name}: checksum errors {e1:.3e} {e2:.3e}"
