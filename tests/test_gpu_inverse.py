"""Batched explicit inverse (khp_inverse): blocked LU with partial pivoting, A^-1 = U^-1 L^-1 P,
against numpy's inverse, at sizes that end on and off the 32-column panels, with the 256-row
register panels and the shared-memory panels above them, in FP64 and FP32."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import __graft_entry__
    __graft_entry__.build()
    from khepri_gb300 import _capi
    return _capi.load()


def _inverse(lib, A, precision):
    import torch
    from khepri_gb300 import _capi
    batch, n, _ = A.shape
    dt = torch.complex128 if precision == 0 else torch.complex64
    a = torch.from_numpy(A).to(dt).cuda().contiguous()
    x = torch.empty_like(a)
    st = torch.zeros(batch, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.khp_inverse_workspace(batch, n), dtype=torch.uint8, device="cuda")
    code = lib.khp_inverse(batch, n, precision, _capi.ptr(a), n * n, _capi.ptr(x), n * n, _capi.ptr(st), _capi.ptr(ws),
                           ws.numel(), _capi.stream_ptr())
    _capi.check(code, "khp_inverse")
    torch.cuda.synchronize()
    return x.cpu().numpy().astype(np.complex128), st.cpu().numpy()


@pytest.mark.parametrize("n", [1, 7, 32, 33, 100, 242, 256, 300])
@pytest.mark.parametrize("precision", [0, 1])
def test_matches_numpy_inverse(lib, n, precision):
    rng = np.random.default_rng(1000 + n)
    batch = 5
    A = rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))
    A += 0.5 * np.sqrt(n) * np.eye(n)  # moderately conditioned, pivoting still active
    X, st = _inverse(lib, A, precision)
    assert (st == 0).all()
    ref = np.linalg.inv(A)
    # normwise bound: |X - inv(A)| <= c n eps cond(A) |inv(A)|
    eps = 2.0 ** -52 if precision == 0 else 2.0 ** -23
    cond = np.linalg.cond(A)
    err = np.abs(X - ref).max(axis=(1, 2)) / np.abs(ref).max(axis=(1, 2))
    assert (err <= 8 * n * eps * cond).all(), (err, cond)
    resid = np.abs(A @ X - np.eye(n)).max()
    assert resid <= 8 * n * eps * cond.max()


def test_pivoting_on_a_permuted_matrix(lib):
    # a row-permuted well-conditioned matrix whose leading entries are zero: every column must pivot
    n, batch = 64, 3
    rng = np.random.default_rng(7)
    base = np.triu(rng.standard_normal((n, n))) + 4 * np.eye(n) + 0j
    A = np.stack([base[rng.permutation(n)] for _ in range(batch)])
    X, st = _inverse(lib, A, 0)
    assert (st == 0).all()
    assert np.abs(A @ X - np.eye(n)).max() < 1e-10


def test_singular_and_nonfinite_status(lib):
    n = 40
    rng = np.random.default_rng(3)
    A = rng.standard_normal((3, n, n)) + 0j
    A[1, :, 5] = 0.0        # a zero column: singular
    A[2, 3, 3] = np.nan     # a NaN
    _, st = _inverse(lib, A, 0)
    assert st[0] == 0
    assert st[1] & 1
    assert st[2] & 4


def test_bad_arguments(lib):
    from khepri_gb300 import _capi
    assert lib.khp_inverse(1, 0, 0, None, 0, None, 0, None, None, 0, None) == 1
    assert lib.khp_inverse(1, 4, 2, None, 16, None, 16, None, None, 0, None) == 1
    assert lib.khp_inverse_workspace(2, 8) == 2 * 8 * 4
    assert _capi  # the module loaded the symbol table
