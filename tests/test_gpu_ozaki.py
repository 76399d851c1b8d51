"""FP64-accurate complex products on the tensor cores (khp_zgemm_fp64_tc) against torch's FP64
matmul.  The mixed-precision solve forms its eigen-residuals M W and V = Q W with this kernel,
so it must agree with an FP64 product to that product's own rounding bound:
|dC_ij| <= 4 * 2k * 2^-53 * max_l |A_il| * max_l |B_lj| (plus the FP64 reference's own error,
which the same bound covers).  On integer inputs whose products are exact in FP64 the kernel
must be bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, A, B, ldc=None):
    import torch

    from khepri_gb300 import _capi
    batch, m, k = A.shape
    n = B.shape[2]
    ldc = ldc or n
    C = torch.full((batch, m, ldc), complex("nan"), dtype=torch.complex128, device="cuda")
    ws = torch.empty(lib.khp_zgemm_fp64_tc_workspace(batch, m, n, k), dtype=torch.uint8, device="cuda")
    code = lib.khp_zgemm_fp64_tc(batch, m, n, k, _capi.ptr(A), A.stride(1), A.stride(0), _capi.ptr(B), B.stride(1),
                                 B.stride(0), _capi.ptr(C), ldc, m * ldc, _capi.ptr(ws), ws.numel(),
                                 _capi.stream_ptr())
    assert code == 0, _capi.status_string(code)
    torch.cuda.synchronize()
    return C[:, :, :n]


def _bound(A, B):
    import torch
    k = A.shape[2]
    amax = torch.maximum(A.real.abs(), A.imag.abs()).amax(dim=2, keepdim=True)  # [b, m, 1]
    bmax = torch.maximum(B.real.abs(), B.imag.abs()).amax(dim=1, keepdim=True)  # [b, 1, n]
    return 4 * 2 * k * 2.0 ** -53 * amax * bmax


@pytest.fixture(scope="module")
def lib(khp):
    from khepri_gb300 import _capi
    return _capi.load()


@pytest.mark.parametrize("batch,m,n,k", [(3, 242, 242, 242), (2, 37, 19, 53), (1, 64, 64, 64), (4, 121, 242, 121),
                                         (2, 130, 70, 300)])
def test_matches_fp64_product(lib, batch, m, n, k):
    import torch
    g = torch.Generator(device="cpu").manual_seed(m * 1000 + n + k)
    # rows and columns spanning many orders of magnitude, as the k^4 / eps rows of P Q do
    ra = torch.exp(6 * torch.rand(batch, m, 1, generator=g, dtype=torch.float64))
    cb = torch.exp(-6 * torch.rand(batch, 1, n, generator=g, dtype=torch.float64))
    A = (torch.randn(batch, m, k, generator=g, dtype=torch.complex128) * ra).cuda()
    B = (torch.randn(batch, k, n, generator=g, dtype=torch.complex128) * cb).cuda()
    C = _run(lib, A, B)
    ref = A @ B
    err = (C - ref).abs()
    assert torch.isfinite(C).all()
    assert (err <= _bound(A, B)).all(), float((err / _bound(A, B)).max())


def test_strided_operands_and_padded_output(lib):
    """B as the upper half of a wider matrix (the V = Q W shape), C with a row stride > n."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(7)
    batch, nh, n = 3, 61, 122
    A = torch.randn(batch, nh, nh, generator=g, dtype=torch.complex128).cuda()
    W = torch.randn(batch, n, n, generator=g, dtype=torch.complex128).cuda()
    B = W[:, :nh, :]  # row stride n, batch stride n * n
    C = _run(lib, A, B, ldc=n + 5)
    ref = A @ B
    assert ((C - ref).abs() <= _bound(A, B)).all()


def test_exact_on_integer_inputs(lib):
    """Small integers: every product and sum is exact in FP64, so the result must be too."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(11)
    batch, m, n, k = 2, 100, 90, 250
    A = torch.complex(torch.randint(-1000, 1000, (batch, m, k), generator=g).double(),
                      torch.randint(-1000, 1000, (batch, m, k), generator=g).double()).cuda()
    B = torch.complex(torch.randint(-1000, 1000, (batch, k, n), generator=g).double(),
                      torch.randint(-1000, 1000, (batch, k, n), generator=g).double()).cuda()
    C = _run(lib, A, B)
    assert torch.equal(C, A @ B)


def test_zero_rows_columns_and_bad_arguments(lib):
    import torch

    from khepri_gb300 import _capi
    A = torch.zeros(1, 20, 30, dtype=torch.complex128, device="cuda")
    A[0, 3, :] = 1.5 - 2j
    B = torch.zeros(1, 30, 10, dtype=torch.complex128, device="cuda")
    B[0, :, 4] = 0.25j
    C = _run(lib, A, B)
    assert torch.equal(C, A @ B)
    ws = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    bad = lib.khp_zgemm_fp64_tc(1, 20, 10, 5000, _capi.ptr(A), 30, 600, _capi.ptr(B), 10, 300, _capi.ptr(C), 10,
                                200, _capi.ptr(ws), ws.numel(), None)
    assert bad == 1
    small = lib.khp_zgemm_fp64_tc(1, 20, 10, 30, _capi.ptr(A), 30, 600, _capi.ptr(B), 10, 300, _capi.ptr(C), 10,
                                  200, _capi.ptr(ws), 16, None)
    assert small == 2
