"""FP32-accurate complex products by 3xTF32 on the tcgen05 tensor cores (khp_cgemm_tf32x3)
against torch's FP64 product of the same FP32 inputs.  Bound per element, with the operands'
row / column maxima: |dC_ij| <= 2^-19 * 2k * max_l |A_il| * max_l |B_lj| (the dropped lo lo'
term and the TF32 rounding of lo are ~2^-21 each, FP32 accumulation ~2k 2^-24); the test also
states the measured error relative to that bound and to an FP32 SIMT product's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, A, B, ldc=None):
    import torch

    from khepri_gb300 import _capi
    batch, m, k = A.shape
    n = B.shape[2]
    ldc = ldc or n
    C = torch.full((batch, m, ldc), complex("nan"), dtype=torch.complex64, device="cuda")
    ws = torch.empty(lib.khp_cgemm_tf32x3_workspace(batch, m, n, k), dtype=torch.uint8, device="cuda")
    code = lib.khp_cgemm_tf32x3(batch, m, n, k, _capi.ptr(A), A.stride(1), A.stride(0), _capi.ptr(B), B.stride(1),
                                B.stride(0), _capi.ptr(C), ldc, m * ldc, _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
    assert code == 0, _capi.status_string(code)
    torch.cuda.synchronize()
    return C[:, :, :n]


@pytest.fixture(scope="module")
def lib(khp):
    from khepri_gb300 import _capi
    return _capi.load()


@pytest.mark.parametrize("batch,m,n,k", [(3, 242, 242, 242), (2, 37, 19, 53), (1, 128, 64, 16), (4, 121, 242, 121),
                                         (2, 300, 130, 578)])
def test_matches_fp64_product(lib, batch, m, n, k):
    import torch
    g = torch.Generator(device="cpu").manual_seed(m * 1000 + n + k)
    ra = torch.exp(3 * torch.rand(batch, m, 1, generator=g))
    cb = torch.exp(3 * torch.rand(batch, 1, n, generator=g))
    A = (torch.randn(batch, m, k, generator=g) + 1j * torch.randn(batch, m, k, generator=g)) * ra
    B = (torch.randn(batch, k, n, generator=g) + 1j * torch.randn(batch, k, n, generator=g)) * cb
    A, B = A.to(torch.complex64).cuda(), B.to(torch.complex64).cuda()
    C = _run(lib, A, B)
    ref = A.to(torch.complex128) @ B.to(torch.complex128)
    amax = torch.maximum(A.real.abs(), A.imag.abs()).amax(dim=2, keepdim=True).double()
    bmax = torch.maximum(B.real.abs(), B.imag.abs()).amax(dim=1, keepdim=True).double()
    bound = 2.0 ** -19 * 2 * k * amax * bmax
    err = (C.to(torch.complex128) - ref).abs()
    simt = ((A @ B).to(torch.complex128) - ref).abs()
    print(f"{batch}x{m}x{n}x{k}: max err / bound {(err / bound).max().item():.3f}, "
          f"max err {err.max().item():.2e} (FP32 product {simt.max().item():.2e})")
    assert torch.isfinite(C).all()
    assert (err <= bound).all()


def test_strided_operands(lib):
    """Row strides larger than the row and batch strides larger than the matrix."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(5)
    Abig = (torch.randn(2, 70, 90, generator=g) + 1j * torch.randn(2, 70, 90, generator=g)).to(torch.complex64).cuda()
    Bbig = (torch.randn(2, 60, 50, generator=g) + 1j * torch.randn(2, 60, 50, generator=g)).to(torch.complex64).cuda()
    A, B = Abig[:, :64, :40], Bbig[:, :40, :33]
    C = _run(lib, A, B, ldc=40)
    ref = A.to(torch.complex128) @ B.to(torch.complex128)
    assert (C.to(torch.complex128) - ref).abs().max().item() < 2.0 ** -19 * 80 * 4 * 4


def test_argument_errors(lib):
    from khepri_gb300 import _capi
    assert lib.khp_cgemm_tf32x3(1, 0, 4, 4, None, 4, 16, None, 4, 16, None, 4, 16, None, 0, None) == 1
    assert lib.khp_cgemm_tf32x3_workspace(1, 4, 4, 0) == 0
    assert _capi.status_string(1) == "invalid argument"
