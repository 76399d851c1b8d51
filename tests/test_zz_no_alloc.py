"""The star product entry point that allocates nothing (khp_star_product_noalloc).

Some callers cannot give libkhp a workspace: their device memory is partitioned up front, or
they run a latency-critical loop where a cudaMalloc (which may synchronise the device) is not
allowed.  khp_star_product_noalloc takes its scratch from a fixed device array inside the
library instead.  This test calls it through the C ABI twice in a row (the shared scratch keeps
the previous call's contents) and compares each result with the workspace-based
khp_star_product on the same inputs.  It sits in its own file so that pytest collects it last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # both entry points run the same FP64 kernels; agreement is to rounding


def _random_smatrix(rng, batch, n, scale):
    a = rng.standard_normal((batch, 2, 2, n, n)) + 1j * rng.standard_normal((batch, 2, 2, n, n))
    return a * (scale / n)


def test_noalloc_star_product_matches_workspace_version():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from khepri_gb300 import build as kb
    kb.build()
    from khepri_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(5)
    for batch, n, scale in [(7, 50, 0.8), (3, 98, 0.6)]:
        assert lib.khp_star_product_workspace(batch, n) <= 32 * 1024 * 1024
        for _ in range(2):  # two calls in a row on the same shared scratch
            sa = torch.tensor(_random_smatrix(rng, batch, n, scale), device="cuda")
            sb = torch.tensor(_random_smatrix(rng, batch, n, scale), device="cuda")
            ref = torch.empty_like(sa)
            out = torch.full_like(sa, float("nan"))
            st_ref = torch.zeros(batch, dtype=torch.int32, device="cuda")
            st = torch.zeros(batch, dtype=torch.int32, device="cuda")
            ws = torch.empty(lib.khp_star_product_workspace(batch, n), dtype=torch.uint8, device="cuda")
            sp = _capi.stream_ptr()
            nn4 = 4 * n * n
            assert lib.khp_star_product(batch, n, _capi.ptr(sa), nn4, _capi.ptr(sb), nn4, _capi.ptr(ref),
                                        _capi.ptr(st_ref), _capi.ptr(ws), ws.numel(), sp) == 0
            assert lib.khp_star_product_noalloc(batch, n, _capi.ptr(sa), nn4, _capi.ptr(sb), nn4, _capi.ptr(out),
                                                _capi.ptr(st), sp) == 0
            torch.cuda.synchronize()
            assert not st.any() and not st_ref.any()
            err = (out - ref).abs().max().item() / ref.abs().max().item()
            assert err < TOL, err


def test_noalloc_rejects_oversized_batch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from khepri_gb300 import build as kb
    kb.build()
    from khepri_gb300 import _capi
    lib = _capi.load()
    # 64 problems of n = 242 need ~300 MB of scratch: beyond the fixed capacity, refused before any launch.
    dummy = torch.empty(1, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.khp_star_product_noalloc(64, 242, _capi.ptr(dummy), 0, _capi.ptr(dummy), 0, _capi.ptr(dummy),
                                        _capi.ptr(st), None) == 7
