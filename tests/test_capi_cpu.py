"""CPU-side checks of the boundary: libkhp loads and exports every symbol the header declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^[A-Za-z_][\w \*]*?\b(khp_\w+)\s*\(", text, re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    from khepri_gb300 import build as kb
    kb.build()
    from khepri_gb300 import _capi
    return _capi.load()


def test_header_declares_entry_points():
    names = _declared()
    assert {"khp_version", "khp_status_string", "khp_convmat", "khp_layer_modes", "khp_layer_smatrix",
            "khp_closed_form_smatrix", "khp_star_product", "khp_flux"} <= names


def test_every_declared_symbol_is_exported(lib):
    for name in sorted(_declared()):
        assert hasattr(lib, name), name


def test_binding_covers_header(lib):
    from khepri_gb300 import _capi
    assert set(_capi.exported_symbols()) == _declared()


def test_version_and_status_strings(lib):
    from khepri_gb300 import _capi
    assert lib.khp_version() >= 100
    assert _capi.status_string(0) == "ok"
    assert "workspace" in _capi.status_string(2)
    assert _capi.decode_status(5) == "singular pivot, non-finite value"


def test_workspace_sizes_are_monotone(lib):
    for f, args in [(lib.khp_layer_modes_workspace, (8, 25)), (lib.khp_layer_smatrix_workspace, (8, 25)),
                    (lib.khp_star_product_workspace, (8, 50)), (lib.khp_convmat_workspace, (8, 5, 5))]:
        small = f(*args)
        big = f(args[0] * 2, *args[1:])
        assert 0 < small < big and small % 256 == 0


def test_invalid_arguments_rejected_without_gpu(lib):
    # Validation happens before any CUDA call: even-sized harmonic sets and null pointers.
    assert lib.khp_convmat(1, 16, 16, None, 4, 3, None, None, 0, None) == 1
    assert lib.khp_star_product(1, 10, None, 0, None, 0, None, None, None, 0, None) == 1
    assert lib.khp_flux(1, 3, 3, None, 0, None, None, None, None, None, None, 1.0, 0.0, 1.0, 0.0, None, None, None,
                        None, None) == 1


def test_newer_entry_points_validate_before_any_gpu_work(lib):
    # Each call below returns before it touches a pointer or the GPU: a bad argument (1), an
    # empty batch (0) or missing scratch (2).  P is a non-null placeholder that is never used.
    P = ctypes.c_void_p(256)
    # batched inverse: null operands, unknown precision, short stride, empty batch, no workspace
    assert lib.khp_inverse(1, 8, 0, None, 64, None, 64, None, None, 0, None) == 1
    assert lib.khp_inverse(1, 8, 3, P, 64, P, 64, P, None, 0, None) == 1
    assert lib.khp_inverse(1, 8, 0, P, 63, P, 64, P, None, 0, None) == 1
    assert lib.khp_inverse(0, 8, 0, P, 64, P, 64, P, None, 0, None) == 0
    assert lib.khp_inverse(2, 8, 0, P, 64, P, 64, P, None, 0, None) == 2
    # FP64-accurate tensor-core product: inner size above 4096, empty batch, no workspace
    assert lib.khp_zgemm_fp64_tc(1, 4, 4, 4097, P, 4097, 0, P, 4, 0, P, 4, 0, None, 0, None) == 1
    assert lib.khp_zgemm_fp64_tc(0, 4, 4, 4, P, 4, 16, P, 4, 16, P, 4, 16, None, 0, None) == 0
    assert lib.khp_zgemm_fp64_tc(1, 4, 4, 4, P, 4, 16, P, 4, 16, P, 4, 16, None, 0, None) == 2
    # band structure from S: null S, empty batch
    assert lib.khp_scattering_eig(1, 2, None, 64, None, None, None, None, None, 0, None) == 1
    assert lib.khp_scattering_eig(0, 2, P, 64, P, None, None, P, None, 0, None) == 0
    # beams: empty supercell, no workspace
    assert lib.khp_bzi_amplitudes(0, 1, 4, P, P, P, P, 9, P, P, P, None, 0, None) == 1
    assert lib.khp_bzi_amplitudes(2, 2, 4, P, P, P, P, 9, P, P, P, None, 0, None) == 2
    # tmat star product and S assembly: short stride, empty batch
    assert lib.khp_tmat_multS(1, 2, P, 63, P, 64, P, P, None, 0, None) == 1
    assert lib.khp_tmat_matrix_s(0, 2, P, P, P, None, 0, None) == 0


def test_no_gpu_means_loud_failure():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from khepri_gb300 import Crystal, KhpError
    with pytest.raises(KhpError):
        Crystal((3, 3))


def test_problem_arrays_are_row_major():
    """Problems.make copies its inputs row-major, whatever their memory order (a kp built by
    broadcasting against a transposed array is column-major; the kernels read it as [B][2])."""
    import numpy as np
    from khepri_gb300 import engine
    g = np.random.default_rng(1).standard_normal((2, 9))
    kp = (np.array([[0.3, 0.1]], dtype=complex)[:, None, :] + g.T[None, :, :]).reshape(9, 2)
    assert not kp.flags["C_CONTIGUOUS"]
    p = engine.Problems.make(np.ones(9), kp, 1.0, 0.0, "cpu")
    assert p.kp.is_contiguous() and p.kp.stride() == (2, 1)
    np.testing.assert_array_equal(p.kp.numpy(), kp)
