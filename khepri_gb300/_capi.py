"""ctypes binding of libkhp (include/khepri_gb300.h).

The library is the only compute path: if it is missing or no CUDA device is present the
calls fail loudly (ImportError / KhpError); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import torch

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libkhp.so")

_c_i64 = ctypes.c_int64
_c_i32 = ctypes.c_int32
_c_p = ctypes.c_void_p
_c_sz = ctypes.c_size_t
_c_d = ctypes.c_double

_SIGNATURES = {
    "khp_version": (ctypes.c_int, []),
    "khp_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "khp_convmat_workspace": (_c_sz, [_c_i64, _c_i32, _c_i32]),
    "khp_convmat": (ctypes.c_int, [_c_i64, _c_i64, _c_i64, _c_p, _c_i32, _c_i32, _c_p, _c_p, _c_sz, _c_p]),
    "khp_structure_prep_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_structure_prep": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_sz,
                                          _c_p]),
    "khp_layer_modes_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_layer_modes": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                       _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_layer_smatrix_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_layer_smatrix": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                         _c_p, _c_sz, _c_p]),
    "khp_closed_form_smatrix": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                               _c_p, _c_p, _c_p, _c_p]),
    "khp_star_product_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_star_product": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_i64, _c_p, _c_i64, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_star_product_noalloc": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_i64, _c_p, _c_i64, _c_p, _c_p, _c_p]),
    "khp_flux": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_p, _c_i64, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_d, _c_d,
                                _c_d, _c_d, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "khp_fields_amplitudes_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_fields_amplitudes": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                             _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_fields_fourier": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                          _c_p, _c_p, _c_p, _c_p]),
    "khp_fields_idft": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_i64, _c_p, _c_p, _c_p, _c_p]),
    "khp_solve_batched_workspace": (_c_sz, [_c_i64, _c_i32, _c_i32, _c_p, _c_p]),
    "khp_solve_batched": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_i64,
                                         _c_p, _c_p,
                                         _c_p, _c_p, _c_p, _c_d, _c_d, _c_d, _c_d, _c_p, _c_p, _c_i32, _c_p, _c_p,
                                         _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_solve_batched_mixed_workspace": (_c_sz, [_c_i64, _c_i32, _c_i32, _c_p, _c_p]),
    "khp_solve_batched_mixed": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                               _c_i64, _c_p,
                                               _c_p, _c_p, _c_p, _c_p, _c_d, _c_d, _c_d, _c_d, _c_p, _c_p, _c_i32,
                                               _c_p, _c_p, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    # khp_solve_batched's arguments up to tm, then mixed_batch, mixed_index, mixed_workspace, mixed_ws_bytes,
    # R, T, status, ws, ws_bytes, stream
    "khp_solve_batched_mixed_repair": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p,
                                                      _c_p, _c_i64, _c_p, _c_p, _c_p, _c_p, _c_p, _c_d, _c_d, _c_d,
                                                      _c_d, _c_p, _c_p, _c_i32, _c_p, _c_p, _c_i64, _c_p, _c_p,
                                                      _c_sz, _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_solve_batched_mixed_grad_workspace": (_c_sz, [_c_i64, _c_i32, _c_i32, _c_p, _c_p, _c_i64]),
    # batch, px, py, nlayers, kind, map, eps, depth, pmap, pdepth, nmaps, conv, ic, hx, hy, gx, gy, epsi (2),
    # epse (2), kp, k0, npol, te, tm, refine, dR, dT, R, T, R_orders, T_orders, dconv, status, ws, ws_bytes, stream
    "khp_solve_batched_mixed_grad": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p,
                                                    _c_p, _c_i64, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_d, _c_d,
                                                    _c_d, _c_d, _c_p, _c_p, _c_i32, _c_p, _c_p, _c_i32, _c_p, _c_p,
                                                    _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_convmat_islands_workspace": (_c_sz, [_c_i64, _c_i32, _c_i32]),
    "khp_convmat_islands": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_p, _c_p, _c_d, _c_d, _c_d, _c_d, _c_d,
                                           _c_p, _c_p, _c_sz, _c_p]),
    "khp_convmat_bwd_workspace": (_c_sz, [_c_i64, _c_i64, _c_i32, _c_i32]),
    "khp_convmat_bwd": (ctypes.c_int, [_c_i64, _c_i64, _c_i64, _c_p, _c_i32, _c_i32, _c_p, _c_p, _c_sz, _c_p]),
    "khp_twisted_rt_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_twisted_rt": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_i32, _c_p, _c_p, _c_d, _c_d,
                                      _c_d, _c_d, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_launch_count": (ctypes.c_longlong, []),
    "khp_tune": (ctypes.c_int, [_c_i32, _c_i32, _c_i32]),
    "khp_probe_fp64_tflops": (ctypes.c_double, [_c_p, _c_i64, _c_p]),
    "khp_probe_fp32_tflops": (ctypes.c_double, [_c_p, _c_i64, _c_p]),
    "khp_stage_timing": (ctypes.c_int, [_c_i32]),
    "khp_stage_timing_read": (ctypes.c_int, [_c_i32, _c_p, _c_p]),
    "khp_scattering_eig_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_scattering_eig": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_i64, _c_p, _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_bzi_amplitudes_workspace": (_c_sz, [_c_i32, _c_i32, _c_i32]),
    "khp_bzi_amplitudes": (ctypes.c_int, [_c_i32, _c_i32, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_i32, _c_p, _c_p, _c_p,
                                          _c_p, _c_sz, _c_p]),
    "khp_tmat_layer_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_tmat_layer_smatrix": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p,
                                              _c_p, _c_p, _c_p, _c_d, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                              _c_sz, _c_p]),
    "khp_tmat_multS_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_tmat_matrix_s": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_tmat_multS": (ctypes.c_int, [_c_i64, _c_i32, _c_p, _c_i64, _c_p, _c_i64, _c_p, _c_p, _c_p, _c_sz, _c_p]),
    "khp_inverse_workspace": (_c_sz, [_c_i64, _c_i32]),
    "khp_inverse": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_p, _c_i64, _c_p, _c_i64, _c_p, _c_p, _c_sz, _c_p]),
    "khp_cgemm_tf32x3_workspace": (_c_sz, [_c_i64, _c_i32, _c_i32, _c_i32]),
    "khp_cgemm_tf32x3": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_p, _c_i64, _c_i64, _c_p, _c_i64, _c_i64,
                                        _c_p, _c_i64, _c_i64, _c_p, _c_sz, _c_p]),
    "khp_zgemm_fp64_tc_workspace": (_c_sz, [_c_i64, _c_i32, _c_i32, _c_i32]),
    "khp_zgemm_fp64_tc": (ctypes.c_int, [_c_i64, _c_i32, _c_i32, _c_i32, _c_p, _c_i64, _c_i64, _c_p, _c_i64, _c_i64,
                                         _c_p, _c_i64, _c_i64, _c_p, _c_sz, _c_p]),
}

_lib = None


class KhpError(RuntimeError):
    """A libkhp call or a per-problem status reported a failure."""


def load():
    """Load libkhp.so (built by khepri_gb300.build) and declare its C signatures."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libkhp is not built ({LIB_PATH} missing): run khepri_gb300.build.build()")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def exported_symbols():
    """Names of the C entry points this binding declares."""
    return sorted(_SIGNATURES)


def status_string(code: int) -> str:
    """Static description of a return code (khp_status_string)."""
    return load().khp_status_string(int(code)).decode()


def check(code: int, what: str):
    """Raise KhpError for a non-zero return code of a libkhp call."""
    if code != 0:
        raise KhpError(f"{what} failed: {status_string(code)} (code {code})")


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    """The CUDA stream handle for a libkhp call (torch's current stream by default)."""
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def require_cuda():
    """Raise KhpError when no CUDA device is present: the path has no CPU fallback."""
    if not torch.cuda.is_available():
        raise KhpError("libkhp needs a CUDA device; none is available (there is no CPU fallback)")
    load()


STATUS_BITS = {1: "singular pivot", 2: "eigensolver not converged", 4: "non-finite value",
               8: "mixed-precision refinement not converged", 16: "per-problem input out of range",
               32: "mixed-precision eigen-refinement not converged"}


def decode_status(word: int) -> str:
    """The per-problem status bits of a status word, in words."""
    return ", ".join(v for k, v in STATUS_BITS.items() if word & k) or "ok"


STAGES = {"modes": 0, "eigensolve": 1, "tc_product": 2, "recursion": 3, "refine": 4}


def stage_times():
    """{stage name: (total ms, intervals)} recorded since the last khp_stage_timing call."""
    lib = load()
    out = {}
    for name, sid in STAGES.items():
        ms = ctypes.c_double(0.0)
        marks = ctypes.c_int64(0)
        check(lib.khp_stage_timing_read(sid, ctypes.byref(ms), ctypes.byref(marks)), "khp_stage_timing_read")
        out[name] = (ms.value, marks.value)
    return out
