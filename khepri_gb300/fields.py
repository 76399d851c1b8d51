"""Field reconstruction of the Crystal path (fields_coords_xy / fields_volume) on the GPU.

Follows khepri/crystal.py:208-343 (locate_layer, _fourier_fields, fields_coords_xy,
fields_volume), khepri/fields.py:18-76 and khepri/fourier.py:136-142, in three libkhp launches
per call: per-layer mode amplitudes, Fourier fields at every requested depth, inverse DFT.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _capi, engine


def incident_vector(pw, te, tm, k_vector):
    """Source vector [ex, ey] of a plane wave: delta at harmonic (Nh-1)//2 times the normalised
    te*aTE + tm*aTM polarisation (khepri/alternative.py:101-128); host-side set-up data."""
    norm = math.hypot(abs(te), abs(tm))
    te, tm = te / norm, tm / norm
    kvec = np.asarray(k_vector, dtype=complex)
    kp_norm = np.linalg.norm(kvec[:2])
    kbar = kvec / np.linalg.norm(kvec)
    if abs(kp_norm) < 1e-8:
        a_te = np.array([1.0, 0.0, 0.0], dtype=complex)
        a_tm = np.array([0.0, 1.0, 0.0], dtype=complex)
    else:
        a_te = np.array([-kbar[1], kbar[0], 0.0], dtype=complex)
        a_te = a_te / np.linalg.norm(a_te)
        a_tm = np.array([a_te[1] * kbar[2], -a_te[0] * kbar[2], a_te[0] * kbar[1] - a_te[1] * kbar[0]])
        a_tm = a_tm / np.linalg.norm(a_tm)
    nh = pw[0] * pw[1]
    pol = te * a_te + tm * a_tm
    out = np.zeros(2 * nh, dtype=complex)
    out[(nh - 1) // 2] = pol[0]
    out[nh + (nh - 1) // 2] = pol[1]
    return out



def _locate(cl, z):
    """crystal.py:208-232: layer index and depth relative to the layer's start."""
    idx = int(np.searchsorted(cl.stack_positions, z)) - 1
    zr = z if z <= 0 else z - cl.stack_positions[idx]
    return idx, zr


def _i64(ptrs, device):
    return torch.tensor(ptrs, dtype=torch.int64, device=device)


def fourier_fields(cl, zs, incident_fields):
    """Device tensor [Nz, 6, nh] of (sx, sy, sz, ux, uy, uz) at the depths zs."""
    struct, prob = cl._struct, cl._prob
    dev, nh, n = struct.device, struct.nh, struct.n
    k0 = 2 * np.pi / cl.source.wavelength
    slots, slot_of_z, zbar = {}, [], []
    for z in zs:
        idx, zr = _locate(cl, z)
        name = cl.global_stacking[idx]
        layer = cl.layers[name]
        assert layer.fields, f"Layer at {z} did not store eigenspace."
        slot = slots.setdefault(idx, len(slots))
        slot_of_z.append(slot)
        zbar.append(k0 * (layer.depth - zr))
    if cl._rev is None:  # the reverse chain is built on first use (only fields need it)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        cl._rev = engine.reverse_chain(cl._states, cl.global_stacking, cl.stack_retain_mask, status)
        cl.stacking_reverse_matrices = [None if s is None else s[0] for s in cl._rev]
    order = sorted(slots, key=slots.get)
    names = [cl.global_stacking[i] for i in order]
    st = [cl._states[nm] for nm in names]
    sl = [cl._fwd[i][0] for i in order]
    sr = [cl._rev[i][0] for i in order]
    lib = _capi.load()
    sp = _capi.stream_ptr()
    kp = torch.view_as_real(prob.kp[0]).contiguous()
    k0t = prob.k0[:1].contiguous()
    inc = torch.tensor(np.asarray(incident_fields, dtype=complex).ravel(), dtype=torch.complex128, device=dev)
    L = len(order)
    amps = torch.empty((L, 2 * n), dtype=torch.complex128, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = engine.workspace(lib.khp_fields_amplitudes_workspace(L, nh), dev)
    vref = cl._states["Sref"].V[0]
    # Every argument tensor is held in a local until the launches are enqueued: a temporary
    # would return its storage to the caching allocator while its address is still in use.
    sl_p = _i64([s.data_ptr() for s in sl], dev)
    sr_p = _i64([s.data_ptr() for s in sr], dev)
    w_p = _i64([s.W[0].data_ptr() for s in st], dev)
    v_p = _i64([s.V[0].data_ptr() for s in st], dev)
    lam_p = _i64([s.lam[0].data_ptr() for s in st], dev)
    ic_p = _i64([s.IC.data_ptr() if torch.is_tensor(s.IC) else 0 for s in st], dev)
    ic_sc = torch.tensor([0j if torch.is_tensor(s.IC) else complex(s.IC) for s in st], dtype=torch.complex128,
                         device=dev)
    slot_t = torch.tensor(slot_of_z, dtype=torch.int32, device=dev)
    zbar_t = torch.tensor(zbar, dtype=torch.float64, device=dev)
    _capi.check(lib.khp_fields_amplitudes(
        L, nh, _capi.ptr(sl_p), _capi.ptr(sr_p), _capi.ptr(w_p), _capi.ptr(v_p), _capi.ptr(vref), _capi.ptr(inc),
        _capi.ptr(struct.gx), _capi.ptr(struct.gy), _capi.ptr(kp), _capi.ptr(k0t), _capi.ptr(amps),
        _capi.ptr(status), _capi.ptr(ws), ws.numel(), sp), "khp_fields_amplitudes")
    ff = torch.empty((len(zs), 6, nh), dtype=torch.complex128, device=dev)
    _capi.check(lib.khp_fields_fourier(
        len(zs), nh, _capi.ptr(slot_t), _capi.ptr(zbar_t), _capi.ptr(w_p), _capi.ptr(v_p), _capi.ptr(lam_p),
        _capi.ptr(ic_p), _capi.ptr(ic_sc), _capi.ptr(amps), _capi.ptr(struct.gx), _capi.ptr(struct.gy),
        _capi.ptr(kp), _capi.ptr(k0t), _capi.ptr(ff), sp), "khp_fields_fourier")
    word = int(status.item())
    if word:
        raise _capi.KhpError(f"fields: {_capi.decode_status(word)}")
    return ff


def idft(cl, ff, x, y, kp=None):
    """Real-space fields [rows, X, Y] from Fourier rows [rows, nh] (fourier.py:136-142)."""
    struct = cl._struct
    dev = struct.device
    shape = np.shape(x)
    xs = torch.tensor(np.asarray(x, dtype=float).ravel(), dtype=torch.float64, device=dev)
    ys = torch.tensor(np.asarray(y, dtype=float).ravel(), dtype=torch.float64, device=dev)
    kpv = cl.kp if kp is None else kp
    kpt = torch.tensor([complex(kpv[0]), complex(kpv[1])], dtype=torch.complex128, device=dev)
    rows = ff.reshape(-1, struct.nh).contiguous()
    out = torch.empty((rows.shape[0], xs.numel()), dtype=torch.complex128, device=dev)
    kpr = torch.view_as_real(kpt).contiguous()
    lib = _capi.load()
    _capi.check(lib.khp_fields_idft(rows.shape[0], struct.nh, _capi.ptr(rows), _capi.ptr(struct.gx),
                                    _capi.ptr(struct.gy), _capi.ptr(kpr), xs.numel(), _capi.ptr(xs), _capi.ptr(ys),
                                    _capi.ptr(out), _capi.stream_ptr()), "khp_fields_idft")
    return out.reshape(rows.shape[0], *shape)


def _incident(cl, incident_fields):
    if incident_fields is None:
        return np.hstack(cl.get_source_as_field_vectors())
    if isinstance(incident_fields, tuple) and len(incident_fields) == 2:
        return np.hstack(incident_fields)
    return np.asarray(incident_fields)


def fields_coords_xy(cl, x, y, z, incident_fields=None, kp=None, return_fourier=False):
    """crystal.py:297-333: [E, H] with E, H of shape [3, X, Y] at depth z."""
    x = np.asarray(x)
    y = np.asarray(y)
    assert x.shape == y.shape and (len(x.shape) == 2), "x and y must be 2D meshgrids"
    assert cl.solved, "Call solve first."
    ff = fourier_fields(cl, [z], _incident(cl, incident_fields))
    if return_fourier:
        return tuple(ff[0, i].cpu().numpy() for i in range(6))
    f = idft(cl, ff, x, y, kp).cpu().numpy()
    return np.split(f, 2, axis=0)


def fields_volume(cl, x, y, z, incident_fields=None):
    """crystal.py:335-343: (E, H), each [Nz, 3, X, Y]; every depth in one launch."""
    x = np.asarray(x)
    y = np.asarray(y)
    assert x.shape == y.shape and (len(x.shape) == 2), "x and y must be 2D meshgrids"
    assert cl.solved, "Call solve first."
    zs = [float(v) for v in np.asarray(list(z), dtype=float)]
    ff = fourier_fields(cl, zs, _incident(cl, incident_fields))
    f = idft(cl, ff, x, y).cpu().numpy().reshape(len(zs), 6, *x.shape)
    return f[:, :3], f[:, 3:]
