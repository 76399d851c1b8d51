"""Brillouin-zone-integrated beams on the GPU (khepri/beams.py:164-207).

``amplitudes_from_fields`` decomposes a beam sampled over a supercell of bzs[0] x bzs[1] unit
cells into plane-wave amplitudes of the expansion's harmonics (khp_bzi_amplitudes: one launch
for the phase division and the sample gather, one CTA per harmonic for the DFT sums);
``gen_bzi_grid`` is the cell-centred Bloch grid of the integration (host arithmetic).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi, engine


def gen_bzi_grid(shape, a=1, reciproc=None):
    """beams.py:193-207: [2, shape[0], shape[1]] cell-centred Bloch vectors of the first zone."""
    if reciproc is None:
        b1 = [2 * np.pi / a, 0]
        b2 = [0, 2 * np.pi / a]
    else:
        b1, b2 = reciproc
    si, sj = 1 / shape[0], 1 / shape[1]
    i, j = np.meshgrid(np.arange(-0.5 + si / 2, 0.5, si), np.arange(-0.5 + sj / 2, 0.5, sj), indexing="ij")
    return np.stack([b1[0] * i + b2[0] * j, b1[1] * i + b2[1] * j])


def _g_vectors(e):
    if hasattr(e, "g_vectors"):
        return np.asarray(e.g_vectors, dtype=float)
    return np.asarray(e, dtype=float)


def amplitudes_from_fields(fields, e, wl, kp, x, y, bzs, a=1, device="cuda"):
    """beams.py:164-190.  fields: complex [X, Y, 2, 3] (E, H; x, y, z) sampled at x, y [X, Y],
    X = bzs[1] * ns, Y = bzs[0] * ns; e: an Expansion (or its g vectors [2, ng]); kp: the
    incident planar wavevector.  Returns complex [4, ng]: the amplitudes of (Ex, Ey, Hx, Hy).
    ``wl`` and ``a`` are unused, as in the reference."""
    _capi.require_cuda()
    lib = _capi.load()
    dev = torch.device(device)
    fields = np.asarray(fields)
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    X, Y = x.shape
    if fields.shape != (X, Y, 2, 3) or y.shape != (X, Y):
        raise ValueError("fields must be [X, Y, 2, 3] and x, y [X, Y]")
    b0, b1 = int(bzs[0]), int(bzs[1])
    if X % b1 or Y % b0 or X // b1 != Y // b0:
        raise ValueError("the sample grid must hold bzs[1] x bzs[0] square cells")
    ns = X // b1
    g = _g_vectors(e)
    ng = g.shape[1]
    ft = torch.as_tensor(np.ascontiguousarray(fields), dtype=torch.complex128).to(dev)
    xt = torch.as_tensor(np.ascontiguousarray(x)).to(dev)
    yt = torch.as_tensor(np.ascontiguousarray(y)).to(dev)
    kpt = torch.as_tensor(np.asarray(kp, dtype=complex).reshape(2)).to(dev)
    gxt = torch.as_tensor(np.ascontiguousarray(g[0])).to(dev)
    gyt = torch.as_tensor(np.ascontiguousarray(g[1])).to(dev)
    out = torch.empty((4, ng), dtype=torch.complex128, device=dev)
    ws = engine.workspace(lib.khp_bzi_amplitudes_workspace(b0, b1, ns), dev)
    with engine._stage("khp_bzi_amplitudes"):
        code = lib.khp_bzi_amplitudes(b0, b1, ns, _capi.ptr(ft), _capi.ptr(xt), _capi.ptr(yt), _capi.ptr(kpt), ng,
                                      _capi.ptr(gxt), _capi.ptr(gyt), _capi.ptr(out), _capi.ptr(ws), ws.numel(),
                                      _capi.stream_ptr())
    _capi.check(code, "khp_bzi_amplitudes")
    return out.cpu().numpy()
