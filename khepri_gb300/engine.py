"""Device-side RCWA solve over a batch of problems that share one layer structure.

A *problem* is (wavelength, in-plane wavevector kp, polarisation).  Everything here drives
libkhp through its C ABI on torch CUDA tensors; torch supplies device memory and streams.

Work is split the GB300 way:
* per structure (once): G vectors, and for each distinct pixmap its convolution matrix C,
  C^-1 and the products C^-1 diag(g) C (khp_convmat, khp_structure_prep);
* per problem batch: patterned-layer modes (one eigensolve per distinct pixmap, shared by
  every layer that uses the map), layer S-matrices, closed-form homogeneous media, the
  star-product chain and the fluxes.

Reference layout of the same steps: khepri/crystal.py:180-206 (solve), layer.py:35-60
(stack_layers), layer.py:145-194 (Layer.solve).
"""
from __future__ import annotations

import cmath
import hashlib
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _capi

TWOPI = 2.0 * math.pi
C128 = torch.complex128
F64 = torch.float64


# ------------------------------------------------------------------------------------------
# Basis (khepri/expansion.py, khepri/tools.py:64-69)
# ------------------------------------------------------------------------------------------
def lattice_vectors(lattice="square", pitch=1.0):
    """Rows are lattice vectors; khepri/crystal.py:60-74."""
    if isinstance(lattice, str):
        if lattice == "square":
            return pitch * np.asarray([[1.0, 0.0], [0.0, 1.0]])
        if lattice == "hexagonal":
            return pitch * np.asarray([[math.sqrt(3) / 2, 0.5], [math.sqrt(3) / 2, -0.5]])
        raise NotImplementedError(f"This {lattice} magic-string is not emplemented.")
    return np.asarray(lattice, dtype=float)


def reciprocal_basis(lat):
    """Reciprocal lattice vectors (tools.py:64-69, reciproc)."""
    a1, a2 = lat[0], lat[1]
    s = TWOPI / (a1[0] * a2[1] - a1[1] * a2[0])
    return np.array([[a2[1] * s, -a2[0] * s], [-a1[1] * s, a1[0] * s]])


def expansion_indices(pw):
    """Harmonic index set, m fastest (expansion.py:4-16); odd counts only, as the reference asserts."""
    px, py = pw
    if px % 2 != 1 or py % 2 != 1:
        raise AssertionError("harmonic counts must be odd")
    m = np.arange(-(px - 1) // 2, (px - 1) // 2 + 1)
    n = np.arange(-(py - 1) // 2, (py - 1) // 2 + 1)
    mm, nn = np.meshgrid(m, n)
    return np.vstack([mm.ravel(), nn.ravel()])


def g_vectors(pw, lat):
    """G vectors of the expansion, [2][Nh] (expansion.py:76-84)."""
    rec = reciprocal_basis(lat)
    idx = expansion_indices(pw)
    return rec[0][:, None] * idx[0][None, :] + rec[1][:, None] * idx[1][None, :]


def compute_kplanar(eps_inc, wavelength, theta_deg=0.0, phi_deg=0.0):
    """khepri/tools.py:17-21 (complex result)."""
    phi, theta = math.radians(phi_deg), math.radians(theta_deg)
    s = cmath.sqrt(eps_inc) * TWOPI / wavelength * math.sin(theta)
    return (complex(math.cos(phi)) * s, complex(math.sin(phi)) * s)


# ------------------------------------------------------------------------------------------
# Optional per-entry-point timing with CUDA events on the launching stream (used by bench.py)
# ------------------------------------------------------------------------------------------
class StageTimer:
    """Collects (start, end) CUDA events around each libkhp entry point while active."""

    def __init__(self):
        self.events = {}

    def __enter__(self):
        global _TIMER
        _TIMER = self
        return self

    def __exit__(self, *exc):
        global _TIMER
        _TIMER = None

    def record(self, name):
        """A CUDA event recorded now on the current stream."""
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    def add(self, name, e0, e1):
        """An interval of stage ``name`` between two recorded events."""
        self.events.setdefault(name, []).append((e0, e1))

    def totals_ms(self):
        """{stage: (total ms, intervals)} (synchronises)."""
        torch.cuda.synchronize()
        return {k: (sum(a.elapsed_time(b) for a, b in v), len(v)) for k, v in self.events.items()}


_TIMER = None


class _stage:
    def __init__(self, name):
        self.name = name

    def __enter__(self):
        self.e0 = _TIMER.record(self.name) if _TIMER is not None else None
        return self

    def __exit__(self, *exc):
        if self.e0 is not None and _TIMER is not None:
            _TIMER.add(self.name, self.e0, _TIMER.record(self.name))


# ------------------------------------------------------------------------------------------
# Workspace: one growing device byte buffer per device (caller-owned scratch for libkhp)
# ------------------------------------------------------------------------------------------
_WS = {}


def workspace(nbytes, device, slot=0):
    """A reusable device byte buffer of at least ``nbytes`` per device, slot and current stream
    (grown, never shrunk).  Calls whose workspaces must coexist use different slots: a
    mixed-precision solve keeps its refined modes in its workspace until its flagged problems are
    re-solved, and a pipelined caller alternates two slots between consecutive chunks.  Work
    enqueued on different streams gets different buffers, so concurrent streams never share
    scratch (work on one stream runs in order, so its calls may share a buffer)."""
    dev = torch.device(device)
    stream = torch.cuda.current_stream(dev).cuda_stream if dev.type == "cuda" else 0
    key = (str(device), int(slot), stream)
    buf = _WS.get(key)
    if buf is None or buf.numel() < nbytes:
        _WS[key] = buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
    return buf


class AnalyticalMap:
    """Permittivity of an analytical layer (Layer.analytical, khepri/layer.py:121-129): islands
    as Drawing.islands() describes them (dicts with "type" "disc" | "rectangle", "params",
    "epsilon") in a host medium.  Used in place of a pixmap; its convolution matrix comes from
    the closed-form island transforms (khp_convmat_islands)."""

    _TYPES = {"disc": 0, "rectangle": 1}

    def __init__(self, islands, eps_host):
        self.islands = [dict(type=i["type"], params=list(i["params"]), epsilon=i["epsilon"]) for i in islands]
        self.eps_host = complex(eps_host)
        for i in self.islands:
            if i["type"] not in self._TYPES:
                raise NotImplementedError(f"island type {i['type']!r}")
        self.key = "islands:" + repr((self.islands, self.eps_host))

    def rows(self, map_index=0):
        """[n][8] rows of khp_convmat_islands."""
        out = []
        for i in self.islands:
            p = list(i["params"]) + [0.0] * (4 - len(i["params"]))
            e = complex(i["epsilon"])
            out.append([map_index, self._TYPES[i["type"]], e.real, e.imag] + p)
        return np.asarray(out, dtype=np.float64).reshape(-1, 8)


def _digest(a):
    if isinstance(a, AnalyticalMap):
        return a.key
    a = np.ascontiguousarray(a)
    return hashlib.blake2b(a.tobytes(), digest_size=16).hexdigest() + str(a.shape) + str(a.dtype)


# ------------------------------------------------------------------------------------------
# Layer descriptors
# ------------------------------------------------------------------------------------------
@dataclass
class LayerSpec:
    """One layer of a stack: kind, permittivity (map or scalar) and depth."""
    kind: str  # "pixmap" | "uniform" | "inc" | "trn"
    eps: object  # 2-D array for pixmaps, complex scalar otherwise
    depth: float


class StructureGPU:
    """Per-structure device state: G vectors and, per distinct pixmap, C, C^-1, Hx, Hy."""

    def __init__(self, pw, lattice, device="cuda"):
        _capi.require_cuda()
        self.pw = (int(pw[0]), int(pw[1]))
        self.nh = self.pw[0] * self.pw[1]
        self.n = 2 * self.nh
        self.device = torch.device(device)
        self.lattice = np.asarray(lattice, dtype=float)
        g = g_vectors(self.pw, lattice)
        self.gx = torch.tensor(g[0], dtype=F64, device=self.device)
        self.gy = torch.tensor(g[1], dtype=F64, device=self.device)
        self._maps = {}  # digest -> dict(conv, ic, hx, hy)

    def prepare_map(self, eps_map):
        """Device C, C^-1, Hx, Hy of a pixmap (cached by content)."""
        key = _digest(eps_map)
        hit = self._maps.get(key)
        if hit is not None:
            return hit
        px, py = self.pw
        nh = self.nh
        conv = torch.empty((1, nh, nh), dtype=C128, device=self.device)
        lib = _capi.load()
        sp = _capi.stream_ptr()
        if isinstance(eps_map, AnalyticalMap):
            rows = torch.tensor(eps_map.rows(), dtype=F64, device=self.device)
            host = torch.tensor([eps_map.eps_host], dtype=C128, device=self.device)
            b = reciprocal_basis(self.lattice)
            area = abs(self.lattice[0, 0] * self.lattice[1, 1] - self.lattice[0, 1] * self.lattice[1, 0])
            ws = workspace(lib.khp_convmat_islands_workspace(1, px, py), self.device)
            _capi.check(lib.khp_convmat_islands(1, px, py, rows.shape[0], _capi.ptr(rows), _capi.ptr(host),
                                                float(b[0, 0]), float(b[0, 1]), float(b[1, 0]), float(b[1, 1]), area,
                                                _capi.ptr(conv), _capi.ptr(ws), ws.numel(), sp), "khp_convmat_islands")
        else:
            eps = torch.as_tensor(np.asarray(eps_map), device=self.device).to(C128).contiguous()
            nx, ny = eps.shape
            ws = workspace(lib.khp_convmat_workspace(1, px, py), self.device)
            _capi.check(lib.khp_convmat(1, nx, ny, _capi.ptr(eps), px, py, _capi.ptr(conv), _capi.ptr(ws), ws.numel(),
                                        sp), "khp_convmat")
        ic = torch.empty_like(conv)
        hx = torch.empty_like(conv)
        hy = torch.empty_like(conv)
        st = torch.zeros(1, dtype=torch.int32, device=self.device)
        ws = workspace(lib.khp_structure_prep_workspace(1, nh), self.device)
        _capi.check(lib.khp_structure_prep(1, nh, _capi.ptr(conv), _capi.ptr(self.gx), _capi.ptr(self.gy),
                                           _capi.ptr(ic), _capi.ptr(hx), _capi.ptr(hy), _capi.ptr(st), _capi.ptr(ws),
                                           ws.numel(), sp), "khp_structure_prep")
        code = int(st.item())
        if code:
            raise _capi.KhpError(f"convolution matrix of a pixmap: {_capi.decode_status(code)}")
        entry = dict(conv=conv, ic=ic, hx=hx, hy=hy, key=key)
        self._maps[key] = entry
        return entry


# Pinned host copies of inputs whose host-to-device copies are still queued, with the event that
# follows them on the stream.  A pinned buffer must outlive its copy (released early, the next
# staging could take the same buffer and overwrite the bytes before the device reads them), so
# each is held here until its event has completed.
_STAGED = []


def _to_device_async(arrays, device):
    """Copies of host numpy arrays on ``device``, staged through pinned memory and queued on the
    current stream without a host wait; the staging buffers are kept until their copies ran."""
    pinned = [torch.from_numpy(a).pin_memory() for a in arrays]
    out = [h.to(device, non_blocking=True) for h in pinned]
    ev = torch.cuda.Event()
    ev.record()
    _STAGED[:] = [(h, e) for h, e in _STAGED if not e.query()]
    _STAGED.append((pinned, ev))
    return out


@dataclass
class Problems:
    """Device arrays describing a batch of problems."""

    k0: torch.Tensor  # [B] float64
    kp: torch.Tensor  # [B, 2] complex128 (absolute units)
    te: torch.Tensor  # [B] complex128
    tm: torch.Tensor  # [B] complex128

    @property
    def batch(self):
        """Number of problems."""
        return int(self.k0.shape[0])

    def subset(self, idx: torch.Tensor) -> "Problems":
        """The problems at device indices ``idx``."""
        return Problems(k0=self.k0[idx].contiguous(), kp=self.kp[idx].contiguous(), te=self.te[idx].contiguous(),
                        tm=self.tm[idx].contiguous())

    @classmethod
    def make(cls, wavelengths, kp, te, tm, device):
        """Problems from host wavelengths, in-plane k (crystal.py:345-360 conventions) and sources."""
        wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
        B = wl.shape[0]
        kpa = np.asarray(kp, dtype=complex).reshape(B, 2)
        te = np.broadcast_to(np.asarray(te, dtype=complex), (B,))
        tm = np.broadcast_to(np.asarray(tm, dtype=complex), (B,))
        d = torch.device(device)
        # row-major copies: an input built by broadcasting can be column-major (kp of the twisted
        # path), and the kernels read kp as [B][2]
        host = [np.array(TWOPI / wl, dtype=np.float64, order="C"), np.array(kpa, dtype=np.complex128, order="C"),
                np.array(te, dtype=np.complex128, order="C"), np.array(tm, dtype=np.complex128, order="C")]
        if d.type != "cuda":
            return cls(*(torch.from_numpy(h).to(d) for h in host))
        return cls(*_to_device_async(host, d))


@dataclass
class LayerState:
    """A solved layer: its S-matrix and, for field reconstruction, its modes."""
    S: torch.Tensor  # [B, 2, 2, n, n]
    W: torch.Tensor | None = None
    V: torch.Tensor | None = None
    lam: torch.Tensor | None = None
    IC: object = None  # [nh, nh] tensor for pixmaps, complex scalar 1/eps otherwise


def _kp_real_view(kp):
    return torch.view_as_real(kp).contiguous()


def layer_modes(struct: StructureGPU, entry, prob: Problems, status):
    """W, V, lam of a patterned layer for every problem (khp_layer_modes)."""
    B, nh, n = prob.batch, struct.nh, struct.n
    dev = struct.device
    W = torch.empty((B, n, n), dtype=C128, device=dev)
    V = torch.empty_like(W)
    lam = torch.empty((B, n), dtype=C128, device=dev)
    mi = torch.zeros(B, dtype=torch.int32, device=dev)
    lib = _capi.load()
    ws = workspace(lib.khp_layer_modes_workspace(B, nh), dev)
    with _stage("khp_layer_modes"):
        code = lib.khp_layer_modes(B, nh, _capi.ptr(mi), _capi.ptr(entry["conv"]), _capi.ptr(entry["hx"]),
                                    _capi.ptr(entry["hy"]), _capi.ptr(struct.gx), _capi.ptr(struct.gy),
                                    _capi.ptr(prob.kp), _capi.ptr(prob.k0), _capi.ptr(W), _capi.ptr(V),
                                    _capi.ptr(lam), _capi.ptr(status), _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
    _capi.check(code, "khp_layer_modes")
    return W, V, lam


def layer_smatrix(struct: StructureGPU, W, V, lam, depth, prob: Problems, status):
    """S-matrix of a patterned layer from its modes (alternative.py:181-195, build_scatmat)."""
    B, nh, n = prob.batch, struct.nh, struct.n
    dev = struct.device
    S = torch.empty((B, 2, 2, n, n), dtype=C128, device=dev)
    d = torch.full((B,), float(depth), dtype=F64, device=dev)
    lib = _capi.load()
    ws = workspace(lib.khp_layer_smatrix_workspace(B, nh), dev)
    with _stage("khp_layer_smatrix"):
        code = lib.khp_layer_smatrix(B, nh, _capi.ptr(W), _capi.ptr(V), _capi.ptr(lam), _capi.ptr(d),
                                      _capi.ptr(struct.gx), _capi.ptr(struct.gy), _capi.ptr(prob.kp),
                                      _capi.ptr(prob.k0), _capi.ptr(S), _capi.ptr(status), _capi.ptr(ws), ws.numel(),
                                      _capi.stream_ptr())
    _capi.check(code, "khp_layer_smatrix")
    return S


_KIND = {"uniform": 0, "inc": 1, "trn": 2}


def closed_form(struct: StructureGPU, kind, eps, depth, prob: Problems, status, want_modes=False):
    """S-matrix of a uniform layer or a half-space in closed form (alternative.py:32-82, 130-156)."""
    B, nh, n = prob.batch, struct.nh, struct.n
    dev = struct.device
    S = torch.empty((B, 2, 2, n, n), dtype=C128, device=dev)
    e = torch.full((B,), complex(eps), dtype=C128, device=dev)
    d = torch.full((B,), float(depth), dtype=F64, device=dev)
    W = V = lam = None
    if want_modes:
        W = torch.empty((B, n, n), dtype=C128, device=dev)
        V = torch.empty_like(W)
        lam = torch.empty((B, n), dtype=C128, device=dev)
    lib = _capi.load()
    with _stage("khp_closed_form_smatrix"):
        code = lib.khp_closed_form_smatrix(B, nh, _KIND[kind], _capi.ptr(e), _capi.ptr(d), _capi.ptr(struct.gx),
                                            _capi.ptr(struct.gy), _capi.ptr(prob.kp), _capi.ptr(prob.k0), _capi.ptr(S),
                                            _capi.ptr(W), _capi.ptr(V), _capi.ptr(lam), _capi.ptr(status),
                                            _capi.stream_ptr())
    _capi.check(code, "khp_closed_form_smatrix")
    return S, W, V, lam


def star(SA, SB, status, out=None):
    """Redheffer star product SA * SB over the batch (khp_star_product)."""
    B, n = SA.shape[0], SA.shape[-1]
    if out is None:
        out = torch.empty_like(SA)
    lib = _capi.load()
    ws = workspace(lib.khp_star_product_workspace(B, n), SA.device)
    nn4 = 4 * n * n
    with _stage("khp_star_product"):
        code = lib.khp_star_product(B, n, _capi.ptr(SA), nn4, _capi.ptr(SB), nn4, _capi.ptr(out), _capi.ptr(status),
                                     _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
    _capi.check(code, "khp_star_product")
    return out


def identity_smatrix(B, n, device):
    """[[0, I], [I, 0]] (khepri/alternative.py:220-232)."""
    S = torch.zeros((B, 2, 2, n, n), dtype=C128, device=device)
    eye = torch.eye(n, dtype=C128, device=device)
    S[:, 0, 1] = eye
    S[:, 1, 0] = eye
    return S


def flux(struct: StructureGPU, Stot, prob: Problems, epsi, epse, orders=False):
    """R, T (and per-order powers) from the global S (crystal.py:363-396; alternative.py:235-245)."""
    B, nh, n = prob.batch, struct.nh, struct.n
    dev = struct.device
    R = torch.empty(B, dtype=F64, device=dev)
    T = torch.empty(B, dtype=F64, device=dev)
    ro = to = None
    if orders:
        ro = torch.empty((B, nh), dtype=F64, device=dev)
        to = torch.empty((B, nh), dtype=F64, device=dev)
    epsi, epse = complex(epsi), complex(epse)
    lib = _capi.load()
    with _stage("khp_flux"):
        code = lib.khp_flux(B, struct.pw[0], struct.pw[1], _capi.ptr(Stot), 4 * n * n, _capi.ptr(struct.gx),
                             _capi.ptr(struct.gy), _capi.ptr(prob.kp), _capi.ptr(prob.k0), _capi.ptr(prob.te),
                             _capi.ptr(prob.tm), epsi.real, epsi.imag, epse.real, epse.imag, _capi.ptr(R), _capi.ptr(T),
                             _capi.ptr(ro), _capi.ptr(to), _capi.stream_ptr())
    _capi.check(code, "khp_flux")
    return R, T, ro, to


def solve_layers(struct: StructureGPU, specs: dict, stack: list, prob: Problems, status, keep_modes=()):
    """S-matrix (and, for names in keep_modes, W, V, lam, IC) of every distinct layer in stack."""
    states = {}
    modes = {}
    for name in dict.fromkeys(stack):
        sp = specs[name]
        want = name in keep_modes
        if sp.kind == "pixmap":
            entry = struct.prepare_map(sp.eps)
            key = entry["key"]
            if key not in modes:
                modes[key] = layer_modes(struct, entry, prob, status)
            W, V, lam = modes[key]
            S = layer_smatrix(struct, W, V, lam, sp.depth, prob, status)
            states[name] = LayerState(S, W if want else None, V if want else None, lam if want else None,
                                      entry["ic"][0] if want else None)
        else:
            S, W, V, lam = closed_form(struct, sp.kind, sp.eps, sp.depth, prob, status, want)
            states[name] = LayerState(S, W, V, lam, 1.0 / complex(sp.eps) if want else None)
    return states


def chain(states, stack, mask, status, reverse=False):
    """Forward chain S_0 * S_1 * ... (copies where mask) and, optionally, the reverse chain
    (khepri/layer.py:35-60).  The first product with the identity is exact and skipped."""
    Stot = states[stack[0]].S
    fwd = [Stot if mask[0] else None]
    for i, name in enumerate(stack[1:], start=1):
        Stot = star(Stot, states[name].S, status)
        fwd.append(Stot if mask[i] else None)
    rev = reverse_chain(states, stack, mask, status) if reverse else None
    return fwd, rev, Stot


def reverse_chain(states, stack, mask, status):
    """Reverse chain of khepri/layer.py:49-59: entry i is the product of the layers right of i."""
    S0 = states[stack[0]].S
    B, n = S0.shape[0], S0.shape[-1]
    srev = identity_smatrix(B, n, S0.device)
    rmask = list(reversed(mask[1:]))
    rev = []
    for i, name in enumerate(reversed(stack[1:])):
        rev.append(srev if rmask[i] else None)
        srev = star(states[name].S, srev, status)
    rev.append(srev)
    return list(reversed(rev))
