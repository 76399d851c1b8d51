"""Batched RCWA solves: many (wavelength, k-point, polarisation) problems of one structure per launch.

``solve_rt`` is the batched counterpart of the reference's one-problem-per-call loop
(README.md:52-58: set_source -> solve -> poynting_flux_end).  Problems are processed in chunks;
inside a chunk every kernel launch covers all problems.  The star-product chain is streamed
left to right (only the running S-matrix and one layer S-matrix are live), and patterned layers
that share a pixmap share one eigensolve per problem.
"""
from __future__ import annotations

import contextlib
import ctypes
import functools

import numpy as np
import torch

from . import _capi, autotune, engine
from .engine import LayerSpec


def _spec(kind, eps, depth):
    """("pixmap", map, d) | ("uniform", eps, d) | ("analytical", (islands, eps_host) or AnalyticalMap, d)."""
    if kind == "analytical":
        amap = eps if isinstance(eps, engine.AnalyticalMap) else engine.AnalyticalMap(*eps)
        return LayerSpec("pixmap", amap, depth)
    return LayerSpec(kind, eps, depth)


def _specs(layers, epsi, epse):
    specs = {name: _spec(kind, eps, depth) for name, (kind, eps, depth) in layers.items()}
    specs["__inc__"] = LayerSpec("inc", epsi, 0.0)
    specs["__trn__"] = LayerSpec("trn", epse, 0.0)
    return specs


def global_smatrix(struct, specs, stack, prob, status):
    """Global S-matrix of every problem of the chunk, streamed left to right."""
    modes = {}
    Stot, _, _, _ = engine.closed_form(struct, "inc", specs["__inc__"].eps, 0.0, prob, status)
    for name in list(stack) + ["__trn__"]:
        sp = specs[name]
        if sp.kind == "pixmap":
            entry = struct.prepare_map(sp.eps)
            if entry["key"] not in modes:
                modes[entry["key"]] = engine.layer_modes(struct, entry, prob, status)
            W, V, lam = modes[entry["key"]]
            S = engine.layer_smatrix(struct, W, V, lam, sp.depth, prob, status)
        else:
            S, _, _, _ = engine.closed_form(struct, sp.kind, sp.eps, sp.depth, prob, status)
        Stot = engine.star(Stot, S, status)
        del S
    return Stot


def solve_chunk(struct, specs, stack, prob, status, orders=False, epsi=1.0, epse=1.0):
    """R, T (and per-order powers) of one chunk of problems on the device."""
    Stot = global_smatrix(struct, specs, stack, prob, status)
    return engine.flux(struct, Stot, prob, epsi, epse, orders=orders)


def solve_chunk_both_pols(struct, specs, stack, prob, status, epsi=1.0, epse=1.0):
    """R, T for (te, tm) = (1, 0) and (0, 1) from one S-matrix per problem: each [B, 2]."""
    Stot = global_smatrix(struct, specs, stack, prob, status)
    one, zero = torch.ones_like(prob.te), torch.zeros_like(prob.te)
    out = []
    for te, tm in ((one, zero), (zero, one)):
        p = engine.Problems(prob.k0, prob.kp, te, tm)
        r, t, _, _ = engine.flux(struct, Stot, p, epsi, epse)
        out.append((r, t))
    return torch.stack([out[0][0], out[1][0]], 1), torch.stack([out[0][1], out[1][1]], 1)


class StackPlan:
    """Host description of a layer stack for khp_solve_batched, with the stacked per-pixmap
    device matrices (C, Hx, Hy) it reads."""

    def __init__(self, struct, specs, stack):
        kinds, maps, eps, depth = [], [], [], []
        keys, entries = [], []
        for name in stack:
            sp = specs[name]
            if sp.kind == "pixmap":
                e = struct.prepare_map(sp.eps)
                if e["key"] not in keys:
                    keys.append(e["key"])
                    entries.append(e)
                kinds.append(1)
                maps.append(keys.index(e["key"]))
                eps.append(0j)
            else:
                kinds.append(0)
                maps.append(0)
                eps.append(complex(sp.eps))
            depth.append(float(sp.depth))
        self.kinds = np.asarray(kinds, dtype=np.int32)
        self.maps = np.asarray(maps, dtype=np.int32)
        self.eps = np.asarray(eps, dtype=np.complex128)
        self.depth = np.asarray(depth, dtype=np.float64)
        self.nmaps = len(entries)
        if entries:
            self.conv = torch.cat([e["conv"] for e in entries]).contiguous()
            self.ic = torch.cat([e["ic"] for e in entries]).contiguous()
            self.hx = torch.cat([e["hx"] for e in entries]).contiguous()
            self.hy = torch.cat([e["hy"] for e in entries]).contiguous()
        else:
            self.conv = self.ic = self.hx = self.hy = None


def _host(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def solve_chunk_gamma(struct, plan, prob, status, epsi=1.0, epse=1.0, te=None, tm=None, precision="fp64",
                      refine=2, pmap=None, pdepth=None, repair=True, ws_slot=0, defer_repair=False):
    """R, T of one chunk by the reflection-matrix recursion (khp_solve_batched).

    te, tm: optional [B, npol] complex device tensors (default: prob.te, prob.tm as one
    polarisation); the recursion runs once and every polarisation is read from it.
    pmap, pdepth: optional device tensors [L, B] (int32 map index into plan's maps, float64
    depth) giving every problem its own maps and depths.
    repair: re-solve the problems the mixed path flagged (status bits 8 and 32, see
    _repair_unconverged).  ws_slot: workspace slot of the call (engine.workspace).
    defer_repair: return (R, T, repair_fn) instead, where repair_fn() checks the flags and
    re-solves later (it reads this call's workspace, so the slot must not be reused before).
    Returns R, T of shape [B] (one polarisation) or [B, npol].
    """
    B = prob.batch
    dev = struct.device
    one_pol = te is None
    if one_pol:
        te, tm = prob.te.reshape(B, 1), prob.tm.reshape(B, 1)
    te, tm = te.contiguous(), tm.contiguous()
    npol = te.shape[1]
    R = torch.empty((B, npol), dtype=torch.float64, device=dev)
    T = torch.empty((B, npol), dtype=torch.float64, device=dev)
    lib = _capi.load()
    L = len(plan.kinds)
    epsi, epse = complex(epsi), complex(epse)
    if pmap is not None:
        pmap = pmap.to(torch.int32).contiguous()
        assert tuple(pmap.shape) == (L, B)
    if pdepth is not None:
        pdepth = pdepth.to(torch.float64).contiguous()
        assert tuple(pdepth.shape) == (L, B)
    common = (B, struct.pw[0], struct.pw[1], L, _host(plan.kinds), _host(plan.maps), _host(plan.eps),
              _host(plan.depth), _capi.ptr(pmap) if pmap is not None else None,
              _capi.ptr(pdepth) if pdepth is not None else None, plan.nmaps, _capi.ptr(plan.conv),
              _capi.ptr(plan.hx), _capi.ptr(plan.hy),
              _capi.ptr(struct.gx), _capi.ptr(struct.gy), epsi.real, epsi.imag, epse.real, epse.imag,
              _capi.ptr(prob.kp), _capi.ptr(prob.k0), npol, _capi.ptr(te), _capi.ptr(tm))
    fix = None
    if precision == "mixed":
        ws = engine.workspace(lib.khp_solve_batched_mixed_workspace(B, struct.nh, L, _host(plan.kinds),
                                                                     _host(plan.maps)), dev, ws_slot)
        with engine._stage("khp_solve_batched_mixed"):
            code = lib.khp_solve_batched_mixed(*common, int(refine), _capi.ptr(R), _capi.ptr(T), _capi.ptr(status),
                                               _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
        _capi.check(code, "khp_solve_batched_mixed")
        if repair or defer_repair:
            fix = functools.partial(_repair_unconverged, struct, plan, prob, status, epsi, epse, te, tm, R, T, pmap,
                                    pdepth, ws)
            if not defer_repair:
                fix()
                fix = None
    else:
        ws = engine.workspace(lib.khp_solve_batched_workspace(B, struct.nh, L, _host(plan.kinds), _host(plan.maps)),
                              dev, ws_slot)
        with engine._stage("khp_solve_batched"):
            code = lib.khp_solve_batched(*common, _capi.ptr(R), _capi.ptr(T), _capi.ptr(status), _capi.ptr(ws),
                                         ws.numel(), _capi.stream_ptr())
        _capi.check(code, "khp_solve_batched")
    if one_pol:
        R, T = R[:, 0], T[:, 0]
    if defer_repair:
        return R, T, (fix if fix is not None else (lambda: None))
    return R, T


REFINE_BIT = 8
MODES_BIT = 32
# Problems re-solved after the mixed path flagged them: "refine_repairs" (status bit 8, the stack
# refinement did not converge) are re-solved in FP64 from the mixed path's refined modes;
# "fp64_repairs" (status bit 32, a refined mode missed its residual test) by the full FP64 path.
STATS = {"refine_repairs": 0, "fp64_repairs": 0, "grad_repairs": 0}
# Rounds of stack refinement for the gradient call's second pass over problems whose refinement
# did not converge in the first (status bit 8; typically next to a Wood anomaly, where the FP32
# factors make each round gain only a factor ~0.3)
GRAD_REPAIR_ROUNDS = 40
REPAIR_WS_SLOT = 7  # workspace slot of the re-solves (the flagged call's own slot must stay intact)


def _sub_args(pmap, pdepth, te, tm, idx):
    pm = None if pmap is None else pmap[:, idx].contiguous()
    pd = None if pdepth is None else pdepth[:, idx].contiguous()
    return pm, pd, te[idx].contiguous(), tm[idx].contiguous()


def resolve_fp64(struct, plan, prob, sel, te, tm, epsi=1.0, epse=1.0, pmap=None, pdepth=None, mixed_ws=None):
    """R, T [K, npol] and status [K] of the problems at device indices ``sel`` of a chunk, by the
    FP64 reflection-matrix recursion.  With ``mixed_ws`` (the workspace of the chunk's
    khp_solve_batched_mixed call, unchanged since) the recursion starts from that call's refined
    FP64 modes (khp_solve_batched_mixed_repair); without, it runs its own FP64 eigensolve
    (khp_solve_batched).  te, tm: the chunk's [B, npol] source weights."""
    lib = _capi.load()
    dev = struct.device
    epsi, epse = complex(epsi), complex(epse)
    K, L, npol = int(sel.numel()), len(plan.kinds), te.shape[1]
    sub = prob.subset(sel)
    pm, pd, te_s, tm_s = _sub_args(pmap, pdepth, te, tm, sel)
    st = torch.zeros(K, dtype=torch.int32, device=dev)
    r = torch.empty((K, npol), dtype=torch.float64, device=dev)
    t = torch.empty_like(r)
    common = (K, struct.pw[0], struct.pw[1], L, _host(plan.kinds), _host(plan.maps), _host(plan.eps),
              _host(plan.depth), _capi.ptr(pm), _capi.ptr(pd), plan.nmaps, _capi.ptr(plan.conv),
              _capi.ptr(plan.hx), _capi.ptr(plan.hy), _capi.ptr(struct.gx), _capi.ptr(struct.gy),
              epsi.real, epsi.imag, epse.real, epse.imag, _capi.ptr(sub.kp), _capi.ptr(sub.k0), npol,
              _capi.ptr(te_s), _capi.ptr(tm_s))
    ws = engine.workspace(lib.khp_solve_batched_workspace(K, struct.nh, L, _host(plan.kinds), _host(plan.maps)),
                          dev, REPAIR_WS_SLOT)
    if mixed_ws is None:
        code = lib.khp_solve_batched(*common, _capi.ptr(r), _capi.ptr(t), _capi.ptr(st), _capi.ptr(ws), ws.numel(),
                                     _capi.stream_ptr())
        _capi.check(code, "khp_solve_batched")
    else:
        rows = sel.to(torch.int32).contiguous()
        code = lib.khp_solve_batched_mixed_repair(*common, prob.batch, _capi.ptr(rows), _capi.ptr(mixed_ws),
                                                  mixed_ws.numel(), _capi.ptr(r), _capi.ptr(t), _capi.ptr(st),
                                                  _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
        _capi.check(code, "khp_solve_batched_mixed_repair")
    return r, t, st


def _repair_unconverged(struct, plan, prob, status, epsi, epse, te, tm, R, T, pmap, pdepth, mixed_ws):
    """Re-solve the problems a mixed-precision call flagged; R, T and status in place.

    Status bit 8 (the stack refinement did not converge: an ill-conditioned stack, e.g. next to a
    Wood anomaly, where the FP32 factors make the refinement converge too slowly): the FP64
    reflection-matrix recursion from that call's refined FP64 modes, read from its workspace
    (no second eigensolve).  Status bit 32 (a refined mode missed its FP64 residual test): the
    full FP64 path with its own FP64 eigensolve."""
    flagged = (status & (REFINE_BIT | MODES_BIT)) != 0
    if not bool(flagged.any()):
        return
    idx = torch.nonzero(flagged).flatten()
    modes_bad = (status[idx] & MODES_BIT) != 0
    for sel, full in ((idx[~modes_bad], False), (idx[modes_bad], True)):
        K = int(sel.numel())
        if K == 0:
            continue
        STATS["fp64_repairs" if full else "refine_repairs"] += K
        r, t, st = resolve_fp64(struct, plan, prob, sel, te, tm, epsi, epse, pmap, pdepth,
                                None if full else mixed_ws)
        R[sel] = r
        T[sel] = t
        status[sel] = (status[sel] & ~(REFINE_BIT | MODES_BIT)) | st


def both_pol_weights(B, device):
    """te, tm [B, 2] for the polarisations (te, tm) = (1, 0) and (0, 1)."""
    te = torch.zeros((B, 2), dtype=torch.complex128, device=device)
    tm = torch.zeros((B, 2), dtype=torch.complex128, device=device)
    te[:, 0] = 1.0
    tm[:, 1] = 1.0
    return te, tm


def solve_chunk_gamma_both_pols(struct, plan, prob, status, epsi=1.0, epse=1.0, precision="fp64", refine=2, **kw):
    """R, T [B, 2] for (te, tm) = (1, 0) and (0, 1) from one recursion per problem (keyword
    arguments as solve_chunk_gamma: repair, ws_slot, defer_repair)."""
    te, tm = both_pol_weights(prob.batch, struct.device)
    return solve_chunk_gamma(struct, plan, prob, status, epsi, epse, te, tm, precision, refine, **kw)


def _no_repair():
    return None


_CAPTURE_STREAMS = {}
_CHUNK_STREAMS = {}


def _chunk_streams(device, count):
    """``count`` side streams of ``device`` that solve_rt deals its chunks (and solve_structures
    its shape groups) to; the same streams on every call, so that engine.workspace's per-stream
    cache finds their workspaces again."""
    key = str(device)
    have = _CHUNK_STREAMS.setdefault(key, [])
    while len(have) < count:
        have.append(torch.cuda.Stream(device=device))
    return have[:count]


def _capture_stream(device):
    """The side stream ChunkGraph captures on (one per device, so that every capture, and the
    eager call before it, find the same workspaces in engine.workspace's per-stream cache)."""
    key = str(device)
    if key not in _CAPTURE_STREAMS:
        _CAPTURE_STREAMS[key] = torch.cuda.Stream(device=device)
    return _CAPTURE_STREAMS[key]


class ChunkGraph:
    """One full-size chunk of the batched recursion (khp_solve_batched(_mixed), one or both
    polarisations) captured as a CUDA graph: the ~1000 launches of a chunk are replayed as one
    graph launch, with the next chunk's problems copied into the graph's input buffers first.

    The capture follows one eager call of the same chunk on the same side stream, which sizes
    the workspace (the graph then uses that buffer) and sets the kernels' attributes; outputs (R,
    T, status) live in the graph's memory and are overwritten by the next replay.  The deferred
    re-solve of flagged problems (mixed path) runs eagerly after a replay.  Library stage timing
    (khp_stage_timing) must be off while a graph is captured or replayed."""

    def __init__(self, struct, plan, B, precision, refine, epsi, epse, both_pols, ws_slot, prob0):
        self.B = B
        dev = struct.device
        self.prob = engine.Problems(k0=prob0.k0.clone(), kp=prob0.kp.clone(), te=prob0.te.clone(),
                                    tm=prob0.tm.clone())
        self.status = torch.zeros(B, dtype=torch.int32, device=dev)
        kw = dict(ws_slot=ws_slot, defer_repair=precision == "mixed", repair=False)

        def call():
            if both_pols:
                return solve_chunk_gamma_both_pols(struct, plan, self.prob, self.status, epsi, epse, precision,
                                                   refine, **kw)
            return solve_chunk_gamma(struct, plan, self.prob, self.status, epsi, epse, precision=precision,
                                     refine=refine, **kw)

        # the eager call solves prob0 (its results are first()'s), sizes the side stream's workspace
        # and sets the kernel attributes, so the capture allocates and configures nothing
        cap = _capture_stream(dev)
        cap.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(cap):
            out = call()
        # (the status buffer is shared with the graph: a replay clears it, so the caller reads these
        # results before the next replay)
        self._first = (out[0], out[1], self.status, out[2] if len(out) > 2 else _no_repair)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=cap, capture_error_mode="relaxed"):
            out = call()
        self.R, self.T = out[0], out[1]
        self.fix = out[2] if len(out) > 2 else _no_repair

    def first(self):
        """R, T, status and deferred re-solve of the eager call that preceded the capture."""
        return self._first

    def replay(self, prob):
        """Solve ``prob`` (B problems): returns R, T, status and the deferred re-solve."""
        for dst, src in ((self.prob.k0, prob.k0), (self.prob.kp, prob.kp), (self.prob.te, prob.te),
                         (self.prob.tm, prob.tm)):
            dst.copy_(src)
        self.status.zero_()
        self.graph.replay()
        return self.R, self.T, self.status, self.fix


def solve_rt(pw, layers, stack, wavelengths, kp, te=1.0, tm=0.0, lattice="square", epsi=1.0, epse=1.0,
             chunk=256, orders=False, device="cuda", struct=None, strict=True, both_pols=False, method="gamma",
             refine=2, graphs=False, streams=2):
    """R and T of every problem (host numpy arrays); problems share ``layers``/``stack``.

    layers: name -> ("pixmap", eps_map, depth) | ("uniform", eps, depth); stack: layer names
    from the incidence side.  wavelengths [P], kp [P, 2] (absolute, complex allowed), te/tm
    scalars or [P].  Returns (R, T, status) or (R, T, r_orders, t_orders, status) with
    ``orders=True``.  ``both_pols=True`` returns R, T of shape [P, 2] for (te, tm) = (1, 0)
    and (0, 1).  ``method``: "gamma" (reflection-matrix recursion in FP64, khp_solve_batched),
    "mixed" (the same recursion in FP32 with FP64 eigen-refinement and ``refine`` rounds of FP64
    iterative refinement, khp_solve_batched_mixed) or "chain" (layer S-matrices and the
    star-product chain, as the reference; needed for per-order powers).  With ``strict`` a
    non-zero per-problem status raises KhpError.  ``graphs=True`` (methods "gamma" and "mixed"):
    every full-size chunk after the first replays a CUDA graph of the chunk solve (ChunkGraph, one
    per workspace slot) instead of enqueueing its launches one by one; the results are the same.
    ``streams`` (methods "gamma" and "mixed" without graphs): chunk c is enqueued on side stream
    c mod ``streams``, so that one chunk's stages run beside the next one's on the device; each
    stream has its own workspaces, and the results do not depend on it.
    """
    if orders:
        method = "chain"
    _capi.require_cuda()
    wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
    P = wl.shape[0]
    kpa = np.asarray(kp, dtype=complex).reshape(P, 2)
    te = np.broadcast_to(np.asarray(te, dtype=complex), (P,))
    tm = np.broadcast_to(np.asarray(tm, dtype=complex), (P,))
    if struct is None:
        struct = engine.StructureGPU(pw, engine.lattice_vectors(lattice), device)
    specs = _specs(layers, epsi, epse)
    plan = StackPlan(struct, specs, stack) if method in ("gamma", "mixed") else None
    prec = "mixed" if method == "mixed" else "fp64"
    R = np.empty((P, 2) if both_pols else P)
    T = np.empty((P, 2) if both_pols else P)
    ro = np.empty((P, struct.nh)) if orders else None
    to = np.empty((P, struct.nh)) if orders else None
    st = np.zeros(P, dtype=np.int32)

    def finish(job):
        # the chunk's deferred re-solve of flagged problems, then its results to the host (on the
        # chunk's stream, which orders the copies after its work)
        sc, s, e, r, t, r_o, t_o, status, fix = job
        with torch.cuda.stream(sc):
            fix()
            R[s:e] = r.cpu().numpy()
            T[s:e] = t.cpu().numpy()
            if orders:
                ro[s:e] = r_o.cpu().numpy()
                to[s:e] = t_o.cpu().numpy()
            st[s:e] = status.cpu().numpy()

    # Chunk c is finished (flags read, flagged problems re-solved, results copied back) only after
    # the next max(1, S - 1) chunks are enqueued (S streams), so the device never waits for the
    # host's look at the flags.  The chunks in flight use distinct workspace slots; the next chunk
    # on a stream reuses a slot only after the chunk that held it was finished.
    use_graphs = graphs and method in ("gamma", "mixed")
    nstreams = max(1, int(streams)) if method in ("gamma", "mixed") and not use_graphs else 1
    cur = torch.cuda.current_stream(struct.device)
    side = _chunk_streams(struct.device, nstreams) if nstreams > 1 else None
    nslots, lag = max(2, nstreams), max(1, nstreams - 1)
    pending = []
    cgraphs = {}
    for c, s in enumerate(range(0, P, chunk)):
        e = min(P, s + chunk)
        sc = side[c % nstreams] if side else cur
        if side:
            sc.wait_stream(cur)
        with torch.cuda.stream(sc):
            prob = engine.Problems.make(wl[s:e], kpa[s:e], te[s:e], tm[s:e], struct.device)
            status = torch.zeros(e - s, dtype=torch.int32, device=struct.device)
            r_o = t_o = None
            fix = _no_repair
            if use_graphs and e - s == chunk and c > 0:
                g = cgraphs.get(c % 2)
                if g is None:
                    while pending:  # the capture waits for the device anyway
                        finish(pending.pop(0))
                    g = cgraphs[c % 2] = ChunkGraph(struct, plan, chunk, prec, refine, epsi, epse, both_pols,
                                                    c % 2, prob)
                    r, t, status, fix = g.first()
                else:
                    r, t, status, fix = g.replay(prob)
            elif method in ("gamma", "mixed"):
                kw = dict(ws_slot=c % nslots, defer_repair=prec == "mixed")
                if both_pols:
                    out = solve_chunk_gamma_both_pols(struct, plan, prob, status, epsi, epse, prec, refine, **kw)
                else:
                    out = solve_chunk_gamma(struct, plan, prob, status, epsi, epse, precision=prec, refine=refine,
                                            **kw)
                r, t = out[0], out[1]
                if prec == "mixed":
                    fix = out[2]
            elif both_pols:
                r, t = solve_chunk_both_pols(struct, specs, stack, prob, status, epsi, epse)
            else:
                r, t, r_o, t_o = solve_chunk(struct, specs, stack, prob, status, orders, epsi, epse)
        pending.append((sc, s, e, r, t, r_o, t_o, status, fix))
        while len(pending) > lag:
            finish(pending.pop(0))
    while pending:
        finish(pending.pop(0))
    for sc in side or ():
        cur.wait_stream(sc)
    if strict and st.any():
        bad = int(np.flatnonzero(st)[0])
        raise _capi.KhpError(f"problem {bad}: {_capi.decode_status(int(st[bad]))}")
    if orders:
        return R, T, ro, to, st
    return R, T, st


# ------------------------------------------------------------------------------------------
# Many structures of one shape per launch
# ------------------------------------------------------------------------------------------
class _ChunkPlan:
    """StackPlan-like description of one chunk of problems over several structures of one shape:
    per-layer kinds and uniform eps shared, maps and depths per problem."""

    def __init__(self, kinds, slots, eps, conv, hx, hy):
        self.kinds = np.asarray(kinds, dtype=np.int32)
        self.maps = np.asarray(slots, dtype=np.int32)
        self.eps = np.asarray(eps, dtype=np.complex128)
        self.depth = np.zeros(len(kinds), dtype=np.float64)  # per-problem depths are passed instead
        self.nmaps = 0 if conv is None else int(conv.shape[0])
        self.conv, self.hx, self.hy = conv, hx, hy
        self.ic = None


def _shape_key(layers, stack):
    """Layer kinds, uniform eps and which patterned layers share a pixmap (first-use slots)."""
    kinds, slots, eps, digests = [], [], [], []
    for name in stack:
        kind, e, _ = layers[name]
        if kind == "pixmap":
            d = engine._digest(e)
            if d not in digests:
                digests.append(d)
            kinds.append(1)
            slots.append(digests.index(d))
            eps.append(0j)
        else:
            kinds.append(0)
            slots.append(0)
            eps.append(complex(e))
    return (tuple(kinds), tuple(slots), tuple(eps)), digests


def prepare_maps(struct, eps_maps):
    """C, C^-1, Hx, Hy of a stack of pixmaps [M, nx, ny] in two batched launches (khp_convmat,
    khp_structure_prep).  Raises KhpError when a convolution matrix is singular."""
    lib = _capi.load()
    sp = _capi.stream_ptr()
    eps = torch.as_tensor(np.asarray(eps_maps), device=struct.device).to(torch.complex128).contiguous()
    M, nx, ny = eps.shape
    px, py = struct.pw
    nh = struct.nh
    conv = torch.empty((M, nh, nh), dtype=torch.complex128, device=struct.device)
    ws = engine.workspace(lib.khp_convmat_workspace(M, px, py), struct.device)
    _capi.check(lib.khp_convmat(M, nx, ny, _capi.ptr(eps), px, py, _capi.ptr(conv), _capi.ptr(ws), ws.numel(), sp),
                "khp_convmat")
    ic, hx, hy = torch.empty_like(conv), torch.empty_like(conv), torch.empty_like(conv)
    st = torch.zeros(M, dtype=torch.int32, device=struct.device)
    ws = engine.workspace(lib.khp_structure_prep_workspace(M, nh), struct.device)
    _capi.check(lib.khp_structure_prep(M, nh, _capi.ptr(conv), _capi.ptr(struct.gx), _capi.ptr(struct.gy),
                                       _capi.ptr(ic), _capi.ptr(hx), _capi.ptr(hy), _capi.ptr(st), _capi.ptr(ws),
                                       ws.numel(), sp), "khp_structure_prep")
    if bool(st.any()):
        bad = int(torch.nonzero(st).flatten()[0])
        raise _capi.KhpError(f"convolution matrix of pixmap {bad}: {_capi.decode_status(int(st[bad]))}")
    return conv, ic, hx, hy


def convmat_bwd(struct, dconv, nx, ny):
    """Gradient with respect to pixmaps [M, nx, ny] from the convolution-matrix gradient
    [M, nh, nh] (khp_convmat_bwd; both in the convention dL = Re sum(d o delta))."""
    lib = _capi.load()
    M = int(dconv.shape[0])
    px, py = struct.pw
    deps = torch.empty((M, nx, ny), dtype=torch.complex128, device=dconv.device)
    ws = engine.workspace(lib.khp_convmat_bwd_workspace(M, ny, px, py), dconv.device)
    _capi.check(lib.khp_convmat_bwd(M, nx, ny, _capi.ptr(dconv.contiguous()), px, py, _capi.ptr(deps), _capi.ptr(ws),
                                    ws.numel(), _capi.stream_ptr()), "khp_convmat_bwd")
    return deps


def _group_plan(structures, which, chunk):
    """The shape groups of the problems (host only): a list of (key, [problem index arrays, one
    per chunk]) and the per-structure map digests."""
    keys, digests = [], []
    for pw, layers, stack in structures:
        k, d = _shape_key(layers, stack)
        keys.append((tuple(pw),) + k)
        digests.append(d)
    groups = {}
    for p in range(len(which)):
        groups.setdefault(keys[which[p]], []).append(p)
    out = []
    for key, members in groups.items():
        pw, kinds, slots = key[0], key[1], key[2]
        members = np.asarray(members)
        nslots = len({s for k, s in zip(kinds, slots) if k == 1}) or 1
        step = chunk if chunk else autotune.chunk_for(2 * pw[0] * pw[1], nslots)
        out.append((key, [members[s:s + step] for s in range(0, len(members), step)]))
    return out, digests


def _chunk_item(structures, which, digests, key, idx, struct):
    """(struct, idx, plan, pmap, pdepth, maps, eps_maps) of one chunk: the chunk's pixmaps prepared
    on the device (C, C^-1, Hx, Hy), per-problem map indices and depths."""
    kinds, slots, eps = key[1], key[2], key[3]
    L = len(kinds)
    B = len(idx)
    mpos, eps_maps = {}, []
    for sid in dict.fromkeys(which[idx].tolist()):
        _, layers, stack = structures[sid]
        for name in stack:
            kind, e, _ = layers[name]
            if kind != "pixmap":
                continue
            slot = digests[sid].index(engine._digest(e))
            if (sid, slot) not in mpos:
                mpos[(sid, slot)] = len(eps_maps)
                eps_maps.append(np.asarray(e))
    conv = ic = hx = hy = None
    if eps_maps:
        conv, ic, hx, hy = prepare_maps(struct, np.stack(eps_maps))
    pm = np.zeros((L, B), dtype=np.int32)
    pd = np.zeros((L, B), dtype=np.float64)
    for j, p in enumerate(idx):
        sid = which[p]
        _, layers, stack = structures[sid]
        for l, name in enumerate(stack):
            pd[l, j] = layers[name][2]
            if kinds[l] == 1:
                pm[l, j] = mpos[(sid, slots[l])]
    plan = _ChunkPlan(kinds, slots, eps, conv, hx, hy)
    plan.ic = ic
    maps = sorted(mpos, key=mpos.get)
    return (struct, idx, plan, torch.tensor(pm, device=struct.device), torch.tensor(pd, device=struct.device),
            maps, eps_maps)


def _group_chunks(structures, which, chunk, lattice, device):
    """Yield (struct, idx, plan, pmap, pdepth, maps, eps_maps) for every chunk of every shape group:
    ``maps`` lists the (structure, slot) of each prepared map, ``plan`` carries C, C^-1, Hx, Hy."""
    groups, digests = _group_plan(structures, which, chunk)
    lat = engine.lattice_vectors(lattice)
    for key, chunks in groups:
        struct = engine.StructureGPU(key[0], lat, device)
        for idx in chunks:
            yield _chunk_item(structures, which, digests, key, idx, struct)


def _prep_args(wavelengths, kp, which, te, tm):
    wl = np.atleast_1d(np.asarray(wavelengths, dtype=float))
    P = wl.shape[0]
    kpa = np.asarray(kp, dtype=complex).reshape(P, 2)
    which = np.arange(P) if which is None else np.asarray(which, dtype=np.int64).reshape(P)
    te = np.broadcast_to(np.asarray(te, dtype=complex), (P,))
    tm = np.broadcast_to(np.asarray(tm, dtype=complex), (P,))
    return wl, P, kpa, which, te, tm


def solve_structures(structures, wavelengths, kp, which=None, te=1.0, tm=0.0, lattice="square", epsi=1.0,
                     epse=1.0, chunk=None, both_pols=False, method="mixed", refine=2, strict=True, device="cuda",
                     streams=4):
    """R and T of problems spread over many structures, batched across structures.

    structures: list of (pw, layers, stack) (``layers`` as in solve_rt); which: [P] structure of
    each problem (default: problem i uses structure i).  Structures with the same harmonic set,
    layer kinds, uniform media and pixmap-sharing pattern form one group; each chunk of a group is
    one khp_solve_batched(_mixed) call with per-problem maps and depths (maps of the chunk
    prepared in one batched launch).  chunk: problems per call (None: the autotuned number of
    mode matrices per call for the group's size, divided by its maps per problem).
    method: "mixed" (default) or "gamma" (FP64).
    streams: CUDA streams the shape groups are dealt to in turn, each stream with its own
    workspaces; a group's chunks stay on its stream.  Many small groups (structures of uneven
    sizes) then fill the GPU together instead of one after the other; a chunk's flags are read
    (and its flagged problems re-solved) only when its stream takes its next chunk.
    Returns R, T ([P] or [P, 2] with ``both_pols``) and status [P].
    """
    _capi.require_cuda()
    wl, P, kpa, which, te, tm = _prep_args(wavelengths, kp, which, te, tm)
    prec = "mixed" if method == "mixed" else "fp64"
    R = np.empty((P, 2) if both_pols else P)
    T = np.empty((P, 2) if both_pols else P)
    st_all = np.zeros(P, dtype=np.int32)
    dev = torch.device(device)
    if dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    main = torch.cuda.current_stream(dev)
    K = max(1, int(streams))
    # the same side streams on every call: engine.workspace keys its buffers by stream, so fresh
    # streams (torch cycles through a pool of 32) would leave a workspace behind for each
    ss = [main] + _chunk_streams(dev, K - 1)
    for s in ss[1:]:
        s.wait_stream(main)  # the caller's earlier work on the inputs comes first
    pending = [None] * K

    def finish(k):
        """Repairs and results of the chunk in flight on stream k (on that stream)."""
        if pending[k] is None:
            return
        idx, r, t, status, fix, keep = pending[k]
        pending[k] = None
        with torch.cuda.stream(ss[k]):
            fix()
            R[idx] = r.cpu().numpy()
            T[idx] = t.cpu().numpy()
            st_all[idx] = status.cpu().numpy()

    # a shape group's chunks run on one stream (they share the group's device data); groups are
    # dealt to the streams in turn
    groups, digests = _group_plan(structures, which, chunk)
    lat = engine.lattice_vectors(lattice)
    for gi, (key, chunk_idx) in enumerate(groups):
        k = gi % K
        struct_k = None
        for idx in chunk_idx:
            finish(k)  # the stream's workspaces are reused by its next chunk
            with torch.cuda.stream(ss[k]):
                if struct_k is None:
                    struct_k = engine.StructureGPU(key[0], lat, dev)
                _, _, plan, pmap, pdepth, _, _ = _chunk_item(structures, which, digests, key, idx, struct_k)
                B = len(idx)
                prob = engine.Problems.make(wl[idx], kpa[idx], te[idx], tm[idx], dev)
                status = torch.zeros(B, dtype=torch.int32, device=dev)
                # the autotuned chunk comes with its tuned eigensolver team size
                with (autotune.tuned_team(struct_k.n) if chunk is None else contextlib.nullcontext()):
                    if both_pols:
                        tt, tmm = both_pol_weights(B, dev)
                        r, t, fix = solve_chunk_gamma(struct_k, plan, prob, status, epsi, epse, tt, tmm, prec, refine,
                                                      pmap, pdepth, defer_repair=True)
                    else:
                        r, t, fix = solve_chunk_gamma(struct_k, plan, prob, status, epsi, epse, precision=prec,
                                                      refine=refine, pmap=pmap, pdepth=pdepth, defer_repair=True)
                pending[k] = (idx, r, t, status, fix, (struct_k, plan, prob, pmap, pdepth))
    for k in range(K):
        finish(k)
    for s in ss[1:]:
        main.wait_stream(s)
    if strict and st_all.any():
        bad = int(np.flatnonzero(st_all)[0])
        raise _capi.KhpError(f"problem {bad}: {_capi.decode_status(int(st_all[bad]))}")
    return R, T, st_all


def solve_structures_grad(structures, wavelengths, kp, which=None, dR=None, dT=None, te=1.0, tm=0.0,
                          lattice="square", epsi=1.0, epse=1.0, chunk=256, refine=2, strict=True, device="cuda"):
    """Solve + gradient over many structures (khp_solve_batched_mixed_grad + khp_convmat_bwd).

    dR, dT: [P, nh] weights of the per-order reflected / transmitted powers in the loss
    L = sum dR * R_orders + dT * T_orders (None = 0); every structure in a call has the same
    harmonic count.  Returns R [P], T [P], R_orders [P, nh], T_orders [P, nh], grads, status:
    grads[s][name] = dL/d(eps map) of structure s's pixmap layer ``name`` as a complex [nx, ny]
    array in the convention dL = Re sum(grad * d eps) (for a real map, dL/deps = grad.real);
    layers sharing one pixmap get the total gradient with respect to that pixmap.  A problem whose
    stack refinement does not converge adds nothing to the first call's gradients; it is solved
    again with more refinement rounds and its share added (``STATS["grad_repairs"]``); what stays
    unconverged keeps status bit 8.
    """
    _capi.require_cuda()
    wl, P, kpa, which, te, tm = _prep_args(wavelengths, kp, which, te, tm)
    lib = _capi.load()
    R = np.empty(P)
    T = np.empty(P)
    Ro = To = None
    st_all = np.zeros(P, dtype=np.int32)
    grads = [dict() for _ in structures]
    for struct, idx, plan, pmap, pdepth, maps, eps_maps in _group_chunks(structures, which, chunk, lattice, device):
        B, nh = len(idx), struct.nh
        if Ro is None:
            Ro, To = np.empty((P, nh)), np.empty((P, nh))
        dev = struct.device
        prob = engine.Problems.make(wl[idx], kpa[idx], te[idx], tm[idx], dev)
        wr = None if dR is None else torch.tensor(np.asarray(dR, dtype=float)[idx].reshape(B, 1, nh), device=dev)
        wt = None if dT is None else torch.tensor(np.asarray(dT, dtype=float)[idx].reshape(B, 1, nh), device=dev)
        L = len(plan.kinds)
        ei, ee = complex(epsi), complex(epse)

        def run(sel, rounds):
            """The gradient call on the chunk's problems at device indices ``sel`` (None: all)."""
            pb = prob if sel is None else prob.subset(sel)
            K = pb.batch
            pm = pmap if sel is None else pmap[:, sel].contiguous()
            pd = pdepth if sel is None else pdepth[:, sel].contiguous()
            ted, tmd = pb.te.reshape(K, 1).contiguous(), pb.tm.reshape(K, 1).contiguous()
            wrs = None if wr is None else (wr if sel is None else wr[sel].contiguous())
            wts = None if wt is None else (wt if sel is None else wt[sel].contiguous())
            st_k = torch.zeros(K, dtype=torch.int32, device=dev)
            r_k = torch.empty((K, 1), dtype=torch.float64, device=dev)
            t_k = torch.empty((K, 1), dtype=torch.float64, device=dev)
            ro_k = torch.empty((K, 1, nh), dtype=torch.float64, device=dev)
            to_k = torch.empty((K, 1, nh), dtype=torch.float64, device=dev)
            dconv_k = torch.empty((plan.nmaps, nh, nh), dtype=torch.complex128, device=dev)
            ws = engine.workspace(lib.khp_solve_batched_mixed_grad_workspace(K, nh, L, _host(plan.kinds),
                                                                             _host(plan.maps), plan.nmaps), dev)
            with engine._stage("khp_solve_batched_mixed_grad"):
                code = lib.khp_solve_batched_mixed_grad(
                    K, struct.pw[0], struct.pw[1], L, _host(plan.kinds), _host(plan.maps), _host(plan.eps),
                    _host(plan.depth), _capi.ptr(pm), _capi.ptr(pd), plan.nmaps, _capi.ptr(plan.conv),
                    _capi.ptr(plan.ic), _capi.ptr(plan.hx), _capi.ptr(plan.hy), _capi.ptr(struct.gx),
                    _capi.ptr(struct.gy), ei.real, ei.imag, ee.real, ee.imag, _capi.ptr(pb.kp), _capi.ptr(pb.k0), 1,
                    _capi.ptr(ted), _capi.ptr(tmd), int(rounds), _capi.ptr(wrs), _capi.ptr(wts), _capi.ptr(r_k),
                    _capi.ptr(t_k), _capi.ptr(ro_k), _capi.ptr(to_k), _capi.ptr(dconv_k), _capi.ptr(st_k),
                    _capi.ptr(ws), ws.numel(), _capi.stream_ptr())
            _capi.check(code, "khp_solve_batched_mixed_grad")
            return r_k, t_k, ro_k, to_k, dconv_k, st_k

        r, t, ro, to, dconv, status = run(None, refine)
        # A problem whose stack refinement did not converge (status bit 8; the modes are good)
        # adds nothing to the call's map gradients; it is solved again with GRAD_REPAIR_ROUNDS
        # rounds and its share added.
        flagged = (status & REFINE_BIT) != 0
        if bool(flagged.any()):
            sel = torch.nonzero(flagged).flatten()
            r2, t2, ro2, to2, dconv_new, st2 = run(sel, max(int(refine), GRAD_REPAIR_ROUNDS))
            dconv = dconv + dconv_new
            r[sel], t[sel], ro[sel], to[sel] = r2, t2, ro2, to2
            status[sel] = (status[sel] & ~REFINE_BIT) | st2
            STATS["grad_repairs"] += int(sel.numel())
        R[idx] = r[:, 0].cpu().numpy()
        T[idx] = t[:, 0].cpu().numpy()
        Ro[idx] = ro[:, 0].cpu().numpy()
        To[idx] = to[:, 0].cpu().numpy()
        st_all[idx] = status.cpu().numpy()
        if maps:
            shapes = {np.asarray(e).shape for e in eps_maps}
            for shp in shapes:
                sel = [k for k, e in enumerate(eps_maps) if np.asarray(e).shape == shp]
                deps = convmat_bwd(struct, dconv[sel], shp[0], shp[1]).cpu().numpy()
                for k, d in zip(sel, deps):
                    sid, slot = maps[k]
                    _, layers, stack = structures[sid]
                    for l, name in enumerate(stack):
                        if plan.kinds[l] == 1 and plan.maps[l] == slot:
                            grads[sid][name] = grads[sid].get(name, 0) + d
    if strict and st_all.any():
        bad = int(np.flatnonzero(st_all)[0])
        raise _capi.KhpError(f"problem {bad}: {_capi.decode_status(int(st_all[bad]))}")
    return R, T, Ro, To, grads, st_all
