"""Per-size launch schedules for the batched solve, measured on the GPU.

Two choices decide the speed of khp_solve_batched_mixed at a given mode-matrix size n = 2 Px Py
and depend on the GPU rather than on the problem:

* ``eig_threads``: threads per CTA of the eigensolver (khp_tune, KHP_TUNE_EIG_THREADS).  One CTA
  works on one matrix; a small matrix leaves most of a 256-thread team idle, and a smaller team
  lets more matrices share an SM.
* ``matrices``: mode matrices per call (problems per call x distinct maps per problem).  More
  matrices fill the GPU better until the workspace or the tail of the last wave costs more.

``tune()`` times every candidate pair on synthetic problems of each size (one smoothed, lossy
random map per structure, the uneven-batch shapes) and writes the fastest per size to
``tuning.json`` beside this file; ``batch.solve_structures`` applies that table when it picks
the chunk itself (``chunk_for``, ``tuned_team``).  Run it on the GPU the library will use:

    python -m khepri_gb300.autotune [--sizes 3 5 ... 17] [--out path]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import time

import numpy as np
import torch

from . import _capi

TUNING_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")
_table = None


def load(path=TUNING_PATH):
    """The tuning table {n: {"eig_threads": T, "matrices": M, ...}} ({} when there is none)."""
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        data = json.load(f)
    return {int(k): v for k, v in data.get("sizes", {}).items()}


def table():
    """The committed table, read once per process."""
    global _table
    if _table is None:
        _table = load()
    return _table


class tuned_team:
    """Context manager: the tuned eigensolver team size for matrices of size n inside, the default
    after.  The team size is tuned together with the matrices per call, so it applies only to
    calls that also take ``chunk_for``'s chunk (a 128-thread team that wins at 912 matrices per
    call loses at 456)."""

    def __init__(self, n):
        self.n = int(n)
        self.threads = int(table().get(self.n, {}).get("eig_threads", 0))

    def __enter__(self):
        if self.threads:
            _capi.check(_capi.load().khp_tune(1, self.n, self.threads), "khp_tune")
        return self

    def __exit__(self, *exc):
        if self.threads:
            _capi.load().khp_tune(1, self.n, 0)
        return False


def chunk_for(n, slots=1, default=256):
    """Problems per call for mode matrices of size n with ``slots`` distinct maps per problem."""
    e = table().get(int(n))
    if e is None:
        return default
    return max(1, int(e["matrices"]) // max(1, int(slots)))


def _problems(p, count, rng):
    """``count`` one-layer structures at Px = Py = p (smoothed lossy maps, one in-cone problem each),
    as solve_structures takes them."""
    from . import workloads
    ents, wl, kp = [], [], []
    for _ in range(count):
        re = workloads.periodic_gaussian_blur(rng.uniform(1.0, 12.0, size=(64, 64)), 4.0)
        im = -workloads.periodic_gaussian_blur(rng.uniform(0.0, 0.1, size=(64, 64)), 4.0)
        ents.append(((p, p), {"L0": ("pixmap", re + 1j * im, float(rng.uniform(0.2, 1.0)))}, ["L0"]))
        f = float(rng.uniform(0.3, 0.8))
        while True:
            k = (rng.uniform(0.0, 1.0, size=2) - 0.5) * 2 * np.pi
            if np.hypot(*k) < 0.98 * 2 * np.pi * f:
                break
        wl.append(1.0 / f)
        kp.append(k)
    return ents, np.array(wl), np.array(kp)


def _time_call(ents, wl, kp, chunk):
    from . import batch
    # an explicit chunk: the team size set by tune() stays in force
    batch.solve_structures(ents, wl, kp, chunk=chunk, strict=False)  # warm-up (maps, workspace, modules)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.solve_structures(ents, wl, kp, chunk=chunk, strict=False)
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def tune(sizes=(3, 5, 7, 9, 11, 13, 15, 17), threads=(64, 128, 256), matrices=(152, 304, 456, 912),
         budget_gb=48.0, out=TUNING_PATH, seed=0, verbose=True):
    """Time every (eig_threads, matrices) pair per size and write the fastest to ``out``."""
    global _table
    lib = _capi.load()
    rng = np.random.default_rng(seed)
    result = {}
    for p in sizes:
        n = 2 * p * p
        kinds, maps = np.array([1], np.int32), np.array([0], np.int32)
        per = lib.khp_solve_batched_mixed_workspace(1, p * p, 1, kinds.ctypes.data_as(ctypes.c_void_p),
                                                    maps.ctypes.data_as(ctypes.c_void_p))
        cands = [m for m in matrices if m * per <= budget_gb * 2 ** 30] or [matrices[0]]
        ents, wl, kp = _problems(p, max(cands), rng)
        best = None
        rows = []
        for th in threads:
            _capi.check(lib.khp_tune(1, n, th), "khp_tune")
            for m in cands:
                t = _time_call(ents[:m], wl[:m], kp[:m], m)
                us = 1e6 * t / m
                rows.append({"eig_threads": th, "matrices": m, "us_per_problem": us})
                if best is None or us < best["us_per_problem"]:
                    best = rows[-1]
        _capi.check(lib.khp_tune(1, n, 0), "khp_tune")
        result[n] = dict(best, pw=p, candidates=rows)
        if verbose:
            print(f"n={n}: eig_threads {best['eig_threads']}, {best['matrices']} matrices per call, "
                  f"{best['us_per_problem']:.1f} us per problem", flush=True)
    data = {"device": torch.cuda.get_device_name(), "note": "one-layer structures, khp_solve_batched_mixed, "
            "wall clock per call after a warm-up call; the fastest (eig_threads, matrices) per size",
            "sizes": {str(k): v for k, v in sorted(result.items())}}
    with open(out, "w") as f:
        json.dump(data, f, indent=1)
    _table = None
    return result


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", type=int, nargs="*", default=[3, 5, 7, 9, 11, 13, 15, 17])
    ap.add_argument("--out", default=TUNING_PATH)
    args = ap.parse_args()
    tune(tuple(args.sizes), out=args.out)


if __name__ == "__main__":
    main()
