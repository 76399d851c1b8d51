"""Benchmark: batched RCWA solves/s at 11x11 harmonics on GB300 (one JSON line on stdout).

Workload (the batched sweep): one seed of the 11x11 structure — a 256x256 binary pixmap (union
of 1-4 periodic discs, eps 12 in eps 1) shared by 3 patterned layers, 2 uniform layers, depths
U(0.2, 1.0) — over 64 frequencies 0.3-0.7 c/a x a 32x32 Bloch grid (65,536 problems), both
polarisations from one S-matrix per problem.  A step solves one chunk of ``--batch`` problems
(successive chunks of the sweep, dealt to two CUDA streams in turn so that two chunks are in
flight).  Synthetic seeded inputs: no dataset is involved.

* value: problems (S-matrix solves) per second with the problem arrays resident in HBM,
  timed with CUDA events over exactly K steps (barrier + synchronize on both sides).
* e2e: the same metric through the public batched API (khepri_gb300.batch.solve_rt) from host
  numpy inputs to host R/T, host<->device copies inside the timed region.
* roofline: the dominant kernels, the FP32 eigensolver of the modes stage (k_gehrd +
  k_geev_schur): its algorithmic flops per call (100 n^3 per matrix) / its mean launch duration, timed by CUDA
  events that libkhp records on its stream around each stage (khp_stage_timing), against the
  FP32 FMA throughput measured in this run (khp_probe_fp32_tflops).  The per-stage times and
  the tensor-core products' fraction of the bf16 peak ride along.
* cpu_baseline: the CPU oracle (numpy/LAPACK restatement of the reference) on a bounded sample.

``--impl reference`` times that CPU restatement alone (all host threads), same metric/config.
Multi-GPU (torchrun): independent replicas, each rank solving its own chunks; no collective on
the data path; value = problems of all ranks / max over ranks of the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RCWA solves/s + solve+grad/s, 11×11 harmonics, batched vs plain GPU, |ΔT|≤1e-6"
UNIT = "solves/s"
PW = (11, 11)
N_MAT = 2 * PW[0] * PW[1]
# Algorithmic flops per problem of each entry point (real flops, complex MAC = 8; conventions:
# GEMM 8n^3, LU 8/3 n^3, eig 100 n^3; P build 1, P.Q 8, eig 100, V 8 -> modes 117 n^3;
# build_scatmat 85.3 n^3; star product 106.7 n^3).
FLOPS_PER_CALL = {
    "khp_layer_modes": 117.0 * N_MAT ** 3,
    "khp_layer_smatrix": 85.3 * N_MAT ** 3,
    "khp_star_product": 106.7 * N_MAT ** 3,
}


def _up64(x):
    return (x + 63) // 64 * 64


def _up128(x):
    return (x + 127) // 128 * 128


# bf16 tensor flops issued per modes matrix by the FP64-accurate products of the mixed solve
# (k_tc_digits: 8 digits, the 36 pairs i + j < 8, rows padded to 128, real columns and inner
# index to 64): M W twice (m = k = n) and C W twice (m = k = n/2, n complex columns)
TC_PAIRS = 36
TC_FLOPS_PER_MATRIX = TC_PAIRS * 2 * (2 * _up128(N_MAT) * _up64(2 * N_MAT) * _up64(2 * N_MAT)
                                      + 2 * _up128(N_MAT // 2) * _up64(2 * N_MAT) * _up64(N_MAT))
BF16_PEAK = 1935.4  # TFLOP/s, MEASURED_PEAKS.json bf16_tflops (burst)
# DRAM bytes per matrix of the FP32 eigensolver (read + write of k_gehrd, k_geev_schur and
# k_hqr_apply_log) at 912 matrices per launch and 128-thread teams, from one ncu capture of the
# bench's eigensolver launches (dram__bytes_read.sum + dram__bytes_write.sum, one pass)
GEEV_TRAFFIC_PER_MATRIX = (70947202816 + 18853817088 + 80481979392 + 95487486208 + 1118951936 + 392237056) / 912


def solve_mixed_flops(n, nmaps, npattern, nhomog):
    """Algorithmic flops per problem of khp_solve_batched_mixed (FP32 and FP64 together): the
    recursion as in solve_batched_flops, plus per map the eigen-refinement (FP64 residual GEMM
    8 n^3, FP32 solve 10.67 n^3, FP32 correction GEMM 8 n^3, FP64 V = QW 4 n^3)."""
    return solve_batched_flops(n, nmaps, npattern, nhomog) + n ** 3 * nmaps * (8.0 + 10.67 + 8.0 + 4.0)


def solve_batched_flops(n, nmaps, npattern, nhomog):
    """Algorithmic flops per problem of khp_solve_batched: per distinct map the modes (117 n^3)
    and W^-1, V^-1 (2 x 10.67 n^3); per patterned layer 4 GEMMs + 2 LU + 2 right-solves
    (53.3 n^3); per homogeneous layer an LU and a right-solve (10.67 n^3); the incidence LU."""
    return n ** 3 * (nmaps * (117.0 + 21.33) + 53.33 * npattern + 10.67 * nhomog + 2.67)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=912,
                    help="problems per call (912 = 6 x 152 SMs: six 128-thread eigensolver CTAs per SM)")
    ap.add_argument("--eig-threads", type=int, default=128,
                    help="eigensolver threads per CTA for the sweep's 242 x 242 matrices (khp_tune; 0 = the "
                         "library default, 256)")
    ap.add_argument("--mode-digits", type=int, default=0, choices=[0, 6, 8],
                    help="7-bit digits per operand of the eigen-refinement steps' M W products (khp_tune; 0 = "
                         "library default)")
    ap.add_argument("--tf32-min-n", type=int, default=-1,
                    help="smallest n whose recursion products run as 3xTF32 on the tensor cores (khp_tune; 0 = "
                         "never; -1 = the library default)")
    ap.add_argument("--impl", default="khepri_gb300", choices=["khepri_gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=6)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--refine", type=int, default=2)
    ap.add_argument("--plain", type=int, default=2, help="single-problem drop-in solves timed for comparison")
    ap.add_argument("--grad-designs", type=int, default=64,
                    help="inverse-design structures (x 16 frequencies) for the solve+grad measurement (0 = skip)")
    ap.add_argument("--uneven", type=int, default=1024,
                    help="uneven structures (config 3's shapes) for the many-structure measurement (0 = skip)")
    ap.add_argument("--twisted7", type=int, default=4,
                    help="twisted-bilayer problems at 7x7 base harmonics (n = 4802) for the extended-crystal "
                         "measurement (0 = skip)")
    ap.add_argument("--twisted", type=int, default=16,
                    help="twisted-bilayer problems (5x5 base harmonics, n = 1250) for the extended-crystal measurement")
    ap.add_argument("--tc-product", type=int, default=0,
                    help="only time khp_zgemm_fp64_tc (FP64-accurate tensor-core product) on this many random "
                         "242 x 242 complex problems (kernel profiling)")
    ap.add_argument("--cpu-rate-only", type=int, default=0,
                    help="time the CPU oracle alone on this many in-cone sweep problems and print the seconds "
                         "(used in a child process whose BLAS threads are pinned)")
    ap.add_argument("--tf32-product", type=int, default=0,
                    help="only time khp_cgemm_tf32x3 (3xTF32 tensor-core complex product) on this many random "
                         "242 x 242 complex64 problems against torch's complex64 matmul (kernel profiling)")
    ap.add_argument("--graphs-check", type=int, default=1,
                    help="time the 5x5 sweep in small chunks with and without CUDA-graph replay (0 = skip)")
    ap.add_argument("--streams", type=int, default=2,
                    help="CUDA streams the chunks are dealt to in turn (chunk k on stream k mod S, each with its "
                         "own workspace), so that one chunk's stages run beside the next one's (1 = one stream)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="run only the warm-up and timed steps and print the line (for kernel profiling)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ------------------------------------------------------------------------------------------
# CPU oracle timing (reported baseline / reference arm)
# ------------------------------------------------------------------------------------------
def time_oracle(problems, st, wl, kp):
    from oracle import khepri_oracle as ko
    cl = ko.OracleCrystal(st.pw)
    for name, (kind, eps, depth) in st.layers.items():
        (cl.add_layer_uniform if kind == "uniform" else cl.add_layer_pixmap)(name, eps, depth)
    cl.set_device(st.stack, False)
    t0 = time.perf_counter()
    for p in problems:
        cl.set_source(wl[p], 1.0, 0.0, kp=tuple(kp[p]))
        cl.solve()
        cl.poynting_flux_end()
        cl.source.te, cl.source.tm = 0.0, 1.0
        cl.poynting_flux_end()
    return time.perf_counter() - t0


def cpu_sample(count):
    """The bench's seeded sample of in-cone 11x11 sweep problems for the CPU oracle."""
    from khepri_gb300 import workloads
    st = workloads.batched_structure(0)
    wl_all, kp_all = workloads.batched_problems()
    inside = np.flatnonzero(np.hypot(kp_all[:, 0], kp_all[:, 1]) < 2 * np.pi / wl_all)
    return np.random.default_rng(1).choice(inside, count, replace=False), st, wl_all, kp_all


def cpu_rate_one_thread(count):
    """Solves/s of the CPU oracle on the sample with one BLAS/OpenMP thread, timed in a child
    process (the thread count of numpy's BLAS is fixed when it loads)."""
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1", MKL_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-rate-only", str(count)], env=env,
                       capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return None
    return count / float(r.stdout.strip().splitlines()[-1])


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------------------------------
# Clock sampling during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------
# Reference arm
# ------------------------------------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from khepri_gb300 import workloads
    st = workloads.batched_structure(0)
    wl, kp = workloads.batched_problems()
    inside = np.flatnonzero(np.hypot(kp[:, 0], kp[:, 1]) < 2 * np.pi / wl)
    per_step = 2
    rng = np.random.default_rng(0)
    for _ in range(args.warmup):
        time_oracle(rng.choice(inside, per_step, replace=False), st, wl, kp)
    total = 0.0
    for _ in range(args.steps):
        total += time_oracle(rng.choice(inside, per_step, replace=False), st, wl, kp)
    value = per_step * args.steps / total
    cores = cpu_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded)",
        "config": {"workload": "batched sweep 11x11, 256x256 multi-disc map, [P,U,P,U,P], both polarisations",
                   "batch": per_step, "harmonics": "11x11", "parallelism": "host cores (numpy/LAPACK)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{per_step} in-cone (f, k) problems per step of the 11x11 sweep, CPU oracle"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def bench_grad(args, struct11, st11, wl_all, kp_all):
    """Solve + gradient through the public API (host inputs -> host R, T, per-order powers and
    pixmap gradients), host wall clock, after one untimed pass of the same call:
    (a) the 11x11 sweep structure, loss = sum of T (te) over one chunk of problems, gradient with
        respect to its 256x256 pixmap; (b) inverse design 9x9: designs x 16 frequencies, normal
        incidence, loss = mean over f of the zeroth-order T, gradient w.r.t. each design."""
    from khepri_gb300 import batch, workloads
    out = {}
    B = args.batch
    inside = np.flatnonzero(np.hypot(kp_all[:, 0], kp_all[:, 1]) < 2 * np.pi / wl_all)
    idx = np.sort(np.random.default_rng(4).choice(inside, B, replace=False))
    entries = [(st11.pw, st11.layers, st11.stack)]
    nh = st11.pw[0] * st11.pw[1]
    dT = np.ones((B, nh))

    def g11():
        return batch.solve_structures_grad(entries, wl_all[idx], kp_all[idx], which=np.zeros(B, int), dT=dT,
                                           chunk=B, strict=False)

    def s11():
        return batch.solve_structures(entries, wl_all[idx], kp_all[idx], which=np.zeros(B, int), chunk=B,
                                      strict=False)

    g11()
    _, tg = _timed(g11)
    s11()
    rep0 = dict(batch.STATS)
    _, ts = _timed(s11)
    out["sweep_11x11"] = {"solve_grad_per_s": B / tg, "solve_per_s_same_call_path": B / ts,
                          "repairs_in_timed_solve": {k: batch.STATS[k] - rep0[k] for k in batch.STATS},
                          "problems": B, "loss": "sum of T (te) over the chunk",
                          "wrt": "the 256x256 pixmap shared by the 3 patterned layers"}
    if args.grad_designs > 0:
        thetas, structs, freqs = workloads.inverse_design(args.grad_designs, seed=0)
        D, F = len(structs), len(freqs)
        ents = [(s.pw, s.layers, s.stack) for s in structs]
        which = np.repeat(np.arange(D), F)
        wl = np.tile(1.0 / freqs, D)
        kp = np.zeros((D * F, 2))
        nh9 = 81
        dT9 = np.zeros((D * F, nh9))
        dT9[:, (nh9 - 1) // 2] = 1.0 / F

        def g9():
            return batch.solve_structures_grad(ents, wl, kp, which=which, dT=dT9, chunk=1024, strict=False)

        def s9():
            return batch.solve_structures(ents, wl, kp, which=which, chunk=1024, strict=False)

        g9()
        res, tg9 = _timed(g9)
        s9()
        _, ts9 = _timed(s9)
        out["inverse_design_9x9"] = {"solve_grad_per_s": D * F / tg9, "solve_per_s_same_call_path": D * F / ts9,
                                     "problems": D * F, "designs": D, "frequencies": F,
                                     "problems_with_status": int((res[5] != 0).sum()),
                                     "loss": "mean over f of the zeroth-order T (te, normal incidence)",
                                     "wrt": "each design's 64x64 eps map (shared by its 2 patterned layers)"}
    return out


def bench_uneven(args):
    """Config 3's uneven batch: structures of 3x3..17x17 harmonics with 1-8 lossy smoothed 128x128
    layers, one problem each, through solve_structures (mixed; grouped by shape, chunks of the
    autotuned size), host wall clock; R, T and A = 1 - R - T against the CPU oracle on the first
    structure of every harmonic count."""
    from khepri_gb300 import batch, workloads
    from oracle import khepri_oracle as ko
    if args.uneven <= 0:
        return None
    sts = workloads.uneven_structures(args.uneven, seed=0)
    ents = [(s.pw, s.layers, s.stack) for s, _, _ in sts]
    wl = np.array([w for _, w, _ in sts])
    kp = np.array([k for _, _, k in sts])

    def run(sel):
        return batch.solve_structures([ents[i] for i in sel], wl[sel], kp[sel], te=1.0, tm=1.0, strict=False)

    run(np.arange(min(64, len(ents))))
    res, t = _timed(lambda: run(np.arange(len(ents))))
    R, T, st = res
    first = {}
    for i, (s, _, _) in enumerate(sts):
        first.setdefault(s.pw[0], i)
    errs = {"R": 0.0, "T": 0.0, "A": 0.0}
    t_cpu = time.perf_counter()
    for p_, i in sorted(first.items()):
        r0, t0 = ko.solve_rt(ents[i][0], ents[i][1], ents[i][2], wl[i], 1.0, 1.0, kp=tuple(kp[i]))
        errs["R"] = max(errs["R"], abs(R[i] - r0))
        errs["T"] = max(errs["T"], abs(T[i] - t0))
        errs["A"] = max(errs["A"], abs((1 - R[i] - T[i]) - (1 - r0 - t0)))
    t_cpu = time.perf_counter() - t_cpu
    return {"structures_per_s": len(ents) / t, "structures": len(ents), "seconds": t,
            "problems_with_status": int((st != 0).sum()),
            "sizes": "pw 3..17 odd, 1..8 layers of 128x128 maps; grouped by shape, autotuned chunks",
            "max_abs_err_vs_oracle": errs,
            "err_sample": f"the first structure of each of the {len(first)} harmonic counts, CPU oracle "
                          f"({t_cpu:.1f} s)"}


def bench_graphs(args):
    """Chunk solves replayed as CUDA graphs (one stream) against enqueued launch by launch on one
    and on two streams (batch.solve_rt: graphs=True; graphs=False with streams=1, 2), host wall
    clock through the public API: the 5x5 drop-in structure's 151 frequencies, eight times over,
    in chunks of 16 (small chunks, where launch overhead counts)."""
    if args.graphs_check <= 0:
        return None
    from khepri_gb300 import batch, workloads
    out = {}
    sw = workloads.plain_sweep()
    wl = np.tile(sw.wavelengths, 8)
    kp = np.tile(np.asarray(sw.kp).reshape(-1, 2), (8, 1))
    for name, g, ns in (("eager", False, 1), ("eager_2_streams", False, 2), ("graphs", True, 1)):
        batch.solve_rt((5, 5), sw.structure.layers, sw.structure.stack, wl[:64], kp[:64], chunk=16, method="mixed",
                       graphs=g, streams=ns)
        _, t = _timed(lambda: batch.solve_rt((5, 5), sw.structure.layers, sw.structure.stack, wl, kp, chunk=16,
                                             method="mixed", graphs=g, streams=ns))
        out.setdefault("plain_5x5_chunk16", {})[name] = len(wl) / t
    return out


def bench_twisted(args):
    """Twisted bilayers at 5x5 base harmonics (product expansion of 625 orders, n = 1250): a disc
    grating (eps 12 in 1, 128x128 map, depth 0.3) on each side of a gap (d 0.3), twist 13 deg,
    frequencies 0.4-0.7 at normal incidence, both polarisations; host wall clock through
    TwistedBilayer.solve_rt after one untimed problem."""
    from khepri_gb300 import twisted
    if args.twisted <= 0:
        return None
    x = np.linspace(-0.5, 0.5, 128)
    X, Y = np.meshgrid(x, x, indexing="ij")
    disc = np.where(X ** 2 + Y ** 2 < 0.3 ** 2, 12.0, 1.0)
    tw = twisted.TwistedBilayer((5, 5), "square", np.deg2rad(13.0), [("pixmap", disc, 0.3)],
                                [("uniform", 1.0, 0.3)], [("pixmap", disc, 0.3)])
    f = np.linspace(0.4, 0.7, args.twisted)
    tw.solve_rt(1.0 / f[:1], np.zeros((1, 2)), both_pols=True)
    res, t = _timed(lambda: tw.solve_rt(1.0 / f, np.zeros((len(f), 2)), both_pols=True, chunk=16, strict=False))
    R, T, st = res
    return {"solves_per_s": len(f) / t, "problems": len(f), "seconds": t, "n_extended": 1250,
            "max_abs_R_plus_T_minus_1": float(np.abs(R + T - 1).max()), "problems_with_status": int((st != 0).sum())}


def bench_twisted7(args):
    """Twisted bilayers at 7x7 base harmonics (product expansion of 2401 orders, n = 4802): disc
    gratings eps 12 in 1 (64x64 map, r 0.3, depth 0.3) on each side of a gap (d 0.3), twist 13
    deg, frequencies 0.4-0.7 at normal incidence, both polarisations; host wall clock through
    TwistedBilayer.solve_rt after one untimed problem."""
    from khepri_gb300 import twisted
    if args.twisted7 <= 0:
        return None
    x = np.linspace(-0.5, 0.5, 64)
    X, Y = np.meshgrid(x, x, indexing="ij")
    disc = np.where(X ** 2 + Y ** 2 < 0.3 ** 2, 12.0, 1.0)
    tw = twisted.TwistedBilayer((7, 7), "square", np.deg2rad(13.0), [("pixmap", disc, 0.3)],
                                [("uniform", 1.0, 0.3)], [("pixmap", disc, 0.3)])
    f = np.linspace(0.4, 0.7, args.twisted7)
    tw.solve_rt(1.0 / f[:1], np.zeros((1, 2)), both_pols=True)
    res, t = _timed(lambda: tw.solve_rt(1.0 / f, np.zeros((len(f), 2)), both_pols=True, chunk=4, strict=False))
    R, T, st = res
    return {"solves_per_s": len(f) / t, "problems": len(f), "seconds": t, "n_extended": 4802,
            "max_abs_R_plus_T_minus_1": float(np.abs(R + T - 1).max()), "problems_with_status": int((st != 0).sum())}


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    import __graft_entry__
    __graft_entry__.build()
    from khepri_gb300 import _capi, batch, engine, replicas, workloads

    lib = _capi.load()
    if args.eig_threads:
        _capi.check(lib.khp_tune(1, N_MAT, args.eig_threads), "khp_tune")
    if args.tf32_min_n >= 0:
        _capi.check(lib.khp_tune(2, 1, args.tf32_min_n), "khp_tune")
    if args.mode_digits:
        _capi.check(lib.khp_tune(3, 1, args.mode_digits), "khp_tune")
    st = workloads.batched_structure(0)
    wl_all, kp_all = workloads.batched_problems()
    P = wl_all.shape[0]
    B = args.batch
    struct = engine.StructureGPU(st.pw, engine.lattice_vectors("square"), dev)
    specs = batch._specs(st.layers, 1.0, 1.0)
    for name, sp in specs.items():
        if sp.kind == "pixmap":
            struct.prepare_map(sp.eps)  # per-structure preparation, outside the timed region

    def chunk(step):
        return replicas.chunk_indices(P, B, step, rank, world)

    nsteps = args.warmup + args.steps
    probs = [engine.Problems.make(wl_all[chunk(k)], kp_all[chunk(k)], 1.0, 0.0, dev) for k in range(nsteps)]
    statuses = [torch.zeros(B, dtype=torch.int32, device=dev) for _ in range(nsteps)]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > L2 (129 MB)

    plan = batch.StackPlan(struct, specs, st.stack)
    npat = int((plan.kinds == 1).sum())
    FLOPS_PER_CALL["khp_solve_batched"] = solve_batched_flops(N_MAT, plan.nmaps, npat, len(plan.kinds) - npat)
    FLOPS_PER_CALL["khp_solve_batched_mixed"] = solve_mixed_flops(N_MAT, plan.nmaps, npat, len(plan.kinds) - npat)
    prec = args.precision

    # chunk k on stream k mod S with workspace slot k mod max(2, S); its deferred repair (the flags
    # read, flagged problems re-solved) runs after the next max(1, S - 1) chunks are enqueued, so
    # the device never idles while the host looks at them, and before the next chunk that reuses
    # its stream and slot (the same schedule as batch.solve_rt)
    nstreams = max(1, args.streams)
    streams = [torch.cuda.Stream(dev) for _ in range(nstreams)] if nstreams > 1 else None
    nslots, lag = max(2, nstreams), max(1, nstreams - 1)

    def step(k, between=None):
        """Enqueue chunk k (after ``between``, on the chunk's stream); returns its deferred repair."""
        s = streams[k % nstreams] if streams else torch.cuda.current_stream(dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(s):
            if between is not None:
                between()
            out = batch.solve_chunk_gamma_both_pols(struct, plan, probs[k], statuses[k], precision=prec,
                                                    refine=args.refine, ws_slot=k % nslots,
                                                    defer_repair=prec == "mixed")
        fix = out[2] if prec == "mixed" else (lambda: None)

        def on_stream():
            with torch.cuda.stream(s):
                fix()
        return on_stream

    def run_steps(ks, between=None):
        pending = []
        for k in ks:
            pending.append(step(k, between))
            while len(pending) > lag:
                pending.pop(0)()
        while pending:
            pending.pop(0)()
        for s in streams or ():
            torch.cuda.current_stream(dev).wait_stream(s)

    run_steps(range(args.warmup))
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    _capi.check(lib.khp_stage_timing(1), "khp_stage_timing")
    launches0 = lib.khp_launch_count()
    repairs0 = dict(batch.STATS)
    with ClockSampler(local) as clocks:
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        run_steps(range(args.warmup, nsteps), between=flush.zero_)
        e1.record()
        torch.cuda.synchronize()
        barrier()
    launches = lib.khp_launch_count() - launches0
    stage_ms = _capi.stage_times()
    lib.khp_stage_timing(0)
    repairs = {k: batch.STATS[k] - repairs0[k] for k in batch.STATS}
    ms = e0.elapsed_time(e1)
    ms = replicas.max_over_ranks(ms, dev)
    value = world * B * args.steps / (ms * 1e-3)
    bad = int(sum(int((s != 0).sum().item()) for s in statuses))
    if args.kernels_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": ms / args.steps, "kernels_only": True,
                              "config": {"batch": B, "problems_with_status": bad}}), flush=True)
        return

    # roofline of the dominant kernels: the FP32 eigensolver of the modes stage (k_gehrd +
    # k_geev_schur + k_hqr_apply_log, ~31 % of the step in the launch list), timed live by the
    # library's stage events
    scratch = torch.empty(2048 * 1024, dtype=torch.float64, device=dev)
    fp64_peak = lib.khp_probe_fp64_tflops(_capi.ptr(scratch), scratch.numel(), _capi.stream_ptr())
    fp32_peak = lib.khp_probe_fp32_tflops(_capi.ptr(scratch), 2 * scratch.numel(), _capi.stream_ptr())
    roof = None
    eig_ms, eig_calls = stage_ms["eigensolve"]
    if prec == "mixed" and eig_calls > 0:
        mats = B * plan.nmaps  # modes matrices per call (one per problem and distinct map)
        eig_flops = 100.0 * N_MAT ** 3 * mats  # convention: complex eig with vectors = 100 n^3
        achieved = eig_flops / (eig_ms / eig_calls * 1e-3) / 1e12
        stages = {k: {"ms_per_call": v[0] / args.steps, "share": round(v[0] / ms, 4)}
                  for k, v in stage_ms.items() if v[1] > 0}
        roof = {"bound": "fp32", "kernel": "k_gehrd<float> + k_geev_schur<float> + k_hqr_apply_log<float> (eigensolve "
                         "stage of khp_solve_batched_mixed)",
                "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak if fp32_peak > 0 else None,
                "traffic": GEEV_TRAFFIC_PER_MATRIX * mats if GEEV_TRAFFIC_PER_MATRIX else None,
                "traffic_source": "DRAM read + write per matrix from one ncu capture at 912 matrices per launch "
                                  "(128-thread teams), scaled by the matrices of this launch",
                "peak_source": "FP32 FMA pipe measured in this run (khp_probe_fp32_tflops); MEASURED_PEAKS.json "
                               "lists only HBM and bf16",
                "note": "latency-bound (one CTA per matrix; barriers and dependent loads inside each QR "
                        "window), not pipe-bound; with chunks on %d streams a stage's events span the share of "
                        "the SMs the other stream's kernels take meanwhile, so stage times overlap" % nstreams,
                "flops_per_launch": eig_flops, "launch_ms": eig_ms / eig_calls, "stages": stages,
                "fp64_peak_tflops": fp64_peak}
        tc_ms, tc_calls = stage_ms["tc_product"]
        if tc_calls > 0:
            tc_flops = mats * TC_FLOPS_PER_MATRIX
            tc_rate = tc_flops / (tc_ms / args.steps * 1e-3) / 1e12
            roof["tensor_stage"] = {
                "bound": "tensor", "kernel": "k_tc_digits (FP64-accurate products M W, C W: tcgen05 bf16 digit products in TMEM)",
                "achieved": tc_rate, "peak": BF16_PEAK, "unit": "TFLOP/s", "frac": tc_rate / BF16_PEAK,
                "flops": "bf16 flops issued: 36 digit pairs x 2 Mp N2p K2p per product (rows padded to 128, columns and inner index to 64)",
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)",
                "fp64_equivalent_tflops": mats * 20.0 * N_MAT ** 3 / (tc_ms / args.steps * 1e-3) / 1e12}

    # error of the timed path against the FP64 recursion on the first timed chunk (untimed)
    err = None
    fp64_rate = None
    if prec == "mixed":
        inside = np.flatnonzero(np.hypot(kp_all[:, 0], kp_all[:, 1]) < 2 * np.pi / wl_all)
        sel = np.sort(np.random.default_rng(2).choice(inside, B, replace=False))
        pchk = engine.Problems.make(wl_all[sel], kp_all[sel], 1.0, 0.0, dev)
        st_a = torch.zeros(B, dtype=torch.int32, device=dev)
        st_b = torch.zeros(B, dtype=torch.int32, device=dev)
        Rm, Tm = batch.solve_chunk_gamma_both_pols(struct, plan, pchk, st_a, precision="mixed", refine=args.refine)
        torch.cuda.synchronize()
        e2 = torch.cuda.Event(enable_timing=True)
        e3 = torch.cuda.Event(enable_timing=True)
        e2.record()
        R64, T64 = batch.solve_chunk_gamma_both_pols(struct, plan, pchk, st_b, precision="fp64")
        e3.record()
        torch.cuda.synchronize()
        fp64_rate = B / (e2.elapsed_time(e3) * 1e-3)
        err = max((Rm - R64).abs().max().item(), (Tm - T64).abs().max().item())

    # the plain drop-in path: one Crystal.solve + poynting_flux_end per call (FP64 chain)
    plain_rate = None
    if rank == 0 and args.plain > 0:
        from khepri_gb300 import Crystal
        cl = Crystal(st.pw, device=dev)
        for name, (kind, eps, depth) in st.layers.items():
            (cl.add_layer_uniform if kind == "uniform" else cl.add_layer_pixmap)(name, eps, depth)
        cl.set_device(st.stack, False)
        idx = chunk(args.warmup)[: args.plain + 1]
        cl.set_source(wl_all[idx[0]], 1.0, 0.0, kp=tuple(kp_all[idx[0]]))
        cl.solve()
        cl.poynting_flux_end()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for p_ in idx[1:]:
            cl.set_source(wl_all[p_], 1.0, 0.0, kp=tuple(kp_all[p_]))
            cl.solve()
            cl.poynting_flux_end()
        torch.cuda.synchronize()
        plain_rate = args.plain / (time.perf_counter() - t0)

    # end to end through the public API: host numpy inputs -> host R, T, over exactly the chunks of
    # the timed region (one solve_rt call; it pipelines the chunks as the timed loop does)
    e2e_idx = np.concatenate([chunk(k) for k in range(args.warmup, nsteps)])
    torch.cuda.synchronize()
    barrier()
    rep_e0 = dict(batch.STATS)
    t0 = time.perf_counter()
    batch.solve_rt(st.pw, st.layers, st.stack, wl_all[e2e_idx], kp_all[e2e_idx], chunk=B, struct=struct,
                   strict=False, both_pols=True, method="mixed" if prec == "mixed" else "gamma", refine=args.refine,
                   streams=nstreams)
    torch.cuda.synchronize()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_repairs = {k: batch.STATS[k] - rep_e0[k] for k in batch.STATS}
    h2d = B * (8 + 32 + 16 + 16)  # k0, kp, te, tm per problem
    d2h = B * (2 * 2 * 8 + 4)      # R, T for two polarisations, status

    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        sample, _, _, _ = cpu_sample(args.cpu_sample)
        t_cpu = time_oracle(sample, st, wl_all, kp_all)
        one = cpu_rate_one_thread(args.cpu_sample)
        cpu = {"value": args.cpu_sample / t_cpu, "unit": UNIT, "cores": cpu_threads(), "kind": "port",
               "sample": f"{args.cpu_sample} in-cone problems of the 11x11 sweep, both polarisations, CPU oracle "
                         f"(numpy/LAPACK), {t_cpu:.1f} s",
               "one_thread": {"value": one, "unit": UNIT, "cores": 1,
                              "sample": "the same problems, BLAS and OpenMP pinned to one thread"}}

    grad_info = uneven_info = twisted_info = twisted7_info = graphs_info = None
    if rank == 0:
        graphs_info = bench_graphs(args)
        grad_info = bench_grad(args, struct, st, wl_all, kp_all)
        uneven_info = bench_uneven(args)
        twisted_info = bench_twisted(args)
        twisted7_info = bench_twisted7(args)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)",
            "config": {"workload": "batched sweep 11x11 (n=242), 256x256 multi-disc map, [P,U,P,U,P], 64 f x "
                                   "32x32 k, both polarisations per S-matrix",
                       "batch": B, "harmonics": "11x11", "eig_threads": args.eig_threads or 256,
                       "recursion_products": ("3xTF32 tensor cores" if (args.tf32_min_n < 0 and N_MAT >= 128)
                                              or 0 < args.tf32_min_n <= N_MAT else "FP32 pipe"),
                       "precision": ("mixed: FP32 O(n^3) work, FP64 eigen-refinement and %d rounds of FP64 "
                                     "iterative refinement" % args.refine) if prec == "mixed"
                       else "fp64 (complex128) throughout",
                       "max_abs_err_vs_fp64": err,
                       "err_sample": "R and T, both polarisations, of %d random in-cone problems of the sweep, "
                                     "mixed vs the FP64 recursion" % B,
                       "fp64_recursion_solves_per_s": fp64_rate,
                       "plain_dropin_gpu_solves_per_s": plain_rate,
                       "method": "reflection-matrix recursion (khp_solve_batched%s), one eigensolve per problem"
                                 % ("_mixed" if prec == "mixed" else ""),
                       "l2": "256 MB buffer written between steps (> 129 MB L2)",
                       "parallelism": f"replicas x{world}", "streams": nstreams,
                       "problems_with_status": bad,
                       "repairs": repairs,
                       "solve_grad": grad_info, "uneven": uneven_info, "twisted_5x5": twisted_info,
                       "twisted_7x7": twisted7_info, "graphs": graphs_info},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": world * len(e2e_idx) / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.steps, "repairs": e2e_repairs,
                    "path": "batch.solve_rt, host numpy in (pinned staging) -> host R, T, status out"},
            "gpu_launches": int(launches), "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_tc_product(args):
    """Times the FP64-accurate tensor-core product alone: C = A B for args.tc_product random
    complex 242 x 242 pairs, against torch's FP64 matmul for the error."""
    import torch

    import __graft_entry__
    __graft_entry__.build()
    from khepri_gb300 import _capi
    lib = _capi.load()
    b, n = args.tc_product, N_MAT
    g = torch.Generator(device="cpu").manual_seed(3)
    A = torch.randn(b, n, n, generator=g, dtype=torch.complex128).cuda()
    Bm = torch.randn(b, n, n, generator=g, dtype=torch.complex128).cuda()
    C = torch.empty_like(A)
    ws = torch.empty(lib.khp_zgemm_fp64_tc_workspace(b, n, n, n), dtype=torch.uint8, device="cuda")

    def call():
        _capi.check(lib.khp_zgemm_fp64_tc(b, n, n, n, _capi.ptr(A), n, n * n, _capi.ptr(Bm), n, n * n, _capi.ptr(C), n,
                                          n * n, _capi.ptr(ws), ws.numel(), _capi.stream_ptr()), "khp_zgemm_fp64_tc")

    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        call()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ref = A @ Bm
    rel = ((C - ref).abs().max() / ref.abs().max()).item()
    print(json.dumps({"metric": "FP64-accurate complex products (242^3) per second", "value": b / (ms * 1e-3),
                      "unit": "products/s", "ms_per_call": ms, "problems": b, "steps": args.steps,
                      "warmup": args.warmup, "fp64_equivalent_tflops": 8.0 * n ** 3 * b / (ms * 1e-3) / 1e12,
                      "max_rel_err_vs_torch_fp64": rel}), flush=True)


def run_tf32_product(args):
    """Times the 3xTF32 product alone: C = A B for args.tf32_product random complex64 242 x 242
    pairs (split and product together), against torch's complex64 matmul, with the error of both
    against an FP64 product."""
    import torch

    import __graft_entry__
    __graft_entry__.build()
    from khepri_gb300 import _capi
    lib = _capi.load()
    b, n = args.tf32_product, N_MAT
    g = torch.Generator(device="cpu").manual_seed(3)
    A = torch.randn(b, n, n, generator=g, dtype=torch.complex64).cuda()
    Bm = torch.randn(b, n, n, generator=g, dtype=torch.complex64).cuda()
    C = torch.empty_like(A)
    ws = torch.empty(lib.khp_cgemm_tf32x3_workspace(b, n, n, n), dtype=torch.uint8, device="cuda")

    def call():
        _capi.check(lib.khp_cgemm_tf32x3(b, n, n, n, _capi.ptr(A), n, n * n, _capi.ptr(Bm), n, n * n, _capi.ptr(C), n,
                                         n * n, _capi.ptr(ws), ws.numel(), _capi.stream_ptr()), "khp_cgemm_tf32x3")

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms = timed(call)
    ms_ref = timed(lambda: torch.matmul(A, Bm))
    ref = A.to(torch.complex128) @ Bm.to(torch.complex128)
    scale = ref.abs().max().item()
    err = ((C.to(torch.complex128) - ref).abs().max() / scale).item()
    err_ref = (((A @ Bm).to(torch.complex128) - ref).abs().max() / scale).item()
    print(json.dumps({"metric": "FP32-accurate complex products (242^3) per second", "value": b / (ms * 1e-3),
                      "unit": "products/s", "ms_per_call": ms, "problems": b, "steps": args.steps,
                      "warmup": args.warmup, "fp32_equivalent_tflops": 8.0 * n ** 3 * b / (ms * 1e-3) / 1e12,
                      "max_rel_err_vs_fp64": err, "torch_complex64_ms": ms_ref,
                      "torch_complex64_tflops": 8.0 * n ** 3 * b / (ms_ref * 1e-3) / 1e12,
                      "torch_complex64_max_rel_err": err_ref}), flush=True)


def main():
    args = parse()
    if args.cpu_rate_only > 0:
        sample, st, wl_all, kp_all = cpu_sample(args.cpu_rate_only)
        print(time_oracle(sample, st, wl_all, kp_all), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    elif args.tc_product > 0:
        run_tc_product(args)
    elif args.tf32_product > 0:
        run_tf32_product(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
