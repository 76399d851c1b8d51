"""Chunks of batch.solve_rt dealt to several CUDA streams (chunk c on stream c mod S, each stream
with its own workspaces, deferred re-solves on the chunk's own stream): the same R, T and status
as one stream, for the mixed and FP64 recursions, including chunks whose flagged problems are
re-solved."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RT_TOL = 1e-6


@pytest.mark.parametrize("method", ["mixed", "gamma"])
def test_streams_match_one_stream(khp, golden, method):
    from khepri_gb300 import batch, workloads
    g = golden("plain_5x5")
    sw = workloads.plain_sweep()
    args = ((5, 5), sw.structure.layers, sw.structure.stack, sw.wavelengths, sw.kp, 1.0, 0.0)
    R1, T1, s1 = batch.solve_rt(*args, chunk=24, method=method, streams=1)
    assert max(np.abs(R1 - g["R"]).max(), np.abs(T1 - g["T"]).max()) < RT_TOL
    for S in (2, 3):
        R, T, s = batch.solve_rt(*args, chunk=24, method=method, streams=S)
        assert np.array_equal(s, s1) and not s.any()
        assert np.abs(R - R1).max() < 1e-12 and np.abs(T - T1).max() < 1e-12


def test_streams_with_deferred_resolves(khp):
    """Three-problem chunks of sweep problems next to a Wood anomaly and a close conjugate pair
    (the mixed path flags and re-solves some of them): every stream count gives the results of
    one stream, with every status clear and the re-solves counted."""
    from khepri_gb300 import batch, workloads
    st = workloads.batched_structure(0)
    wl, kp = workloads.batched_problems()
    inside = np.flatnonzero(np.hypot(kp[:, 0], kp[:, 1]) < 2 * np.pi / wl)
    idx = np.concatenate([[50517, 38308, 47259, 1400, 4469, 7987], inside[inside > 20000][:3]])
    args = (st.pw, st.layers, st.stack, wl[idx], kp[idx])
    results = {}
    for S in (1, 2, 3):
        before = dict(batch.STATS)
        R, T, s = batch.solve_rt(*args, chunk=3, both_pols=True, method="mixed", streams=S)
        resolved = sum(batch.STATS[k] - before[k] for k in ("refine_repairs", "fp64_repairs"))
        assert not s.any()
        results[S] = (R, T, resolved)
    R1, T1, n1 = results[1]
    print("re-solved per run:", n1)
    for S in (2, 3):
        R, T, n = results[S]
        assert n == n1
        assert np.abs(R - R1).max() < 1e-12 and np.abs(T - T1).max() < 1e-12


def test_repeated_calls_reuse_stream_workspaces(khp):
    """solve_structures and solve_rt take their side streams from one persistent set, so calling
    them again adds no workspace (engine.workspace keys its buffers by stream)."""
    from khepri_gb300 import batch, engine, workloads
    structs = workloads.uneven_structures(12, seed=3, n_pix=32, max_pw=5, max_layers=2)
    entries = [(st.pw, st.layers, st.stack) for st, _, _ in structs]
    wl = np.array([w for _, w, _ in structs])
    kp = np.array([k for _, _, k in structs])
    sw = workloads.plain_sweep(nfreq=40)
    rt_args = ((5, 5), sw.structure.layers, sw.structure.stack, sw.wavelengths, sw.kp)
    first = None
    for _ in range(3):
        R, T, s = batch.solve_structures(entries, wl, kp, chunk=4, streams=4, strict=False)
        R2, T2, s2 = batch.solve_rt(*rt_args, chunk=8, method="mixed", streams=2)
        assert not s2.any()
        if first is None:
            first = (len(engine._WS), R, T, R2, T2)
        else:
            assert len(engine._WS) == first[0]
            assert np.array_equal(R, first[1], equal_nan=True) and np.array_equal(T, first[2], equal_nan=True)
            assert np.array_equal(R2, first[3]) and np.array_equal(T2, first[4])
