"""CUDA-graph replay of the batched recursion's chunk solve (batch.ChunkGraph via
batch.solve_rt(graphs=True)): the same R, T and status as launching every kernel, for the mixed
and FP64 paths and both polarisations, and the graphs are really replayed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RT_TOL = 1e-6


@pytest.mark.parametrize("method", ["mixed", "gamma"])
def test_graph_replay_matches_eager(khp, golden, method, monkeypatch):
    from khepri_gb300 import batch, workloads
    g = golden("plain_5x5")
    sw = workloads.plain_sweep()
    replays = []
    real_replay = batch.ChunkGraph.replay

    def counting_replay(self, prob):
        replays.append(self.B)
        return real_replay(self, prob)

    monkeypatch.setattr(batch.ChunkGraph, "replay", counting_replay)
    args = ((5, 5), sw.structure.layers, sw.structure.stack, sw.wavelengths, sw.kp, 1.0, 0.0)
    # 151 problems in chunks of 24: chunk 0 eager, chunks 1 and 2 capture a graph each (their
    # results from the eager call before the capture), chunks 3-5 replay, the short last chunk eager
    R0, T0, s0 = batch.solve_rt(*args, chunk=24, method=method)
    R1, T1, s1 = batch.solve_rt(*args, chunk=24, method=method, graphs=True)
    assert replays == [24, 24, 24]
    assert not s1.any() and np.array_equal(s0, s1)
    assert np.abs(R1 - R0).max() < 1e-12 and np.abs(T1 - T0).max() < 1e-12
    assert max(np.abs(R1 - g["R"]).max(), np.abs(T1 - g["T"]).max()) < RT_TOL


def test_graph_replay_both_polarisations(khp):
    from khepri_gb300 import batch, workloads
    st = workloads.batched_structure(0, pw=(5, 5), n_pix=64)
    wl, kp = workloads.batched_problems(nfreq=8, nk=8)
    sel = np.arange(0, 512, 8)
    args = (st.pw, st.layers, st.stack, wl[sel], kp[sel])
    R0, T0, s0 = batch.solve_rt(*args, chunk=16, method="mixed", both_pols=True, strict=False)
    R1, T1, s1 = batch.solve_rt(*args, chunk=16, method="mixed", both_pols=True, strict=False, graphs=True)
    assert R1.shape == (64, 2)
    assert np.array_equal(s0, s1)
    ok = np.isfinite(R0)
    assert np.abs(R1[ok] - R0[ok]).max() < 1e-12 and np.abs(T1[ok] - T0[ok]).max() < 1e-12
