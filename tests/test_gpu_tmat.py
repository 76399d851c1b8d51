"""tmat formulation on the GPU (khepri_gb300.tmat, khp_tmat_*) against the reference's own
MATLAB fixtures (test/integration/fixtures/pair_pw, via tests/golden/tmat.npz, with the
tolerances of test/integration/test_pair_pw.py:103-131) and against the reference run on a
5x5 oblique two-island case, plus multS / matrix_s against the oracle."""
import numpy as np
import pytest

from oracle import khepri_oracle as ko
from pins import check_pinned

pytestmark = pytest.mark.gpu


def test_pair_pw_matlab_fixtures(khp, golden):
    from khepri_gb300 import tmat
    g = golden("tmat")
    pw, a, wl, kp, depth, sp = (8, 8), tmat.nanometers(100), tmat.nanometers(200), (0, 0), 1e-7, 3
    lat = tmat.CartesianLattice(pw, a1=(a, 0.0), a2=(0.0, a), eps_emerg=1.0, eps_incid=1.0, dtype=np.float64)
    assert np.allclose(lat.gx, g["mat_gx"]) and np.allclose(lat.Gy, g["mat_Gy"])
    bf = tmat.transform("disc", [0.5 * a, 0.5 * a, 0.2 * a], lat.Gx, lat.Gy, lat.area)
    assert np.allclose(bf, g["mat_Omega_g"])
    check_pinned(g, "mat_U_in", lat.U(wl, kp), 1, rtol=1e-7)
    check_pinned(g, "mat_V_in", lat.Vi(wl, kp), 1, rtol=1e-7)
    S, A, E, T = tmat.scattering_matrices(pw, lat, [(bf, 8.9)], 1.0, [wl], [kp], depth, sp, intermediates=True)
    check_pinned(g, "mat_A", A[0].cpu().numpy(), 1, rtol=1e-7)
    check_pinned(g, "mat_T_xyz", E[0].cpu().numpy(), 1, rtol=1e-7, atol=1e-10)
    check_pinned(g, "mat_Tslice", T[0].cpu().numpy(), 1, rtol=1e-7, atol=4e-10)
    check_pinned(g, "mat_Sslice", S[0].cpu().numpy(), 1, rtol=1e-7, atol=1e-11)
    Si = tmat.scattering_interface(lat, wl, kp).numpy()
    check_pinned(g, "mat_S_interface", Si, 1, rtol=1e-7, atol=1e-12)


def test_reference_5x5_oblique_two_islands(khp, golden):
    from khepri_gb300 import tmat
    g = golden("tmat")
    pw = tuple(int(v) for v in g["ref_pw"])
    a, wl, kp = float(g["ref_a"]), float(g["ref_wl"]), tuple(g["ref_kp"])
    depth, sp = float(g["ref_depth"]), int(g["ref_slicing"])
    lat = tmat.CartesianLattice(pw, a1=(a, 0.0), a2=(0.0, a), eps_emerg=float(g["ref_eps_emerg"]),
                                eps_incid=float(g["ref_eps_incid"]), dtype=np.float64)
    isl = [(tmat.transform("disc", [0.3 * a, 0.45 * a, 0.22 * a], lat.Gx, lat.Gy, lat.area), 6.0),
           (tmat.transform("rectangle", [0.6 * a, 0.1 * a, 0.9 * a, 0.35 * a], lat.Gx, lat.Gy, lat.area), 3.0 + 0.1j)]
    _, q = tmat.grid_size(pw)
    assert np.allclose(tmat.epsilon_g(q, isl, 1.5), g["ref_epsg"], rtol=1e-13, atol=1e-15)
    # a batch of three problems: the fixture's and two others (each checked where pinned)
    S, A, E, T = tmat.scattering_matrices(pw, lat, isl, 1.5, [wl, wl * 1.1, wl], [kp, (0.0, 0.0), kp], depth, sp,
                                          intermediates=True)
    # the exponential is a different scaling-and-squaring variant from scipy's: entries agree to
    # ~1e-11 of the matrix's largest entry
    def scale(name):
        return np.abs(g[f"{name}_val"]).max()

    for b in (0, 2):
        check_pinned(g, "ref_A", A[b].cpu().numpy(), 2, rtol=1e-12)
        check_pinned(g, "ref_E", E[b].cpu().numpy(), 2, rtol=1e-9, atol=1e-11 * scale("ref_E"))
        check_pinned(g, "ref_T", T[b].cpu().numpy(), 2, rtol=1e-9, atol=1e-11 * scale("ref_T"))
        check_pinned(g, "ref_S", S[b].cpu().numpy(), 2, rtol=1e-8, atol=1e-10 * scale("ref_S"))
    # the second problem against the oracle
    A1 = ko.tmat_matrix_a(pw, lat.gx, lat.gy, tmat.epsilon_g(q, isl, 1.5), tmat.epsilon_g(q, isl, 1.5, True),
                          wl * 1.1, (0.0, 0.0))
    U, Vi, _ = ko.tmat_uv(ko.tmat_lattice(pw, (a, 0.0), (0.0, a)), wl * 1.1, (0.0, 0.0), 1.0, 2.25)
    S1, E1 = ko.tmat_layer_smatrix(A1, U, Vi, depth, sp)
    assert np.abs(A[1].cpu().numpy() - A1).max() <= 1e-12 * np.abs(A1).max()
    assert np.abs(S[1].cpu().numpy() - S1).max() <= 1e-8 * max(1.0, np.abs(S1).max())


def test_multS_and_matrix_s_match_oracle(khp):
    from khepri_gb300 import tmat
    rng = np.random.default_rng(3)
    ng, B = 9, 4
    N = 4 * ng
    S1 = (rng.standard_normal((B, N, N)) + 1j * rng.standard_normal((B, N, N))) * 0.3 / np.sqrt(N)
    S2 = (rng.standard_normal((B, N, N)) + 1j * rng.standard_normal((B, N, N))) * 0.3 / np.sqrt(N)
    out = tmat.multS(S1, S2)
    for b in range(B):
        ref = ko.tmat_multS(S1[b], S2[b])
        assert np.abs(out[b] - ref).max() < 1e-12 * np.abs(ref).max()
    T = np.eye(N) + (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.2 / np.sqrt(N)
    assert np.abs(tmat.matrix_s(T) - ko.tmat_matrix_s(T)).max() < 1e-12 * np.abs(ko.tmat_matrix_s(T)).max()
    L = tmat.LayerMatrix(S1[0]) @ tmat.LayerMatrix(S2[0])
    assert np.abs(L.numpy() - ko.tmat_multS(S1[0], S2[0])).max() < 1e-12
