"""Pin the CPU oracle to golden vectors made by running the reference on the same inputs."""
import numpy as np
import pytest

from oracle import khepri_oracle as ko
from khepri_gb300 import workloads as wk


def _solve(pw, layers, stack, wl, te, tm, theta=0.0, phi=0.0, kp=None, lattice="square", epsi=1, epse=1,
           only_total=True):
    return ko.solve_rt(pw, layers, stack, wl, te, tm, theta, phi, kp, lattice, epsi, epse, only_total)


def test_fresnel_film_known_answer(golden):
    """The reference's own known-answer test (test/integration/test_complex_eps.py:13-42)."""
    g = golden("fresnel_1x1")
    R = []
    for wl, eps in zip(g["wavelength"], g["eps"]):
        r, t = _solve((1, 1), {"1": ("uniform", eps, float(g["depth"]))}, ["1"], wl, 1, 1)
        R.append(r)
    R = np.array(R)
    np.testing.assert_allclose(R, g["R"], rtol=1e-10, atol=1e-13)
    wls = g["wavelength"]
    eps_c = np.conj(g["eps"])
    n2 = np.conj(np.sqrt(eps_c))
    r12 = (1 - n2) / (1 + n2)
    r23 = (n2 - 1) / (n2 + 1)
    ph = np.exp(-2j * 2 * np.pi / wls * n2 * float(g["depth"]))
    fres = np.abs((r12 + r23 * ph) / (1 + r12 * r23 * ph)) ** 2
    np.testing.assert_allclose(R, fres, rtol=1e-7)


def test_convolution_matrix(golden):
    g = golden("convmat")
    C = ko.convolution_matrix(g["eps_map"], tuple(g["pw"]))
    np.testing.assert_allclose(C, g["C"], rtol=0, atol=1e-14)


def test_plain_sweep_rt(golden):
    g = golden("plain_5x5")
    sw = wk.plain_sweep()
    cl = ko.OracleCrystal((5, 5))
    for name, (kind, eps, depth) in sw.structure.layers.items():
        (cl.add_layer_uniform if kind == "uniform" else cl.add_layer_pixmap)(name, eps, depth)
    cl.set_device(sw.structure.stack, [True] * 3)
    idx = np.arange(0, 151, 10)
    for i in idx:
        cl.set_source(sw.wavelengths[i], 1.0, 0, 0.0, 0.0)
        cl.solve()
        r, t = cl.poynting_flux_end()
        assert abs(r - g["R"][i]) < 1e-10 and abs(t - g["T"][i]) < 1e-10
        if i == 0:
            np.testing.assert_allclose(cl.Stot, g["stot_0"], atol=1e-10)
    np.testing.assert_allclose(g["R"] + g["T"], 1.0, atol=1e-10)


def test_plain_layer_smatrices(golden):
    g = golden("plain_5x5")
    sw = wk.plain_sweep()
    cl = ko.OracleCrystal((5, 5))
    for name, (kind, eps, depth) in sw.structure.layers.items():
        (cl.add_layer_uniform if kind == "uniform" else cl.add_layer_pixmap)(name, eps, depth)
    cl.set_device(sw.structure.stack, [True] * 3)
    cl.set_source(sw.wavelengths[75], 1.0, 0, 0.0, 0.0)
    cl.solve()
    np.testing.assert_allclose(cl.layers["Scyl"].S, g["s_cyl_75"], atol=1e-10)
    np.testing.assert_allclose(cl.layers["S1"].S, g["s_uniform_75"], atol=1e-12)
    np.testing.assert_allclose(cl.layers["Sref"].S, g["s_ref_75"], atol=1e-12)
    np.testing.assert_allclose(cl.layers["Strans"].S, g["s_trn_75"], atol=1e-12)
    np.testing.assert_allclose(np.sort_complex(cl.layers["Scyl"].L), np.sort_complex(g["lam_cyl_75"]), atol=1e-10)
    np.testing.assert_allclose(cl.Stot, g["stot_75"], atol=1e-10)


def test_fields(golden):
    g = golden("fields_5x5")
    sw = wk.plain_sweep()
    cl = ko.OracleCrystal((5, 5))
    for name, (kind, eps, depth) in sw.structure.layers.items():
        (cl.add_layer_uniform if kind == "uniform" else cl.add_layer_pixmap)(name, eps, depth)
    cl.set_device(sw.structure.stack, [True] * 3)
    cl.set_source(float(g["wavelength"]), 1.0, 0.0, 0, 0)
    cl.solve()
    E, H = cl.fields_volume(g["x"], g["y"], g["z"])
    scale = np.abs(g["E"]).max()
    np.testing.assert_allclose(E, g["E"], atol=1e-9 * scale)
    np.testing.assert_allclose(H, g["H"], atol=1e-9 * np.abs(g["H"]).max())


def test_oblique_orders(golden):
    g = golden("oblique_5x5")
    emap, d, eu = g["eps_map"], g["depths"], g["eps_u"]
    layers = {"P1": ("pixmap", emap, d[0]), "U1": ("uniform", eu[0], d[1]), "P2": ("pixmap", emap, d[2]),
              "U2": ("uniform", eu[1], d[3]), "P3": ("pixmap", emap, d[4])}
    stack = ["P1", "U1", "P2", "U2", "P3"]
    for i in range(len(g["R"])):
        (r, ro), (t, to) = _solve((5, 5), layers, stack, g["wavelength"][i], g["te"][i], g["tm"][i],
                                  g["theta"][i], g["phi"][i], epsi=g["epsi"][i], epse=g["epse"][i],
                                  only_total=False)
        assert abs(r - g["R"][i]) < 1e-10 and abs(t - g["T"][i]) < 1e-10
        np.testing.assert_allclose(ro, g["r_orders"][i], atol=1e-10)
        np.testing.assert_allclose(to, g["t_orders"][i], atol=1e-10)


def test_hexagonal(golden):
    g = golden("hex_3x3")
    for i in range(len(g["R"])):
        r, t = _solve((3, 3), {"H": ("pixmap", g["eps_map"], 0.4)}, ["H"], g["wavelength"][i], 1.0, 1.0,
                      kp=tuple(g["kp"][i]), lattice="hexagonal")
        assert abs(r - g["R"][i]) < 1e-10 and abs(t - g["T"][i]) < 1e-10


def test_uneven_lossy(golden):
    g = golden("uneven_small")
    structs = wk.uneven_structures(int(g["count"]), seed=int(g["seed"]), n_pix=int(g["n_pix"]),
                                   max_pw=int(g["max_pw"]), max_layers=int(g["max_layers"]))
    for i, (st, wl, kp) in enumerate(structs):
        r, t = _solve(st.pw, st.layers, st.stack, wl, 1.0, 1.0, kp=tuple(kp))
        assert abs(r - g["R"][i]) < 1e-9 and abs(t - g["T"][i]) < 1e-9
        assert r + t < 1.0  # lossy: Im eps < 0


def test_inverse_design_zeroth_order(golden):
    g = golden("design_9x9")
    _, structs, freqs = wk.inverse_design(int(g["count"]), seed=int(g["seed"]))
    k = 0
    for st in structs:
        for f in freqs[[0, 7, 15]]:
            (r, _), (t, to) = _solve(st.pw, st.layers, st.stack, 1.0 / f, 1.0, 0.0, only_total=False)
            assert abs(f - g["freq"][k]) < 1e-15
            assert abs(r - g["R"][k]) < 1e-9 and abs(t - g["T"][k]) < 1e-9
            assert abs(to[40] - g["t0"][k]) < 1e-9
            k += 1


@pytest.mark.slow
def test_batched_11x11_points(golden):
    g = golden("batched_11x11")
    st = wk.batched_structure(int(g["seed"]))
    assert abs(st.layers["P1"][1].sum() - float(g["map_sum"])) == 0
    wl, kp = wk.batched_problems()
    for j, p in enumerate(g["problems"][:2]):
        r, t = _solve(st.pw, st.layers, st.stack, wl[p], 1.0, 0.0, kp=tuple(kp[p]))
        assert abs(r - g["R_te"][j]) < 1e-9 and abs(t - g["T_te"][j]) < 1e-9


def test_oracle_twisted_bilayer(golden):
    """Extended (twisted) crystal: e1 + rotated e2, pixmap gratings on each, uniform gap;
    reference fixture from examples/crystal_api/twisted_phc.py's construction."""
    g = golden("twisted_3x3")
    n_pix = int(g["n_pix"])
    x = np.linspace(-0.5, 0.5, n_pix)
    X, Y = np.meshgrid(x, x, indexing="ij")
    for k, (lat, ang, f, dg, r, kx, ky) in enumerate(g["cases"]):
        disc = np.where(X ** 2 + Y ** 2 < r ** 2, 4.0, 1.0)
        R, T, S = ko.twisted_solve_rt((3, 3), ["square", "hexagonal"][int(lat)], np.deg2rad(ang),
                                      [("pixmap", disc, 0.3)], [("uniform", 1.0, dg)], [("pixmap", disc, 0.3)],
                                      1.0 / f, 1.0, 1.0, kp=(kx, ky))
        assert abs(R - g["RT"][k, 0]) < 1e-12 and abs(T - g["RT"][k, 1]) < 1e-12
        if k == 0:
            np.testing.assert_allclose(S, g["S0"], atol=1e-12)


def _islands(rows):
    out = []
    for row in rows:
        t = int(row[0])
        out.append({"type": ["disc", "rectangle"][t], "params": list(row[2:6] if t == 1 else row[2:5]),
                    "epsilon": float(row[1])})
    return out


def test_oracle_analytical_layers(golden):
    """Analytical layers (closed-form disc / rectangle transforms, layer.py:161-168): C exactly and
    R, T of [A, U, A] against the reference."""
    g = golden("analytical")
    for tag, lattice, pw in (("sq", "square", (3, 5)), ("hex", "hexagonal", (5, 5))):
        isl = _islands(g[tag + "_islands"])
        np.testing.assert_allclose(ko.analytical_convolution_matrix(isl, 1.5, pw, lattice), g[tag + "_C"], atol=1e-14)
        cl = ko.OracleCrystal(pw, lattice=lattice)
        cl.add_layer_analytical("A", isl, 1.5, 0.4)
        cl.add_layer_uniform("U", 2.0, 0.3)
        cl.set_device(["A", "U", "A"], False)
        for k, (f, kx, ky) in enumerate(((0.45, 0.1, 0.0), (0.62, 0.05, -0.12))):
            cl.set_source(1.0 / f, 1.0, 1.0, kp=(kx * 2 * np.pi * f, ky * 2 * np.pi * f))
            cl.solve()
            r, t = cl.poynting_flux_end()
            assert abs(r - g[tag + "_RT"][k, 0]) < 1e-10 and abs(t - g[tag + "_RT"][k, 1]) < 1e-10


def test_oracle_band_structure_matches_reference(golden):
    """eigentricks.py: pencil eigenvalues, determinant and band_structure of dense global
    S-matrices from the reference's Crystal solve (tests/golden/bands_3x3.npz)."""
    g = golden("bands_3x3")
    for i in range(len(g["S"])):
        w, v, d = ko.scattering_eigenvalues(g["S"][i], dos=True)
        assert ko.match_eigenvalues(w, g["w"][i]) < 1e-9
        assert abs(d - g["det"][i]) <= 1e-9 * abs(g["det"][i])
        Sl, Sr = ko.scattering_splitlr(g["S"][i])
        assert np.abs(Sl @ v - (Sr @ v) * w).max() < 1e-9
        assert ko.band_structure(g["S"][i]).size == g["band_counts"][i]


def test_oracle_beams_match_reference(golden):
    """beams.py: amplitudes_from_fields (square and rectangular supercells, with the reference's
    cell pairing) and gen_bzi_grid (tests/golden/beams.npz)."""
    g = golden("beams")
    for name in ("sq", "rect"):
        F = ko.amplitudes_from_fields(g[f"{name}_fields"], g[f"{name}_g"], g[f"{name}_kp"], g[f"{name}_x"],
                                      g[f"{name}_y"], tuple(g[f"{name}_bzs"]))
        assert np.abs(F - g[f"{name}_F"]).max() < 1e-12 * np.abs(g[f"{name}_F"]).max()
    assert np.allclose(ko.gen_bzi_grid((4, 3)), g["grid_a"], rtol=0, atol=1e-15)
    assert np.allclose(ko.gen_bzi_grid((3, 3), a=2), g["grid_b"], rtol=0, atol=1e-15)
    assert np.allclose(ko.gen_bzi_grid((2, 5), reciproc=((1.0, 0.5), (-0.3, 2.0))), g["grid_c"], rtol=0, atol=1e-15)



def test_oracle_tmat_matches_matlab_and_reference(golden):
    """tmat formulation: the oracle against the reference's MATLAB fixtures (fixtures/pair_pw,
    with the reference test's tolerances, test_pair_pw.py:40-131) and against the reference run
    on a 5x5 oblique two-island case (tests/golden/tmat.npz)."""
    from pins import check_pinned
    g = golden("tmat")
    pw, a, wl, kp, depth, sp = (8, 8), 100e-9, 200e-9, (0.0, 0.0), 1e-7, 3
    lat = ko.tmat_lattice(pw, (a, 0.0), (0.0, a))
    assert np.allclose(lat.b1, g["mat_b1"]) and np.allclose(lat.b2, g["mat_b2"])
    assert np.allclose(lat.gx, g["mat_gx"]) and np.allclose(lat.gy, g["mat_gy"])
    assert np.allclose(lat.Gx, g["mat_Gx"]) and np.allclose(lat.Gy, g["mat_Gy"])
    disc = {"type": "disc", "params": (0.5 * a, 0.5 * a, 0.2 * a)}
    bf = ko.island_transform(disc, lat.Gx, lat.Gy, lat.area)
    assert np.allclose(bf, g["mat_Omega_g"], rtol=1e-7)
    _, q = ko.tmat_grid_size(pw)
    epsg = ko.tmat_epsilon_g(q, [(bf, 8.9)], 1.0)
    iepsg = ko.tmat_epsilon_g(q, [(bf, 8.9)], 1.0, inverse=True)
    assert np.allclose(epsg, g["mat_eps_g"], rtol=1e-7) and np.allclose(iepsg, g["mat_epsinv_g"], rtol=1e-7)
    kz = ko.tmat_kz(lat.gx, lat.gy, 1.0, wl, kp)
    assert np.allclose(kz, g["mat_kgz_in"], rtol=1e-7)
    eta = ko.tmat_eta(lat.gx, lat.gy, kp)
    assert np.allclose(eta[0], g["mat_etagx"], rtol=1e-7) and np.allclose(eta[1], g["mat_etagy"], rtol=1e-7)
    U, Vi, Ve = ko.tmat_uv(lat, wl, kp, 1.0, 1.0)
    check_pinned(g, "mat_U_in", U, 1, rtol=1e-7)
    check_pinned(g, "mat_V_in", Vi, 1, rtol=1e-7)
    A = ko.tmat_matrix_a(pw, lat.gx, lat.gy, epsg, iepsg, wl, kp)
    check_pinned(g, "mat_A", A, 1, rtol=1e-7)
    S, E = ko.tmat_layer_smatrix(A, U, Vi, depth, sp)
    # numpy's assert_allclose defaults (rtol 1e-7) with the test's atol values
    check_pinned(g, "mat_T_xyz", E, 1, rtol=1e-7, atol=1e-10)
    check_pinned(g, "mat_Tslice", U @ E @ Vi, 1, rtol=1e-7, atol=4e-10)
    check_pinned(g, "mat_Sslice", S, 1, rtol=1e-7, atol=1e-11)
    check_pinned(g, "mat_S_interface", ko.tmat_matrix_s(U @ Ve), 1, rtol=1e-7, atol=1e-12)
    # the reference itself on pw 5x5, oblique kp, a disc and a lossy rectangle
    pw = tuple(g["ref_pw"])
    a, wl, kp, depth, sp = float(g["ref_a"]), float(g["ref_wl"]), tuple(g["ref_kp"]), float(g["ref_depth"]), \
        int(g["ref_slicing"])
    lat = ko.tmat_lattice(pw, (a, 0.0), (0.0, a))
    assert np.allclose(lat.gx, g["ref_gx"]) and np.allclose(lat.Gy, g["ref_Gy"])
    A = ko.tmat_matrix_a(pw, lat.gx, lat.gy, g["ref_epsg"], g["ref_iepsg"], wl, kp)
    check_pinned(g, "ref_A", A, 2, rtol=1e-12)
    U, Vi, Ve = ko.tmat_uv(lat, wl, kp, float(g["ref_eps_incid"]), float(g["ref_eps_emerg"]))
    for name, M in (("ref_U", U), ("ref_Vi", Vi), ("ref_Ve", Ve)):
        check_pinned(g, name, M, 2, rtol=1e-12)
    S, E = ko.tmat_layer_smatrix(A, U, Vi, depth, sp)
    check_pinned(g, "ref_E", E, 2, rtol=1e-10, atol=1e-12)
    check_pinned(g, "ref_S", S, 2, rtol=1e-9, atol=1e-11)
