"""Generate golden vectors by running the reference (Kaeryv/Khepri) on seeded inputs.

Run in a container where the reference source is available (read-only):

    python tests/golden/make_golden.py /root/reference

The reference imports numba at module load; ``tests/golden/_shim`` provides an identity
``njit`` (the decorated functions are not on the Crystal solve path).  Inputs come from
``khepri_gb300.workloads`` (deterministic, seeded) or are stored in the fixture itself; each
fixture holds the reference's outputs for them.  The fixtures are small (< 1 MB each) and are
the pins for the oracle (tests/test_oracle_golden.py) and for the GPU parity tests.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _import_reference(ref_root):
    sys.path.insert(0, os.path.join(HERE, "_shim"))
    sys.path.insert(0, ref_root)
    from khepri.crystal import Crystal  # noqa: E402
    from khepri.draw import Drawing  # noqa: E402
    from khepri import tools  # noqa: E402
    return Crystal, Drawing, tools


def _crystal(Crystal, st_pw, layers, stack, mask=False, lattice="square", epsi=1, epse=1):
    cl = Crystal(st_pw, lattice=lattice, epsi=epsi, epse=epse)
    for name, (kind, eps, depth) in layers.items():
        if kind == "uniform":
            cl.add_layer_uniform(name, eps, depth)
        else:
            cl.add_layer_pixmap(name, eps, depth)
    cl.set_device(stack, mask)
    return cl


def main(ref_root):
    sys.path.insert(0, ROOT)
    from khepri_gb300 import workloads as wk

    Crystal, Drawing, tools = _import_reference(ref_root)
    t0 = time.time()

    # A. thin lossy film, test/integration/test_complex_eps.py:13-42 (1x1 harmonics).
    c, e0, sigma, h = 299792458, 8.85418782e-12, 0.01e6, 1.2
    wls = np.linspace(0.7, 2.0)
    R, T, EPS = [], [], []
    for wl in wls:
        omega = np.pi * 2 * (c / 1e-6) / wl
        eps = 1.6 ** 2 - 1j * sigma / omega / e0
        cl = Crystal((1, 1))
        cl.add_layer_uniform("1", eps, h)
        cl.set_device(["1"])
        cl.set_source(wl, 1, 1)
        cl.solve()
        r, t = cl.poynting_flux_end()
        R.append(r); T.append(t); EPS.append(eps)
    np.savez_compressed(os.path.join(HERE, "fresnel_1x1.npz"), wavelength=wls, eps=np.array(EPS),
                        depth=h, R=np.array(R), T=np.array(T))

    # B. plain 5x5 sweep, 151 frequencies (examples/crystal_api/test_crystal.py:23-43 at 128^2).
    d = Drawing((128, 128), 12)
    d.disc((0.0, 0.0), 0.4, 1.0)
    canvas = d.canvas()
    sw = wk.plain_sweep()
    assert np.array_equal(canvas, sw.structure.layers["Scyl"][1]), "disc_canvas disagrees with Drawing"
    cl = _crystal(Crystal, (5, 5), sw.structure.layers, sw.structure.stack, [True] * 3)
    R, T = [], []
    stots = {}
    for i, wl in enumerate(sw.wavelengths):
        cl.set_source(wl, 1.0, 0, 0.0, 0.0)
        cl.solve()
        r, t = cl.poynting_flux_end()
        R.append(r); T.append(t)
        if i in (0, 75):
            stots[i] = cl.Stot.copy()
            if i == 75:
                s_cyl = cl.layers["Scyl"].S.copy()
                lam_cyl = cl.layers["Scyl"].L.copy()
                s_u = cl.layers["S1"].S.copy()
                s_ref = cl.layers["Sref"].S.copy()
                s_trn = cl.layers["Strans"].S.copy()
    np.savez_compressed(os.path.join(HERE, "plain_5x5.npz"), wavelength=sw.wavelengths, R=np.array(R),
                        T=np.array(T), stot_0=stots[0], stot_75=stots[75], s_cyl_75=s_cyl, lam_cyl_75=lam_cyl,
                        s_uniform_75=s_u, s_ref_75=s_ref, s_trn_75=s_trn)

    # C. fields of the plain structure at wl = 2.04 (examples/crystal_api/test_crystal.py:49-57).
    cl.set_source(2.04, 1.0, 0.0, 0, 0)
    cl.solve()
    xs = np.linspace(0, 1, 6)
    ys = np.linspace(0, 1, 5)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    Z = np.array([-0.3, 0.0, 0.2, 0.55, 0.9, 1.65, 2.0, 2.4])
    E, H = cl.fields_volume(X, Y, Z)
    np.savez_compressed(os.path.join(HERE, "fields_5x5.npz"), wavelength=2.04, x=X, y=Y, z=Z, E=E, H=H)

    # D. oblique incidence, both polarisations, per-order output, multi-disc map, non-unit media.
    rng = np.random.default_rng(7)
    emap = wk.multi_disc_map(rng, n=48)
    layers = {"P1": ("pixmap", emap, 0.31), "U1": ("uniform", 2.2, 0.45), "P2": ("pixmap", emap, 0.27),
              "U2": ("uniform", 3.1 - 0.05j, 0.2), "P3": ("pixmap", emap, 0.6)}
    stack = ["P1", "U1", "P2", "U2", "P3"]
    cases = []
    for (epsi, epse) in [(1.0, 1.0), (2.25, 1.5)]:
        cl = _crystal(Crystal, (5, 5), layers, stack, False, epsi=epsi, epse=epse)
        for (wl, te, tm, theta, phi) in [(1.9, 1.0, 0.0, 0.0, 0.0), (1.9, 0.0, 1.0, 0.0, 0.0),
                                         (2.3, 1.0, 0.0, 17.0, 30.0), (2.3, 0.0, 1.0, 17.0, 30.0),
                                         (1.6, 0.6, 0.8, 35.0, -60.0)]:
            cl.set_source(wl, te, tm, theta, phi)
            cl.solve()
            (r, ro), (t, to) = cl.poynting_flux_end(only_total=False)
            cases.append((epsi, epse, wl, te, tm, theta, phi, r.real, t.real, ro.real, to.real))
    arr = lambda k: np.array([cs[k] for cs in cases])
    np.savez_compressed(os.path.join(HERE, "oblique_5x5.npz"), eps_map=emap,
                        depths=np.array([0.31, 0.45, 0.27, 0.2, 0.6]), eps_u=np.array([2.2, 3.1 - 0.05j]),
                        epsi=arr(0), epse=arr(1), wavelength=arr(2), te=arr(3), tm=arr(4), theta=arr(5),
                        phi=arr(6), R=arr(7), T=arr(8), r_orders=arr(9), t_orders=arr(10))

    # E. hexagonal lattice, 3x3, explicit kp.
    dh = Drawing((64, 64), 4.0)
    dh.disc((0.0, 0.0), 0.3, 1.0)
    cl = _crystal(Crystal, (3, 3), {"H": ("pixmap", dh.canvas(), 0.4)}, ["H"], False, lattice="hexagonal")
    hx = []
    for wl, kp in [(1.4, (0.0, 0.0)), (1.2, (0.5, -0.3)), (0.95, (1.1, 0.4))]:
        cl.set_source(wl, 1.0, 1.0, kp=kp)
        cl.solve()
        hx.append((wl, kp[0], kp[1]) + tuple(cl.poynting_flux_end()))
    hx = np.array(hx)
    np.savez_compressed(os.path.join(HERE, "hex_3x3.npz"), eps_map=dh.canvas(), wavelength=hx[:, 0],
                        kp=hx[:, 1:3], R=hx[:, 3], T=hx[:, 4])

    # F. uneven batch, small maps (lossy, absorption = 1 - R - T).
    structs = wk.uneven_structures(8, seed=3, n_pix=32, max_pw=9, max_layers=4)
    out = {}
    for i, (st, wl, kp) in enumerate(structs):
        cl = _crystal(Crystal, st.pw, st.layers, st.stack, False)
        cl.set_source(wl, 1.0, 1.0, kp=tuple(kp))
        cl.solve()
        r, t = cl.poynting_flux_end()
        out[f"R_{i}"] = r; out[f"T_{i}"] = t
    np.savez_compressed(os.path.join(HERE, "uneven_small.npz"), count=8, seed=3, n_pix=32, max_pw=9,
                        max_layers=4, R=np.array([out[f"R_{i}"] for i in range(8)]),
                        T=np.array([out[f"T_{i}"] for i in range(8)]))

    # G. the 11x11 batched-sweep structure (seed 0, full 256^2 map), a few (f, k) problems.
    st = wk.batched_structure(0)
    wl_all, kp_all = wk.batched_problems()
    pick = np.array([16 * 32 + 16, 20 * 1024 + 15 * 32 + 17, 40 * 1024 + 300, 63 * 1024 + 1023])
    cl = _crystal(Crystal, st.pw, st.layers, st.stack, False)
    Rte, Tte, Rtm, Ttm = [], [], [], []
    for p in pick:
        for (te, tm, RR, TT) in [(1.0, 0.0, Rte, Tte), (0.0, 1.0, Rtm, Ttm)]:
            cl.set_source(wl_all[p], te, tm, kp=tuple(kp_all[p]))
            cl.solve()
            r, t = cl.poynting_flux_end()
            RR.append(r); TT.append(t)
    np.savez_compressed(os.path.join(HERE, "batched_11x11.npz"), seed=0, problems=pick,
                        map_sum=st.layers["P1"][1].sum(), R_te=np.array(Rte), T_te=np.array(Tte),
                        R_tm=np.array(Rtm), T_tm=np.array(Ttm))

    # H. convolution matrix of a non-square complex map, non-square harmonic set.
    rng = np.random.default_rng(11)
    cmap = rng.uniform(1, 5, size=(20, 14)) - 1j * rng.uniform(0, 0.2, size=(20, 14))
    conv = tools.convolution_matrix(cmap, (5, 3))
    np.savez_compressed(os.path.join(HERE, "convmat.npz"), eps_map=cmap, pw=np.array([5, 3]), C=conv)

    # I. inverse-design structures (9x9), zeroth-order transmission.
    thetas, dstructs, freqs = wk.inverse_design(2, seed=0)
    res = []
    for st in dstructs:
        cl = _crystal(Crystal, st.pw, st.layers, st.stack, False)
        for f in freqs[[0, 7, 15]]:
            cl.set_source(1.0 / f, 1.0, 0.0, 0.0, 0.0)
            cl.solve()
            (r, ro), (t, to) = cl.poynting_flux_end(only_total=False)
            res.append((f, r.real, t.real, to[(81 - 1) // 2].real))
    res = np.array(res)
    np.savez_compressed(os.path.join(HERE, "design_9x9.npz"), count=2, seed=0, freq=res[:, 0], R=res[:, 1],
                        T=res[:, 2], t0=res[:, 3])
    print(f"golden vectors written in {time.time() - t0:.1f} s")


def twisted(ref_root):
    """Twisted bilayer (examples/crystal_api/twisted_phc.py:35-57 with pixmap gratings): extended
    crystal over e1 + e2, e2 rotated; R, T and the global S at 3x3 base harmonics."""
    sys.path.insert(0, ROOT)
    Crystal, Drawing, tools = _import_reference(ref_root)
    from khepri.expansion import Expansion
    from khepri.layer import Layer
    rng = np.random.default_rng(11)
    x = np.linspace(-0.5, 0.5, 32)
    X, Y = np.meshgrid(x, x, indexing="ij")
    cases, out = [], []
    for lattice in ("square", "hexagonal"):
        for angle_deg, f, d_gap, r in ((7.0, 0.62, 0.25, 0.3), (23.0, 0.71, 0.4, 0.22)):
            disc = np.where(X ** 2 + Y ** 2 < r ** 2, 4.0, 1.0)
            lat = Crystal((1, 1), lattice=lattice).lattice
            e1 = Expansion((3, 3), lattice=lat)
            e2 = Expansion((3, 3), lattice=lat)
            e2.rotate(np.deg2rad(angle_deg))
            cl = Crystal.from_expansion(e1 + e2)
            etw = cl.expansion
            cl.add_layer("Sref", Layer.half_infinite(e1, "reflexion", 1), True)
            cl.add_layer("G1", Layer.pixmap(e1, disc, 0.3), True)
            cl.add_layer("Gap", Layer.uniform(etw, 1.0, d_gap), False)
            cl.add_layer("G2", Layer.pixmap(e2, disc, 0.3), True)
            cl.add_layer("Strans", Layer.half_infinite(e2, "transmission", 1), True)
            cl.set_device(["G1", "Gap", "G2"], [False] * 3)
            kp = (0.21 * 2 * np.pi * f, -0.08 * 2 * np.pi * f)
            cl.set_source(1.0 / f, 1.0, 1.0, kp=kp)
            cl.solve()
            R, T = cl.poynting_flux_end()
            cases.append((0 if lattice == "square" else 1, angle_deg, f, d_gap, r, kp[0], kp[1]))
            out.append((R, T))
            if len(out) == 1:
                S0 = np.asarray(cl.Stot)
    np.savez_compressed(os.path.join(HERE, "twisted_3x3.npz"), cases=np.array(cases), RT=np.array(out), S0=S0,
                        n_pix=32)


def twisted7(ref_root):
    """One twisted bilayer at 7x7 base harmonics (product expansion of 2401 orders, n = 4802):
    disc gratings eps 12 in eps 1 (r = 0.3, depth 0.3) on both sides of a gap (eps 1, d = 0.3),
    twist 13 deg, square lattice, f = 0.5, oblique kp; R and T of the reference."""
    sys.path.insert(0, ROOT)
    Crystal, Drawing, tools = _import_reference(ref_root)
    from khepri.expansion import Expansion
    from khepri.layer import Layer
    x = np.linspace(-0.5, 0.5, 64)
    X, Y = np.meshgrid(x, x, indexing="ij")
    r, angle_deg, f, d_gap = 0.3, 13.0, 0.5, 0.3
    disc = np.where(X ** 2 + Y ** 2 < r ** 2, 12.0, 1.0)
    lat = Crystal((1, 1), lattice="square").lattice
    e1 = Expansion((7, 7), lattice=lat)
    e2 = Expansion((7, 7), lattice=lat)
    e2.rotate(np.deg2rad(angle_deg))
    cl = Crystal.from_expansion(e1 + e2)
    etw = cl.expansion
    cl.add_layer("Sref", Layer.half_infinite(e1, "reflexion", 1), True)
    cl.add_layer("G1", Layer.pixmap(e1, disc, 0.3), True)
    cl.add_layer("Gap", Layer.uniform(etw, 1.0, d_gap), False)
    cl.add_layer("G2", Layer.pixmap(e2, disc, 0.3), True)
    cl.add_layer("Strans", Layer.half_infinite(e2, "transmission", 1), True)
    cl.set_device(["G1", "Gap", "G2"], [False] * 3)
    kp = (0.11 * 2 * np.pi * f, 0.05 * 2 * np.pi * f)
    cl.set_source(1.0 / f, 1.0, 1.0, kp=kp)
    t0 = time.time()
    cl.solve()
    R, T = cl.poynting_flux_end()
    print(f"twisted 7x7: R {R}, T {T}, R + T - 1 = {R + T - 1:.2e}, {time.time() - t0:.0f} s")
    np.savez_compressed(os.path.join(HERE, "twisted_7x7.npz"), case=np.array([0, angle_deg, f, d_gap, r, kp[0], kp[1]]),
                        RT=np.array([R, T]), n_pix=64, eps_disc=12.0)


def analytical(ref_root):
    """Analytical layers (closed-form island transforms, layer.py:161-168): C and R, T of a stack
    [analytical, uniform, analytical] for square (3x5 harmonics) and hexagonal (5x5) lattices."""
    sys.path.insert(0, ROOT)
    Crystal, Drawing, tools = _import_reference(ref_root)
    out = {}
    for tag, lattice, pw in (("sq", "square", (3, 5)), ("hex", "hexagonal", (5, 5))):
        dr = Drawing((64, 64), 1.5)
        dr.disc((0.1, -0.05), 0.25, 8.0)
        dr.rectangle((-0.2, 0.15), (0.2, 0.3), 3.0)
        islands = dr.islands()
        cl = Crystal(pw, lattice=lattice)
        cl.add_layer_analytical("A", islands, 1.5, 0.4)
        cl.add_layer_uniform("U", 2.0, 0.3)
        cl.set_device(["A", "U", "A"], [False] * 3)
        RT, C = [], None
        for f, kx, ky in ((0.45, 0.1, 0.0), (0.62, 0.05, -0.12)):
            cl.set_source(1.0 / f, 1.0, 1.0, kp=(kx * 2 * np.pi * f, ky * 2 * np.pi * f))
            cl.solve()
            RT.append(cl.poynting_flux_end())
            C = np.asarray(cl.layers["A"].C)
        out[tag + "_RT"] = np.array(RT)
        out[tag + "_C"] = C
        out[tag + "_islands"] = np.array([[0 if i["type"] == "disc" else 1, i["epsilon"]] + list(i["params"]) +
                                          [0.0] * (4 - len(i["params"])) for i in islands])
    np.savez_compressed(os.path.join(HERE, "analytical.npz"), **out)


def bands(ref_root):
    """Band structure from S (khepri/eigentricks.py:5-55): pencil eigenvalues, determinant and
    band_structure of the dense global S of a patterned slab (3x3 harmonics, disc eps 8 in air,
    d = 0.4) at four (f, kx) points, from the reference's Crystal solve."""
    sys.path.insert(0, ROOT)
    Crystal, Drawing, tools = _import_reference(ref_root)
    from khepri import eigentricks as et
    x = np.linspace(-0.5, 0.5, 64)
    X, Y = np.meshgrid(x, x, indexing="ij")
    emap = np.where(X ** 2 + Y ** 2 < 0.3 ** 2, 8.0, 1.0)
    cl = _crystal(Crystal, (3, 3), {"P": ("pixmap", emap, 0.4)}, ["P"])
    points = [(0.3, 0.0), (0.45, 0.3), (0.6, 0.8), (0.7, 1.5)]
    Ss, ws, dets, bs, counts = [], [], [], [], []
    for f, kx in points:
        cl.set_source(1.0 / f, 1.0, 0.0, kp=(kx, 0.0))
        cl.solve()
        S = np.asarray(cl.Stot)
        n = S.shape[2]
        Sd = S.transpose(0, 2, 1, 3).reshape(2 * n, 2 * n)
        w, _, d = et.scattering_eigenvalues(Sd, dos=True)
        b = et.band_structure(Sd)
        Ss.append(Sd)
        ws.append(w)
        dets.append(d)
        bs.extend(list(b))
        counts.append(len(b))
    np.savez_compressed(os.path.join(HERE, "bands_3x3.npz"), S=np.array(Ss), w=np.array(ws), det=np.array(dets),
                        bands=np.array(bs, dtype=float), band_counts=np.array(counts), points=np.array(points))
    print("bands_3x3: eigenvalues of", len(points), "S-matrices of size", Ss[0].shape)


def beams(ref_root):
    """Brillouin-zone-integrated beams (khepri/beams.py:164-207): amplitudes_from_fields on seeded
    random fields over 3x3 and 2x3 supercells (3x3 harmonics), and gen_bzi_grid."""
    sys.path.insert(0, ROOT)
    _import_reference(ref_root)
    from khepri.beams import amplitudes_from_fields, gen_bzi_grid
    from khepri.expansion import Expansion
    rng = np.random.default_rng(21)
    out = {}
    for name, bzs, ns, kp in [("sq", (3, 3), 4, (0.4, -0.25)), ("rect", (2, 3), 4, (-0.1, 0.3))]:
        X, Y = bzs[1] * ns, bzs[0] * ns
        fields = rng.standard_normal((X, Y, 2, 3)) + 1j * rng.standard_normal((X, Y, 2, 3))
        x, y = np.meshgrid((np.arange(X) + 0.5) / ns, (np.arange(Y) + 0.5) / ns * 1.1, indexing="ij")
        e = Expansion((3, 3))
        F = amplitudes_from_fields(fields, e, 1.0, kp, x, y, bzs)
        out.update({f"{name}_fields": fields, f"{name}_x": x, f"{name}_y": y, f"{name}_kp": np.array(kp),
                    f"{name}_bzs": np.array(bzs), f"{name}_g": e.g_vectors, f"{name}_F": F})
    out["grid_a"] = gen_bzi_grid((4, 3))
    out["grid_b"] = gen_bzi_grid((3, 3), a=2)
    out["grid_c"] = gen_bzi_grid((2, 5), reciproc=((1.0, 0.5), (-0.3, 2.0)))
    np.savez_compressed(os.path.join(HERE, "beams.npz"), **out)
    print("beams: amplitudes of", out["sq_F"].shape, out["rect_F"].shape)


def _pin(out, name, M, rng_seed=0):
    """A large matrix pinned by seeded sampled entries and two seeded matrix-vector checksums."""
    rng = np.random.default_rng(rng_seed)
    M = np.asarray(M)
    idx = rng.choice(M.size, size=min(M.size, 6000), replace=False)
    r = rng.standard_normal(M.shape[1]) + 1j * rng.standard_normal(M.shape[1])
    l = rng.standard_normal(M.shape[0]) + 1j * rng.standard_normal(M.shape[0])
    out[f"{name}_idx"] = idx
    out[f"{name}_val"] = M.flat[idx]
    out[f"{name}_Mr"] = M @ r
    out[f"{name}_lM"] = l @ M


def tmat(ref_root):
    """tmat expm formulation (khepri/tmat/*.py): the MATLAB fixtures of the reference's own test
    (test/integration/test_pair_pw.py, fixtures/pair_pw: pw 8x8, a = 100 nm, lambda = 200 nm,
    disc r = 0.2 a, eps 8.9, depth 100 nm / 2^3 slices) and the reference run on a second case
    (pw 5x5, oblique kp, two islands).  Large matrices are stored as seeded samples plus
    matrix-vector checksums (_pin)."""
    sys.path.insert(0, ROOT)
    _import_reference(ref_root)
    from scipy.io import loadmat
    from scipy.linalg import expm
    from khepri.tmat.lattice import CartesianLattice
    from khepri.tmat.tools import epsilon_g, grid_size, coords_from_index
    from khepri.tmat.matrices import matrix_a, matrix_s, multS
    from khepri.fourier import transform
    fx = os.path.join(ref_root, "test", "integration", "fixtures", "pair_pw")
    out = {}
    # (1) the MATLAB values
    d = {}
    for f in ("S", "T", "UV", "epsg", "eta", "gvectors", "kz", "mu", "reciproc", "interface", "fourier"):
        d.update({k: v for k, v in loadmat(os.path.join(fx, f + ".mat")).items() if not k.startswith("__")})
    for k in ("A", "Tslice", "Sslice", "T_xyz", "U_in", "V_in", "V_em", "S_interface"):
        _pin(out, "mat_" + k, d[k], rng_seed=1)
    for k in ("eps_g", "epsinv_g", "etagx", "etagy", "gx", "gy", "Gx", "Gy", "kgz_in", "kgz_em", "mugx_in",
              "mugy_in", "b1", "b2"):
        out["mat_" + k] = np.asarray(d[k])
    out["mat_Omega_g"] = np.vectorize(lambda c: complex(np.asarray(c).item()), otypes=[complex])(d["Omega_g"])
    # (2) the reference on pw 5x5, oblique incidence, a disc and a rectangle
    pw, a, wl, kp, depth, sp = (5, 5), 100e-9, 310e-9, (2.1e6, -1.3e6), 80e-9, 2
    lat = CartesianLattice(pw, a1=(a, 0.0), a2=(0.0, a), eps_emerg=2.25, eps_incid=1.0, dtype=np.float64)
    isl = [(transform("disc", [0.3 * a, 0.45 * a, 0.22 * a], lat.Gx, lat.Gy, lat.area), 6.0),
           (transform("rectangle", [0.6 * a, 0.1 * a, 0.9 * a, 0.35 * a], lat.Gx, lat.Gy, lat.area), 3.0 + 0.1j)]
    _, q = grid_size(pw)
    epsg = epsilon_g(q, isl, 1.5)
    iepsg = epsilon_g(q, isl, 1.5, inverse=True)
    nx, ny = lat.gx.shape[0] // 2, lat.gx.shape[1] // 2
    ind = np.array([coords_from_index(pw, (nx, ny), i) for i in range(pw[0] * pw[1])])
    A = matrix_a(ind, lat.gx, lat.gy, epsg, iepsg, wl, kx=kp[0], ky=kp[1])
    E = expm(-A * (depth / 2 ** sp))
    U, Vi, Ve = lat.U(wl, kp), lat.Vi(wl, kp), lat.Ve(wl, kp)
    T = U @ E @ Vi
    S = matrix_s(T)
    for _ in range(sp):
        S = multS(S, S)
    Si = matrix_s(U @ Ve)
    out.update({"ref_pw": np.array(pw), "ref_a": a, "ref_wl": wl, "ref_kp": np.array(kp), "ref_depth": depth,
                "ref_slicing": sp, "ref_eps_incid": 1.0, "ref_eps_emerg": 2.25, "ref_eps_host": 1.5,
                "ref_epsg": epsg, "ref_iepsg": iepsg, "ref_gx": lat.gx, "ref_gy": lat.gy, "ref_Gx": lat.Gx,
                "ref_Gy": lat.Gy})
    for k, M in (("A", A), ("E", E), ("U", U), ("Vi", Vi), ("Ve", Ve), ("T", T), ("S", S), ("Sint", Si)):
        _pin(out, "ref_" + k, M, rng_seed=2)
    np.savez_compressed(os.path.join(HERE, "tmat.npz"), **out)
    print("tmat: MATLAB pair_pw pins and a 5x5 reference case;", A.shape)


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "tmat":
        tmat(sys.argv[1])
    elif len(sys.argv) > 2 and sys.argv[2] == "beams":
        beams(sys.argv[1])
    elif len(sys.argv) > 2 and sys.argv[2] == "bands":
        bands(sys.argv[1])
    elif len(sys.argv) > 2 and sys.argv[2] == "analytical":
        analytical(sys.argv[1])
    elif len(sys.argv) > 2 and sys.argv[2] == "twisted":
        twisted(sys.argv[1])
    elif len(sys.argv) > 2 and sys.argv[2] == "twisted7":
        twisted7(sys.argv[1])
    elif len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        sys.exit("usage: make_golden.py <reference source root> [tmat|beams|bands|analytical|twisted]")
