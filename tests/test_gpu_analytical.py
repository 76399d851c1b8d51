"""Analytical layers (closed-form disc / rectangle Fourier coefficients, khepri/layer.py:161-168)
against the reference's complex128 values: C, and R, T through the drop-in facade and the
batched API."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _islands(rows):
    out = []
    for row in rows:
        t = int(row[0])
        out.append({"type": ["disc", "rectangle"][t], "params": list(row[2:6] if t == 1 else row[2:5]),
                    "epsilon": float(row[1])})
    return out


CASES = (("sq", "square", (3, 5)), ("hex", "hexagonal", (5, 5)))
PROBLEMS = ((0.45, 0.1, 0.0), (0.62, 0.05, -0.12))


def test_analytical_convolution_matrix(khp, golden):
    from khepri_gb300 import engine
    g = golden("analytical")
    for tag, lattice, pw in CASES:
        st = engine.StructureGPU(pw, engine.lattice_vectors(lattice))
        entry = st.prepare_map(engine.AnalyticalMap(_islands(g[tag + "_islands"]), 1.5))
        C = entry["conv"][0].cpu().numpy()
        np.testing.assert_allclose(C, g[tag + "_C"], atol=1e-13)


def test_analytical_layers_rt(khp, golden):
    from khepri_gb300 import Crystal, batch
    g = golden("analytical")
    for tag, lattice, pw in CASES:
        isl = _islands(g[tag + "_islands"])
        cl = Crystal(pw, lattice=lattice)
        cl.add_layer_analytical("A", isl, 1.5, 0.4)
        cl.add_layer_uniform("U", 2.0, 0.3)
        cl.set_device(["A", "U", "A"], [False] * 3)
        for k, (f, kx, ky) in enumerate(PROBLEMS):
            cl.set_source(1.0 / f, 1.0, 1.0, kp=(kx * 2 * np.pi * f, ky * 2 * np.pi * f))
            cl.solve()
            r, t = cl.poynting_flux_end()
            assert abs(r - g[tag + "_RT"][k, 0]) < 1e-9 and abs(t - g[tag + "_RT"][k, 1]) < 1e-9
        layers = {"A": ("analytical", (isl, 1.5), 0.4), "U": ("uniform", 2.0, 0.3)}
        wl = np.array([1.0 / f for f, _, _ in PROBLEMS])
        kp = np.array([[kx * 2 * np.pi * f, ky * 2 * np.pi * f] for f, kx, ky in PROBLEMS])
        for method, tol in (("gamma", 1e-9), ("mixed", 1e-6)):
            R, T, s = batch.solve_rt(pw, layers, ["A", "U", "A"], wl, kp, 1.0, 1.0, lattice=lattice, method=method)
            np.testing.assert_allclose(R, g[tag + "_RT"][:, 0], atol=tol)
            np.testing.assert_allclose(T, g[tag + "_RT"][:, 1], atol=tol)
