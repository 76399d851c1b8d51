"""Brillouin-zone-integrated beams on the GPU (khepri_gb300.beams, khp_bzi_amplitudes) against
the reference's amplitudes_from_fields on the same samples (tests/golden/beams.npz: square and
rectangular supercells, so the reference's pairing of cell samples and coordinates is
exercised), and against the oracle on a larger case."""
import numpy as np
import pytest

from oracle import khepri_oracle as ko

pytestmark = pytest.mark.gpu


def test_amplitudes_match_reference(khp, golden):
    from khepri_gb300 import beams
    from khepri_gb300.expansion import Expansion
    g = golden("beams")
    e = Expansion((3, 3))
    assert np.allclose(e.g_vectors, g["sq_g"], rtol=0, atol=1e-14)
    for name in ("sq", "rect"):
        F = beams.amplitudes_from_fields(g[f"{name}_fields"], e, 1.0, g[f"{name}_kp"], g[f"{name}_x"],
                                         g[f"{name}_y"], tuple(g[f"{name}_bzs"]))
        ref = g[f"{name}_F"]
        assert F.shape == ref.shape
        assert np.abs(F - ref).max() < 1e-12 * np.abs(ref).max()
    assert np.allclose(beams.gen_bzi_grid((4, 3)), g["grid_a"], rtol=0, atol=1e-15)
    assert np.allclose(beams.gen_bzi_grid((2, 5), reciproc=((1.0, 0.5), (-0.3, 2.0))), g["grid_c"], rtol=0,
                       atol=1e-15)


def test_amplitudes_larger_supercell_vs_oracle(khp):
    from khepri_gb300 import beams, Crystal
    rng = np.random.default_rng(5)
    bzs, ns = (5, 4), 8
    X, Y = bzs[1] * ns, bzs[0] * ns
    fields = rng.standard_normal((X, Y, 2, 3)) + 1j * rng.standard_normal((X, Y, 2, 3))
    x, y = np.meshgrid(np.arange(X) / ns, np.arange(Y) / ns, indexing="ij")
    cl = Crystal((5, 5))
    kp = (0.2 + 0.01j, -0.35)
    F = beams.amplitudes_from_fields(fields, cl.expansion, 1.0, kp, x, y, bzs)
    ref = ko.amplitudes_from_fields(fields, cl.expansion.g_vectors, np.asarray(kp), x, y, bzs)
    assert np.abs(F - ref).max() < 1e-12 * np.abs(ref).max()
