"""Twisted bilayers (extended crystal over e1 + rotated e2) against the reference's complex128
values: square and hexagonal lattices, two twist angles, pixmap gratings on both sides."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_twisted_bilayer_golden(khp, golden):
    from khepri_gb300 import twisted
    g = golden("twisted_3x3")
    n_pix = int(g["n_pix"])
    x = np.linspace(-0.5, 0.5, n_pix)
    X, Y = np.meshgrid(x, x, indexing="ij")
    for k, (lat, ang, f, dg, r, kx, ky) in enumerate(g["cases"]):
        disc = np.where(X ** 2 + Y ** 2 < r ** 2, 4.0, 1.0)
        tw = twisted.TwistedBilayer((3, 3), ["square", "hexagonal"][int(lat)], np.deg2rad(ang),
                                    [("pixmap", disc, 0.3)], [("uniform", 1.0, dg)], [("pixmap", disc, 0.3)])
        R, T, st = tw.solve_rt([1.0 / f], [[kx, ky]], 1.0, 1.0)
        assert not st.any()
        print(k, R[0] - g["RT"][k, 0], T[0] - g["RT"][k, 1])
        assert abs(R[0] - g["RT"][k, 0]) < 1e-9 and abs(T[0] - g["RT"][k, 1]) < 1e-9


def test_twisted_batch_both_pols_lossless(khp):
    """A batch of frequencies at 5x5 base harmonics (n = 1250): R + T = 1 for a lossless stack,
    and the (1, 1) polarisation's R is the mean of the two unit polarisations' when the cross
    terms cancel is not assumed: only energy conservation is checked here."""
    from khepri_gb300 import twisted
    x = np.linspace(-0.5, 0.5, 64)
    X, Y = np.meshgrid(x, x, indexing="ij")
    disc = np.where(X ** 2 + Y ** 2 < 0.3 ** 2, 12.0, 1.0)
    tw = twisted.TwistedBilayer((5, 5), "square", np.deg2rad(13.0), [("pixmap", disc, 0.3)],
                                [("uniform", 1.0, 0.25)], [("pixmap", disc, 0.3)])
    f = np.linspace(0.4, 0.7, 4)
    R, T, st = tw.solve_rt(1.0 / f, np.zeros((4, 2)), both_pols=True)
    assert not st.any()
    np.testing.assert_allclose(R + T, 1.0, atol=1e-8)


def test_twisted_bilayer_7x7_golden(khp, golden):
    """The larger basis of the twisted-bilayer config: 7x7 base harmonics, a product expansion of
    2401 orders (n = 4802), disc gratings eps 12 in eps 1 on both sides of a gap, 13 deg, oblique
    incidence: R, T against the reference's complex128 values at 1e-9, and R + T = 1 to 1e-8."""
    from khepri_gb300 import twisted
    g = golden("twisted_7x7")
    _, ang, f, dg, r, kx, ky = g["case"]
    x = np.linspace(-0.5, 0.5, int(g["n_pix"]))
    X, Y = np.meshgrid(x, x, indexing="ij")
    disc = np.where(X ** 2 + Y ** 2 < r ** 2, float(g["eps_disc"]), 1.0)
    tw = twisted.TwistedBilayer((7, 7), "square", np.deg2rad(ang), [("pixmap", disc, 0.3)], [("uniform", 1.0, dg)],
                                [("pixmap", disc, 0.3)])
    R, T, st = tw.solve_rt([1.0 / f], [[kx, ky]], 1.0, 1.0)
    assert not st.any()
    print("7x7 twisted: dR", R[0] - g["RT"][0], "dT", T[0] - g["RT"][1], "R + T - 1", R[0] + T[0] - 1)
    assert abs(R[0] - g["RT"][0]) < 1e-9 and abs(T[0] - g["RT"][1]) < 1e-9
    assert abs(R[0] + T[0] - 1) < 1e-8
