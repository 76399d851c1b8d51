"""Band structure from S on the GPU (khepri_gb300.eigentricks, khp_scattering_eig) against the
reference's eigentricks on the same dense S-matrices (tests/golden/bands_3x3.npz: the global S
of a patterned slab at four (f, kx) points).  The eigenvalues of the pencil (Sl, Sr) are an
unordered set: each reference eigenvalue must have one of ours within 1e-8 relative."""
import numpy as np
import pytest

from oracle import khepri_oracle as ko

pytestmark = pytest.mark.gpu

TOL = 1e-8


def test_pencil_eigenvalues_and_det_match_reference(khp, golden):
    from khepri_gb300 import eigentricks as et
    g = golden("bands_3x3")
    S = g["S"]
    w, v, d = et.scattering_eigenvalues(S, dos=True)  # the four S-matrices in one batch
    for i in range(len(S)):
        assert ko.match_eigenvalues(w[i], g["w"][i]) < TOL
        assert ko.match_eigenvalues(g["w"][i], w[i]) < TOL
        assert abs(d[i] - g["det"][i]) <= TOL * abs(g["det"][i])
        Sl, Sr = et.scattering_splitlr(S[i])
        scale = np.abs(Sl).max() + np.abs(Sr).max() * np.abs(w[i]).max()
        assert np.abs(Sl @ v[i] - (Sr @ v[i]) * w[i]).max() < 1e-10 * scale
        assert np.allclose(np.linalg.norm(v[i], axis=0), 1.0)
        b = et.band_structure(S[i])
        assert b.size == g["band_counts"][i]


def test_single_matrix_crystal_layout_and_nan(khp, golden):
    from khepri_gb300 import eigentricks as et
    g = golden("bands_3x3")
    Sd = g["S"][1]
    n = Sd.shape[0] // 2
    S4 = Sd.reshape(2, n, 2, n).transpose(0, 2, 1, 3)  # [2, 2, n, n]
    w, v = et.scattering_eigenvalues(S4)
    assert w.shape == (2 * n,) and v.shape == (2 * n, 2 * n)
    assert ko.match_eigenvalues(w, g["w"][1]) < TOL
    assert abs(et.scattering_det(Sd) - g["det"][1]) <= TOL * abs(g["det"][1])
    bad = Sd.copy()
    bad[0, 0] = np.nan
    assert et.scattering_eigenvalues(bad) is None
    assert et.band_structure(bad) is None
    wb, _ = et.scattering_eigenvalues(np.stack([bad, Sd]))
    assert np.isnan(wb[0]).all() and ko.match_eigenvalues(wb[1], g["w"][1]) < TOL
