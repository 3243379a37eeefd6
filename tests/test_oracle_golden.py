"""Pin the CPU oracle against the reference's own golden files.

test/setup_operator/0/{divT_Serial, gradT_Serial} are NeoN's Serial-executor
results of Gauss-linear div and grad on the 5x5x1 fixture mesh with T = cell
index, phi = internal-face index and zero boundary flux (the inputs of
test/setup_operator/0/T and 0/phi).  The files print 16 significant digits.
Tolerances follow test/test_operators.cpp:61,77-80,113,131 (1e-15 absolute on
O(1) data there; relative here because div is O(1e8)).
"""
import numpy as np

from conftest import load_polymesh
from oracle.pyoracle import Oracle


def sig16(x):
    return np.array([float(f"{v:.16g}") for v in np.ravel(x)])


def _operator_case():
    hm, d = load_polymesh("setup_operator")
    T = d["field_T"].copy()
    Tb = np.ascontiguousarray(T[hm.bcells])          # zeroGradient walls: T_b = T_P
    flux = np.zeros(hm.nif + hm.nbf)
    flux[:hm.nif] = d["field_phi"]                     # calculated 0 on the walls
    return hm, d, T, Tb, flux


def test_mesh_fixture_geometry():
    hm, d = load_polymesh("setup_operator")
    assert (hm.n, hm.nif, hm.nbf, hm.npatch) == (25, 40, 20, 1)   # empty frontAndBack has no faces
    np.testing.assert_allclose(hm.V, 4e-6, rtol=1e-14)
    np.testing.assert_allclose(hm.w, 0.5, rtol=1e-14)
    np.testing.assert_allclose(hm.delta, 50.0, rtol=1e-14)
    np.testing.assert_allclose(hm.bdelta, 100.0, rtol=1e-14)


def test_div_linear_matches_divT_Serial():
    hm, d, T, Tb, flux = _operator_case()
    out = Oracle(hm).div(0, 1, flux, T, Tb, 1.0, np.zeros(hm.n))
    g = d["field_divT_Serial"]
    assert np.max(np.abs(out - g)) / np.max(np.abs(g)) < 2e-15
    assert np.sum(sig16(out) == g) >= 24              # identical to the printed digits in 24 of 25 cells


def test_grad_linear_matches_gradT_Serial():
    hm, d, T, Tb, flux = _operator_case()
    out = Oracle(hm).grad(T, Tb, 1.0, np.zeros(3 * hm.n)).reshape(-1, 3)
    g = d["field_gradT_Serial"]
    np.testing.assert_array_equal(sig16(out), g.ravel())   # all 75 components, z round-off included


def test_against_openfoam_fvc():
    hm, d, T, Tb, flux = _operator_case()
    o = Oracle(hm)
    div = o.div(0, 1, flux, T, Tb, 1.0, np.zeros(hm.n))
    np.testing.assert_allclose(div, d["field_ofDivT"], rtol=0, atol=2e-15 * np.abs(d["field_ofDivT"]).max())
    grad = o.grad(T, Tb, 1.0, np.zeros(3 * hm.n)).reshape(-1, 3)
    np.testing.assert_allclose(grad[:, :2], d["field_ofGradT"][:, :2], rtol=0, atol=1e-12)
    np.testing.assert_allclose(grad[:, 2], d["field_ofGradT"][:, 2], rtol=0, atol=1e-6)


def test_sparsity_stencil3D():
    """nnz == nCells + 2*nInternalFaces (test/test_sparsityPattern.cpp:42-62)."""
    hm, _ = load_polymesh("setup_stencil3D")
    assert hm.n == 27
    ro, col, do, oo, no = Oracle(hm).csr_arrays()
    assert ro[-1] == hm.n + 2 * hm.nif == 135
    for c in range(hm.n):
        row = col[ro[c]:ro[c + 1]]
        assert np.all(np.diff(row) > 0) and row[do[c]] == c
    for f in range(hm.nif):
        assert col[ro[hm.own[f]] + oo[f]] == hm.nei[f]
        assert col[ro[hm.nei[f]] + no[f]] == hm.own[f]
