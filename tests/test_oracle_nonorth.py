"""Non-orthogonal correction (`Gauss linear corrected`) in the oracle, on the
CPU: properties of OpenFOAM's correctedSnGrad that hold whatever the mesh."""
import numpy as np
import pytest

from foamadapter_gb300 import abi, mesh
from oracle.pyoracle import Oracle


def linear_field(hm, a, b=2.0):
    return hm.C @ a + b, hm.bCf @ a + b


def test_orthogonal_box_has_no_correction():
    hm = mesh.box(9, 7, 5, jitter=0.0)
    o = Oracle(hm)
    assert np.abs(o.nonorth_vectors()).max() < 1e-13
    rng = np.random.default_rng(0)
    T, Tb = rng.standard_normal(hm.n), rng.standard_normal(hm.nbf)
    gamma = np.exp(rng.standard_normal(hm.nif + hm.nbf))
    lu = o.laplacian(1, gamma, T, Tb, 1.0, np.zeros(hm.n))
    lc = o.laplacian_corrected(1, gamma, T, Tb, 1.0, np.zeros(hm.n))
    np.testing.assert_allclose(lc, lu, rtol=0, atol=1e-11 * np.abs(lu).max())


@pytest.mark.parametrize("jitter,gain", [(0.1, 10.0), (0.3, 4.0)])
def test_correction_recovers_linear_field_gradient(jitter, gain):
    """On a jittered mesh the uncorrected snGrad of a linear field is off by the
    non-orthogonality; the corrected one is `gain` times closer to n.grad(T)."""
    hm = mesh.box(12, 11, 10, jitter=jitter, seed=4)
    o = Oracle(hm)
    a = np.array([0.3, -1.2, 0.7])
    T, Tb = linear_field(hm, a)
    exact = (hm.Sf / hm.magSf[:, None]) @ a
    eu = np.abs(o.sngrad(T, Tb)[:hm.nif] - exact).mean()
    ec = np.abs(o.sngrad_corrected(T, Tb)[:hm.nif] - exact).mean()
    assert ec * gain < eu
    # boundary faces are not corrected
    np.testing.assert_array_equal(o.sngrad_corrected(T, Tb)[hm.nif:], o.sngrad(T, Tb)[hm.nif:])


def test_corrected_laplacian_is_uncorrected_plus_flux_correction():
    """laplacian_corrected = laplacian + div(faceFluxCorrection)/V (the split the
    implicit assembly uses), per component of a vector field."""
    hm = mesh.box(8, 7, 6, jitter=0.2, seed=1)
    o = Oracle(hm)
    rng = np.random.default_rng(2)
    U, Ub = rng.standard_normal(3 * hm.n), rng.standard_normal(3 * hm.nbf)
    gamma = np.exp(rng.standard_normal(hm.nif + hm.nbf))
    full = o.laplacian_corrected(3, gamma, U, Ub, 1.0, np.zeros(3 * hm.n))
    unc = o.laplacian(3, gamma, U, Ub, 1.0, np.zeros(3 * hm.n))
    fc = o.nonorth_flux(3, gamma, U, Ub, 1.0, np.zeros(3 * (hm.nif + hm.nbf)))
    div = np.zeros((hm.n, 3))
    np.add.at(div, hm.own, fc[:3 * hm.nif].reshape(-1, 3))
    np.subtract.at(div, hm.nei, fc[:3 * hm.nif].reshape(-1, 3))
    np.testing.assert_allclose(full, unc + (div / hm.V[:, None]).ravel(), rtol=0, atol=1e-11 * np.abs(full).max())
    assert not fc[3 * hm.nif:].any()


def test_corrected_implicit_laplacian_reproduces_explicit_one():
    """A x - b of the assembled corrected laplacian equals the explicit
    corrected laplacian of x (volume integrated) when x is the field the
    correction was evaluated on."""
    hm = mesh.box(7, 6, 5, jitter=0.2, seed=3)
    o = Oracle(hm)
    rng = np.random.default_rng(4)
    T = rng.standard_normal(hm.n)
    Tb = rng.standard_normal(hm.nbf)
    gamma = np.exp(rng.standard_normal(hm.nif + hm.nbf))
    types = [abi.BC_FIXED_VALUE] * hm.npatch
    terms = [(abi.TERM_LAPLACIAN, abi.SCHEME_CORRECTED, 1.0, T, gamma)]
    values, rhs, _, _ = o.assemble(1, terms, 1.0, types, Tb, Tb)
    Ax_b = o.apply_operator(values, rhs, 1, T)
    lap = o.laplacian_corrected(1, gamma, T, Tb, 1.0, np.zeros(hm.n)) * hm.V
    np.testing.assert_allclose(Ax_b, lap, rtol=0, atol=1e-10 * np.abs(lap).max())


@pytest.mark.parametrize("corrected,ddt_corr,n_non_orth", [(False, False, 0), (True, False, 0), (True, True, 1),
                                                           (False, True, 0)])
def test_cavity_loop_keeps_continuity(corrected, ddt_corr, n_non_orth):
    """phi = phiHbyA - pEqn.flux() conserves mass in every cell to the pressure
    solver's tolerance, with or without the corrected laplacian (its face-flux
    correction taken with the pressure the matrix was assembled with) and ddtCorr."""
    from oracle.apps import CavityPisoCPU

    hm = mesh.box(14, 13, 1, 1.0, 1.0, 1.0 / 14, jitter=0.25, seed=5, two_d=True)
    cpu = CavityPisoCPU(hm, dt=5e-3, n_corr=2, p_rel_tol=1e-12, ddt_corr=ddt_corr, corrected=corrected,
                        n_non_orth=n_non_orth)
    for _ in range(3):
        cpu.step()
    assert len(cpu.stats) == 3 * 2 * (n_non_orth + 1)
    div = np.zeros(hm.n)
    np.add.at(div, hm.own, cpu.phi[:hm.nif])
    np.subtract.at(div, hm.nei, cpu.phi[:hm.nif])
    np.add.at(div, hm.bcells, cpu.phi[hm.nif:])
    assert np.abs(div).max() < 1e-9 * np.abs(cpu.phi).max()
