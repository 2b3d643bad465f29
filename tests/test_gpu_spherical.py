"""Real solid-harmonic output (an option beyond the reference's Cartesian basis).

The GPU path builds Cartesian integrals and transforms them; the check is the
oracle's Cartesian integrals and SCF transformed the same way in numpy.  The
spherical space is a subspace of the Cartesian one (a Cartesian d shell also
holds x^2 + y^2 + z^2), so its RHF energy lies above the Cartesian one.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(geom, basis, spherical):
    import slowquant_gb300.SlowQuant as sq

    A = sq.SlowQuant()
    A.set_molecule(geom, distance_unit="angstrom")
    A.set_basis_set(basis, spherical=spherical)
    A.init_hartree_fock()
    A.hartree_fock.logger.print_output = False
    A.hartree_fock.run_restricted_hartree_fock()
    return A


@pytest.mark.parametrize("basis", ["cc-pvdz", "cc-pvtz"])
def test_spherical_scf_matches_oracle(gpu_lib, basis):
    from oracle import oracle as O
    from slowquant_gb300 import spherical, systems

    geom = systems.water_monomer()
    A = _run(geom, basis, True)
    cart = _run(geom, basis, False)
    T = spherical.transform_matrix(A.molecule.shells)
    assert A.integral.number_bf == T.shape[1] == (24 if basis == "cc-pvdz" else 58)
    o = O.OracleMolecule(geom, basis, "angstrom")
    S, Tk, Vn = o.one_electron()
    S, Tk, Vn = (T.T @ M @ T for M in (S, Tk, Vn))
    np.testing.assert_allclose(A.integral.overlap_matrix, S, atol=1e-12)

    def jk(D):
        J, K = o.jk_direct(T @ D @ T.T, 1e-12)
        return T.T @ J @ T, T.T @ K @ T

    E = O.run_hartree_fock(S, Tk, Vn, jk, o.number_electrons)[0]
    assert abs(A.hartree_fock.E_hf - E) < 1e-8
    assert A.hartree_fock.E_hf > cart.hartree_fock.E_hf


def test_spherical_dense_tensor_is_the_transformed_cartesian_one(gpu_lib):
    from slowquant_gb300 import spherical, systems

    A = _run(systems.water_monomer(), "cc-pvdz", True)
    cart = _run(systems.water_monomer(), "cc-pvdz", False)
    T = spherical.transform_matrix(A.molecule.shells)
    V = np.einsum("pqrs,pi,qj,rk,sl->ijkl", cart.integral.electron_repulsion_tensor, T, T, T, T, optimize=True)
    np.testing.assert_allclose(A.integral.electron_repulsion_tensor, V, atol=1e-11)
