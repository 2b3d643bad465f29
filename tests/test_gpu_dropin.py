"""Option A of the integration guide: SlowQuant's own module names, served by this package.

``slowquant_gb300.dropin.install()`` registers the package under the names the
reference's code imports; the tests then import ``slowquant.SlowQuant`` and
``slowquant.hartreefock.hartreefock_in_memory`` as a SlowQuant user would, and
follow the call sequences of the reference's own tests:

* tests/test_hartreefock.py:4-80 -- SlowQuant(), set_molecule(..., bohr),
  set_basis_set, init_hartree_fock, run_restricted_hartree_fock; nuclear
  repulsion and E_hf against the published energies (1e-6);
* tests/test_integral.py:7-68 -- the H6/DZP chain's ERI tensor at Schwarz
  thresholds 1e-8, 1e-3 (within the threshold of the unscreened tensor) and
  1e10 (all zero);
* the free function run_hartree_fock(S, T, V, ERI, Ne, log, ...) of
  hartreefock_in_memory.py:7-18 on the stored tensor, and DIIS from diis.py.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WATER = """O 0.000000000000  -0.143225816552   0.000000000000;
           H 1.638036840407   1.136548822547  -0.000000000000;
           H -1.638036840407   1.136548822547  -0.000000000000;"""
METHANE = """C  -0.000000000000   0.000000000000   0.000000000000;
           H   1.183771681898  -1.183771681898  -1.183771681898;
           H   1.183771681898   1.183771681898   1.183771681898;
           H  -1.183771681898   1.183771681898  -1.183771681898;
           H  -1.183771681898  -1.183771681898   1.183771681898"""
# published energies quoted by the reference's tests (tests/test_hartreefock.py:19-79)
CASES = [(WATER, "sto-3g", 8.0023670618, -82.944446990003), (WATER, "dz", 8.0023670618, -83.980246037187),
         (WATER, "dzp", 8.0023670618, -84.01054766778844), (METHANE, "sto-3g", 13.4973044620, -53.224154786383)]
CHAIN = ";".join(f"H {x:.12f} 0.000000000000 0.000000000000" for x in range(6))


@pytest.fixture
def slowquant_names(gpu_lib):
    from slowquant_gb300 import dropin

    saved = dropin.install()
    try:
        yield
    finally:
        dropin.uninstall(saved)


@pytest.mark.parametrize("geom,basis,enuc,ehf", CASES)
def test_reference_hartree_fock_calls(slowquant_names, geom, basis, enuc, ehf):
    import slowquant.SlowQuant as sq

    A = sq.SlowQuant()
    A.set_molecule(geom, distance_unit="bohr")
    A.set_basis_set(basis)
    A.init_hartree_fock()
    A.hartree_fock.logger.print_output = False
    A.hartree_fock.run_restricted_hartree_fock()
    assert type(A).__module__ == "slowquant_gb300.SlowQuant"
    assert abs(A.molecule.nuclear_repulsion - enuc) < 1e-6
    assert abs(A.hartree_fock.E_hf - ehf) < 1e-6


def test_reference_screening_calls(slowquant_names):
    import slowquant.SlowQuant as sq

    def tensor(threshold):
        A = sq.SlowQuant()
        A.set_molecule(CHAIN, distance_unit="bohr")
        A.set_basis_set("dzp")
        A.integral.cauchy_schwarz_threshold = threshold
        return A.integral.electron_repulsion_tensor

    ref = tensor(1e-20)
    np.testing.assert_allclose(tensor(1e-8), ref, atol=1e-8)
    np.testing.assert_allclose(tensor(1e-3), ref, atol=1e-3)
    np.testing.assert_allclose(tensor(1e10), np.zeros(np.shape(ref)), atol=1e-8)


def test_reference_free_functions(slowquant_names):
    import slowquant.SlowQuant as sq
    from slowquant.hartreefock.diis import DIIS
    from slowquant.hartreefock.hartreefock_in_memory import run_hartree_fock
    from slowquant.logger import _Logger

    A = sq.SlowQuant()
    A.set_molecule(WATER, distance_unit="bohr")
    A.set_basis_set("sto-3g")
    log = _Logger()
    log.print_output = False
    E, C, F, D = run_hartree_fock(A.integral.overlap_matrix, A.integral.kinetic_energy_matrix,
                                  A.integral.nuclear_attraction_matrix, A.integral.electron_repulsion_tensor,
                                  A.molecule.number_electrons, log, 1e-9, 1e-9, 100, True)
    assert abs(E - (-82.944446990003)) < 1e-6  # electronic energy, as E_hf
    assert isinstance(D, np.ndarray) and D.shape == (7, 7)
    assert DIIS(7).get_extrapolated_fock_matrix is not None
