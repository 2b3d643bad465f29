"""Multipole integrals against the reference's own matrices.

tests/golden/multipole.npz holds the unmodified reference's
get_multipole_matrix (integralclass.py:99-108 -> multipole.py:10-135, about
its centre of mass) for water in 6-31G* and H2O2 in cc-pVTZ (f shells):
dipoles, quadrupoles and mixed orders up to (1, 2, 3).
"""

import numpy as np
import pytest

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tag", ["h2o_631gs", "h2o2_ccpvtz"])
def test_multipole_matrices_match_reference(gpu_lib, tag):
    import slowquant_gb300.SlowQuant as sq

    g = load_golden("multipole")
    A = sq.SlowQuant()
    A.set_molecule(str(g[f"{tag}_geometry"]), distance_unit=str(g[f"{tag}_unit"]))
    A.set_basis_set(str(g[f"{tag}_basis"]))
    np.testing.assert_allclose(A.molecule.center_of_mass, g[f"{tag}_com"], atol=1e-12)
    for order, ref in zip(g[f"{tag}_orders"], g[f"{tag}_M"]):
        M = A.integral.get_multipole_matrix(order)
        np.testing.assert_allclose(M, ref, atol=1e-10 * max(1.0, np.abs(ref).max()), err_msg=str(order))
    # order (0, 0, 0) is the overlap
    np.testing.assert_allclose(A.integral.get_multipole_matrix([0, 0, 0]), A.integral.overlap_matrix, atol=1e-12)
