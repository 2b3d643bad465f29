"""RHF through the reference's public API on the GPU path.

Energies: 1e-8 Eh against the reference's own outputs (golden), 1e-6 Eh
against the reference test suite's literature values.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KNOWN = {
    "h2o_sto3g_crawford": -82.944446990003,
    "h2o_dz": -83.980246037187,
    "h2o_dzp": -84.01054766778844,
    "ch4_sto3g": -53.224154786383,
}


def _run(geom, basis, unit, **kw):
    import slowquant_gb300.SlowQuant as sq

    A = sq.SlowQuant()
    A.set_molecule(geom, distance_unit=unit)
    A.set_basis_set(basis)
    A.init_hartree_fock()
    A.hartree_fock.logger.print_output = False
    for k, v in kw.items():
        setattr(A.hartree_fock, k, v)
    A.hartree_fock.run_restricted_hartree_fock()
    return A


@pytest.mark.parametrize("name", ["h2o_sto3g_crawford", "h2o_sto3g_c1", "ch4_sto3g", "h2o_631gs", "h2o_dz",
                                  "h2o_ccpvdz_c1", "h2o_dzp", "h6_dzp"])
def test_rhf_energy_direct(name, gpu_lib, golden_energies):
    e = golden_energies[name]
    A = _run(e["geometry"], e["basis"], e["unit"])
    assert abs(A.molecule.nuclear_repulsion - e["E_nuc"]) < 1e-10
    assert abs(A.hartree_fock.E_hf - e["E_hf"]) < 1e-8
    if name in KNOWN:
        assert abs(A.hartree_fock.E_hf - KNOWN[name]) < 1e-6
    assert A.hartree_fock.rdm1.shape == (e["nbf"], e["nbf"])


@pytest.mark.parametrize("name", ["h2o_sto3g_crawford", "h2o_631gs"])
def test_rhf_energy_stored_tensor_path(name, gpu_lib, golden_energies):
    e = golden_energies[name]
    A = _run(e["geometry"], e["basis"], e["unit"], direct_jk=False)
    assert abs(A.hartree_fock.E_hf - e["E_hf"]) < 1e-8


def test_run_hartree_fock_signature_with_numpy_inputs(gpu_lib, golden_energies):
    from slowquant_gb300.hartreefock import run_hartree_fock
    from slowquant_gb300.logger import _Logger
    from tests.conftest import load_golden

    e = golden_energies["h2o_sto3g_crawford"]
    d = load_golden("h2o_sto3g_crawford")
    log = _Logger()
    log.print_output = False
    E, C, F, D = run_hartree_fock(d["S"], d["T"], d["V"], d["eri"], 10, log, 1e-9, 1e-9, 100, True)
    assert abs(E - e["E_hf"]) < 1e-9
    np.testing.assert_allclose(D, d["D"], atol=1e-7)
    assert "Iter" in log.log


def test_mixed_precision_energy(gpu_lib):
    from slowquant_gb300 import systems

    g = systems.water_cluster(2, 5.0, seed=2)
    ref = _run(g, "cc-pvdz", "angstrom").hartree_fock.E_hf
    for prec in ("mixed", "mixed_boys32"):
        A = _run(g, "cc-pvdz", "angstrom", precision=prec, fp32_schwarz_threshold=1e-4)
        builds = A.hartree_fock.fock_builds
        assert builds[0] != "fp64" and builds[-1] == "fp64"
        assert abs(A.hartree_fock.E_hf - ref) < 1e-6


UHF_KNOWN = {  # E_uhf + E_nuc from the reference's tests/test_unrestrictedhartreefock.py
    "uhf_n2_631gs": (-108.942686389118, 1e-6),
    "uhf_n2cation_631gs": (-108.36597, 1e-5),
    "uhf_li_631gss": (-7.4313707537, 1e-5),
}


def _run_uhf(e, **kw):
    import slowquant_gb300.SlowQuant as sq

    A = sq.SlowQuant()
    A.set_molecule(e["geometry"], distance_unit=e["unit"])
    A.set_basis_set(e["basis"])
    A.molecule.molecular_charge = e["charge"]
    A.init_hartree_fock()
    A.hartree_fock.logger.print_output = False
    A.hartree_fock.uhf_lumo_homo_mix_coeff = e["mix"]
    for k, v in kw.items():
        setattr(A.hartree_fock, k, v)
    A.hartree_fock.run_unrestricted_hartree_fock()
    return A


@pytest.mark.parametrize("name", ["uhf_h2o_sto3g_mix0", "uhf_n2_631gs", "uhf_n2cation_631gs", "uhf_li_631gss"])
def test_uhf_energy_direct(name, gpu_lib, golden_energies):
    from tests.conftest import load_golden

    e = golden_energies[name]
    d = load_golden(name)
    A = _run_uhf(e)
    hf = A.hartree_fock
    assert abs(hf.E_uhf - e["E_uhf"]) < 1e-8
    np.testing.assert_allclose(hf.rdm1_alpha, d["D_alpha"], atol=1e-6)
    np.testing.assert_allclose(hf.rdm1_beta, d["D_beta"], atol=1e-6)
    np.testing.assert_allclose(hf.rdm1_charge, d["D_alpha"] + d["D_beta"], atol=2e-6)
    np.testing.assert_allclose(hf.rdm1_spin, d["D_alpha"] - d["D_beta"], atol=2e-6)
    if name in UHF_KNOWN:
        ref, tol = UHF_KNOWN[name]
        assert abs(hf.E_uhf + A.molecule.nuclear_repulsion - ref) < tol
    # <S^2> contamination is non-negative; zero for the closed-shell solutions
    assert hf.spin_contamination > -1e-8
    if name in ("uhf_h2o_sto3g_mix0", "uhf_n2_631gs"):
        assert abs(hf.spin_contamination) < 1e-6


def test_uhf_equals_rhf_closed_shell_and_stored_tensor(gpu_lib, golden_energies):
    e = golden_energies["uhf_h2o_sto3g_mix0"]
    A = _run_uhf(e, direct_jk=False)
    A.hartree_fock.run_restricted_hartree_fock()
    assert abs(A.hartree_fock.E_uhf - e["E_uhf"]) < 1e-8
    assert abs(A.hartree_fock.E_hf - A.hartree_fock.E_uhf) < 1e-6


def test_uhf_mixed_precision(gpu_lib, golden_energies):
    e = golden_energies["uhf_n2cation_631gs"]
    A = _run_uhf(e, precision="mixed", fp32_schwarz_threshold=1e-4)
    builds = A.hartree_fock.fock_builds
    assert builds[0] == "mixed" and builds[-1] == "fp64"
    assert abs(A.hartree_fock.E_uhf - e["E_uhf"]) < 1e-6


def test_ao_to_mo_transforms_match_einsum(gpu_lib, golden_energies):
    """integralfunctions.py:186-211 against the reference's einsum contractions."""
    from slowquant_gb300.integralfunctions import one_electron_integral_transform, two_electron_integral_transform

    e = golden_energies["h2o_631gs"]
    A = _run(e["geometry"], e["basis"], e["unit"])
    C = A.hartree_fock.mo_coeff
    h = A.integral.kinetic_energy_matrix + A.integral.nuclear_attraction_matrix
    g = A.integral.electron_repulsion_tensor
    h_mo = one_electron_integral_transform(C, h)
    g_mo = two_electron_integral_transform(C, g)
    np.testing.assert_allclose(h_mo, np.einsum("ai,bj,ab->ij", C, C, h), atol=1e-11)
    ref = np.einsum("ai,bj,ck,dl,abcd->ijkl", C, C, C, C, g, optimize=True)
    np.testing.assert_allclose(g_mo, ref, atol=1e-11)
    # a rectangular (active-space) C as well
    Ca = C[:, 2:9]
    np.testing.assert_allclose(two_electron_integral_transform(Ca, g),
                               np.einsum("ai,bj,ck,dl,abcd->ijkl", Ca, Ca, Ca, Ca, g, optimize=True), atol=1e-11)


def test_dense_jk_kernel_matches_einsum(gpu_lib):
    """sq_jk_dense (one pass over the stored tensor) against the reference's two einsums,
    with D in shared memory (n = 37) and read through the caches (n = 120)."""
    import torch

    from slowquant_gb300.hartreefock import dense_jk

    rng = np.random.default_rng(6)
    for n in (37, 120):
        G = torch.tensor(rng.standard_normal((n, n, n, n)), device="cuda")
        D = torch.tensor(rng.standard_normal((n, n)), device="cuda")
        J, K = dense_jk(G, D)
        Jr = torch.einsum("pqrs,sr->pq", G, D)
        Kr = torch.einsum("psqr,sr->pq", G, D)
        torch.testing.assert_close(J, Jr, rtol=0, atol=1e-10 * float(Jr.abs().max()))
        torch.testing.assert_close(K, Kr, rtol=0, atol=1e-10 * float(Kr.abs().max()))


def test_ao_to_mo_rotate_kernel_ragged_sizes(gpu_lib):
    """sq_ao2mo_rotate at sizes that are not multiples of its 64 x 64 x 16 tiles, against numpy."""
    import torch

    from slowquant_gb300.integralfunctions import one_electron_integral_transform, two_electron_integral_transform

    rng = np.random.default_rng(4)
    for n, m in ((37, 23), (17, 17), (65, 3), (5, 70)):
        C = rng.standard_normal((n, m))
        g = rng.standard_normal((n, n, n, n)) if n <= 40 else None
        h = rng.standard_normal((n, n))
        np.testing.assert_allclose(one_electron_integral_transform(C, h), C.T @ h @ C, atol=1e-11)
        if g is not None:
            ref = np.einsum("ai,bj,ck,dl,abcd->ijkl", C, C, C, C, g, optimize=True)
            out = two_electron_integral_transform(torch.tensor(C, device="cuda"), torch.tensor(g, device="cuda"))
            assert isinstance(out, torch.Tensor)
            np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-9 * np.abs(ref).max())


H6_BOHR = ";".join(f"H   {float(i):.12f}   0.000000000000   0.000000000000" for i in range(6))


def _h6_tensor(threshold):
    import slowquant_gb300.SlowQuant as sq

    A = sq.SlowQuant()
    A.set_molecule(H6_BOHR, distance_unit="bohr")
    A.set_basis_set("dzp")
    A.integral.cauchy_schwarz_threshold = threshold
    return A.integral.electron_repulsion_tensor


def test_cauchy_schwarz_inequality_like_reference(gpu_lib):
    """The reference's tests/test_integral.py case: H6 chain in DZP, screened tensors stay
    within the threshold of the (almost) unscreened one, and a huge threshold gives zeros."""
    ref = _h6_tensor(1e-20)
    np.testing.assert_allclose(_h6_tensor(1e-8), ref, atol=1e-8)
    np.testing.assert_allclose(_h6_tensor(1e-3), ref, atol=1e-3)
    np.testing.assert_allclose(_h6_tensor(1e10), np.zeros(ref.shape), atol=1e-8)


def test_edge_cases_small_systems(gpu_lib):
    """H2 (two basis functions: DIIS passes F through), a lone H atom in UHF, and a
    J/K build whose screening removes every quartet."""
    import torch

    from oracle import oracle as O

    # H2 STO-3G RHF against the oracle (nbf = 2 -> the reference's DIIS returns F unchanged)
    geom = "H 0.0 0.0 0.0;H 1.4 0.0 0.0"
    A = _run(geom, "sto-3g", "bohr")
    o = O.OracleMolecule(geom, "sto-3g", "bohr")
    V = o.eri_dense(1e-12)
    S, T, Vn = o.one_electron()
    E_ref = O.run_hartree_fock(S, T, Vn, lambda D: O.jk_from_eri(V, D), o.number_electrons)[0]
    assert A.molecule.number_bf == 2
    assert abs(A.hartree_fock.E_hf - E_ref) < 1e-8
    # a lone H atom: one alpha electron, no beta electrons
    e = {"geometry": "H 0.0 0.0 0.0;", "unit": "bohr", "basis": "6-31G", "charge": 0, "mix": 0.15}
    B = _run_uhf(e)
    o = O.OracleMolecule(e["geometry"], e["basis"], "bohr")
    V = o.eri_dense(1e-12)
    S, T, Vn = o.one_electron()
    E_u = O.run_unrestricted_hartree_fock(S, T, Vn, lambda D: O.jk_from_eri(V, D), 1, 0)[0]
    assert abs(B.hartree_fock.E_uhf - E_u) < 1e-8
    np.testing.assert_allclose(B.hartree_fock.rdm1_beta, 0.0, atol=1e-14)
    # screening that keeps nothing: J = K = 0
    eng = B.integral.engine
    D = torch.eye(eng.nbf, dtype=torch.float64, device="cuda")
    J, K = eng.jk(D, 1e30, "mixed", 1e-4)
    assert float(J.abs().max()) == 0.0 and float(K.abs().max()) == 0.0


def test_torch_operators_match_the_package_calls(gpu_lib):
    """torch.ops.slowquant_gb300.* give the package functions' results on CUDA tensors."""
    import torch

    import slowquant_gb300.torch_ops as ops
    from slowquant_gb300 import systems
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.hartreefock import dense_jk
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(systems.water_monomer(), 0, "angstrom")
    m._set_basis_set("6-31G*")
    eng = IntegralEngine(m)
    V = eng.eri_dense(1e-12)
    rng = np.random.default_rng(8)
    C = rng.standard_normal((eng.nbf, eng.nbf // 2))
    D = torch.tensor(2 * C @ C.T, device="cuda")
    Jo, Ko = torch.ops.slowquant_gb300.jk_dense(V, D)
    Jd, Kd = dense_jk(V, D)
    torch.testing.assert_close(Jo, Jd, rtol=0, atol=0)
    h = ops.register_engine(eng)
    Jx, Kx = torch.ops.slowquant_gb300.direct_jk(h, D, 1e-12, "fp64", 1e-4)
    torch.testing.assert_close(Jx, Jd, rtol=0, atol=1e-10)
    torch.testing.assert_close(Kx, Kd, rtol=0, atol=1e-10)
    Ct = torch.tensor(C, device="cuda")
    torch.testing.assert_close(torch.ops.slowquant_gb300.ao2mo(Ct, V),
                               torch.einsum("ai,bj,ck,dl,abcd->ijkl", Ct, Ct, Ct, Ct, V), rtol=0, atol=1e-10)
