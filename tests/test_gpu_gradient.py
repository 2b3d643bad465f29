"""Adjoint RHF nuclear gradients against finite differences.

The reference has no gradients; its energies are the check: central finite
differences (step 1e-4 bohr) of the oracle's energies, which reproduce the
reference's own energies to 1e-14 Eh.  Tolerance 1e-6 Eh/bohr.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

H2O_BOHR = [("O", (0.0, -0.143225816552, 0.0)), ("H", (1.638036840407, 1.136548822547, 0.0)),
            ("H", (-1.638036840407, 1.136548822547, 0.0))]


def _geom(symbols, xyz):
    return ";".join(f"{s} {x:.17g} {y:.17g} {z:.17g}" for s, (x, y, z) in zip(symbols, xyz))


def oracle_energy(symbols, xyz, basis):
    m = O.OracleMolecule(_geom(symbols, xyz), basis, "bohr")
    V = m.eri_dense(1e-14)
    S, T, Vn = m.one_electron()
    E = O.run_hartree_fock(S, T, Vn, lambda D: O.jk_from_eri(V, D), m.number_electrons, 1e-13, 1e-11, 200)[0]
    return E + m.nuclear_repulsion


def fd_gradient(symbols, xyz, basis, comps=None, h=1e-4):
    xyz = np.array(xyz, dtype=np.float64)
    g = np.full(xyz.shape, np.nan)
    comps = comps or [(a, d) for a in range(len(xyz)) for d in range(3)]
    for a, d in comps:
        xp = xyz.copy()
        xm = xyz.copy()
        xp[a, d] += h
        xm[a, d] -= h
        g[a, d] = (oracle_energy(symbols, xp, basis) - oracle_energy(symbols, xm, basis)) / (2 * h)
    return g


def gpu_gradient(symbols, xyz, basis):
    from slowquant_gb300.gradient import molecule_from_coords, rhf_gradient

    return rhf_gradient(molecule_from_coords(symbols, xyz, basis), conv=1e-11)


@pytest.mark.parametrize("basis", ["sto-3g", "6-31G*", "cc-pvdz"])
def test_water_gradient_matches_fd_of_reference_energies(basis, gpu_lib):
    symbols = [s for s, _ in H2O_BOHR]
    xyz = [list(c) for _, c in H2O_BOHR]
    xyz[1][2] += 0.05  # break the symmetry so every component is non-zero
    g = gpu_gradient(symbols, xyz, basis)
    fd = fd_gradient(symbols, xyz, basis)
    np.testing.assert_allclose(g, fd, atol=1e-6)
    np.testing.assert_allclose(g.sum(axis=0), 0.0, atol=1e-8)


def test_f_shell_gradient_matches_fd_of_reference_energies(gpu_lib):
    """cc-pVTZ puts f shells on O: every f class of the adjoint kernels, (ff|ff)
    on one-warp blocks, the high-order Boys grid for m > 8 and the
    one-electron kernel at l = 3, against finite differences of the oracle."""
    symbols = [s for s, _ in H2O_BOHR]
    xyz = [list(c) for _, c in H2O_BOHR]
    xyz[1][2] += 0.05
    g = gpu_gradient(symbols, xyz, "cc-pvtz")
    fd = fd_gradient(symbols, xyz, "cc-pvtz")
    np.testing.assert_allclose(g, fd, atol=1e-6)
    np.testing.assert_allclose(g.sum(axis=0), 0.0, atol=1e-8)


def test_f_shell_gradient_per_thread_classes_match_warp_kernel(gpu_lib):
    """With f shells present, the light classes on per-thread kernels == all on the warp kernel."""
    from slowquant_gb300 import _lib
    from slowquant_gb300.gradient import molecule_from_coords, rhf_gradient

    symbols = [s for s, _ in H2O_BOHR]
    xyz = [list(c) for _, c in H2O_BOHR]
    xyz[2][2] -= 0.03
    m = molecule_from_coords(symbols, xyz, "cc-pvtz")
    L = _lib.lib()
    try:
        _lib.check(L.sq_set_option(_lib.SQ_OPT_GRAD_THREAD, 0), "sq_set_option")
        g_warp = rhf_gradient(m, conv=1e-11)
        _lib.check(L.sq_set_option(_lib.SQ_OPT_GRAD_THREAD, 1), "sq_set_option")
        g_thread = rhf_gradient(m, conv=1e-11)
    finally:
        L.sq_set_option(_lib.SQ_OPT_GRAD_THREAD, 1)
    np.testing.assert_allclose(g_thread, g_warp, atol=1e-10)


def test_water_dimer_gradient_multicentre(gpu_lib):
    from slowquant_gb300 import systems
    from slowquant_gb300.molecule import ANGSTROM_TO_BOHR

    geom = systems.water_cluster(2, 5.0, seed=2)
    symbols = [a.split()[0] for a in geom.split(";")]
    xyz = np.array([[float(v) * ANGSTROM_TO_BOHR for v in a.split()[1:]] for a in geom.split(";")])
    g = gpu_gradient(symbols, xyz, "cc-pvdz")
    comps = [(0, 0), (1, 1), (3, 2), (5, 0)]
    fd = fd_gradient(symbols, xyz, "cc-pvdz", comps)
    for a, d in comps:
        assert abs(g[a, d] - fd[a, d]) < 1e-6, (a, d, g[a, d], fd[a, d])
    np.testing.assert_allclose(g.sum(axis=0), 0.0, atol=1e-8)


def test_hydrogen_chain_gradient(gpu_lib):
    from slowquant_gb300 import systems
    from slowquant_gb300.molecule import ANGSTROM_TO_BOHR

    geom = systems.hydrogen_chain(12, seed=24)
    xyz = np.array([[float(v) * ANGSTROM_TO_BOHR for v in a.split()[1:]] for a in geom.split(";")])
    symbols = ["H"] * len(xyz)
    g = gpu_gradient(symbols, xyz, "sto-3g")
    comps = [(0, 0), (5, 0), (11, 0)]
    fd = fd_gradient(symbols, xyz, "sto-3g", comps)
    for a, d in comps:
        assert abs(g[a, d] - fd[a, d]) < 1e-6
    np.testing.assert_allclose(g[:, 1:], 0.0, atol=1e-9)  # linear chain: no transverse force


def test_autograd_function_backward(gpu_lib):
    import torch

    from slowquant_gb300.gradient import rhf_energy

    symbols = [s for s, _ in H2O_BOHR]
    xyz = torch.tensor([list(c) for _, c in H2O_BOHR], dtype=torch.float64, requires_grad=True)
    E = rhf_energy(xyz, symbols, "sto-3g")
    E.backward()
    assert abs(float(E) - (-82.94444701585452 + 8.00236706181077)) < 1e-7
    g_ref = gpu_gradient(symbols, xyz.detach().numpy(), "sto-3g")
    np.testing.assert_allclose(xyz.grad.numpy(), g_ref, atol=1e-10)


def test_per_thread_gradient_classes_match_warp_kernel(gpu_lib):
    """The light classes' per-thread gradient kernels == the warp kernel (all classes)."""
    from slowquant_gb300 import _lib, systems
    from slowquant_gb300.gradient import rhf_gradient
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(systems.water_cluster(2, 5.0, seed=2), 0, "angstrom")
    m._set_basis_set("cc-pvdz")
    L = _lib.lib()
    try:
        _lib.check(L.sq_set_option(_lib.SQ_OPT_GRAD_THREAD, 0), "sq_set_option")
        g_warp = rhf_gradient(m, conv=1e-11)
        _lib.check(L.sq_set_option(_lib.SQ_OPT_GRAD_THREAD, 1), "sq_set_option")
        g_thread = rhf_gradient(m, conv=1e-11)
    finally:
        L.sq_set_option(_lib.SQ_OPT_GRAD_THREAD, 1)
    np.testing.assert_allclose(g_thread, g_warp, atol=1e-10)
