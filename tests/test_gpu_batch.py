"""Batched SCF over independent molecules of uneven size against single-molecule SCF."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mols(sizes, basis="6-31G*"):
    from slowquant_gb300 import systems
    from slowquant_gb300.molecule import _Molecule

    out = []
    for i, n in enumerate(sizes):
        box = 9.0 * (n / 8.0) ** (1.0 / 3.0) + 1.0
        m = _Molecule(systems.water_cluster(n, box, seed=100 + i), 0, "angstrom")
        m._set_basis_set(basis)
        out.append(m)
    return out


def _single_energy(m):
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.hartreefock import DirectJK, run_hartree_fock
    from slowquant_gb300.logger import _Logger

    eng = IntegralEngine(m)
    S, T, V = eng.one_electron()
    log = _Logger()
    log.print_output = False
    return run_hartree_fock(S, T, V, DirectJK(eng), m.number_electrons, log, 1e-10, 1e-10, 100, True)[0]


@pytest.mark.parametrize("use_graphs", [False, True])
def test_batch_energies_match_single_molecule(gpu_lib, use_graphs):
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    sizes = [2, 1, 3, 1, 2]
    mols = _mols(sizes)
    be = BatchEngine(mols)
    E = BatchSCF(be, "fp64", use_graphs=use_graphs).run(1e-10, 1e-10)
    ref = np.array([_single_energy(m) for m in mols])
    np.testing.assert_allclose(E, ref, atol=1e-8)


def test_batch_one_electron_blocks(gpu_lib):
    from slowquant_gb300.batch import BatchEngine
    from slowquant_gb300.engine import IntegralEngine

    mols = _mols([1, 2])
    be = BatchEngine(mols)
    S, T, V = be.one_electron()
    for mi, m in enumerate(be.mols):
        n = m.number_bf
        blk = slice(be.mol_base[mi], be.mol_base[mi] + n * n)
        Sr, Tr, Vr = IntegralEngine(m).one_electron()
        np.testing.assert_allclose(S[blk].view(n, n).cpu().numpy(), Sr.cpu().numpy(), atol=1e-12)
        np.testing.assert_allclose(T[blk].view(n, n).cpu().numpy(), Tr.cpu().numpy(), atol=1e-12)
        np.testing.assert_allclose(V[blk].view(n, n).cpu().numpy(), Vr.cpu().numpy(), atol=1e-11)


def test_batch_mixed_precision(gpu_lib):
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    mols = _mols([3, 2, 4])
    be = BatchEngine(mols)
    E64 = BatchSCF(be, "fp64").run()
    scf = BatchSCF(be, "mixed", fp32_threshold=1e-4)
    Em = scf.run()
    assert scf.builds[0] == "mixed" and scf.builds[-1] == "fp64"
    assert np.max(np.abs(Em - E64)) < 1e-6


@pytest.mark.parametrize("precision", ["df64", "mixed_df"])
def test_batch_double_float_modes(gpu_lib, precision):
    """Double-float arithmetic in place of FP64 on a packed batch: the FP64 batch energies
    (1e-9 Eh for df64; mixed_df ends in df64 after its mixed phase, 1e-8 Eh)."""
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    mols = _mols([3, 1, 4, 2])
    be = BatchEngine(mols)
    E64 = BatchSCF(be, "fp64").run(1e-10, 1e-10)
    scf = BatchSCF(be, precision, fp32_threshold=1e-3)
    E = scf.run(1e-10, 1e-10)
    if precision == "mixed_df":
        assert scf.builds[0] == "mixed" and scf.builds[-1] == "fp64"  # the batch's phase names
    assert np.max(np.abs(E - E64)) < (1e-9 if precision == "df64" else 1e-8)


@pytest.mark.parametrize("dims", [[1, 2, 7, 19, 38, 57, 114, 128],  # eigenvectors rotated in global memory
                                  [3, 18, 55, 76, 95, 114, 118]])     # eigenvectors in shared memory
def test_batched_eigh_ragged_matches_numpy(gpu_lib, dims):
    """sq_batched_eigh on matrices of mixed sizes against numpy eigh."""
    import torch

    from slowquant_gb300 import _lib

    rng = np.random.default_rng(3)
    offs = np.concatenate([[0], np.cumsum([d * d for d in dims])[:-1]]).astype(np.int64)
    woff = np.concatenate([[0], np.cumsum(dims)[:-1]]).astype(np.int64)
    mats = []
    for d in dims:
        M = rng.normal(size=(d, d))
        mats.append((M + M.T) / 2)
    A = torch.tensor(np.concatenate([m.ravel() for m in mats]), dtype=torch.float64, device="cuda")
    V = torch.zeros_like(A)
    W = torch.zeros(sum(dims), dtype=torch.float64, device="cuda")
    # every argument tensor stays referenced until the results are read back
    t_off = torch.tensor(offs, device="cuda")
    t_dims = torch.tensor(np.array(dims, np.int32), device="cuda")
    t_woff = torch.tensor(woff, device="cuda")
    sweeps = torch.zeros(len(dims), dtype=torch.int32, device="cuda")
    _lib.check(_lib.lib().sq_batched_eigh(len(dims), t_off.data_ptr(), t_dims.data_ptr(), max(dims), A.data_ptr(),
                                          W.data_ptr(), V.data_ptr(), t_woff.data_ptr(), 1e-15, 40,
                                          sweeps.data_ptr(), _lib.stream_handle()), "sq_batched_eigh")
    torch.cuda.synchronize()
    Wh, Vh, sw = W.cpu().numpy(), V.cpu().numpy(), sweeps.cpu().numpy()
    assert np.all(sw >= 0) and np.all(sw < 40)
    for i, d in enumerate(dims):
        w = Wh[woff[i]:woff[i] + d]
        v = Vh[offs[i]:offs[i] + d * d].reshape(d, d)
        wr = np.linalg.eigvalsh(mats[i])
        np.testing.assert_allclose(w, wr, atol=1e-12 * max(1.0, np.abs(wr).max()))
        # eigenvector residual and orthonormality
        np.testing.assert_allclose(mats[i] @ v, v * w[None, :], atol=1e-11)
        np.testing.assert_allclose(v.T @ v, np.eye(d), atol=1e-12)


def test_batched_eigh_helper_uniform_stack(gpu_lib):
    import torch

    from slowquant_gb300.batch import batched_eigh

    rng = np.random.default_rng(5)
    M = rng.normal(size=(16, 66, 66))
    M = (M + M.transpose(0, 2, 1)) / 2
    Mt = torch.tensor(M, device="cuda")
    W, V = batched_eigh(Mt)
    W, V = W.cpu().numpy(), V.cpu().numpy()
    np.testing.assert_allclose(W, np.linalg.eigvalsh(M), atol=1e-12)
    np.testing.assert_allclose(M @ V, V * W[:, None, :], atol=1e-11)


def test_autotuned_launch_shapes_keep_results(gpu_lib):
    """The autotuner's launch shapes change timing only: batch energies stay the same."""
    from slowquant_gb300 import autotune
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    mols = _mols([2, 1, 3])
    be = BatchEngine(mols)
    E0 = BatchSCF(be, "mixed").run()
    scf = BatchSCF(be, "mixed")
    try:
        table = scf.autotune(threads=(64, 128), waves=(1, 8))
        assert table and all(ms > 0 for _, _, ms in table.values())
        E1 = scf.run()
    finally:
        autotune.reset()
    np.testing.assert_allclose(E1, E0, atol=1e-9)


def test_batch_of_one_molecule(gpu_lib):
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    mols = _mols([2])
    E = BatchSCF(BatchEngine(mols), "fp64").run(1e-10, 1e-10)
    np.testing.assert_allclose(E, [_single_energy(mols[0])], atol=1e-8)


def test_captured_iterations_replay_and_match_eager_iterations(gpu_lib):
    """Whole SCF iterations replayed from CUDA graphs give the eager iterations' energies and
    iteration counts; a second run replays the first run's graphs; the host reads the
    convergence flag only every few iterations."""
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    be = BatchEngine(_mols([2, 1, 3, 2]))
    for prec in ("fp64", "mixed"):
        eager = BatchSCF(be, prec, use_graphs=False)
        E_eager = eager.run()
        scf = BatchSCF(be, prec, check_every=4)
        E1 = scf.run()
        graphs = dict(scf.graphs)
        E2 = scf.run()
        np.testing.assert_allclose(E1, E_eager, atol=1e-10)
        np.testing.assert_allclose(E2, E1, atol=1e-12)
        assert scf.iterations == eager.iterations
        assert all(scf.graphs[k] is graphs[k] for k in graphs)  # replayed, not captured again
        if prec == "fp64":
            assert scf.host_syncs < scf.iterations
