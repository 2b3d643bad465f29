"""Restricted and unrestricted Hartree-Fock on the GPU: SCF loops, DIIS, the HF class.

Drop-in for slowquant/hartreefock/{hartreefock_in_memory.py,
unrestricted_hartreefock_in_memory.py, diis.py,
hartreefockclass.py}: same names, arguments, iteration semantics and log lines.
Linear algebra runs on the device in FP64 (torch: cuSOLVER eigh, cuBLAS
products).  The two-electron part comes either from a dense ERI tensor (the
reference's einsums, hartreefock_in_memory.py:55-56, as one pass of the
library's ``sq_jk_dense`` over the tensor) or from the integral-direct J/K
kernels (``DirectJK``), optionally in mixed precision.
"""

from __future__ import annotations

import numpy as np
import torch

from .logger import _Logger


def dense_jk(G: torch.Tensor, D: torch.Tensor):
    """J = einsum("pqrs,sr->pq", G, D) and K = einsum("psqr,sr->pq", G, D)
    (hartreefock_in_memory.py:55-56) from a stored (n,)*4 tensor in one pass over it
    (the library's sq_jk_dense)."""
    from . import _lib

    n = G.shape[0]
    G = G.contiguous()
    D = D.to(dtype=torch.float64).contiguous()
    J = torch.empty((n, n), dtype=torch.float64, device=G.device)
    K = torch.empty_like(J)
    _lib.check(_lib.lib().sq_jk_dense(n, _lib.ptr(G), _lib.ptr(D), _lib.ptr(J), _lib.ptr(K), _lib.stream_handle()),
               "sq_jk_dense")
    return J, K


def _dev_tensor(x, device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float64)
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device=device)


class DIIS:
    """Pulay DIIS with error FDS - SDF (slowquant/hartreefock/diis.py:4-66)."""

    def __init__(self, number_bf: int, number_fock_saved_: int = 6) -> None:
        self.fock_matrices: list[torch.Tensor] = []
        self.density_matrices: list[torch.Tensor] = []
        self.error_matrices: list[torch.Tensor] = []
        self.number_fock_saved = number_fock_saved_
        self.num_bf = number_bf
        self.last_error: float | None = None

    def get_extrapolated_fock_matrix(self, fock_matrix, density_matrix, S):
        if len(fock_matrix) == 2:
            return fock_matrix
        err = fock_matrix @ density_matrix @ S - S @ density_matrix @ fock_matrix
        self.last_error = float(err.abs().max())
        self.fock_matrices.append(fock_matrix)
        self.density_matrices.append(density_matrix)
        self.error_matrices.append(err)
        if len(self.fock_matrices) == 1:
            return fock_matrix
        if len(self.fock_matrices) > self.number_fock_saved:
            self.fock_matrices.pop(0)
            self.density_matrices.pop(0)
            self.error_matrices.pop(0)
        m = len(self.fock_matrices)
        E = torch.stack(self.error_matrices)  # [m, n, n]
        # B_ij = trace(e_i e_j) = sum_pq e_i[p,q] e_j[q,p]
        Bm = torch.einsum("ipq,jqp->ij", E, E)
        B = torch.zeros((m + 1, m + 1), dtype=torch.float64, device=E.device)
        B[-1, :] = -1
        B[:, -1] = -1
        B[-1, -1] = 0
        B[:m, :m] = Bm
        b0 = torch.zeros(m + 1, dtype=torch.float64, device=E.device)
        b0[-1] = -1
        coefficients = torch.linalg.solve(B, b0)
        return torch.einsum("i,ipq->pq", coefficients[:-1], torch.stack(self.fock_matrices))


class DirectJK:
    """Integral-direct J/K callable for run_hartree_fock.

    precision: "fp64", "mixed" (quartets with Schwarz bound < fp32_threshold in
    FP32 with FP64 Boys recursion), "mixed_boys32", "mixed_chunk",
    "mixed_prim" (the bound test per primitive quartet inside the large-bound
    quartets), "df64" (double-float arithmetic in place of FP64) or
    "mixed_df" ("mixed_prim" with double-float in place of FP64), see
    IntegralEngine._lists_for.  In mixed modes the SCF switches to the
    accurate arithmetic (FP64; double-float for "mixed_df") once the DIIS
    error max|FDS - SDF| drops below ``fp64_tail_diis_error`` (call
    ``switch_to_fp64``).
    """

    def __init__(self, engine, threshold: float = 1e-12, precision: str = "fp64", fp32_threshold: float = 1e-4,
                 fp64_tail_diis_error: float = 1e-5):
        self.engine = engine
        self.threshold = threshold
        self.precision = precision
        self.fp32_threshold = fp32_threshold
        self.fp64_tail_diis_error = fp64_tail_diis_error
        self.builds: list[str] = []

    @property
    def mixed(self) -> bool:
        return self.precision not in ("fp64", "df64")

    def switch_to_fp64(self) -> None:
        self.precision = "df64" if self.precision == "mixed_df" else "fp64"

    def __call__(self, D: torch.Tensor):
        self.builds.append(self.precision)
        return self.engine.jk(D, self.threshold, self.precision, self.fp32_threshold)

    def multi(self, Ds: torch.Tensor):
        """(J_i, K_i) for a stack of densities from one integral pass (sq_jk_multi)."""
        self.builds.append(self.precision)
        return self.engine.jk_multi(Ds, self.threshold, self.precision, self.fp32_threshold)


class SphericalJK:
    """J/K in real solid harmonics around a Cartesian J/K callable (DirectJK):
    D_cart = T D T^T, then J = T^T J_cart T, K = T^T K_cart T, with T the
    (n_cartesian, n_spherical) transform of slowquant_gb300.spherical."""

    def __init__(self, cartesian_jk, T: torch.Tensor):
        self.inner = cartesian_jk
        self.T = T

    def __getattr__(self, name):  # builds, mixed, fp64_tail_diis_error, switch_to_fp64 ...
        return getattr(self.inner, name)

    def __call__(self, D: torch.Tensor):
        Tm = self.T
        J, K = self.inner((Tm @ D @ Tm.T).contiguous())
        return Tm.T @ J @ Tm, Tm.T @ K @ Tm

    def multi(self, Ds: torch.Tensor):
        Tm = self.T
        J, K = self.inner.multi((Tm @ Ds @ Tm.T).contiguous())
        return Tm.T @ J @ Tm, Tm.T @ K @ Tm


def run_hartree_fock(S, T, V, ERI, number_electrons: int, log, dE_threshold: float, rmsd_threshold: float,
                     max_scf_iterations: int, use_diis: bool = True):
    """Restricted Hartree-Fock (hartreefock_in_memory.py:7-94).

    ERI is a dense (nbf,)*4 tensor (numpy or torch) or a callable D -> (J, K)
    such as DirectJK.  Returns (E_elec, C, F, D) as numpy arrays.
    """
    device = torch.device("cuda", torch.cuda.current_device())
    log.add_to_log(f"{'Iter':^4}    {'E_HF':^18}    {'DeltaE':^13}    {'RMS_D':^12}")
    S = _dev_tensor(S, device)
    Hcore = _dev_tensor(T, device) + _dev_tensor(V, device)
    if callable(ERI):
        jk = ERI
    else:
        G = _dev_tensor(ERI, device)

        def jk(D):
            return dense_jk(G, D)

    Lambda_S, L_S = torch.linalg.eigh(S)
    S_sqrt = L_S @ torch.diag(Lambda_S ** (-1 / 2)) @ L_S.T
    F0prime = S_sqrt.T @ Hcore @ S_sqrt.T
    _, C0prime = torch.linalg.eigh(F0prime)
    C0 = (S_sqrt @ C0prime).T
    nocc = int(number_electrons / 2)
    C0 = C0[0:nocc]
    D0 = 2 * C0.T @ C0
    E0 = torch.sum(D0 * Hcore)
    number_bf = len(S)
    diis_acceleration = DIIS(number_bf) if use_diis else None
    mixed = getattr(jk, "mixed", False)
    for iteration in range(1, max_scf_iterations + 1):
        J, K = jk(D0)
        F = Hcore + J - 0.5 * K
        if diis_acceleration is not None:
            F = diis_acceleration.get_extrapolated_fock_matrix(F, D0, S)
            if mixed and getattr(jk, "mixed", False):
                err = diis_acceleration.last_error
                if err is not None and err < jk.fp64_tail_diis_error:
                    jk.switch_to_fp64()
                    diis_acceleration = DIIS(number_bf)
        elif mixed and getattr(jk, "mixed", False):
            err = float((F @ D0 @ S - S @ D0 @ F).abs().max())
            if err < jk.fp64_tail_diis_error:
                jk.switch_to_fp64()
        Fprime = S_sqrt.T @ F @ S_sqrt
        _, Cprime = torch.linalg.eigh(Fprime)
        C = S_sqrt @ Cprime
        Cocc = C[:, 0:nocc]
        D = 2 * Cocc @ Cocc.T
        E = 0.5 * torch.sum(D * (Hcore + F))
        dE = float(E - E0)
        rmsd = float(torch.sum((D - D0) ** 2) ** 0.5)
        Ef = float(E)
        log.add_to_log(f"{iteration:>4}    {Ef: 18.12f}    {dE: 1.6e}    {rmsd:1.6e}")
        D0 = D
        E0 = E
        still_mixed = mixed and getattr(jk, "mixed", False)
        if np.abs(dE) < dE_threshold and rmsd < rmsd_threshold and not still_mixed:
            break
    else:
        log.add_to_log(
            f"Restricted Hartree-Fock did not meet convergence requirements in {max_scf_iterations} iterations",
            is_warning=True,
        )
    return float(E), C.cpu().numpy(), F.cpu().numpy(), D.cpu().numpy()


class _HartreeFock:
    """HF driver (hartreefockclass.py:14-136: RHF, UHF, spin densities and contamination).

    Extra knobs beyond the reference: ``direct_jk`` (default True: integral-
    direct Fock builds instead of the stored ERI tensor), ``precision``
    (a DirectJK precision: "fp64", "mixed", "mixed_prim", "df64", "mixed_df",
    ...), ``fp32_schwarz_threshold``, ``fp64_tail_diis_error``.
    """

    def __init__(self, molecule_obj, integral_obj) -> None:
        self.mol_obj = molecule_obj
        self.int_obj = integral_obj
        self.de_threshold = 10**-9
        self.rmsd_threshold = 10**-9
        self.max_scf_iterations = 100
        self.uhf_lumo_homo_mix_coeff = 0.15
        self.use_diis = True
        self.logger = _Logger()
        self.direct_jk = True
        self.precision = "fp64"
        self.fp32_schwarz_threshold = 1e-4
        self.fp64_tail_diis_error = 1e-5
        self.fock_builds: list[str] = []

    @property
    def log(self) -> str:
        return self.logger.log

    def _direct_jk(self):
        jk = DirectJK(self.int_obj.engine, self.int_obj.cauchy_schwarz_threshold, self.precision,
                      self.fp32_schwarz_threshold, self.fp64_tail_diis_error)
        if getattr(self.int_obj, "spherical", False):
            return SphericalJK(jk, self.int_obj.cart_to_sph)
        return jk

    def run_restricted_hartree_fock(self) -> None:
        if self.direct_jk:
            eri = self._direct_jk()
            S, T, V = self.int_obj.one_electron_device()
        else:
            eri = self.int_obj.electron_repulsion_tensor
            S, T, V = (self.int_obj.overlap_matrix, self.int_obj.kinetic_energy_matrix,
                       self.int_obj.nuclear_attraction_matrix)
        E, C, F, D = run_hartree_fock(S, T, V, eri, self.mol_obj.number_electrons, self.logger, self.de_threshold,
                                      self.rmsd_threshold, self.max_scf_iterations, self.use_diis)
        if self.direct_jk:
            self.fock_builds = list(eri.builds)
        self.E_hf = E
        self.mo_coeff = C
        self.rdm1 = D
        self.fock_matrix = F

    def run_unrestricted_hartree_fock(self) -> None:
        """UHF (hartreefockclass.py:67-91): sets E_uhf and the alpha/beta MOs, 1-RDMs and Fock matrices."""
        if self.direct_jk:
            eri = self._direct_jk()
            S, T, V = self.int_obj.one_electron_device()
        else:
            eri = self.int_obj.electron_repulsion_tensor
            S, T, V = (self.int_obj.overlap_matrix, self.int_obj.kinetic_energy_matrix,
                       self.int_obj.nuclear_attraction_matrix)
        E, Ca, Cb, Fa, Fb, Da, Db = run_unrestricted_hartree_fock(
            S, T, V, eri, self.mol_obj.number_electrons_alpha, self.mol_obj.number_electrons_beta,
            self.uhf_lumo_homo_mix_coeff, self.logger, self.de_threshold, self.rmsd_threshold,
            self.max_scf_iterations, self.use_diis)
        if self.direct_jk:
            self.fock_builds = list(eri.builds)
        self.E_uhf = E
        self.mo_coeff_alpha = Ca
        self.mo_coeff_beta = Cb
        self.rdm1_alpha = Da
        self.rdm1_beta = Db
        self.fock_matrix_alpha = Fa
        self.fock_matrix_beta = Fb

    @property
    def rdm1_charge(self) -> np.ndarray:
        """D_alpha + D_beta (hartreefockclass.py:93-103)."""
        return self.rdm1_alpha + self.rdm1_beta

    @property
    def rdm1_spin(self) -> np.ndarray:
        """D_alpha - D_beta (hartreefockclass.py:105-115)."""
        return self.rdm1_alpha - self.rdm1_beta

    @property
    def spin_contamination(self) -> float:
        """N_beta - sum_ij |C^a_ai C^b_bj S_ab|^2 over occupied i, j (hartreefockclass.py:117-136)."""
        na = self.mol_obj.number_electrons_alpha
        nb = self.mol_obj.number_electrons_beta
        Sab = self.mo_coeff_alpha[:, :na].T @ np.asarray(self.int_obj.overlap_matrix) @ self.mo_coeff_beta[:, :nb]
        return self.mol_obj.number_electrons_beta - float(np.sum(Sab**2))


def run_unrestricted_hartree_fock(S, T, V, ERI, number_electrons_alpha: int, number_electrons_beta: int,
                                  lumo_homo_mix_coeff: float, log, dE_threshold: float, rmsd_threshold: float,
                                  max_scf_iterations: int, use_diis: bool = True):
    """Unrestricted Hartree-Fock (unrestricted_hartreefock_in_memory.py:7-125).

    Same start (core guess, HOMO/LUMO rotation by ``lumo_homo_mix_coeff``
    when N_alpha == N_beta), Fock matrices F_s = H + J[D_a + D_b] - K[D_s],
    one DIIS per spin, energy, convergence test and log lines.  ERI is a dense
    tensor or a callable D -> (J, K) such as DirectJK; DirectJK digests both
    spin densities in one pass over the integrals (sq_jk_multi), another
    callable is called once per spin density (J is linear in D, so
    J[D_a] + J[D_b] is the total Coulomb matrix).  Returns
    (E_elec, C_a, C_b, F_a, F_b, D_a, D_b) as numpy arrays.
    """
    device = torch.device("cuda", torch.cuda.current_device())
    log.add_to_log(
        f"{'Iter':^4}    {'E_UHF':^18}    {'DeltaE':^13}    {'RMS_D_alpha':^12}    {'RMS_D_beta':^12}"
    )
    S = _dev_tensor(S, device)
    Hcore = _dev_tensor(T, device) + _dev_tensor(V, device)
    if callable(ERI):
        jk = ERI
    else:
        G = _dev_tensor(ERI, device)

        def jk(D):
            return dense_jk(G, D)

    na, nb = int(number_electrons_alpha), int(number_electrons_beta)
    Lambda_S, L_S = torch.linalg.eigh(S)
    S_sqrt = L_S @ torch.diag(Lambda_S ** (-1 / 2)) @ L_S.T
    F0prime = S_sqrt.T @ Hcore @ S_sqrt.T
    _, C0prime = torch.linalg.eigh(F0prime)
    C0_alpha = (S_sqrt @ C0prime).T.clone()  # rows are MOs
    C0_beta = (S_sqrt @ C0prime).T.clone()
    if na == nb:
        # break the alpha/beta symmetry by rotating HOMO and LUMO
        c_homo = C0_alpha[na - 1].clone()
        c_lumo = C0_alpha[na].clone()
        x = lumo_homo_mix_coeff
        C0_alpha[na - 1] = 1 / (1 + x**2) ** 0.5 * (c_homo + x * c_lumo)
        C0_alpha[na] = 1 / (1 + x**2) ** 0.5 * (-x * c_homo + c_lumo)
    C0_alpha = C0_alpha[0:na]
    C0_beta = C0_beta[0:nb]
    D0_alpha = C0_alpha.T @ C0_alpha
    D0_beta = C0_beta.T @ C0_beta
    E0 = torch.sum(D0_alpha * Hcore) + torch.sum(D0_beta * Hcore)
    number_bf = len(S)
    diis_alpha = DIIS(number_bf) if use_diis else None
    diis_beta = DIIS(number_bf) if use_diis else None
    mixed = getattr(jk, "mixed", False)
    for iteration in range(1, max_scf_iterations + 1):
        if hasattr(jk, "multi"):
            # both spin densities against one evaluation of the integrals
            Js, Ks = jk.multi(torch.stack([D0_alpha, D0_beta]))
            J_alpha, J_beta, K_alpha, K_beta = Js[0], Js[1], Ks[0], Ks[1]
        else:
            J_alpha, K_alpha = jk(D0_alpha)
            J_beta, K_beta = jk(D0_beta)
        F_alpha = Hcore + J_alpha + J_beta - K_alpha
        F_beta = Hcore + J_beta + J_alpha - K_beta
        if diis_alpha is not None:
            F_alpha = diis_alpha.get_extrapolated_fock_matrix(F_alpha, D0_alpha, S)
            F_beta = diis_beta.get_extrapolated_fock_matrix(F_beta, D0_beta, S)
            if mixed and getattr(jk, "mixed", False):
                errs = (diis_alpha.last_error, diis_beta.last_error)
                if all(e is not None for e in errs) and max(errs) < jk.fp64_tail_diis_error:
                    jk.switch_to_fp64()
                    diis_alpha, diis_beta = DIIS(number_bf), DIIS(number_bf)
        elif mixed and getattr(jk, "mixed", False):
            err = max(float((F @ D0 @ S - S @ D0 @ F).abs().max())
                      for F, D0 in ((F_alpha, D0_alpha), (F_beta, D0_beta)))
            if err < jk.fp64_tail_diis_error:
                jk.switch_to_fp64()
        _, Cprime_alpha = torch.linalg.eigh(S_sqrt.T @ F_alpha @ S_sqrt)
        _, Cprime_beta = torch.linalg.eigh(S_sqrt.T @ F_beta @ S_sqrt)
        C_alpha = S_sqrt @ Cprime_alpha
        C_beta = S_sqrt @ Cprime_beta
        Cocc_alpha = C_alpha[:, 0:na]
        Cocc_beta = C_beta[:, 0:nb]
        D_alpha = Cocc_alpha @ Cocc_alpha.T
        D_beta = Cocc_beta @ Cocc_beta.T
        E = 0.5 * torch.sum(D_alpha * (Hcore + F_alpha)) + 0.5 * torch.sum(D_beta * (Hcore + F_beta))
        dE = float(E - E0)
        rmsd_alpha = float(torch.sum((D_alpha - D0_alpha) ** 2) ** 0.5)
        rmsd_beta = float(torch.sum((D_beta - D0_beta) ** 2) ** 0.5)
        log.add_to_log(
            f"{iteration:>4}    {float(E): 18.12f}    {dE: 1.6e}    {rmsd_alpha:1.6e}     {rmsd_beta:1.6e}"
        )
        D0_alpha, D0_beta, E0 = D_alpha, D_beta, E
        still_mixed = mixed and getattr(jk, "mixed", False)
        if (np.abs(dE) < dE_threshold and rmsd_alpha < rmsd_threshold and rmsd_beta < rmsd_threshold
                and not still_mixed):
            break
    else:
        log.add_to_log(
            f"Unrestricted Hartree-Fock did not meet convergence requirements in {max_scf_iterations} iterations",
            is_warning=True,
        )
    return (float(E), C_alpha.cpu().numpy(), C_beta.cpu().numpy(), F_alpha.cpu().numpy(), F_beta.cpu().numpy(),
            D_alpha.cpu().numpy(), D_beta.cpu().numpy())
