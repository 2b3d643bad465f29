"""Oracle for SlowQuant's integral / RHF hot path -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker (or the timed CPU
baseline).  The product package never imports it.

It restates the reference independently of the product's host code:

* molecule parsing and the Angstrom->bohr factor 1.889725989
  (slowquant/molecule/moleculeclass.py:12-80), nuclear repulsion (:167-184);
* basis reading (slowquant/molecule/basis_reader.py:6-75) from the JSON
  tables of published basis-set data shipped with the package;
* per-Cartesian-component normalisation (moleculeclass.py:269-301,
  moleculefunctions.py:7-88);
* the MD integrals through ``sq_oracle.c`` (compiled to ``liboracle.so``);
* J/K by the reference's einsums and the RHF SCF + DIIS loop
  (slowquant/hartreefock/hartreefock_in_memory.py:7-94, diis.py:4-66).
"""

from __future__ import annotations

import ctypes
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BASIS_DIR = os.path.join(os.path.dirname(HERE), "slowquant_gb300", "basisset")
LIB_PATH = os.path.join(HERE, "liboracle.so")

ANGSTROM_TO_BOHR = 1.889725989  # moleculeclass.py:27
CHARGES = {"H": 1, "He": 2, "Li": 3, "Be": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "Ne": 10,
           "Na": 11, "Mg": 12, "Al": 13, "Si": 14, "P": 15, "S": 16, "Cl": 17, "Ar": 18}
CART = {  # basis_reader.py:50-70 component order
    "s": [[0, 0, 0]],
    "p": [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
    "d": [[2, 0, 0], [1, 1, 0], [1, 0, 1], [0, 2, 0], [0, 1, 1], [0, 0, 2]],
    "f": [[3, 0, 0], [2, 1, 0], [2, 0, 1], [1, 2, 0], [1, 1, 1], [1, 0, 2], [0, 3, 0], [0, 2, 1],
          [0, 1, 2], [0, 0, 3]],
}


def build_oracle(force: bool = False) -> str:
    """Compile sq_oracle.c into liboracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "sq_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


class _Basis(ctypes.Structure):
    _fields_ = [
        ("nshell", ctypes.c_int), ("center", ctypes.c_void_p), ("nprim", ctypes.c_void_p),
        ("prim_off", ctypes.c_void_p), ("ncart", ctypes.c_void_p), ("cart_off", ctypes.c_void_p),
        ("bf_off", ctypes.c_void_p), ("norm_off", ctypes.c_void_p), ("exps", ctypes.c_void_p),
        ("coefs", ctypes.c_void_p), ("cart", ctypes.c_void_p), ("norm", ctypes.c_void_p),
        ("nbf", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(LIB_PATH)
        L.sqo_boys.restype = ctypes.c_double
        L.sqo_boys.argtypes = [ctypes.c_int, ctypes.c_double]
        L.sqo_factorial2.restype = ctypes.c_double
        L.sqo_factorial2.argtypes = [ctypes.c_double]
        _lib = L
    return _lib


def factorial2(n: float) -> float:
    """moleculefunctions.py:7-26."""
    out = 1.0
    if n > 0:
        for i in range(int(n + 1) // 2):
            out *= n - 2 * i
    return out


def primitive_normalization(exponent: float, ang) -> float:
    """moleculefunctions.py:29-47."""
    l, m, n = ang
    return ((2 / np.pi) ** (3 / 4) * (2 ** (l + m + n) * exponent ** ((2 * l + 2 * m + 2 * n + 3) / 4))
            / (factorial2(2 * l - 1) * factorial2(2 * m - 1) * factorial2(2 * n - 1)) ** (1 / 2))


def contracted_normalization(exponents, coefficients, ang) -> float:
    """moleculefunctions.py:50-88."""
    ax, ay, az = ang
    f = 0.0
    for i in range(len(exponents)):
        for j in range(len(exponents)):
            f += coefficients[i] * coefficients[j] / (exponents[i] + exponents[j]) ** (ax + ay + az + 3 / 2)
    f *= (np.pi ** (3 / 2) * factorial2(2 * ax - 1) * factorial2(2 * ay - 1) * factorial2(2 * az - 1)) / (
        2 ** (ax + ay + az))
    return f ** (-1 / 2)


class OracleMolecule:
    """Atoms + shells, restated from moleculeclass.py / basis_reader.py."""

    def __init__(self, geometry: str, basis: str, distance_unit: str = "bohr", charge: int = 0):
        unit = {"angstrom": ANGSTROM_TO_BOHR, "bohr": 1.0, "au": 1.0}[distance_unit.lower()]
        self.atoms = []
        for line in geometry.split(";"):
            if not line.strip():
                continue
            f = line.split()
            self.atoms.append((f[0], np.array([float(f[1]) * unit, float(f[2]) * unit, float(f[3]) * unit]),
                               CHARGES[f[0]]))
        self.charge = charge
        name = basis.replace("*", "_st_").lower()
        table = json.load(open(os.path.join(BASIS_DIR, name + ".json"), encoding="UTF-8"))["elements"]
        self.shells = []  # (center, exps, coefs, cart[ncart,3], norm[ncart,nprim], bf_off)
        nbf = 0
        for sym, xyz, _ in self.atoms:
            for sh in table[sym.lower()]:
                exps = np.array(sh["exponents"])
                coefs = np.array(sh["coefficients"])
                cart = np.array(CART[sh["l"]])
                norm = np.zeros((len(cart), len(exps)))
                for b, ang in enumerate(cart):
                    for i, e in enumerate(exps):
                        norm[b, i] = primitive_normalization(e, ang)
                    norm[b, :] *= contracted_normalization(exps, coefs * norm[b, :], ang)
                self.shells.append((xyz, exps, coefs, cart, norm, nbf))
                nbf += len(cart)
        self.nbf = nbf
        self._keep = None

    @property
    def number_electrons(self) -> int:
        return sum(a[2] for a in self.atoms) - self.charge

    @property
    def nuclear_repulsion(self) -> float:
        """moleculeclass.py:167-184."""
        V = 0.0
        for i, (_, Ri, Zi) in enumerate(self.atoms):
            for j, (_, Rj, Zj) in enumerate(self.atoms):
                if i >= j:
                    continue
                V += Zi * Zj / np.einsum("k->", (Ri - Rj) ** 2) ** 0.5
        return V

    def cbasis(self) -> _Basis:
        sh = self.shells
        center = np.ascontiguousarray(np.array([s[0] for s in sh], dtype=np.float64))
        nprim = np.array([len(s[1]) for s in sh], dtype=np.int32)
        ncart = np.array([len(s[3]) for s in sh], dtype=np.int32)
        prim_off = np.concatenate([[0], np.cumsum(nprim)[:-1]]).astype(np.int32)
        cart_off = np.concatenate([[0], np.cumsum(ncart)[:-1]]).astype(np.int32)
        norm_off = np.concatenate([[0], np.cumsum(nprim * ncart)[:-1]]).astype(np.int32)
        bf_off = np.array([s[5] for s in sh], dtype=np.int32)
        exps = np.concatenate([s[1] for s in sh]).astype(np.float64)
        coefs = np.concatenate([s[2] for s in sh]).astype(np.float64)
        cart = np.ascontiguousarray(np.concatenate([s[3] for s in sh]).astype(np.int32))
        norm = np.concatenate([s[4].ravel() for s in sh]).astype(np.float64)
        self._keep = (center, nprim, ncart, prim_off, cart_off, norm_off, bf_off, exps, coefs, cart, norm)
        p = lambda a: a.ctypes.data  # noqa: E731
        return _Basis(len(sh), p(center), p(nprim), p(prim_off), p(ncart), p(cart_off), p(bf_off),
                      p(norm_off), p(exps), p(coefs), p(cart), p(norm), self.nbf)

    # --- integrals through the C restatement ---------------------------------
    def schwarz(self, nthreads: int = 0, faithful: bool = False) -> np.ndarray:
        n = len(self.shells)
        cs = np.zeros((n, n))
        B = self.cbasis()
        rc = lib().sqo_schwarz(ctypes.byref(B), cs.ctypes.data_as(ctypes.c_void_p), nthreads, int(faithful))
        assert rc == 0
        return cs

    def eri_dense(self, threshold: float = 1e-12, use_schwarz: bool = True, nthreads: int = 0,
                  faithful: bool = False) -> np.ndarray:
        n = self.nbf
        V = np.zeros((n, n, n, n))
        cs = self.schwarz(nthreads, faithful) if use_schwarz else None
        B = self.cbasis()
        rc = lib().sqo_eri_dense(ctypes.byref(B), None if cs is None else cs.ctypes.data_as(ctypes.c_void_p),
                                 ctypes.c_double(threshold), V.ctypes.data_as(ctypes.c_void_p), nthreads,
                                 int(faithful))
        assert rc == 0
        return V

    def eri_quartets(self, quartets: np.ndarray, nthreads: int = 0, faithful: bool = True) -> np.ndarray:
        """Contracted blocks of explicit shell quartets, concatenated (C order per block)."""
        q = np.ascontiguousarray(quartets, dtype=np.int32).reshape(-1, 4)
        sizes = np.array([np.prod([len(self.shells[s][3]) for s in row]) for row in q], dtype=np.int64)
        off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        out = np.zeros(int(sizes.sum()))
        B = self.cbasis()
        rc = lib().sqo_eri_quartets(ctypes.byref(B), q.ctypes.data_as(ctypes.c_void_p), ctypes.c_long(len(q)),
                                    out.ctypes.data_as(ctypes.c_void_p), off.ctypes.data_as(ctypes.c_void_p),
                                    nthreads, int(faithful))
        assert rc == 0
        return out

    def jk_direct(self, D: np.ndarray, threshold: float = 1e-12, nthreads: int = 0, accurate: bool = True,
                  cs: np.ndarray | None = None):
        """J, K of hartreefock_in_memory.py:55-56 from the screened unique quartets, no stored tensor.

        ``accurate`` evaluates the Boys function to full double precision (the
        oracle's mode 1) instead of the reference's truncated series; the
        Schwarz matrix ``cs`` (default: computed here) screens as the driver does.
        """
        L = lib()
        L.sqo_set_boys_mode(1 if accurate else 0)
        try:
            if cs is None:
                cs = self.schwarz(nthreads)
            n = self.nbf
            Dc = np.ascontiguousarray(D, dtype=np.float64)
            J, K = np.zeros((n, n)), np.zeros((n, n))
            B = self.cbasis()
            rc = L.sqo_jk_direct(ctypes.byref(B), cs.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(threshold),
                                 Dc.ctypes.data_as(ctypes.c_void_p), J.ctypes.data_as(ctypes.c_void_p),
                                 K.ctypes.data_as(ctypes.c_void_p), nthreads)
            assert rc == 0
        finally:
            L.sqo_set_boys_mode(0)
        return J, K

    def one_electron(self):
        n = self.nbf
        S, T, V = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
        B = self.cbasis()
        xyz = np.ascontiguousarray(np.array([a[1] for a in self.atoms], dtype=np.float64))
        Z = np.array([float(a[2]) for a in self.atoms])
        L = lib()
        L.sqo_overlap(ctypes.byref(B), S.ctypes.data_as(ctypes.c_void_p))
        L.sqo_kinetic(ctypes.byref(B), T.ctypes.data_as(ctypes.c_void_p))
        L.sqo_nuclear(ctypes.byref(B), len(self.atoms), xyz.ctypes.data_as(ctypes.c_void_p),
                      Z.ctypes.data_as(ctypes.c_void_p), V.ctypes.data_as(ctypes.c_void_p))
        return S, T, V


def boys(n: int, z: float) -> float:
    return lib().sqo_boys(int(n), float(z))


def jk_from_eri(ERI: np.ndarray, D: np.ndarray):
    """hartreefock_in_memory.py:55-56."""
    J = np.einsum("pqrs,sr->pq", ERI, D)
    K = np.einsum("psqr,sr->pq", ERI, D)
    return J, K


class OracleDIIS:
    """diis.py:4-66."""

    def __init__(self, number_bf: int, number_fock_saved: int = 6):
        self.F, self.D = [], []
        self.nsave = number_fock_saved
        self.nbf = number_bf

    def extrapolate(self, F, D, S):
        if len(F) == 2:
            return F
        self.F.append(F)
        self.D.append(D)
        if len(self.F) == 1:
            return F
        if len(self.F) > self.nsave:
            self.F.pop(0)
            self.D.pop(0)
        errs = [Fi @ Di @ S - S @ Di @ Fi for Fi, Di in zip(self.F, self.D)]
        m = len(self.F)
        B = np.zeros((m + 1, m + 1))
        B[-1, :] = B[:, -1] = -1
        B[-1, -1] = 0
        b0 = np.zeros(m + 1)
        b0[-1] = -1
        for i in range(m):
            for j in range(m):
                B[i, j] = np.trace(errs[i] @ errs[j])
        c = np.linalg.solve(B, b0)
        out = np.zeros((self.nbf, self.nbf))
        for ci, Fi in zip(c[:-1], self.F):
            out += ci * Fi
        return out


def run_hartree_fock(S, T, V, jk, number_electrons, dE_threshold=1e-9, rmsd_threshold=1e-9,
                     max_scf_iterations=100, use_diis=True):
    """hartreefock_in_memory.py:7-94; ``jk(D) -> (J, K)`` supplies the two-electron part.

    Returns (E_elec, C, F, D, per-iteration energies).
    """
    Hcore = T + V
    lam, LS = np.linalg.eigh(S)
    S_sqrt = LS @ np.diag(lam ** (-1 / 2)) @ LS.T
    F0p = S_sqrt.T @ Hcore @ S_sqrt.T
    _, C0p = np.linalg.eigh(F0p)
    C0 = (S_sqrt @ C0p).T[: number_electrons // 2]
    D0 = 2 * C0.T @ C0
    E0 = np.einsum("ij,ij->", D0, Hcore)
    diis = OracleDIIS(len(S)) if use_diis else None
    energies = []
    for _ in range(1, max_scf_iterations + 1):
        J, K = jk(D0)
        F = Hcore + J - 0.5 * K
        if diis is not None:
            F = diis.extrapolate(F, D0, S)
        Fp = S_sqrt.T @ F @ S_sqrt
        _, Cp = np.linalg.eigh(Fp)
        C = S_sqrt @ Cp
        Cocc = C[:, : number_electrons // 2]
        D = 2 * Cocc @ Cocc.T
        E = 0.5 * np.einsum("ij,ij->", D, Hcore + F)
        dE = E - E0
        rmsd = np.einsum("ij->", (D - D0) ** 2) ** 0.5
        energies.append(E)
        D0, E0 = D, E
        if abs(dE) < dE_threshold and rmsd < rmsd_threshold:
            break
    return E, C, F, D, energies


def run_unrestricted_hartree_fock(S, T, V, jk, number_electrons_alpha, number_electrons_beta,
                                  lumo_homo_mix_coeff=0.15, dE_threshold=1e-9, rmsd_threshold=1e-9,
                                  max_scf_iterations=100, use_diis=True):
    """unrestricted_hartreefock_in_memory.py:7-125; ``jk(D) -> (J, K)``.

    Returns (E_elec, C_alpha, C_beta, D_alpha, D_beta, per-iteration energies).
    """
    na, nb = int(number_electrons_alpha), int(number_electrons_beta)
    Hcore = T + V
    lam, LS = np.linalg.eigh(S)
    S_sqrt = LS @ np.diag(lam ** (-1 / 2)) @ LS.T
    _, C0p = np.linalg.eigh(S_sqrt.T @ Hcore @ S_sqrt.T)
    Ca0 = (S_sqrt @ C0p).T.copy()
    Cb0 = (S_sqrt @ C0p).T.copy()
    if na == nb:
        h, lu = Ca0[na - 1].copy(), Ca0[na].copy()
        x = lumo_homo_mix_coeff
        Ca0[na - 1] = (h + x * lu) / (1 + x**2) ** 0.5
        Ca0[na] = (-x * h + lu) / (1 + x**2) ** 0.5
    Da0 = Ca0[:na].T @ Ca0[:na]
    Db0 = Cb0[:nb].T @ Cb0[:nb]
    E0 = np.einsum("ij,ij->", Da0 + Db0, Hcore)
    diis_a = OracleDIIS(len(S)) if use_diis else None
    diis_b = OracleDIIS(len(S)) if use_diis else None
    energies = []
    for _ in range(1, max_scf_iterations + 1):
        Ja, Ka = jk(Da0)
        Jb, Kb = jk(Db0)
        Fa = Hcore + Ja + Jb - Ka
        Fb = Hcore + Ja + Jb - Kb
        if diis_a is not None:
            Fa = diis_a.extrapolate(Fa, Da0, S)
            Fb = diis_b.extrapolate(Fb, Db0, S)
        _, Cpa = np.linalg.eigh(S_sqrt.T @ Fa @ S_sqrt)
        _, Cpb = np.linalg.eigh(S_sqrt.T @ Fb @ S_sqrt)
        Ca, Cb = S_sqrt @ Cpa, S_sqrt @ Cpb
        Da = Ca[:, :na] @ Ca[:, :na].T
        Db = Cb[:, :nb] @ Cb[:, :nb].T
        E = 0.5 * np.einsum("ij,ij->", Da, Hcore + Fa) + 0.5 * np.einsum("ij,ij->", Db, Hcore + Fb)
        dE = E - E0
        rmsd_a = np.sum((Da - Da0) ** 2) ** 0.5
        rmsd_b = np.sum((Db - Db0) ** 2) ** 0.5
        energies.append(E)
        Da0, Db0, E0 = Da, Db, E
        if abs(dE) < dE_threshold and rmsd_a < rmsd_threshold and rmsd_b < rmsd_threshold:
            break
    return E, Ca, Cb, Da, Db, energies
