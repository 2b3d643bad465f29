"""Device-side integral engine: basis upload, shell-pair data, Schwarz screening,
shell-quartet work lists, dense ERIs and the integral-direct J/K build.

Work layout in HBM (all arrays are torch tensors owned by the engine and handed
to the C ABI as raw device pointers):

* basis: shell centres, angular momenta, primitive offsets, exponents and
  component-independent contraction coefficients (``sq_basis``);
* pairs: every shell pair (a, b), l[a] >= l[b], sorted by pair class, with per
  primitive pair p, P, U (``prim``, 8 doubles) and the Hermite-expanded
  E^{ab}_{tuv} x component normalisation (``herm``), in FP64 and FP32;
* quartets: per quartet class a contiguous segment of (bra pair, ket pair)
  int32 pairs.  Pairs are grouped by (class, primitive counts) and sorted by
  descending Schwarz factor inside a group, so each bra pair's surviving ket
  pairs are a prefix of every ket group (the screening test
  Q_bra Q_ket >= threshold of electronrepulsion.py:44-49), and warps see
  uniform loop trip counts.  With a second threshold the prefix splits into an
  FP64 part (large bounds) and an FP32 part (small bounds).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, screening
from ._lib import SqBasis, SqPairs, SqQuartets, SqSlots, check, ptr
from .molecule import _Molecule

NCART = [1, 3, 6, 10]


def herm_size(la: int, lb: int) -> int:
    """Hermite terms per primitive pair of class (la, lb): sum over component pairs of prod_d (a_d+b_d+1)."""
    from .molecule import CARTESIAN

    ca = CARTESIAN["spdf"[la]]
    cb = CARTESIAN["spdf"[lb]]
    return int(sum((a[0] + b[0] + 1) * (a[1] + b[1] + 1) * (a[2] + b[2] + 1) for a in ca for b in cb))


def pair_class(la: int, lb: int) -> int:
    return la * (la + 1) // 2 + lb


def quartet_class(cb: int, ck: int) -> int:
    return cb * (cb + 1) // 2 + ck


@dataclass
class QuartetList:
    """Device quartet list + host class offsets, ready for the C ABI."""

    pairs: torch.Tensor  # [n, 2] int32 on device
    class_off: np.ndarray  # [SQ_MAX_QCLASS + 1] int64

    @property
    def nquartet(self) -> int:
        return int(self.class_off[-1])

    def cstruct(self) -> SqQuartets:
        q = SqQuartets()
        q.nquartet = self.nquartet
        q.pairs = ptr(self.pairs) if self.nquartet > 0 else None
        for i, v in enumerate(self.class_off):
            q.class_off[i] = int(v)
        return q

    def class_counts(self) -> np.ndarray:
        return np.diff(self.class_off)


class IntegralEngine:
    """Integrals and Fock builds for one molecule on one GPU."""

    def __init__(self, mol: _Molecule, device: int | str | torch.device | None = None, fp32: bool = True):
        if not torch.cuda.is_available():
            raise RuntimeError("slowquant_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = _lib.lib()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.mol = mol
        self.nbf = int(mol.number_bf)
        self.nshell = int(mol.number_shell)
        shells = mol.shells
        self.l = np.array([s.angular_momentum for s in shells], dtype=np.int32)
        self.lmax_eri = _lib.SQ_MAX_L
        dev = self.device
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        # Integrals are translation invariant: centre the coordinates so the
        # FP32 copies of P and Q keep more significant bits.
        coords = mol.atom_coordinates
        self.origin = coords.mean(axis=0) if len(coords) else np.zeros(3)
        centers = np.array([s.center for s in shells], dtype=np.float64).reshape(-1, 3) - self.origin
        nprim = np.array([len(s.exponents) for s in shells], dtype=np.int32)
        prim_off = np.concatenate([[0], np.cumsum(nprim)[:-1]]).astype(np.int32)
        bf_off = np.array([s.bf_idx[0] for s in shells], dtype=np.int32)
        exps = np.concatenate([s.exponents for s in shells]).astype(np.float64)
        coefs = np.concatenate([s.component_independent_coefficients() for s in shells]).astype(np.float64)
        self.nprim = nprim
        self.bf_off_host = bf_off
        self.t_center = torch.tensor(centers, **f64)
        self.t_l = torch.tensor(self.l, **i32)
        self.t_nprim = torch.tensor(nprim, **i32)
        self.t_prim_off = torch.tensor(prim_off, **i32)
        self.t_bf_off = torch.tensor(bf_off, **i32)
        self.t_exps = torch.tensor(exps, **f64)
        self.t_coefs = torch.tensor(coefs, **f64)
        self.t_atom_xyz = torch.tensor(coords - self.origin, **f64).reshape(-1, 3).contiguous()
        self.t_atom_charge = torch.tensor(mol.atom_charges, **f64)
        self.shell_atom = np.array([mol.atoms.index(s.origin_atom) for s in shells], dtype=np.int32)
        self.t_shell_atom = torch.tensor(self.shell_atom, **i32)
        b = SqBasis()
        b.nshell, b.nbf, b.natom, b.nprim_total = self.nshell, self.nbf, len(mol.atoms), len(exps)
        b.center, b.l, b.nprim, b.prim_off, b.bf_off = (ptr(self.t_center), ptr(self.t_l), ptr(self.t_nprim),
                                                       ptr(self.t_prim_off), ptr(self.t_bf_off))
        b.exps, b.coefs = ptr(self.t_exps), ptr(self.t_coefs)
        b.atom_xyz, b.atom_charge = ptr(self.t_atom_xyz), ptr(self.t_atom_charge)
        b.shell_atom = ptr(self.t_shell_atom)
        self.cbasis = b

        # Boys grid tables
        self.tab64 = torch.empty(_lib.SQ_BOYS_TAB64_SIZE, **f64)
        self.tab32 = torch.empty(_lib.SQ_BOYS_TAB32_SIZE, dtype=torch.float32, device=dev)
        check(self.lib.sq_boys_table(ptr(self.tab64), ptr(self.tab32), self._stream()), "sq_boys_table")

        self.fp32 = fp32
        self._build_pairs()
        self._q = None
        self._quartet_cache: dict = {}
        self._jk_scratch = None
        self._slots = None

    # ------------------------------------------------------------------ utils
    def _stream(self) -> int:
        return _lib.stream_handle(self.device)

    def eri_supported(self) -> bool:
        return bool(self.nshell == 0 or self.l.max() <= self.lmax_eri)

    def _require_eri(self) -> None:
        if not self.eri_supported():
            raise NotImplementedError(
                f"two-electron kernels support shells up to l={self.lmax_eri}; basis has l={int(self.l.max())}")

    # ------------------------------------------------------------------ pairs
    def _build_pairs(self) -> None:
        ns = self.nshell
        i, j = np.triu_indices(ns)
        li, lj = self.l[i], self.l[j]
        a = np.where(li >= lj, i, j)
        b = np.where(li >= lj, j, i)
        la, lb = self.l[a], self.l[b]
        pc = la * (la + 1) // 2 + lb
        order = np.argsort(pc, kind="stable")
        a, b, pc = a[order], b[order], pc[order]
        self.pair_shells = np.stack([a, b], axis=1).astype(np.int32)
        self.pair_class = pc.astype(np.int32)
        self.pair_np = (self.nprim[a] * self.nprim[b]).astype(np.int64)
        self.pair_npa = self.nprim[a]
        self.pair_npb = self.nprim[b]
        self.npair = len(a)
        hs = np.array([herm_size(min(x, 3), min(y, 3)) if x <= 3 else 0 for x, y in zip(self.l[a], self.l[b])],
                      dtype=np.int64)
        pp_off = np.concatenate([[0], np.cumsum(self.pair_np)]).astype(np.int64)
        herm_off = np.concatenate([[0], np.cumsum(self.pair_np * hs)[:-1]]).astype(np.int64)
        nprimpair = int(pp_off[-1])
        nherm = int((self.pair_np * hs).sum())
        if nprimpair >= 2**31:
            raise RuntimeError("too many primitive pairs for int32 indexing")
        dev = self.device
        self.t_pair_shells = torch.tensor(self.pair_shells, dtype=torch.int32, device=dev)
        self.t_pp_off = torch.tensor(pp_off.astype(np.int32), dtype=torch.int32, device=dev)
        self.t_herm_off = torch.tensor(herm_off, dtype=torch.int64, device=dev)
        self.t_prim = torch.empty(max(nprimpair, 1) * 8, dtype=torch.float64, device=dev)
        self.t_herm = torch.empty(max(nherm, 1), dtype=torch.float64, device=dev)
        self.t_prim32 = torch.empty(max(nprimpair, 1) * 8, dtype=torch.float32, device=dev) if self.fp32 else None
        self.t_herm32 = torch.empty(max(nherm, 1), dtype=torch.float32, device=dev) if self.fp32 else None
        p = SqPairs()
        p.npair, p.nprimpair = self.npair, nprimpair
        p.shells, p.pp_off, p.herm_off = ptr(self.t_pair_shells), ptr(self.t_pp_off), ptr(self.t_herm_off)
        p.prim, p.herm = ptr(self.t_prim), ptr(self.t_herm)
        p.prim32, p.herm32 = ptr(self.t_prim32), ptr(self.t_herm32)
        self.cpairs = p
        if self.npair:
            check(self.lib.sq_pair_prep(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), self._stream()),
                  "sq_pair_prep")

    # --------------------------------------------------------------- schwarz
    def _class_lists(self, lists: dict[int, np.ndarray]) -> QuartetList:
        """Concatenate per-class (n,2) int32 arrays into one device list."""
        off = np.zeros(_lib.SQ_MAX_QCLASS + 1, dtype=np.int64)
        parts = []
        for c in range(_lib.SQ_MAX_QCLASS):
            arr = lists.get(c)
            n = 0 if arr is None else len(arr)
            off[c + 1] = off[c] + n
            if n:
                parts.append(arr)
        host = np.concatenate(parts).astype(np.int32) if parts else np.zeros((0, 2), dtype=np.int32)
        t = torch.tensor(host, dtype=torch.int32, device=self.device).reshape(-1, 2).contiguous()
        return QuartetList(t, off)

    @property
    def pair_q(self) -> np.ndarray:
        """Schwarz factor sqrt(max (ab|ab)) of every pair (pair order)."""
        if self._q is None:
            self._require_eri()
            lists = {}
            for pc in np.unique(self.pair_class):
                idx = np.nonzero(self.pair_class == pc)[0].astype(np.int32)
                lists[quartet_class(int(pc), int(pc))] = np.stack([idx, idx], axis=1)
            ql = self._class_lists(lists)
            q = torch.zeros(max(self.npair, 1), dtype=torch.float64, device=self.device)
            qs = ql.cstruct()
            check(self.lib.sq_schwarz(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(qs),
                                      ptr(self.tab64), ptr(q), self._stream()), "sq_schwarz")
            self._q = q[: self.npair].cpu().numpy()
        return self._q

    def schwarz_matrix(self) -> np.ndarray:
        """(nshell, nshell) Cauchy-Schwarz matrix (get_cauchy_schwarz_matrix)."""
        cs = np.zeros((self.nshell, self.nshell))
        q = self.pair_q
        a, b = self.pair_shells[:, 0], self.pair_shells[:, 1]
        cs[a, b] = q
        cs[b, a] = q
        return cs

    # ----------------------------------------------------------------- slots
    @property
    def slots(self) -> SqSlots:
        """Slot layout (pairs in Schwarz-sorted group order, field-major data)."""
        if self._slots is None:
            self._build_slots()
        return self._slots

    def _build_slots(self) -> None:
        q = self.pair_q
        groups = screening.pair_groups(self.pair_class, self.pair_npa, self.pair_npb, q)
        slot_pair = np.concatenate([g[1] for g in groups]).astype(np.int32) if groups else np.zeros(0, np.int32)
        nslot = len(slot_pair)
        npp = np.zeros(nslot, np.int32)
        pbase = np.zeros(nslot, np.int32)
        pstride = np.zeros(nslot, np.int32)
        hbase = np.zeros(nslot, np.int64)
        pos = 0
        poff = 0
        hoff = 0
        for cls, members in groups:
            n = len(members)
            nppg = int(self.pair_np[members[0]])
            la, lb = int(self.l[self.pair_shells[members[0], 0]]), int(self.l[self.pair_shells[members[0], 1]])
            E = herm_size(la, lb)
            sl = slice(pos, pos + n)
            npp[sl] = nppg
            pbase[sl] = poff + np.arange(n)
            pstride[sl] = n
            hbase[sl] = hoff + np.arange(n)
            pos += n
            poff += n * nppg
            hoff += n * nppg * E
        if poff >= 2**31:
            raise RuntimeError("too many primitive pairs for int32 slot indexing")
        self.slot_pair = slot_pair
        self.slot_of_pair = np.empty(nslot, np.int32)
        self.slot_of_pair[slot_pair] = np.arange(nslot, dtype=np.int32)
        dev = self.device
        i32 = dict(dtype=torch.int32, device=dev)
        self.t_slot_pair = torch.tensor(slot_pair, **i32)
        self.t_slot_of_pair = torch.tensor(self.slot_of_pair, **i32)
        self.t_slot_npp = torch.tensor(npp, **i32)
        self.t_slot_pbase = torch.tensor(pbase, **i32)
        self.t_slot_pstride = torch.tensor(pstride, **i32)
        self.t_slot_hbase = torch.tensor(hbase, dtype=torch.int64, device=dev)
        self.t_slot_prim = torch.empty(max(5 * poff, 1), dtype=torch.float64, device=dev)
        self.t_slot_herm = torch.empty(max(hoff, 1), dtype=torch.float64, device=dev)
        self.t_slot_prim32 = torch.empty(max(5 * poff, 1), dtype=torch.float32, device=dev) if self.fp32 else None
        self.t_slot_herm32 = torch.empty(max(hoff, 1), dtype=torch.float32, device=dev) if self.fp32 else None
        s = SqSlots()
        s.nslot, s.npp_total, s.nherm_total = nslot, poff, hoff
        s.pair, s.npp, s.pbase, s.pstride, s.hbase = (ptr(self.t_slot_pair), ptr(self.t_slot_npp),
                                                      ptr(self.t_slot_pbase), ptr(self.t_slot_pstride),
                                                      ptr(self.t_slot_hbase))
        s.prim, s.herm = ptr(self.t_slot_prim), ptr(self.t_slot_herm)
        s.prim32, s.herm32 = ptr(self.t_slot_prim32), ptr(self.t_slot_herm32)
        self._slots = s
        if nslot:
            check(self.lib.sq_slots_fill(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(s),
                                         self._stream()), "sq_slots_fill")

    # -------------------------------------------------------------- quartets
    def quartets(self, threshold: float, fp32_threshold: float | None = None, q: np.ndarray | None = None):
        """Unique screened quartets.  Returns one QuartetList, or (fp64, fp32) lists
        when fp32_threshold is given (bound >= fp32_threshold goes to FP64).
        ``q`` overrides the per-pair Schwarz factors (None: the engine's own)."""
        key = (float(threshold), None if fp32_threshold is None else float(fp32_threshold))
        if q is None and key in self._quartet_cache:
            return self._quartet_cache[key]
        self._require_eri()
        own = q is None
        qv = self.pair_q if own else np.asarray(q, dtype=np.float64)
        lists, ket_list = screening.build_tasks(self.pair_class, self.pair_npa, self.pair_npb, qv, threshold,
                                                fp32_threshold)
        self.slots  # canonical slot numbering (from the engine's own Schwarz factors)
        out = [self._expand(t, ket_list) for t in lists]
        res = out[0] if len(out) == 1 else (out[0], out[1])
        if own:
            self._quartet_cache[key] = res
        return res

    def _expand(self, tasks: dict, ket_list: np.ndarray) -> QuartetList:
        bra, kst, cnt, toff, off = screening.flatten_tasks(tasks)
        nq = int(off[-1])
        dev = self.device
        pairs = torch.empty((max(nq, 1), 2), dtype=torch.int32, device=dev)
        if nq:
            # quartet entries are slot ids: map bra pair ids and the ket order
            t_bra = torch.tensor(self.slot_of_pair[bra], dtype=torch.int32, device=dev)
            t_kst = torch.tensor(kst, dtype=torch.int32, device=dev)
            t_cnt = torch.tensor(cnt.astype(np.int32), dtype=torch.int32, device=dev)
            t_off = torch.tensor(toff, dtype=torch.int64, device=dev)
            t_ket = torch.tensor(self.slot_of_pair[ket_list], dtype=torch.int32, device=dev)
            check(self.lib.sq_quartets_expand(len(bra), ptr(t_bra), ptr(t_kst), ptr(t_cnt), ptr(t_off),
                                              ptr(t_ket), ptr(pairs), nq, self._stream()), "sq_quartets_expand")
        return QuartetList(pairs, off)

    # ------------------------------------------------------------ integrals
    def one_electron(self):
        """S, T, V (nbf x nbf FP64 device tensors)."""
        n = self.nbf
        S = torch.zeros((n, n), dtype=torch.float64, device=self.device)
        T = torch.zeros_like(S)
        V = torch.zeros_like(S)
        check(self.lib.sq_one_electron(ctypes.byref(self.cbasis), ptr(self.tab64), ptr(S), ptr(T), ptr(V),
                                       self._stream()), "sq_one_electron")
        return S, T, V

    def eri_dense(self, threshold: float = 1e-12) -> torch.Tensor:
        """Dense (nbf,)*4 FP64 ERI tensor on the device, screened like the reference driver."""
        return self.eri_dense_with_q(self.pair_q, threshold)

    def eri_dense_with_q(self, q: np.ndarray | None, threshold: float) -> torch.Tensor:
        """Dense tensor screened with per-pair factors q (None: no screening)."""
        n = self.nbf
        V = torch.zeros((n, n, n, n), dtype=torch.float64, device=self.device)
        if q is None:
            ql = self.quartets(0.0, q=np.ones(self.npair))
        elif q is self.pair_q:
            ql = self.quartets(threshold)
        else:
            ql = self.quartets(threshold, q=q)
        qs = ql.cstruct()
        check(self.lib.sq_eri_dense(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                    ctypes.byref(qs), ptr(self.tab64), ptr(V), self._stream()), "sq_eri_dense")
        return V

    def _scratch(self):
        n = self.nbf
        if self._jk_scratch is None:
            dev = self.device
            self._jk_scratch = (
                torch.empty((n, n), dtype=torch.float64, device=dev),
                torch.empty((n, n), dtype=torch.float64, device=dev),
                torch.empty((n, n), dtype=torch.float32, device=dev),
            )
        return self._jk_scratch

    def jk_accumulate(self, D: torch.Tensor, lists, precisions, Jacc=None, Kacc=None):
        """Run sq_jk for each (quartet list, precision); returns (Jacc, Kacc)."""
        Ja, Ka, D32 = self._scratch()
        if Jacc is None:
            Jacc, Kacc = Ja, Ka
        Jacc.zero_()
        Kacc.zero_()
        D = D.contiguous()
        for ql, prec in zip(lists, precisions):
            if ql.nquartet == 0:
                continue
            qs = ql.cstruct()
            check(self.lib.sq_jk(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                 ctypes.byref(qs), ptr(self.tab64), ptr(self.tab32), ptr(D), ptr(D32), ptr(Jacc),
                                 ptr(Kacc), _lib.PRECISIONS[prec], self._stream()), "sq_jk")
        return Jacc, Kacc

    def jk(self, D: torch.Tensor, threshold: float = 1e-12, precision: str = "fp64",
           fp32_threshold: float = 1e-4):
        """Coulomb and exchange matrices J, K (symmetrised) for density D.

        precision: "fp64" (every quartet FP64), "mixed" (bound < fp32_threshold
        in FP32 with FP64 Boys), "mixed_boys32" (those quartets fully FP32).
        """
        if precision == "fp64":
            lists, precs = [self.quartets(threshold)], ["fp64"]
        else:
            q64, q32 = self.quartets(threshold, fp32_threshold)
            lists = [q64, q32]
            precs = ["fp64", "fp32" if precision == "mixed" else "fp32_boys32"]
        Jacc, Kacc = self.jk_accumulate(D, lists, precs)
        J = torch.empty_like(Jacc)
        K = torch.empty_like(Kacc)
        check(self.lib.sq_fock_build(self.nbf, None, ptr(Jacc), ptr(Kacc), None, ptr(J), ptr(K), self._stream()),
              "sq_fock_build")
        return J, K

    def fock(self, H: torch.Tensor, D: torch.Tensor, threshold: float = 1e-12, precision: str = "fp64",
             fp32_threshold: float = 1e-4) -> torch.Tensor:
        """F = H + J - K/2 built directly from screened ERIs."""
        if precision == "fp64":
            lists, precs = [self.quartets(threshold)], ["fp64"]
        else:
            q64, q32 = self.quartets(threshold, fp32_threshold)
            lists = [q64, q32]
            precs = ["fp64", "fp32" if precision == "mixed" else "fp32_boys32"]
        Jacc, Kacc = self.jk_accumulate(D, lists, precs)
        F = torch.empty_like(Jacc)
        check(self.lib.sq_fock_build(self.nbf, ptr(H.contiguous()), ptr(Jacc), ptr(Kacc), ptr(F), None, None,
                                     self._stream()), "sq_fock_build")
        return F

    # -------------------------------------------------------------- gradient
    def nuclear_gradient(self, D: torch.Tensor, threshold: float = 1e-12) -> np.ndarray:
        """RHF nuclear gradient dE_total/dR (natom x 3, Eh/bohr) at the converged density D.

        Electronic part from the adjoint kernels (sq_grad_1e, sq_grad_2e) with
        W = D F D / 2, F = H + J - K/2 built from D; nuclear-repulsion part on
        the host.
        """
        self._require_eri()
        D = D.to(device=self.device, dtype=torch.float64).contiguous()
        S, T, V = self.one_electron()
        F = self.fock(T + V, D, threshold, "fp64")
        W = (0.5 * D @ F @ D).contiguous()
        natom = len(self.mol.atoms)
        grad = torch.zeros((natom, 3), dtype=torch.float64, device=self.device)
        check(self.lib.sq_grad_1e(ctypes.byref(self.cbasis), ptr(self.tab64), ptr(D), ptr(W), ptr(grad),
                                  self._stream()), "sq_grad_1e")
        ql = self.quartets(threshold)
        qs = ql.cstruct()
        check(self.lib.sq_grad_2e(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                  ctypes.byref(qs), ptr(self.tab64), ptr(D), ptr(grad), self._stream()),
              "sq_grad_2e")
        return grad.cpu().numpy() + nuclear_repulsion_gradient(self.mol)


def nuclear_repulsion_gradient(mol: _Molecule) -> np.ndarray:
    """d/dR_A of sum_{i<j} Z_i Z_j / R_ij."""
    Z = mol.atom_charges
    R = mol.atom_coordinates
    g = np.zeros_like(R)
    for i in range(len(Z)):
        for j in range(len(Z)):
            if i != j:
                d = R[i] - R[j]
                g[i] -= Z[i] * Z[j] * d / np.linalg.norm(d) ** 3
    return g
