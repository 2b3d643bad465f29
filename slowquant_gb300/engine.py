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
* slots: the per-thread class kernels read primitive-pair data through the
  slot layout, which keeps only the primitive pairs that can matter: pair
  (i, j) is dropped when its primitive Schwarz factor times the largest one
  in the basis is below PRIM_SCREEN (far-apart tight primitives), and pairs
  are grouped by the surviving count.
* split quartets: one thread per contracted quartet leaves the heavy ones
  (e.g. (ss|ss) over 8-primitive oxygen s shells: 4096 primitive quartets)
  as a long tail.  A J/K quartet whose primitive count exceeds SPLIT_TARGET
  is emitted S times with bra "sub-slots" that cover consecutive chunks of
  the bra primitive pairs; J and K are linear in the integrals, so the S
  partial epilogues add up to the full contribution.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, flops, screening
from ._lib import SqBasis, SqPairs, SqQuartets, SqSlots, check, ptr
from .molecule import _Molecule

NCART = [1, 3, 6, 10]
# bound on |(ij|kl)| of a primitive quartet below which primitive pair ij is left out
PRIM_SCREEN = 1e-17
# work per thread, in (ss|ss) primitive quartets, above which a J/K quartet is
# split over its bra primitives (a class's primitive quartet weighs its model
# FLOPs over those of (ss|ss))
SPLIT_TARGET = 512
# primitive pairs per chunk (at least) in the per-chunk precision mode
CHUNK_MIN = 2
# heavy per-thread classes, (dp|pp) to (dd|ds): a short list of them is bound by
# one thread's serial, spilled quartet; below KET_SPLIT_PER_SM entries per SM
# their quartets can be cut into ket sub-slot chunks (at most KET_SPLIT_MAX),
# which multiplies the threads in flight.  Off (0) by default: on (H2O)16
# cc-pVDZ, 256 per SM halved those launches timed alone (0.77 -> 0.42 ms for
# (dp|pp)) but the concurrent builds took longer (mixed_df 6.09 -> 6.40 ms),
# because the extra digestion work competes with the other classes' launches.
KET_SPLIT_CLASSES = frozenset(range(12, 19))
KET_SPLIT_PER_SM = 0
KET_SPLIT_MAX = 8
# f-shell classes with per-thread J/K kernels in every precision: (fs|ss), (fs|ps), (fp|ss)
F_PER_THREAD = frozenset({21, 22, 28})
_W_SSSS = flops.flops_per_primitive_quartet(0, 0, 0, 0)
CLASS_WEIGHT = [flops.flops_per_primitive_quartet(*flops.quartet_class_l(c)) / _W_SSSS
                for c in range(screening.NQCLASS)]


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
        self.prim_off_host = prim_off
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
        self.pp_off_host = pp_off
        self.pair_hs = hs
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

    @property
    def prim_q(self) -> np.ndarray:
        """sqrt(max (ij|ij)) of every primitive pair, indexed like the pair table's
        primitive pairs (pp_off[P] + i * nprim_b + j).

        Each primitive i of shell a with coefficient c_i is one single-primitive
        pseudo-shell; the Schwarz kernel then gives the factor of the product
        c_i c_j g_i g_j directly, in the normalisation of the contracted pair.
        """
        if getattr(self, "_prim_q", None) is None:
            self._require_eri()
            dev = self.device
            total = int(self.pp_off_host[-1])
            if total == 0:
                self._prim_q = np.zeros(0)
                return self._prim_q
            shell_of_prim = np.repeat(np.arange(self.nshell), self.nprim)
            nps = len(shell_of_prim)
            i32 = dict(dtype=torch.int32, device=dev)
            t_center = self.t_center[torch.tensor(shell_of_prim, device=dev)].contiguous()
            t_l = torch.tensor(self.l[shell_of_prim], **i32)
            t_np = torch.ones(nps, **i32)
            t_poff = torch.arange(nps, **i32)
            t_bf = torch.zeros(nps, **i32)
            t_satom = torch.tensor(self.shell_atom[shell_of_prim], **i32)
            b = SqBasis()
            b.nshell, b.nbf, b.natom, b.nprim_total = nps, self.nbf, self.cbasis.natom, nps
            b.center, b.l, b.nprim, b.prim_off, b.bf_off = ptr(t_center), ptr(t_l), ptr(t_np), ptr(t_poff), ptr(t_bf)
            b.exps, b.coefs = ptr(self.t_exps), ptr(self.t_coefs)
            b.atom_xyz, b.atom_charge, b.shell_atom = ptr(self.t_atom_xyz), ptr(self.t_atom_charge), ptr(t_satom)
            rep = np.repeat(np.arange(self.npair), self.pair_np)
            local = np.arange(total) - self.pp_off_host[:-1][rep]
            npb = self.pair_npb[rep]
            sa = self.prim_off_host[self.pair_shells[rep, 0]] + local // npb
            sb = self.prim_off_host[self.pair_shells[rep, 1]] + local % npb
            hs = self.pair_hs[rep]
            t_shells = torch.tensor(np.stack([sa, sb], 1).astype(np.int32), **i32)
            t_ppoff = torch.arange(total + 1, **i32)
            t_hoff = torch.tensor(np.concatenate([[0], np.cumsum(hs)[:-1]]).astype(np.int64), dtype=torch.int64,
                                  device=dev)
            t_prim = torch.empty(total * 8, dtype=torch.float64, device=dev)
            t_herm = torch.empty(max(int(hs.sum()), 1), dtype=torch.float64, device=dev)
            pp = SqPairs()
            pp.npair, pp.nprimpair = total, total
            pp.shells, pp.pp_off, pp.herm_off = ptr(t_shells), ptr(t_ppoff), ptr(t_hoff)
            pp.prim, pp.herm = ptr(t_prim), ptr(t_herm)
            check(self.lib.sq_pair_prep(ctypes.byref(b), ctypes.byref(pp), self._stream()), "sq_pair_prep")
            # diagonal quartets of the pseudo pairs, grouped by class (pairs are class-sorted)
            cls = self.pair_class[rep]
            lists = {}
            for pc in np.unique(cls):
                idx = np.nonzero(cls == pc)[0].astype(np.int32)
                lists[quartet_class(int(pc), int(pc))] = np.stack([idx, idx], axis=1)
            ql = self._class_lists(lists)
            q = torch.zeros(total, dtype=torch.float64, device=dev)
            qs = ql.cstruct()
            check(self.lib.sq_schwarz(ctypes.byref(b), ctypes.byref(pp), ctypes.byref(qs), ptr(self.tab64), ptr(q),
                                      self._stream()), "sq_schwarz")
            self._prim_q = q.cpu().numpy()
        return self._prim_q

    def _prim_keep(self) -> np.ndarray:
        """Primitive pairs kept in the slot data: q_ij * max q >= PRIM_SCREEN bounds what a
        dropped pair adds to any primitive quartet; each pair keeps at least its largest one."""
        qp = self.prim_q
        keep = qp * (qp.max() if len(qp) else 0.0) >= PRIM_SCREEN
        if len(qp):
            rep = np.repeat(np.arange(self.npair), self.pair_np)
            # index of each pair's largest primitive factor
            order = np.lexsort((-qp, rep))
            first = order[np.concatenate([[0], np.cumsum(self.pair_np)[:-1]])[self.pair_np > 0]]
            keep[first] = True
        return keep

    @property
    def pair_npp_eff(self) -> np.ndarray:
        """Primitive pairs of each pair that survive primitive screening."""
        if getattr(self, "_npp_eff", None) is None:
            keep = self._prim_keep()
            self._keep = keep
            self._npp_eff = np.add.reduceat(keep.astype(np.int64), self.pp_off_host[:-1]) if len(keep) else \
                np.zeros(self.npair, np.int64)
            self._npp_eff[self.pair_np == 0] = 0
        return self._npp_eff

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
        npp_eff = self.pair_npp_eff
        groups = screening.pair_groups(self.pair_class, npp_eff, np.ones_like(npp_eff), q)
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
            nppg = int(npp_eff[members[0]])
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
        # kept primitive pairs of every slot (local indices in the pair's table)
        starts = self.pp_off_host[:-1][slot_pair]
        lens = self.pair_np[slot_pair]
        first = np.repeat(np.concatenate([[0], np.cumsum(lens)[:-1]]), lens)
        gidx = np.repeat(starts, lens) + (np.arange(int(lens.sum())) - first)
        kept = self._keep[gidx]
        # each slot's kept primitive pairs in descending primitive Schwarz factor,
        # so that chunk 0 of a sub-slot split holds the largest ones
        slot_of_entry = np.repeat(np.arange(nslot), lens)[kept]
        gk = gidx[kept]
        order = np.lexsort((-self.prim_q[gk], slot_of_entry))
        gk = gk[order]
        prim_src = (gk - np.repeat(starts, npp)).astype(np.int32)
        prim_src_off = np.concatenate([[0], np.cumsum(npp)[:-1]]).astype(np.int64)
        assert len(prim_src) == int(npp.sum())
        # prefix sums of the sorted factors: the bound sum_ij q_ij of any chunk
        qsorted = self.prim_q[gk]
        qcum = np.concatenate([[0.0], np.cumsum(qsorted)])
        self.slot_of_pair = np.empty(nslot, np.int32)
        self.slot_of_pair[slot_pair] = np.arange(nslot, dtype=np.int32)
        # sub-slots: S (a power of two) chunks of a slot's primitive pairs, for the
        # S a quartet with the heaviest ket group can ask for; sub-slot k of S covers
        # primitive pairs [k*n//S, (k+1)*n//S) of its parent and shares its data
        max_np = int(npp.max()) if nslot else 0
        la_s = self.l[self.pair_shells[slot_pair, 0]] if nslot else np.zeros(0, np.int32)
        lb_s = self.l[self.pair_shells[slot_pair, 1]] if nslot else np.zeros(0, np.int32)
        E_s = np.array([herm_size(int(a), int(b)) for a, b in zip(la_s, lb_s)], dtype=np.int64)
        # heaviest quartet class a slot can be the bra of: (its pair class | its pair class)
        pc_s = self.pair_class[slot_pair] if nslot else np.zeros(0, np.int64)
        w_s = np.array([CLASS_WEIGHT[screening.quartet_class(int(c), int(c))] for c in pc_s], dtype=np.float64)
        self.sub_first, subs = screening.sub_slot_table(npp, pbase, pstride, hbase, E_s, w_s, qcum, prim_src_off,
                                                        max_np, SPLIT_TARGET, CHUNK_MIN)
        sub_pair = [slot_pair[subs["parent"]]] if len(subs["parent"]) else []
        sub_npp, sub_pb, sub_ps, sub_hb = [subs["npp"]], [subs["pbase"]], [subs["pstride"]], [subs["hbase"]]
        sub_code, sub_qsum = [subs["code"]], [subs["qsum"]]
        nsub = len(subs["parent"])
        self.nslot_base = nslot
        if nsub:
            slot_pair = np.concatenate([slot_pair] + sub_pair).astype(np.int32)
            npp = np.concatenate([npp] + sub_npp).astype(np.int32)
            pbase = np.concatenate([pbase] + sub_pb).astype(np.int32)
            pstride = np.concatenate([pstride] + sub_ps).astype(np.int32)
            hbase = np.concatenate([hbase] + sub_hb).astype(np.int64)
        sub = np.concatenate([np.zeros(self.nslot_base, np.int64)] + sub_code).astype(np.int32)
        self.slot_sub = sub
        # sum of the primitive Schwarz factors of every slot and sub-slot: a bound on
        # its partial contracted factor, |(chunk|ket)| <= qsum[chunk] * qsum[ket]
        base_qsum = qcum[prim_src_off + npp[: self.nslot_base]] - qcum[prim_src_off] if self.nslot_base else \
            np.zeros(0)
        self.slot_qsum = np.concatenate([base_qsum] + sub_qsum) if nsub else base_qsum
        self.slot_pair = slot_pair
        self.slot_npp = npp
        nslot = len(slot_pair)
        dev = self.device
        i32 = dict(dtype=torch.int32, device=dev)
        self.t_slot_pair = torch.tensor(slot_pair, **i32)
        self.t_slot_of_pair = torch.tensor(self.slot_of_pair, **i32)
        self.t_slot_npp = torch.tensor(npp, **i32)
        self.t_slot_pbase = torch.tensor(pbase, **i32)
        self.t_slot_pstride = torch.tensor(pstride, **i32)
        self.t_slot_hbase = torch.tensor(hbase, dtype=torch.int64, device=dev)
        self.t_slot_sub = torch.tensor(sub if nslot else np.zeros(1, np.int32), **i32)
        self.t_slot_prim_src = torch.tensor(prim_src if len(prim_src) else np.zeros(1, np.int32), **i32)
        self.t_slot_prim_src_off = torch.tensor(prim_src_off if nslot else np.zeros(1, np.int64), dtype=torch.int64,
                                                device=dev)
        self.t_slot_prim = torch.empty(max(5 * poff, 1), dtype=torch.float64, device=dev)
        self.t_slot_herm = torch.empty(max(hoff, 1), dtype=torch.float64, device=dev)
        self.t_slot_prim32 = torch.empty(max(5 * poff, 1), dtype=torch.float32, device=dev) if self.fp32 else None
        self.t_slot_herm32 = torch.empty(max(hoff, 1), dtype=torch.float32, device=dev) if self.fp32 else None
        self.t_slot_prim32v = torch.empty(max(8 * poff, 1), dtype=torch.float32, device=dev) if self.fp32 else None
        # double-float copies (hi, lo) for the df64 J/K kernels
        self.t_slot_primdf = torch.empty(max(10 * poff, 2), dtype=torch.float32, device=dev) if self.fp32 else None
        self.t_slot_hermdf = torch.empty(max(2 * hoff, 2), dtype=torch.float32, device=dev) if self.fp32 else None
        self.t_slot_desc = torch.empty(max(8 * nslot, 8), dtype=torch.int32, device=dev)
        # primitive Schwarz factors in the pair table's order, copied into the packed FP32 slot data
        self.t_prim_q = torch.tensor(self.prim_q if len(self.prim_q) else np.zeros(1), dtype=torch.float64,
                                     device=dev)
        self.cpairs.pq = ptr(self.t_prim_q)
        s = SqSlots()
        s.nslot, s.npp_total, s.nherm_total = nslot, poff, hoff
        s.pair, s.npp, s.pbase, s.pstride, s.hbase = (ptr(self.t_slot_pair), ptr(self.t_slot_npp),
                                                      ptr(self.t_slot_pbase), ptr(self.t_slot_pstride),
                                                      ptr(self.t_slot_hbase))
        s.prim, s.herm = ptr(self.t_slot_prim), ptr(self.t_slot_herm)
        s.prim32, s.herm32 = ptr(self.t_slot_prim32), ptr(self.t_slot_herm32)
        s.prim_src, s.prim_src_off = ptr(self.t_slot_prim_src), ptr(self.t_slot_prim_src_off)
        s.sub = ptr(self.t_slot_sub)
        s.desc, s.mbase, s.prim32v = ptr(self.t_slot_desc), None, ptr(self.t_slot_prim32v)
        s.primdf, s.hermdf = ptr(self.t_slot_primdf), ptr(self.t_slot_hermdf)
        self._slots = s
        if self.nslot_base:
            # fill the parents' data only: sub-slots point into it
            fill = SqSlots.from_buffer_copy(s)
            fill.nslot = self.nslot_base
            check(self.lib.sq_slots_fill(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(fill),
                                         self._stream()), "sq_slots_fill")
            check(self.lib.sq_slots_describe(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(s),
                                             self._stream()), "sq_slots_describe")

    # -------------------------------------------------------------- quartets
    def quartets(self, threshold: float, fp32_threshold: float | None = None, q: np.ndarray | None = None,
                 split: bool = True, chunks: bool = False):
        """Unique screened quartets.  Returns one QuartetList, or (fp64, fp32) lists
        when fp32_threshold is given (bound >= fp32_threshold goes to FP64).
        ``q`` overrides the per-pair Schwarz factors (None: the engine's own).
        ``split``: heavy quartets of the per-thread J/K classes are emitted as
        bra sub-slot chunks (J/K lists only; dense tensors and gradients need
        whole quartets).  ``chunks`` (with fp32_threshold): the precision test
        is applied per bra chunk of the FP64 quartets of the per-thread classes:
        a chunk goes to FP32 when the sum of its primitive Schwarz factors times
        the ket's is below fp32_threshold."""
        s64, s32 = self._split_classes()
        key = (float(threshold), None if fp32_threshold is None else float(fp32_threshold), bool(split),
               bool(chunks), s64)
        if q is None and key in self._quartet_cache:
            return self._quartet_cache[key]
        self._require_eri()
        own = q is None
        qv = self.pair_q if own else np.asarray(q, dtype=np.float64)
        npp_eff = self.pair_npp_eff
        lists, ket_list = screening.build_tasks(self.pair_class, npp_eff, np.ones_like(npp_eff), qv, threshold,
                                                fp32_threshold)
        self.slots  # canonical slot numbering (from the engine's own Schwarz factors)
        # classes with per-thread kernels: 0-18 (FP64: 12-18 unless switched off), FP32 0-18,
        # and the light f classes in both
        split_sets = [s64, s32] if split else [frozenset(), frozenset()]
        if chunks and fp32_threshold is not None:
            out = self._chunk_lists(lists, ket_list, float(fp32_threshold), s64)
        else:
            out = [self._expand(t, ket_list, split_sets[li]) for li, t in enumerate(lists)]
        if split:
            out = [self._ket_split(ql, split_sets[li] & KET_SPLIT_CLASSES) for li, ql in enumerate(out)]
        res = out[0] if len(out) == 1 else (out[0], out[1])
        if own:
            self._quartet_cache[key] = res
        return res

    def _ket_split(self, ql: QuartetList, classes) -> QuartetList:
        """Cut the ket of every quartet of a short heavy-class segment into sub-slot chunks.

        A class segment of n < KET_SPLIT_PER_SM * SMs entries asks for S = the
        power of two (at most KET_SPLIT_MAX) that brings it to that size; each
        entry (bra, ket) with a whole ket slot becomes (bra, chunk j of S') for
        the largest S' <= S its ket has chunks for.  J and K are linear in the
        ket's primitive pairs, so the partial quartets add up to the whole."""
        target = KET_SPLIT_PER_SM * torch.cuda.get_device_properties(self.device).multi_processor_count
        counts = ql.class_counts()
        todo = [c for c in sorted(classes) if 0 < counts[c] < target]
        if not todo or not self.sub_first:
            return ql
        host = ql.pairs[: ql.nquartet].cpu().numpy()
        parts, off = [], np.zeros_like(ql.class_off)
        for c in range(_lib.SQ_MAX_QCLASS):
            seg = host[ql.class_off[c]:ql.class_off[c + 1]]
            if c in todo:
                want = 1
                while want < KET_SPLIT_MAX and len(seg) * want < target:
                    want *= 2
                seg = screening.ket_chunk_entries(seg, self.sub_first, self.nslot_base, want)
            parts.append(seg)
            off[c + 1] = off[c] + len(seg)
        allp = np.concatenate(parts).astype(np.int32) if int(off[-1]) else np.zeros((0, 2), np.int32)
        t = torch.tensor(allp, dtype=torch.int32, device=self.device).reshape(-1, 2).contiguous()
        return QuartetList(t, off)

    def _split_classes(self):
        """(FP64, FP32) sets of the classes whose J/K quartets may be split into
        sub-slot chunks: those on per-thread kernels in that precision."""
        hi = self._fp64_per_thread_max()
        return frozenset(range(hi + 1)) | F_PER_THREAD, frozenset(range(19)) | F_PER_THREAD

    def _fp64_per_thread_max(self) -> int:
        """Highest class index up to which every FP64 J/K launch runs on a per-thread kernel
        (18 with the default SQ_OPT_FP64_UNROLLED_HIGH, 11 otherwise).  Sub-slot chunks
        of one quartet must all go through kernels of the same kind, which number a
        slot's primitive pairs the same way."""
        mask = int(self.lib.sq_get_option(_lib.SQ_OPT_FP64_UNROLLED_HIGH))
        return 18 if all((mask >> c) & 1 for c in range(12, 19)) else 11

    def _chunk_lists(self, lists, ket_list: np.ndarray, tau: float, split64=None):
        """(FP64, FP32) lists with the precision test per bra primitive chunk.

        FP64 quartets of the per-thread classes (split64: 0-18 and F_PER_THREAD) are cut into S chunks of
        their bra's primitive pairs (sorted by descending factor, CHUNK_MIN to
        2 CHUNK_MIN per chunk, more when the quartet is heavy), kets are cut the same way where
        a ket straddles the threshold, and each (bra chunk, ket chunk) is placed
        by its own bound; FP32 quartets stay whole.
        """
        t64, t32 = lists
        if split64 is None:
            split64 = self._split_classes()[0]
        q32 = self._expand(t32, ket_list, split64)
        npp = self.slot_npp
        ket_slots = self.slot_of_pair[ket_list]
        keep64 = {c: [] for c in range(screening.NQCLASS)}
        move32 = {c: [] for c in range(screening.NQCLASS)}
        whole64 = {c: [] for c in range(screening.NQCLASS)}
        for c in range(screening.NQCLASS):
            for m, st, n in t64[c]:
                slots = self.slot_of_pair[m]
                if c not in split64 or len(m) == 0:
                    whole64[c].append((m, st, n))  # pair ids: _expand maps them to slots
                    continue
                nb = int(npp[slots[0]])
                cost = nb * int(npp[ket_slots[st[0]]]) * CLASS_WEIGHT[c]
                S = 1
                while (2 * S) in self.sub_first and self.sub_first[2 * S][slots[0]] >= 0 and \
                        (nb >= 2 * CHUNK_MIN * S or cost > SPLIT_TARGET * S):
                    S *= 2
                pairs = screening.expand_host(slots.astype(np.int32), st.astype(np.int32), n.astype(np.int64),
                                              ket_slots)
                if S == 1:
                    chunk = pairs
                else:
                    first = self.sub_first[S][pairs[:, 0]]
                    chunk = np.concatenate([np.stack([(first + k).astype(np.int32), pairs[:, 1]], 1)
                                            for k in range(S)])
                k64, k32 = self._ket_chunks(chunk, tau)
                keep64[c].append(k64)
                move32[c].append(k32)
        # FP64 list: whole-quartet blocks of the warp classes (device expand) and
        # the kept chunks; FP32 list: the quartet-level FP32 list plus the moved chunks
        q64w = self._expand(whole64, ket_list)
        dev = self.device

        def merge(base, extra):
            parts, off = [], np.zeros(screening.NQCLASS + 1, dtype=np.int64)
            for c in range(screening.NQCLASS):
                seg = base.pairs[base.class_off[c]:base.class_off[c + 1]] if base is not None else None
                ex = np.concatenate(extra[c]) if extra[c] else np.zeros((0, 2), np.int32)
                n = (0 if seg is None else int(base.class_off[c + 1] - base.class_off[c])) + len(ex)
                off[c + 1] = off[c] + n
                if seg is not None and len(seg):
                    parts.append(seg[: int(base.class_off[c + 1] - base.class_off[c])])
                if len(ex):
                    parts.append(torch.tensor(ex.astype(np.int32), device=dev))
            pairs = torch.cat(parts).contiguous() if parts else torch.empty((1, 2), dtype=torch.int32, device=dev)
            return QuartetList(pairs, off)

        return [merge(q64w, keep64), merge(q32, move32)]

    def _ket_chunks(self, entries: np.ndarray, tau: float):
        """Partition (bra, ket) entries by bound into (FP64, FP32) entries.

        An entry whose whole ket passes or fails the test stays whole; otherwise
        its ket is cut into chunks of CHUNK_MIN to 2 CHUNK_MIN primitive pairs (ket sub-slots)
        and each chunk is placed by qsum[bra] * qsum[ket chunk].
        """
        qs = self.slot_qsum
        qb = qs[entries[:, 0]]
        whole = qb * qs[entries[:, 1]]
        # the largest and smallest ket chunk bounds decide whether the ket must be cut
        npp = self.slot_npp
        kslot = entries[:, 1]
        nk = npp[kslot].astype(np.int64)
        Sk = np.ones(len(entries), np.int64)
        for S in sorted(self.sub_first):
            ok = (nk >= 2 * CHUNK_MIN * S) & (self.sub_first[S][kslot] >= 0)
            Sk[ok] = S
        out64, out32 = [], []
        one = Sk == 1
        big = whole >= tau
        out64.append(entries[one & big])
        out32.append(entries[one & ~big])
        for S in sorted(set(Sk[~one].tolist())):
            sel = np.nonzero(Sk == S)[0]
            first = self.sub_first[S][kslot[sel]]
            kc = first[:, None] + np.arange(S)[None, :]  # ket chunk ids per entry
            b = qb[sel, None] * qs[kc]
            all_big = (b >= tau).all(axis=1)
            all_small = (b < tau).all(axis=1)
            out64.append(entries[sel[all_big]])
            out32.append(entries[sel[all_small]])
            mix = ~(all_big | all_small)
            if mix.any():
                bras = np.repeat(entries[sel[mix], 0], S)
                kets = kc[mix].ravel()
                bm = b[mix].ravel() >= tau
                pairs = np.stack([bras, kets], 1).astype(np.int32)
                out64.append(pairs[bm])
                out32.append(pairs[~bm])
        cat = lambda xs: np.concatenate(xs).astype(np.int32) if xs else np.zeros((0, 2), np.int32)  # noqa: E731
        return cat(out64), cat(out32)

    def _split_tasks(self, tasks: dict, ket_list: np.ndarray, split_classes=frozenset()) -> dict:
        """Bra slot ids of every task block, heavy blocks replaced by their sub-slot chunks."""
        npp = self.slot_npp
        out = {}
        for c in range(screening.NQCLASS):
            blocks = []
            for m, st, n in tasks[c]:
                slots = self.slot_of_pair[m]
                if c in split_classes and len(m):
                    cost = int(npp[slots[0]]) * int(npp[self.slot_of_pair[ket_list[st[0]]]]) * CLASS_WEIGHT[c]
                    S = 1
                    while cost > SPLIT_TARGET * S and (2 * S) in self.sub_first and \
                            self.sub_first[2 * S][slots[0]] >= 0:
                        S *= 2
                    if S > 1:
                        first = self.sub_first[S][slots]
                        for k in range(S):
                            blocks.append(((first + k).astype(np.int32), st, n))
                        continue
                blocks.append((slots.astype(np.int32), st, n))
            out[c] = blocks
        return out

    def _expand(self, tasks: dict, ket_list: np.ndarray, split_classes=frozenset()) -> QuartetList:
        bra, kst, cnt, toff, off = screening.flatten_tasks(self._split_tasks(tasks, ket_list, split_classes))
        nq = int(off[-1])
        dev = self.device
        pairs = torch.empty((max(nq, 1), 2), dtype=torch.int32, device=dev)
        if nq:
            # quartet entries are slot ids: bra slots (or sub-slots) and the ket order
            t_bra = torch.tensor(bra, dtype=torch.int32, device=dev)
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

    def multipole(self, order, origin=None) -> torch.Tensor:
        """Multipole matrix <a| (x-Cx)^ex (y-Cy)^ey (z-Cz)^ez |b> (nbf x nbf FP64 device tensor).

        origin: C in bohr, in the molecule's own coordinates (default: its
        centre of mass, as multipole.py:10-45 uses)."""
        n = self.nbf
        o = np.asarray(order, dtype=np.int32).reshape(3)
        c = (self.mol.center_of_mass if origin is None else np.asarray(origin, dtype=np.float64)) - self.origin
        c = np.ascontiguousarray(c, dtype=np.float64)
        M = torch.zeros((n, n), dtype=torch.float64, device=self.device)
        check(self.lib.sq_multipole(ctypes.byref(self.cbasis), o.ctypes.data, c.ctypes.data, ptr(M), self._stream()),
              "sq_multipole")
        return M

    def eri_dense(self, threshold: float = 1e-12) -> torch.Tensor:
        """Dense (nbf,)*4 FP64 ERI tensor on the device, screened like the reference driver."""
        return self.eri_dense_with_q(self.pair_q, threshold)

    def eri_dense_with_q(self, q: np.ndarray | None, threshold: float) -> torch.Tensor:
        """Dense tensor screened with per-pair factors q (None: no screening)."""
        n = self.nbf
        V = torch.zeros((n, n, n, n), dtype=torch.float64, device=self.device)
        if q is None:
            ql = self.quartets(0.0, q=np.ones(self.npair), split=False)
        elif q is self.pair_q:
            ql = self.quartets(threshold, split=False)
        else:
            ql = self.quartets(threshold, q=q, split=False)
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

    def jk_accumulate(self, D: torch.Tensor, lists, precisions, Jacc=None, Kacc=None, prim_tau: float = 0.0):
        """Run sq_jk for each (quartet list, precision); returns (Jacc, Kacc).

        Precision "fp64_prim" runs sq_jk_prim with bound ``prim_tau``, "df64_prim"
        sq_jk_df with that bound and "df64" sq_jk_df with none."""
        Ja, Ka, D32 = self._scratch()
        if Jacc is None:
            Jacc, Kacc = Ja, Ka
        Jacc.zero_()
        Kacc.zero_()
        D = D.contiguous()
        work = [(ql, prec) for ql, prec in zip(lists, precisions) if ql.nquartet]
        main = torch.cuda.current_stream(self.device)
        # the lists after the first run from side streams, concurrently with the
        # first (all of them only add into Jacc/Kacc)
        side = self._side_streams(len(work) - 1)
        for s in side:
            s.wait_stream(main)  # after the zeroing, before the first list's launches
        for i, (ql, prec) in enumerate(work):
            s = main if i == 0 else side[i - 1]
            qs = ql.cstruct()
            if prec == "fp64_prim":
                check(self.lib.sq_jk_prim(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs),
                                          ctypes.byref(self.slots), ctypes.byref(qs), ptr(self.tab64), ptr(self.tab32),
                                          ptr(D), ptr(Jacc), ptr(Kacc), float(prim_tau), s.cuda_stream), "sq_jk_prim")
                continue
            if prec in ("df64", "df64_prim"):
                if getattr(self, "_ddf", None) is None:
                    self._ddf = torch.empty(2 * self.nbf * self.nbf, dtype=torch.float32, device=self.device)
                tau = float(prim_tau) if prec == "df64_prim" else 0.0
                check(self.lib.sq_jk_df(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                        ctypes.byref(qs), ptr(self.tab64), ptr(self.tab32), ptr(D), ptr(self._ddf),
                                        ptr(Jacc), ptr(Kacc), tau, s.cuda_stream), "sq_jk_df")
                continue
            check(self.lib.sq_jk(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                 ctypes.byref(qs), ptr(self.tab64), ptr(self.tab32), ptr(D), ptr(D32), ptr(Jacc),
                                 ptr(Kacc), _lib.PRECISIONS[prec], s.cuda_stream), "sq_jk")
        for s in side:
            main.wait_stream(s)
        return Jacc, Kacc

    def df_class(self, qclass: int, nquartets: int) -> bool:
        """True when a "df64"/"df64_prim" launch of this class and length runs in double-float (sq_df_class)."""
        return bool(self.lib.sq_df_class(int(qclass), int(nquartets)))

    def _side_streams(self, n: int):
        if not hasattr(self, "_sides"):
            self._sides = []
        while len(self._sides) < n:
            self._sides.append(torch.cuda.Stream(self.device))
        return self._sides[:n]

    def _lists_for(self, precision: str, threshold: float, fp32_threshold: float):
        """Quartet lists and their launch precisions for a J/K precision mode.

        "fp64": every quartet FP64; "mixed": quartets with bound < fp32_threshold
        in FP32 (FP64 Boys recursion); "mixed_boys32": the same, recursion in FP32
        too; "mixed_chunk": the "mixed" test applied per bra primitive chunk of
        the large-bound quartets (classes with per-thread kernels);
        "mixed_prim": the "mixed" lists, with the large-bound quartets' primitive
        quartets of bound q_ij q_kl < fp32_threshold run in FP32 inside the FP64
        launch (sq_jk_prim); "df64": every quartet in double-float arithmetic on
        the FP32 pipe (sq_jk_df, classes (ss|ss)-(dd|ds); the others FP64);
        "mixed_df": "mixed_prim" with double-float in place of FP64.
        """
        if precision == "fp64":
            return [self.quartets(threshold)], ["fp64"]
        if precision == "df64":
            return [self.quartets(threshold)], ["df64"]
        if precision in ("mixed_prim", "mixed_df"):
            q64, q32 = self.quartets(threshold, fp32_threshold)
            return [q64, q32], ["fp64_prim" if precision == "mixed_prim" else "df64_prim", "fp32"]
        if precision not in ("mixed", "mixed_boys32", "mixed_chunk"):
            raise ValueError(f"unknown precision {precision!r}")
        q64, q32 = self.quartets(threshold, fp32_threshold, chunks=precision == "mixed_chunk")
        return [q64, q32], ["fp64", "fp32_boys32" if precision == "mixed_boys32" else "fp32"]

    def jk_multi(self, Ds: torch.Tensor, threshold: float = 1e-12, precision: str = "fp64",
                 fp32_threshold: float = 1e-4):
        """J_i, K_i (symmetrised, [nd, nbf, nbf]) for a stack of densities Ds [nd, nbf, nbf],
        with each quartet's integrals evaluated once for all of them (sq_jk_multi)."""
        if precision in ("mixed_prim", "mixed_df", "df64"):
            raise ValueError(f"precision {precision!r} serves one density per call (use 'mixed' for several)")
        lists, precs = self._lists_for(precision, threshold, fp32_threshold)
        Ds = Ds.to(device=self.device, dtype=torch.float64).contiguous()
        nd = Ds.shape[0]
        Jacc = torch.zeros_like(Ds)
        Kacc = torch.zeros_like(Ds)
        D32 = torch.empty(Ds.shape, dtype=torch.float32, device=self.device)
        for ql, prec in zip(lists, precs):
            if ql.nquartet == 0:
                continue
            qs = ql.cstruct()
            check(self.lib.sq_jk_multi(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                       ctypes.byref(qs), ptr(self.tab64), ptr(self.tab32), nd, ptr(Ds), ptr(D32),
                                       ptr(Jacc), ptr(Kacc), _lib.PRECISIONS[prec], self._stream()), "sq_jk_multi")
        J = 0.5 * (Jacc + Jacc.transpose(1, 2))
        K = 0.5 * (Kacc + Kacc.transpose(1, 2))
        return J, K

    def jk(self, D: torch.Tensor, threshold: float = 1e-12, precision: str = "fp64",
           fp32_threshold: float = 1e-4):
        """Coulomb and exchange matrices J, K (symmetrised) for density D.

        precision: "fp64" (every quartet FP64), "mixed" (bound < fp32_threshold
        in FP32 with FP64 Boys), "mixed_boys32" (those quartets fully FP32),
        "mixed_chunk" and "mixed_prim" (the same test at finer grain), "df64" and
        "mixed_df" (double-float arithmetic in place of FP64), see _lists_for.
        """
        lists, precs = self._lists_for(precision, threshold, fp32_threshold)
        Jacc, Kacc = self.jk_accumulate(D, lists, precs, prim_tau=fp32_threshold)
        J = torch.empty_like(Jacc)
        K = torch.empty_like(Kacc)
        check(self.lib.sq_fock_build(self.nbf, None, ptr(Jacc), ptr(Kacc), None, ptr(J), ptr(K), self._stream()),
              "sq_fock_build")
        return J, K

    def fock(self, H: torch.Tensor, D: torch.Tensor, threshold: float = 1e-12, precision: str = "fp64",
             fp32_threshold: float = 1e-4) -> torch.Tensor:
        """F = H + J - K/2 built directly from screened ERIs."""
        lists, precs = self._lists_for(precision, threshold, fp32_threshold)
        Jacc, Kacc = self.jk_accumulate(D, lists, precs, prim_tau=fp32_threshold)
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
        if self.nshell and self.l.max() > _lib.SQ_MAX_L_GRAD:
            raise NotImplementedError(
                f"gradient kernels support shells up to l={_lib.SQ_MAX_L_GRAD}; basis has l={int(self.l.max())}")
        D = D.to(device=self.device, dtype=torch.float64).contiguous()
        S, T, V = self.one_electron()
        F = self.fock(T + V, D, threshold, "fp64")
        W = (0.5 * D @ F @ D).contiguous()
        natom = len(self.mol.atoms)
        grad = torch.zeros((natom, 3), dtype=torch.float64, device=self.device)
        check(self.lib.sq_grad_1e(ctypes.byref(self.cbasis), ptr(self.tab64), ptr(D), ptr(W), ptr(grad),
                                  self._stream()), "sq_grad_1e")
        ql = self.quartets(threshold, split=False)
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
