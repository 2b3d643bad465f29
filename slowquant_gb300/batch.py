"""Many independent molecules in one set of kernel launches.

A batch is one block-diagonal system: shells of all molecules are
concatenated, shell pairs and shell quartets exist only inside a molecule, and
the n_i x n_i matrices (D, J, K, S, T, V, F) of molecule i are packed blocks
of one flat device buffer.  Molecules are ordered by basis size, so the
blocks of equal-size molecules form a [count, n, n] tensor view: the SCF's
linear algebra (DIIS, eigh) runs batched per size group (eigh on the
library's one-CTA-per-matrix Jacobi kernel), and every Fock
build of the whole batch is one launch per quartet class over all molecules'
quartets (heavy-first order across molecules).  Setup (pairs, Schwarz,
one-electron integrals) is also one launch each for the batch.

The steady-state Fock build (zeroing, the class launches, F assembly) is
captured once in a CUDA graph and replayed every SCF iteration.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, screening
from ._lib import SqBasis, SqPairs, SqQuartets, SqSlots, check, ptr
from .engine import CLASS_WEIGHT, F_PER_THREAD, SPLIT_TARGET, QuartetList, herm_size
from .molecule import _Molecule


@dataclass
class SizeGroup:
    nbf: int
    mols: list[int]  # molecule indices (batch order)
    offset: int  # element offset of the group's first block in the packed buffers
    nocc: int


class BatchEngine:
    """Integral engine for a batch of independent molecules on one GPU."""

    def __init__(self, molecules: list[_Molecule], device=None, fp32: bool = True):
        if not torch.cuda.is_available():
            raise RuntimeError("slowquant_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = _lib.lib()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        order = sorted(range(len(molecules)), key=lambda i: (molecules[i].number_bf, i))
        self.order = order
        self.mols = [molecules[i] for i in order]
        self.nmol = len(self.mols)
        self.fp32 = fp32
        dev = self.device
        # ---- concatenated basis with packed matrix addressing
        l, nprim, bf_off, centers, exps, coefs = [], [], [], [], [], []
        mat_base, mat_ld, atom_begin, atom_end, shell_atom, shell_mol = [], [], [], [], [], []
        atom_xyz, atom_charge = [], []
        base = 0
        natom = 0
        self.mol_base, self.mol_nbf, self.mol_shell0 = [], [], []
        for mi, m in enumerate(self.mols):
            n = m.number_bf
            self.mol_base.append(base)
            self.mol_nbf.append(n)
            self.mol_shell0.append(len(l))
            coords = m.atom_coordinates
            origin = coords.mean(axis=0)
            for s in m.shells:
                l.append(s.angular_momentum)
                nprim.append(len(s.exponents))
                bf_off.append(int(s.bf_idx[0]))
                centers.append(np.asarray(s.center) - origin)
                exps.append(s.exponents)
                coefs.append(s.component_independent_coefficients())
                mat_base.append(base)
                mat_ld.append(n)
                atom_begin.append(natom)
                atom_end.append(natom + len(m.atoms))
                shell_atom.append(natom + m.atoms.index(s.origin_atom))
                shell_mol.append(mi)
            atom_xyz.append(coords - origin)
            atom_charge.append(m.atom_charges)
            natom += len(m.atoms)
            base += n * n
        self.mat_total = base
        self.l = np.array(l, dtype=np.int32)
        if self.l.max() > _lib.SQ_MAX_L:
            raise NotImplementedError(f"ERI kernels support shells up to l={_lib.SQ_MAX_L}")
        self.nprim = np.array(nprim, dtype=np.int32)
        self.shell_mol = np.array(shell_mol, dtype=np.int32)
        prim_off = np.concatenate([[0], np.cumsum(self.nprim)[:-1]]).astype(np.int32)
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        self._keep = [
            torch.tensor(np.array(centers), **f64), torch.tensor(self.l, **i32), torch.tensor(self.nprim, **i32),
            torch.tensor(prim_off, **i32), torch.tensor(np.array(bf_off, dtype=np.int32), **i32),
            torch.tensor(np.concatenate(exps), **f64), torch.tensor(np.concatenate(coefs), **f64),
            torch.tensor(np.concatenate(atom_xyz), **f64).reshape(-1, 3).contiguous(),
            torch.tensor(np.concatenate(atom_charge), **f64), torch.tensor(np.array(shell_atom, np.int32), **i32),
            torch.tensor(np.array(mat_base, np.int64), dtype=torch.int64, device=dev),
            torch.tensor(np.array(mat_ld, np.int32), **i32), torch.tensor(np.array(atom_begin, np.int32), **i32),
            torch.tensor(np.array(atom_end, np.int32), **i32),
        ]
        k = self._keep
        b = SqBasis()
        b.nshell, b.nbf, b.natom, b.nprim_total = len(l), max(self.mol_nbf), natom, int(self.nprim.sum())
        b.center, b.l, b.nprim, b.prim_off, b.bf_off = ptr(k[0]), ptr(k[1]), ptr(k[2]), ptr(k[3]), ptr(k[4])
        b.exps, b.coefs, b.atom_xyz, b.atom_charge, b.shell_atom = ptr(k[5]), ptr(k[6]), ptr(k[7]), ptr(k[8]), ptr(k[9])
        b.mat_base, b.mat_ld, b.mat_total = ptr(k[10]), ptr(k[11]), self.mat_total
        b.atom_begin, b.atom_end = ptr(k[12]), ptr(k[13])
        self.cbasis = b
        self.tab64 = torch.empty(_lib.SQ_BOYS_TAB64_SIZE, **f64)
        self.tab32 = torch.empty(_lib.SQ_BOYS_TAB32_SIZE, dtype=torch.float32, device=dev)
        check(self.lib.sq_boys_table(ptr(self.tab64), ptr(self.tab32), self._stream()), "sq_boys_table")
        # size groups (contiguous in the packed buffers)
        self.groups: list[SizeGroup] = []
        for mi, m in enumerate(self.mols):
            n = m.number_bf
            if not self.groups or self.groups[-1].nbf != n:
                self.groups.append(SizeGroup(n, [], self.mol_base[mi], m.number_electrons // 2))
            self.groups[-1].mols.append(mi)
        self._build_pairs()
        self._schwarz()
        self._build_slots()
        self._lists: dict = {}
        self._graphs: dict = {}

    def _stream(self) -> int:
        return _lib.stream_handle(self.device)

    # ------------------------------------------------------------- pairs
    def _build_pairs(self) -> None:
        a_all, b_all = [], []
        for mi, m in enumerate(self.mols):
            s0 = self.mol_shell0[mi]
            ns = m.number_shell
            i, j = np.triu_indices(ns)
            i += s0
            j += s0
            li, lj = self.l[i], self.l[j]
            a_all.append(np.where(li >= lj, i, j))
            b_all.append(np.where(li >= lj, j, i))
        a = np.concatenate(a_all)
        b = np.concatenate(b_all)
        la, lb = self.l[a], self.l[b]
        pc = la * (la + 1) // 2 + lb
        order = np.argsort(pc, kind="stable")
        a, b, pc = a[order], b[order], pc[order]
        self.pair_shells = np.stack([a, b], 1).astype(np.int32)
        self.pair_class = pc.astype(np.int32)
        self.pair_mol = self.shell_mol[a]
        self.pair_npa, self.pair_npb = self.nprim[a], self.nprim[b]
        self.pair_np = (self.pair_npa * self.pair_npb).astype(np.int64)
        self.npair = len(a)
        hs = np.array([herm_size(int(x), int(y)) for x, y in zip(la[order], lb[order])], dtype=np.int64)
        pp_off = np.concatenate([[0], np.cumsum(self.pair_np)]).astype(np.int64)
        herm_off = np.concatenate([[0], np.cumsum(self.pair_np * hs)[:-1]]).astype(np.int64)
        nprimpair, nherm = int(pp_off[-1]), int((self.pair_np * hs).sum())
        dev = self.device
        self.t_pair = [
            torch.tensor(self.pair_shells, dtype=torch.int32, device=dev),
            torch.tensor(pp_off.astype(np.int32), dtype=torch.int32, device=dev),
            torch.tensor(herm_off, dtype=torch.int64, device=dev),
            torch.empty(nprimpair * 8, dtype=torch.float64, device=dev),
            torch.empty(max(nherm, 1), dtype=torch.float64, device=dev),
            torch.empty(nprimpair * 8, dtype=torch.float32, device=dev) if self.fp32 else None,
            torch.empty(max(nherm, 1), dtype=torch.float32, device=dev) if self.fp32 else None,
        ]
        t = self.t_pair
        p = SqPairs()
        p.npair, p.nprimpair = self.npair, nprimpair
        p.shells, p.pp_off, p.herm_off, p.prim, p.herm = ptr(t[0]), ptr(t[1]), ptr(t[2]), ptr(t[3]), ptr(t[4])
        p.prim32, p.herm32 = ptr(t[5]), ptr(t[6])
        self.cpairs = p
        check(self.lib.sq_pair_prep(ctypes.byref(self.cbasis), ctypes.byref(p), self._stream()), "sq_pair_prep")

    def _schwarz(self) -> None:
        lists = {}
        for pc in np.unique(self.pair_class):
            idx = np.nonzero(self.pair_class == pc)[0].astype(np.int32)
            lists[screening.quartet_class(int(pc), int(pc))] = np.stack([idx, idx], 1)
        off = np.zeros(_lib.SQ_MAX_QCLASS + 1, np.int64)
        parts = []
        for c in range(_lib.SQ_MAX_QCLASS):
            arr = lists.get(c)
            off[c + 1] = off[c] + (0 if arr is None else len(arr))
            if arr is not None:
                parts.append(arr)
        ql = QuartetList(torch.tensor(np.concatenate(parts), dtype=torch.int32, device=self.device), off)
        q = torch.zeros(self.npair, dtype=torch.float64, device=self.device)
        qs = ql.cstruct()
        check(self.lib.sq_schwarz(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(qs),
                                  ptr(self.tab64), ptr(q), self._stream()), "sq_schwarz")
        self.pair_q = q.cpu().numpy()

    def _build_slots(self) -> None:
        # groups keyed by (molecule, class, primitive counts), sorted by descending q
        key_class = self.pair_mol.astype(np.int64) * 64 + self.pair_class
        groups = screening.pair_groups(key_class, self.pair_npa, self.pair_npb, self.pair_q)
        self.slot_groups = groups
        slot_pair = np.concatenate([g[1] for g in groups]).astype(np.int32)
        nslot = len(slot_pair)
        npp, pbase, pstride = (np.zeros(nslot, np.int32) for _ in range(3))
        hbase = np.zeros(nslot, np.int64)
        pos = poff = hoff = 0
        for _, members in groups:
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
        self.slot_of_pair = np.empty(nslot, np.int32)
        self.slot_of_pair[slot_pair] = np.arange(nslot, dtype=np.int32)
        # bra sub-slots for splitting heavy quartets (as in IntegralEngine)
        la_s = self.l[self.pair_shells[slot_pair, 0]]
        lb_s = self.l[self.pair_shells[slot_pair, 1]]
        E_s = np.array([herm_size(int(a), int(b)) for a, b in zip(la_s, lb_s)], dtype=np.int64)
        pc_s = self.pair_class[slot_pair]
        w_s = np.array([CLASS_WEIGHT[screening.quartet_class(int(c), int(c))] for c in pc_s], dtype=np.float64)
        qzero = np.zeros(int(npp.sum()) + 1)
        off = np.concatenate([[0], np.cumsum(npp)[:-1]]).astype(np.int64)
        self.sub_first, subs = screening.sub_slot_table(npp, pbase, pstride, hbase, E_s, w_s, qzero, off,
                                                        int(npp.max()), SPLIT_TARGET)
        self.nslot_base = nslot
        slot_pair = np.concatenate([slot_pair, slot_pair[subs["parent"]]]).astype(np.int32)
        npp = np.concatenate([npp, subs["npp"]]).astype(np.int32)
        pbase = np.concatenate([pbase, subs["pbase"]]).astype(np.int32)
        pstride = np.concatenate([pstride, subs["pstride"]]).astype(np.int32)
        hbase = np.concatenate([hbase, subs["hbase"]]).astype(np.int64)
        sub = np.concatenate([np.zeros(nslot, np.int64), subs["code"]]).astype(np.int32)
        self.slot_pair = slot_pair
        self.slot_npp = npp
        dev = self.device
        i32 = dict(dtype=torch.int32, device=dev)
        self.t_slot = [
            torch.tensor(slot_pair, **i32), torch.tensor(npp, **i32), torch.tensor(pbase, **i32),
            torch.tensor(pstride, **i32), torch.tensor(hbase, dtype=torch.int64, device=dev),
            torch.empty(5 * poff, dtype=torch.float64, device=dev), torch.empty(max(hoff, 1), dtype=torch.float64, device=dev),
            torch.empty(5 * poff, dtype=torch.float32, device=dev) if self.fp32 else None,
            torch.empty(max(hoff, 1), dtype=torch.float32, device=dev) if self.fp32 else None,
            torch.tensor(sub, **i32),
            torch.empty(8 * len(slot_pair), **i32),  # descriptors
            torch.empty(len(slot_pair), dtype=torch.int64, device=dev),  # matrix block offsets
            torch.empty(max(8 * poff, 1), dtype=torch.float32, device=dev) if self.fp32 else None,
            # double-float (hi, lo) copies for the df64 J/K kernels
            torch.empty(max(10 * poff, 2), dtype=torch.float32, device=dev) if self.fp32 else None,
            torch.empty(max(2 * hoff, 2), dtype=torch.float32, device=dev) if self.fp32 else None,
        ]
        t = self.t_slot
        s = SqSlots()
        s.nslot, s.npp_total, s.nherm_total = len(slot_pair), poff, hoff
        s.pair, s.npp, s.pbase, s.pstride, s.hbase = ptr(t[0]), ptr(t[1]), ptr(t[2]), ptr(t[3]), ptr(t[4])
        s.prim, s.herm, s.prim32, s.herm32 = ptr(t[5]), ptr(t[6]), ptr(t[7]), ptr(t[8])
        s.sub = ptr(t[9])
        s.desc, s.mbase, s.prim32v = ptr(t[10]), ptr(t[11]), ptr(t[12])
        s.primdf, s.hermdf = ptr(t[13]), ptr(t[14])
        self.slots = s
        fill = SqSlots.from_buffer_copy(s)
        fill.nslot = nslot  # the parents' data only: sub-slots point into it
        check(self.lib.sq_slots_fill(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(fill),
                                     self._stream()), "sq_slots_fill")
        check(self.lib.sq_slots_describe(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(s),
                                         self._stream()), "sq_slots_describe")

    # ---------------------------------------------------------- quartets
    def quartets(self, threshold: float, fp32_threshold: float | None = None):
        """Screened unique quartets of every molecule (slot ids), one segment per class,
        tasks of all molecules merged heaviest first."""
        mask_now = int(self.lib.sq_get_option(_lib.SQ_OPT_FP64_UNROLLED_HIGH))
        key = (threshold, fp32_threshold, mask_now)
        if key in self._lists:
            return self._lists[key]
        nl = 1 if fp32_threshold is None else 2
        # FP64 classes 12-18 split only while all of them run on per-thread kernels
        mask = int(self.lib.sq_get_option(_lib.SQ_OPT_FP64_UNROLLED_HIGH))
        hi = 18 if all((mask >> c) & 1 for c in range(12, 19)) else 11
        split_set = frozenset(range(hi + 1)) | F_PER_THREAD
        merged = [{c: [] for c in range(screening.NQCLASS)} for _ in range(nl)]
        for mi in range(self.nmol):
            sel = np.nonzero(self.pair_mol == mi)[0]
            lists, ket = screening.build_tasks(self.pair_class[sel], self.pair_npa[sel], self.pair_npb[sel],
                                               self.pair_q[sel], threshold, fp32_threshold)
            # a molecule's groups are consecutive slots in the same order, so the
            # kets of one task are consecutive slots starting at slot_of_pair[ket[start]]
            ket_slots = self.slot_of_pair[sel[ket]]
            for li in range(nl):
                for c in range(screening.NQCLASS):
                    for bra, kst, cnt in lists[li][c]:
                        cost = int(self.pair_np[sel[bra[0]]] * self.pair_np[sel[ket[kst[0]]]])
                        bslots = self.slot_of_pair[sel[bra]]
                        # heavy quartets of the per-thread classes: bra sub-slot chunks
                        S = 1
                        if c in split_set:
                            while cost * CLASS_WEIGHT[c] > SPLIT_TARGET * S and (2 * S) in self.sub_first and \
                                    self.sub_first[2 * S][bslots[0]] >= 0:
                                S *= 2
                        if S == 1:
                            merged[li][c].append((cost, bslots, ket_slots[kst], cnt))
                        else:
                            first = self.sub_first[S][bslots]
                            for k in range(S):
                                merged[li][c].append((cost / S, (first + k).astype(np.int32), ket_slots[kst], cnt))
        out = []
        for li in range(nl):
            tasks = {c: [(b, k, n) for _, b, k, n in sorted(merged[li][c], key=lambda t: -t[0])]
                     for c in range(screening.NQCLASS)}
            bra, kst, cnt, toff, off = screening.flatten_tasks(tasks)
            nq = int(off[-1])
            pairs = torch.empty((max(nq, 1), 2), dtype=torch.int32, device=self.device)
            if nq:
                dev = self.device
                tb = torch.tensor(bra, dtype=torch.int32, device=dev)
                tk = torch.tensor(kst, dtype=torch.int32, device=dev)
                tc = torch.tensor(cnt.astype(np.int32), dtype=torch.int32, device=dev)
                to = torch.tensor(toff, dtype=torch.int64, device=dev)
                check(self.lib.sq_quartets_expand(len(bra), ptr(tb), ptr(tk), ptr(tc), ptr(to), None, ptr(pairs),
                                                  nq, self._stream()), "sq_quartets_expand")
                torch.cuda.current_stream(self.device).synchronize()
            out.append(QuartetList(pairs, off))
        res = out[0] if nl == 1 else (out[0], out[1])
        self._lists[key] = res
        return res

    # ---------------------------------------------------------- matrices
    def one_electron(self):
        S = torch.zeros(self.mat_total, dtype=torch.float64, device=self.device)
        T = torch.zeros_like(S)
        V = torch.zeros_like(S)
        check(self.lib.sq_one_electron(ctypes.byref(self.cbasis), ptr(self.tab64), ptr(S), ptr(T), ptr(V),
                                       self._stream()), "sq_one_electron")
        return S, T, V

    def view(self, flat: torch.Tensor, g: SizeGroup) -> torch.Tensor:
        n = g.nbf
        return flat[g.offset:g.offset + len(g.mols) * n * n].view(len(g.mols), n, n)

    def jk_accumulate(self, D: torch.Tensor, Jacc: torch.Tensor, Kacc: torch.Tensor, D32: torch.Tensor,
                      lists, precs, prim_tau: float = 0.0) -> None:
        """sq_jk for each (list, precision); "df64" / "df64_prim" run sq_jk_df (double-float,
        the latter with the primitive split at prim_tau)."""
        Jacc.zero_()
        Kacc.zero_()
        work = [(ql, prec) for ql, prec in zip(lists, precs) if ql.nquartet]
        main = torch.cuda.current_stream(self.device)
        # lists after the first run concurrently from side streams (all only add into Jacc/Kacc);
        # the fork/join is stream-ordered, so it also holds inside a CUDA-graph capture
        if not hasattr(self, "_sides"):
            self._sides = []
        while len(self._sides) < len(work) - 1:
            self._sides.append(torch.cuda.Stream(self.device))
        side = self._sides[: max(len(work) - 1, 0)]
        for s in side:
            s.wait_stream(main)
        for i, (ql, prec) in enumerate(work):
            st = main if i == 0 else side[i - 1]
            qs = ql.cstruct()
            if prec in ("df64", "df64_prim"):
                if getattr(self, "_ddf", None) is None:  # first made in a warm-up call, before any capture
                    self._ddf = torch.empty(2 * self.mat_total, dtype=torch.float32, device=self.device)
                check(self.lib.sq_jk_df(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                        ctypes.byref(qs), ptr(self.tab64), ptr(self.tab32), ptr(D), ptr(self._ddf),
                                        ptr(Jacc), ptr(Kacc), float(prim_tau) if prec == "df64_prim" else 0.0,
                                        st.cuda_stream), "sq_jk_df")
                continue
            check(self.lib.sq_jk(ctypes.byref(self.cbasis), ctypes.byref(self.cpairs), ctypes.byref(self.slots),
                                 ctypes.byref(qs), ptr(self.tab64), ptr(self.tab32), ptr(D), ptr(D32), ptr(Jacc),
                                 ptr(Kacc), _lib.PRECISIONS[prec], st.cuda_stream), "sq_jk")
        for s in side:
            main.wait_stream(s)


_EIGH_MAX_N = 128
_eigh_desc: dict = {}


def batched_eigh(M: torch.Tensor, tol: float = 1e-15, max_sweeps: int = 40):
    """Eigenvalues (ascending) and eigenvectors (columns) of a [B, n, n] FP64 symmetric stack.

    Replaces torch/numpy eigh in the SCF step (hartreefock_in_memory.py:63-66)
    with sq_batched_eigh, one CTA per matrix, for n <= 128.  Larger blocks use
    torch.linalg.eigh (cuSOLVER).
    """
    B, n, _ = M.shape
    if n > _EIGH_MAX_N:
        return torch.linalg.eigh(M)
    M = M.contiguous()
    key = (B, n, M.device)
    if key not in _eigh_desc:
        dev = M.device
        _eigh_desc[key] = (torch.arange(B, dtype=torch.int64, device=dev) * (n * n),
                           torch.full((B,), n, dtype=torch.int32, device=dev),
                           torch.arange(B, dtype=torch.int64, device=dev) * n)
    offs, dims, woffs = _eigh_desc[key]
    W = torch.empty((B, n), dtype=torch.float64, device=M.device)
    V = torch.empty_like(M)
    check(_lib.lib().sq_batched_eigh(B, ptr(offs), ptr(dims), n, ptr(M), ptr(W), ptr(V), ptr(woffs), tol,
                                     max_sweeps, None, _lib.stream_handle()), "sq_batched_eigh")
    return W, V


class _BatchDIIS:
    """Pulay DIIS (diis.py:4-66 semantics) for a [count, n, n] group, entirely on the device.

    The six stored (F, error) pairs live in a ring buffer whose write position
    and fill count are device tensors, and the bordered system always has the
    full 7 x 7 shape: a slot not yet written gets a unit diagonal and a zero
    border, so its coefficient is 0.  The coefficients solve the same system
    as the reference's (the order of the stored vectors does not change the
    solution), one vector gives c = 1 (F unchanged, as the reference's first
    call), and nothing depends on host state, so a whole SCF iteration can be
    captured in a CUDA graph and replayed.  Blocks of 2 functions skip DIIS,
    as the reference does.
    """

    def __init__(self, count: int, n: int, device, nsave: int = 6):
        self.n = n
        self.nsave = nsave
        self.F = torch.zeros((nsave, count, n, n), dtype=torch.float64, device=device)
        self.E = torch.zeros_like(self.F)
        self.head = torch.zeros(1, dtype=torch.int64, device=device)
        self.k = torch.zeros(1, dtype=torch.int64, device=device)
        self.slots = torch.arange(nsave, device=device)
        self.last_error = torch.zeros(count, dtype=torch.float64, device=device)

    def reset(self) -> None:
        self.head.zero_()
        self.k.zero_()

    def extrapolate(self, F, D, S):
        if self.n == 2:
            return F
        err = F @ D @ S - S @ D @ F
        self.last_error.copy_(err.abs().amax(dim=(1, 2)))
        self.F.index_copy_(0, self.head, F[None])
        self.E.index_copy_(0, self.head, err[None])
        self.head.copy_(torch.remainder(self.head + 1, self.nsave))
        self.k.copy_(torch.clamp(self.k + 1, max=self.nsave))
        valid = self.slots < self.k  # slots are written 0, 1, 2, ... then reused
        m = self.nsave
        Bm = torch.einsum("icpq,jcqp->cij", self.E, self.E)
        pair = valid[:, None] & valid[None, :]
        Bm = torch.where(pair, Bm, torch.zeros_like(Bm)) + torch.diag_embed((~valid).to(Bm.dtype)).expand_as(Bm)
        count = F.shape[0]
        border = torch.where(valid, -1.0, 0.0).to(torch.float64)
        B = torch.zeros((count, m + 1, m + 1), dtype=torch.float64, device=F.device)
        B[:, :m, :m] = Bm
        B[:, m, :m] = border
        B[:, :m, m] = border
        b0 = torch.zeros((count, m + 1), dtype=torch.float64, device=F.device)
        b0[:, m] = -1
        # solve_ex: no singularity check, so no host synchronisation
        c = torch.linalg.solve_ex(B, b0)[0]
        return torch.einsum("ci,icpq->cpq", c[:, :m], self.F)


class BatchSCF:
    """Restricted HF of every molecule of a BatchEngine (hartreefock_in_memory.py:7-94 semantics,
    batched per size group).  precision: "fp64" or "mixed" (FP32 quartets below fp32_threshold
    until every molecule's DIIS error is below fp64_tail_diis_error, then FP64), and the
    same two with double-float arithmetic on the FP32 pipe in place of FP64: "df64" and
    "mixed_df" (quartet-level, as "mixed": the batch carries no primitive Schwarz factors).

    With ``use_graphs`` (default) a whole SCF iteration -- the Fock build, DIIS,
    the orthogonalised eigensolve, the new density, the energies and the
    convergence test -- is captured once per precision in a CUDA graph and
    replayed.  Convergence is a device flag: once every molecule meets the
    thresholds the state stops changing, so the host reads the flag only every
    ``check_every`` iterations and the results equal stopping at the converged
    iteration.  In mixed precision the host reads the FP64-switch test every
    iteration until the switch.
    """

    def __init__(self, be: BatchEngine, precision: str = "fp64", threshold: float = 1e-12,
                 fp32_threshold: float = 1e-4, fp64_tail_diis_error: float = 1e-5, use_graphs: bool = True,
                 check_every: int = 4):
        self.be = be
        self.precision = precision
        self.threshold = threshold
        self.fp32_threshold = fp32_threshold
        self.tail = fp64_tail_diis_error
        self.use_graphs = use_graphs
        self.check_every = max(1, int(check_every))
        dev = be.device
        tot = be.mat_total
        self.S, T, V = be.one_electron()
        self.H = T + V
        self.D = torch.zeros(tot, dtype=torch.float64, device=dev)
        self.F = torch.zeros_like(self.D)
        self.Jacc = torch.zeros_like(self.D)
        self.Kacc = torch.zeros_like(self.D)
        self.D32 = torch.zeros(tot, dtype=torch.float32, device=dev)
        if precision not in ("fp64", "mixed", "df64", "mixed_df"):
            raise ValueError(f"unknown batch precision {precision!r}")
        df = precision in ("df64", "mixed_df")
        # the accurate phase ("fp64") and the mixed phase, in FP64 or double-float
        self.lists = {"fp64": ([be.quartets(threshold)], ["df64" if df else "fp64"])}
        if precision in ("mixed", "mixed_df"):
            q64, q32 = be.quartets(threshold, fp32_threshold)
            self.lists["mixed"] = ([q64, q32], ["df64" if df else "fp64", "fp32"])
        self.graphs: dict = {}
        self.builds: list[str] = []
        self.tuning: dict = {}
        self.host_syncs = 0

    def autotune(self, threads=None, waves=None) -> dict:
        """Pick each quartet class's launch shape (threads per block, grid cap) for this
        batch's lists with the project's autotuner, install it, and return the table
        {(class, precision): (threads, blocks, ms)}.  Call before the first SCF so the
        captured graphs use the tuned shapes; ``autotune.reset()`` restores the defaults."""
        from . import autotune

        kw = {}
        if threads is not None:
            kw["threads"] = threads
        if waves is not None:
            kw["waves"] = waves
        be = self.be

        def run_class(sub, prec):
            be.jk_accumulate(self.D, self.Jacc, self.Kacc, self.D32, [sub], [prec])

        table = {}
        for mode in self.lists:
            # double-float launches have no tunable shape
            pairs = [(ql, p) for ql, p in zip(*self.lists[mode]) if not p.startswith("df")]
            if pairs:
                table.update(autotune.tune(run_class, [q for q, _ in pairs], [p for _, p in pairs], **kw))
        self.tuning = table
        self.graphs = {}  # re-capture with the tuned shapes
        self.fock_graphs = {}
        return table

    def _fock_into_F(self, mode: str) -> None:
        be = self.be
        lists, precs = self.lists[mode]
        be.jk_accumulate(self.D, self.Jacc, self.Kacc, self.D32, lists, precs, self.fp32_threshold)
        for g in be.groups:
            J = be.view(self.Jacc, g)
            K = be.view(self.Kacc, g)
            F = be.view(self.F, g)
            F.copy_(be.view(self.H, g) + 0.5 * (J + J.transpose(1, 2)) - 0.25 * (K + K.transpose(1, 2)))

    def fock(self, mode: str) -> None:
        """F <- H + J(D) - K(D)/2 for the whole batch alone (replayed from its own CUDA graph);
        the SCF iterations capture the build inside their iteration graphs instead."""
        if not self.use_graphs:
            self._fock_into_F(mode)
            return
        if not hasattr(self, "fock_graphs"):
            self.fock_graphs = {}
        if mode not in self.fock_graphs:
            # warm up on a side stream, then capture the build once
            s = torch.cuda.Stream(self.be.device)
            s.wait_stream(torch.cuda.current_stream(self.be.device))
            with torch.cuda.stream(s):
                self._fock_into_F(mode)
            torch.cuda.current_stream(self.be.device).wait_stream(s)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._fock_into_F(mode)
            self.fock_graphs[mode] = g
        self.fock_graphs[mode].replay()

    def _eigh_all(self, A_flat: torch.Tensor):
        """Eigenvectors of every molecule's block of a packed buffer in one launch (sq_batched_eigh).

        The matrices are handed to the kernel largest first: its shared memory
        is sized by the largest one, so few CTAs fit per SM, and the large
        matrices should take the first wave with the small ones behind them."""
        be = self.be
        if not hasattr(self, "_eig_desc"):
            dev = be.device
            nbf = np.array(be.mol_nbf, dtype=np.int64)
            base = np.array(be.mol_base, dtype=np.int64)
            woff = np.concatenate([[0], np.cumsum(nbf)[:-1]]).astype(np.int64)
            order = np.argsort(-nbf, kind="stable")
            self._eig_desc = (torch.tensor(base[order], device=dev),
                              torch.tensor(nbf[order].astype(np.int32), device=dev),
                              torch.tensor(woff[order], device=dev), int(nbf.sum()), int(nbf.max()))
        offs, dims, woffs, ntot, nmax = self._eig_desc
        if nmax > _EIGH_MAX_N:
            out = torch.empty_like(A_flat)
            for g in be.groups:
                be.view(out, g).copy_(torch.linalg.eigh(be.view(A_flat, g))[1])
            return out
        W = torch.empty(ntot, dtype=torch.float64, device=be.device)
        V = torch.empty_like(A_flat)
        check(_lib.lib().sq_batched_eigh(be.nmol, ptr(offs), ptr(dims), nmax, ptr(A_flat), ptr(W), ptr(V),
                                         ptr(woffs), 1e-14, 40, None, _lib.stream_handle()), "sq_batched_eigh")
        return V

    def _setup_state(self) -> None:
        """Core-Hamiltonian guess and the per-group state (hartreefock_in_memory.py:30-42).

        A second run of the same object writes into the first run's tensors,
        so the iteration graphs captured then stay valid and are replayed."""
        be = self.be
        first = not hasattr(self, "X")
        if first:
            self.X, self.U, self.E, self.diis, self.nocc = [], [], [], [], []
        for gi, g in enumerate(be.groups):
            S = be.view(self.S, g)
            H = be.view(self.H, g)
            lam, L = batched_eigh(S)
            Xg = L @ torch.diag_embed(lam ** (-0.5)) @ L.transpose(1, 2)
            _, C0p = batched_eigh(Xg.transpose(1, 2) @ H @ Xg.transpose(1, 2))
            C0 = Xg @ C0p
            Co = C0[:, :, : g.nocc]
            be.view(self.D, g).copy_(2 * Co @ Co.transpose(1, 2))
            E0 = torch.sum(be.view(self.D, g) * H, dim=(1, 2))
            if first:
                self.E.append(E0)
                self.X.append(Xg)
                self.U.append(C0p.contiguous())
                self.diis.append(_BatchDIIS(len(g.mols), g.nbf, be.device))
                self.nocc.append(g.nocc)
            else:
                self.E[gi].copy_(E0)
                self.X[gi].copy_(Xg)
                self.U[gi].copy_(C0p)
                self.diis[gi].reset()
        if first:
            dev = be.device
            self.Fp = torch.zeros_like(self.F)  # packed orthogonalised Fock matrices
            self.done = torch.zeros(1, dtype=torch.bool, device=dev)
            self.tail_ok = torch.zeros(1, dtype=torch.bool, device=dev)
            self.iters = torch.zeros(1, dtype=torch.int64, device=dev)
        else:
            self.done.zero_()
            self.tail_ok.zero_()
            self.iters.zero_()

    def _iterate(self, mode: str, dE_threshold: float, rmsd_threshold: float) -> None:
        """One SCF iteration of every molecule, device work only (graph-capturable)."""
        be = self.be
        self._fock_into_F(mode)
        Fx = []
        for gi, g in enumerate(be.groups):
            F = self.diis[gi].extrapolate(be.view(self.F, g).clone(), be.view(self.D, g).clone(),
                                          be.view(self.S, g))
            Fx.append(F)
            # in the previous iteration's orbital basis U the Fock matrix is nearly
            # diagonal, so the Jacobi sweeps converge in a few sweeps
            XU = self.X[gi] @ self.U[gi]
            be.view(self.Fp, g).copy_(XU.transpose(1, 2) @ F @ XU)
        V = self._eigh_all(self.Fp)  # one eigensolver launch for all molecules
        live = ~self.done
        conv = torch.ones(1, dtype=torch.bool, device=be.device)
        tail = torch.ones(1, dtype=torch.bool, device=be.device)
        for gi, g in enumerate(be.groups):
            Un = self.U[gi] @ be.view(V, g)
            C = self.X[gi] @ Un
            Co = C[:, :, : self.nocc[gi]]
            Dn = 2 * Co @ Co.transpose(1, 2)
            Dv = be.view(self.D, g)
            En = 0.5 * torch.sum(Dn * (be.view(self.H, g) + Fx[gi]), dim=(1, 2))
            dE = (En - self.E[gi]).abs().amax()
            rmsd = torch.sqrt(torch.sum((Dn - Dv) ** 2, dim=(1, 2))).amax()
            conv = conv & (dE < dE_threshold) & (rmsd < rmsd_threshold)
            tail = tail & (self.diis[gi].last_error.amax() < self.tail)
            # a converged batch keeps its state: later replays change nothing
            self.U[gi].copy_(torch.where(live, Un, self.U[gi]))
            Dv.copy_(torch.where(live, Dn, Dv))
            self.E[gi].copy_(torch.where(live, En, self.E[gi]))
        self.iters.add_(live.to(torch.int64))
        self.tail_ok.copy_(tail)
        if mode == "fp64":  # the mixed phase never stops: it ends with the switch to FP64
            self.done.copy_(self.done | conv)

    def _step(self, mode: str, dE_threshold: float, rmsd_threshold: float) -> None:
        self.builds.append(mode)
        if not self.use_graphs:
            self._iterate(mode, dE_threshold, rmsd_threshold)
            return
        if mode not in self.graphs:
            # the first iteration in this precision runs on a side stream (warming up
            # every library handle), then the iteration is captured once
            s = torch.cuda.Stream(self.be.device)
            s.wait_stream(torch.cuda.current_stream(self.be.device))
            with torch.cuda.stream(s):
                self._iterate(mode, dE_threshold, rmsd_threshold)
            torch.cuda.current_stream(self.be.device).wait_stream(s)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._iterate(mode, dE_threshold, rmsd_threshold)
            self.graphs[mode] = g
            return
        self.graphs[mode].replay()

    def run(self, dE_threshold: float = 1e-9, rmsd_threshold: float = 1e-9, max_iter: int = 100):
        be = self.be
        self._setup_state()
        mode = "fp64" if self.precision in ("fp64", "df64") else "mixed"
        self.host_syncs = 0
        for it in range(1, max_iter + 1):
            self._step(mode, dE_threshold, rmsd_threshold)
            if mode == "mixed":
                self.host_syncs += 1
                if bool(self.tail_ok.item()):
                    mode = "fp64"
                    for d in self.diis:
                        d.reset()
            elif it % self.check_every == 0 or it == max_iter:
                self.host_syncs += 1
                if bool(self.done.item()):
                    break
        self.iterations = int(self.iters.item())
        if not bool(self.done.item()):
            import warnings

            warnings.warn(f"batched RHF did not converge in {max_iter} iterations", stacklevel=2)
        E = self.E
        # energies back in the caller's molecule order
        Eb = torch.cat(E).cpu().numpy()
        out = np.empty(be.nmol)
        out[np.array(be.order)] = Eb
        return out
