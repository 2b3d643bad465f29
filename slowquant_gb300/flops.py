"""Algorithmic work model for the MD ERI + J/K build (roofline numerator).

Per surviving primitive quartet of class (la lb | lc ld), Cartesian MD:
  F_boys = 30 + 3L
  F_R    = 3 * sum_{m=0}^{L} H(m) - 3           (Hermite Coulomb recurrences)
  F_ket  = 2 * H(L_ab) * K_cd                     (ket Hermite contraction)
  F_bra  = 2 * K_ab * C(lc) C(ld)                 (bra Hermite contraction)
  F_acc  = 2 * C(la) C(lb) C(lc) C(ld)            (primitive accumulation)
with H(n) = (n+1)(n+2)(n+3)/6, C(l) = (l+1)(l+2)/2 and K_xy the number of
Hermite terms over all Cartesian pairs of the pair.  Per contracted quartet
the J/K digestion adds 12 C(la) C(lb) C(lc) C(ld).  Pair data are amortised
and not counted.
"""

from __future__ import annotations

from .molecule import CARTESIAN


def H(n: int) -> int:
    return (n + 1) * (n + 2) * (n + 3) // 6


def C(l: int) -> int:
    return (l + 1) * (l + 2) // 2


def K(la: int, lb: int) -> int:
    ca, cb = CARTESIAN["spdf"[la]], CARTESIAN["spdf"[lb]]
    return sum((a[0] + b[0] + 1) * (a[1] + b[1] + 1) * (a[2] + b[2] + 1) for a in ca for b in cb)


def flops_per_primitive_quartet(la: int, lb: int, lc: int, ld: int) -> int:
    lab, lcd = la + lb, lc + ld
    L = lab + lcd
    f_boys = 30 + 3 * L
    f_r = 3 * sum(H(m) for m in range(L + 1)) - 3
    f_ket = 2 * H(lab) * K(lc, ld)
    f_bra = 2 * K(la, lb) * C(lc) * C(ld)
    f_acc = 2 * C(la) * C(lb) * C(lc) * C(ld)
    return f_boys + f_r + f_ket + f_bra + f_acc


def flops_per_contracted_quartet_jk(la: int, lb: int, lc: int, ld: int) -> int:
    return 12 * C(la) * C(lb) * C(lc) * C(ld)


PAIR_CLASSES = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2), (3, 0), (3, 1), (3, 2), (3, 3)]


def quartet_class_l(qc: int):
    cb = 0
    while (cb + 1) * (cb + 2) // 2 <= qc:
        cb += 1
    ck = qc - cb * (cb + 1) // 2
    return (*PAIR_CLASSES[cb], *PAIR_CLASSES[ck])
