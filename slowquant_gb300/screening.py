"""Schwarz screening and shell-quartet work-list construction (host side).

Replaces the shell-quartet loops of electron_repulsion_integral_driver
(slowquant/molecularintegrals/electronrepulsion.py:32-49): the reference visits
i <= j, k <= l with "ij >= kl" and skips a quartet when
cs[i,j] * cs[k,l] < threshold.  Here the unique quartets are enumerated as
(bra pair, ket pair) combinations of pair *groups*:

* a group is the set of shell pairs with the same pair class (la, lb) and the
  same primitive counts, sorted by descending Schwarz factor q;
* bra group g1 meets ket groups g2 <= g1 whose class is not above g1's class
  (so bra class >= ket class), and inside one group only ket position <= bra
  position, which makes every unordered pair of pairs appear once;
* for a bra pair with factor x the surviving kets of a group are the prefix
  with x * q_ket >= threshold (the same product test as the reference), and
  with a second threshold that prefix splits into a large-bound (FP64) part
  and a small-bound (FP32) part;
* inside a quartet class, group pairs are emitted heaviest first (primitive
  quartets per contracted quartet), so the device's block scheduler balances
  the load across SMs.

``build_tasks`` returns per quartet class the (bra pair, ket start, count)
tasks; the device kernel sq_quartets_expand turns them into the flat list.
"""

from __future__ import annotations

import numpy as np

NQCLASS = 55  # quartet classes of s, p, d and f shells (10 pair classes)


def quartet_class(cb: int, ck: int) -> int:
    return cb * (cb + 1) // 2 + ck


def prefix_counts(x: np.ndarray, qk: np.ndarray, thr: float) -> np.ndarray:
    """For each bra factor x: number of leading ket factors (descending qk) with x*qk >= thr."""
    n = len(qk)
    if n == 0 or len(x) == 0:
        return np.zeros(len(x), dtype=np.int64)
    with np.errstate(divide="ignore", over="ignore"):
        lim = np.where(x > 0, thr / np.where(x > 0, x, 1.0), np.inf)
    cnt = np.searchsorted(-qk, -lim, side="right").astype(np.int64)
    # exact product test at the boundary, the comparison the reference uses
    # (the division above can round either way by one position)
    for _ in range(4):
        last = qk[np.maximum(cnt - 1, 0)]
        dec = (cnt > 0) & (x * last < thr)
        nxt = qk[np.minimum(cnt, n - 1)]
        inc = (cnt < n) & (x * nxt >= thr)
        if not (dec.any() or inc.any()):
            break
        cnt = cnt - dec + inc
    return cnt


def pair_groups(pair_class: np.ndarray, npa: np.ndarray, npb: np.ndarray, q: np.ndarray):
    """[(class, member pair indices sorted by descending q)], ordered by (class, npa, npb).

    One stable sort by (class, npa, npb, -q), then a split at the key changes
    (O(n log n); many thousands of groups occur in a batch of molecules).
    """
    pair_class = np.asarray(pair_class)
    npa = np.asarray(npa)
    npb = np.asarray(npb)
    q = np.asarray(q, dtype=np.float64)
    n = len(pair_class)
    if n == 0:
        return []
    order = np.lexsort((np.arange(n), -q, npb, npa, pair_class))
    kc, ka, kb = pair_class[order], npa[order], npb[order]
    change = np.nonzero((kc[1:] != kc[:-1]) | (ka[1:] != ka[:-1]) | (kb[1:] != kb[:-1]))[0] + 1
    bounds = np.concatenate([[0], change, [n]])
    return [(int(kc[bounds[i]]), order[bounds[i]:bounds[i + 1]].astype(np.int32)) for i in range(len(bounds) - 1)]


def build_tasks(pair_class, npa, npb, q, threshold: float, fp32_threshold: float | None = None):
    """Tasks per list and quartet class.

    Returns (lists, ket_list): lists[li][qc] = list of (bra ids, ket starts,
    counts) arrays, li = 0 for the FP64 (or only) list, 1 for the FP32 list;
    ket_list is the concatenation of the groups' sorted members.
    """
    q = np.asarray(q, dtype=np.float64)
    groups = pair_groups(np.asarray(pair_class), np.asarray(npa), np.asarray(npb), q)
    ket_list = np.concatenate([g[1] for g in groups]).astype(np.int32) if groups else np.zeros(0, np.int32)
    gstart = np.concatenate([[0], np.cumsum([len(g[1]) for g in groups])]).astype(np.int64)
    nlists = 1 if fp32_threshold is None else 2
    lists = [{c: [] for c in range(NQCLASS)} for _ in range(nlists)]
    npp = np.asarray(npa, dtype=np.int64) * np.asarray(npb, dtype=np.int64)
    pending = [{c: [] for c in range(NQCLASS)} for _ in range(nlists)]
    for g1, (c1, m1) in enumerate(groups):
        x = q[m1]
        for g2 in range(g1 + 1):
            c2, m2 = groups[g2]
            if c2 > c1:
                continue
            qk = q[m2]
            cnt = prefix_counts(x, qk, threshold)
            if g2 == g1:
                cnt = np.minimum(cnt, np.arange(1, len(m1) + 1))
            if fp32_threshold is None:
                bounds = [(np.zeros_like(cnt), cnt)]
            else:
                c64 = np.minimum(prefix_counts(x, qk, fp32_threshold), cnt)
                bounds = [(np.zeros_like(cnt), c64), (c64, cnt)]
            qc = quartet_class(c1, c2)
            # primitive quartets per contracted quartet of this group pair
            cost = int(npp[m1[0]] * npp[m2[0]])
            for li, (lo, hi) in enumerate(bounds):
                n = hi - lo
                keep = n > 0
                if keep.any():
                    pending[li][qc].append((cost, g1, g2, (m1[keep], gstart[g2] + lo[keep], n[keep])))
    # Heaviest group pairs first inside each class: every quartet of a group pair
    # costs the same, so this is longest-processing-time-first order for the
    # hardware block scheduler (light blocks fill the tail).
    for li in range(nlists):
        for qc in range(NQCLASS):
            for _, _, _, task in sorted(pending[li][qc], key=lambda t: (-t[0], t[1], t[2])):
                lists[li][qc].append(task)
    return lists, ket_list


def flatten_tasks(tasks: dict):
    """Concatenate one list's tasks: (bra, ket_start, count, task offsets, class offsets)."""
    bra, kst, cnt = [], [], []
    off = np.zeros(NQCLASS + 1, dtype=np.int64)
    for c in range(NQCLASS):
        tot = 0
        for m, s, n in tasks[c]:
            bra.append(m)
            kst.append(s)
            cnt.append(n)
            tot += int(n.sum())
        off[c + 1] = off[c] + tot
    if bra:
        bra = np.concatenate(bra).astype(np.int32)
        kst = np.concatenate(kst).astype(np.int32)
        cnt = np.concatenate(cnt).astype(np.int64)
    else:
        bra = np.zeros(0, np.int32)
        kst = np.zeros(0, np.int32)
        cnt = np.zeros(0, np.int64)
    toff = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int64) if len(cnt) else np.zeros(0, np.int64)
    return bra, kst, cnt, toff, off


def expand_host(bra, kst, cnt, ket_list) -> np.ndarray:
    """Host restatement of sq_quartets_expand (for tests and small checks)."""
    if len(bra) == 0:
        return np.zeros((0, 2), dtype=np.int32)
    rep_bra = np.repeat(bra, cnt)
    starts = np.repeat(kst.astype(np.int64), cnt)
    first = np.repeat(np.concatenate([[0], np.cumsum(cnt)[:-1]]), cnt)
    k = np.arange(int(cnt.sum())) - first
    return np.stack([rep_bra, ket_list[starts + k]], axis=1).astype(np.int32)


def ket_chunk_entries(seg: np.ndarray, sub_first: dict, nslot: int, want: int) -> np.ndarray:
    """Quartet entries (bra, ket) with each whole ket slot cut into sub-slot chunks.

    For every entry whose ket is a whole slot (id < nslot), S' is the largest
    chunk count S <= want with sub_first[S][ket] >= 0; the entry becomes S'
    entries (bra, sub_first[S'][ket] + j), j < S' (chunk j of S' covers the
    ket's primitive pairs [j n / S', (j+1) n / S')).  Entries without chunks
    (sub-slot kets, or slots with no chunk table up to want) are kept.  Order:
    each entry's chunks in place of the entry."""
    seg = np.asarray(seg, dtype=np.int64).reshape(-1, 2)
    ket = seg[:, 1]
    whole = ket < nslot
    S = np.ones(len(seg), np.int64)
    first = np.full(len(seg), -1, np.int64)
    for s in sorted(sub_first):
        if s > want:
            break
        f = np.full(len(seg), -1, np.int64)
        f[whole] = np.asarray(sub_first[s])[ket[whole]]
        ok = f >= 0
        S[ok] = s
        first[ok] = f[ok]
    rep = np.repeat(np.arange(len(seg)), S)
    j = np.arange(len(rep)) - np.repeat(np.cumsum(S) - S, S)
    newket = np.where(np.repeat(S, S) > 1, np.repeat(first, S) + j, np.repeat(ket, S))
    return np.stack([seg[rep, 0], newket], axis=1).astype(np.int32)


def sub_slot_table(npp, pbase, pstride, hbase, herm_per_prim, weight, qcum, prim_off, max_np: int,
                   split_target: float, min_chunk: int = 4):
    """Sub-slots: chunk k of S (a power of two) of a slot's primitive pairs.

    Sub-slot k of S covers the slot's primitive pairs [k*n//S, (k+1)*n//S)
    (n = npp of the slot) and points into the slot's data (field-major layout
    with stride pstride: primitive i at pbase + i*pstride, its Hermite block at
    hbase + i*herm_per_prim*pstride).  Chunk counts are made for the S a split
    can ask for: the slot's heaviest quartet (npp * max_np * weight) above
    split_target * S/2, or chunks of at least min_chunk primitive pairs (for
    the per-chunk precision test).  qcum is the prefix sum of the slots' primitive
    Schwarz factors in slot order (prim_off[s] = start of slot s), which gives
    each sub-slot's bound sum.

    Returns (first, table): first[S][s] = id of sub-slot 0 of S of slot s (-1:
    none; ids continue after the nslot slots), and the table's arrays (parent,
    npp, pbase, pstride, hbase, code = k << 16 | S, qsum).
    """
    npp = np.asarray(npp, dtype=np.int64)
    nslot = len(npp)
    max_np = int(max_np)
    first_of = {}
    cols = {k: [] for k in ("parent", "npp", "pbase", "pstride", "hbase", "code", "qsum")}
    nsub = 0
    S = 2
    while nslot:
        want = ((npp * max_np * weight > split_target * (S // 2)) | (npp >= min_chunk * S)) & (npp >= S)
        idx = np.nonzero(want)[0]
        if len(idx) == 0:
            break
        first = np.full(nslot, -1, np.int64)
        first[idx] = nslot + nsub + S * np.arange(len(idx))
        first_of[S] = first
        k = np.tile(np.arange(S), len(idx))
        par = np.repeat(idx, S)
        lo = (k * npp[par]) // S
        hi = ((k + 1) * npp[par]) // S
        cols["parent"].append(par)
        cols["npp"].append(hi - lo)
        cols["pbase"].append(pbase[par] + lo * pstride[par])
        cols["pstride"].append(pstride[par])
        cols["hbase"].append(hbase[par] + lo * herm_per_prim[par] * pstride[par])
        cols["code"].append((k << 16) | S)
        cols["qsum"].append(qcum[prim_off[par] + hi] - qcum[prim_off[par] + lo])
        nsub += S * len(idx)
        S *= 2
    dtypes = {"parent": np.int64, "npp": np.int32, "pbase": np.int32, "pstride": np.int32, "hbase": np.int64,
              "code": np.int64, "qsum": np.float64}
    table = {k: (np.concatenate(v).astype(dtypes[k]) if v else np.zeros(0, dtypes[k])) for k, v in cols.items()}
    return first_of, table
