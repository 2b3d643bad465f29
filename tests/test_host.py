"""Host-side logic on CPU: molecule/basis layer, screening work lists, C ABI exports."""

import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from slowquant_gb300 import molecule, screening, systems
from tests.conftest import ROOT, load_golden


def test_molecule_matches_oracle_restatement():
    geom = systems.water_cluster(3, 6.0, seed=3)
    m = molecule._Molecule(geom, 0, "angstrom")
    m._set_basis_set("cc-pvdz")
    o = O.OracleMolecule(geom, "cc-pvdz", "angstrom")
    assert m.number_bf == o.nbf == 75
    assert m.number_shell == len(o.shells) == 36
    assert m.number_electrons == o.number_electrons == 30
    assert abs(m.nuclear_repulsion - o.nuclear_repulsion) < 1e-10
    for s, t in zip(m.shells, o.shells):
        np.testing.assert_allclose(s.normalization, t[4], rtol=1e-13)
        np.testing.assert_array_equal(s.angular_moments, t[3])


def test_normalization_factorises_per_component():
    """N[bf,i] = g(alpha_i) / sqrt((2x-1)!!(2y-1)!!(2z-1)!!): the identity the kernels use."""
    m = molecule._Molecule(systems.water_monomer(), 0, "angstrom")
    m._set_basis_set("cc-pvdz")
    g = load_golden("primitives")
    np.testing.assert_allclose(np.concatenate([s.normalization.ravel() for s in m.shells]), g["ccpvdz_h2o_norms"],
                               rtol=1e-13)
    for s in m.shells:
        base = s.component_independent_coefficients()
        for b, ang in enumerate(s.angular_moments):
            df = np.prod([molecule.factorial2(2 * a - 1) for a in ang])
            np.testing.assert_allclose(base / np.sqrt(df), s.contraction_coefficients * s.normalization[b], rtol=1e-13)


def test_molecule_errors_follow_reference():
    with pytest.raises(ValueError):
        molecule._Molecule("H 0 0 0;H 0 0 1", 0, "parsec")
    with pytest.raises(ValueError):
        molecule._Molecule("H 0 0 0", 0, "bohr")
    m = molecule._Molecule("Xe 0 0 0;", 0, "bohr")
    with pytest.raises(ValueError):
        m._set_basis_set("cc-pvdz")
    m = molecule._Molecule("H 0 0 0;H 0 0 1.4;", 0, "bohr")
    m._set_basis_set("6-31G**")
    assert m.number_bf == 10


def test_angstrom_factor_and_geometries():
    m = molecule._Molecule("H 0 0 0;H 0 0 1", 0, "angstrom")
    assert m.atom_coordinates[1, 2] == 1.889725989
    c = systems.water_cluster(16, 11.0, seed=16)
    xyz = np.array([[float(v) for v in a.split()[1:]] for a in c.split(";")])
    o = xyz[0::3]
    d = np.linalg.norm(o[:, None] - o[None], axis=-1) + np.eye(len(o)) * 10
    assert d.min() >= 2.7 and xyz.min() > -1.0 and xyz.max() < 12.0
    oh = np.linalg.norm(xyz[1::3] - o, axis=1)
    np.testing.assert_allclose(oh, 0.96, atol=1e-9)
    assert len(systems.octane().split(";")) == 26
    assert len(systems.hydrogen_chain(24, seed=24).split(";")) == 24


def _brute_force(pc, q, thr):
    n = len(q)
    out = set()
    for P in range(n):
        for Q in range(n):
            if pc[Q] > pc[P] or (pc[Q] == pc[P] and Q > P):
                continue
            if q[P] * q[Q] >= thr:
                out.add((P, Q))
    return out


@pytest.mark.parametrize("seed,npc", [(0, 6), (1, 6), (2, 6), (3, 10), (4, 10)])
def test_quartet_lists_unique_and_complete(seed, npc):
    """npc = 6: s, p, d pair classes; 10: with the f pair classes (quartet classes up to 54)."""
    rng = np.random.default_rng(seed)
    n = 60
    pc = np.sort(rng.integers(0, npc, n)).astype(np.int32)
    npa = rng.choice([1, 3, 8], n)
    npb = rng.choice([1, 3], n)
    q = 10.0 ** rng.uniform(-9, 0.5, n)
    thr = 1e-6
    lists, ket = screening.build_tasks(pc, npa, npb, q, thr)
    bra, kst, cnt, toff, off = screening.flatten_tasks(lists[0])
    pairs = screening.expand_host(bra, kst, cnt, ket)
    got = {tuple(sorted(p, key=lambda x: (pc[x], x), reverse=True)) for p in pairs}
    assert len(got) == len(pairs)  # no quartet twice
    ref = {tuple(sorted(p, key=lambda x: (pc[x], x), reverse=True)) for p in _brute_force(pc, q, thr)}
    assert got == ref
    # each class segment holds only its class, bra class >= ket class
    for c in range(screening.NQCLASS):
        seg = pairs[off[c]:off[c + 1]]
        for P, Q in seg:
            assert screening.quartet_class(pc[P], pc[Q]) == c and pc[P] >= pc[Q]
    # the fp64 / fp32 split partitions the same set by the bound
    l2, ket2 = screening.build_tasks(pc, npa, npb, q, thr, fp32_threshold=1e-3)
    p64 = screening.expand_host(*screening.flatten_tasks(l2[0])[:3], ket2)
    p32 = screening.expand_host(*screening.flatten_tasks(l2[1])[:3], ket2)
    assert len(p64) + len(p32) == len(pairs)
    assert np.all(q[p64[:, 0]] * q[p64[:, 1]] >= 1e-3)
    assert np.all(q[p32[:, 0]] * q[p32[:, 1]] < 1e-3)


def test_screening_boundary_uses_product_test():
    q = np.array([1e-3, 1e-3 * (1 + 1e-16), 2e-3])
    x = np.array([1e-3])
    thr = float(x[0] * q[0])
    c = screening.prefix_counts(x, np.sort(q)[::-1], thr)
    assert c[0] == int(np.sum(x[0] * q >= thr))


def _header_functions():
    text = open(os.path.join(ROOT, "include", "slowquant_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:[A-Za-z_]\w*[\s*]+)+(sq_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_bound_entry_points():
    from slowquant_gb300 import _lib

    assert set(_header_functions()) == set(_lib.EXPORTED)


def test_library_exports_every_header_symbol():
    from slowquant_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for name in _header_functions():
        assert hasattr(lib, name), name
    assert lib.sq_version() >= 1


def test_sub_slot_table_partitions_each_slot():
    """Sub-slot chunks tile their parent's primitive pairs exactly and carry the right bound sums."""
    import numpy as np

    from slowquant_gb300 import screening

    rng = np.random.default_rng(11)
    nslot = 40
    npp = rng.integers(1, 65, nslot)
    pstride = rng.integers(1, 9, nslot)
    pbase = np.cumsum(np.concatenate([[0], npp[:-1] * pstride[:-1]]))
    E = rng.integers(1, 12, nslot)
    hbase = np.cumsum(np.concatenate([[0], (npp * E * pstride)[:-1]]))
    w = rng.uniform(1, 50, nslot)
    q = rng.uniform(0, 1, int(npp.sum()))
    qcum = np.concatenate([[0.0], np.cumsum(q)])
    off = np.concatenate([[0], np.cumsum(npp)[:-1]])
    first, t = screening.sub_slot_table(npp, pbase, pstride, hbase, E, w, qcum, off, int(npp.max()), 512)
    assert first, "some slots must be split"
    for S, f in first.items():
        for s in np.nonzero(f >= 0)[0]:
            ids = f[s] - nslot + np.arange(S)
            assert np.all(t["parent"][ids] == s)
            assert t["npp"][ids].sum() == npp[s]
            assert np.all((t["code"][ids] & 0xFFFF) == S) and np.all((t["code"][ids] >> 16) == np.arange(S))
            lo = np.concatenate([[0], np.cumsum(t["npp"][ids])[:-1]])
            np.testing.assert_array_equal(t["pbase"][ids], pbase[s] + lo * pstride[s])
            np.testing.assert_array_equal(t["hbase"][ids], hbase[s] + lo * E[s] * pstride[s])
            np.testing.assert_allclose(t["qsum"][ids].sum(), q[off[s]:off[s] + npp[s]].sum(), rtol=1e-12)
            assert npp[s] >= S


def test_ket_chunk_partition():
    """_ket_chunks: every (bra, ket) entry is kept whole or cut into all of its ket
    chunks, and each piece lands in FP64 exactly when its bound reaches tau."""
    from types import SimpleNamespace

    import numpy as np

    from slowquant_gb300 import screening
    from slowquant_gb300.engine import IntegralEngine

    rng = np.random.default_rng(5)
    nslot = 30
    npp = rng.integers(1, 40, nslot)
    pstride = np.ones(nslot, np.int64)
    pbase = np.concatenate([[0], np.cumsum(npp)[:-1]])
    E = np.ones(nslot, np.int64)
    q = np.sort(rng.uniform(0, 0.2, int(npp.sum())))[::-1]
    qcum = np.concatenate([[0.0], np.cumsum(q)])
    first, t = screening.sub_slot_table(npp, pbase, pstride, pbase, E, np.ones(nslot), qcum, pbase,
                                        int(npp.max()), 512, 2)
    qs = np.concatenate([qcum[pbase + npp] - qcum[pbase], t["qsum"]])
    fake = SimpleNamespace(slot_qsum=qs, slot_npp=np.concatenate([npp, t["npp"]]), sub_first=first)
    fake._ket_chunks = IntegralEngine._ket_chunks.__get__(fake)
    entries = np.stack([rng.integers(0, nslot, 400), rng.integers(0, nslot, 400)], 1).astype(np.int32)
    tau = 0.05
    e64, e32 = fake._ket_chunks(entries, tau)
    # bounds on the right side of tau: FP64 pieces reach it; an FP32 piece is below it,
    # or is a whole ket each of whose chunks is below it (same arithmetic as its chunks)
    assert np.all(qs[e64[:, 0]] * qs[e64[:, 1]] >= tau)
    for b, k in e32:
        if qs[b] * qs[k] < tau:
            continue
        assert k < nslot
        S = max(S for S in first if first[S][k] >= 0 and npp[k] >= 4 * S)
        chunks = first[S][k] + np.arange(S)
        assert np.all(qs[b] * qs[chunks] < tau)
    # every entry's ket primitive pairs are covered exactly once
    npp_all = fake.slot_npp
    got = {}
    for b, k in np.concatenate([e64, e32]):
        parent = k if k < nslot else t["parent"][k - nslot]
        got[(b, parent)] = got.get((b, parent), 0) + int(npp_all[k])
    want = {}
    for b, k in entries:
        want[(b, k)] = want.get((b, k), 0) + int(npp[k])
    assert got == want


def _header_defines():
    """Integer #defines of the public header, expressions evaluated in order."""
    text = open(os.path.join(ROOT, "include", "slowquant_gb300.h")).read()
    vals = {}
    for name, expr in re.findall(r"^#define\s+(SQ_\w+)\s+([^/\n]+)", text, flags=re.M):
        expr = expr.strip()
        try:
            vals[name] = eval(expr, {"__builtins__": {}}, dict(vals))
        except (NameError, SyntaxError):
            continue
    return vals


def test_header_constants_match_python_bindings():
    from slowquant_gb300 import _lib

    d = _header_defines()
    names = [n for n in dir(_lib) if n.startswith("SQ_") and isinstance(getattr(_lib, n), (int, float))]
    assert len(names) > 20
    for n in names:
        if n in d:
            assert getattr(_lib, n) == d[n], n
    for n in ("SQ_MAX_L", "SQ_MAX_QCLASS", "SQ_MAX_L_GRAD", "SQ_BOYS_TAB64_SIZE", "SQ_BOYS_TAB32_SIZE",
              "SQ_BOYS_HI64_OFF", "SQ_BOYS_TAY64_OFF", "SQ_BOYS_DF_OFF", "SQ_DF64", "SQ_ERR_UNSUPPORTED",
              "SQ_OPT_JK_STREAMS"):
        assert n in d and getattr(_lib, n) == d[n], n
    # 10 pair classes (la >= lb, l <= 3) -> 55 quartet classes; the grids fit the orders used
    npc = (d["SQ_MAX_L"] + 1) * (d["SQ_MAX_L"] + 2) // 2
    assert d["SQ_MAX_QCLASS"] == npc * (npc + 1) // 2
    assert d["SQ_BOYS_HI_NCOL"] - 1 >= 4 * d["SQ_MAX_L"] + 7  # F_m + 6 Taylor orders + exp column
    assert (d["SQ_BOYS_HI_NGRID"] - 1) / d["SQ_BOYS_STEP_INV"] >= d["SQ_BOYS_HI_TMAX"] + 0.5 / d["SQ_BOYS_STEP_INV"]


def test_ctypes_structs_match_c_layout(tmp_path):
    """sizeof / offsetof of every ABI struct, from gcc on the public header, equal the ctypes mirrors."""
    import shutil
    import subprocess

    from slowquant_gb300 import _lib

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    structs = {"sq_basis": _lib.SqBasis, "sq_pairs": _lib.SqPairs, "sq_slots": _lib.SqSlots,
               "sq_quartets": _lib.SqQuartets}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "slowquant_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "abi"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    for line in out:
        if not line:
            continue
        cname, field, val = line.split()
        py = structs[cname]
        want = ctypes.sizeof(py) if field == "size" else getattr(py, field).offset
        assert int(val) == want, (cname, field)


def test_quartet_class_indexing_covers_f():
    from slowquant_gb300 import engine, flops, screening

    assert screening.NQCLASS == 55 and len(engine.CLASS_WEIGHT) == 55
    seen = set()
    for c in range(screening.NQCLASS):
        la, lb, lc, ld = flops.quartet_class_l(c)
        assert la >= lb and lc >= ld and engine.pair_class(la, lb) >= engine.pair_class(lc, ld)
        assert screening.quartet_class(engine.pair_class(la, lb), engine.pair_class(lc, ld)) == c
        seen.add((la, lb, lc, ld))
    assert len(seen) == 55
    assert sum(1 for c in range(55) if max(flops.quartet_class_l(c)) == 3) == 34
    assert all(max(flops.quartet_class_l(c)) <= 2 for c in range(21))
    assert engine.F_PER_THREAD == {21, 22, 28}
    assert [flops.quartet_class_l(c) for c in sorted(engine.F_PER_THREAD)] == [(3, 0, 0, 0), (3, 0, 1, 0),
                                                                              (3, 1, 0, 0)]


def test_abi_refuses_bad_arguments_before_touching_the_device():
    """Argument errors come back as status codes with a message (no device work is started)."""
    from slowquant_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    L = _lib.lib()
    defaults = {k: L.sq_get_option(k) for k in (_lib.SQ_OPT_GENERIC_MIN_L, _lib.SQ_OPT_JK_STREAMS,
                                                _lib.SQ_OPT_FP64_UNROLLED_HIGH, _lib.SQ_OPT_GRAD_THREAD,
                                                _lib.SQ_OPT_DF_CLASSES)}
    try:
        assert defaults[_lib.SQ_OPT_JK_STREAMS] == 8 and defaults[_lib.SQ_OPT_GENERIC_MIN_L] == 5
        assert defaults[_lib.SQ_OPT_FP64_UNROLLED_HIGH] == 0x7F << 12
        assert defaults[_lib.SQ_OPT_DF_CLASSES] == -1  # the measured per-class policy
        assert L.sq_set_option(_lib.SQ_OPT_DF_CLASSES, -2) == _lib.SQ_ERR_ARG
        assert L.sq_set_option(_lib.SQ_OPT_JK_STREAMS, 0) == _lib.SQ_ERR_ARG
        assert L.sq_set_option(_lib.SQ_OPT_JK_STREAMS, 17) == _lib.SQ_ERR_ARG
        assert L.sq_set_option(_lib.SQ_OPT_FP64_UNROLLED_HIGH, 1 << _lib.SQ_MAX_QCLASS) == _lib.SQ_ERR_ARG
        assert L.sq_set_option(99, 1) == _lib.SQ_ERR_ARG
        assert b"unknown key" in L.sq_last_error()
        assert L.sq_set_option(_lib.SQ_OPT_JK_STREAMS, 3) == _lib.SQ_OK and L.sq_get_option(_lib.SQ_OPT_JK_STREAMS) == 3
        assert L.sq_set_launch_config(_lib.SQ_MAX_QCLASS, 0, 64, 100) == _lib.SQ_ERR_ARG
        assert L.sq_set_launch_config(_lib.SQ_MAX_QCLASS - 1, 0, 48, 100) == _lib.SQ_ERR_ARG
        assert L.sq_set_launch_config(_lib.SQ_MAX_QCLASS - 1, 0, 0, 0) == _lib.SQ_OK  # back to the built-in shape
        buf = (ctypes.c_double * 64)()
        p = ctypes.addressof(buf)
        assert L.sq_boys(2, None, 1, p, 0, p, None) == _lib.SQ_ERR_ARG
        assert L.sq_boys(9, p, 1, p, 0, p, None) == _lib.SQ_ERR_ARG  # beyond the d grid
        assert L.sq_boys(17, p, 1, p, 2, p, None) == _lib.SQ_ERR_ARG  # beyond the high-order grid
        assert L.sq_boys(2, p, 1, p, 3, p, None) == _lib.SQ_ERR_ARG  # unknown mode
        L.sq_boys(9, p, 1, p, 0, p, None)
        assert b"n_max 9 out of range" in L.sq_last_error()
        assert L.sq_jk(None, None, None, None, None, None, None, None, None, None, 0, None) == _lib.SQ_ERR_ARG
        assert b"NULL" in L.sq_last_error()
        assert L.sq_grad_2e(None, None, None, None, None, None, None, None) == _lib.SQ_ERR_ARG
        assert L.sq_jk_df(None, None, None, None, None, None, None, None, None, None, 0.0, None) == _lib.SQ_ERR_ARG
        assert L.sq_batched_eigh(1, p, p, 129, p, p, p, p, 1e-12, 10, None, None) == _lib.SQ_ERR_ARG
        assert b"dimension" in L.sq_last_error()
    finally:
        for k, v in defaults.items():
            L.sq_set_option(k, v)


def test_noalloc_refuses_packed_density_beyond_scratch_before_device_work():
    """sq_jk_noalloc bounds the packed density length, not only nbf.

    A batch basis (mat_base set) has nbf = its largest molecule, while its
    matrices hold sum_i n_i^2 elements; the static FP32 scratch holds
    SQ_NOALLOC_MAX_ELEMS.  The refusal must come back as SQ_ERR_ARG before any
    CUDA call: no pointer below is dereferenced and no GPU is needed.
    """
    from slowquant_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    L = _lib.lib()
    b = _lib.SqBasis()
    b.nbf = 50  # small largest molecule ...
    b.mat_base = 0x1000  # ... in a packed batch (never read: refused first)
    b.mat_ld = 0x1000
    b.mat_total = _lib.SQ_NOALLOC_MAX_ELEMS + 1  # ... whose matrices overflow the scratch
    for prec in (_lib.SQ_FP32, _lib.SQ_FP64):
        rc = L.sq_jk_noalloc(ctypes.byref(b), None, None, None, None, None, None, None, None, prec, None)
        assert rc == _lib.SQ_ERR_ARG
        assert b"static scratch limit" in L.sq_last_error() and b"elements" in L.sq_last_error()
    b.mat_total = -1
    assert L.sq_jk_noalloc(ctypes.byref(b), None, None, None, None, None, None, None, None, 1, None) == \
        _lib.SQ_ERR_ARG
    one = _lib.SqBasis()
    one.nbf = _lib.SQ_NOALLOC_MAX_NBF + 1
    assert L.sq_jk_noalloc(ctypes.byref(one), None, None, None, None, None, None, None, None, 1, None) == \
        _lib.SQ_ERR_ARG
    assert b"basis functions" in L.sq_last_error()


def test_solid_harmonic_transform_is_orthonormal_per_shell():
    """T^T S T is the identity inside every shell (d and f included), and the
    spherical counts are those published for cc-pVXZ (24 per water in cc-pVDZ)."""
    from slowquant_gb300 import spherical

    m = molecule._Molecule("O 0 0 0;", 0, "bohr")
    m._set_basis_set("cc-pvtz")
    T = spherical.transform_matrix(m.shells)
    assert T.shape == (35, 30)
    S = O.OracleMolecule("O 0 0 0;", "cc-pvtz", "bohr").one_electron()[0]
    Ss = T.T @ S @ T
    off = 0
    for s in m.shells:
        n = 2 * int(np.sum(s.angular_moments[0])) + 1
        np.testing.assert_allclose(Ss[off:off + n, off:off + n], np.eye(n), atol=1e-13)
        off += n
    w = molecule._Molecule(systems.water_cluster(16, 11.0, seed=16), 0, "angstrom")
    w._set_basis_set("cc-pvdz")
    assert spherical.n_spherical(w.shells) == 384 and w.number_bf == 400


def test_headline_fixtures_match_the_synthetic_generators():
    """The oracle fixtures of the two headline clusters were made from the same seeded geometries."""
    for name, (nw, box, seed, nbf) in {"headline_c2": (8, 9.0, 8, 200), "headline_c3": (16, 11.0, 16, 400)}.items():
        g = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
        assert str(g["geometry"]) == systems.water_cluster(nw, box, seed)
        assert int(g["nbf"]) == nbf and g["C_occ"].shape == (nbf, 5 * nw)
        assert g["JR"].shape == (nbf, 8) and float(g["screen"]) == 1e-12
        # the SCF converged: the last two iteration energies agree to the SCF threshold
        assert abs(g["energies"][-1] - g["energies"][-2]) < 1e-9
        assert abs(float(g["E_at_D"]) - float(g["E_hf"])) < 1e-9


def test_dropin_aliases_resolve_and_uninstall_cleanly():
    """Option A: the reference's module names import this package's objects; uninstall restores sys.modules."""
    import sys

    from slowquant_gb300 import dropin, hartreefock

    before = {k: v for k, v in sys.modules.items() if k == "slowquant" or k.startswith("slowquant.")}
    saved = dropin.install()
    try:
        import slowquant.SlowQuant as sq
        from slowquant.hartreefock.diis import DIIS
        from slowquant.hartreefock.hartreefock_in_memory import run_hartree_fock
        from slowquant.molecularintegrals.electronrepulsion import get_cauchy_schwarz_matrix  # noqa: F401
        from slowquant.molecularintegrals.integralclass import _Integral  # noqa: F401

        assert sq.SlowQuant.__module__ == "slowquant_gb300.SlowQuant"
        assert DIIS is hartreefock.DIIS and run_hartree_fock is hartreefock.run_hartree_fock
    finally:
        dropin.uninstall(saved)
    after = {k: v for k, v in sys.modules.items() if k == "slowquant" or k.startswith("slowquant.")}
    assert after == before


def test_centre_of_mass_uses_the_reference_masses():
    """The multipole origin: the reference's centre of mass (its mass table) for the golden molecules."""
    g = load_golden("multipole")
    for tag in ("h2o_631gs", "h2o2_ccpvtz"):
        m = molecule._Molecule(str(g[f"{tag}_geometry"]), 0, str(g[f"{tag}_unit"]))
        np.testing.assert_allclose(m.center_of_mass, g[f"{tag}_com"], atol=1e-12)


def test_torch_operators_are_registered_with_shape_rules():
    """torch.ops.slowquant_gb300.* exist and give output shapes on fake tensors (no device needed)."""
    import torch
    from torch._subclasses.fake_tensor import FakeTensorMode

    import slowquant_gb300.torch_ops as ops

    with FakeTensorMode():
        V = torch.empty(6, 6, 6, 6, dtype=torch.float64)
        D = torch.empty(6, 6, dtype=torch.float64)
        J, K = torch.ops.slowquant_gb300.jk_dense(V, D)
        assert J.shape == K.shape == (6, 6)
        C = torch.empty(6, 4, dtype=torch.float64)
        assert torch.ops.slowquant_gb300.ao2mo(C, V).shape == (4, 4, 4, 4)
        J, K = torch.ops.slowquant_gb300.direct_jk(1, D, 1e-12, "fp64", 1e-4)
        assert J.shape == (6, 6)
    assert ops.register_engine(object()) >= 1


def test_double_float_class_policy():
    """Which classes an SQ_DF64 launch runs in double-float (host-side dispatch, no device work)."""
    from slowquant_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    L = _lib.lib()
    big = 1 << 40
    assert L.sq_get_option(_lib.SQ_OPT_DF_CLASSES) == -1
    always = (0, 1, 2, 3, 6, 7, 10, 15, 16)
    long_only = (4, 5, 8, 9, 11)
    never = (12, 13, 14, 17, 18)
    for c in always:
        assert L.sq_df_class(c, 1) == 1 and L.sq_df_class(c, big) == 1
    for c in long_only:
        assert L.sq_df_class(c, 1) == 0 and L.sq_df_class(c, big) == 1
    for c in never + tuple(range(19, _lib.SQ_MAX_QCLASS)) + (-1, _lib.SQ_MAX_QCLASS):
        assert L.sq_df_class(c, big) == 0
    try:
        assert L.sq_set_option(_lib.SQ_OPT_DF_CLASSES, (1 << 12) | (1 << 3) | (1 << 20)) == _lib.SQ_OK
        assert [c for c in range(19) if L.sq_df_class(c, 1)] == [3, 12]
        assert L.sq_df_class(20, 1) == 0  # no double-float kernel, whatever the mask
    finally:
        L.sq_set_option(_lib.SQ_OPT_DF_CLASSES, -1)
    assert L.sq_df_class(12, big) == 0


def test_ket_chunk_entries_cut_whole_kets_only():
    """screening.ket_chunk_entries: each whole ket with chunks becomes its chunks, in place; others stay."""
    from slowquant_gb300 import screening

    nslot = 5
    # chunk tables: S = 2 for slots 1, 3; S = 4 for slot 3 only (ids continue after the slots)
    sub_first = {2: np.array([-1, 5, -1, 7, -1]), 4: np.array([-1, -1, -1, 9, -1])}
    seg = np.array([[0, 1], [2, 3], [4, 0], [1, 8]], dtype=np.int32)  # the last ket is a sub-slot already
    out = screening.ket_chunk_entries(seg, sub_first, nslot, want=4)
    assert out.tolist() == [[0, 5], [0, 6], [2, 9], [2, 10], [2, 11], [2, 12], [4, 0], [1, 8]]
    out2 = screening.ket_chunk_entries(seg, sub_first, nslot, want=2)
    assert out2.tolist() == [[0, 5], [0, 6], [2, 7], [2, 8], [4, 0], [1, 8]]
    assert screening.ket_chunk_entries(seg, sub_first, nslot, want=1).tolist() == seg.tolist()
    assert screening.ket_chunk_entries(np.zeros((0, 2), np.int32), sub_first, nslot, 4).shape == (0, 2)
