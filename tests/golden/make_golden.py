"""Generate the golden fixtures in this folder by running the SlowQuant reference itself.

This script is test infrastructure. It imports the unmodified reference package
(``slowquant``, pure Python + numba) from the checkout given as
``--reference``.  numba is not installed in the build container, so a
no-op stand-in module is registered under ``sys.modules['numba']`` before the
import: ``jit(...)`` returns the function unchanged and the numba type objects
are inert.  The reference arithmetic then runs as CPython floats / numpy, which
differs from numba-compiled code only at the ulp level.

Outputs (``*.npz``, ``golden_energies.json``) are small and committed; the
parity tests read them on machines where the reference is absent.

Run:  python tests/golden/make_golden.py --reference PATH [--only NAME ...]
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def install_numba_standin() -> None:
    """Register a no-op ``numba`` module (jit returns the function unchanged)."""

    class _Type:
        def __getitem__(self, item):
            return self

        def __call__(self, *args, **kwargs):
            return self

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not isinstance(args[0], _Type) and not kwargs:
            return args[0]

        def deco(fn):
            return fn

        return deco

    mod = types.ModuleType("numba")
    mod.jit = jit
    mod.njit = jit
    mod.float64 = _Type()
    mod.int64 = _Type()
    mod.prange = range
    sys.modules["numba"] = mod


class ListLog:
    """Captures the reference's log lines (``add_to_log`` contract)."""

    def __init__(self):
        self.lines: list[str] = []

    def add_to_log(self, content: str, is_warning: bool = False) -> None:
        self.lines.append(("WARNING: " if is_warning else "") + content)


# Geometries -------------------------------------------------------------------
# H2O in bohr as used by the reference's RHF known-answer tests
# (tests/test_hartreefock.py:13-18).
H2O_CRAWFORD_BOHR = """O 0.000000000000  -0.143225816552   0.000000000000;
           H 1.638036840407   1.136548822547  -0.000000000000;
           H -1.638036840407   1.136548822547  -0.000000000000;"""
# CH4 in bohr (tests/test_hartreefock.py:70-75).
CH4_BOHR = """C  -0.000000000000   0.000000000000   0.000000000000;
           H   1.183771681898  -1.183771681898  -1.183771681898;
           H   1.183771681898   1.183771681898   1.183771681898;
           H  -1.183771681898   1.183771681898  -1.183771681898;
           H  -1.183771681898  -1.183771681898   1.183771681898"""
# H6 chain, 1 bohr spacing (tests/test_integral.py:15-22).
H6_BOHR = ";".join(f"H   {float(i):.12f}   0.000000000000   0.000000000000" for i in range(6))


def water_monomer_angstrom() -> str:
    """Single H2O: O at origin, O-H 0.96 A, H-O-H 104.5 deg, in the xy plane."""
    r = 0.96
    half = np.deg2rad(104.5) / 2.0
    h1 = (r * np.sin(half), r * np.cos(half), 0.0)
    h2 = (-r * np.sin(half), r * np.cos(half), 0.0)
    return (
        f"O 0.0 0.0 0.0;H {h1[0]:.15f} {h1[1]:.15f} {h1[2]:.15f};H {h2[0]:.15f} {h2[1]:.15f} {h2[2]:.15f}"
    )


def unique_eri(V: np.ndarray) -> np.ndarray:
    """Pack a dense (n,n,n,n) ERI tensor into its 8-fold unique elements.

    Order: i>=j, k>=l, ij>=kl with ij=i(i+1)/2+j, loops i,j,k,l ascending.
    """
    n = V.shape[0]
    ii, jj = np.tril_indices(n)
    npair = len(ii)
    P, Q = np.tril_indices(npair)
    return V[ii[P], jj[P], ii[Q], jj[Q]].copy()


def run_system(sq, name, geom, unit, basis, *, eri=True, eri_store="full", scf=True, out=None):
    t0 = time.time()
    A = sq.SlowQuant()
    A.set_molecule(geom, distance_unit=unit)
    A.set_basis_set(basis)
    res = {"basis": basis, "unit": unit, "geometry": geom, "nbf": int(A.molecule.number_bf),
           "nshell": int(A.molecule.number_shell), "E_nuc": float(A.molecule.nuclear_repulsion)}
    arrays = {"schwarz": A.integral._cauchy_schwarz_matrix,
              "S": A.integral.overlap_matrix, "T": A.integral.kinetic_energy_matrix,
              "V": A.integral.nuclear_attraction_matrix}
    if eri:
        V = A.integral.electron_repulsion_tensor
        arrays["eri_unique" if eri_store == "unique" else "eri"] = (
            unique_eri(V) if eri_store == "unique" else V
        )
    if scf:
        import slowquant.hartreefock.hartreefock_in_memory as hfm

        log = ListLog()
        E, C, F, D = hfm.run_hartree_fock(
            A.integral.overlap_matrix, A.integral.kinetic_energy_matrix,
            A.integral.nuclear_attraction_matrix, A.integral.electron_repulsion_tensor,
            A.molecule.number_electrons, log, 10**-9, 10**-9, 100, True,
        )
        iters = []
        for line in log.lines[1:]:
            parts = line.split()
            if len(parts) == 4 and parts[0].isdigit():
                iters.append(float(parts[1]))
        res.update({"E_hf": float(E), "scf_energies": iters, "n_iter": len(iters)})
        arrays["D"] = D
        arrays["F"] = F
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **arrays)
    res["seconds"] = round(time.time() - t0, 2)
    print(name, res.get("E_hf"), res["nbf"], res["seconds"], flush=True)
    return res


def run_uhf_system(sq, name, geom, unit, basis, *, charge=0, mix=0.15, out=None):
    """Reference UHF (unrestricted_hartreefock_in_memory.py) energy, trajectory and spin densities."""
    t0 = time.time()
    A = sq.SlowQuant()
    A.set_molecule(geom, distance_unit=unit)
    A.set_basis_set(basis)
    A.molecule.molecular_charge = charge
    import slowquant.hartreefock.unrestricted_hartreefock_in_memory as uhfm

    log = ListLog()
    E, Ca, Cb, Fa, Fb, Da, Db = uhfm.run_unrestricted_hartree_fock(
        A.integral.overlap_matrix, A.integral.kinetic_energy_matrix, A.integral.nuclear_attraction_matrix,
        A.integral.electron_repulsion_tensor, A.molecule.number_electrons_alpha,
        A.molecule.number_electrons_beta, mix, log, 10**-9, 10**-9, 100, True,
    )
    iters = []
    for line in log.lines[1:]:
        parts = line.split()
        if len(parts) == 5 and parts[0].isdigit():
            iters.append(float(parts[1]))
    res = {"basis": basis, "unit": unit, "geometry": geom, "charge": charge, "mix": mix,
           "nbf": int(A.molecule.number_bf), "E_nuc": float(A.molecule.nuclear_repulsion),
           "n_alpha": int(A.molecule.number_electrons_alpha), "n_beta": int(A.molecule.number_electrons_beta),
           "E_uhf": float(E), "scf_energies": iters, "n_iter": len(iters)}
    np.savez_compressed(os.path.join(out, f"{name}.npz"), D_alpha=Da, D_beta=Db)
    res["seconds"] = round(time.time() - t0, 2)
    print(name, E, res["nbf"], res["seconds"], flush=True)
    return res


# H2O2 without symmetry (angstrom): two O centres carry f shells in cc-pVTZ.
H2O2_ANGSTROM = """O   0.000000000000   0.000000000000   0.000000000000;
           O   1.452000000000   0.081000000000   0.033000000000;
           H  -0.262000000000   0.912000000000   0.187000000000;
           H   1.698000000000  -0.457000000000   0.811000000000"""


def f_shell_quartets(ref_eri, mol, budget_s: float = 1200.0) -> dict:
    """Contracted blocks of shell quartets with f shells, from the reference's
    electron_repulsion_integral (electronrepulsion.py:107-297).

    Every class with an f shell that the basis offers is sampled: for each
    (la, lb, lc, ld) with la >= lb, lc >= ld, (la,lb) >= (lc,ld) and max l = 3,
    up to two quartets whose shells sit on different centres where possible,
    cheapest first (the reference runs as plain Python here).
    """
    shells = mol.shells
    ls = [int(s.angular_moments.sum(1)[0]) for s in shells]
    atom = [mol.atoms.index(s.origin_atom) for s in shells]
    npr = [len(s.exponents) for s in shells]
    by_l = {l: [i for i in range(len(shells)) if ls[i] == l] for l in range(4)}
    quartets = []
    for la in range(4):
        for lb in range(la + 1):
            for lc in range(la + 1):
                for ld in range(lc + 1):
                    if (la, lb) < (lc, ld) or max(la, lb, lc, ld) < 3:
                        continue
                    cands = []
                    for a in by_l[la]:
                        for b in by_l[lb]:
                            for c in by_l[lc]:
                                for d in by_l[ld]:
                                    ncent = len({atom[a], atom[b], atom[c], atom[d]})
                                    cost = npr[a] * npr[b] * npr[c] * npr[d]
                                    cands.append((-ncent, cost, (a, b, c, d)))
                    cands.sort()
                    quartets += [c[2] for c in cands[:2]]
    keys, blocks = [], []
    t0 = time.time()
    for a, b, c, d in quartets:
        if time.time() - t0 > budget_s:
            break
        s1, s2, s3, s4 = shells[a], shells[b], shells[c], shells[d]
        V = ref_eri(s1.center, s2.center, s3.center, s4.center, s1.exponents, s2.exponents, s3.exponents,
                    s4.exponents, s1.contraction_coefficients, s2.contraction_coefficients,
                    s3.contraction_coefficients, s4.contraction_coefficients, s1.normalization,
                    s2.normalization, s3.normalization, s4.normalization, s1.angular_moments,
                    s2.angular_moments, s3.angular_moments, s4.angular_moments)
        keys.append((a, b, c, d))
        blocks.append(np.asarray(V).ravel())
    off = np.concatenate([[0], np.cumsum([len(b) for b in blocks])]).astype(np.int64)
    return {"quartets": np.array(keys, dtype=np.int64), "block_off": off, "blocks": np.concatenate(blocks),
            "seconds": time.time() - t0}


def boys_grid(ref_boys) -> dict:
    zs = np.concatenate([
        [0.0, 1e-12, 9.9e-11, 1.1e-10, 1e-8, 1e-6, 1e-4, 1e-3, 0.01],
        np.linspace(0.05, 5.0, 25), np.linspace(5.5, 24.5, 20),
        [24.99, 25.0, 25.01, 26.0, 30.0, 35.0, 40.0, 50.0, 80.0, 150.0, 400.0, 1e4],
    ])
    ns = np.arange(0, 17)
    F = np.array([[ref_boys(int(n), float(z)) for z in zs] for n in ns])
    return {"boys_z": zs, "boys_n": ns, "boys_F": F}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of a SlowQuant checkout (the directory holding slowquant/)")
    ap.add_argument("--only", nargs="*", default=None)
    args = ap.parse_args()
    install_numba_standin()
    sys.path.insert(0, args.reference)
    import slowquant.SlowQuant as sq
    from slowquant.molecularintegrals import integralfunctions as ifn
    from slowquant.molecule.moleculeclass import _Molecule

    out = HERE
    energies_path = os.path.join(out, "golden_energies.json")
    energies = json.load(open(energies_path)) if os.path.exists(energies_path) else {}

    def want(name):
        return args.only is None or name in args.only

    if want("primitives"):
        prim = boys_grid(ifn.boys_function)
        rng = np.random.default_rng(7)
        ecases = []
        for la in range(3):
            for lb in range(3):
                A_x, B_x = rng.uniform(-2, 2, 2)
                a, b = rng.uniform(0.1, 20.0, 2)
                E = ifn.expansion_coefficients(A_x, B_x, a, b, la, lb)
                ecases.append(((A_x, B_x, a, b, la, lb), E))
        prim["ecoef_params"] = np.array([c[0] for c in ecases])
        prim["ecoef_values"] = np.concatenate([c[1].ravel() for c in ecases])
        rcases = []
        for L in range(0, 9):
            p = float(rng.uniform(0.2, 30.0))
            PC = rng.uniform(-1.5, 1.5, 3)
            R = ifn.hermite_coulomb_integral(L, L, L, p, PC)
            rcases.append((np.array([L, p, *PC]), R))
        prim["hermite_params"] = np.array([c[0] for c in rcases])
        prim["hermite_values"] = np.concatenate([c[1].ravel() for c in rcases])
        mol = _Molecule(water_monomer_angstrom(), 0, "angstrom")
        mol._set_basis_set("cc-pvdz")
        prim["ccpvdz_h2o_norms"] = np.concatenate([s.normalization.ravel() for s in mol.shells])
        prim["ccpvdz_h2o_centers"] = mol.atom_coordinates
        np.savez_compressed(os.path.join(out, "primitives.npz"), **prim)
        print("primitives done", flush=True)

    if want("multipole"):
        # the reference's multipole matrices (about its centre of mass) for water in 6-31G* and
        # H2O2 in cc-pVTZ (f shells): dipole, quadrupole and some higher mixed orders
        orders = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0), (0, 1, 1), (0, 0, 2),
                  (3, 0, 0), (1, 2, 3)]
        sets = {"h2o_631gs": orders, "h2o2_ccpvtz": [(1, 0, 0), (0, 1, 1), (0, 0, 2), (1, 2, 3)]}
        res = {}
        for tag, geom, unit, basis in (("h2o_631gs", H2O_CRAWFORD_BOHR, "bohr", "6-31G*"),
                                       ("h2o2_ccpvtz", H2O2_ANGSTROM, "angstrom", "cc-pvtz")):
            orders = sets[tag]
            res[f"{tag}_orders"] = np.array(orders)
            A = sq.SlowQuant()
            A.set_molecule(geom, distance_unit=unit)
            A.set_basis_set(basis)
            res[f"{tag}_com"] = A.molecule.center_of_mass
            res[f"{tag}_M"] = np.stack([A.integral.get_multipole_matrix(np.array(o)) for o in orders])
            res[f"{tag}_geometry"] = np.array(geom)
            res[f"{tag}_unit"] = np.array(unit)
            res[f"{tag}_basis"] = np.array(basis)
        np.savez_compressed(os.path.join(out, "multipole.npz"), **res)
        print("multipole done", flush=True)

    if want("h2o2_ccpvtz_f"):
        from slowquant.molecularintegrals.electronrepulsion import electron_repulsion_integral

        mol = _Molecule(H2O2_ANGSTROM, 0, "angstrom")
        mol._set_basis_set("cc-pvtz")
        res = f_shell_quartets(electron_repulsion_integral, mol)
        secs = res.pop("seconds")
        from slowquant.molecularintegrals.kineticenergy import kinetic_energy_integral_driver
        from slowquant.molecularintegrals.multipole import multipole_integral_driver
        from slowquant.molecularintegrals.nuclearattraction import nuclear_attraction_integral_driver

        res["S"] = multipole_integral_driver(mol, np.array([0, 0, 0]))
        res["T"] = kinetic_energy_integral_driver(mol)
        res["V"] = nuclear_attraction_integral_driver(mol)
        np.savez_compressed(os.path.join(out, "h2o2_ccpvtz_f.npz"), **res)
        energies["h2o2_ccpvtz_f"] = {"basis": "cc-pvtz", "unit": "angstrom", "geometry": H2O2_ANGSTROM,
                                     "nbf": int(mol.number_bf), "nshell": int(mol.number_shell),
                                     "E_nuc": float(mol.nuclear_repulsion),
                                     "n_quartets": int(len(res["quartets"])), "seconds": round(secs, 2)}
        json.dump(energies, open(energies_path, "w"), indent=1)
        print("h2o2_ccpvtz_f", len(res["quartets"]), "quartets", round(secs, 1), "s", flush=True)

    systems = [
        ("h2o_sto3g_crawford", H2O_CRAWFORD_BOHR, "bohr", "sto-3g", dict(eri_store="full")),
        ("h2o_sto3g_c1", water_monomer_angstrom(), "angstrom", "sto-3g", dict(eri_store="full")),
        ("ch4_sto3g", CH4_BOHR, "bohr", "sto-3g", dict(eri_store="unique")),
        ("h2o_631gs", H2O_CRAWFORD_BOHR, "bohr", "6-31G*", dict(eri_store="unique")),
        ("h2o_dz", H2O_CRAWFORD_BOHR, "bohr", "dz", dict(eri_store="unique")),
        ("h2o_ccpvdz_c1", water_monomer_angstrom(), "angstrom", "cc-pvdz", dict(eri_store="unique")),
        ("h2o_dzp", H2O_CRAWFORD_BOHR, "bohr", "dzp", dict(eri_store="unique")),
        ("h6_dzp", H6_BOHR, "bohr", "dzp", dict(eri_store="unique", scf=True)),
    ]
    for name, geom, unit, basis, kw in systems:
        if want(name):
            energies[name] = run_system(sq, name, geom, unit, basis, out=out, **kw)
            json.dump(energies, open(energies_path, "w"), indent=1)
    # UHF known-answer cases of the reference (tests/test_unrestrictedhartreefock.py)
    n2 = """N   0.000000000000  0.000000000000   0.000000000000;
                      N  2.074000000000   0.000000000000  -0.000000000000"""
    uhf_systems = [
        ("uhf_h2o_sto3g_mix0", H2O_CRAWFORD_BOHR, "bohr", "sto-3g", dict(mix=0.0)),
        ("uhf_n2_631gs", n2, "bohr", "6-31G*", {}),
        ("uhf_n2cation_631gs", n2, "bohr", "6-31G*", dict(charge=1)),
        ("uhf_li_631gss", "Li   0.000000000000  0.000000000000   0.000000000000;", "bohr", "6-31G**", {}),
    ]
    for name, geom, unit, basis, kw in uhf_systems:
        if want(name):
            energies[name] = run_uhf_system(sq, name, geom, unit, basis, out=out, **kw)
            json.dump(energies, open(energies_path, "w"), indent=1)


if __name__ == "__main__":
    main()
