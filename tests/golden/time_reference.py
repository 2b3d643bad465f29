"""Time the unmodified SlowQuant reference on the small configurations -- TEST INFRASTRUCTURE.

The reference is pure Python + numba.  numba is not installed in the build
container, so (as in make_golden.py) a no-op stand-in is registered and the
reference runs as plain CPython/numpy, single-threaded (OMP/BLAS threads are
pinned to 1 before numpy loads).  The Python reference cannot be installed on
the GPU hosts, so its timings are recorded here, with the machine they were
taken on, in ``reference_timings.json``; the benchmark's reference arm prints
them beside its own CPU measurement.

Workloads (BASELINE C1 and the next size up):
* H2O, O-H 0.96 A, H-O-H 104.5 deg, STO-3G (7 functions): ERI tensor
  (``_Integral.electron_repulsion_tensor``) and the RHF SCF
  (``run_restricted_hartree_fock``, thresholds 1e-9);
* the same water in cc-pVDZ (25 functions): ERI tensor and SCF.

Run:  python tests/golden/time_reference.py --reference PATH
"""

from __future__ import annotations

import os

for _v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ[_v] = "1"

import argparse  # noqa: E402
import json  # noqa: E402
import platform  # noqa: E402
import sys  # noqa: E402
import time  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of a SlowQuant checkout (the directory holding slowquant/)")
    args = ap.parse_args()
    from slowquant_gb300 import systems
    from tests.golden.make_golden import install_numba_standin

    install_numba_standin()
    sys.path.insert(0, args.reference)
    import slowquant.SlowQuant as sq

    geom = systems.water_monomer()
    out = {"machine": {"platform": platform.platform(), "processor": platform.processor() or platform.machine(),
                       "nproc": os.cpu_count(), "threads_used": 1,
                       "python": platform.python_version()},
           "note": "unmodified reference, numba replaced by a no-op stand-in (pure CPython/numpy), one thread",
           "runs": []}
    for basis in ("sto-3g", "cc-pvdz"):
        A = sq.SlowQuant()
        A.set_molecule(geom, distance_unit="angstrom")
        t0 = time.time()
        A.set_basis_set(basis)  # builds the Schwarz matrix eagerly (integralclass.py:38)
        t_setup = time.time() - t0
        t0 = time.time()
        eri = A.integral.electron_repulsion_tensor
        t_eri = time.time() - t0
        A.init_hartree_fock()
        A.hartree_fock.logger.print_output = False
        t0 = time.time()
        A.hartree_fock.run_restricted_hartree_fock()
        t_scf = time.time() - t0
        n = eri.shape[0]
        out["runs"].append({"system": "H2O (O-H 0.96 A, 104.5 deg)", "basis": basis, "nbf": n,
                            "setup_with_schwarz_s": round(t_setup, 3), "eri_tensor_s": round(t_eri, 3),
                            "scf_s": round(t_scf, 3), "E_hf": A.hartree_fock.E_hf})
        print(out["runs"][-1], flush=True)
    with open(os.path.join(HERE, "reference_timings.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
