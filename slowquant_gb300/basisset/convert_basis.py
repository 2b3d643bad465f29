"""Convert Turbomole-format basis-set text files into this package's JSON tables.

The basis sets are published data (Basis Set Exchange exports); the JSON keeps
every exponent and contraction coefficient as the same IEEE double that a
``float(text.replace("D", "e"))`` parse of the text produces, so integrals
built from either source are identical.  Shell order per element is file
order, as the reference's reader keeps it
(slowquant/molecule/basis_reader.py:6-75).

Run once where the text files exist:
    python slowquant_gb300/basisset/convert_basis.py SRC_DIR
SRC_DIR defaults to the reference's ``slowquant/molecule/basisset``.
"""

from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_turbomole(path: str) -> dict[str, list[dict]]:
    """Return {element_lowercase: [{"l": "s", "exponents": [...], "coefficients": [...]}, ...]}."""
    elements: dict[str, list[dict]] = {}
    current: list[dict] | None = None
    pending = 0
    shell: dict | None = None
    with open(path, encoding="UTF-8") as fh:
        for raw in fh:
            line = raw.rstrip("\n")
            if line.startswith("$ecp") or line.startswith("$end"):
                # Only the $basis section is read (effective core potentials are not used).
                break
            if not line or line.startswith("#") or line.startswith("$"):
                continue
            if line[0] == "*":
                continue
            if line[0] != " ":
                # "<element> <basis name>" header line
                current = []
                elements[line.split()[0].lower()] = current
                pending = 0
                continue
            fields = line.split()
            if pending == 0:
                # "<nprim> <l>" shell header
                shell = {"l": fields[1].lower(), "exponents": [], "coefficients": []}
                pending = int(fields[0])
                assert current is not None
                current.append(shell)
                continue
            assert shell is not None
            shell["exponents"].append(float(fields[0].replace("D", "e")))
            shell["coefficients"].append(float(fields[1].replace("D", "e")))
            pending -= 1
    return elements


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: python convert_basis.py <SlowQuant checkout>/slowquant/molecule/basisset")
    src = sys.argv[1]
    for fname in sorted(os.listdir(src)):
        if not fname.endswith(".basis"):
            continue
        data = parse_turbomole(os.path.join(src, fname))
        name = fname[: -len(".basis")]
        with open(os.path.join(HERE, name + ".json"), "w", encoding="UTF-8") as out:
            json.dump({"name": name, "elements": data}, out, separators=(",", ":"))
        print(name, len(data), "elements")


if __name__ == "__main__":
    main()
