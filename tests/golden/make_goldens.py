"""Extracts the reference's own golden values for the DG transport tests.

Reads the doctest sources of the reference as text (nothing is compiled or
run) and writes tests/golden/transport_goldens.json:
  - dynamics/test/Advection_test.cpp   (rotating smooth bump, DG 1/3/6,
    regular and distorted meshes, tolerance 1e-7)
  - dynamics/test/AdvectionPeriodicBC_test.cpp (ring with a periodic edge)
Only the first two resolutions of each table are exercised by the reference
tests (the loop runs it = 0, 1); the json keeps all six values and marks the
checked ones.

Usage: python tests/golden/make_goldens.py [reference source tree]
(default: $NSDG_REFERENCE, else the location the oracle build recipe uses)
"""
import json
import re
import sys
from pathlib import Path

NUM = r"[-+]?\d+\.\d+e[-+]\d+"


def _tables(text):
    out = []
    for block in re.findall(r"std::array<double, 6>\(\s*\{([^}]*)\}", text):
        vals = [float(v) for v in re.findall(NUM, block)]
        assert len(vals) == 6, block
        out.append(vals)
    return out


def main(root):
    root = Path(root)
    adv = (root / "dynamics/test/Advection_test.cpp").read_text()
    per = (root / "dynamics/test/AdvectionPeriodicBC_test.cpp").read_text()
    adv_cases = adv.split('TEST_CASE("Distorted Mesh")')
    regular, distorted = _tables(adv_cases[0]), _tables(adv_cases[1])
    periodic = _tables(per)
    assert len(regular) == 3 and len(distorted) == 3 and len(periodic) == 3
    tol = float(re.search(r"double TOL = ([0-9.e-]+);", adv).group(1))
    dgs = [1, 3, 6]
    data = {
        "source": {
            "advection": "dynamics/test/Advection_test.cpp:274-301",
            "periodic": "dynamics/test/AdvectionPeriodicBC_test.cpp:281-290",
        },
        "tolerance": tol,
        "checked_resolutions": [0, 1],
        "advection_regular": {str(dg): regular[i] for i, dg in enumerate(dgs)},
        "advection_distorted": {str(dg): distorted[i] for i, dg in enumerate(dgs)},
        "periodic": {str(dg): periodic[i] for i, dg in enumerate(dgs)},
    }
    dst = Path(__file__).with_name("transport_goldens.json")
    dst.write_text(json.dumps(data, indent=1) + "\n")
    print("wrote", dst)


def _reference() -> str:
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent.parent))
    from oracle import pyref
    root = pyref.reference_root()
    if root is None:
        sys.exit("give the reference source tree as the argument or in NSDG_REFERENCE")
    return str(root)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else _reference())
