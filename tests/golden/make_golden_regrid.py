"""Regenerate tests/golden/regrid_ah_n32.json from the reference's own
known-answer file src/test/test_regrid/reference_results.txt.

Run once in a container that has the reference checked out:
    python tests/golden/make_golden_regrid.py REFERENCE_CHECKOUT
The JSON keeps the Ah-grid entries (the grid of the hot path): the maximum
lat-lon interpolation errors of the xyz scalar field and of the solid
rotation vector field (covariant and contravariant components), for linear
and cubic interpolation, printed by test_regrid_mod.f90 at N=32, nz=3,
Nlon=4N, Nlat=2N+1 with list-directed output (full precision).
"""
import json
import os
import sys


def main(ref_root):
    path = os.path.join(ref_root, "src/test/test_regrid/reference_results.txt")
    lines = open(path).read().splitlines()
    out = []
    k = 0
    while k < len(lines):
        head = lines[k].strip()
        kind = None
        if head == "scalar latlon regrid test, staggering: Ah":
            kind, comps = "scalar", None
        elif head.startswith("vector latlon regrid test, staggering: Ah, components type: "):
            kind, comps = "vector", head.rsplit(" ", 1)[1]
        if kind:
            for off, interp in ((1, "linear"), (2, "cubic")):
                line = lines[k + off]
                assert "(%s)" % interp in line, line
                vals = [float(x) for x in line.split(")")[1].split()]
                out.append({"kind": kind, "components": comps, "interp": interp, "N": 32, "nz": 3,
                            "Nlon": 128, "Nlat": 65, "values": vals,
                            "source": f"src/test/test_regrid/reference_results.txt:{k + off + 1}"})
            k += 3
        else:
            k += 1
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "regrid_ah_n32.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(out)} entries to {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_regrid.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
