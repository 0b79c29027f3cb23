"""Pin the .re2 reader on the reference's own genbox output: read
short_tests/lpm_one/uniform.re2 from the reference tree, check it against
the box its uniform.box describes (element counts, uniform spacing on the
given ranges, x fastest, preprocessor corner order, the given wall type on
every outside face), and write the figures tests/test_meshio.py compares
(re2_reference.json).  Run where a Nek5000 source tree is present, naming
its root on the command line or in NEK5000_REFERENCE:

    python tests/golden/make_re2_reference.py <path to the Nek5000 tree>
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))


def parse_box(path):
    lines = [l.split("!")[0].strip() for l in open(path)]
    lines = [l for l in lines if l and not l.startswith("#")]
    ndim = abs(int(lines[0].split()[0]))
    i = [k for k, l in enumerate(lines) if l.lower().startswith("box")][0]
    nel = [abs(int(v)) for v in lines[i + 1].replace(",", " ").split()[:ndim]]
    ranges = [[float(v) for v in lines[i + 2 + d].replace(",", " ").split()[:3]]
              for d in range(ndim)]
    bcs = [b.strip() for b in lines[i + 2 + ndim].split(",")][:2 * ndim]
    return ndim, nel, ranges, bcs


def main(ref_root):
    from nek5000_gb300 import build, meshio
    from re2_util import box_elements
    build.build()
    d = os.path.join(ref_root, "short_tests", "lpm_one")
    ndim, nel, ranges, bcs = parse_box(os.path.join(d, "uniform.box"))
    assert ndim == 3 and all(r[2] == 1.0 and r[0] == 0.0 and r[1] == 1.0 for r in ranges)
    R = meshio.read_re2(os.path.join(d, "uniform.re2"))
    xc, yc, zc, _, walls = box_elements(*nel)
    assert R["nelgt"] == int(np.prod(nel)) and R["ndim"] == 3
    for a, b in ((R["xc"], xc), (R["yc"], yc), (R["zc"], zc)):
        assert np.max(np.abs(a - b)) <= 1e-15
    cbc, bc = R["bcs"][0]
    assert all(t == "W" for t in bcs)
    assert all(cbc[el - 1, f - 1] == "W  " for (el, f, _, _) in walls)
    assert (cbc == "W  ").sum() == len(walls) and (cbc == "E  ").sum() == cbc.size - len(walls)
    out = {"uniform.re2": {
        "source": "short_tests/lpm_one/uniform.re2 (genbox output of uniform.box)",
        "header": [R["nelgt"], R["ndim"], R["nelgv"], R["wdsize"]],
        "n_wall_faces": int((cbc == "W  ").sum()),
        "n_bc_sections": len(R["bcs"]),
        "corner_sum": float(np.sum(R["xc"] + 2 * R["yc"] + 3 * R["zc"])),
    }}
    json.dump(out, open(os.path.join(HERE, "re2_reference.json"), "w"), indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NEK5000_REFERENCE")
    if not root:
        sys.exit("name the Nek5000 source tree: an argument or NEK5000_REFERENCE")
    main(root)
