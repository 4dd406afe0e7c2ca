"""Extract the reference's known-answer values for the projection path from its
own test sources and write known_answers.json next to this script.

The reference's GPU tests cannot run here (wgpu needs a graphics adapter), so
the golden values are the literal expectations its tests assert:
  * hierarchy sizes: src/fluid/multigrid/tests.rs,
    hierarchy_uses_exact_ceil_half_workspace_and_checked_indices
  * gauge anchors on tiny masks: src/fluid/tests.rs,
    pressure_failure_rolls_back_and_disconnected_components_get_gauges
  * acceptance tolerances of the analytic projection tests.
Run: python tests/golden/make_known_answers.py <reference root>
(or set MHD_REFERENCE_ROOT to the reference checkout).
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MHD_REFERENCE_ROOT")
if not ROOT:
    sys.exit("usage: make_known_answers.py <reference root>  (or set MHD_REFERENCE_ROOT)")
HERE = os.path.dirname(os.path.abspath(__file__))


def read(rel):
    with open(os.path.join(ROOT, rel)) as f:
        return f.read()


def main():
    mg = read("src/fluid/multigrid/tests.rs")
    m = re.search(r"fn hierarchy_uses_exact_ceil_half_workspace_and_checked_indices\(\) \{(.*?)\n\}", mg, re.S)
    body = m.group(1)
    cases = []
    for dims, expected in re.findall(r"\(\[([^\]]+)\],\s*([0-9_]+)(?:u64)?\)", body):
        parts = [p.strip() for p in dims.split(",")]

        def val(p):
            p = p.replace("u32", "")
            if ".pow(" in p:
                b, e = re.match(r"(\d+)\.pow\((\d+)\)", p).groups()
                return int(b) ** int(e)
            return int(p)

        cases.append({"dims": [val(p) for p in parts], "coarse_cells": int(expected.replace("_", ""))})
    rejected = []
    for dims in re.findall(r"assert!\(hierarchy\(\[([^\]]+)\]", body):
        vals = []
        for p in dims.split(";") if ";" in dims else dims.split(","):
            p = p.strip()
            vals.append(p)
        if len(vals) == 2 and vals[0] == "u32::MAX":  # [u32::MAX; 4]
            rejected.append([0xFFFFFFFF] * 4)
        else:
            rejected.append([0xFFFFFFFF if v == "u32::MAX" else int(v) for v in vals])
    ft = read("src/fluid/tests.rs")
    anchors = []
    for block in re.findall(r"let mut mask = vec!\[([^\]]+)\];\s*assert_eq!\(anchors\(&mut mask, \[([^\]]+)\], \[([^\]]+)\]\), (\d+)\);", ft):
        mask = [int(v) for v in block[0].split(",")]
        dims = [int(v) for v in block[1].split(",")]
        per = block[2].strip()
        periodic = [True, False, False] if per.startswith("true") else [False, False, False]
        anchors.append({"mask": mask, "dims": dims, "periodic": periodic, "components": int(block[3])})
    m = re.search(r"mask\.iter\(\)\.map\(\|v\| v & 3\)\.collect::<Vec<_>>\(\),\s*vec!\[([^\]]+)\]", ft)
    classes = [int(v) for v in m.group(1).split(",")]
    roots = [int(v) for v in re.findall(r"assert_eq!\(mask\[\d\] >> 2, (\d+)\);", ft)]
    out = {
        "source": "sdfgeoff/mhd-simulator tests (literal expectations)",
        "hierarchy": cases,
        "hierarchy_rejected": rejected,
        "anchors": anchors,
        "anchors_first_case_classes": classes,
        "anchors_first_case_roots": roots,
        "tolerances": {
            "periodic_cosine_pressure_rel_l2": 1e-4,
            "periodic_cosine_max_speed": 2e-6,
            "manufactured_projection_rel_l2": 2e-4,
            "galerkin_rel": 2e-6,
            "vcycle_symmetry": 3e-6,
            "fused_coarse_rel": 2e-6,
            "cached_operator_rel": 2e-7,
        },
    }
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
