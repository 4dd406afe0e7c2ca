"""The C-ABI library loads and exports every entry point the header declares;
host-only utilities answer the reference's known answers (no GPU needed)."""
import json
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            with open(os.path.join(ROOT, "include", f)) as fh:
                text = re.sub(r"/\*.*?\*/", "", fh.read(), flags=re.S)
            names |= set(re.findall(r"\b(mhdproj_[a-z0-9_]+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    from mhdproj import build
    import mhdproj

    build.build()
    return mhdproj.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 19
    for n in sorted(names):
        assert hasattr(lib, n), n
    import mhdproj

    assert set(mhdproj.EXPORTED) <= names


def test_hierarchy_matches_reference_known_answers(lib):
    import mhdproj

    with open(os.path.join(ROOT, "tests", "golden", "known_answers.json")) as f:
        k = json.load(f)
    for case in k["hierarchy"]:
        assert mhdproj.hierarchy(case["dims"])[1] == case["coarse_cells"]
    for dims in k["hierarchy_rejected"]:
        with pytest.raises(ValueError):
            mhdproj.hierarchy(dims)


def test_anchors_match_reference_known_answers(lib):
    import mhdproj

    with open(os.path.join(ROOT, "tests", "golden", "known_answers.json")) as f:
        k = json.load(f)
    a = k["anchors"][0]
    comps, mask = mhdproj.anchors(a["mask"], a["dims"], 0)
    assert comps == a["components"] and list(mask & 3) == k["anchors_first_case_classes"]
    assert [int(mask[0] >> 2), int(mask[2] >> 2)] == k["anchors_first_case_roots"]
    b = k["anchors"][1]
    assert mhdproj.anchors(b["mask"], b["dims"], 1)[0] == b["components"]


def test_product_anchors_match_oracle_on_random_masks(lib, oracle_lib):
    import numpy as np
    import mhdproj

    rng = np.random.default_rng(0)
    for dims, per in [((9, 7, 5), 0), ((9, 7, 5), 5), ((4, 4, 4), 7)]:
        m = (rng.random(dims[0] * dims[1] * dims[2]) < 0.55).astype(np.uint32)
        a = mhdproj.anchors(m, dims, per)
        b = oracle_lib.anchors(m, dims, per)
        assert a[0] == b[0] and np.array_equal(a[1], b[1])


def test_create_without_gpu_fails_loudly(lib):
    import torch
    import mhdproj

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(Exception):
        mhdproj.PressureProjection((8, 8, 8), 1e-3)


def test_em_create_without_gpu_fails_loudly(lib):
    import torch
    import mhdproj

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(Exception):
        mhdproj.EmInduction((8, 8, 8), 1e-3)


def test_chain_objective_names_match_the_header():
    """The Python objective names map to the header's MHDPROJ_CHAIN_* values."""
    import mhdproj

    with open(os.path.join(ROOT, "include", "mhdproj.h")) as f:
        text = f.read()
    values = {m.group(1): int(m.group(2)) for m in re.finditer(r"MHDPROJ_CHAIN_(\w+) = (\d+)", text)}
    assert values == {"FINAL_OUTLET": 0, "SUMMED_OUTLET": 1}
    names = mhdproj.PressureProjection.CHAIN_OBJECTIVES
    assert names["final"] == values["FINAL_OUTLET"] and names["summed"] == values["SUMMED_OUTLET"]
