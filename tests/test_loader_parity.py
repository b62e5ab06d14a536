"""The tetgen loader against the reference's own (TetMesh.cpp:14-151).

TetMesh::initNodesFromFile / initTetsFromFile read the shipped meshes
model/*/*.node/.ele into FP32 positions scaled by 0.1 and tets in file
order.  meshes.load_tetgen(stem, scale=0.1, orient=False) must give the same
bits: the digests of the reference loader's arrays are frozen in
tests/golden/loader_models.json (``make_golden.py loader``), and where the
reference's headless build is present the arrays are also compared
directly.  The meshes themselves belong to the reference checkout
(PHYBS_REFERENCE); without it the test skips.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from phybs_gb300 import meshes as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIGESTS = json.load(open(os.path.join(ROOT, "tests", "golden", "loader_models.json")))


def _model_dir():
    tree = os.environ.get("PHYBS_REFERENCE")
    d = os.path.join(tree, "model") if tree else None
    if not d or not os.path.isdir(d):
        pytest.skip("the reference checkout (PHYBS_REFERENCE) with its model/ meshes is not present")
    return d


@pytest.mark.parametrize("rel", sorted(DIGESTS))
def test_load_tetgen_equals_reference_loader(rel):
    stem = os.path.join(_model_dir(), rel)
    want = DIGESTS[rel]
    m = M.load_tetgen(stem, scale=0.1, orient=False)
    assert m.rest.dtype == np.float32 and m.rest.shape == (want["n_nodes"], 3)
    assert m.tets.shape == (want["n_tets"], 4)
    assert hashlib.sha256(np.ascontiguousarray(m.rest).tobytes()).hexdigest() == want["rest_sha256"]
    assert hashlib.sha256(np.ascontiguousarray(m.tets, np.int32).tobytes()).hexdigest() == want["tets_sha256"]
    # the oriented form (what the device path takes) differs only by corner
    # swaps of negatively oriented tets
    mo = M.load_tetgen(stem, scale=0.1)
    assert np.array_equal(mo.rest, m.rest)
    assert (M.signed_volumes(mo.rest, mo.tets) > 0).all()
    assert np.array_equal(np.sort(mo.tets, axis=1), np.sort(m.tets, axis=1))
    # the loader's hard-coded pin rule (TetMesh.cpp:38-39) selects these
    # nodes; load_tetgen leaves pins to the caller
    rest = m.rest
    rule = np.nonzero((rest[:, 2] > 0) & (rest[:, 1] > np.float32(8.5)))[0]
    assert rule.tolist() == want["pins"]


def test_load_tetgen_equals_reference_build():
    from oracle import ref as R
    d = _model_dir()
    if not R.available():
        pytest.skip("the reference's headless build (oracle/_ref) is not present")
    for rel in ("bar/bar.1", "asiandragon/asiandragon.1"):
        stem = os.path.join(d, rel)
        rest, tets, pins = R.load_model(stem)
        m = M.load_tetgen(stem, scale=0.1, orient=False)
        assert np.array_equal(rest, m.rest) and np.array_equal(tets, m.tets)
