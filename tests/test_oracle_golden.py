"""The CPU oracle (integer restatement of the reference) against the golden
fixtures of tests/golden/, which a float32 transliteration of the reference
kernels produced (tests/golden/gen_golden.py): pyramid traversals, contour
taggers, the GM_REF update sequence and the contour marching cubes.
Bit-exact for the grids and the triangle indices; vertices within 1e-6
relative (float32)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(HERE, "manifest.json")))


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_closing_matches_reference_transliteration(name):
    case = MANIFEST[name]
    g = np.load(os.path.join(HERE, name + ".npz"))
    res = case["res"]
    D, S, C = O.close(g["X"], res, case["data_res"], g["scale"], 0, 1 if case["cube"] else 0)
    assert np.array_equal(D, g["D"])
    assert np.array_equal(S, g["S"])
    assert np.array_equal(C, g["C"])


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_mc_matches_reference_transliteration(name):
    g = np.load(os.path.join(HERE, name + ".npz"))
    res = MANIFEST[name]["res"]
    V, T = O.mc(g["C"], res, np.array([0.25, -0.5, 1.0], np.float32), 0.0625)
    assert np.array_equal(T, g["T"])
    np.testing.assert_allclose(V, g["V"], rtol=1e-6, atol=0)


def test_fixtures_are_nontrivial():
    for name, case in MANIFEST.items():
        assert case["nt"] > 100, name
