"""The benchmark's input generator without a GPU: configuration 2's blob
isosurface (marching cubes on the seeded Gaussian field, torch on the CPU),
its grid attributes and its voxelization by the oracle give the same grid
as the CUDA path that produced tests/golden/bench_manifest.json (digest,
triangle count, data extent)."""
import hashlib
import json
import os

import numpy as np

from broxy_gb300 import synth
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bench_manifest.json")


def test_config2_input_grid_matches_manifest():
    m = json.load(open(GOLDEN))["blob_512_uniform_12"]
    res, seed = m["res"], m["seed"]
    assert seed == synth.CONFIGS[2]["seed"]
    P, T = synth.blob_mesh(synth.mesh_samples(2, res), seed, count=200, device="cpu")
    P, T = P.numpy(), T.numpy().astype(np.uint32)
    assert len(T) == m["input_triangles"]
    bmin, _, cell, data_res = O.grid_attributes(P, res, synth.MESH_MARGIN)
    assert [int(v) for v in data_res] == m["data_res"]
    X = O.voxelize(P, T, res, bmin, cell)
    assert hashlib.sha256(np.ascontiguousarray(X).tobytes()).hexdigest() == m["X"]
