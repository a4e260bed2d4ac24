"""The oracle against the fixtures the reference's own source produced
(tests/golden/ref/): extraction with every output, depth maps, voxel
initialisation + integration of three frames, RLE slices -- bit for bit."""
import numpy as np
import pytest

from ref_golden_util import load, mesh_cases, poses


def _same_mesh(o, g):
    n = len(g["soup"])
    assert len(o["soup"]) == n
    assert np.array_equal(o["soup"].view(np.uint8).reshape(-1, 28), g["soup"])
    assert np.array_equal(o["normals"].view(np.uint32), g["normals"].view(np.uint32))
    assert np.array_equal(o["vi2vox"], g["vi2vox"])
    assert np.array_equal(o["ver_voxel"].reshape(-1), g["ver_voxel"].reshape(-1))


@pytest.mark.parametrize("name", mesh_cases())
def test_oracle_extraction_matches_reference_fixture(orc, name):
    g = load(name)
    _same_mesh(orc.mc_extract(g["vol"], float(g["cell"])), g)


def test_oracle_fusion_chain_matches_reference_fixture(orc):
    g = load("fusion_48.npz")
    fx, fy, cx, cy = (float(x) for x in g["intrinsic"])
    k = orc.intrinsic(fx, fy, cx, cy)
    m0 = orc.depth_to_meter(g["depth"][0])
    assert np.array_equal(m0.view(np.uint32), g["meter0"].view(np.uint32))
    v0 = orc.meter_to_vertex(k, m0)
    assert np.array_equal(v0.view(np.uint32), g["vertex0"].view(np.uint32))
    assert np.array_equal(orc.vertex_to_normal(v0).view(np.uint32), g["normal0"].view(np.uint32))
    n = g["vol"].shape[0]
    vol = orc.voxel_init(n ** 3).reshape(n, n, n, 2)
    trunc, grid_s = float(g["trunc"]), float(g["grid_s"])
    for d, (R, t) in zip(g["depth"], poses(g)):
        orc.integrate(vol, trunc, trunc, grid_s, k, orc.extrinsic(R, t), orc.depth_to_meter(d))
    assert np.array_equal(vol, g["vol"])
    enc = [orc.rle_encode_slice(s) for s in vol.reshape(n, -1, 2)]
    assert np.array_equal(np.array([len(e) for e in enc]), g["rle_sizes"])
    assert np.array_equal(np.frombuffer(b"".join(enc), np.uint8), g["rle"])
    _same_mesh(orc.mc_extract(vol, grid_s), g)
