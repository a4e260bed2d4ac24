"""The CUDA library against the fixtures the reference's own source produced
(tests/golden/ref/, made where the reference tree is present): extraction
with every output, depth maps, voxel initialisation + integration of three
frames, the RLE image of the integrated volume -- bit for bit."""
import numpy as np
import pytest
import torch

from mc_util import gpu_extract
from ref_golden_util import load, mesh_cases, poses, rle_body

pytestmark = pytest.mark.gpu


def _same_mesh(out, g):
    assert len(out["soup"]) == len(g["soup"])
    assert np.array_equal(out["soup"].view(np.uint8).reshape(-1, 28), g["soup"])
    assert np.array_equal(out["normals"].view(np.uint32), g["normals"].view(np.uint32))
    assert np.array_equal(out["vi2vox"], g["vi2vox"])
    assert np.array_equal(out["ver_voxel"].reshape(-1), g["ver_voxel"].reshape(-1))


@pytest.mark.parametrize("name", mesh_cases())
def test_gpu_extraction_matches_reference_fixture(mcg, name):
    g = load(name)
    _same_mesh(gpu_extract(mcg, g["vol"], float(g["cell"])), g)


def test_gpu_fusion_chain_matches_reference_fixture(mcg):
    g = load("fusion_48.npz")
    fx, fy, cx, cy = (float(x) for x in g["intrinsic"])
    k = mcg.intrinsic(fx, fy, cx, cy)
    n = g["vol"].shape[0]
    trunc, grid_s = float(g["trunc"]), float(g["grid_s"])
    v = mcg.voxel_new((n, n, n), trunc, trunc, grid_s)
    for i, (d, (R, t)) in enumerate(zip(g["depth"], poses(g))):
        dt = torch.from_numpy(d.view(np.int16)).cuda()
        m, vert, nrm = mcg.depth_to_maps(dt, k)
        if i == 0:
            assert np.array_equal(m.cpu().numpy().view(np.uint32), g["meter0"].view(np.uint32))
            assert np.array_equal(vert.cpu().numpy().view(np.uint32), g["vertex0"].view(np.uint32))
            assert np.array_equal(nrm.cpu().numpy().view(np.uint32), g["normal0"].view(np.uint32))
        mcg.volumetric_integration(v, k, mcg.extrinsic(R, t), m)
    torch.cuda.synchronize()
    assert np.array_equal(v.data.cpu().numpy(), g["vol"])
    sizes, body = rle_body(mcg.rle_encode(v), n)
    assert np.array_equal(sizes, g["rle_sizes"]) and np.array_equal(body, g["rle"])
    _same_mesh(gpu_extract(mcg, g["vol"], grid_s), g)
