"""The 512^3 fusion workload at full size: the exact inputs of bench.py's
headline volume (60 seeded 640x480 depth frames of the 20-sphere + box
scene integrated into a 512^3 short2 volume over a 3 m cube, truncation
0.03 m), integrated on the GPU and by the oracle, compared bit for bit after
every frame's metre map and after the last frame's volume; then the
extraction of that volume, with every output of the reference's run() (soup,
normals, vi2vox, ver_voxel) and the cube ids, compared with the oracle's.

Reference: cu_kinect_fusion_v1.cu:99-112 (depth -> metre), :427-532
(integrate), cu_marching_cubes_v1.cu:416-467 (MarchingCubes::run)."""
import numpy as np
import pytest
import torch

import bench
from marching_cube_gb300 import synthetic
from mc_util import assert_same_mesh, gpu_extract

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fused(mcg, orc):
    n = bench.N_VOX
    grid_s = bench.EXTENT / n
    v = mcg.voxel_new((n, n, n), bench.TRUNC, bench.TRUNC, grid_s)
    ref = orc.voxel_init(n ** 3).reshape(n, n, n, 2)
    k = mcg.intrinsic(bench.FX, bench.FY, bench.CX, bench.CY)
    ko = orc.intrinsic(bench.FX, bench.FY, bench.CX, bench.CY)
    for R, t, d in bench.fusion_frames(synthetic, bench.N_FRAMES, seed=0):
        m, _, _ = mcg.depth_to_maps(d, k, vertex=False, normal=False)
        mcg.volumetric_integration(v, k, mcg.extrinsic(R, t), m)
        mo = orc.depth_to_meter(d.cpu().numpy().view(np.uint16))
        assert np.array_equal(m.cpu().numpy().view(np.uint32), mo.view(np.uint32))
        orc.integrate(ref, bench.TRUNC, bench.TRUNC, grid_s, ko, orc.extrinsic(R, t), mo)
    torch.cuda.synchronize()
    yield v, ref, grid_s
    del v
    torch.cuda.empty_cache()


def test_fused_volume_matches_oracle(fused):
    v, ref, _ = fused
    got = v.data.cpu().numpy()
    diff = (got.reshape(-1, 2) != ref.reshape(-1, 2)).any(axis=1)
    assert int(diff.sum()) == 0, int(diff.sum())
    # the fusion observed the scene: a surface band of updated voxels
    assert (ref[..., 1] != 0).mean() > 0.01


def test_fused_extraction_matches_oracle(mcg, orc, fused):
    v, ref, cell = fused
    g = gpu_extract(mcg, ref, cell)
    o = orc.mc_extract(ref, cell)
    assert g["counts"]["triangles"] > 500000
    assert_same_mesh(g, o)
    # the headline step's configuration (soup + normals only) writes the
    # same soup and normals as the full output set
    mesh = mcg.extract(v.data, cell, soup=True, normals=True)
    torch.cuda.synchronize()
    full = mcg.extract(v.data, cell, soup=True, normals=True, tri_cube=True)
    torch.cuda.synchronize()
    assert torch.equal(mesh.soup, full.soup) and torch.equal(mesh.normals, full.normals)
