"""The batched workload at full size: 64 volumes with edges log-uniform in
[32, 256] per axis (1-8 spheres / boxes each, seed 7: the volumes bench.py
times), extracted in one batched call with every output of the reference's
run() (soup, normals, vi2vox, ver_voxel) and the cube ids, and each volume
compared bit for bit with the oracle's extraction of that volume.

Reference: the per-volume loop of cu_kinect_fusion_v1.cu:3511-3737
(cu_voxel_to_mesh: MarchingCubes::run + normals per volume)."""
import pytest
import torch

from marching_cube_gb300 import synthetic
from mc_util import assert_same_mesh, mesh_arrays

pytestmark = pytest.mark.gpu


def test_batched_64_volumes_match_oracle(mcg, orc):
    vols = synthetic.batch_volumes(64, seed=7, lo=32, hi=256, device="cuda")
    cells = [0.01] * len(vols)
    meshes = mcg.extract_batched(vols, cells, soup=True, normals=True, vi2vox=True, ver_voxel=True,
                                 tri_cube=True)
    torch.cuda.synchronize()
    total = 0
    for v, c, m in zip(vols, cells, meshes):
        g = mesh_arrays(m)
        o = orc.mc_extract(v.cpu().numpy(), c)
        assert_same_mesh(g, o)
        total += m.num_triangles
    assert total > 1000000
