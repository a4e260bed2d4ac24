"""Ray casting on the GPU against the oracle's restatement, bit for bit:
analytic planes, a fused scene from cameras outside and inside the volume,
the 512^3 fusion volume at 640x480, a singular camera."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic
from test_raycast_oracle import _plane_volume

pytestmark = pytest.mark.gpu


def _check(mcg, orc, vol_np, grid_s, K, R, t, w, h):
    vol = torch.from_numpy(np.ascontiguousarray(vol_np)).cuda()
    v = mcg.Voxel(vol, 0.03, 0.03, grid_s)
    d, n = mcg.raycast(v, mcg.intrinsic(*K), mcg.extrinsic(R, t), w, h)
    torch.cuda.synchronize()
    ref = orc.raycast(vol_np, grid_s, orc.intrinsic(*K), orc.extrinsic(R, t), w, h)
    assert ref is not None
    assert np.array_equal(d.cpu().numpy().view(np.uint32), ref[0].view(np.uint32))
    assert np.array_equal(n.cpu().numpy().view(np.uint32), ref[1].view(np.uint32))
    return ref


def test_planes(mcg, orc):
    K = (40.0, 40.0, 15.5, 15.5)
    d, _ = _check(mcg, orc, _plane_volume(), 0.01, K, np.eye(3), [0.32, 0.32, 0.02], 32, 32)
    assert (d > 0).all()
    R = np.stack([[0, 0, -1.0], [0, 1.0, 0], [1.0, 0, 0]], axis=1)
    _check(mcg, orc, _plane_volume(axis=0), 0.01, K, R, [0.05, 0.32, 0.32], 32, 32)


@pytest.fixture(scope="module")
def fused(mcg):
    n, extent = 128, 3.0
    scene = synthetic.FusionScene(seed=11, extent=extent)
    v = mcg.voxel_new((n, n, n), 0.09, 0.09, extent / n)
    k = mcg.intrinsic(131.25, 131.25, 79.5, 59.5)
    for i in range(8):
        R, t = scene.pose(i, 8)
        mm = synthetic.mm_to_u16_bits(scene.depth_frame(R, t, w=160, h=120, fx=131.25, fy=131.25, cx=79.5,
                                                        cy=59.5, seed=i, device="cuda"))
        meter = mcg.depth_to_maps(mm, k, vertex=False, normal=False)[0]
        mcg.volumetric_integration(v, k, mcg.extrinsic(R, t), meter)
    torch.cuda.synchronize()
    return v.data.cpu().numpy(), extent / n, scene


def test_fused_scene(mcg, orc, fused):
    vol_np, g, scene = fused
    hits = 0
    for i in range(0, 16, 3):
        R, t = scene.pose(i, 16)
        d, _ = _check(mcg, orc, vol_np, g, (131.25, 131.25, 79.5, 59.5), R, t, 160, 120)
        hits += int((d > 0).sum())
    assert hits > 10000
    # a camera inside the volume, looking along a diagonal
    R, _ = scene.pose(3, 16)
    _check(mcg, orc, vol_np, g, (131.25, 131.25, 79.5, 59.5), R, scene.center + 0.3, 160, 120)


def test_fusion_512_full_size(mcg, orc):
    import bench
    v, _ = bench.build_volume(mcg, synthetic, torch, 512, 60, seed=0)
    vol_np = v.data.cpu().numpy()
    scene = synthetic.FusionScene(seed=0, extent=bench.EXTENT)
    R, t = scene.pose(5, 60)
    d, _ = _check(mcg, orc, vol_np, v.grid_s, (bench.FX, bench.FY, bench.CX, bench.CY), R, t, bench.W, bench.H)
    assert (d > 0).mean() > 0.2


def test_singular_camera_writes_nothing(mcg):
    vol = torch.from_numpy(_plane_volume()).cuda()
    v = mcg.Voxel(vol, 0.03, 0.03, 0.01)
    d = torch.full((8, 8), 7.0, device="cuda")
    n = torch.full((8, 8, 3), 7.0, device="cuda")
    mcg.raycast(v, mcg.intrinsic(0.0, 40.0, 15.5, 15.5), mcg.extrinsic(np.eye(3), [0.3, 0.3, 0.0]), 8, 8,
                out_depth=d, out_normal=n)
    assert (d == 7.0).all() and (n == 7.0).all()
