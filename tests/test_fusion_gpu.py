"""Parity of the CUDA fusion kernels (voxel init, depth -> metre / vertex /
normal maps, integrate) with the CPU oracle, bit-exact."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _frames(n_frames, w, h, f, extent=3.0, seed=0):
    scene = synthetic.FusionScene(seed=seed, extent=extent)
    cx, cy = (w - 1) / 2.0, (h - 1) / 2.0
    out = []
    for i in range(n_frames):
        R, t = scene.pose(i, n_frames)
        mm = scene.depth_frame(R, t, w=w, h=h, fx=f, fy=f, cx=cx, cy=cy, seed=seed * 1000 + i)
        out.append((R, t, mm))
    return out, (f, f, cx, cy)


def test_voxel_init(mcg, orc):
    v = mcg.voxel_new((37, 5, 3), 0.03, 0.03, 0.01)
    ref = orc.voxel_init(37 * 5 * 3)
    assert np.array_equal(v.data.cpu().numpy().reshape(-1, 2), ref)
    f = mcg.voxel_new((10, 3, 3), 0.03, 0.03, 0.01, dtype=torch.float32)
    assert (f.data[..., 0] == -1.0).all() and (f.data[..., 1] == 0).all()
    # misaligned start (tail path)
    big = torch.zeros(1001 * 2, dtype=torch.int16, device="cuda")
    view = big[2:].view(1000, 1, 1, 2)
    mcg.voxel_init(view)
    assert np.array_equal(view.cpu().numpy().reshape(-1, 2), orc.voxel_init(1000))
    assert int(big[0]) == 0 and int(big[1]) == 0


def test_depth_maps(mcg, orc):
    frames, (fx, fy, cx, cy) = _frames(2, 160, 120, 131.25)
    for R, t, mm in frames:
        mm_np = mm.numpy().astype(np.uint16)
        mm_np[5, 7] = 2001   # just beyond the 2 m range
        mm_np[6, 9] = 40000  # far out of range (negative as the reference's short)
        d = torch.from_numpy(mm_np.view(np.int16)).cuda()
        k = mcg.intrinsic(fx, fy, cx, cy)
        m, v, n = mcg.depth_to_maps(d, k)
        ko = orc.intrinsic(fx, fy, cx, cy)
        mo = orc.depth_to_meter(mm_np)
        vo = orc.meter_to_vertex(ko, mo)
        no = orc.vertex_to_normal(vo)
        assert np.array_equal(m.cpu().numpy().view(np.uint32), mo.view(np.uint32))
        assert np.array_equal(v.cpu().numpy().view(np.uint32), vo.view(np.uint32))
        assert np.array_equal(n.cpu().numpy().view(np.uint32), no.view(np.uint32))
        assert (mo > 0).mean() > 0.3
        # the unfused entry points give the same maps
        v2 = mcg.meter_to_vertex(m, k)
        n2 = mcg.vertex_to_normal(v2)
        assert torch.equal(v2, v) and torch.equal(n2, n)


def test_plane_normal_known_answer(mcg):
    # fronto-parallel plane at 1.2 m: every interior normal is (0, 0, -1)
    w, h = 64, 48
    d = torch.full((h, w), 1200, dtype=torch.int16, device="cuda")
    m, v, n = mcg.depth_to_maps(d, mcg.intrinsic(60.0, 60.0, 31.5, 23.5))
    nn = n.cpu().numpy()
    assert np.allclose(nn[:-1, :-1], [0.0, 0.0, -1.0], atol=1e-6)
    assert (nn[-1] == 0).all() and (nn[:, -1] == 0).all()
    assert np.allclose(m.cpu().numpy(), 1.2)


@pytest.mark.parametrize("vtype,use_normals,dynamic", [(torch.int16, False, False), (torch.int16, True, False),
                                                       (torch.int16, False, True), (torch.float32, False, False),
                                                       (torch.float32, True, True)])
def test_integrate_parity(mcg, orc, vtype, use_normals, dynamic):
    n = 72
    extent = 3.0
    grid_s = extent / n
    trunc = 0.09
    frames, (fx, fy, cx, cy) = _frames(3, 160, 120, 131.25, extent=extent, seed=1)
    v = mcg.voxel_new((n, n, n), trunc, trunc, grid_s, dtype=vtype)
    ref = v.data.cpu().numpy().copy()
    k = mcg.intrinsic(fx, fy, cx, cy)
    ko = orc.intrinsic(fx, fy, cx, cy)
    for R, t, mm in frames:
        mm_np = mm.numpy().astype(np.uint16)
        d = torch.from_numpy(mm_np.view(np.int16)).cuda()
        m, _, nrm = mcg.depth_to_maps(d, k, vertex=False, normal=use_normals)
        e = mcg.extrinsic(R, t)
        mcg.volumetric_integration(v, k, e, m, normals=nrm if use_normals else None, is_dynamic=dynamic)
        mo = orc.depth_to_meter(mm_np)
        no = orc.vertex_to_normal(orc.meter_to_vertex(ko, mo)) if use_normals else None
        orc.integrate(ref, trunc, trunc, grid_s, ko, orc.extrinsic(R, t), mo, normals=no, is_dynamic=dynamic)
        got = v.data.cpu().numpy()
        diff = (got.view(np.uint32) != ref.view(np.uint32)).reshape(-1) if vtype == torch.float32 else \
            (got.reshape(-1, 2) != ref.reshape(-1, 2)).any(axis=1)
        assert int(diff.sum()) == 0, int(diff.sum())
    # the fusion actually observed surfaces
    w = ref[..., 1]
    assert (w != 0).mean() > 0.02


def test_integrate_then_extract(mcg, orc):
    n = 64
    extent = 3.0
    frames, (fx, fy, cx, cy) = _frames(4, 160, 120, 131.25, extent=extent, seed=2)
    v = mcg.voxel_new((n, n, n), 0.1, 0.1, extent / n)
    k = mcg.intrinsic(fx, fy, cx, cy)
    for R, t, mm in frames:
        d = torch.from_numpy(mm.numpy().astype(np.uint16).view(np.int16)).cuda()
        m, _, _ = mcg.depth_to_maps(d, k, vertex=False, normal=False)
        mcg.volumetric_integration(v, k, mcg.extrinsic(R, t), m)
    mesh = mcg.MarchingCubes().run(v)
    o = orc.mc_extract(v.data.cpu().numpy(), v.grid_s)
    assert mesh.num_vertices == len(o["soup"]) > 0
