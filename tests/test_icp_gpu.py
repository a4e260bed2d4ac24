"""Depth pyramid and ICP on the GPU against the oracle: the pyramid step,
the masks and one correspondence pass (v21, A, b, inlier) bit-exact; the
whole ICP loop with the same outcome and iterations and the pose within
1e-5 (the normal equations are binary64 sums in another order); tracking
recovers the known relative pose at 640 x 480."""
import math

import numpy as np
import pytest
import torch

import oracle
from icp_util import frames, pyramid_maps, rot_angle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mcg():
    import marching_cube_gb300 as m
    return m


@pytest.fixture(scope="module")
def scene_maps():
    d1, d2, rel, (f, cx, cy) = frames(seed=1, step=1)
    return d1, d2, rel, pyramid_maps(d1, f, cx, cy), pyramid_maps(d2, f, cx, cy)


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_pyramid_and_masks(mcg, scene_maps):
    d1 = scene_maps[0].copy()
    d1[::7, ::5] = 0.0  # holes
    m = mcg.float_data_to_mask(cu(d1))
    assert np.array_equal(m.cpu().numpy(), oracle.float_data_to_mask(d1))
    for sigma in (0.06, 0.005):
        d, dm = mcg.pyramid_down(cu(d1), m, sigma=sigma)
        od, odm = oracle.pyramid_down(d1, oracle.float_data_to_mask(d1), (60, 80), sigma)
        assert np.array_equal(dm.cpu().numpy(), odm)
        assert np.array_equal(d.cpu().numpy().view(np.uint32), od.view(np.uint32))
    x = cu(d1)
    mcg.float_mask_to_data(cu(np.where(d1 > 0.7, 255, 0).astype(np.uint8)), x)
    assert np.array_equal(x.cpu().numpy(), oracle.float_mask_to_data(np.where(d1 > 0.7, 255, 0), d1))


@pytest.mark.parametrize("bilinear", [False, True])
def test_correspond_bit_exact(mcg, scene_maps, bilinear):
    _, _, (R, t), m1, m2 = scene_maps
    v1, n1, k, _ = m1[0]
    v2, n2, _, _ = m2[0]
    nt, dt = math.cos(math.radians(20)), 0.10
    for RR, tt in ((np.eye(3), np.zeros(3)), (R, t + 0.003)):
        e = oracle.extrinsic(RR, tt)
        ov21, oA, ob, oin = oracle.icp_correspond(nt, dt, k, e, v1, n1, v2, n2, bilinear)
        p = mcg.icp_params(1, bilinear)
        g = mcg.icp_correspond(p, mcg.intrinsic(k.fx, k.fy, k.cx, k.cy), mcg.extrinsic(RR, tt), cu(v1), cu(n1),
                               cu(v2), cu(n2))
        assert np.array_equal(g["inlier"].cpu().numpy(), oin)
        assert oin.sum() > 1000 * 255
        assert np.array_equal(g["v21"].cpu().numpy().view(np.uint32), ov21.view(np.uint32))
        assert np.array_equal(g["A"].cpu().numpy().view(np.uint32), oA.view(np.uint32))
        assert np.array_equal(g["b"].cpu().numpy().view(np.uint32), ob.view(np.uint32))


@pytest.mark.parametrize("bilinear", [False, True])
def test_icp_loop_matches_oracle(mcg, scene_maps, bilinear):
    _, _, (R, t), m1, m2 = scene_maps
    e = oracle.extrinsic(np.eye(3), np.zeros(3))
    ge = mcg.extrinsic(np.eye(3), np.zeros(3))
    for lv, it_max in ((2, 8), (1, 11), (0, 15)):
        v1, n1, k, _ = m1[lv]
        v2, n2, _, _ = m2[lv]
        ok, (r, tt), iters, oin = oracle.icp(math.cos(math.radians(20)), 0.10, math.radians(20), 0.10, it_max, k, e,
                                             v1, n1, v2, n2, bilinear)
        inl = torch.zeros(v1.shape[:2], dtype=torch.uint8, device="cuda")
        gok, ge, giters = mcg.icp(mcg.icp_params(it_max, bilinear), mcg.intrinsic(k.fx, k.fy, k.cx, k.cy), ge,
                                  cu(v1), cu(n1), cu(v2), cu(n2), inlier=inl)
        assert gok == ok and giters == iters, (lv, iters, giters)
        assert np.allclose(np.array(list(ge.r)), r, atol=1e-5) and np.allclose(np.array(list(ge.t)), tt, atol=1e-5)
        if np.array_equal(np.array(list(ge.r), np.float32), r) and np.array_equal(np.array(list(ge.t), np.float32), tt):
            assert np.array_equal(inl.cpu().numpy(), oin)
        e = oracle.Extrinsic()
        for i in range(9):
            e.r[i] = float(r[i])
        for i in range(3):
            e.t[i] = float(tt[i])
    Re = np.array(list(ge.r)).reshape(3, 3).T
    assert rot_angle(Re.T @ R) < 2e-3 and np.linalg.norm(np.array(list(ge.t)) - t) < 2e-3


def test_icp_pyramid_640(mcg):
    """Tracking at full size: depth, masks, pyramid, maps and ICP all on the
    GPU (icp_pyramid: 3 levels, 8 / 11 / 15 iterations)."""
    from marching_cube_gb300 import synthetic
    from icp_util import rel_pose
    scene = synthetic.BlendedSpheres(seed=3)
    w, h, f = 640, 480, 525.0
    k0 = mcg.intrinsic(f, f, 319.5, 239.5)
    P1, P2 = scene.pose(0, 200), scene.pose(1, 200)
    R, t = rel_pose(P1, P2)
    maps = []
    for P in (P1, P2):
        d = scene.depth_frame(*P, w=w, h=h, fx=f, fy=f, cx=319.5, cy=239.5, device="cuda").float().contiguous()
        lv, k = [], k0
        for i in range(3):
            if i > 0:
                m = mcg.float_data_to_mask(d)
                d, dm = mcg.pyramid_down(d, m)
                mcg.float_mask_to_data(dm, d)
                k = mcg.intrinsic_pyramid_down(k)
            v = mcg.meter_to_vertex(d, k)
            lv.append((v, mcg.vertex_to_normal(v)))
        maps.append(lv)
    inl = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
    ok, e, iters = mcg.icp_pyramid(k0, mcg.extrinsic(np.eye(3), np.zeros(3)), maps[0], maps[1], inlier=inl)
    assert ok and len(iters) == 3
    Re = np.array(list(e.r)).reshape(3, 3).T
    assert rot_angle(Re.T @ R) < 1e-3 and np.linalg.norm(np.array(list(e.t)) - t) < 1e-3
    # inliers: level-0 pixels with a match, all of them with a valid normal
    assert int((inl == 255).sum()) > 20000 and bool(((inl == 255) <= (maps[0][0][1].abs().sum(-1) > 0)).all())
