"""Adjoints on the GPU against the oracle's binary64 adjoints.

FP32 accumulation on the device, binary64 on the host; bound: relative error
(2-norm over all outputs) <= 1e-4.  Topology and every discrete integrate
choice come from the FP32 path, which the oracle mirrors bit for bit."""
import numpy as np
import pytest
import torch

from adjoint_util import Scene, rel_err, smooth_volume
from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _canonical_order(mcg, vol_t, cell):
    m = mcg.extract(vol_t, cell, soup=False, normals=False, tri_cube=True)
    tc = m.tri_cube.cpu().numpy()
    order = np.argsort(tc, kind="stable")
    return (order[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)


def _mc_case(mcg, orc, vol_np, cell, seed=0):
    vol_t = torch.from_numpy(vol_np).cuda()
    idx = _canonical_order(mcg, vol_t, cell)  # canonical slot i <- device vertex idx[i]
    n = len(idx)
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((n, 3)).astype(np.float32)
    Gd = np.zeros_like(G)
    Gd[idx] = G
    g_dev = mcg.mc_backward(vol_t, cell, torch.from_numpy(Gd).cuda()).cpu().numpy()
    g64 = orc.mc_backward_f64(vol_np, cell, G.astype(np.float64))
    return g_dev, g64, vol_t, Gd


@pytest.mark.parametrize("n", [24, 64, 128])
def test_mc_backward_float2(mcg, orc, n):
    vol, cell = smooth_volume(n, seed=n)
    g_dev, g64, _, _ = _mc_case(mcg, orc, vol, cell)
    assert np.count_nonzero(g64) > 100
    assert rel_err(g_dev, g64) <= TOL
    # voxels off the surface get exactly nothing
    assert np.array_equal(g_dev != 0, g64 != 0)


def test_mc_backward_short2(mcg, orc):
    vol = synthetic.sphere_volume(48, radius=15.0, trunc=4.0, seed=3)
    g_dev, g64, _, _ = _mc_case(mcg, orc, vol, 0.01)
    assert np.count_nonzero(g64) > 100
    assert rel_err(g_dev, g64) <= TOL


def test_mc_backward_ragged_and_reuse(mcg, orc):
    """odd sizes (partial bricks, no TMA), zero weights; reclassify=False
    reuses the count phase; accumulation into a given grad_f."""
    rng = np.random.default_rng(5)
    vol, cell = smooth_volume(40, seed=7)
    vol = np.ascontiguousarray(vol[:37, :29, :33])
    vol[..., 1][rng.random(vol.shape[:3]) < 0.02] = 0.0
    g_dev, g64, vol_t, Gd = _mc_case(mcg, orc, vol, cell, seed=1)
    assert rel_err(g_dev, g64) <= TOL
    # the count phase of the last call is still the one for vol_t
    acc = torch.from_numpy(g_dev).cuda().clone()
    mcg.mc_backward(vol_t, cell, torch.from_numpy(Gd).cuda(), grad_f=acc, reclassify=False)
    assert rel_err(acc.cpu().numpy(), 2 * g64) <= TOL


def test_mc_backward_linearity_large(mcg):
    """size-independent property at 256^3: the adjoint is linear in dL/dP."""
    vol, cell = smooth_volume(256, seed=11)
    vol_t = torch.from_numpy(vol).cuda()
    n = mcg.extract(vol_t, cell, soup=True, normals=False).num_vertices
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    G1 = torch.randn((n, 3), device="cuda", generator=g)
    G2 = torch.randn((n, 3), device="cuda", generator=g)
    a = mcg.mc_backward(vol_t, cell, G1)
    b = mcg.mc_backward(vol_t, cell, G2)
    c = mcg.mc_backward(vol_t, cell, 2.0 * G1 - 0.5 * G2)
    ref = 2.0 * a.double() - 0.5 * b.double()
    assert float((c.double() - ref).norm() / ref.norm()) <= TOL


def _scene_tensors(sc):
    depth = torch.from_numpy(sc.depth).cuda()
    poses = torch.from_numpy(sc.pose_rows()).cuda()
    return depth, poses


def _normals_np(orc, sc):
    return np.stack([orc.vertex_to_normal(orc.meter_to_vertex(sc.k_orc, sc.depth[f]))
                     for f in range(sc.depth.shape[0])])


@pytest.mark.parametrize("variant", ["plain", "normals", "dynamic"])
def test_integrate_backward(mcg, orc, variant):
    sc = Scene(n=48, frames=4, w=80, h=60, seed=6)
    depth, poses = _scene_tensors(sc)
    k = mcg.intrinsic(sc.fx, sc.fy, sc.cx, sc.cy)
    nrm_np = _normals_np(orc, sc) if variant == "normals" else None
    nrm = torch.from_numpy(nrm_np).cuda() if nrm_np is not None else None
    dyn = variant == "dynamic"
    vol = mcg.integrate_frames(depth, poses, sc.shape, sc.min_t, sc.max_t, sc.grid_s, k, normals=nrm,
                               is_dynamic=dyn)
    # the forward is the FP32 mirror, bit for bit
    ref = np.zeros(sc.shape + (2,), np.float32)
    ref[..., 0] = -1.0
    for f in range(sc.depth.shape[0]):
        orc.integrate(ref, sc.min_t, sc.max_t, sc.grid_s, sc.k_orc, sc.e_orc[f], sc.depth[f],
                      normals=None if nrm_np is None else nrm_np[f], is_dynamic=dyn)
    got = vol.cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    W = ref[..., 1]
    assert (W > 0).mean() > 0.01
    rng = np.random.default_rng(2)
    gF = np.where(W > 0, rng.standard_normal(sc.shape), 0).astype(np.float32)
    gW = np.where(W > 0, 0.1 * rng.standard_normal(sc.shape), 0).astype(np.float32)
    gd, _, _ = mcg.integrate_backward(sc.shape, sc.min_t, sc.max_t, sc.grid_s, k, poses, depth,
                                      torch.from_numpy(gF).cuda(), torch.from_numpy(gW).cuda(), normals=nrm,
                                      is_dynamic=dyn)
    gd64, _, _ = orc.integrate_seq_backward_f64(sc.shape, sc.min_t, sc.max_t, sc.grid_s, sc.k_orc, sc.e_orc,
                                                sc.depth.astype(np.float64), gF.astype(np.float64),
                                                gW.astype(np.float64), normals=nrm_np, is_dynamic=dyn)
    assert np.count_nonzero(gd64) > 100
    assert rel_err(gd.cpu().numpy(), gd64) <= TOL


def test_integrate_backward_initial_volume_and_chunks(mcg, orc):
    """grad of the starting volume, and a sequence split in two calls chained
    through vol0 / grad_f0 / grad_w0 equals the one-call adjoint."""
    sc = Scene(n=40, frames=4, w=80, h=60, seed=8)
    depth, poses = _scene_tensors(sc)
    k = mcg.intrinsic(sc.fx, sc.fy, sc.cx, sc.cy)
    vol = mcg.integrate_frames(depth, poses, sc.shape, sc.min_t, sc.max_t, sc.grid_s, k)
    mid = mcg.integrate_frames(depth[:2], poses[:2], sc.shape, sc.min_t, sc.max_t, sc.grid_s, k)
    W = vol[..., 1].cpu().numpy()
    rng = np.random.default_rng(4)
    gF = torch.from_numpy(np.where(W > 0, rng.standard_normal(sc.shape), 0).astype(np.float32)).cuda()
    full, _, _ = mcg.integrate_backward(sc.shape, sc.min_t, sc.max_t, sc.grid_s, k, poses, depth, gF)
    g2 = torch.zeros_like(depth)
    _, gf_mid, gw_mid = mcg.integrate_backward(sc.shape, sc.min_t, sc.max_t, sc.grid_s, k, poses[2:], depth[2:], gF,
                                               vol0=mid, grad_depth=g2[2:], want_grad_vol0=True)
    mcg.integrate_backward(sc.shape, sc.min_t, sc.max_t, sc.grid_s, k, poses[:2], depth[:2], gf_mid, gw_mid,
                           grad_depth=g2[:2])
    assert rel_err(g2.cpu().numpy(), full.cpu().numpy()) <= TOL
    # against binary64, with the starting volume
    gd64, gF0, gW0 = orc.integrate_seq_backward_f64(sc.shape, sc.min_t, sc.max_t, sc.grid_s, sc.k_orc,
                                                    sc.e_orc[2:], sc.depth[2:].astype(np.float64),
                                                    gF.cpu().numpy().astype(np.float64), None,
                                                    vol0=mid.cpu().numpy())
    assert rel_err(gf_mid.cpu().numpy(), gF0) <= TOL
    assert rel_err(gw_mid.cpu().numpy(), gW0) <= TOL


def test_autograd_chain(mcg, orc):
    """depth -> integrate_frames -> mesh_positions -> L = sum G . P, through
    torch.autograd, against the binary64 adjoint chain."""
    sc = Scene(n=48, frames=3, w=80, h=60, seed=9)
    depth, poses = _scene_tensors(sc)
    k = mcg.intrinsic(sc.fx, sc.fy, sc.cx, sc.cy)
    d = depth.clone().requires_grad_(True)
    vol = mcg.integrate_frames(d, poses, sc.shape, sc.min_t, sc.max_t, sc.grid_s, k)
    pos = mcg.mesh_positions(vol, sc.grid_s)
    n = pos.shape[0]
    assert n > 300
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    G = torch.randn((n, 3), device="cuda", generator=g)
    (pos * G).sum().backward()
    vol_np = vol.detach().cpu().numpy()
    idx = _canonical_order(mcg, vol.detach().contiguous(), sc.grid_s)
    G_can = G.cpu().numpy()[idx].astype(np.float64)
    gF = orc.mc_backward_f64(vol_np, sc.grid_s, G_can)
    gd64, _, _ = orc.integrate_seq_backward_f64(sc.shape, sc.min_t, sc.max_t, sc.grid_s, sc.k_orc, sc.e_orc,
                                                sc.depth.astype(np.float64), gF, None)
    assert np.count_nonzero(gd64) > 100
    assert rel_err(d.grad.cpu().numpy(), gd64) <= TOL


def test_autograd_volume_leaf(mcg, orc):
    """gradient into a leaf float32 volume through mesh_positions, and into
    the starting volume through integrate_frames."""
    vol, cell = smooth_volume(32, seed=12)
    v = torch.from_numpy(vol).cuda().requires_grad_(True)
    pos = mcg.mesh_positions(v, cell)
    G = torch.ones_like(pos)
    (pos * G).sum().backward()
    idx = _canonical_order(mcg, v.detach(), cell)
    g64 = orc.mc_backward_f64(vol, cell, G.cpu().numpy()[idx].astype(np.float64))
    assert rel_err(v.grad[..., 0].cpu().numpy(), g64) <= TOL
    assert not v.grad[..., 1].any()


def test_blended_spheres_full_size(mcg, orc):
    """The differentiable-fusion workload at its full size: 10 sphere-traced
    320x240 frames (f 262.5) of 8 blended spheres -> 256^3 float32 volume ->
    soup positions P -> L = sum phi(P)^2 (phi the analytic field); the
    autograd gradient w.r.t. every depth pixel against the binary64 adjoint
    chain fed the same dL/dP."""
    scene = synthetic.BlendedSpheres(seed=0)
    w, h, f, n, frames = 320, 240, 262.5, 256, 10
    depth64, poses = scene.frames(frames, w=w, h=h, fx=f, fy=f, device="cuda")
    depth = depth64.to(torch.float32).contiguous()
    k = mcg.intrinsic(f, f, (w - 1) / 2.0, (h - 1) / 2.0)
    pt = torch.stack([mcg.extrinsic_tensor(R, t) for R, t in poses]).contiguous()
    shape, gs = (n, n, n), 1.0 / n
    trunc = 4 * gs
    d = depth.clone().requires_grad_(True)
    vol = mcg.integrate_frames(d, pt, shape, trunc, trunc, gs, k)
    pos = mcg.mesh_positions(vol, gs)
    assert pos.shape[0] > 100000
    pos.retain_grad()
    (scene.sdf(pos) ** 2).sum().backward()
    G = pos.grad
    vol_np = vol.detach().cpu().numpy()
    idx = _canonical_order(mcg, vol.detach().contiguous(), gs)
    gF = orc.mc_backward_f64(vol_np, gs, G.cpu().numpy()[idx].astype(np.float64))
    k_orc = orc.intrinsic(f, f, (w - 1) / 2.0, (h - 1) / 2.0)
    e_orc = [orc.extrinsic(R, t) for R, t in poses]
    gd64, _, _ = orc.integrate_seq_backward_f64(shape, trunc, trunc, gs, k_orc, e_orc,
                                                depth.cpu().numpy().astype(np.float64), gF, None)
    assert np.count_nonzero(gd64) > 10000
    assert rel_err(d.grad.cpu().numpy(), gd64) <= TOL
