"""Indexed extraction on the GPU against the oracle: the vertex set is the
set of grid edges the soup uses, each exactly once; triangles are the soup's
(order, winding) as vertex indices; positions, normals and voxels of the
vertices are bit-exact with the oracle's lower -> upper interpolation."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _check(mcg, orc, vol_np, cell):
    vol = torch.from_numpy(np.ascontiguousarray(vol_np)).cuda()
    m = mcg.extract_indexed(vol, cell, normals=True, vi2vox=True, vertex_edge=True, tri_cube=True)
    torch.cuda.synchronize()
    keys, tri_keys = orc.mc_indexed(vol_np)
    nv, nt = m.num_vertices, m.num_triangles
    assert nv == len(keys) and nt == len(tri_keys)
    if nt == 0:
        return m
    ve = m.vertex_edge.cpu().numpy()
    assert len(np.unique(ve)) == nv
    assert np.array_equal(np.sort(ve), keys)
    tri = m.triangles.cpu().numpy().astype(np.int64)
    assert tri.min() >= 0 and tri.max() < nv
    tc = m.tri_cube.cpu().numpy()
    order = np.argsort(tc, kind="stable")
    assert np.array_equal(ve[tri[order]], tri_keys)
    # soup order: the indexed triangles follow the soup's triangles one to one
    soup = mcg.extract(vol, cell, soup=False, normals=False, tri_cube=True)
    assert np.array_equal(soup.tri_cube.cpu().numpy(), tc)
    pos, nrm, v2v = orc.mc_edge_vertices(vol_np, cell, ve)
    assert np.array_equal(m.positions.cpu().numpy().view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(m.normals.cpu().numpy().view(np.uint32), nrm.view(np.uint32))
    assert np.array_equal(m.vi2vox.cpu().numpy(), v2v)
    return m


@pytest.mark.parametrize("n", [33, 48, 64, 65])
def test_sphere(mcg, orc, n):
    vol = synthetic.sphere_volume(n, radius=n * 0.3, trunc=4.0, seed=n)
    m = _check(mcg, orc, vol, 0.01)
    # closed 2-manifold: V - E + F = 2
    tri = m.triangles.cpu().numpy().astype(np.int64)
    e = np.sort(np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]]), axis=1)
    assert m.num_vertices - len(np.unique(e, axis=0)) + m.num_triangles == 2


@pytest.mark.parametrize("shape", [(9, 17, 65), (17, 9, 40), (33, 33, 33), (2, 2, 2), (6, 7, 9), (41, 10, 97)])
def test_random_and_ragged(mcg, orc, shape):
    vol = synthetic.random_volume(shape, seed=sum(shape))
    _check(mcg, orc, vol, 0.02)


def test_corner_sphere_and_float2(mcg, orc):
    # surface through the volume faces and edges (last-brick ownership)
    vol = synthetic.sphere_volume(65, radius=40.0, trunc=4.0, seed=2, center=(0.0))
    _check(mcg, orc, vol, 0.01)
    f = synthetic.sphere_volume(72, radius=20.0, trunc=4.0, seed=3)
    f32 = np.stack([f[..., 0].astype(np.float32) / 32766.0, (f[..., 1] != 0).astype(np.float32)], axis=-1)
    _check(mcg, orc, f32, 0.01)


def test_capacity_and_state(mcg, orc):
    vol = torch.from_numpy(synthetic.sphere_volume(48, radius=14.0, trunc=4.0)).cuda()
    ctx = mcg.Context()
    full = mcg.extract_indexed(vol, 0.01, ctx=ctx, vertex_edge=True)
    nv, nt = full.num_vertices, full.num_triangles
    out = {"positions": torch.zeros((nv // 2, 3), device="cuda"),
           "triangles": torch.zeros((nt // 2, 3), dtype=torch.int32, device="cuda")}
    mcg.extract_indexed_into(vol, 0.01, out, nv // 2, nt // 2, ctx=ctx)
    import ctypes
    c = mcg._capi.MeshCounts()
    assert mcg._lib.mcg_mc_counts(ctx.handle, ctypes.byref(c)) == mcg.MCG_ERR_CAPACITY
    assert c.vertices == nv and c.triangles == nt
    # what was written is the prefix of the full result
    assert torch.equal(out["triangles"], full.triangles[: nt // 2])
    assert torch.equal(out["positions"], full.positions[: nv // 2])
    # the soup generate refuses an indexed count phase
    o = {"soup": torch.empty((3 * nt, 28), dtype=torch.uint8, device="cuda")}
    cv = mcg._cvol(vol, 0.01)
    mo = mcg._mesh_out({**{k: None for k in ("normals", "vi2vox", "ver_voxel", "tri_cube")}, **o}, 3 * nt)
    st = mcg._lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), mcg._stream())
    assert st == mcg.MCG_ERR_STATE


def test_fusion_volume_matches_soup(mcg):
    """512-class property without the oracle: on a fused volume every soup
    vertex's edge is one indexed vertex and the soup positions agree with the
    indexed ones to the last bits (the soup interpolates some edges from the
    upper voxel)."""
    scene = synthetic.FusionScene(seed=3, extent=3.0)
    n = 192
    v = mcg.voxel_new((n, n, n), 0.03, 0.03, 3.0 / n)
    k = mcg.intrinsic(525.0, 525.0, 319.5, 239.5)
    for i in range(6):
        R, t = scene.pose(i, 6)
        mm = synthetic.mm_to_u16_bits(scene.depth_frame(R, t, seed=i, device="cuda"))
        meter = mcg.depth_to_maps(mm, k, vertex=False, normal=False)[0]
        mcg.volumetric_integration(v, k, mcg.extrinsic(R, t), meter)
    cell = 3.0 / n
    m = mcg.extract_indexed(v.data, cell, vertex_edge=True, tri_cube=True)
    s = mcg.extract(v.data, cell, normals=False, tri_cube=True)
    assert s.num_triangles == m.num_triangles and m.num_triangles > 10000
    assert torch.equal(s.tri_cube, m.tri_cube)
    sp = s.positions.reshape(-1, 3, 3)
    ip = m.positions[m.triangles.long()]
    assert float((sp - ip).abs().max()) <= 8 * 3.0 * 2.0 ** -23
    # unique vertices: at most the soup count, on a closed-ish surface far fewer
    assert m.num_vertices < 3 * m.num_triangles / 4
