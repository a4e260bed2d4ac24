"""Slab extraction: the cubes of z0 <= z < z1 only.  Slabs of consecutive
ranges, concatenated in order, are the whole volume's soup bit for bit
(records, normals, cube ids); invalid ranges are rejected."""
import ctypes

import numpy as np
import pytest
import torch

from marching_cube_gb300 import shard, synthetic

pytestmark = pytest.mark.gpu


def _whole(mcg, vol, cell):
    m = mcg.extract(vol, cell, soup=True, normals=True, tri_cube=True)
    return m.soup.cpu(), m.normals.cpu(), m.tri_cube.cpu()


@pytest.mark.parametrize("shape,parts", [((96, 96, 96), 3), ((97, 41, 67), 2), ((41, 10, 97), 5), ((24, 40, 40), 4)])
def test_slabs_concatenate_to_the_whole(mcg, shape, parts):
    if shape[0] == shape[1] == shape[2]:
        vol_np = synthetic.sphere_volume(shape[0], radius=shape[0] * 0.3, trunc=4.0, seed=1)
    else:
        vol_np = synthetic.random_volume(shape, seed=sum(shape))
    vol = torch.from_numpy(vol_np).cuda()
    soup, nrm, tc = _whole(mcg, vol, 0.01)
    parts_out = []
    for z0, z1 in shard.slab_bounds(shape[0], parts):
        if z1 <= z0:
            continue
        m = mcg.extract_slab(vol, 0.01, z0, z1, soup=True, normals=True, tri_cube=True)
        if m.num_vertices:
            parts_out.append((m.soup.cpu(), m.normals.cpu(), m.tri_cube.cpu()))
            # every cube of the slab lies in its range
            z = m.tri_cube.cpu() // (shape[1] * shape[2])
            assert int(z.min()) >= z0 and int(z.max()) < z1
    assert torch.equal(torch.cat([p[0] for p in parts_out]), soup)
    assert torch.equal(torch.cat([p[1] for p in parts_out]).view(torch.int32), nrm.view(torch.int32))
    assert torch.equal(torch.cat([p[2] for p in parts_out]), tc)


def test_slab_adjoint_matches_the_whole(mcg):
    """MC adjoint after a slab count phase: the slab's share of the whole
    volume's gradient (same voxels, same dL/dP per vertex)."""
    vol_np = synthetic.sphere_volume(64, radius=20.0, trunc=4.0, seed=2)
    f32 = np.stack([vol_np[..., 0].astype(np.float32) / 32766.0, np.ones(vol_np.shape[:3], np.float32)], -1)
    vol = torch.from_numpy(f32).cuda()
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    whole = mcg.extract(vol, 0.01, soup=True, normals=False)
    G = torch.randn((whole.num_vertices, 3), device="cuda", generator=g)
    gw = mcg.mc_backward(vol, 0.01, G)
    acc = torch.zeros_like(gw)
    off = 0
    for z0, z1 in shard.slab_bounds(64, 3):
        m = mcg.extract_slab(vol, 0.01, z0, z1, soup=True, normals=False)
        n = m.num_vertices
        mcg.mc_backward(vol, 0.01, G[off:off + n].contiguous(), grad_f=acc, reclassify=False)
        off += n
    assert off == whole.num_vertices
    assert float((acc - gw).abs().max()) <= 1e-4 * float(gw.abs().max())


def test_slab_rejects_bad_ranges(mcg):
    vol = torch.from_numpy(synthetic.sphere_volume(40, radius=12.0, trunc=4.0)).cuda()
    ctx = mcg.Context()
    cv = mcg._cvol(vol, 0.01)
    for z0, z1 in ((4, 16), (0, 0), (8, 40), (-8, 8), (16, 8)):
        assert mcg._lib.mcg_mc_classify_slab(ctx.handle, ctypes.byref(cv), z0, z1, mcg._stream()) == \
            mcg.MCG_ERR_INVALID_ARG
    # ver_voxel is whole-volume state: not with a partial slab
    assert mcg._lib.mcg_mc_classify_slab(ctx.handle, ctypes.byref(cv), 8, 24, mcg._stream()) == mcg.MCG_OK
    c = mcg.counts(ctx)
    vv = torch.zeros(40 ** 3, dtype=torch.int16, device="cuda")
    soup = torch.empty((max(c["vertices"], 1), 28), dtype=torch.uint8, device="cuda")
    mo = mcg._mesh_out({"soup": soup, "normals": None, "vi2vox": None, "ver_voxel": vv, "tri_cube": None},
                       c["vertices"])
    assert mcg._lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), mcg._stream()) == \
        mcg.MCG_ERR_INVALID_ARG
