"""Volumes that TMA cannot describe, filled into shared-memory tiles by 16-byte
words shifted into place: rows that are not a multiple of 16 bytes, bases
that are not 16-byte aligned (views 1, 2 or 3 voxels into a buffer), and
volumes whose last 16-byte word lies partly past the end of the view.
Every output of the extraction (soup, normals, vi2vox, ver_voxel, cube
ids), the batched extraction, the indexed extraction's counts and the
adjoint against the oracle or against an aligned copy of the same volume
(the adjoint within the run-to-run variation of its FP32 atomic sums).

Reference: cu_marching_cubes_v1.cu:416-467 (MarchingCubes::run)."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic
from mc_util import assert_same_mesh, mesh_arrays

pytestmark = pytest.mark.gpu

SHAPES = [(37, 23, 19), (64, 20, 18), (33, 17, 40), (70, 9, 11), (5, 7, 3)]


def _view(vol_np, off, dtype=torch.int16):
    """A device view of vol_np starting `off` voxels into a larger buffer,
    with one voxel of slack after it."""
    nz, ny, nx, _ = vol_np.shape
    n = nx * ny * nz
    buf = torch.full(((n + off + 1) * 2,), 7, dtype=dtype, device="cuda")
    v = buf[2 * off:2 * off + 2 * n].view(nz, ny, nx, 2)
    v.copy_(torch.from_numpy(np.ascontiguousarray(vol_np)).cuda())
    return buf, v


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("off", [1, 2, 3])
def test_misaligned_views_match_oracle(mcg, orc, shape, off):
    nx, ny, nz = shape
    vol = synthetic.random_volume((nz, ny, nx), seed=nx * 7 + off, sentinel_frac=0.02)
    buf, v = _view(vol, off)
    assert v.data_ptr() % 16 != 0
    cell = 0.03
    m = mcg.extract(v, cell, soup=True, normals=True, vi2vox=True, ver_voxel=True, tri_cube=True)
    torch.cuda.synchronize()
    g = mesh_arrays(m)
    o = orc.mc_extract(vol, cell)
    assert len(o["soup"]) > 0
    assert_same_mesh(g, o)
    # the indexed path reads the same tiles
    idx = mcg.extract_indexed(v, cell)
    torch.cuda.synchronize()
    assert idx.counts["triangles"] == len(o["soup"]) // 3
    del buf


def test_misaligned_batch_matches_single(mcg):
    vols, bufs, cells = [], [], []
    for i, (nx, ny, nz) in enumerate(SHAPES):
        vol = synthetic.random_volume((nz, ny, nx), seed=100 + i, sentinel_frac=0.0)
        buf, v = _view(vol, 1 + i % 3)
        vols.append(v)
        bufs.append(buf)
        cells.append(0.02 + 0.001 * i)
    meshes = mcg.extract_batched(vols, cells, normals=True)
    torch.cuda.synchronize()
    for v, c, mb in zip(vols, cells, meshes):
        ms = mcg.extract(v.clone(), c, soup=True, normals=True)  # aligned copy: TMA where it can
        torch.cuda.synchronize()
        assert ms.counts["vertices"] == mb.counts["vertices"] > 0
        assert torch.equal(ms.soup, mb.soup) and torch.equal(ms.normals, mb.normals)


def test_misaligned_float2_adjoint_matches_aligned(mcg):
    nx, ny, nz = 41, 19, 23
    vol = synthetic.random_volume((nz, ny, nx), seed=9, sentinel_frac=0.0).astype(np.float32) / 32766.0
    vol[..., 1] = (vol[..., 1] != 0).astype(np.float32)
    buf, v = _view(vol, 1, dtype=torch.float32)
    assert v.data_ptr() % 16 != 0
    a = v.clone()
    cell = 0.05
    pa = mcg.mesh_positions(a, cell)
    pv = mcg.mesh_positions(v, cell)
    torch.cuda.synchronize()
    assert torch.equal(pa, pv) and pa.shape[0] > 0
    G = torch.randn(pa.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    ga = mcg.mc_backward(a, cell, G)
    gv = mcg.mc_backward(v, cell, G)
    torch.cuda.synchronize()
    # the adjoint accumulates with FP32 atomics, so the order of its sums
    # (and their last bits) varies from run to run
    assert torch.equal(ga != 0, gv != 0) and int((ga != 0).sum()) > 0
    assert float((ga - gv).norm() / ga.norm()) <= 1e-6
    del buf
