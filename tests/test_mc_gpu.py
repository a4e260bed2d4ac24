"""Parity of the CUDA marching-cubes path (through the C ABI) with the CPU
oracle: cube indices, counts, topology and every output bit-exact against
the FP32 mirror; positions within 1e-5 voxel of the FP64 oracle."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic
from mc_util import assert_same_mesh, gpu_extract

pytestmark = pytest.mark.gpu

POS_TOL_VOXEL = 1e-5   # |p_gpu - p_fp64| / cell
NRM_TOL = 1e-5         # abs, on unit normals away from degenerate gradients


def test_sphere_128_parity(mcg, orc):
    vol = synthetic.sphere_volume(128, seed=0)
    cell = 0.01
    g = gpu_extract(mcg, vol, cell)
    o = orc.mc_extract(vol, cell)
    occ, tri = orc.mc_count(vol)
    assert g["counts"]["triangles"] == tri and g["counts"]["occupied"] == occ
    assert tri > 10000
    assert_same_mesh(g, o)


def test_sphere_fp64_tolerance(mcg, orc):
    vol = synthetic.sphere_volume(64, radius=20.0, seed=3)
    cell = 0.01
    g = gpu_extract(mcg, vol, cell)
    pos64, nrm64 = orc.mc_extract_f64(vol, cell)
    pos = g["soup"]["pos"].astype(np.float64)
    err = np.abs(pos - pos64).max() / cell
    assert err <= POS_TOL_VOXEL, err
    good = np.linalg.norm(nrm64, axis=1) > 0.5
    nerr = np.abs(g["normals"][good].astype(np.float64) - nrm64[good]).max()
    assert nerr <= NRM_TOL, nerr


# (nz, ny, nx): nx*4 a multiple of 16 and every dim >= the tile box takes the
# TMA path; the others take the plain-load path
@pytest.mark.parametrize("shape,seed", [((2, 2, 2), 1), ((3, 5, 7), 2), ((9, 33, 65), 3),
                                        ((17, 40, 31), 4), ((8, 8, 96), 5), ((40, 3, 2), 6),
                                        ((11, 13, 40), 7), ((30, 17, 100), 8), ((12, 12, 64), 9),
                                        ((19, 41, 200), 10)])
def test_random_volumes(mcg, orc, shape, seed):
    vol = synthetic.random_volume(shape, seed=seed)
    cell = 0.0037
    g = gpu_extract(mcg, vol, cell)
    o = orc.mc_extract(vol, cell)
    assert_same_mesh(g, o)


def test_classification_bit_exact(mcg, orc):
    # per-cube triangle count recovered from the GPU's tri_cube histogram
    vol = synthetic.random_volume((19, 21, 70), seed=11, p_zero_weight=0.1)
    g = gpu_extract(mcg, vol, 1.0)
    ci, nv = orc.mc_classify(vol)
    nz, ny, nx, _ = vol.shape
    counts = np.bincount(g["tri_cube"], minlength=nx * ny * nz).reshape(nz, ny, nx)
    assert np.array_equal(counts[:-1, :-1, :-1], nv.astype(np.int64) // 3)
    assert counts[-1].sum() == 0 and counts[:, -1].sum() == 0 and counts[:, :, -1].sum() == 0


def test_empty_and_full(mcg, orc):
    vol = np.zeros((10, 12, 14, 2), np.int16)
    vol[..., 0] = 1000
    vol[..., 1] = 7
    g = gpu_extract(mcg, vol, 0.1)
    assert g["counts"]["triangles"] == 0 and len(g["soup"]) == 0
    assert (g["ver_voxel"] == 0).all()
    vol[..., 0] = -5
    g = gpu_extract(mcg, vol, 0.1)
    assert g["counts"]["triangles"] == 0


def test_zero_weight_kills_cube(mcg, orc):
    vol = synthetic.sphere_volume(24, radius=7.0, seed=5)
    vol[12, 12, 5, 1] = 0
    g = gpu_extract(mcg, vol, 0.02)
    o = orc.mc_extract(vol, 0.02)
    assert_same_mesh(g, o)
    full = orc.mc_count(synthetic.sphere_volume(24, radius=7.0, seed=5))[1]
    assert g["counts"]["triangles"] < full


def test_surface_through_max_faces(mcg, orc):
    # sphere centred near the max corner: vertices on the last cube layer,
    # normals sampled past the faces use the reference's linear addressing
    vol = synthetic.sphere_volume(40, radius=12.0, seed=9, center=38.0)
    g = gpu_extract(mcg, vol, 0.01)
    o = orc.mc_extract(vol, 0.01)
    assert_same_mesh(g, o)


@pytest.mark.parametrize("shape", [(13, 17, 45), (14, 20, 46)])
def test_float2_volume(mcg, orc, shape):
    rng = np.random.default_rng(7)
    vol = np.stack([rng.standard_normal(shape).astype(np.float32),
                    (rng.random(shape) > 0.03).astype(np.float32)], axis=-1)
    g = gpu_extract(mcg, vol, 0.5)
    o = orc.mc_extract(vol, 0.5)
    assert_same_mesh(g, o)


def test_deterministic_order(mcg):
    vol = synthetic.random_volume((20, 30, 50), seed=12)
    a = gpu_extract(mcg, vol, 0.01, canonical=False)
    b = gpu_extract(mcg, vol, 0.01, canonical=False)
    assert np.array_equal(a["soup"].view(np.uint8), b["soup"].view(np.uint8))
    assert np.array_equal(a["tri_cube"], b["tri_cube"])


def test_capacity_truncation(mcg, orc):
    vol = torch.from_numpy(synthetic.sphere_volume(48, radius=15.0, seed=2)).cuda()
    full = mcg.extract(vol, 0.01, normals=True)
    n = full.num_vertices
    cap = n // 2 + 1
    soup = torch.zeros((n, 28), dtype=torch.uint8, device="cuda")
    nrm = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    ctx = mcg.Context()
    mcg.extract_into(vol, 0.01, {"soup": soup, "normals": nrm}, cap, ctx=ctx)
    c = mcg.counts(ctx)
    assert c["status"] == mcg.MCG_ERR_CAPACITY and c["vertices"] == n
    assert torch.equal(soup[:cap], full.soup[:cap])
    assert torch.equal(nrm[:cap], full.normals[:cap])
    assert int(soup[cap:].abs().sum()) == 0
    ctx.close()


def test_normals_entry_point(mcg, orc):
    vol = synthetic.sphere_volume(32, radius=9.0, seed=4)
    g = gpu_extract(mcg, vol, 0.01)
    tv = torch.from_numpy(vol).cuda()
    soup_t = torch.from_numpy(g["soup"].view(np.uint8).reshape(-1, 28).copy()).cuda()
    n = mcg.extract_surface_normals(tv, 0.01, soup_t).cpu().numpy()
    assert np.array_equal(n.view(np.uint32), g["normals"].view(np.uint32))
    for i in range(0, len(n), 97):
        assert np.array_equal(orc.surface_normal(vol, 0.01, g["soup"]["pos"][i]).view(np.uint32),
                              n[i].view(np.uint32))


def test_reference_class_api(mcg, orc):
    v = mcg.Voxel(torch.from_numpy(synthetic.sphere_volume(32, radius=10.0, seed=1)).cuda(), 0.03, 0.03, 0.01)
    mesh = mcg.MarchingCubes().run(v)
    o = orc.mc_extract(v.data.cpu().numpy(), 0.01)
    assert mesh.num_vertices == len(o["soup"])
    assert mesh.positions.shape == (mesh.num_vertices, 3)
    assert mesh.ver_voxel.shape == (32 * 32 * 32,)
    assert np.array_equal(mesh.ver_voxel.cpu().numpy(), o["ver_voxel"])
