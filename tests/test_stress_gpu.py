"""The 1024^3 stress volume (4 GiB short2: 200 spheres + gradient noise) at
full size: soup extraction bit-exact with the oracle over the whole volume,
and the RLE codec's round trips (lossless: bit-exact; reference format:
tsdf-exact)."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu
N = 1024


@pytest.fixture(scope="module")
def stress():
    vol = synthetic.stress_volume(N, seed=0)
    yield vol
    del vol
    torch.cuda.empty_cache()


def test_stress_extraction_matches_oracle(mcg, orc, stress):
    cell = 1.0 / N
    m = mcg.extract(stress, cell, normals=True, tri_cube=True)
    torch.cuda.synchronize()
    vol_np = stress.cpu().numpy()
    occ, ntri = orc.mc_count(vol_np)
    assert m.num_triangles == ntri and m.counts["occupied"] == occ and ntri > 1000000
    o = orc.mc_extract(vol_np, cell, normals=True, vi2vox=False, ver_voxel=False, tri_cube=True)
    tc = m.tri_cube.cpu().numpy()
    order = np.argsort(tc, kind="stable")
    assert np.array_equal(tc[order], o["tri_cube"])
    idx = (order[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
    soup = m.soup.cpu().numpy()[idx]
    assert np.array_equal(soup.reshape(-1).view(np.uint8), o["soup"].view(np.uint8))
    nrm = m.normals.cpu().numpy()[idx]
    assert np.array_equal(nrm.view(np.uint32), o["normals"].view(np.uint32))


def test_stress_rle_round_trips(mcg, stress):
    cell = 1.0 / N
    v = mcg.Voxel(stress, 5 * cell, 5 * cell, cell)
    img = mcg.rle_encode(v, lossless=True)
    back = mcg.rle_decode(img)
    assert torch.equal(back.data, stress)
    del back
    img = mcg.rle_encode(v, lossless=False)
    back = mcg.rle_decode(img)
    assert torch.equal(back.data[..., 0], stress[..., 0])


def test_stress_fp32_mc_adjoint_matches_binary64(mcg, orc, stress):
    """The MC adjoint at the full 1024^3 size, on the FP32 volume the bench
    times (tsdf / 32766, weight 0 or 1): dL/df from the GPU against the
    oracle's binary64 adjoint for the same dL/dP (canonical vertex order),
    relative 2-norm error <= 1e-4, and the same set of voxels touched."""
    cell = 1.0 / N
    f32 = torch.empty((N, N, N, 2), dtype=torch.float32, device="cuda")
    f32[..., 0] = stress[..., 0].to(torch.float32) / 32766.0
    f32[..., 1] = (stress[..., 1] != 0).to(torch.float32)
    m = mcg.extract(f32, cell, soup=False, normals=False, tri_cube=True)
    torch.cuda.synchronize()
    tc = m.tri_cube.cpu().numpy()
    del m
    order = np.argsort(tc, kind="stable")
    idx = (order[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
    n = len(idx)
    assert n > 3000000
    rng = np.random.default_rng(11)
    G = rng.standard_normal((n, 3)).astype(np.float32)
    Gd = np.empty_like(G)
    Gd[idx] = G
    g_dev = mcg.mc_backward(f32, cell, torch.from_numpy(Gd).cuda()).cpu().numpy().reshape(-1)
    vol_np = f32.cpu().numpy()
    del f32
    torch.cuda.empty_cache()
    g64 = orc.mc_backward_f64(vol_np, cell, G.astype(np.float64)).reshape(-1)
    del vol_np
    # chunked 2-norms (the arrays hold 2^30 voxels)
    num = den = 0.0
    touched_64 = 0
    step = 1 << 26
    for i in range(0, g64.size, step):
        a = g_dev[i:i + step].astype(np.float64)
        b = g64[i:i + step]
        num += float(np.dot(a - b, a - b))
        den += float(np.dot(b, b))
        assert np.array_equal(a != 0, b != 0)
        touched_64 += int(np.count_nonzero(b))
    assert touched_64 > 1000000
    assert (num / den) ** 0.5 <= 1e-4
