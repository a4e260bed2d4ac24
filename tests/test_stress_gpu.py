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
