"""RLE codec on device volumes through the C ABI: the same bytes as the
host codec, bit-exact round trips, file I/O wrappers."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_device_encode_decode(mcg, tmp_path):
    vol = synthetic.random_volume((20, 33, 70), seed=7, sentinel_frac=0.4)
    v = mcg.Voxel(torch.from_numpy(vol).cuda(), 0.03, 0.03, 0.01)
    for lossless in (False, True):
        img = mcg.rle_encode(v, lossless=lossless)
        assert img == mcg.rle_encode_host(vol, 0.03, 0.03, 0.01, lossless=lossless)
    img = mcg.rle_encode(v, lossless=True)
    back = mcg.rle_decode(img)
    assert torch.equal(back.data, v.data)
    assert (back.min_t, back.max_t) == pytest.approx((0.03, 0.03))
    f = str(tmp_path / "vol.rle")
    mcg.run_length_encode(v, f, lossless=True)
    back = mcg.run_length_decode(f)
    assert torch.equal(back.data, v.data)


def test_fused_volume_round_trip(mcg):
    # a fusion volume is in the reference format's domain after one frame:
    # observed voxels are literal runs, unobserved ones the -32766 sentinel
    v = mcg.voxel_new((64, 48, 40), 0.1, 0.1, 3.0 / 64)
    img = mcg.rle_encode(v)
    back = mcg.rle_decode(img)
    assert torch.equal(back.data, v.data)
    assert len(img) < 40 + 40 * (4 + 2 * 64 * 48 // 16383 + 8)
