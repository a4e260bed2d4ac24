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


def _runs_volume(shape, seed, mean_run, values):
    """Slices of runs with geometric lengths (mean mean_run) over `values`
    (a few tsdf values, sentinels among them), weights varying inside runs."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    n = nx * ny * nz
    t = np.empty(n, np.int16)
    i = 0
    while i < n:
        L = int(rng.geometric(1.0 / mean_run))
        t[i:i + L] = rng.choice(values)
        i += L
    w = rng.integers(0, 3, size=n).astype(np.uint16)
    w[rng.random(n) < 0.7] = 1
    return np.stack([t.reshape(shape), w.reshape(shape).view(np.int16)], axis=-1)


@pytest.mark.parametrize("shape,mean_run", [((3, 128, 256), 40000), ((4, 257, 129), 3000), ((5, 64, 61), 7),
                                            ((2, 1, 9000), 20000), ((7, 3, 5), 2)])
def test_device_encoder_runs_and_splits(mcg, shape, mean_run):
    """Runs longer than the 14-bit count (split every 16383 voxels), runs
    across the encoder's 4096-voxel chunks and slices, odd slice sizes: the
    device encoder writes the host encoder's bytes."""
    vol = _runs_volume(shape, seed=mean_run, mean_run=mean_run, values=np.array([32766, -32766, 5, -7, 0], np.int16))
    v = mcg.Voxel(torch.from_numpy(vol).cuda(), 0.03, 0.03, 0.01)
    for lossless in (False, True):
        img = mcg.rle_encode(v, lossless=lossless)
        assert img == mcg.rle_encode_host(vol, 0.03, 0.03, 0.01, lossless=lossless)
    back = mcg.rle_decode(mcg.rle_encode(v, lossless=True))
    assert torch.equal(back.data, v.data)


def test_device_encoder_uniform_slices(mcg):
    """Whole slices of one value: one split record every 16383 voxels."""
    vol = np.zeros((3, 200, 300, 2), np.int16)
    vol[0, ..., 0] = 32766
    vol[1, ..., 0] = -32766
    vol[2, ..., 0] = 1234
    vol[..., 1] = 7
    v = mcg.Voxel(torch.from_numpy(vol).cuda(), 0.03, 0.03, 0.01)
    for lossless in (False, True):
        assert mcg.rle_encode(v, lossless=lossless) == mcg.rle_encode_host(vol, 0.03, 0.03, 0.01, lossless=lossless)
