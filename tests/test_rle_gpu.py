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


def _split(img):
    """(header bytes, [slice record bytes]) of a well-formed image."""
    img = bytes(img)
    nz = int(np.frombuffer(img[16:28], np.int32)[2])
    p, out = 40, []
    for _ in range(nz):
        n = int(np.frombuffer(img[p:p + 4], np.uint32)[0])
        out.append(img[p + 4:p + 4 + n])
        p += 4 + n
    return img[:40], out


def _join(head, slices):
    return head + b"".join(np.uint32(len(s)).tobytes() + s for s in slices)


def _host_decode(mcg, img):
    try:
        vol, _ = mcg.rle_decode_host(img)
        return 0, vol
    except mcg.MCGError as e:
        return e.status, None


def _gpu_decode(mcg, img):
    try:
        return 0, mcg.rle_decode(img).data.cpu().numpy()
    except mcg.MCGError as e:
        return e.status, None


def test_gpu_decoder_malformed_like_host(mcg):
    """The GPU decoder accepts and rejects exactly what the host decoder
    does: zero-length and overlong runs, truncated literals and streams, odd
    trailing bytes and records after a full slice, cut directories."""
    vol = _runs_volume((3, 40, 50), seed=3, mean_run=30, values=np.array([32766, -32766, 5, -7], np.int16))
    v = mcg.Voxel(torch.from_numpy(vol).cuda(), 0.03, 0.03, 0.01)
    head, sl = _split(mcg.rle_encode(v, lossless=False))
    rec = lambda cnt, kind: np.uint16(cnt | (kind << 14)).tobytes()
    cases = {
        "valid": sl,
        "zero_count": [sl[0], rec(0, 1) + sl[1], sl[2]],
        "overlong": [sl[0], sl[1], rec(1500, 1) + rec(600, 2)],
        "short_stream": [sl[0], sl[1][:-2], sl[2]],
        "cut_literal": [sl[0], sl[1], rec(1, 3) + b"\x01\x02"],
        "odd_trailing": [sl[0], sl[1] + b"\x07", sl[2]],
        "after_full": [sl[0] + rec(3, 1) + rec(0, 2), sl[1], sl[2] + rec(9, 3) + b"\x01"],
        "literal_kind0": [rec(2000, 0) + b"\x05\x00\x01\x00", sl[1], sl[2]],
    }
    for name, slices in cases.items():
        img = _join(head, slices)
        hs, hv = _host_decode(mcg, img)
        gs, gv = _gpu_decode(mcg, img)
        assert hs == gs, name
        if hs == 0:
            assert np.array_equal(hv, gv), name
    img = _join(head, sl)
    for cut in (39, 45, len(img) - 1):
        assert _gpu_decode(mcg, img[:cut])[0] == _host_decode(mcg, img[:cut])[0] == mcg.MCG_ERR_FORMAT


def test_gpu_decoder_literal_slices(mcg):
    """512 x 512 slices of literals (six bytes a voxel, ~380 chunks of 4096
    words a slice) and of long runs."""
    rng = np.random.default_rng(9)
    vol = np.empty((3, 512, 512, 2), np.int16)
    vol[..., 0] = rng.integers(-30000, 30000, size=(3, 512, 512))
    vol[..., 1] = rng.integers(1, 100, size=(3, 512, 512))
    vol[1, 100:400, :, 0] = -32766
    vol[1, 100:400, :, 1] = 0
    v = mcg.Voxel(torch.from_numpy(vol).cuda(), 0.03, 0.03, 0.01)
    for lossless in (True, False):
        img = mcg.rle_encode(v, lossless=lossless)
        hs, hv = _host_decode(mcg, img)
        gs, gv = _gpu_decode(mcg, img)
        assert hs == gs == 0 and np.array_equal(hv, gv)
    assert np.array_equal(_gpu_decode(mcg, mcg.rle_encode(v, lossless=True))[1], vol)


def test_gpu_decode_file_pieces(mcg, tmp_path):
    """A 68 MB image read in 64 MiB pieces: slices straddle the piece end and
    one slice byte count is split by it (bytes 2 + 2)."""
    nz, ny, nx = 114, 100, 1000
    xy = nx * ny
    rng = np.random.default_rng(10)
    vol = np.empty((nz, ny, nx, 2), np.int16)
    vol[..., 0] = rng.integers(-30000, 30000, size=(nz, ny, nx))
    vol[..., 1] = (np.arange(xy).reshape(ny, nx) % 2 + 1)[None]  # neighbours always differ
    flat0 = vol[0].reshape(-1, 2)
    flat0[84728:, 0] = 1234  # slice 0: 84728 literals, then one run of 15272
    flat0[84728:, 1] = 7
    v = mcg.Voxel(torch.from_numpy(vol).cuda(), 0.03, 0.03, 0.01)
    img = bytes(mcg.rle_encode(v, lossless=True))
    cnt_at = 40 + (4 + 6 * 84729) + 111 * (4 + 6 * xy)  # byte count of slice 112
    assert cnt_at == (64 << 20) - 2 and len(img) > (64 << 20)
    assert int(np.frombuffer(img[cnt_at:cnt_at + 4], np.uint32)[0]) == 6 * xy
    f = tmp_path / "pieces.rle"
    f.write_bytes(img)
    back = mcg.run_length_decode(str(f))
    assert torch.equal(back.data, v.data)
    assert torch.equal(mcg.rle_decode(img).data, v.data)
    # a file cut inside the directory, and a missing file
    f.write_bytes(img[: cnt_at + 3])
    with pytest.raises(mcg.MCGError) as e:
        mcg.run_length_decode(str(f))
    assert e.value.status == mcg.MCG_ERR_FORMAT
    with pytest.raises(mcg.MCGError) as e:
        mcg.run_length_decode(str(tmp_path / "missing.rle"))
    assert e.value.status == mcg.MCG_ERR_IO
