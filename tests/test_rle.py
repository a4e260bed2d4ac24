"""RLE volume codec of the library (host entry points, no GPU): byte-exact
with the oracle, bit-exact round trips in the domain of each format, and
malformed input rejected."""
import numpy as np
import pytest

from marching_cube_gb300 import synthetic

MAX_TSDF = 32766


def reference_domain(vol):
    """Normalise a volume into the domain the reference format round-trips:
    every run of equal tsdf along x (inside a slice) carries the weight of its
    first voxel, and sentinel voxels (+-32766) have weight 0."""
    v = vol.copy()
    nz = v.shape[0]
    flat = v.reshape(nz, -1, 2)
    for z in range(nz):
        s = flat[z]
        t = s[:, 0]
        start = np.r_[True, t[1:] != t[:-1]]
        idx = np.maximum.accumulate(np.where(start, np.arange(len(t)), 0))
        s[:, 1] = s[idx, 1]
        sent = (t == MAX_TSDF) | (t == -MAX_TSDF)
        s[sent, 1] = 0
    return v


@pytest.mark.parametrize("shape,seed", [((4, 5, 6), 1), ((16, 33, 17), 2), ((3, 200, 300), 3)])
def test_host_codec_matches_oracle(mcg, orc, shape, seed):
    vol = synthetic.random_volume(shape, seed=seed, sentinel_frac=0.5)
    for lossless in (False, True):
        a = mcg.rle_encode_host(vol, 0.03, 0.04, 0.005, lossless=lossless)
        b = orc.rle_encode_volume(vol, 0.03, 0.04, 0.005, lossless=lossless)
        assert a == b


def test_lossless_round_trip_any_volume(mcg):
    vol = synthetic.random_volume((12, 40, 50), seed=4, sentinel_frac=0.3)
    img = mcg.rle_encode_host(vol, 0.03, 0.03, 0.01, lossless=True)
    back, params = mcg.rle_decode_host(img)
    assert np.array_equal(back, vol)
    assert img[:16] == b"VOLUME_TSDF_W32\x00"


def test_reference_format_round_trip_in_its_domain(mcg):
    # long runs so runs actually form, with sentinels and split runs
    rng = np.random.default_rng(5)
    vol = np.zeros((6, 64, 300, 2), np.int16)
    vol[..., 0] = rng.choice([MAX_TSDF, -MAX_TSDF, 1200, -300], size=(6, 64, 300), p=[0.5, 0.3, 0.1, 0.1])
    vol[..., 1] = rng.integers(1, 9, size=(6, 64, 300))
    dom = reference_domain(vol)
    img = mcg.rle_encode_host(dom, 0.03, 0.03, 0.01)
    back, _ = mcg.rle_decode_host(img)
    assert np.array_equal(back, dom)
    # outside the domain the reference format keeps tsdf exactly
    img2 = mcg.rle_encode_host(vol, 0.03, 0.03, 0.01)
    back2, _ = mcg.rle_decode_host(img2)
    assert np.array_equal(back2[..., 0], vol[..., 0])
    assert not np.array_equal(back2[..., 1], vol[..., 1])


def test_compression_of_fusion_like_volume(mcg):
    # free space (+32766, w>0 -> literal runs), unobserved (-32766, w=0)
    vol = np.zeros((8, 128, 128, 2), np.int16)
    vol[..., 0] = -MAX_TSDF
    vol[:, :, :64, 0] = MAX_TSDF
    vol[:, :, :64, 1] = 3
    img = mcg.rle_encode_host(vol, 0.03, 0.03, 0.01)
    assert len(img) < vol.nbytes / 100


def test_malformed_images_rejected(mcg):
    vol = synthetic.random_volume((3, 4, 5), seed=6)
    img = bytearray(mcg.rle_encode_host(vol, 0.03, 0.03, 0.01))
    with pytest.raises(mcg.MCGError) as e:
        mcg.rle_decode_host(bytes(img[:-3]))           # truncated
    assert e.value.status == mcg.MCG_ERR_FORMAT
    bad = bytearray(img)
    bad[0:16] = b"NOT_A_VOLUME\x00\x00\x00\x00"
    with pytest.raises(mcg.MCGError):
        mcg.rle_decode_host(bytes(bad))                 # wrong tag
    bad = bytearray(img)
    bad[44:46] = (0 | (1 << 14)).to_bytes(2, "little")  # zero-length run in slice 0
    with pytest.raises(mcg.MCGError):
        mcg.rle_decode_host(bytes(bad))


def test_image_larger_than_2gib_round_trips(mcg):
    """A file image past 2^31 bytes (every voxel a 6-byte literal) encodes and
    decodes whole."""
    import numpy as np
    nz = (2 ** 31) // (6 * 1024 * 1024) + 2
    rng = np.random.default_rng(0)
    vol = np.empty((nz, 1024, 1024, 2), np.int16)
    vol[..., 0] = rng.integers(-32767, 32768, size=(nz, 1024, 1024), dtype=np.int16)
    vol[..., 1] = 1
    vol[:, :, 1::2, 0] = vol[:, :, 0::2, 0] ^ 1  # no two neighbours share a tsdf
    img = mcg.rle_encode_host(vol, 0.01, 0.01, 0.002, lossless=True)
    assert len(img) > 2 ** 31
    back, _ = mcg.rle_decode_host(img)
    assert np.array_equal(back, vol)
