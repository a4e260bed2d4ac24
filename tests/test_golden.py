"""The CPU oracle reproduces the golden fixtures: cube indices, topology and
RLE bytes exactly, positions / normals within tolerance of binary64."""
import os

import numpy as np
import pytest

from golden_util import cases, check_mesh, load


@pytest.mark.parametrize("path", cases(), ids=lambda p: os.path.basename(p))
def test_oracle_matches_golden(orc, path):
    g = load(path)
    vol = g["vol"]
    ci, _ = orc.mc_classify(vol)
    assert np.array_equal(ci, g["ci"])
    out = orc.mc_extract(vol, float(g["cell"]))
    check_mesh(g, out["soup"]["pos"], out["normals"], out["tri_cube"])
    slices = vol.reshape(vol.shape[0], -1, 2)
    enc = b"".join(orc.rle_encode_slice(s) for s in slices)
    assert enc == g["rle"].tobytes()


@pytest.mark.parametrize("path", cases(), ids=lambda p: os.path.basename(p))
def test_library_host_rle_matches_golden(path):
    import marching_cube_gb300 as mcg
    g = load(path)
    vol = g["vol"]
    img = mcg.rle_encode_host(vol, 0.03, 0.03, float(g["cell"]))
    # skip the 40-byte header, then per slice: uint32 size + records
    body, off = b"", 40
    for sz in g["rle_sizes"]:
        n = int.from_bytes(img[off:off + 4], "little")
        assert n == sz
        body += img[off + 4:off + 4 + n]
        off += 4 + n
    assert off == len(img)
    assert body == g["rle"].tobytes()
