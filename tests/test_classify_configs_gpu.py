"""Every classify configuration (mcg_mc_config.classify_shape: item width,
in-box or separate halo box, stage ring and CTA size) and a range of
generate start rounds give the oracle's counts and soup, on volumes that take
the TMA path with and without the halo column inside the volume, the
plain-copy path, and float2."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu

SHAPES = [((20, 33, 300), 1), ((17, 40, 130), 2), ((11, 13, 45), 3), ((24, 24, 128), 4)]


def _check(mcg, orc, ctx, vol, cell=0.01):
    m = mcg.extract(torch.from_numpy(vol).cuda(), cell, normals=True, tri_cube=True, ctx=ctx)
    torch.cuda.synchronize()
    occ, tri = orc.mc_count(vol)
    assert m.counts["occupied"] == occ and m.counts["triangles"] == tri
    o = orc.mc_extract(vol, cell)
    tc = m.tri_cube.cpu().numpy()
    order = np.argsort(tc, kind="stable")
    idx = (order[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
    soup = m.soup.cpu().numpy().reshape(-1, 28)[idx]
    assert np.array_equal(soup.reshape(-1), o["soup"].view(np.uint8).reshape(-1))


@pytest.mark.parametrize("shape_cfg", [0, 1, 2, 3, 4, 5])
def test_classify_config_matches_oracle(mcg, orc, shape_cfg):
    ctx = mcg.Context()
    ctx.set_config(classify_shape=shape_cfg, fused=0)
    for shape, seed in SHAPES:
        _check(mcg, orc, ctx, synthetic.random_volume(shape, seed=seed))
    rng = np.random.default_rng(5)
    f2 = np.stack([rng.standard_normal((14, 20, 200)).astype(np.float32),
                   (rng.random((14, 20, 200)) > 0.03).astype(np.float32)], axis=-1)
    m = mcg.extract(torch.from_numpy(f2).cuda(), 0.5, normals=False, ctx=ctx)
    torch.cuda.synchronize()
    occ, tri = orc.mc_count(f2)
    assert m.counts["occupied"] == occ and m.counts["triangles"] == tri
    ctx.close()


@pytest.mark.parametrize("rounds", [0, 1, 5, 16])
def test_generate_start_rounds_match_oracle(mcg, orc, rounds):
    ctx = mcg.Context()
    ctx.set_config(gen_fixed_rounds=rounds, fused=0)
    _check(mcg, orc, ctx, synthetic.sphere_volume(96, radius=30.0, seed=rounds))
    _check(mcg, orc, ctx, synthetic.random_volume((20, 33, 300), seed=9))
    ctx.close()
