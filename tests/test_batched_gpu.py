"""Batched extraction (one launch per pass over many volumes) through the
C ABI equals per-volume extraction, bit for bit."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a.num_vertices == b.num_vertices
    for k in ("soup", "normals", "vi2vox", "ver_voxel", "tri_cube"):
        x, y = getattr(a, k), getattr(b, k)
        assert (x is None) == (y is None)
        if x is not None:
            assert torch.equal(x, y), k


def test_batched_equals_plain(mcg):
    vols = synthetic.batch_volumes(12, seed=3, lo=20, hi=100, device="cuda")
    # a few extra cases: empty volume, odd sizes (plain loads), float2 elsewhere
    e = torch.zeros((9, 10, 11, 2), dtype=torch.int16, device="cuda")
    e[..., 0] = 500
    e[..., 1] = 1
    vols.append(e)
    vols.append(torch.from_numpy(synthetic.random_volume((7, 9, 13), seed=5)).cuda())
    cells = [0.01 * (1 + i % 3) for i in range(len(vols))]
    kw = dict(soup=True, normals=True, vi2vox=True, ver_voxel=True, tri_cube=True)
    batched = mcg.extract_batched(vols, cells, **kw)
    for v, c, m in zip(vols, cells, batched):
        _same(m, mcg.extract(v, c, **kw))
    assert sum(m.num_vertices for m in batched) > 1000
    assert batched[-2].num_vertices == 0


def test_batched_float2(mcg):
    rng = np.random.default_rng(9)
    vols = []
    for shape in [(12, 14, 40), (20, 9, 33), (11, 11, 48)]:
        v = np.stack([rng.standard_normal(shape).astype(np.float32),
                      (rng.random(shape) > 0.05).astype(np.float32)], axis=-1)
        vols.append(torch.from_numpy(v).cuda())
    batched = mcg.extract_batched(vols, 0.5, tri_cube=True)
    for v, m in zip(vols, batched):
        _same(m, mcg.extract(v, 0.5, tri_cube=True))


def test_batched_capacity_per_volume(mcg):
    vols = synthetic.batch_volumes(4, seed=11, lo=32, hi=64, device="cuda")
    full = [mcg.extract(v, 0.01) for v in vols]
    caps = [m.num_vertices // 2 for m in full]
    outs = [{"soup": torch.zeros((max(m.num_vertices, 1), 28), dtype=torch.uint8, device="cuda")} for m in full]
    ctx = mcg.Context()
    mcg.extract_batched_into(vols, 0.01, outs, caps, ctx=ctx)
    counts = mcg.counts_batched(ctx, len(vols))
    for c, m, o, cap in zip(counts, full, outs, caps):
        assert c["vertices"] == m.num_vertices
        if m.num_vertices > cap:
            assert c["status"] == mcg.MCG_ERR_CAPACITY
        assert torch.equal(o["soup"][:cap], m.soup[:cap])
    ctx.close()
