"""The autotuner on the GPU: it times the candidates on a volume, applies the
fastest to the context, caches it, and a tuned extraction gives the same
mesh as the default configuration, bit for bit."""
import pytest
import torch

from marching_cube_gb300 import synthetic, tune

pytestmark = pytest.mark.gpu


def test_autotune_applies_caches_and_preserves_output(mcg, tmp_path):
    path = str(tmp_path / "tune.json")
    vol = torch.from_numpy(synthetic.sphere_volume(160, radius=50.0, seed=9)).cuda()
    ref = mcg.extract(vol, 0.01, normals=True)
    ctx = mcg.Context()
    r = tune.autotune(vol, 0.01, ctx=ctx, reps=3, warmup=1, path=path)
    assert not r["cached"] and r["ms"] > 0 and len(r["timings"]) >= 8
    assert ctx.config == r["config"]
    assert r["config"]["fused"] in (0, 1, 2) and 0 <= r["config"]["classify_shape"] <= 5
    # the tuned configuration extracts the same mesh
    n = ref.num_vertices
    o = {"soup": torch.zeros((n, 28), dtype=torch.uint8, device="cuda"),
         "normals": torch.zeros((n, 3), dtype=torch.float32, device="cuda")}
    mcg.extract_into(vol, 0.01, o, n, ctx=ctx)
    c = mcg.counts(ctx)
    torch.cuda.synchronize()
    assert c["status"] == 0 and c["vertices"] == n
    assert torch.equal(o["soup"], ref.soup) and torch.equal(o["normals"], ref.normals)
    # a second context of the same shape class takes the cached choice
    ctx2 = mcg.Context()
    r2 = tune.autotune(vol, 0.01, ctx=ctx2, path=path)
    assert r2["cached"] and ctx2.config == r["config"]
    ctx3 = mcg.Context()
    assert tune.apply_cached(ctx3, vol, path=path) == r["config"] and ctx3.config == r["config"]
    for x in (ctx, ctx2, ctx3):
        x.close()
