"""The fused extraction (one persistent launch: count, look-back offsets and
generation from the count pass's tiles) against the count + generate
launches and the oracle: every output bit for bit, in the same order, with
capacity truncation, on volumes whose work items span many look-back
groups, on consecutive calls on one context (the per-launch epochs of the
look-back state, the totals it accumulates), mixed with two-launch calls on
the same context, and the fused launch's state rules (generate / backward
need a count phase)."""
import ctypes

import pytest
import torch

from marching_cube_gb300 import _capi, synthetic
from mc_util import assert_same_mesh, mesh_arrays

pytestmark = pytest.mark.gpu

KEYS = ("soup", "normals", "vi2vox", "ver_voxel", "tri_cube")


def _outputs(n, nvox):
    n = max(n, 3)
    return {"soup": torch.zeros((n, 28), dtype=torch.uint8, device="cuda"),
            "normals": torch.zeros((n, 3), dtype=torch.float32, device="cuda"),
            "vi2vox": torch.zeros((n, 3), dtype=torch.int32, device="cuda"),
            "ver_voxel": torch.full((nvox,), 77, dtype=torch.int16, device="cuda"),
            "tri_cube": torch.zeros((n // 3,), dtype=torch.int64, device="cuda")}


def _extract(mcg, ctx, vol, cell, n, cap, mode):
    ctx.set_config(fused=mode)
    nz, ny, nx, _ = vol.shape
    o = _outputs(n, nx * ny * nz)
    cv = _capi.Volume(vol.data_ptr(), nx, ny, nz, 0, float(cell))
    mo = _capi.MeshOut(*(o[k].data_ptr() for k in KEYS), cap)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ctx.check(mcg._lib.mcg_mc_extract(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "mcg_mc_extract")
    c = _capi.MeshCounts()
    st = mcg._lib.mcg_mc_counts(ctx.handle, ctypes.byref(c))
    torch.cuda.synchronize()
    return o, c, st


def _same_both(mcg, vol, cell, cap_frac=None, mode=1):
    """The fused launch (mode 1: 4-brick items, 2: 2-brick items) against the
    two launches, same capacity."""
    a, b = mcg.Context(), mcg.Context()
    n = mcg.extract(vol, cell).num_vertices
    cap = n if cap_frac is None else int(n * cap_frac)
    o1, c1, s1 = _extract(mcg, a, vol, cell, n, cap, mode)
    o2, c2, s2 = _extract(mcg, b, vol, cell, n, cap, 0)
    assert s1 == s2 and (c1.occupied, c1.triangles, c1.vertices, c1.active_bricks) == \
        (c2.occupied, c2.triangles, c2.vertices, c2.active_bricks)
    for k in KEYS:
        assert torch.equal(o1[k], o2[k]), k
    a.close()
    b.close()
    return n, s1


@pytest.mark.parametrize("mode", [1, 2])
def test_fused_matches_two_pass_and_oracle(mcg, orc, mode):
    vol = synthetic.sphere_volume(160, radius=50.0, seed=3)
    t = torch.from_numpy(vol).cuda()
    n, st = _same_both(mcg, t, 0.01, mode=mode)
    assert n > 10000 and st == 0
    ctx = mcg.Context()
    ctx.set_config(fused=mode)
    o = _outputs(n, t.shape[0] * t.shape[1] * t.shape[2])
    mcg.extract_into(t, 0.01, o, n, ctx=ctx)
    torch.cuda.synchronize()
    m = mcg.Mesh(o["soup"][:n], o["normals"][:n], o["vi2vox"][:n], o["ver_voxel"], o["tri_cube"][:n // 3],
                 mcg.counts(ctx))
    assert_same_mesh(mesh_arrays(m), orc.mc_extract(vol, 0.01))
    ctx.close()


@pytest.mark.parametrize("mode", [1, 2])
def test_fused_many_groups_and_odd_sizes(mcg, mode):
    # more items than one window of look-back groups reaches, edges that are
    # not whole bricks or items, weight-0 holes, sentinel regions
    for shape, seed in [((70, 90, 300), 1), ((48, 40, 260), 2), ((41, 64, 388), 4), ((20, 12, 100), 6)]:
        v = synthetic.random_volume(shape, seed=seed, p_zero_weight=0.02, sentinel_frac=0.3)
        _same_both(mcg, torch.from_numpy(v).cuda(), 0.02, mode=mode)
    _same_both(mcg, synthetic.stress_volume(256, seed=5, n_spheres=40), 1.0 / 256, mode=mode)


@pytest.mark.parametrize("mode", [1, 2])
def test_fused_capacity_truncation(mcg, mode):
    vol = torch.from_numpy(synthetic.sphere_volume(140, radius=45.0, seed=6)).cuda()
    n, st = _same_both(mcg, vol, 0.01, cap_frac=0.37, mode=mode)
    assert st == mcg.MCG_ERR_CAPACITY


def test_fused_consecutive_calls_and_state(mcg):
    ctx = mcg.Context()
    vols = [torch.from_numpy(synthetic.sphere_volume(n, radius=n * 0.3, seed=n)).cuda() for n in (160, 200, 176)]
    refs = [mcg.extract(v, 0.01, soup=True, normals=True) for v in vols]
    # fused calls on one context, with a two-launch call between some of them
    for k, (v, ref) in enumerate(zip(vols + vols, refs + refs)):
        n = ref.num_vertices
        ctx.set_config(fused=[1, 2, 1, 0, 2, 1][k])
        o = {"soup": torch.zeros((n, 28), dtype=torch.uint8, device="cuda"),
             "normals": torch.zeros((n, 3), dtype=torch.float32, device="cuda")}
        mcg.extract_into(v, 0.01, o, n, ctx=ctx)
        c = mcg.counts(ctx)
        torch.cuda.synchronize()
        assert c["status"] == 0 and c["vertices"] == n and c["triangles"] == ref.num_triangles, (k, c, n)
        assert c["occupied"] == ref.counts["occupied"] and c["active_bricks"] == ref.counts["active_bricks"]
        assert torch.equal(o["soup"], ref.soup) and torch.equal(o["normals"], ref.normals)
    # the fused launch keeps no brick list: generate needs a count phase first
    v = vols[0]
    cv = _capi.Volume(v.data_ptr(), v.shape[2], v.shape[1], v.shape[0], 0, 0.01)
    mo = _capi.MeshOut(None, None, None, None, None, 0)
    assert ctx.config["fused"] == 1
    st = mcg._lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), None)
    assert st == mcg.MCG_ERR_STATE
    ctx.close()


def test_config_round_trip_and_validation(mcg):
    ctx = mcg.Context()
    assert ctx.config == {"fused": 0, "classify_shape": 4, "gen_fixed_rounds": 3}
    ctx.set_config(classify_shape=2, gen_fixed_rounds=0, fused=0)
    assert ctx.config == {"fused": 0, "classify_shape": 2, "gen_fixed_rounds": 0}
    with pytest.raises(mcg.MCGError):
        ctx.set_config(classify_shape=6)
    with pytest.raises(mcg.MCGError):
        ctx.set_config(fused=3)
    with pytest.raises(KeyError):
        ctx.set_config(stages=2)
    ctx.close()
