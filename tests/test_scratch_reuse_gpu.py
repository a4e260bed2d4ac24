"""One context across calls that share its scratch.

The count phase's per-chunk sums are cleared by the scan that read them, the
generate launch resets its own work counter when its last CTA leaves, and the
totals reach the host through mapped memory written by the kernels.  These
tests chain calls that would expose a sum, counter or total left behind by
the call before."""
import ctypes

import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic
from mc_util import VERTEX_DTYPE, assert_same_mesh, gpu_extract

pytestmark = pytest.mark.gpu


def _classify(mcg, ctx, vol_t, cell):
    cv = mcg._cvol(vol_t, cell)
    ctx.check(mcg._lib.mcg_mc_classify(ctx.handle, ctypes.byref(cv), None), "mcg_mc_classify")
    return cv


def _generate(mcg, ctx, cv, vol_t, n):
    nz, ny, nx, _ = vol_t.shape
    o = mcg._alloc_outputs(n, nx * ny * nz, vol_t.device, True, True, False, False, True)
    mo = mcg._mesh_out(o, n)
    ctx.check(mcg._lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), None), "mcg_mc_generate")
    torch.cuda.synchronize()
    return o


def test_counts_of_a_classify_without_generate(mcg, orc):
    ctx = mcg.Context(0)
    cell = 0.01
    for shape, seed in [((40, 70, 150), 11), ((33, 64, 200), 12), ((40, 70, 150), 13)]:
        vol = synthetic.random_volume(shape, seed=seed)
        _classify(mcg, ctx, torch.from_numpy(vol).cuda(), cell)
        c = mcg.counts(ctx)
        occ, tri = orc.mc_count(vol)
        assert (c["occupied"], c["triangles"], c["vertices"], c["status"]) == (occ, tri, 3 * tri, 0)
    ctx.close()


def test_generate_twice_after_one_classify(mcg, orc):
    ctx = mcg.Context(0)
    cell = 0.01
    vol = synthetic.sphere_volume(128, seed=0)
    vt = torch.from_numpy(vol).cuda()
    cv = _classify(mcg, ctx, vt, cell)
    n = mcg.counts(ctx)["vertices"]
    first = _generate(mcg, ctx, cv, vt, n)
    second = _generate(mcg, ctx, cv, vt, n)
    c = mcg.counts(ctx)
    assert c["status"] == 0 and c["vertices"] == n
    assert torch.equal(first["soup"], second["soup"])
    assert torch.equal(first["normals"].view(torch.int32), second["normals"].view(torch.int32))
    assert torch.equal(first["tri_cube"], second["tri_cube"])
    # and the soup is the oracle's
    o = orc.mc_extract(vol, cell)
    tc = first["tri_cube"].cpu().numpy()
    order = np.argsort(tc, kind="stable")
    idx = (order[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
    soup = first["soup"].cpu().numpy().reshape(-1).view(VERTEX_DTYPE)[idx]
    assert np.array_equal(soup.view(np.uint8), o["soup"].view(np.uint8))
    ctx.close()


def test_indexed_then_soup_on_one_context(mcg, orc):
    ctx = mcg.Context(0)
    cell = 0.0037
    a = synthetic.sphere_volume(96, seed=1)
    b = synthetic.random_volume((30, 41, 170), seed=14)
    mcg.extract_indexed(torch.from_numpy(a).cuda(), cell, ctx=ctx)
    torch.cuda.synchronize()
    g = gpu_extract(mcg, b, cell, ctx=ctx)
    assert_same_mesh(g, orc.mc_extract(b, cell))
    # and the indexed path after a soup extraction
    im = mcg.extract_indexed(torch.from_numpy(a).cuda(), cell, ctx=ctx)
    torch.cuda.synchronize()
    occ, tri = orc.mc_count(a)
    assert im.counts["triangles"] == tri and im.counts["occupied"] == occ
    ctx.close()
