"""The opt-in timing of the classify kernel: nothing to report before a
timed count phase, a positive duration after one, and the counts of a timed
count phase are the oracle's."""
import ctypes

import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_count_kernel_timing(mcg, orc):
    ctx = mcg.Context(0)
    ms = ctypes.c_float(0.0)
    assert mcg._lib.mcg_mc_count_kernel_ms(ctx.handle, ctypes.byref(ms)) == mcg.MCG_ERR_STATE
    vol = synthetic.sphere_volume(128, seed=3)
    cv = mcg._cvol(torch.from_numpy(vol).cuda(), 0.01)
    ctx.check(mcg._lib.mcg_set_kernel_timing(ctx.handle, 1), "timing on")
    ctx.check(mcg._lib.mcg_mc_classify(ctx.handle, ctypes.byref(cv), None), "classify")
    ctx.check(mcg._lib.mcg_mc_count_kernel_ms(ctx.handle, ctypes.byref(ms)), "kernel ms")
    assert 0.0 < ms.value < 1000.0
    c = mcg.counts(ctx)
    occ, tri = orc.mc_count(vol)
    assert (c["occupied"], c["triangles"], c["status"]) == (occ, tri, 0)
    ctx.check(mcg._lib.mcg_set_kernel_timing(ctx.handle, 0), "timing off")
    ctx.close()
