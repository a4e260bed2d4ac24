"""mcg_mc_extract_noalloc: the extraction for callers that cannot allocate
device memory (memory owned by another allocator, or a loop that forbids
cudaMalloc once running).  It runs on a fixed static device scratch array,
so it is checked here against the context-based entry point (which
allocates its scratch) through the C ABI, on consecutive calls: the shared
array must not leak state from one call into the next.

This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from marching_cube_gb300 import _capi, synthetic

pytestmark = pytest.mark.gpu

MCG_ERR_TOO_LARGE = 8


def _outputs(n, nvox):
    return {
        "soup": torch.zeros((n, 28), dtype=torch.uint8, device="cuda"),
        "normals": torch.zeros((n, 3), dtype=torch.float32, device="cuda"),
        "vi2vox": torch.zeros((n, 3), dtype=torch.int32, device="cuda"),
        "ver_voxel": torch.full((nvox,), 123, dtype=torch.int16, device="cuda"),
        "tri_cube": torch.zeros((n // 3,), dtype=torch.int64, device="cuda"),
    }


def _mesh_out(o, cap):
    return _capi.MeshOut(o["soup"].data_ptr(), o["normals"].data_ptr(), o["vi2vox"].data_ptr(),
                         o["ver_voxel"].data_ptr(), o["tri_cube"].data_ptr(), cap)


def _run_both(mcg, vol_np, cell):
    lib = mcg._lib
    vol = torch.from_numpy(np.ascontiguousarray(vol_np)).cuda()
    nz, ny, nx, _ = vol.shape
    vt = 0 if vol.dtype == torch.int16 else 1
    cv = _capi.Volume(vol.data_ptr(), nx, ny, nz, vt, float(cell))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # existing entry point (context owns the scratch)
    ctx = mcg.Context()
    assert lib.mcg_mc_classify(ctx.handle, ctypes.byref(cv), stream) == 0
    c_ref = _capi.MeshCounts()
    assert lib.mcg_mc_counts(ctx.handle, ctypes.byref(c_ref)) == 0
    n = c_ref.vertices
    ref = _outputs(n, nx * ny * nz)
    mo = _mesh_out(ref, n)
    assert lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), stream) == 0
    torch.cuda.synchronize()
    ctx.close()
    # no-allocation entry point
    got = _outputs(n, nx * ny * nz)
    mo2 = _mesh_out(got, n)
    c = _capi.MeshCounts()
    st = lib.mcg_mc_extract_noalloc(ctypes.byref(cv), ctypes.byref(mo2), ctypes.byref(c), stream)
    assert st == 0, lib.mcg_status_string(st)
    torch.cuda.synchronize()
    assert (c.occupied, c.triangles, c.vertices, c.active_bricks) == \
        (c_ref.occupied, c_ref.triangles, c_ref.vertices, c_ref.active_bricks)
    for k in ref:
        # bit-exact, the tolerance of every other extraction test
        assert torch.equal(got[k], ref[k]), k
    return n


def test_noalloc_matches_extract_on_consecutive_calls(mcg):
    n1 = _run_both(mcg, synthetic.sphere_volume(96, radius=30.0, seed=1), 0.01)
    n2 = _run_both(mcg, synthetic.random_volume((23, 41, 70), seed=8), 0.02)
    n3 = _run_both(mcg, synthetic.sphere_volume(40, radius=11.0, seed=2), 0.01)
    assert n1 > 0 and n2 > 0 and n3 > 0


def test_noalloc_rejects_oversized_volume(mcg):
    lib = mcg._lib
    small = torch.zeros((2, 2, 2, 2), dtype=torch.int16, device="cuda")
    # 600^3 needs more bricks than the fixed scratch holds; rejected before any launch
    cv = _capi.Volume(small.data_ptr(), 600, 600, 600, 0, 0.01)
    mo = _capi.MeshOut(None, None, None, None, None, 0)
    c = _capi.MeshCounts()
    st = lib.mcg_mc_extract_noalloc(ctypes.byref(cv), ctypes.byref(mo), ctypes.byref(c),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == MCG_ERR_TOO_LARGE
    assert b"fixed scratch" in lib.mcg_status_string(st)
