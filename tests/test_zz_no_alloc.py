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

MCG_ERR_CAPACITY = 2
MCG_ERR_TOO_LARGE = 8


def _outputs(n, nvox):
    n = max(n, 3)
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


def _run_both(mcg, vol, cell, cap_frac=None):
    """Extracts `vol` (a device tensor) through both entry points with the
    same capacity (all vertices, or the fraction cap_frac of them) and checks
    that counts, status and every output array agree bit for bit."""
    lib = mcg._lib
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
    cap = n if cap_frac is None else int(n * cap_frac)
    ref = _outputs(n, nx * ny * nz)
    mo = _mesh_out(ref, cap)
    assert lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), stream) == 0
    st_ref = lib.mcg_mc_counts(ctx.handle, ctypes.byref(c_ref))
    torch.cuda.synchronize()
    ctx.close()
    # no-allocation entry point
    got = _outputs(n, nx * ny * nz)
    mo2 = _mesh_out(got, cap)
    c = _capi.MeshCounts()
    st = lib.mcg_mc_extract_noalloc(ctypes.byref(cv), ctypes.byref(mo2), ctypes.byref(c), stream)
    torch.cuda.synchronize()
    assert st == st_ref == c.status == c_ref.status, (st, st_ref, lib.mcg_status_string(st))
    assert (c.occupied, c.triangles, c.vertices, c.active_bricks) == \
        (c_ref.occupied, c_ref.triangles, c_ref.vertices, c_ref.active_bricks)
    for k in ref:
        # bit-exact, the tolerance of every other extraction test
        assert torch.equal(got[k], ref[k]), k
    return n, st


def _float2_volume(shape, seed):
    rng = np.random.default_rng(seed)
    v = np.stack([rng.standard_normal(shape).astype(np.float32),
                  (rng.random(shape) > 0.05).astype(np.float32)], axis=-1)
    return torch.from_numpy(v).cuda()


def test_noalloc_matches_extract_on_consecutive_calls(mcg):
    cuda = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    n1, _ = _run_both(mcg, cuda(synthetic.sphere_volume(96, radius=30.0, seed=1)), 0.01)
    n2, _ = _run_both(mcg, cuda(synthetic.random_volume((23, 41, 70), seed=8)), 0.02)
    n3, _ = _run_both(mcg, _float2_volume((30, 20, 50), seed=4), 0.5)
    n4, _ = _run_both(mcg, cuda(synthetic.sphere_volume(40, radius=11.0, seed=2)), 0.01)
    n5, _ = _run_both(mcg, _float2_volume((17, 33, 64), seed=5), 0.25)
    assert min(n1, n2, n3, n4, n5) > 0


def test_noalloc_capacity_truncation(mcg):
    # a soup buffer for a third of the vertices: both entry points report the
    # capacity status, the full counts, and write the same prefix
    vol = torch.from_numpy(synthetic.sphere_volume(80, radius=25.0, seed=3)).cuda()
    n, st = _run_both(mcg, vol, 0.01, cap_frac=1.0 / 3.0)
    assert n > 0 and st == MCG_ERR_CAPACITY
    # and the next call with room for everything is whole again
    n2, st2 = _run_both(mcg, vol, 0.01)
    assert n2 == n and st2 == 0


def _sphere_torch(nx, ny, nz, radius, trunc=5.0):
    """(nz, ny, nx, 2) int16 sphere volume built on the device (the shape of
    synthetic.sphere_volume, weights constant 1)."""
    def ax(n):
        return torch.arange(n, device="cuda", dtype=torch.float32) + 0.5
    z, y, x = ax(nz)[:, None, None], ax(ny)[None, :, None], ax(nx)[None, None, :]
    sd = torch.sqrt((x - nx / 2) ** 2 + (y - ny / 2) ** 2 + (z - nz / 2) ** 2) - radius
    t = torch.trunc(torch.clamp(sd / trunc, -1.0, 1.0) * 32767).to(torch.int16)
    return torch.stack([t, torch.ones_like(t)], dim=-1).contiguous()


def test_noalloc_largest_volume(mcg):
    # 513^3 voxels = 16 x 64 x 64 = 65536 bricks: exactly the fixed limit
    vol = _sphere_torch(513, 513, 513, radius=200.0)
    n, st = _run_both(mcg, vol, 0.01)
    assert n > 0 and st == 0
    del vol
    torch.cuda.empty_cache()


def test_noalloc_rejects_oversized_volume(mcg):
    lib = mcg._lib
    small = torch.zeros((2, 2, 2, 2), dtype=torch.int16, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    mo = _capi.MeshOut(None, None, None, None, None, 0)
    # 600^3, and one brick column past the limit (514 x 513 x 513 = 17 x 64 x 64
    # bricks): rejected before anything is launched, so the small buffer is
    # never read
    for dims in [(600, 600, 600), (514, 513, 513)]:
        cv = _capi.Volume(small.data_ptr(), *dims, 0, 0.01)
        c = _capi.MeshCounts()
        st = lib.mcg_mc_extract_noalloc(ctypes.byref(cv), ctypes.byref(mo), ctypes.byref(c), stream)
        assert st == MCG_ERR_TOO_LARGE
        assert b"fixed scratch" in lib.mcg_status_string(st)
