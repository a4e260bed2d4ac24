"""Helpers shared by the marching-cubes tests: run the CUDA path through the
C ABI and bring its output into the oracle's canonical order."""
import numpy as np
import torch

VERTEX_DTYPE = np.dtype([("pos", "<f4", (3,)), ("vox", "<i4", (3,)), ("tsdf", "<i2"), ("w", "<i2")])


def gpu_extract(mcg, vol_np, cell, canonical=True, **kw):
    vol = torch.from_numpy(np.ascontiguousarray(vol_np)).cuda()
    mesh = mcg.extract(vol, cell, soup=True, normals=True, vi2vox=True, ver_voxel=True, tri_cube=True, **kw)
    torch.cuda.synchronize()
    return mesh_arrays(mesh, canonical)


def mesh_arrays(mesh, canonical=True):
    """A mesh with every output (soup, normals, vi2vox, ver_voxel, tri_cube)
    as numpy arrays, triangles in the oracle's canonical order (by cube id,
    stable) when `canonical`."""
    n = mesh.num_vertices
    soup = mesh.soup.cpu().numpy().reshape(-1).view(VERTEX_DTYPE) if n else np.zeros(0, VERTEX_DTYPE)
    nrm = mesh.normals.cpu().numpy() if n else np.zeros((0, 3), np.float32)
    v2v = mesh.vi2vox.cpu().numpy() if n else np.zeros((0, 3), np.int32)
    tc = mesh.tri_cube.cpu().numpy() if n else np.zeros(0, np.int64)
    vv = mesh.ver_voxel.cpu().numpy()
    out = {"soup": soup, "normals": nrm, "vi2vox": v2v, "ver_voxel": vv, "tri_cube": tc,
           "counts": mesh.counts}
    if canonical and n:
        order = np.argsort(tc, kind="stable")
        idx = (order[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
        out["soup"] = soup[idx]
        out["normals"] = nrm[idx]
        out["vi2vox"] = v2v[idx]
        out["tri_cube"] = tc[order]
    return out


def assert_same_mesh(g, o):
    assert len(g["soup"]) == len(o["soup"])
    assert np.array_equal(g["tri_cube"], o["tri_cube"])
    # whole 28-byte records bit-exact (positions, vox_pos, tsdf, w)
    assert np.array_equal(g["soup"].view(np.uint8), o["soup"].view(np.uint8))
    assert np.array_equal(g["normals"].view(np.uint32), o["normals"].view(np.uint32))
    assert np.array_equal(g["vi2vox"], o["vi2vox"])
    assert np.array_equal(g["ver_voxel"], o["ver_voxel"])
