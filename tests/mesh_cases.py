"""Soups for the mesh-writer tests: 28-byte vertex_voxel records built from
positions, voxel coordinates, tsdf and weights."""
import numpy as np


def soup(pos, vox=None, tsdf=None, w=None):
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    n = len(pos)
    rec = np.zeros((n, 28), np.uint8)
    rec[:, 0:12] = pos.view(np.uint8).reshape(n, 12)
    vox = np.zeros((n, 3), np.int32) if vox is None else np.asarray(vox, np.int32).reshape(n, 3)
    rec[:, 12:24] = vox.view(np.uint8).reshape(n, 12)
    t = np.zeros(n, np.int16) if tsdf is None else np.asarray(tsdf, np.int16)
    ww = np.zeros(n, np.int16) if w is None else np.asarray(w, np.int16)
    rec[:, 24:26] = t.view(np.uint8).reshape(n, 2)
    rec[:, 26:28] = ww.view(np.uint8).reshape(n, 2)
    return rec


def crafted():
    """Key merges across different floats, rounding ties, negative zeros,
    degenerate triangles, the first occurrence's normal winning."""
    p = np.array([
        [0.1, 0.2, 0.3], [0.10001, 0.2, 0.3], [1.0, 2.0, 3.0],        # 0 and 1 merge: a dropped triangle
        [0.03125, 0.0078125, 1.5], [0.0312, 0.0078125, 1.5], [2.0, 2.0, 2.0],  # tie 312.5 -> "0.0312"
        [-0.00001, 0.5, 0.5], [0.0, 0.5, 0.5], [-0.0, 0.5, 0.5],       # "-0.0000" vs "0.0000"
        [99.99995, 12.34565, 0.00005], [99.9999, 12.3457, 0.0001], [7.0, 8.0, 9.0],
        [0.1, 0.2, 0.3], [1.0, 2.0, 3.0], [2.0, 2.0, 2.0],             # all seen before
    ], np.float32)
    n = np.array([[0.0, -0.0, 1.0], [1e-7, -1e-7, 0.5], [-0.6, 0.8, 0.0]] * 5, np.float32)
    n[3] = [1 / 128, -3 / 128, 5 / 128]  # x * 10^6 ends in .5 exactly: ties to even
    vox = np.arange(45, dtype=np.int32).reshape(15, 3) - 7
    tsdf = np.array([-32766, 32766, 0, 1, -1, 5, 100, -100, 7, 8, 9, 10, 11, 12, 13], np.int16)
    w = np.array([0, 1, -1, 65535 - 65536, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12], np.int16)
    return soup(p, vox, tsdf, w), n
