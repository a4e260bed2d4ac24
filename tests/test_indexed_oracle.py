"""The oracle's view of the indexed mesh (edge keys of the soup's vertices)
on CPU: a closed sphere is a 2-manifold of Euler characteristic 2 once the
soup's vertices are merged by grid edge, and every key is a crossed edge."""
import numpy as np

import oracle
from marching_cube_gb300 import synthetic


def _euler(tris):
    V = len(np.unique(tris))
    e = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]), axis=1)
    E = len(np.unique(e, axis=0))
    return V - E + len(tris), e


def test_sphere_is_closed_manifold():
    vol = synthetic.sphere_volume(40, radius=12.0, trunc=4.0, seed=1)
    keys, tris = oracle.mc_indexed(vol)
    chi, e = _euler(tris)
    assert chi == 2
    # every undirected edge is shared by exactly two triangles
    _, cnt = np.unique(e, axis=0, return_counts=True)
    assert np.all(cnt == 2)
    # no degenerate triangle after the merge
    assert np.all((tris[:, 0] != tris[:, 1]) & (tris[:, 1] != tris[:, 2]) & (tris[:, 0] != tris[:, 2]))


def test_keys_are_crossed_edges():
    vol = synthetic.random_volume((9, 11, 13), seed=4)
    keys, _ = oracle.mc_indexed(vol)
    nz, ny, nx, _ = vol.shape
    li, axis = keys // 3, keys % 3
    step = np.where(axis == 0, 1, np.where(axis == 1, nx, nx * ny))
    t = vol[..., 0].reshape(-1)
    assert np.all((t[li] < 0) != (t[li + step] < 0))
    pos, nrm, v2v = oracle.mc_edge_vertices(vol, 0.01, keys)
    # the vertex lies on its edge
    x, y, z = li % nx, (li // nx) % ny, li // (nx * ny)
    lo = (np.stack([x, y, z], 1) + 0.5) * 0.01
    d = pos - lo
    assert np.all(d >= -1e-6) and np.all(d <= 0.01 + 1e-6)
