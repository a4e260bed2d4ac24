"""The rule the indexed count phase rests on, checked with the oracle on CPU:
a brick (32 x 8 x 8 cubes) owns a vertex (the lower voxel of a crossed grid
edge that a valid cube around it uses) only when the brick itself or one of
its neighbours at -x, -y, -z, -x-y, -x-z, -y-z has triangles.  The indexed
count pass counts owned edges of exactly those bricks."""
import numpy as np
import pytest

import oracle
from marching_cube_gb300 import synthetic

BX, BY, BZ = 32, 8, 8


def _bricks(vol):
    nz, ny, nx, _ = vol.shape
    nbx, nby, nbz = (nx - 1 + BX - 1) // BX, (ny - 1 + BY - 1) // BY, (nz - 1 + BZ - 1) // BZ
    _, nv = oracle.mc_classify(vol)  # soup vertices per cube, (nz-1, ny-1, nx-1)
    tris = np.zeros((nbz, nby, nbx), np.int64)
    cz, cy, cx = np.nonzero(nv)
    np.add.at(tris, (cz // BZ, cy // BY, cx // BX), nv[cz, cy, cx] // 3)
    keys, _ = oracle.mc_indexed(vol)
    li = keys // 3
    x, y, z = li % nx, (li // nx) % ny, li // (nx * ny)
    # the brick holding the lower voxel; the last brick along an axis also
    # owns voxel n - 1 when the brick grid stops one short
    owner = (np.minimum(z // BZ, nbz - 1), np.minimum(y // BY, nby - 1), np.minimum(x // BX, nbx - 1))
    owned = np.zeros_like(tris)
    np.add.at(owned, owner, 1)
    return tris, owned


def _candidates(tris):
    cand = np.zeros(tris.shape, bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                if dx and dy and dz:
                    continue
                t = np.zeros_like(cand)
                t[dz:, dy:, dx:] = tris[:tris.shape[0] - dz, :tris.shape[1] - dy, :tris.shape[2] - dx] > 0
                cand |= t
    return cand


CASES = [
    ("random", lambda: synthetic.random_volume((19, 27, 70), seed=1)),
    ("random_sparse_weights", lambda: synthetic.random_volume((33, 17, 65), seed=2, p_zero_weight=0.4)),
    ("sphere", lambda: synthetic.sphere_volume(48, radius=17.0, trunc=3.0, seed=3)),
    ("batch_volume", lambda: synthetic.batch_volumes(3, seed=5, lo=20, hi=80)[2].numpy()),
]


@pytest.mark.parametrize("name", [c[0] for c in CASES])
def test_owned_vertices_lie_in_candidate_bricks(name):
    vol = dict(CASES)[name]()
    tris, owned = _bricks(vol)
    assert owned.sum() > 0
    cand = _candidates(tris)
    assert np.all(cand[owned > 0]), "a brick owns vertices but no brick around it has triangles"


def test_candidates_prune_empty_space():
    # a small sphere in a large volume: most bricks are far from the surface
    vol = synthetic.sphere_volume(96, radius=10.0, trunc=3.0, seed=4)
    tris, owned = _bricks(vol)
    cand = _candidates(tris)
    assert np.all(cand[owned > 0])
    assert cand.sum() < cand.size // 4
