"""The oracle's ray caster (restating cu_kinect_fusion_v1.cu:551-659,
786-986) against closed forms: a fronto-parallel plane at a known depth and
the plane seen from the side, on CPU."""
import numpy as np

import oracle


def _plane_volume(n=64, zp=40.0, trunc=5.0, axis=2):
    """tsdf = clamp((zp - c) / trunc) along `axis` (free space towards c < zp),
    voxel (x, y, z) at grid coordinate (x, y, z), weights 1."""
    c = np.arange(n, dtype=np.float64)
    shape = [1, 1, 1]
    shape[2 - axis] = n
    f = np.clip((zp - c.reshape(shape)) / trunc, -1, 1) * np.ones((n, n, n))
    t = np.trunc(f * 32767).astype(np.int16)
    return np.stack([t, np.ones_like(t)], axis=-1)


def test_fronto_parallel_plane():
    vol = _plane_volume()
    g = 0.01
    k = oracle.intrinsic(40.0, 40.0, 15.5, 15.5)
    e = oracle.extrinsic(np.eye(3), [0.32, 0.32, 0.02])  # camera at grid (32, 32, 2), looking +z
    depth, nrm = oracle.raycast(vol, g, k, e, 32, 32)
    # the surface is grid z = 40: z-depth (40 - 2) cells
    assert np.all(depth > 0)
    assert np.abs(depth - 0.38).max() < 2e-4
    assert np.allclose(nrm[..., 2], -1.0, atol=1e-3) and np.abs(nrm[..., :2]).max() < 1e-3


def test_plane_seen_along_x():
    vol = _plane_volume(axis=0)  # surface at grid x = 40, free space at x < 40
    g = 0.01
    k = oracle.intrinsic(40.0, 40.0, 15.5, 15.5)
    # camera at grid (5, 32, 32) looking +x: camera z = world x
    R = np.stack([[0, 0, -1.0], [0, 1.0, 0], [1.0, 0, 0]], axis=1)  # columns: camera x, y, z in world
    e = oracle.extrinsic(R, [0.05, 0.32, 0.32])
    depth, nrm = oracle.raycast(vol, g, k, e, 32, 32)
    assert np.all(depth > 0)
    assert np.abs(depth - 0.35).max() < 2e-4
    # world normal (-1, 0, 0) in camera coordinates: R^T n
    n_cam = R.T @ np.array([-1.0, 0, 0])
    assert np.allclose(nrm.reshape(-1, 3), n_cam, atol=1e-3)


def test_miss_and_singular_camera():
    vol = _plane_volume()
    k = oracle.intrinsic(40.0, 40.0, 15.5, 15.5)
    # looking away from the plane: no crossing
    e = oracle.extrinsic(np.diag([1.0, -1.0, -1.0]), [0.32, 0.32, 0.02])
    depth, nrm = oracle.raycast(vol, 0.01, k, e, 32, 32)
    assert not depth.any() and not nrm.any()
    assert oracle.raycast(vol, 0.01, oracle.intrinsic(0.0, 40.0, 15.5, 15.5), e, 8, 8) is None
