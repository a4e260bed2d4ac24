"""Depth pyramid and ICP oracle (kf.cu:66-80, 226-261, 988-1301): known
answers for the pyramid step and the rotation, and the tracking property —
ICP from the identity recovers the known relative pose of two rendered
frames.  No GPU needed."""
import math

import numpy as np

import oracle
from icp_util import frames, pyramid_maps, rot_angle


def test_pyramid_down_known_answer():
    src = np.arange(36, dtype=np.float32).reshape(6, 6) / 100.0
    mask = np.full((6, 6), 255, np.uint8)
    mask[0, 1] = 0
    d, dm = oracle.pyramid_down(src, mask, (3, 3), sigma=0.1)
    # (0, 0): window rows 0..2, cols 0..2 clipped to < 3 (tx = min(2*0-2+5, 5) = 3);
    # (0, 1) masked; |v - 0| < 0.1 keeps 0.00, 0.02, 0.06, 0.07, 0.08 ... (< 0.1)
    win = [src[r, c] for r in range(3) for c in range(3) if mask[r, c] and abs(src[r, c] - src[0, 0]) < 0.1]
    assert d[0, 0] == np.float32(sum(np.float32(v) for v in win) / np.float32(len(win))) or \
        abs(d[0, 0] - np.mean(win)) < 1e-7
    assert dm.all()
    mask2 = mask.copy()
    mask2[2, 2] = 0
    d2, dm2 = oracle.pyramid_down(src, mask2, (3, 3), sigma=0.1)
    assert dm2[1, 1] == 0 and d2[1, 1] == 0  # the centre pixel (2, 2) is masked
    assert (oracle.float_data_to_mask(np.array([0.0, -0.0, 1e-30, 2.0], np.float32)) == [0, 0, 255, 255]).all()
    assert (oracle.float_mask_to_data(np.array([0, 255], np.uint8), np.array([3.0, 4.0])) == [0.0, 4.0]).all()


def test_so3_exp():
    w = np.array([0.1, -0.2, 0.3])
    R = np.zeros(9)
    oracle.lib().orc_so3_exp(w.ctypes.data_as(oracle.ctypes.c_void_p), R.ctypes.data_as(oracle.ctypes.c_void_p))
    R = R.reshape(3, 3).T  # column-major -> rows
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    ref = np.eye(3) + math.sin(th) / th * K + (1 - math.cos(th)) / th ** 2 * K @ K
    assert np.allclose(R, ref, atol=1e-15)
    v = np.array([0.3, 0.5, -0.7])
    assert np.allclose(R @ v, v + np.cross(w, v), atol=0.1)  # first order: R v ~ v + w x v


def _icp_levels(maps1, maps2, start, it_max=(15, 11, 8), bilinear=False):
    e = start
    for lv in (2, 1, 0):
        v1, n1, k, _ = maps1[lv]
        v2, n2, _, _ = maps2[lv]
        ok, (r, t), iters, _ = oracle.icp(math.cos(math.radians(20)), 0.10, math.radians(20), 0.10, it_max[lv], k, e,
                                          v1, n1, v2, n2, bilinear)
        assert ok, lv
        e = oracle.Extrinsic()
        for i in range(9):
            e.r[i] = float(r[i])
        for i in range(3):
            e.t[i] = float(t[i])
    return e


def test_icp_recovers_relative_pose():
    d1, d2, (R, t), (f, cx, cy) = frames(seed=1, step=1)
    m1, m2 = pyramid_maps(d1, f, cx, cy), pyramid_maps(d2, f, cx, cy)
    for bilinear in (False, True):
        e = _icp_levels(m1, m2, oracle.extrinsic(np.eye(3), np.zeros(3)), bilinear=bilinear)
        Re = np.array(list(e.r)).reshape(3, 3).T
        te = np.array(list(e.t))
        assert rot_angle(R) > 0.02  # a real motion: ~1.8 degrees, ~4 cm
        assert rot_angle(Re.T @ R) < 2e-3, bilinear
        assert np.linalg.norm(te - t) < 2e-3, bilinear
