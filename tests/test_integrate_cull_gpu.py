"""Integrate's row culling (each voxel row's candidate x interval from the
frustum and the frame's largest depth) never drops an update: the volume
after integration equals the oracle's (which tests every voxel) bit for bit,
for poses whose rotation makes a row parallel to a frustum plane (axis-
aligned, exact zeros in the rotation), cameras inside and outside the
volume looking in every axis direction, depths far beyond the volume, an
all-invalid frame, and a frame with non-finite depths."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N, W, H = 48, 160, 120
F = 131.25
EXTENT = 3.0


def _rot(axis_perm, signs):
    R = np.zeros((3, 3))
    for i, (a, sgn) in enumerate(zip(axis_perm, signs)):
        R[a, i] = sgn
    if np.linalg.det(R) < 0:
        R[:, 0] *= -1
    return R


def _poses():
    rng = np.random.default_rng(4)
    out = []
    c = EXTENT / 2
    # axis-aligned cameras (rotation entries exactly 0 / +-1), inside and outside
    for perm in [(0, 1, 2), (1, 2, 0), (2, 0, 1)]:
        for signs in [(1, 1, 1), (-1, 1, -1)]:
            R = _rot(perm, signs)
            for t in ([c, c, c], [c + 0.4, c - 0.3, c + 0.2], [-0.5, c, c], [c, 3.6, c]):
                out.append((R, np.array(t, float)))
    # random rotations and positions
    for _ in range(6):
        q = rng.standard_normal(4)
        q /= np.linalg.norm(q)
        a, b, cq, d = q
        R = np.array([[a * a + b * b - cq * cq - d * d, 2 * (b * cq - a * d), 2 * (b * d + a * cq)],
                      [2 * (b * cq + a * d), a * a - b * b + cq * cq - d * d, 2 * (cq * d - a * b)],
                      [2 * (b * d - a * cq), 2 * (cq * d + a * b), a * a - b * b - cq * cq + d * d]])
        out.append((R, rng.uniform(-1.0, 4.0, 3)))
    return out


@pytest.mark.parametrize("vtype", [torch.int16, torch.float32])
def test_culling_keeps_every_update(mcg, orc, vtype):
    rng = np.random.default_rng(11)
    grid_s = EXTENT / N
    trunc = 3 * grid_s
    k = mcg.intrinsic(F, F, (W - 1) / 2.0, (H - 1) / 2.0)
    ko = orc.intrinsic(F, F, (W - 1) / 2.0, (H - 1) / 2.0)
    v = mcg.voxel_new((N, N, N), trunc, trunc, grid_s, dtype=vtype)
    ref = v.data.cpu().numpy().copy()
    frames = []
    for i, (R, t) in enumerate(_poses()):
        kind = i % 4
        if kind == 0:
            m = rng.uniform(0.2, 2.0, (H, W)).astype(np.float32)          # depths inside the range
        elif kind == 1:
            m = rng.uniform(0.2, 9.0, (H, W)).astype(np.float32)          # far beyond the volume
        elif kind == 2:
            m = np.where(rng.random((H, W)) < 0.5, rng.uniform(0.5, 1.5, (H, W)), 0.0).astype(np.float32)
        else:
            m = np.zeros((H, W), np.float32)                               # nothing valid
        frames.append((R, t, m))
    # one frame with non-finite depths (the depth bound then culls nothing)
    m = rng.uniform(0.3, 1.8, (H, W)).astype(np.float32)
    m[3, 5] = -1.0
    m[7, 9] = np.nan
    frames.append((np.eye(3), np.array([EXTENT / 2, EXTENT / 2, -0.2]), m))
    for R, t, m in frames:
        mcg.volumetric_integration(v, k, mcg.extrinsic(R, t), torch.from_numpy(m).cuda())
        orc.integrate(ref, trunc, trunc, grid_s, ko, orc.extrinsic(R, t), m)
    got = v.data.cpu().numpy()
    if vtype == torch.float32:
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    else:
        assert np.array_equal(got, ref)
    assert (ref[..., 1] != 0).mean() > 0.05
