"""Two depth frames of the blended-spheres scene and their vertex / normal
pyramids (three levels, as the fusion loop builds them, kf.cu:2105-2145),
for the ICP tests."""
import numpy as np

import oracle
from marching_cube_gb300 import synthetic

W, H, F = 160, 120, 120.0
CX, CY = (W - 1) / 2.0, (H - 1) / 2.0


def rel_pose(P1, P2):
    """camera-2 -> camera-1 of two camera -> global poses (R, t)."""
    R1, t1 = P1
    R2, t2 = P2
    R = R1.T @ R2
    t = R1.T @ (t2 - t1)
    return R, t


def frames(seed=1, step=1, n=200, w=W, h=H, f=F):
    scene = synthetic.BlendedSpheres(seed=seed)
    P1, P2 = scene.pose(0, n), scene.pose(step, n)
    cx, cy = (w - 1) / 2.0, (h - 1) / 2.0
    d1 = scene.depth_frame(*P1, w=w, h=h, fx=f, fy=f, cx=cx, cy=cy).cpu().numpy().astype(np.float32)
    d2 = scene.depth_frame(*P2, w=w, h=h, fx=f, fy=f, cx=cx, cy=cy).cpu().numpy().astype(np.float32)
    return d1, d2, rel_pose(P1, P2), (f, cx, cy)


def pyramid_maps(depth, f, cx, cy, levels=3, sigma=0.06):
    """[(vertex, normal)] per level, oracle arithmetic: masks, pyramid_down,
    mask_to_data, then vmap / nmap with the halved intrinsic."""
    maps, d = [], depth
    k = oracle.intrinsic(f, f, cx, cy)
    for lv in range(levels):
        if lv > 0:
            m = oracle.float_data_to_mask(d)
            h, w = d.shape
            d, dm = oracle.pyramid_down(d, m, (h >> 1, w >> 1), sigma)
            d = oracle.float_mask_to_data(dm, d)
            k = oracle.intrinsic(k.fx / 2, k.fy / 2, k.cx / 2, k.cy / 2)
        v = oracle.meter_to_vertex(k, d)
        maps.append((v, oracle.vertex_to_normal(v), k, d))
    return maps


def rot_angle(R):
    c = (np.trace(R) - 1.0) / 2.0
    return float(np.arccos(np.clip(c, -1.0, 1.0)))
