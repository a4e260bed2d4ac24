"""Shared set-up of the adjoint tests: a blended-spheres scene fused into a
float32 volume, its camera and the oracle's view of the same inputs."""
import numpy as np
import torch

import oracle
from marching_cube_gb300 import synthetic


class Scene:
    def __init__(self, n=32, frames=3, w=80, h=60, seed=0, trunc_voxels=3.0):
        self.n = n
        self.shape = (n, n, n)
        self.grid_s = 1.0 / n
        self.min_t = self.max_t = trunc_voxels * self.grid_s
        f = 262.5 * w / 320.0
        self.fx = self.fy = f
        self.cx, self.cy = (w - 1) / 2.0, (h - 1) / 2.0
        self.w, self.h = w, h
        sc = synthetic.BlendedSpheres(seed=seed)
        self.scene = sc
        depth, poses = sc.frames(frames, w=w, h=h, fx=f, fy=f)
        # the path takes float32 metres; the oracle gets the same values
        self.depth = depth.numpy().astype(np.float32)
        self.poses = poses
        self.k_orc = oracle.intrinsic(self.fx, self.fy, self.cx, self.cy)
        self.e_orc = [oracle.extrinsic(R, t) for R, t in poses]

    def pose_rows(self):
        """(K, 12) float32: rotation column-major, then t."""
        return np.stack([np.array(list(e.r) + list(e.t), np.float32) for e in self.e_orc])

    def integrate_f64(self, depth=None, **kw):
        d = self.depth if depth is None else depth
        return oracle.integrate_seq_f64(self.shape, self.min_t, self.max_t, self.grid_s, self.k_orc, self.e_orc,
                                        d.astype(np.float64) if d.dtype != np.float64 else d, **kw)

    def integrate_f32(self):
        """FP32 mirror of the same frames (float2 volume), frame by frame."""
        vol = np.zeros(self.shape + (2,), np.float32)
        vol[..., 0] = -1.0
        for f in range(len(self.e_orc)):
            oracle.integrate(vol, self.min_t, self.max_t, self.grid_s, self.k_orc, self.e_orc[f], self.depth[f])
        return vol


def smooth_volume(n=24, seed=0):
    """float2 volume: clamped blended-spheres SDF / (3 cells), weight 1."""
    sc = synthetic.BlendedSpheres(seed=seed)
    cell = 1.0 / n
    i = (torch.arange(n, dtype=torch.float64) + 0.5) * cell
    z, y, x = torch.meshgrid(i, i, i, indexing="ij")
    p = torch.stack([x, y, z], dim=-1).reshape(-1, 3)
    f = torch.clamp(sc.sdf(p) / (3 * cell), -1, 1).reshape(n, n, n).numpy().astype(np.float32)
    vol = np.stack([f, np.ones_like(f)], axis=-1)
    return vol, cell


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
