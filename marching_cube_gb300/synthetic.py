"""Seeded synthetic inputs for the TSDF -> mesh workloads.

The reference measures on input files that are not part of it (512dim.vol,
1024dim.vol, sdf.txt); these generators stand in for them with the shapes,
sizes and value ranges of the workloads:

  sphere_volume   128^3 short2 sphere (r 40 voxels, truncation 5 voxels,
                  weights uniform in [1, 128]), cell 1 cm
  fusion_scene    20 random spheres (r 0.1-0.4 m) and axis-aligned boxes in
                  a 3 m cube, depth frames ray-cast from a camera orbiting at
                  1.5 m (pinhole 525/525/319.5/239.5, 640x480), Gaussian
                  noise sigma 2 mm, uint16 millimetres
  random_volume   small random short2 volumes for exhaustive parity cases
  stress_volume   1024^3 short2: union of 200 spheres (r 2-8 % of the side)
                  plus 3-octave gradient noise of amplitude 0.2 voxel added
                  to the signed distance before quantising (trunc 5 voxels,
                  scale 32767, weights uniform in [1, 128])
  blended_spheres smooth union (quadratic polynomial smooth-min, blend
                  radius k = 0.06 m) of 8 spheres in a 1 m cube, float depth
                  frames sphere-traced from a camera orbiting at 1.2 m
                  (pinhole 262.5/262.5/159.5/119.5, 320x240), for the
                  differentiable path

Randomness: numpy.random.default_rng(seed) for scene parameters and
torch.Generator(seed) for per-pixel noise.
"""
import math

import numpy as np
import torch

MAX_TSDF = 32766


def sphere_volume(n=128, radius=40.0, trunc=5.0, seed=0, weight_max=128, scale=32767, center=None):
    """(n, n, n, 2) int16: tsdf = trunc(clamp(sd/trunc, -1, 1) * scale)
    with sd the signed distance (voxel units) of voxel centres (i+0.5) to a
    sphere centred at n/2; w uniform integer in [1, weight_max]."""
    c = n / 2.0 if center is None else center
    i = np.arange(n, dtype=np.float64) + 0.5
    z, y, x = np.meshgrid(i, i, i, indexing="ij")
    sd = np.sqrt((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2) - radius
    t = np.trunc(np.clip(sd / trunc, -1.0, 1.0) * scale).astype(np.int16)
    rng = np.random.default_rng(seed)
    w = rng.integers(1, weight_max + 1, size=t.shape, dtype=np.int64).astype(np.uint16).view(np.int16)
    return np.stack([t, w], axis=-1)


def random_volume(shape, seed=0, p_zero_weight=0.05, sentinel_frac=0.1):
    """Random short2 volume (nz, ny, nx, 2) exercising every cube case,
    zero weights and the +-32766 sentinels."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    t = rng.integers(-32767, 32768, size=(nz, ny, nx), dtype=np.int64)
    s = rng.random((nz, ny, nx))
    t[s < sentinel_frac / 2] = MAX_TSDF
    t[(s >= sentinel_frac / 2) & (s < sentinel_frac)] = -MAX_TSDF
    w = rng.integers(1, 65536, size=(nz, ny, nx), dtype=np.int64)
    w[rng.random((nz, ny, nx)) < p_zero_weight] = 0
    return np.stack([t.astype(np.int16), w.astype(np.uint16).view(np.int16)], axis=-1)


def _mix32(h):
    """32-bit integer hash (multiply-xorshift) on int64 tensors holding
    values in [0, 2^32)."""
    m = 0xFFFFFFFF
    h = ((h ^ (h >> 16)) * 0x7FEB352D) & m
    h = ((h ^ (h >> 15)) * 0x846CA68B) & m
    return h ^ (h >> 16)


def gradient_noise(x, y, z, seed=0):
    """Perlin-style gradient noise (quintic fade 6t^5 - 15t^4 + 10t^3, one
    hashed unit gradient per lattice point) at float tensors x, y, z; roughly
    in [-1, 1]."""
    xi, yi, zi = torch.floor(x), torch.floor(y), torch.floor(z)
    fx, fy, fz = x - xi, y - yi, z - zi
    xi, yi, zi = xi.to(torch.int64), yi.to(torch.int64), zi.to(torch.int64)

    def fade(t):
        return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)

    u, v, w = fade(fx), fade(fy), fade(fz)
    out = torch.zeros_like(x)
    for c in range(8):
        cx, cy, cz = c & 1, (c >> 1) & 1, c >> 2
        h = _mix32(((xi + cx) * 73856093 ^ (yi + cy) * 19349663 ^ (zi + cz) * 83492791 ^ (seed * 2654435761))
                   & 0xFFFFFFFF)
        # gradient from three hashed bytes, normalised
        gx = ((h & 0xFF).to(x.dtype) / 127.5) - 1.0
        gy = (((h >> 8) & 0xFF).to(x.dtype) / 127.5) - 1.0
        gz = (((h >> 16) & 0xFF).to(x.dtype) / 127.5) - 1.0
        gn = torch.rsqrt(gx * gx + gy * gy + gz * gz + 1e-12)
        dot = (gx * (fx - cx) + gy * (fy - cy) + gz * (fz - cz)) * gn
        wgt = (u if cx else 1.0 - u) * (v if cy else 1.0 - v) * (w if cz else 1.0 - w)
        out += wgt * dot
    return out


def stress_volume(n=1024, seed=0, n_spheres=200, trunc=5.0, noise_amp=0.2, slab=32, device="cuda"):
    """(n, n, n, 2) int16 volume built slab by slab on `device`: signed
    distance (voxel units, voxel centres at i + 0.5) to the union of
    n_spheres spheres, plus 3 octaves of gradient noise (periods 32, 16, 8
    voxels, weights 4:2:1) scaled to amplitude noise_amp voxel; tsdf =
    trunc(clamp(sd / trunc, -1, 1) * 32767); w uniform in [1, 128]."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.05, 0.95, size=(n_spheres, 3)) * n
    r = rng.uniform(0.02, 0.08, size=n_spheres) * n
    dev = torch.device(device)
    out = torch.empty((n, n, n, 2), dtype=torch.int16, device=dev)
    g = torch.Generator(device=dev)
    ii = torch.arange(n, device=dev, dtype=torch.float32) + 0.5
    for z0 in range(0, n, slab):
        z1 = min(n, z0 + slab)
        zz = torch.arange(z0, z1, device=dev, dtype=torch.float32)[:, None, None] + 0.5
        yy = ii[None, :, None]
        xx = ii[None, None, :]
        sd = torch.full((z1 - z0, n, n), float(trunc) + 1.0, device=dev)
        # only spheres that can come within trunc + 1 of the slab matter after clamping
        near = np.flatnonzero((c[:, 2] + r + trunc + 1 >= z0) & (c[:, 2] - r - trunc - 1 <= z1))
        for k in near:
            d = torch.sqrt((xx - float(c[k, 0])) ** 2 + (yy - float(c[k, 1])) ** 2 + (zz - float(c[k, 2])) ** 2)
            torch.minimum(sd, d - float(r[k]), out=sd)
        noise = torch.zeros_like(sd)
        X, Y, Z = xx.expand_as(sd), yy.expand_as(sd), zz.expand_as(sd)
        for o, (period, wgt) in enumerate(((32.0, 4.0), (16.0, 2.0), (8.0, 1.0))):
            noise += wgt * gradient_noise(X / period, Y / period, Z / period, seed=seed * 7 + o)
        sd += noise * (noise_amp / 7.0)
        t = torch.trunc(torch.clamp(sd / trunc, -1.0, 1.0) * 32767.0).to(torch.int16)
        g.manual_seed(seed * 100003 + z0)
        w = torch.randint(1, 129, t.shape, generator=g, device=dev, dtype=torch.int32).to(torch.int16)
        out[z0:z1, ..., 0] = t
        out[z0:z1, ..., 1] = w
    return out


def batch_volumes(n=64, seed=0, lo=32, hi=256, device="cpu", trunc=5.0):
    """n short2 volumes (nz, ny, nx, 2), each axis round(exp(U[ln lo, ln hi])),
    each the truncated SDF (trunc voxels, scaled to 32767) of 1-8 random
    spheres and boxes (union), weights uniform in [1, 128]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), size=3))).astype(int)
        nx, ny, nz = (int(d) for d in dims)
        nobj = int(rng.integers(1, 9))
        dev = torch.device(device)
        z = torch.arange(nz, device=dev, dtype=torch.float32)[:, None, None] + 0.5
        y = torch.arange(ny, device=dev, dtype=torch.float32)[None, :, None] + 0.5
        x = torch.arange(nx, device=dev, dtype=torch.float32)[None, None, :] + 0.5
        sd = torch.full((nz, ny, nx), 1e9, device=dev)
        for _ in range(nobj):
            c = rng.uniform(0.2, 0.8, size=3) * np.array([nx, ny, nz])
            if rng.random() < 0.5:
                r = rng.uniform(0.1, 0.35) * min(nx, ny, nz)
                d = torch.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) - r
            else:
                h = rng.uniform(0.05, 0.3, size=3) * np.array([nx, ny, nz])
                qx, qy, qz = (x - c[0]).abs() - h[0], (y - c[1]).abs() - h[1], (z - c[2]).abs() - h[2]
                outside = torch.sqrt(qx.clamp(min=0) ** 2 + qy.clamp(min=0) ** 2 + qz.clamp(min=0) ** 2)
                inside = torch.clamp(torch.maximum(torch.maximum(qx, qy), qz), max=0)
                d = outside + inside
            sd = torch.minimum(sd, d)
        t = torch.trunc(torch.clamp(sd / trunc, -1, 1) * 32767).to(torch.int16)
        g = torch.Generator(device=dev)
        g.manual_seed(seed * 100003 + i)
        w = torch.randint(1, 129, (nz, ny, nx), generator=g, device=dev, dtype=torch.int32).to(torch.int16)
        out.append(torch.stack([t, w], dim=-1).contiguous())
    return out


# ---------------------------------------------------------------------------
# fusion scene
# ---------------------------------------------------------------------------
def orbit_pose(center, frame, n_frames, radius):
    """camera -> global (R, t) of frame `frame` of an orbit looking at `center`
    (camera x right, y down, z forward)."""
    a = 2.0 * math.pi * frame / n_frames
    elev = 0.25 * math.sin(2.0 * a)
    eye = np.asarray(center, np.float64) + radius * np.array([math.cos(a) * math.cos(elev), math.sin(elev),
                                                               math.sin(a) * math.cos(elev)])
    fwd = center - eye
    fwd /= np.linalg.norm(fwd)
    up = np.array([0.0, 1.0, 0.0])
    right = np.cross(up, fwd)
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    R = np.stack([right, down, fwd], axis=1)  # columns: camera x, y, z in world
    return R, eye


class BlendedSpheres:
    """Smooth union of n spheres inside a cube of side `extent` metres,
    folded with the quadratic polynomial smooth-min
        smin(a, b) = min(a, b) - h^2 k / 4,  h = max(k - |a - b|, 0) / k
    (blend radius k).  Each fold is a convex combination of its arguments'
    gradients, so the field is 1-Lipschitz and sphere tracing on it is safe."""

    def __init__(self, seed=0, n_spheres=8, extent=1.0, blend=0.06):
        rng = np.random.default_rng(seed)
        c = extent / 2.0
        self.extent = extent
        self.center = np.array([c, c, c])
        self.sph_c = c + rng.uniform(-0.18, 0.18, size=(n_spheres, 3)) * extent
        self.sph_r = rng.uniform(0.07, 0.15, size=n_spheres) * extent
        self.k = blend * extent

    def sdf(self, p):
        c = torch.as_tensor(self.sph_c, dtype=p.dtype, device=p.device)
        r = torch.as_tensor(self.sph_r, dtype=p.dtype, device=p.device)
        d = torch.linalg.norm(p[:, None, :] - c[None, :, :], dim=-1) - r[None, :]
        k = self.k
        f = d[:, 0]
        for i in range(1, d.shape[1]):
            b = d[:, i]
            h = torch.clamp(k - (f - b).abs(), min=0.0) / k
            f = torch.minimum(f, b) - h * h * (k / 4.0)
        return f

    def pose(self, frame, n_frames, radius=1.2):
        return orbit_pose(self.center, frame, n_frames, radius * self.extent)

    def depth_frame(self, R, t, w=320, h=240, fx=262.5, fy=262.5, cx=None, cy=None, steps=160, device="cpu"):
        """Sphere-traced z-depth (h, w) float64 metres, 0 where the ray misses."""
        cx = (w - 1) / 2.0 if cx is None else cx
        cy = (h - 1) / 2.0 if cy is None else cy
        dev = torch.device(device)
        dt = torch.float64
        v, u = torch.meshgrid(torch.arange(h, device=dev, dtype=dt), torch.arange(w, device=dev, dtype=dt),
                              indexing="ij")
        dc = torch.stack([(u - cx) / fx, (v - cy) / fy, torch.ones_like(u)], dim=-1).reshape(-1, 3)
        n = torch.linalg.norm(dc, dim=1)
        d = (dc / n[:, None]) @ torch.as_tensor(R, dtype=dt, device=dev).T
        o = torch.as_tensor(t, dtype=dt, device=dev)
        tr = torch.zeros(d.shape[0], dtype=dt, device=dev)
        far = 3.0 * self.extent + float(np.linalg.norm(np.asarray(t) - self.center))
        for _ in range(steps):
            f = self.sdf(o[None, :] + tr[:, None] * d)
            tr = torch.clamp(tr + f, max=far)
        f = self.sdf(o[None, :] + tr[:, None] * d)
        hit = (f.abs() < 1e-7) & (tr < far)
        z = torch.where(hit, tr / n, torch.zeros_like(tr))
        return z.reshape(h, w)

    def frames(self, n_frames, w=320, h=240, fx=262.5, fy=262.5, device="cpu"):
        """(depth (K, h, w) float64, [(R, t)] * K)."""
        poses = [self.pose(i, n_frames) for i in range(n_frames)]
        depth = torch.stack([self.depth_frame(R, t, w, h, fx, fy, device=device) for R, t in poses])
        return depth, poses


class FusionScene:
    """Spheres and boxes inside a cube of side `extent` metres (volume
    coordinates [0, extent)^3, voxel (x, y, z) at (x, y, z) * grid_s as the
    reference's integrate places it)."""

    def __init__(self, seed=0, n_spheres=20, n_boxes=8, extent=3.0):
        rng = np.random.default_rng(seed)
        c = extent / 2.0
        self.extent = extent
        self.center = np.array([c, c, c])
        # objects stay within 1.1 m of the centre; the camera orbits at 1.5 m
        self.sph_c = c + rng.uniform(-0.7, 0.7, size=(n_spheres, 3))
        self.sph_r = rng.uniform(0.1, 0.4, size=n_spheres)
        self.box_c = c + rng.uniform(-0.7, 0.7, size=(n_boxes, 3))
        self.box_h = rng.uniform(0.05, 0.25, size=(n_boxes, 3))

    def pose(self, frame, n_frames, radius=1.5):
        """camera -> global (R, t) of frame `frame` of an orbit looking at the centre."""
        return orbit_pose(self.center, frame, n_frames, radius)

    def depth_frame(self, R, t, w=640, h=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5,
                    noise_sigma=0.002, seed=0, device="cpu"):
        """Ray-cast z-depth + N(0, sigma), rounded to uint16 millimetres
        (0 where the ray misses)."""
        dev = torch.device(device)
        dt = torch.float64
        v, u = torch.meshgrid(torch.arange(h, device=dev, dtype=dt), torch.arange(w, device=dev, dtype=dt),
                              indexing="ij")
        dc = torch.stack([(u - cx) / fx, (v - cy) / fy, torch.ones_like(u)], dim=-1).reshape(-1, 3)
        Rt = torch.as_tensor(R, dtype=dt, device=dev)
        o = torch.as_tensor(t, dtype=dt, device=dev)
        d = dc @ Rt.T  # world direction, camera-z component 1 -> ray parameter == z-depth
        best = torch.full((d.shape[0],), float("inf"), dtype=dt, device=dev)
        # spheres
        sc = torch.as_tensor(self.sph_c, dtype=dt, device=dev)
        sr = torch.as_tensor(self.sph_r, dtype=dt, device=dev)
        oc = o[None, :] - sc  # (S, 3)
        a = (d * d).sum(-1)[:, None]
        b = 2.0 * (d @ oc.T)
        cc = (oc * oc).sum(-1)[None, :] - sr[None, :] ** 2
        disc = b * b - 4 * a * cc
        sq = torch.sqrt(torch.clamp(disc, min=0.0))
        s0 = (-b - sq) / (2 * a)
        s0 = torch.where((disc >= 0) & (s0 > 1e-6), s0, torch.full_like(s0, float("inf")))
        best = torch.minimum(best, s0.min(dim=1).values)
        # boxes (slab test)
        bc = torch.as_tensor(self.box_c, dtype=dt, device=dev)
        bh = torch.as_tensor(self.box_h, dtype=dt, device=dev)
        lo = bc - bh
        hi = bc + bh
        inv = 1.0 / torch.where(d.abs() < 1e-12, torch.full_like(d, 1e-12), d)
        t1 = (lo[None, :, :] - o[None, None, :]) * inv[:, None, :]
        t2 = (hi[None, :, :] - o[None, None, :]) * inv[:, None, :]
        tmin = torch.minimum(t1, t2).max(dim=-1).values
        tmax = torch.maximum(t1, t2).min(dim=-1).values
        hit = (tmax >= tmin) & (tmin > 1e-6)
        tb = torch.where(hit, tmin, torch.full_like(tmin, float("inf")))
        best = torch.minimum(best, tb.min(dim=1).values)
        g = torch.Generator(device=dev)
        g.manual_seed(int(seed))
        noise = torch.randn(best.shape, generator=g, device=dev, dtype=dt) * noise_sigma
        z = torch.where(torch.isfinite(best), best + noise, torch.zeros_like(best))
        mm = torch.clamp(torch.round(z * 1000.0), 0, 65535)
        return mm.reshape(h, w).to(torch.int32)


def mm_to_u16_bits(mm):
    """int32 millimetre tensor -> int16 tensor holding the uint16 bit
    pattern (the depth kernels read the 16 bits as unsigned)."""
    m = mm.to(torch.int32) & 0xFFFF
    return torch.where(m >= 32768, m - 65536, m).to(torch.int16)


# ---------------------------------------------------------------------------
# text dumps of a volume: "x y z sdf weight\n" per voxel, x outermost, z
# innermost (the record order the loader of cu_voxel_rlc_to_mesh expects,
# kf.cu:3289-3358), formatted on the device with torch ops
# ---------------------------------------------------------------------------
def _format_ints(v, width):
    """(n, width) uint8 right-aligned decimal text of int64 tensor v; unused
    leading columns hold 0 (removed by the caller)."""
    n = v.shape[0]
    out = torch.zeros((n, width), dtype=torch.uint8, device=v.device)
    neg = v < 0
    a = v.abs()
    nd = torch.ones_like(a)
    t = a // 10
    for p in range(1, width):
        nd = nd + (t > 0).to(nd.dtype)
        t = t // 10
    t = a
    for p in range(width):
        col = width - 1 - p
        d = (t % 10).to(torch.uint8) + 48
        out[:, col] = torch.where(p < nd, d, torch.zeros_like(d))
        t = t // 10
    rows = torch.nonzero(neg).squeeze(1)
    if rows.numel():
        out[rows, (width - 1 - nd[rows])] = 45
    return out


def text_dump(values, box_origin=(0, 0, 0), records_per_chunk=1 << 24):
    """uint8 CUDA tensor of the text records of a (nz, ny, nx, 2) int16
    volume whose voxel (0, 0, 0) sits at box_origin; "%d %d %d %d %d\\n" per
    voxel, x outermost, z innermost, weights printed unsigned."""
    nz, ny, nx, _ = values.shape
    dev = values.device
    bx, by, bz = (int(o) for o in box_origin)
    vt = values.permute(2, 1, 0, 3).reshape(-1, 2)  # x, y, z order
    n = vt.shape[0]
    wid = [len(str(max(abs(bx), abs(bx + nx)))) + 1, len(str(max(abs(by), abs(by + ny)))) + 1,
           len(str(max(abs(bz), abs(bz + nz)))) + 1, 6, 5]
    parts = []
    for s in range(0, n, records_per_chunk):
        e = min(n, s + records_per_chunk)
        i = torch.arange(s, e, device=dev, dtype=torch.int64)
        z = i % nz + bz
        y = (i // nz) % ny + by
        x = i // (nz * ny) + bx
        sdf = vt[s:e, 0].to(torch.int64)
        w = vt[s:e, 1].to(torch.int64) & 0xFFFF
        cols = []
        for k, f in enumerate((x, y, z, sdf, w)):
            cols.append(_format_ints(f, wid[k]))
            sep = torch.full((e - s, 1), 10 if k == 4 else 32, dtype=torch.uint8, device=dev)
            cols.append(sep)
        buf = torch.cat(cols, dim=1)
        parts.append(buf[buf != 0])
    return torch.cat(parts) if parts else torch.zeros(0, dtype=torch.uint8, device=dev)
