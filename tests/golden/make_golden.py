"""Generates the golden fixtures in this directory.

An independent restatement of the reference's marching cubes (cube index,
canonical triangle soup, normals) and RLE slice encoder in vectorised numpy
/ plain Python (binary64), written separately from the C oracle so the two
cross-check each other.  Reference lines followed:
cu_marching_cubes_v1.cu:53-95 (cube index), :136 (empty cases), :243-264
(node coordinates, interpolation), :322-333 (reversed winding);
cu_kinect_fusion_v1.cu:3146-3233 (normals), :1367-1417 (RLE slice encoder).
The lookup tables are read from the generated header oracle/mc_tables.h.

    python tests/golden/make_golden.py
"""
import os
import re
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

MAX_TSDF = 32766
CORNERS = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)])
EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


def tables():
    txt = open(os.path.join(REPO, "oracle", "mc_tables.h")).read()
    m = re.search(r"orc_tri_table[^=]*=\s*\{(.*?)\};", txt, re.S)
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    tri = np.array([int(v) for v in re.findall(r"-?\d+", body)], np.int64).reshape(256, 16)
    nv = (tri >= 0).sum(1)
    return tri, nv


def classify(vol):
    t = vol[..., 0].astype(np.int64)
    w = vol[..., 1].astype(np.int64) & 0xFFFF
    nz, ny, nx = t.shape
    ci = np.zeros((nz - 1, ny - 1, nx - 1), np.int64)
    dead = np.zeros_like(ci, dtype=bool)
    for c, (dx, dy, dz) in enumerate(CORNERS):
        sl = (slice(dz, dz + nz - 1), slice(dy, dy + ny - 1), slice(dx, dx + nx - 1))
        ci |= (t[sl] < 0).astype(np.int64) << c
        dead |= w[sl] == 0
    ci[dead] = 0
    return ci


def normal(vol, p):
    """Normal at point p (voxel units, binary64) with the reference's linear
    addressing; zero when a sample is a +-32766 sentinel or leaves [0, N)."""
    nz, ny, nx = vol.shape[:3]
    flat = vol[..., 0].reshape(-1).astype(np.int64)
    pi = np.floor(p).astype(np.int64)
    tf = p - pi
    xy, N = nx * ny, nx * ny * nz
    base = pi[2] * xy + pi[1] * nx + pi[0]
    offs = [0, 1, 1 + nx, nx, xy, xy + 1, xy + 1 + nx, xy + nx]
    slot = [0, 1, 6, 2, 3, 4, 7, 5]
    s = np.zeros(8)
    for k, o in enumerate(offs):
        a = base + o
        if a < 0 or a >= N:
            return np.zeros(3)
        v = flat[a]
        if v in (MAX_TSDF, -MAX_TSDF):
            return np.zeros(3)
        s[slot[k]] = v / MAX_TSDF

    def bil(v0, v1, v2, v3, x, y):
        return v0 * (1 - x) * (1 - y) + v1 * x * (1 - y) + v2 * (1 - x) * y + v3 * x * y

    n = np.array([
        bil(s[1], s[6], s[4], s[7], tf[1], tf[2]) - bil(s[0], s[2], s[3], s[5], tf[1], tf[2]),
        bil(s[2], s[6], s[5], s[7], tf[0], tf[2]) - bil(s[0], s[1], s[3], s[4], tf[0], tf[2]),
        bil(s[3], s[4], s[5], s[7], tf[0], tf[1]) - bil(s[0], s[1], s[2], s[6], tf[0], tf[1]),
    ])
    nn = np.linalg.norm(n)
    normal.last_len = nn
    return n / nn if nn > 1.1920929e-07 else n


def extract(vol, cell):
    tri, nv = tables()
    ci = classify(vol)
    nz, ny, nx = vol.shape[:3]
    f = vol[..., 0].astype(np.float64) / MAX_TSDF
    pos, nrm, tcube, nlen = [], [], [], []
    for z, y, x in zip(*np.nonzero((ci != 0) & (ci != 255))):
        c = ci[z, y, x]
        for j in range(nv[c] // 3):
            tcube.append((z * ny + y) * nx + x)
            for slot in range(3):
                a, b = EDGES[tri[c][3 * j + 2 - slot]]
                pa = np.array((x, y, z)) + CORNERS[a]
                pb = np.array((x, y, z)) + CORNERS[b]
                f0 = f[pa[2], pa[1], pa[0]]
                f1 = f[pb[2], pb[1], pb[0]]
                t = -f0 / (f1 - f0 + 1e-15)
                p = (pa + 0.5) + t * (pb - pa)
                pos.append(p * cell)
                normal.last_len = 0.0
                nrm.append(normal(vol, p))
                nlen.append(normal.last_len)
    return (ci, np.array(pos).reshape(-1, 3), np.array(nrm).reshape(-1, 3), np.array(tcube, np.int64),
            np.array(nlen))


def rle_slice(vox, lossless=False):
    """Byte string of one slice (plain Python, from the record layout)."""
    out = bytearray()

    def run(first, n):
        t, w = int(first[0]), int(first[1]) & 0xFFFF
        kind = 1 if t == MAX_TSDF else 2 if t == -MAX_TSDF else 3
        if lossless and w != 0:
            kind = 3
        out.extend(struct.pack("<H", n | (kind << 14)))
        if kind == 3:
            out.extend(struct.pack("<hH", t, w))

    i = 0
    n = len(vox)
    while i < n:
        j = i
        key = (lambda v: (int(v[0]), int(v[1]))) if lossless else (lambda v: int(v[0]))
        while j < n and key(vox[j]) == key(vox[i]) and j - i < 16383:
            j += 1
        run(vox[i], j - i)
        i = j
    return bytes(out)


CASES = {
    "sphere24": dict(kind="sphere", n=24, radius=7.0, seed=11, cell=0.01),
    "rand_6_7_9": dict(kind="random", shape=(6, 7, 9), seed=21, cell=0.02),
    "rand_9_5_17": dict(kind="random", shape=(9, 5, 17), seed=22, cell=0.005),
    "corner_sphere": dict(kind="sphere", n=20, radius=6.0, seed=12, cell=0.01, center=18.5),
}


def make_volume(c):
    from marching_cube_gb300 import synthetic
    if c["kind"] == "sphere":
        return synthetic.sphere_volume(c["n"], radius=c["radius"], seed=c["seed"], center=c.get("center"))
    return synthetic.random_volume(c["shape"], seed=c["seed"])


def main():
    for name, c in CASES.items():
        vol = make_volume(c)
        ci, pos, nrm, tcube, nlen = extract(vol, c["cell"])
        slices = vol.reshape(vol.shape[0], -1, 2)
        rle = np.frombuffer(b"".join(rle_slice(s) for s in slices), np.uint8)
        rle_sizes = np.array([len(rle_slice(s)) for s in slices], np.int64)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), vol=vol, cell=c["cell"], ci=ci.astype(np.uint8),
                            pos=pos, nrm=nrm, nlen=nlen, tri_cube=tcube, rle=rle, rle_sizes=rle_sizes)
        print(name, vol.shape, "triangles", len(tcube))


if __name__ == "__main__":
    main()
