"""Generates tests/golden/ref/*.npz: input/output vectors produced by the
reference's own source, compiled for the host (oracle/ref/build_ref.py,
oracle/reference.py) -- so the GPU tests, which run where the reference tree
is absent, still compare against the reference itself.  Needs the reference
tree (default /root/reference).

    python tests/golden/make_ref_golden.py

Fixtures:
  fusion_48.npz   three 160x120 depth frames of the fusion scene (uint16 mm)
                  and their poses; the reference's depth -> metre -> vertex ->
                  normal maps of frame 0 (cu_kinect_fusion_v1.cu:95-151); a 48^3
                  short2 volume initialised (:364-379) and integrated with the
                  three frames (:416-532, truncation 3 voxels); the reference's
                  RLE slices of that volume (:1362-1447); its extraction
                  (cu_marching_cubes_v1.cu:228-370 over the cubes in linear order)
                  with every output and the normals (cu_kinect_fusion_v1.cu:3146-3242)
  mc_random.npz   extraction of a random volume with weight-0 voxels and
                  +-32766 sentinels (14 x 12 x 19)
  mc_sphere.npz   extraction of a 40^3 sphere whose surface touches two faces
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

OUT = os.path.join(HERE, "ref")


def mesh_arrays(r):
    return {"soup": r["soup"].view(np.uint8).reshape(-1, 28), "normals": r["normals"], "vi2vox": r["vi2vox"],
            "ver_voxel": r["ver_voxel"]}


def fusion(ref, orc, synthetic):
    n, frames, w, h = 48, 3, 160, 120
    extent = 3.0
    grid_s = extent / n
    trunc = 3 * grid_s
    f = 131.25
    cx, cy = (w - 1) / 2.0, (h - 1) / 2.0
    k = orc.intrinsic(f, f, cx, cy)
    scene = synthetic.FusionScene(seed=6, extent=extent)
    vol = ref.voxel_init((n, n, n))
    depth, poses = [], []
    for i in range(frames):
        R, t = scene.pose(i, frames)
        mm = scene.depth_frame(R, t, w=w, h=h, fx=f, fy=f, cx=cx, cy=cy, seed=60 + i)
        d = mm.numpy().astype(np.uint16)
        m = ref.depth_to_meter(d)
        ref.integrate(vol, trunc, trunc, grid_s, k, orc.extrinsic(R, t), m)
        depth.append(d)
        poses.append(np.concatenate([np.asarray(R, np.float64).reshape(-1), np.asarray(t, np.float64)]))
    m0 = ref.depth_to_meter(depth[0])
    v0 = ref.meter_to_vertex(k, m0)
    n0 = ref.vertex_to_normal(v0)
    slices = vol.reshape(n, -1, 2)
    enc = [ref.rle_encode_slice(s) for s in slices]
    mesh = mesh_arrays(ref.mc_extract(vol, grid_s))
    return dict(depth=np.stack(depth), poses=np.stack(poses), intrinsic=np.array([f, f, cx, cy]),
                trunc=trunc, grid_s=grid_s, meter0=m0, vertex0=v0, normal0=n0, vol=vol,
                rle=np.frombuffer(b"".join(enc), np.uint8), rle_sizes=np.array([len(e) for e in enc], np.int64),
                cell=grid_s, **mesh)


def main():
    import oracle
    import oracle.reference as ref
    from marching_cube_gb300 import synthetic
    oracle.build()
    if not ref.available():
        raise SystemExit("the reference tree is not available")
    os.makedirs(OUT, exist_ok=True)
    np.savez_compressed(os.path.join(OUT, "fusion_48.npz"), **fusion(ref, oracle, synthetic))
    vol = synthetic.random_volume((14, 12, 19), seed=3)
    np.savez_compressed(os.path.join(OUT, "mc_random.npz"), vol=vol, cell=0.02,
                        **mesh_arrays(ref.mc_extract(vol, 0.02)))
    vol = synthetic.sphere_volume(40, radius=13.0, seed=5, center=27.0)
    np.savez_compressed(os.path.join(OUT, "mc_sphere.npz"), vol=vol, cell=0.01,
                        **mesh_arrays(ref.mc_extract(vol, 0.01)))
    for f in sorted(os.listdir(OUT)):
        print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
