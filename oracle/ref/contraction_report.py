"""How much fused multiply-adds move the reference's own results: the
reference's extraction code (oracle/ref) built with -ffp-contract=off (the
convention of the oracle and of the CUDA library) and with
-ffp-contract=fast (the reference's stock nvcc build contracts by default),
run on the 128^3 sphere workload and on the 512^3 fusion workload (60 frames
of 640x480 integrated by the oracle; the frames are drawn on the CPU, so
their noise differs from the GPU-drawn frames of the benchmark).  Prints,
per workload, how many soup vertices differ in position, in vox_pos and in
normal, and the largest position difference in voxels.  TEST INFRASTRUCTURE
ONLY; needs the reference tree.

    python oracle/ref/contraction_report.py [--n 512] [--frames 60]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def compare(name, vol, cell):
    import oracle.reference as ref
    t0 = time.time()
    a = ref.mc_extract(vol, cell)
    b = ref.mc_extract(vol, cell, fma=True)
    assert len(a["soup"]) == len(b["soup"])
    pa, pb = a["soup"]["pos"], b["soup"]["pos"]
    print("%s: %d soup vertices; positions differing %d, vox_pos differing %d, normals differing %d, "
          "max |dP| %.3g voxel, max |dN| %.3g (%.0f s)" % (
              name, len(pa), int((pa != pb).any(axis=1).sum()),
              int((a["soup"]["vox"] != b["soup"]["vox"]).any(axis=1).sum()),
              int((a["normals"] != b["normals"]).any(axis=1).sum()),
              float(np.abs(pa.astype(np.float64) - pb).max() / cell),
              float(np.abs(a["normals"].astype(np.float64) - b["normals"]).max()), time.time() - t0), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--frames", type=int, default=60)
    args = ap.parse_args()
    import torch
    import bench
    import oracle
    import oracle.reference as ref
    from marching_cube_gb300 import synthetic
    oracle.build()
    if not ref.available():
        raise SystemExit("the reference tree is not available")
    compare("sphere_128", synthetic.sphere_volume(128, radius=40.0, trunc=5.0, seed=0), 0.01)
    with torch.no_grad():
        vol = bench.oracle_volume(oracle, synthetic, torch, args.n, args.frames)
    compare("fusion_%d_%dframes" % (args.n, args.frames), vol, bench.EXTENT / args.n)


if __name__ == "__main__":
    main()
