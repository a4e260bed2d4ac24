"""The reference-compatible C++ interface in include/ compiles and links
against libmcg.so (CPU), and a C++ caller gets the same mesh as the oracle
(GPU)."""
import json
import os
import struct
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "marching_cube_gb300")
CUDA_INC = "/usr/local/cuda/include"


def build_dropin(out_dir):
    import marching_cube_gb300  # noqa: F401  (libmcg.so exists)
    exe = os.path.join(out_dir, "dropin_main")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), "-I", CUDA_INC,
           os.path.join(REPO, "tests", "cpp", "dropin_main.cpp"), "-L", PKG, "-lmcg",
           "-Wl,-rpath," + PKG, "-L/usr/local/cuda/lib64", "-lcudart", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_api_compiles_and_links(tmp_path):
    exe = build_dropin(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_cpp_dropin_runs(tmp_path, orc):
    exe = build_dropin(str(tmp_path))
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    # the same sphere as the C++ program, restated here for the oracle
    n = 48
    i = np.arange(n) + 0.5
    z, y, x = np.meshgrid(i, i, i, indexing="ij")
    sd = np.clip((np.sqrt((x - 24) ** 2 + (y - 24) ** 2 + (z - 24) ** 2) - 15.0) / 5.0, -1, 1)
    t = (sd.astype(np.float32) * np.float32(32767.0)).astype(np.int16)
    xi, yi, zi = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="xy")
    w = (1 + (np.arange(n)[None, None, :] + np.arange(n)[None, :, None] + np.arange(n)[:, None, None]) % 100)
    vol = np.stack([t, w.astype(np.int16)], axis=-1)
    _, ntri = orc.mc_count(vol)
    assert res["triangles"] == ntri and res["mesh_size"] == 3 * ntri and res["shared"] == 1
    # MarchingCubes::backward against the binary64 adjoint (constant dL/dP)
    g = np.fromfile(os.path.join(str(tmp_path), "grad_tsdf.bin"), np.float32)
    G = np.tile(np.array([1.0, 0.5, -0.25]), (3 * ntri, 1))
    g64 = orc.mc_backward_f64(vol, 0.01, G).reshape(-1)
    assert np.count_nonzero(g64) > 100
    assert np.linalg.norm(g - g64) <= 1e-4 * np.linalg.norm(g64)
    # PLY: header + 3 vertices per triangle with position and normal
    ply = open(os.path.join(str(tmp_path), "sphere.ply"), "rb").read()
    head, body = ply.split(b"end_header\n", 1)
    assert b"element vertex %d" % (3 * ntri) in head and b"element face %d" % ntri in head
    assert len(body) == 3 * ntri * 24 + ntri * 13
    # the OBJ and qi_volume.txt are the reference writer's bytes for the soup
    import torch
    import marching_cube_gb300 as mcg
    mesh = mcg.extract(torch.from_numpy(vol).cuda(), 0.01, soup=True, normals=True)
    nv = mesh.num_vertices
    obj, qi = orc.mesh_obj(mesh.soup[:nv].cpu().numpy(), mesh.normals[:nv].cpu().numpy())
    assert open(os.path.join(str(tmp_path), "sphere.obj"), "rb").read() == obj
    assert open(os.path.join(str(tmp_path), "qi_volume.txt"), "rb").read() == qi
    assert ply == orc.mesh_ply(mesh.soup[:nv].cpu().numpy(), mesh.normals[:nv].cpu().numpy())
    # cu_voxel_rlc_to_mesh on the same sphere dumped as text records: the
    # same triangles at grid 3 mm instead of 1 cm
    tply = open(os.path.join(str(tmp_path), "text.ply"), "rb").read()
    thead, tbody = tply.split(b"end_header\n", 1)
    assert b"element face %d" % ntri in thead and len(tbody) == len(body)
    P = np.frombuffer(body, np.uint8)[: 3 * ntri * 24].reshape(-1, 6 * 4).copy().view(np.float32)
    Q = np.frombuffer(tbody, np.uint8)[: 3 * ntri * 24].reshape(-1, 6 * 4).copy().view(np.float32)
    assert np.allclose(Q[:, :3] / 0.003, P[:, :3] / 0.01, atol=1e-3) and np.allclose(Q[:, 3:], P[:, 3:], atol=1e-4)
    obj = open(os.path.join(str(tmp_path), "sphere.obj")).read()
    assert obj.count("\nf ") + obj.startswith("f ") > 0.9 * ntri
    # RLE round trip keeps every tsdf; window write / read
    assert res["tsdf_equal"] == res["voxels"]
    assert res["inner"] == [-32766, 0]
    # the reference format keeps tsdf; weights inside a run are the run's first
    assert res["outer"][0] == res["orig"][0]
    # integrate probe: voxel (12, 12, 18) is 0.1 m in front of a 1 m wall
    assert res["probe"][1] > 0 and abs(res["probe"][0] / 32766.0 - 0.1 / 0.15) < 2e-3
    assert res["vtx0"][2] == pytest.approx(1.5)
