"""Pins the oracle to the reference's own source: the reference's functions on
the TSDF -> mesh path, taken from its files by line range and compiled for
the host (oracle/ref/build_ref.py, oracle/reference.py), against the oracle
on the same inputs, bit for bit.  Runs where the reference tree is present;
skips elsewhere.

Covered: cube index (cu_marching_cubes_v1.cu:53-95), the whole extraction
with its side outputs (:228-370 generator driven over the occupied cubes in
linear order), surface normals (cu_kinect_fusion_v1.cu:3146-3242), depth ->
metre / vertex / normal maps (:95-151), voxel initialisation (:364-379),
depth scaling + integration (:416-532), the RLE slice codec (:1362-1447).
All FP32 expressions uncontracted on both sides (the oracle's convention);
test_contraction_effect reports what fused multiply-adds change."""
import numpy as np
import pytest

from marching_cube_gb300 import synthetic
import oracle.reference as ref

pytestmark = pytest.mark.skipif(not ref.available(), reason="the reference tree is not present")


def _same_extract(o, r):
    assert len(o["soup"]) == len(r["soup"])
    assert np.array_equal(o["soup"].view(np.uint8), r["soup"].view(np.uint8))
    assert np.array_equal(o["normals"].view(np.uint32), r["normals"].view(np.uint32))
    assert np.array_equal(o["vi2vox"], r["vi2vox"])
    assert np.array_equal(o["ver_voxel"].reshape(-1), r["ver_voxel"].reshape(-1))


def _fused(orc, n, frames, seed, trunc_vox=4.0, size=(160, 120)):
    """n^3 short2 volume of the fusion scene, integrated by the oracle."""
    extent = 3.0
    grid_s = extent / n
    w, h = size
    f = 525.0 * w / 640.0
    cx, cy = (w - 1) / 2.0, (h - 1) / 2.0
    scene = synthetic.FusionScene(seed=seed, extent=extent)
    vol = orc.voxel_init(n ** 3).reshape(n, n, n, 2)
    k = orc.intrinsic(f, f, cx, cy)
    for i in range(frames):
        R, t = scene.pose(i, frames)
        mm = scene.depth_frame(R, t, w=w, h=h, fx=f, fy=f, cx=cx, cy=cy, seed=seed * 1000 + i)
        m = orc.depth_to_meter(mm.numpy().astype(np.uint16))
        orc.integrate(vol, trunc_vox * grid_s, trunc_vox * grid_s, grid_s, k, orc.extrinsic(R, t), m)
    return vol, grid_s


VOLUMES = {
    "sphere_128": lambda: (synthetic.sphere_volume(128, radius=40.0, trunc=5.0, seed=0), 0.01),
    "random_w0_sentinels": lambda: (synthetic.random_volume((23, 17, 31), seed=3), 0.02),
    "random_dense": lambda: (synthetic.random_volume((40, 9, 33), seed=4, p_zero_weight=0.01,
                                                     sentinel_frac=0.0), 0.5),
}


@pytest.mark.parametrize("name", sorted(VOLUMES))
def test_extraction_matches_reference(orc, name):
    vol, cell = VOLUMES[name]()
    ci, _ = orc.mc_classify(vol)
    assert np.array_equal(ci, ref.mc_cube_index(vol))
    assert orc.mc_count(vol) == ref.mc_count(vol)
    _same_extract(orc.mc_extract(vol, cell), ref.mc_extract(vol, cell))


def test_golden_volumes_match_reference(orc):
    import glob
    import os
    for path in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))):
        g = np.load(path)
        vol, cell = g["vol"], float(g["cell"])
        _same_extract(orc.mc_extract(vol, cell), ref.mc_extract(vol, cell))


def test_max_tsdf_quirk_and_border_reads(orc):
    # stored +-32767 is not the +-32766 sentinel; surfaces touching every face
    # make vertex voxels and normal samples leave the volume
    rng = np.random.default_rng(7)
    vol = np.zeros((12, 10, 14, 2), np.int16)
    vol[..., 0] = rng.choice(np.array([-32767, -32766, -100, 0, 100, 32766, 32767], np.int16), size=vol.shape[:3])
    vol[..., 1] = rng.integers(0, 3, size=vol.shape[:3]).astype(np.int16)
    _same_extract(orc.mc_extract(vol, 0.3), ref.mc_extract(vol, 0.3))


def test_batch_volumes_match_reference(orc):
    # every eighth volume of the 64-volume batch set (each axis log-uniform
    # in 32..256, spheres and boxes), every output
    vols = synthetic.batch_volumes(64, seed=7, lo=32, hi=256, device="cpu")
    total = 0
    for i in range(0, 64, 8):
        v = vols[i].numpy()
        r = ref.mc_extract(v, 0.01)
        total += len(r["soup"])
        _same_extract(orc.mc_extract(v, 0.01), r)
    assert total > 100000


def test_fused_volume_extraction_matches_reference(orc):
    vol, cell = _fused(orc, 96, 4, seed=5)
    r = ref.mc_extract(vol, cell)
    assert len(r["soup"]) > 3000
    _same_extract(orc.mc_extract(vol, cell), r)


def test_surface_normals_of_arbitrary_points(orc):
    vol = synthetic.random_volume((11, 13, 9), seed=2, sentinel_frac=0.05)
    rng = np.random.default_rng(1)
    cell = 0.25
    pts = rng.uniform(-0.2, np.array([9, 13, 11]) * cell + 0.2, size=(500, 3)).astype(np.float32)
    recs = np.zeros(len(pts), ref.VERTEX_DTYPE)
    recs["pos"] = pts
    got = ref.surface_normals(vol, cell, recs)
    for p, n in zip(pts, got):
        assert np.array_equal(orc.surface_normal(vol, cell, p).view(np.uint32), n.view(np.uint32))


def test_depth_maps_match_reference(orc):
    scene = synthetic.FusionScene(seed=3)
    R, t = scene.pose(2, 10)
    mm = scene.depth_frame(R, t, w=160, h=120, fx=131.25, fy=131.25, cx=79.5, cy=59.5, seed=4)
    d = mm.numpy().astype(np.uint16)
    d[3, 4], d[5, 6], d[7, 8], d[9, 10] = 2000, 2001, 40000, 65535
    mo = orc.depth_to_meter(d)
    assert np.array_equal(mo.view(np.uint32), ref.depth_to_meter(d).view(np.uint32))
    k = orc.intrinsic(131.25, 131.25, 79.5, 59.5)
    vo = orc.meter_to_vertex(k, mo)
    assert np.array_equal(vo.view(np.uint32), ref.meter_to_vertex(k, mo).view(np.uint32))
    no = orc.vertex_to_normal(vo)
    assert np.array_equal(no.view(np.uint32), ref.vertex_to_normal(vo).view(np.uint32))


def test_voxel_init_matches_reference(orc):
    assert np.array_equal(orc.voxel_init(7 * 5 * 3).reshape(3, 5, 7, 2), ref.voxel_init((3, 5, 7)))


@pytest.mark.parametrize("use_normals,dynamic", [(False, False), (True, False), (False, True), (True, True)])
def test_integrate_matches_reference(orc, use_normals, dynamic):
    n, frames, w, h = 48, 3, 160, 120
    extent = 3.0
    grid_s = extent / n
    trunc = 3 * grid_s
    f = 131.25
    scene = synthetic.FusionScene(seed=6, extent=extent)
    k = orc.intrinsic(f, f, (w - 1) / 2.0, (h - 1) / 2.0)
    a = orc.voxel_init(n ** 3).reshape(n, n, n, 2)
    b = a.copy()
    for i in range(frames):
        R, t = scene.pose(i, frames)
        mm = scene.depth_frame(R, t, w=w, h=h, fx=f, fy=f, cx=(w - 1) / 2.0, cy=(h - 1) / 2.0, seed=60 + i)
        m = orc.depth_to_meter(mm.numpy().astype(np.uint16))
        nrm = orc.vertex_to_normal(orc.meter_to_vertex(k, m)) if use_normals else None
        e = orc.extrinsic(R, t)
        orc.integrate(a, trunc, trunc, grid_s, k, e, m, normals=nrm, is_dynamic=dynamic)
        ref.integrate(b, trunc, trunc, grid_s, k, e, m, normals=nrm, is_dynamic=dynamic)
        assert np.array_equal(a, b), i
    assert (a[..., 1] != 0).mean() > 0.01


def test_rle_slice_codec_matches_reference(orc):
    rng = np.random.default_rng(11)
    cases = []
    # runs longer than the 14-bit count, all three record kinds, literal runs
    # whose weights differ (the reference format keeps the first)
    s = np.zeros((40000, 2), np.int16)
    s[:20000, 0] = 32766
    s[20000:37000, 0] = -32766
    s[37000:, 0] = rng.integers(-500, 500, size=3000)
    s[:, 1] = rng.integers(0, 3, size=len(s))
    cases.append(s)
    for seed in range(5):
        r = np.random.default_rng(seed)
        v = np.zeros((r.integers(1, 5000), 2), np.int16)
        v[:, 0] = r.choice(np.array([-32766, 32766, 5, -5, 0], np.int16), size=len(v))
        v[:, 1] = r.integers(0, 2, size=len(v))
        cases.append(v)
    for v in cases:
        enc = ref.rle_encode_slice(v)
        assert enc == orc.rle_encode_slice(v)
        assert np.array_equal(ref.rle_decode_slice(enc, len(v)), orc.rle_decode_slice(enc, len(v)))


def test_contraction_effect(orc):
    """The reference's stock nvcc build contracts a*b+c into fused
    multiply-adds; the oracle and the CUDA library evaluate every expression
    as written.  The reference's own code built with contraction gives the
    same topology (cube indices are integer tests) and positions within a
    few ulp; vox_pos (floor of a position) can move at ties.  This measures
    it on the 128^3 sphere and a fused volume; the counts are printed."""
    for name, (vol, cell) in (("sphere_128", VOLUMES["sphere_128"]()), ("fused_96", _fused(orc, 96, 4, seed=5))):
        a = ref.mc_extract(vol, cell)
        b = ref.mc_extract(vol, cell, fma=True)
        assert len(a["soup"]) == len(b["soup"])
        pa, pb = a["soup"]["pos"], b["soup"]["pos"]
        moved = int((pa != pb).any(axis=1).sum())
        vox = int((a["soup"]["vox"] != b["soup"]["vox"]).any(axis=1).sum())
        nrm = int((a["normals"] != b["normals"]).any(axis=1).sum())
        err = float(np.abs(pa.astype(np.float64) - pb).max() / cell)
        print("%s: %d vertices, positions differing %d, vox_pos differing %d, normals differing %d, "
              "max |dP| %.3g voxel" % (name, len(pa), moved, vox, nrm, err))
        assert err < 1e-5
