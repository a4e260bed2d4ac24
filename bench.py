"""Benchmark: marching-cubes extraction of the 512^3 fused TSDF volume.

Workload (the 512^3 fusion configuration): a 512^3 short2 volume over a 3 m
cube (trunc 0.03 m) built by integrating 60 ray-cast 640x480 depth frames of a
seeded scene (20 spheres + boxes, sigma 2 mm noise) with this library's
integrate kernel; then one step = one full extraction (classify, scan,
generate with fused normals) of that volume into preallocated device buffers.
The volume (512 MiB) is larger than L2 (129 MB), so no flush is needed
between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  With torchrun and N > 1 every rank extracts
its own replica (the path has no exchange step), value = all ranks' voxels
/ max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_VOX = 512
EXTENT = 3.0
TRUNC = 0.03
N_FRAMES = 60
W, H = 640, 480
FX = FY = 525.0
CX, CY = 319.5, 239.5
METRIC = "512^3 MC extraction throughput (Gvoxels/s)"
UNIT = "Gvoxels/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_VOX, help="volume edge (default 512)")
    ap.add_argument("--frames", type=int, default=N_FRAMES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-indexed", action="store_true")
    ap.add_argument("--no-stress", action="store_true")
    ap.add_argument("--no-raycast", action="store_true")
    ap.add_argument("--no-text-load", action="store_true")
    ap.add_argument("--no-mesh-write", action="store_true")
    ap.add_argument("--no-icp", action="store_true")
    ap.add_argument("--text-dim", type=int, default=512, help="window of the text-record load (<= volume size)")
    ap.add_argument("--stress-n", type=int, default=1024, help="stress volume edge (default 1024)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# clocks sampler (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        # one nvidia-smi in loop mode (-lms) rather than a process per sample
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                        "--format=csv,noheader,nounits", "-lms", "50"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._p = None
            return
        for line in self._p.stdout:
            if self._stop.is_set():
                break
            line = line.strip()
            if line:
                self.rows.append([x.strip() for x in line.split(",")])

    def __enter__(self):
        self._p = None
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        time.sleep(0.3)  # the sampler is running before the timed region starts
        return self

    def __exit__(self, *a):
        self._stop.set()
        p = self._p
        if p is not None and p.poll() is None:
            p.terminate()  # this sampler's own process, by handle
            try:
                p.wait(timeout=5)
            except Exception:
                p.kill()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ---------------------------------------------------------------------------
# workload construction
# ---------------------------------------------------------------------------
def fusion_frames(synthetic, frames, seed=0, device="cuda"):
    """The fusion workload's depth frames: yields (R, t, depth) per frame,
    R, t the camera -> volume pose of an orbit at 1.5 m around the 3 m
    cube's centre and depth the [H][W] int16 tensor holding the uint16
    millimetre image (ray-cast scene + N(0, 2 mm), seeded)."""
    scene = synthetic.FusionScene(seed=seed, extent=EXTENT)
    for i in range(frames):
        R, t = scene.pose(i, frames)
        mm = scene.depth_frame(R, t, w=W, h=H, fx=FX, fy=FY, cx=CX, cy=CY, seed=seed * 1000 + i, device=device)
        yield R, t, synthetic.mm_to_u16_bits(mm)


def build_volume(mcg, synthetic, torch, n, frames, seed=0):
    v = mcg.voxel_new((n, n, n), TRUNC, TRUNC, EXTENT / n)
    k = mcg.intrinsic(FX, FY, CX, CY)
    t_int = 0.0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for R, t, d in fusion_frames(synthetic, frames, seed):
        ev0.record()
        m, _, _ = mcg.depth_to_maps(d, k, vertex=False, normal=False)
        mcg.volumetric_integration(v, k, mcg.extrinsic(R, t), m)
        ev1.record()
        torch.cuda.synchronize()
        t_int += ev0.elapsed_time(ev1) * 1e-3
    return v, {"frames": frames, "integrate_voxels_per_s": n ** 3 * frames / t_int if t_int else None,
               "integrate_ms_per_frame": 1e3 * t_int / max(frames, 1)}


def host_cores():
    """(cores this process may run on, cores the host reports, machine)."""
    import platform
    try:
        usable = len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        usable = os.cpu_count() or 1
    return usable, os.cpu_count() or usable, platform.machine()


def _time_cpu_extract(orc, vol_np, cell, nthreads, target_s, max_runs=50):
    times = []
    t_all = time.perf_counter()
    ntri = 0
    while not times or (time.perf_counter() - t_all < target_s and len(times) < max_runs):
        t0 = time.perf_counter()
        out = orc.mc_extract(vol_np, cell, normals=True, vi2vox=False, ver_voxel=False, tri_cube=False,
                             nthreads=nthreads)
        times.append(time.perf_counter() - t0)
        ntri = len(out["soup"]) // 3
    return float(np.median(times)), len(times), ntri


def cpu_baseline(orc, vol_np, cell, target_s=8.0):
    """Oracle (FP32 mirror) extraction of the same volume on all host threads
    (OpenMP over z-slabs), repeated for about target_s seconds of CPU work,
    and on one thread; Gvoxels/s."""
    nthreads = orc.max_threads()
    usable, nproc, machine = host_cores()
    vox = vol_np.shape[0] * vol_np.shape[1] * vol_np.shape[2]
    dt, runs, ntri = _time_cpu_extract(orc, vol_np, cell, nthreads, target_s)
    dt1, runs1, _ = _time_cpu_extract(orc, vol_np, cell, 1, target_s / 2, max_runs=5)
    shape = "x".join(map(str, vol_np.shape[:3]))
    return {"value": vox / dt / 1e9, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "oracle FP32-mirror extraction (classify+scan+generate+normals) of the whole %s volume, "
                      "%d triangles, median of %d runs (%.3f s each) on %d threads" % (shape, ntri, runs, dt,
                                                                                   nthreads),
            "single_thread": {"value": vox / dt1 / 1e9, "unit": UNIT, "cores": 1,
                              "sample": "the same extraction on one thread, median of %d runs (%.3f s each)"
                                        % (runs1, dt1)},
            "host": {"nproc": nproc, "usable_cores": usable, "machine": machine}}


def bench_full_outputs(mcg, torch, lib, ctx, vol, cell, nvert, stream, steps=50):
    """One step with every output of the reference's MarchingCubes::run
    (cu_marching_cubes_v1.cu:416-467): soup, vertexindex_to_voxel (vi2vox)
    and the volume-sized ver_voxel (cleared, then scattered), plus the
    normals its driver computes next -- beside the headline step, which
    writes soup + normals only."""
    import ctypes
    from marching_cube_gb300 import _capi
    nz, ny, nx = (int(x) for x in vol.shape[:3])
    soup = torch.empty((nvert, 28), dtype=torch.uint8, device="cuda")
    nrm = torch.empty((nvert, 3), dtype=torch.float32, device="cuda")
    v2v = torch.empty((nvert, 3), dtype=torch.int32, device="cuda")
    vv = torch.empty((nz, ny, nx), dtype=torch.int16, device="cuda")
    cv = _capi.Volume(vol.data_ptr(), nx, ny, nz, 0, float(cell))
    mo = _capi.MeshOut(soup.data_ptr(), nrm.data_ptr(), v2v.data_ptr(), vv.data_ptr(), None, nvert)
    s = ctypes.c_void_p(stream.cuda_stream)

    def step():
        ctx.check(lib.mcg_mc_classify(ctx.handle, ctypes.byref(cv), s), "classify")
        ctx.check(lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "generate")

    for _ in range(3):
        step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    c = mcg.counts(ctx)
    assert c["status"] == 0 and c["vertices"] == nvert
    ms = e0.elapsed_time(e1) / steps
    vox = nx * ny * nz
    del soup, nrm, v2v, vv
    return {"outputs": "soup+normals+vi2vox+ver_voxel (the reference run()'s full set)", "steps": steps,
            "ms_per_step": ms, "gvoxels_per_s": vox / (ms * 1e-3) / 1e9,
            "bytes_out_per_step": nvert * (28 + 12 + 12) + 2 * vox * 2}


def bench_batched(mcg, synthetic, torch, ctx, n=64, reps=30):
    """64 volumes, each axis log-uniform in [32, 256], 1-8 spheres/boxes:
    one batched extraction vs a loop of single-volume extractions (both
    asynchronous, into preallocated soup + normal buffers)."""
    vols = synthetic.batch_volumes(n, seed=7, lo=32, hi=256, device="cuda")
    cells = [0.01] * n
    meshes = mcg.extract_batched(vols, cells, normals=True)
    caps = [max(m.num_vertices, 1) for m in meshes]
    outs = [{"soup": torch.empty((c, 28), dtype=torch.uint8, device="cuda"),
             "normals": torch.empty((c, 3), dtype=torch.float32, device="cuda")} for c in caps]
    del meshes
    ctxs = ctx
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def loop():
        for v, o, c in zip(vols, outs, caps):
            mcg.extract_into(v, 0.01, o, c, ctx=ctxs)

    def batch():
        mcg.extract_batched_into(vols, cells, outs, caps, ctx=ctxs)

    res = {}
    for name, fn in (("loop", loop), ("batched", batch)):
        for _ in range(5):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        res[name + "_ms"] = e0.elapsed_time(e1) / reps
    vox = sum(int(v.shape[0]) * int(v.shape[1]) * int(v.shape[2]) for v in vols)
    tris = sum(c // 3 for c in caps)
    return {"volumes": n, "voxels": vox, "triangles": tris, "loop_ms": res["loop_ms"],
            "batched_ms": res["batched_ms"], "speedup": res["loop_ms"] / res["batched_ms"],
            "batched_gvoxels_per_s": vox / (res["batched_ms"] * 1e-3) / 1e9}


def bench_graph(mcg, synthetic, torch, n=256, frames=20):
    """Per-frame depth maps + integrate + extract of a 256^3 fusion volume,
    eager launches vs one captured CUDA graph replayed per frame."""
    scene = synthetic.FusionScene(seed=1, extent=EXTENT)
    k = mcg.intrinsic(FX, FY, CX, CY)
    depths = []
    poses = []
    for i in range(frames):
        R, t = scene.pose(i, frames)
        depths.append(synthetic.mm_to_u16_bits(scene.depth_frame(R, t, w=W, h=H, fx=FX, fy=FY, cx=CX, cy=CY,
                                                                  seed=i, device="cuda")))
        poses.append(mcg.extrinsic(R, t))
    ctx = mcg.Context()
    v = mcg.voxel_new((n, n, n), TRUNC, TRUNC, EXTENT / n)
    cap = 4 * 1000 * 1000
    out = {"soup": torch.empty((cap, 28), dtype=torch.uint8, device="cuda"),
           "normals": torch.empty((cap, 3), dtype=torch.float32, device="cuda")}
    d_in = torch.empty_like(depths[0])
    meter = torch.empty((H, W), dtype=torch.float32, device="cuda")
    import ctypes
    from marching_cube_gb300 import _capi
    lib = mcg._lib
    pose_all = torch.stack([mcg.extrinsic_tensor(*scene.pose(i, frames)) for i in range(frames)])
    pose_dev = torch.empty(12, dtype=torch.float32, device="cuda")

    def frame(stream):
        mcg.depth_to_maps(d_in, k, vertex=False, normal=False, ctx=ctx, stream=stream, out_meter=meter)
        mcg.volumetric_integration_device_pose(v, k, pose_dev, meter, ctx=ctx, stream=stream)
        mcg.extract_into(v.data, EXTENT / n, out, cap, ctx=ctx, stream=stream)

    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        d_in.copy_(depths[0])
        pose_dev.copy_(pose_all[0])
        frame(st)  # warm-up: scratch allocation, tables
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        e0.record(st)
        for i in range(frames):
            d_in.copy_(depths[i])
            pose_dev.copy_(pose_all[i])
            frame(st)
        e1.record(st)
    torch.cuda.synchronize()
    eager_ms = e0.elapsed_time(e1) / frames
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=st):
        frame(st)
    torch.cuda.synchronize()
    with torch.cuda.stream(st):
        e0.record(st)
        for i in range(frames):
            d_in.copy_(depths[i])
            pose_dev.copy_(pose_all[i])
            g.replay()
        e1.record(st)
    torch.cuda.synchronize()
    graph_ms = e0.elapsed_time(e1) / frames
    return {"volume": [n, n, n], "frames": frames, "eager_ms_per_frame": eager_ms, "graph_ms_per_frame": graph_ms}


def bench_batch_graph(mcg, synthetic, torch, nvol=64, frames=10, seed=11):
    """A multi-volume fusion frame: depth maps of one 640x480 frame, its
    integration into nvol volumes of uneven sizes (each axis log-uniform in
    32..256 voxels, each volume spanning the scene's 3 m cube), and one
    batched extraction of all of them into preallocated buffers; eager calls
    against one captured CUDA graph replayed per frame (the reference runs
    mc.run volume by volume, cu_kinect_fusion_v1.cu:3511-3737)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    dims = [tuple(int(d) for d in np.round(np.exp(rng.uniform(np.log(32), np.log(256), size=3))))
            for _ in range(nvol)]
    scene = synthetic.FusionScene(seed=2, extent=EXTENT)
    k = mcg.intrinsic(FX, FY, CX, CY)
    depths, poses = [], []
    for i in range(frames):
        R, t = scene.pose(i, frames)
        depths.append(synthetic.mm_to_u16_bits(scene.depth_frame(R, t, w=W, h=H, fx=FX, fy=FY, cx=CX, cy=CY,
                                                                  seed=100 + i, device="cuda")))
        poses.append(mcg.extrinsic_tensor(R, t))
    ctx = mcg.Context()
    vols = []
    for (nx, ny, nz) in dims:
        g = EXTENT / max(nx, ny, nz)
        vols.append(mcg.voxel_new((nx, ny, nz), 4 * g, 4 * g, g, ctx=ctx))
    cells = [v.grid_s for v in vols]
    saved = [v.data.clone() for v in vols]
    d_in = torch.empty_like(depths[0])
    meter = torch.empty((H, W), dtype=torch.float32, device="cuda")
    pose_dev = torch.empty(12, dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()
    # capacities: 1.5x the counts after integrating every frame once
    with torch.cuda.stream(st):
        mcg.depth_to_maps(depths[0], k, vertex=False, normal=False, ctx=ctx, stream=st, out_meter=meter)
        for i in range(frames):
            d_in.copy_(depths[i])
            pose_dev.copy_(poses[i])
            mcg.depth_to_maps(d_in, k, vertex=False, normal=False, ctx=ctx, stream=st, out_meter=meter)
            for v in vols:
                mcg.volumetric_integration_device_pose(v, k, pose_dev, meter, ctx=ctx, stream=st)
        meshes = mcg.extract_batched([v.data for v in vols], cells, ctx=ctx, stream=st)
    torch.cuda.synchronize()
    caps = [int(m.counts["vertices"] * 1.5) + 3000 for m in meshes]
    del meshes
    outs = [{"soup": torch.empty((c, 28), dtype=torch.uint8, device="cuda"),
             "normals": torch.empty((c, 3), dtype=torch.float32, device="cuda")} for c in caps]

    def frame():
        mcg.depth_to_maps(d_in, k, vertex=False, normal=False, ctx=ctx, stream=st, out_meter=meter)
        for v in vols:
            mcg.volumetric_integration_device_pose(v, k, pose_dev, meter, ctx=ctx, stream=st)
        mcg.extract_batched_into([v.data for v in vols], cells, outs, caps, ctx=ctx, stream=st)

    def restore():
        for v, s0 in zip(vols, saved):
            v.data.copy_(s0)

    def timed(step):
        restore()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(st):
            e0.record(st)
            for i in range(frames):
                d_in.copy_(depths[i])
                pose_dev.copy_(poses[i])
                step()
            e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / frames

    with torch.cuda.stream(st):
        frame()  # warm-up outside the capture: every buffer and spare sized
    torch.cuda.synchronize()
    eager_ms = timed(frame)
    counts_eager = [c["vertices"] for c in mcg.counts_batched(ctx, nvol)]
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=st):
        frame()
    torch.cuda.synchronize()
    graph_ms = timed(g.replay)
    cnt = mcg.counts_batched(ctx, nvol)
    assert [c["vertices"] for c in cnt] == counts_eager
    assert all(c["status"] == 0 for c in cnt)
    voxels = sum(nx * ny * nz for (nx, ny, nz) in dims)
    return {"volumes": nvol, "voxels": voxels, "frame": [W, H], "frames": frames,
            "triangles_last_frame": int(sum(counts_eager) // 3),
            "launches_per_frame": 1 + 3 * nvol + 6,
            "eager_ms_per_frame": eager_ms, "graph_ms_per_frame": graph_ms,
            "speedup": eager_ms / graph_ms}



def bench_raycast(mcg, synthetic, torch, v, reps=20):
    """Ray casting the headline volume into 640x480 depth + normal maps from
    poses of the orbit that built it (the fusion loop's model prediction)."""
    scene = synthetic.FusionScene(seed=0, extent=EXTENT)
    k = mcg.intrinsic(FX, FY, CX, CY)
    poses = [mcg.extrinsic(*scene.pose(i, reps)) for i in range(reps)]
    d = torch.empty((H, W), dtype=torch.float32, device="cuda")
    n = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    for e in poses[:3]:
        mcg.raycast(v, k, e, W, H, out_depth=d, out_normal=n)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for e in poses:
        mcg.raycast(v, k, e, W, H, out_depth=d, out_normal=n)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    return {"image": [W, H], "ms_per_frame": ms, "rays_per_s": W * H / (ms * 1e-3),
            "hit_fraction": float((d > 0).float().mean())}


def bench_text_load(mcg, synthetic, torch, v, hbm, dim=512, reps=10, sample_bytes=48 << 20):
    """Text-record loader (cu_voxel_rlc_to_mesh's volume load): the headline
    512^3 volume dumped as "x y z sdf weight" records of the window at
    (512, 512, 0), x outermost, z innermost (~3 GB of text), loaded back
    (a) from device memory, (b) from pageable and (c) pinned host memory,
    (d) from a page-cached file; beside it the reference loop over
    libstdc++ streams on a bounded sample, one core."""
    import numpy as np
    n = min(dim, v.data.shape[0])
    if n < v.data.shape[0]:
        v = mcg.Voxel(v.data[:n, :n, :n].contiguous(), v.min_t, v.max_t, v.grid_s)
    text = synthetic.text_dump(v.data, mcg.TEXT_ORIGIN)
    L = text.numel()
    out = torch.empty_like(v.data)
    stats = {}
    mcg.load_text_records(text, n, out=out, stats=stats)
    assert stats["stored"] == n ** 3 and torch.equal(out, v.data)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        mcg.load_text_records(text, n, out=out)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        mcg.load_text_records(text, n, out=out)
    e1.record()
    torch.cuda.synchronize()
    dev_ms = e0.elapsed_time(e1) / reps
    host = np.empty(L, np.uint8)
    host[:] = text.cpu().numpy()
    pinned = torch.empty(L, dtype=torch.uint8, pin_memory=True)
    pinned.copy_(text)
    del text
    torch.cuda.empty_cache()
    res = {}
    for name, src in (("pageable", host), ("pinned", pinned)):
        for _ in range(2):
            mcg.load_text_records(src, n, out=out)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(max(3, reps // 2)):
            mcg.load_text_records(src, n, out=out)
        torch.cuda.synchronize()
        res[name] = (time.perf_counter() - t0) / max(3, reps // 2)
    assert torch.equal(out, v.data)
    # the same text from a file (page cache warm after writing it)
    file_res = None
    try:
        import tempfile
        with tempfile.NamedTemporaryFile(suffix=".vol", delete=True) as f:
            f.write(memoryview(host))
            f.flush()
            mcg.load_text_records(f.name, n, out=out, tail_bytes=None)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(3):
                mcg.load_text_records(f.name, n, out=out, tail_bytes=None)
            torch.cuda.synchronize()
            fs = (time.perf_counter() - t0) / 3
        assert torch.equal(out, v.data)
        file_res = {"ms": fs * 1e3, "gbs": L / fs / 1e9, "h2d_bytes": L, "source": "page-cached file, pread"}
    except Exception as ex:  # pragma: no cover
        file_res = {"error": str(ex)}
    # CPU: the reference loop on the first sample_bytes (cut after a newline)
    cpu = None
    try:
        import oracle as orc
        cut = int(np.flatnonzero(host[:sample_bytes] == 10)[-1]) + 1
        sample = host[:cut].tobytes()
        t0 = time.perf_counter()
        _, st = orc.text_load(sample, n, mcg.TEXT_ORIGIN)
        cs = time.perf_counter() - t0
        cpu = {"value": cut / cs / 1e9, "unit": "GB/s of text", "cores": 1, "kind": "port",
               "sample": "first %d bytes (%d records) of the same dump" % (cut, st["stored"]),
               "seconds": cs}
    except Exception as ex:  # pragma: no cover
        cpu = {"value": None, "error": str(ex)}
    del host, pinned
    alg = L + 4 * n ** 3
    return {"workload": "text dump of the %d^3 window at (512,512,0), %d records" % (n, n ** 3),
            "text_bytes": L, "device_ms": dev_ms, "device_gbs": L / (dev_ms * 1e-3) / 1e9,
            "records_per_s": n ** 3 / (dev_ms * 1e-3),
            "roofline": {"bound": "alu", "alg_bytes": alg, "achieved": alg / (dev_ms * 1e-3) / 1e9,
                         "peak": hbm, "frac": alg / (dev_ms * 1e-3) / 1e9 / hbm,
                         "note": "GB/s of text read once + volume written once over the whole device parse, "
                                 "against the HBM copy peak; the field pass is integer-ALU bound"},
            "e2e_pageable": {"ms": res["pageable"] * 1e3, "gbs": L / res["pageable"] / 1e9,
                             "h2d_bytes": L},
            "e2e_pinned": {"ms": res["pinned"] * 1e3, "gbs": L / res["pinned"] / 1e9, "h2d_bytes": L},
            "e2e_file": file_res,
            "cpu_baseline": cpu}


def bench_mesh_write(mcg, torch, vol, cell, ctx, reps=5, sample_frac=0.25):
    """Mesh writers (kf.cu:3394-3424 PLY, 3625-3726 OBJ) on the headline
    soup: the reference's bytes built on the GPU and copied out (host
    buffers, no file system), beside the reference's writer (std::map of
    "%.4f" keys + fprintf, the oracle) on one core over the first quarter
    of the soup."""
    m = mcg.extract(vol, cell, soup=True, normals=True, ctx=ctx)
    nv = m.num_vertices
    res = {"soup_vertices": nv}
    for name, fn in (("obj", lambda: mcg.mesh_obj(m, ctx=ctx)), ("ply", lambda: mcg.mesh_ply(m, ctx=ctx))):
        out = fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            out = fn()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / reps
        nbytes = sum(len(x) for x in out) if isinstance(out, tuple) else len(out)
        res[name] = {"ms": dt * 1e3, "bytes": nbytes, "mvertices_per_s": nv / dt / 1e6}
    try:
        import oracle as orc
        k = (int(nv * sample_frac) // 3) * 3
        s = m.soup[:k].cpu().numpy()
        n = m.normals[:k].cpu().numpy()
        t0 = time.perf_counter()
        orc.mesh_obj(s, n)
        dt = time.perf_counter() - t0
        res["cpu_obj"] = {"mvertices_per_s": k / dt / 1e6, "cores": 1, "kind": "port",
                          "sample": "first %d soup vertices" % k, "seconds": dt}
    except Exception as ex:  # pragma: no cover
        res["cpu_obj"] = {"error": str(ex)}
    return res


def bench_icp(mcg, synthetic, torch, reps=10):
    """Frame-to-frame tracking (kf.cu:2105-2218): two 640x480 frames of the
    blended-spheres scene 1.8 degrees / 4 cm apart; per frame the depth
    pyramid (masks, pyramid_down, mask_to_data) is built once and timed
    separately, then ICP runs over 3 levels (15 / 11 / 8 iterations at most)
    from the identity; beside it the oracle's ICP (the same algorithm in C,
    one core) on the same maps."""
    import numpy as np
    scene = synthetic.BlendedSpheres(seed=3)
    w, h, f = 640, 480, 525.0
    k0 = mcg.intrinsic(f, f, 319.5, 239.5)
    P1, P2 = scene.pose(0, 200), scene.pose(1, 200)
    depth = [scene.depth_frame(*P, w=w, h=h, fx=f, fy=f, cx=319.5, cy=239.5, device="cuda").float().contiguous()
             for P in (P1, P2)]

    def build(d):
        lv, k = [], k0
        for i in range(3):
            if i > 0:
                m = mcg.float_data_to_mask(d)
                d, dm = mcg.pyramid_down(d, m)
                mcg.float_mask_to_data(dm, d)
                k = mcg.intrinsic_pyramid_down(k)
            v = mcg.meter_to_vertex(d, k)
            lv.append((v, mcg.vertex_to_normal(v)))
        return lv

    maps = [build(d) for d in depth]
    e0 = mcg.extrinsic(np.eye(3), np.zeros(3))
    inl = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        ok, e, iters = mcg.icp_pyramid(k0, e0, maps[0], maps[1], inlier=inl)
        build(depth[1])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        build(depth[1])
    torch.cuda.synchronize()
    pyr_ms = (time.perf_counter() - t0) / reps * 1e3
    t0 = time.perf_counter()
    for _ in range(reps):
        ok, e, iters = mcg.icp_pyramid(k0, e0, maps[0], maps[1], inlier=inl)
    torch.cuda.synchronize()
    icp_ms = (time.perf_counter() - t0) / reps * 1e3
    res = {"frame": [w, h], "levels": 3, "ok": ok, "iterations": iters, "pyramid_and_maps_ms": pyr_ms,
           "icp_ms": icp_ms, "ms_per_iteration": icp_ms / max(1, sum(iters))}
    try:
        import math
        import oracle as orc
        ks = [orc.intrinsic(f, f, 319.5, 239.5)]
        for _ in range(2):
            ks.append(orc.intrinsic(ks[-1].fx / 2, ks[-1].fy / 2, ks[-1].cx / 2, ks[-1].cy / 2))
        hm = [[(v.cpu().numpy(), n.cpu().numpy()) for v, n in lv] for lv in maps]
        oe = orc.extrinsic(np.eye(3), np.zeros(3))
        t0 = time.perf_counter()
        for lv, it_max in ((2, 8), (1, 11), (0, 15)):
            okc, (r, t), _, _ = orc.icp(math.cos(math.radians(20)), 0.10, math.radians(20), 0.10, it_max, ks[lv], oe,
                                        hm[0][lv][0], hm[0][lv][1], hm[1][lv][0], hm[1][lv][1])
            oe = orc.Extrinsic()
            for i in range(9):
                oe.r[i] = float(r[i])
            for i in range(3):
                oe.t[i] = float(t[i])
        res["cpu_icp"] = {"ms": (time.perf_counter() - t0) * 1e3, "cores": 1, "kind": "port",
                          "sample": "the same 3-level ICP on the same maps"}
    except Exception as ex:  # pragma: no cover
        res["cpu_icp"] = {"error": str(ex)}
    return res


def bench_indexed(mcg, torch, vol, cell, ctx, reps=10):
    """Indexed extraction (one vertex per crossed grid edge) of the headline
    volume into preallocated positions + normals + triangles, asynchronous,
    CUDA-event timed; beside it the output bytes of soup and indexed."""
    m = mcg.extract_indexed(vol, cell, normals=True, ctx=ctx)
    nv, nt = m.num_vertices, m.num_triangles
    out = {"positions": m.positions, "normals": m.normals, "triangles": m.triangles}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        mcg.extract_indexed_into(vol, cell, out, nv, nt, ctx=ctx)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        mcg.extract_indexed_into(vol, cell, out, nv, nt, ctx=ctx)
    e1.record()
    torch.cuda.synchronize()
    c = mcg.counts(ctx)
    assert c["status"] == 0 and c["vertices"] == nv
    ms = e0.elapsed_time(e1) / reps
    vox = vol.shape[0] * vol.shape[1] * vol.shape[2]
    return {"ms": ms, "gvoxels_per_s": vox / (ms * 1e-3) / 1e9, "vertices": nv, "triangles": nt,
            "out_bytes": nv * 24 + nt * 12, "soup_out_bytes": 3 * nt * (28 + 12),
            "outputs": "positions + normals (12 B each per vertex) + triangles (12 B)"}


def bench_stress(mcg, synthetic, torch, n=1024, reps=5):
    """1024^3 stress volume (4 GiB short2; 200 spheres + gradient noise):
    extraction (soup + normals) throughput, the FP32 volume's forward
    positions and MC adjoint, and the RLE codec's throughput with a
    bit-exact round trip (lossless variant) and a tsdf-exact one (reference
    format)."""
    vol = synthetic.stress_volume(n, seed=0)
    cell = 1.0 / n
    ctx = mcg.Context()
    m = mcg.extract(vol, cell, normals=True, ctx=ctx)
    nvert = m.num_vertices
    out = {"soup": m.soup, "normals": m.normals}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(2):
        mcg.extract_into(vol, cell, out, nvert, ctx=ctx)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        mcg.extract_into(vol, cell, out, nvert, ctx=ctx)
    e1.record()
    torch.cuda.synchronize()
    ext_ms = e0.elapsed_time(e1) / reps
    res = {"volume": [n, n, n], "triangles": m.num_triangles, "extract_ms": ext_ms,
           "extract_gvoxels_per_s": n ** 3 / (ext_ms * 1e-3) / 1e9}
    del m, out
    # FP32 volume: forward positions + MC adjoint
    f32 = torch.empty((n, n, n, 2), dtype=torch.float32, device="cuda")
    f32[..., 0] = vol[..., 0].to(torch.float32) / 32766.0
    f32[..., 1] = (vol[..., 1] != 0).to(torch.float32)
    pos = mcg.mesh_positions(f32, cell)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    G = torch.randn(pos.shape, device="cuda", generator=g)
    torch.cuda.synchronize()
    e0.record()
    pos = mcg.mesh_positions(f32, cell)
    e1.record()
    torch.cuda.synchronize()
    res["fp32_forward_ms"] = e0.elapsed_time(e1)
    e0.record()
    gf = mcg.mc_backward(f32, cell, G)
    e1.record()
    torch.cuda.synchronize()
    res["fp32_mc_adjoint_ms"] = e0.elapsed_time(e1)
    del f32, pos, G, gf
    # RLE codec (device volume <-> file image in host memory)
    v = mcg.Voxel(vol, 5 * cell, 5 * cell, cell)
    raw = n ** 3 * 4
    for lossless in (True, False):
        # the image buffer is allocated once and reused, as the mesh outputs are
        out = np.empty(len(mcg.rle_encode(v, lossless=lossless, ctx=ctx)), np.uint8)
        mcg.rle_encode(v, lossless=lossless, out=out, ctx=ctx)
        t0 = time.perf_counter()
        img = mcg.rle_encode(v, lossless=lossless, out=out, ctx=ctx)
        t1 = time.perf_counter()
        back = mcg.rle_decode(img, ctx=ctx)  # GPU expansion of the host image
        del back
        torch.cuda.synchronize()
        t1b = time.perf_counter()
        for _ in range(3):
            back = mcg.rle_decode(img, ctx=ctx)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        key = "rle_lossless" if lossless else "rle_reference_format"
        exact = bool(torch.equal(back.data, vol)) if lossless else bool(torch.equal(back.data[..., 0], vol[..., 0]))
        res[key] = {"bytes": len(img), "encode_mb_per_s": raw / (t1 - t0) / 1e6,
                    "decode_mb_per_s": raw / ((t2 - t1b) / 3) / 1e6,
                    "round_trip": "bit-exact" if (lossless and exact) else ("tsdf-exact" if exact else "MISMATCH")}
        del back
        try:
            import tempfile
            with tempfile.NamedTemporaryFile(suffix=".rle", delete=True) as f:
                f.write(img)
                f.flush()
                back = mcg.run_length_decode(f.name, ctx=ctx)
                del back
                torch.cuda.synchronize()
                t3 = time.perf_counter()
                back = mcg.run_length_decode(f.name, ctx=ctx)
                torch.cuda.synchronize()
                t4 = time.perf_counter()
            res[key]["file_decode_mb_per_s"] = raw / (t4 - t3) / 1e6
            res[key]["file_round_trip_exact"] = bool(torch.equal(back.data, vol)) if lossless else \
                bool(torch.equal(back.data[..., 0], vol[..., 0]))
            del back
            t5 = time.perf_counter()
            hv, _ = mcg.rle_decode_host(img)
            res[key]["host_decode_mb_per_s"] = raw / (time.perf_counter() - t5) / 1e6
            del hv
        except Exception as ex:  # pragma: no cover
            res[key]["file_error"] = str(ex)
        del img, out
    return res


def bench_adjoint(mcg, synthetic, torch, n=256, frames=10, reps=5):
    """Differentiable fusion of the blended-spheres scene: 10 sphere-traced
    320x240 depth frames (f 262.5) -> 256^3 float32 volume (trunc 4 voxels)
    -> soup positions P -> L = sum phi(P)^2 with phi the analytic blended
    field; forward and torch.autograd backward (integrate adjoint + MC
    adjoint) timed with CUDA events."""
    scene = synthetic.BlendedSpheres(seed=0)
    w, h, f = 320, 240, 262.5
    depth, poses = scene.frames(frames, w=w, h=h, fx=f, fy=f, device="cuda")
    depth = depth.to(torch.float32).contiguous()
    k = mcg.intrinsic(f, f, (w - 1) / 2.0, (h - 1) / 2.0)
    pt = torch.stack([mcg.extrinsic_tensor(R, t) for R, t in poses]).contiguous()
    shape = (n, n, n)
    gs = 1.0 / n
    trunc = 4 * gs

    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fw, bw = [], []
    for i in range(reps + 2):
        d = depth.clone().requires_grad_(True)
        torch.cuda.synchronize()
        e[0].record()
        vol = mcg.integrate_frames(d, pt, shape, trunc, trunc, gs, k)
        pos = mcg.mesh_positions(vol, gs)
        loss = (scene.sdf(pos) ** 2).sum()
        e[1].record()
        loss.backward()
        e[2].record()
        torch.cuda.synchronize()
        if i >= 2:
            fw.append(e[0].elapsed_time(e[1]))
            bw.append(e[1].elapsed_time(e[2]))
    # the path alone (no loss evaluation): forward integrate + extract, then
    # the two adjoint calls (count phase re-run + MC adjoint, integrate adjoint)
    vol = vol.detach()
    p = pos.detach().requires_grad_(True)
    (scene.sdf(p) ** 2).sum().backward()
    gpos = p.grad.contiguous()
    pf, pb, mb, ib = [], [], [], []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for i in range(reps + 2):
        torch.cuda.synchronize()
        ev[0].record()
        v2 = mcg.integrate_frames(depth, pt, shape, trunc, trunc, gs, k)
        mcg.mesh_positions(v2, gs)
        ev[1].record()
        gf = mcg.mc_backward(v2, gs, gpos)
        ev[2].record()
        mcg.integrate_backward(shape, trunc, trunc, gs, k, pt, depth, gf)
        ev[3].record()
        torch.cuda.synchronize()
        if i >= 2:
            pf.append(ev[0].elapsed_time(ev[1]))
            mb.append(ev[1].elapsed_time(ev[2]))
            ib.append(ev[2].elapsed_time(ev[3]))
            pb.append(ev[1].elapsed_time(ev[3]))
    fms, bms = float(np.median(fw)), float(np.median(bw))
    pfm, pbm = float(np.median(pf)), float(np.median(pb))
    return {"volume": list(shape), "frames": frames, "image": [w, h], "vertices": int(pos.shape[0]),
            "loss": "sum phi(P)^2 (phi: analytic field, torch ops)",
            "autograd_forward_ms": fms, "autograd_backward_ms": bms, "autograd_adjoint_over_forward": bms / fms,
            "path_forward_ms": pfm, "path_backward_ms": pbm, "path_adjoint_over_forward": pbm / pfm,
            "mc_backward_ms": float(np.median(mb)), "integrate_backward_ms": float(np.median(ib)),
            "precision": "fp32 accumulate (atomics)"}


def headline_config(n, frames, **extra):
    """The config dict both arms print for the headline workload."""
    cfg = {"workload": "mc_extract_512_fusion", "volume": [n, n, n], "voxel": "short2",
           "frames_integrated": frames, "outputs": "soup(vertex_voxel)+normals", "l2": "inputs larger than L2"}
    cfg.update(extra)
    return cfg


def oracle_volume(orc, synthetic, torch, n, frames, seed=0):
    """The headline volume built without this library: the same depth frames
    (drawn by torch, on the GPU when there is one, like the GPU arm's), turned
    into metres and integrated by the oracle on the host cores."""
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    vol = orc.voxel_init(n ** 3).reshape(n, n, n, 2)
    ko = orc.intrinsic(FX, FY, CX, CY)
    for R, t, d in fusion_frames(synthetic, frames, seed, device=dev):
        mo = orc.depth_to_meter(d.cpu().numpy().view(np.uint16))
        orc.integrate(vol, TRUNC, TRUNC, EXTENT / n, ko, orc.extrinsic(R, t), mo)
    return vol


def summarize(line):
    """A compact digest of the line's sections (None where a section did not run)."""
    def get(*path):
        x = line
        for k in path:
            if not isinstance(x, dict) or x.get(k) is None:
                return None
            x = x[k]
        return round(x, 4) if isinstance(x, float) else x
    return {
        "headline_gvoxels_per_s": get("value"), "ms_per_step": get("ms_per_step"),
        "launch_config": get("launch_config", "config"),
        "whole_step_frac": get("roofline", "whole_step", "frac"),
        "e2e_gvoxels_per_s": get("e2e", "value"),
        "full_outputs_ms": get("full_outputs", "ms_per_step"),
        "batched_speedup": get("batched", "speedup"), "batched_ms": get("batched", "batched_ms"),
        "loop_ms": get("batched", "loop_ms"),
        "batch_frame_graph_ms": get("graph", "batch", "graph_ms_per_frame"),
        "batch_frame_eager_ms": get("graph", "batch", "eager_ms_per_frame"),
        "adjoint_over_forward": get("adjoint", "path_adjoint_over_forward"),
        "integrate_ms_per_frame": get("integrate", "integrate_ms_per_frame"),
        "indexed_ms": get("indexed", "ms"), "stress_gvoxels_per_s": get("stress", "extract_gvoxels_per_s"),
        "raycast_ms": get("raycast", "ms_per_frame"),
        "cpu_gvoxels_per_s": get("cpu_baseline", "value"),
        "cpu_1thread_gvoxels_per_s": get("cpu_baseline", "single_thread", "value"),
        "cpu_cores": get("cpu_baseline", "cores"),
    }


def run_reference(args):
    """--impl reference: the reference has no CPU marching cubes (MyMarchingCube.h
    is a declaration only) and its GPU code cannot be built with this CUDA;
    its algorithm restated in C (oracle/) runs on all host cores, over the
    same volume (integrated by the oracle from the same frames)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import torch
    import oracle as orc
    from marching_cube_gb300 import synthetic
    orc.build()
    vol_np = oracle_volume(orc, synthetic, torch, args.n, args.frames)
    cell = EXTENT / args.n
    nthreads = orc.max_threads()
    usable, nproc, machine = host_cores()
    vals = []
    vox = vol_np.shape[0] * vol_np.shape[1] * vol_np.shape[2]
    ntri = 0
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        out = orc.mc_extract(vol_np, cell, normals=True, vi2vox=False, ver_voxel=False, tri_cube=False,
                             nthreads=nthreads)
        dt = time.perf_counter() - t0
        ntri = len(out["soup"]) // 3
        if i >= args.warmup:
            vals.append(vox / dt / 1e9)
    value = float(np.median(vals))
    cfg = headline_config(args.n, args.frames, triangles=ntri, parallelism="single")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": vox / value / 1e6,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "each step: oracle extraction (classify+scan+generate+normals) of the "
                                       "whole volume on all %d host threads" % nthreads,
                             "host": {"nproc": nproc, "usable_cores": usable, "machine": machine}},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import marching_cube_gb300 as mcg
    from marching_cube_gb300 import synthetic
    dev = torch.cuda.current_device()

    v, integ = build_volume(mcg, synthetic, torch, args.n, args.frames, seed=0)
    n = args.n
    vox = n ** 3
    cell = v.grid_s
    ctx = mcg.Context(dev)
    stream = torch.cuda.current_stream()

    # size the outputs from one counting pass
    mesh = mcg.extract(v.data, cell, normals=True, ctx=ctx)
    nvert = mesh.num_vertices
    counts = dict(mesh.counts)
    del mesh
    cap = nvert
    soup = torch.empty((cap, 28), dtype=torch.uint8, device="cuda")
    nrm = torch.empty((cap, 3), dtype=torch.float32, device="cuda")
    outs = {"soup": soup, "normals": nrm}

    import ctypes
    from marching_cube_gb300 import _capi
    cv = _capi.Volume(v.data.data_ptr(), n, n, n, 0, float(cell))
    mo = _capi.MeshOut(soup.data_ptr(), nrm.data_ptr(), None, None, None, cap)
    s = ctypes.c_void_p(stream.cuda_stream)
    lib = mcg._lib

    # the launch configuration: the library's autotuner times the candidates
    # on this volume and sets the fastest on ctx (not part of the timed steps)
    from marching_cube_gb300 import tune
    t_tune = time.perf_counter()
    tuned = tune.autotune(v.data, cell, ctx=ctx, reps=5, warmup=2, use_cache=False, store=False)
    t_tune = time.perf_counter() - t_tune
    fused = ctx.config["fused"] != 0

    def step(ev=None):
        """One extraction through mcg_mc_extract (with ev: the count and
        generate launches called apart, events between them)."""
        if ev is None:
            ctx.check(lib.mcg_mc_extract(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "extract")
            return
        ev[0].record(stream)
        ctx.check(lib.mcg_mc_classify(ctx.handle, ctypes.byref(cv), s), "classify")
        ev[1].record(stream)
        ctx.check(lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "generate")
        ev[2].record(stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # the timed steps carry no events between the phases: an event between
    # two launches would stop the second from starting while the first drains
    with Clocks(dev) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            step()
        t1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    total_ms = t0.elapsed_time(t1)
    # the count / generate split, from a separate run of steps with events
    # between the phases
    # between the phases, and the library's events around the classify
    # kernel alone (the count window also holds the scan)
    nsplit = min(args.steps, 50)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(nsplit)]
    ctx.check(lib.mcg_set_kernel_timing(ctx.handle, 1), "kernel timing")
    kms = []
    for i in range(nsplit):
        # with the fused launch: its one kernel timed alone; otherwise the
        # count / generate windows and the classify kernel alone
        step(None if fused else evs[i])
        km = ctypes.c_float(0.0)
        ctx.check(lib.mcg_mc_count_kernel_ms(ctx.handle, ctypes.byref(km)), "count kernel time")
        kms.append(km.value)
    ctx.check(lib.mcg_set_kernel_timing(ctx.handle, 0), "kernel timing")
    torch.cuda.synchronize()
    cls_ms = None if fused else float(np.mean([e[0].elapsed_time(e[1]) for e in evs]))
    gen_ms = None if fused else float(np.mean([e[1].elapsed_time(e[2]) for e in evs]))
    cls_kernel_ms = float(np.mean(kms))
    c = mcg.counts(ctx)
    assert c["status"] == 0 and c["vertices"] == nvert
    full_outputs = bench_full_outputs(mcg, torch, lib, ctx, v.data, cell, nvert, stream,
                                      steps=min(args.steps, 50))
    if world > 1:
        tt = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(tt.item())
    ms_per_step = total_ms / args.steps
    value = vox * world / (ms_per_step * 1e-3) / 1e9

    # ---- roofline --------------------------------------------------------
    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    ntri = counts["triangles"]
    # classify: every voxel read once (4 B) + 8 B per brick of counts
    bricks = ((n - 2) // 32 + 1) * ((n - 2) // 8 + 1) ** 2
    cls_bytes = 4 * vox + 8 * bricks
    # generate: active bricks' 32x8x8 voxels (4 B) + soup (28 B) + normals (12 B) per vertex
    out_bytes = nvert * (28 + 12)
    gen_bytes = out_bytes + 4 * 2048 * c["active_bricks"]
    alg_bytes = 4 * vox + out_bytes
    if fused:
        # the one fused kernel: the volume once + the soup and normals
        f_ach = alg_bytes / (cls_kernel_ms * 1e-3) / 1e9
        per_kernel = {"mc_fused_kernel": {"ms": cls_kernel_ms, "alg_bytes": alg_bytes, "achieved": f_ach,
                                          "frac": f_ach / hbm}}
        dominant = "mc_fused_kernel"
    else:
        # per kernel: classify from the events around it alone, generate from
        # its window (the generate call launches that one kernel)
        cls_ach = cls_bytes / (cls_kernel_ms * 1e-3) / 1e9
        gen_ach = gen_bytes / (gen_ms * 1e-3) / 1e9
        per_kernel = {"mc_classify_kernel": {"ms": cls_kernel_ms, "alg_bytes": cls_bytes, "achieved": cls_ach,
                                             "frac": cls_ach / hbm},
                      "mc_generate_kernel": {"ms": gen_ms, "alg_bytes": gen_bytes, "achieved": gen_ach,
                                             "frac": gen_ach / hbm}}
        dominant = "mc_classify_kernel" if cls_kernel_ms >= gen_ms else "mc_generate_kernel"
    achieved = per_kernel[dominant]["achieved"]
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": None, "kernel": dominant, "peak_source": peak_src, "per_kernel": per_kernel,
                "whole_step": {"alg_bytes": alg_bytes, "achieved_gbs": alg_bytes / (ms_per_step * 1e-3) / 1e9,
                               "frac": alg_bytes / (ms_per_step * 1e-3) / 1e9 / hbm},
                "classify_ms": cls_ms, "classify_kernel_ms": cls_kernel_ms, "generate_ms": gen_ms}

    # ---- e2e: host volume in, host mesh out, through the C ABI ------------
    e2e = None
    try:
        h_vol = torch.empty(v.data.shape, dtype=v.data.dtype, pin_memory=True)
        h_vol.copy_(v.data)
        h_soup = torch.empty((cap, 28), dtype=torch.uint8, pin_memory=True)
        h_nrm = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True)
        d_vol = torch.empty_like(v.data)
        cv2 = _capi.Volume(d_vol.data_ptr(), n, n, n, 0, float(cell))
        reps = max(3, min(args.steps, 10))

        def seq_trial():
            torch.cuda.synchronize()
            ta = time.perf_counter()
            for _ in range(reps):
                d_vol.copy_(h_vol, non_blocking=True)
                ctx.check(lib.mcg_mc_extract(ctx.handle, ctypes.byref(cv2), ctypes.byref(mo), s), "extract")
                h_soup.copy_(soup, non_blocking=True)
                h_nrm.copy_(nrm, non_blocking=True)
                torch.cuda.synchronize()
            return (time.perf_counter() - ta) / reps

        seq_trial()  # warm-up
        # each figure is the median of several timed trials: one trial is a
        # few tens of milliseconds of host-link traffic, which a single stall
        # on the host side would otherwise decide
        seq_t = sorted(seq_trial() for _ in range(3))
        e2e_s = seq_t[1]
        seq = {"value": vox / e2e_s / 1e9, "unit": UNIT, "ms_per_step": e2e_s * 1e3,
               "mode": "sequential: copy in, extract, copy out, then the next volume",
               "trials_ms_per_step": [t * 1e3 for t in seq_t]}
        # the public stream API: volume i+1's copy in overlaps volume i's
        # extraction and copy out (both link directions busy)
        xs = mcg.ExtractStream((n, n, n), float(cell), cap)
        for xc in xs.ctx:
            xc.set_config(**tuned["config"])
        outs = [{"soup": h_soup, "normals": h_nrm}]
        xs.run([h_vol] * 3, outs * 3)
        torch.cuda.synchronize()

        def stream_trial():
            ta = time.perf_counter()
            res = xs.run([h_vol] * reps, outs * reps)
            tb = time.perf_counter()
            assert all(r["vertices"] == ntri * 3 and r["status"] == 0 for r in res)
            return (tb - ta) / reps

        st_t = sorted(stream_trial() for _ in range(5))
        e2e_p = st_t[2]
        e2e = {"value": vox / e2e_p / 1e9, "unit": UNIT, "h2d_bytes_per_step": int(h_vol.numel() * 2),
               "d2h_bytes_per_step": int(cap * 40), "ms_per_step": e2e_p * 1e3,
               "mode": "ExtractStream: each step copies its volume in (pinned) and its soup + normals out; "
                       "step i+1's copy in overlaps step i's extraction and copy out; median of 5 trials "
                       "of %d volumes" % reps,
               "trials_ms_per_step": [t * 1e3 for t in st_t],
               "sequential": seq}
        del h_vol, h_soup, h_nrm, d_vol, xs
    except Exception as ex:  # pragma: no cover
        e2e = {"value": None, "unit": UNIT, "error": str(ex)}

    batched = None
    if not args.no_batched:
        try:
            batched = bench_batched(mcg, synthetic, torch, ctx)
        except Exception as ex:  # pragma: no cover
            batched = {"error": str(ex)}
    graph = None
    if not args.no_graph:
        try:
            graph = bench_graph(mcg, synthetic, torch)
        except Exception as ex:  # pragma: no cover
            graph = {"error": str(ex)}
        try:
            graph["batch"] = bench_batch_graph(mcg, synthetic, torch)
        except Exception as ex:  # pragma: no cover
            graph["batch"] = {"error": str(ex)}

    raycast = None
    if not args.no_raycast:
        try:
            raycast = bench_raycast(mcg, synthetic, torch, v)
        except Exception as ex:  # pragma: no cover
            raycast = {"error": str(ex)}

    text_load = None
    if not args.no_text_load:
        try:
            text_load = bench_text_load(mcg, synthetic, torch, v, hbm, dim=args.text_dim)
        except Exception as ex:  # pragma: no cover
            text_load = {"error": str(ex)}
        torch.cuda.empty_cache()

    mesh_write = None
    if not args.no_mesh_write:
        try:
            mesh_write = bench_mesh_write(mcg, torch, v.data, cell, ctx)
        except Exception as ex:  # pragma: no cover
            mesh_write = {"error": str(ex)}

    icp = None
    if not args.no_icp:
        try:
            icp = bench_icp(mcg, synthetic, torch)
        except Exception as ex:  # pragma: no cover
            icp = {"error": str(ex)}

    indexed = None
    if not args.no_indexed:
        try:
            indexed = bench_indexed(mcg, torch, v.data, cell, ctx)
        except Exception as ex:  # pragma: no cover
            indexed = {"error": str(ex)}

    stress = None
    if not args.no_stress:
        try:
            stress = bench_stress(mcg, synthetic, torch, n=args.stress_n)
        except Exception as ex:  # pragma: no cover
            stress = {"error": str(ex)}
        torch.cuda.empty_cache()

    adjoint = None
    if not args.no_adjoint:
        try:
            adjoint = bench_adjoint(mcg, synthetic, torch)
        except Exception as ex:  # pragma: no cover
            adjoint = {"error": str(ex)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            import oracle as orc
            orc.build()
            cpu = cpu_baseline(orc, v.data.cpu().numpy(), cell)
        except Exception as ex:  # pragma: no cover
            cpu = {"value": None, "error": str(ex)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16", "data": "synthetic",
        "config": headline_config(n, args.frames, triangles=ntri,
                                  parallelism="replicas" if world > 1 else "single"),
        "occupied_cubes": counts["occupied"],
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "clocks": clk.summary(), "gpu_launches": (1 if fused else 3) * args.steps,
        "launch_config": {"config": tuned["config"], "chosen_by": "marching_cube_gb300.tune.autotune on this volume",
                          "tune_s": round(t_tune, 3), "candidates_ms": tuned["timings"]},
        "triangles_per_s": ntri * world / (ms_per_step * 1e-3),
        "full_outputs": full_outputs,
        "integrate": integ,
        "batched": batched,
        "graph": graph,
        "adjoint": adjoint,
        "indexed": indexed,
        "raycast": raycast,
        "text_load": text_load,
        "mesh_write": mesh_write,
        "icp": icp,
        "stress": stress,
    }
    # the figures of the other workloads again, compact and last, so that a
    # reader of the end of the line sees them
    line["summary"] = summarize(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
