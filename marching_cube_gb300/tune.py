"""Autotuner for the marching-cubes launch configuration (mcg_mc_config).

The extraction has three tunable choices, each a field of a context's
configuration (mcg_mc_set_config): whether mcg_mc_extract runs the fused
single launch (and with 4- or 2-brick work items) or the count + generate
launches; the count pass's work-item shape (bricks per item, halo box,
stage ring, CTA size); and how many bricks each generate CTA takes in fixed
rounds before it draws from the counter.  Which is fastest depends on the
part (SM count, memory system) and on the volume (its size, and how much of
it the surface occupies), so the tuner times the candidates on a volume of
the caller's and keeps the winner:

    cfg = tune.autotune(volume, cell, ctx=ctx)      # times, caches, applies
    tune.apply_cached(ctx, volume)                  # later: cache lookup only

Timing is a coordinate search with CUDA events over `reps` extractions per
candidate (into soup + normal buffers sized by one count pass): the count
shape with the default rounds, then the rounds with the best shape, then the
fused modes against the best two-launch configuration.  Every candidate
produces the same mesh bit for bit (tests/test_classify_configs_gpu.py,
tests/test_fused_gpu.py), so the choice is speed alone.

Results are cached in a JSON file (MCG_TUNE_CACHE, default
~/.cache/marching_cube_gb300/tune.json) under the device name and a shape
class: voxel type and each edge rounded up to a power of two.
"""
import ctypes
import json
import os

import torch

from . import _capi

FIELDS = ("fused", "classify_shape", "gen_fixed_rounds")
CLASSIFY_SHAPES = (0, 1, 2, 3, 4, 5)
FIXED_ROUNDS = (0, 1, 2, 3, 5)
FUSED_MODES = (1, 2)


def cache_path():
    return os.environ.get("MCG_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "marching_cube_gb300", "tune.json"))


def _pow2(n):
    p = 1
    while p < n:
        p <<= 1
    return p


def shape_class(shape, voxel_type):
    """Cache key part of a (nz, ny, nx) volume: its voxel type and each edge
    rounded up to a power of two."""
    nz, ny, nx = (int(x) for x in shape)
    return "%s-%dx%dx%d" % ("short2" if voxel_type == 0 else "float2", _pow2(nx), _pow2(ny), _pow2(nz))


def cache_key(device_name, shape, voxel_type):
    return "%s|%s" % (device_name, shape_class(shape, voxel_type))


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def store_cache(key, entry, path=None):
    path = path or cache_path()
    d = load_cache(path)
    d[key] = entry
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _device_name(device):
    return torch.cuda.get_device_name(device)


def apply_cached(ctx, volume, path=None):
    """Sets ctx's configuration from the cache for volume's device and shape
    class; returns the configuration, or None when nothing is cached."""
    vt = 0 if volume.dtype == torch.int16 else 1
    entry = load_cache(path).get(cache_key(_device_name(volume.device), volume.shape[:3], vt))
    if not entry:
        return None
    cfg = {k: int(entry["config"][k]) for k in FIELDS}
    ctx.set_config(**cfg)
    return cfg


def autotune(volume, cell, ctx=None, reps=10, warmup=3, path=None, use_cache=True, store=True):
    """Times the candidate configurations on `volume` (a (nz, ny, nx, 2)
    device tensor) and sets the fastest on ctx (the device's default context
    when None).  Returns {"config": {...}, "ms": best time per extraction,
    "timings": {candidate: ms}, "cached": bool}."""
    from . import default_context, extract, MCG_OK, MCG_ERR_CAPACITY
    from . import _lib, _cvol
    ctx = ctx or default_context(volume.device.index)
    vt = 0 if volume.dtype == torch.int16 else 1
    key = cache_key(_device_name(volume.device), volume.shape[:3], vt)
    if use_cache:
        entry = load_cache(path).get(key)
        if entry:
            cfg = {k: int(entry["config"][k]) for k in FIELDS}
            ctx.set_config(**cfg)
            return {"config": cfg, "ms": entry.get("ms"), "timings": entry.get("timings", {}), "cached": True}
    saved = ctx.config
    n = max(extract(volume, cell, soup=True, normals=False, ctx=ctx).num_vertices, 3)
    soup = torch.empty((n, 28), dtype=torch.uint8, device=volume.device)
    nrm = torch.empty((n, 3), dtype=torch.float32, device=volume.device)
    cv = _cvol(volume, cell)
    mo = _capi.MeshOut(soup.data_ptr(), nrm.data_ptr(), None, None, None, n)
    stream = torch.cuda.current_stream(volume.device)
    s = ctypes.c_void_p(stream.cuda_stream)
    timings = {}

    def run(cfg):
        label = "fused=%d,classify_shape=%d,gen_fixed_rounds=%d" % tuple(cfg[k] for k in FIELDS)
        if label in timings:
            return timings[label]
        ctx.set_config(**cfg)
        for _ in range(warmup):
            ctx.check(_lib.mcg_mc_extract(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "mcg_mc_extract")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            ctx.check(_lib.mcg_mc_extract(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "mcg_mc_extract")
        e1.record(stream)
        torch.cuda.synchronize(volume.device)
        c = _capi.MeshCounts()
        st = _lib.mcg_mc_counts(ctx.handle, ctypes.byref(c))
        if st not in (MCG_OK, MCG_ERR_CAPACITY):
            ctx.check(st, "mcg_mc_counts")
        timings[label] = e0.elapsed_time(e1) / reps
        return timings[label]

    try:
        best = dict(saved, fused=0)
        for cs in CLASSIFY_SHAPES:
            cand = dict(best, classify_shape=cs)
            if run(cand) < run(best):
                best = cand
        for fr in FIXED_ROUNDS:
            cand = dict(best, gen_fixed_rounds=fr)
            if run(cand) < run(best):
                best = cand
        for fm in FUSED_MODES:
            cand = dict(best, fused=fm)
            if run(cand) < run(best):
                best = cand
    except Exception:
        ctx.set_config(**saved)
        raise
    ms = run(best)
    ctx.set_config(**best)
    if store:
        store_cache(key, {"config": best, "ms": ms, "timings": timings, "shape": list(volume.shape[:3]),
                          "cell": float(cell)}, path)
    return {"config": best, "ms": ms, "timings": timings, "cached": False}
