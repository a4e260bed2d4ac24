"""GB300-native TSDF -> mesh path (marching cubes, integrate, depth maps, RLE).

Python host layer over the C ABI of libmcg.so (include/mcg.h).  PyTorch is
used only to own device memory and to supply the current CUDA stream; every
computation runs in the library's CUDA kernels.  The names mirror the
reference's C++ interface:

    MarchingCubes.run                 cu_marching_cubes_v1.h:28-65
    voxel_new / voxel_delete          cu_kinect_fusion_v1.h:215-216
    volumetric_integration            cu_kinect_fusion_v1.h:187-188
    depth_to_maps (+ meter_to_vertex, vertex_to_normal)
                                      cu_kinect_fusion_v1.cu:99-151
    extract_surface_normals           cu_kinect_fusion_v1.cu:3227-3242
    run_length_encode / _decode       cu_kinect_fusion_v1.h:218-219

Adjoints (no counterpart in the reference): mc_backward / integrate_backward
and the autograd Functions behind mesh_positions / integrate_frames.

Volumes are torch tensors of shape (nz, ny, nx, 2): int16 for the reference's
short2 voxels {tsdf, w} (w reinterpreted as uint16), float32 for the FP32
volume of the differentiable path.
"""
import ctypes
import dataclasses
import os
from typing import Optional

import torch

from . import _capi

_lib = _capi.load()

MCG_OK = 0
MCG_ERR_INVALID_ARG = 1
MCG_ERR_CAPACITY = 2
MCG_ERR_CUDA = 3
MCG_ERR_TIMEOUT = 4
MCG_ERR_IO = 5
MCG_ERR_FORMAT = 6
MCG_ERR_STATE = 7
MCG_ERR_TOO_LARGE = 8

VOXEL_SHORT2 = 0
VOXEL_FLOAT2 = 1

MAX_TSDF = 32766                       # cu_kinect_fusion_v1.h:44
DEFAULT_TRIANGLES_BUFFER_SIZE = 9 * 1000 * 1000 * 3   # cu_marching_cubes_v1.h:35
KINECT_DEPTH_MIN = 0.0                 # cu_kinect_fusion_v1.h:32
KINECT_DEPTH_MAX = 2.0                 # cu_kinect_fusion_v1.h:33
VERTEX_VOXEL_BYTES = 28


class MCGError(RuntimeError):
    def __init__(self, status, what, cuda_error=0):
        msg = "%s: %s" % (what, _lib.mcg_status_string(status).decode())
        if status == MCG_ERR_CUDA:
            msg += " (cudaError %d)" % cuda_error
        super().__init__(msg)
        self.status = status
        self.cuda_error = cuda_error


def library_path():
    return _capi.LIB_PATH


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream(stream=None):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


class Context:
    """Owns one mcg_context (scratch buffers, counters) on one device."""

    def __init__(self, device=None):
        if device is None:
            device = torch.cuda.current_device()
        self.device = int(device)
        h = ctypes.c_void_p()
        st = _lib.mcg_create(ctypes.byref(h), self.device)
        if st != MCG_OK:
            raise MCGError(st, "mcg_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def check(self, st, what):
        if st != MCG_OK:
            raise MCGError(st, what, _lib.mcg_last_cuda_error(self._h))

    @property
    def config(self):
        """The marching-cubes launch configuration (mcg_mc_config) as a dict:
        fused, classify_shape, gen_fixed_rounds."""
        c = _capi.McConfig()
        self.check(_lib.mcg_mc_get_config(self._h, ctypes.byref(c)), "mcg_mc_get_config")
        return {"fused": c.fused, "classify_shape": c.classify_shape, "gen_fixed_rounds": c.gen_fixed_rounds}

    def set_config(self, **kw):
        """Changes fields of the launch configuration (the others stay)."""
        cur = self.config
        unknown = set(kw) - set(cur)
        if unknown:
            raise KeyError("unknown configuration fields: %s" % sorted(unknown))
        cur.update(kw)
        c = _capi.McConfig(int(cur["fused"]), int(cur["classify_shape"]), int(cur["gen_fixed_rounds"]), 0)
        self.check(_lib.mcg_mc_set_config(self._h, ctypes.byref(c)), "mcg_mc_set_config")

    def close(self):
        if getattr(self, "_h", None):
            _lib.mcg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = {}


def default_context(device=None):
    if device is None:
        device = torch.cuda.current_device()
    ctx = _default_ctx.get(device)
    if ctx is None:
        ctx = _default_ctx[device] = Context(device)
    return ctx


def _voxel_type(vol):
    if vol.dtype == torch.int16:
        return VOXEL_SHORT2
    if vol.dtype == torch.float32:
        return VOXEL_FLOAT2
    raise TypeError("volume must be int16 (short2) or float32 (float2), got %s" % vol.dtype)


def _check_volume(vol):
    if not vol.is_cuda or vol.dim() != 4 or vol.shape[3] != 2 or not vol.is_contiguous():
        raise ValueError("volume must be a contiguous CUDA tensor of shape (nz, ny, nx, 2)")
    return _voxel_type(vol)


def _cvol(vol, cell):
    vt = _check_volume(vol)
    nz, ny, nx, _ = vol.shape
    return _capi.Volume(vol.data_ptr(), nx, ny, nz, vt, float(cell))


# ---------------------------------------------------------------------------
# voxel volume (structure.h:20-27 cu_voxel)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Voxel:
    """cu_voxel: size (x, y, z), truncation bounds, grid size and the data."""
    data: torch.Tensor
    min_t: float
    max_t: float
    grid_s: float

    @property
    def size(self):
        nz, ny, nx, _ = self.data.shape
        return (nx, ny, nz)

    @property
    def size_xy(self):
        return self.size[0] * self.size[1]


def voxel_init(data, ctx=None, stream=None):
    """Every voxel -> {tsdf=-32766, w=0} (FP32: {-1, 0}); kf.cu:364-379."""
    vt = _check_volume(data)
    ctx = ctx or default_context(data.device.index)
    n = data.numel() // 2
    ctx.check(_lib.mcg_voxel_init(ctx.handle, _ptr(data), vt, n, _stream(stream)), "mcg_voxel_init")


def voxel_new(size, min_t, max_t, grid_s, dtype=torch.int16, device=None, ctx=None, stream=None):
    """cu_voxel_new (kf.cu:381-398): allocate and initialise a volume."""
    nx, ny, nz = (int(s) for s in size)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    data = torch.empty((nz, ny, nx, 2), dtype=dtype, device=device)
    voxel_init(data, ctx, stream)
    return Voxel(data, float(min_t), float(max_t), float(grid_s))


def voxel_delete(v: Voxel):
    """cu_voxel_delete (kf.cu:3245-3258): release the data, zero the fields."""
    v.data = torch.empty((0, 0, 0, 2), dtype=v.data.dtype, device=v.data.device)
    v.min_t = v.max_t = v.grid_s = 0.0


# ---------------------------------------------------------------------------
# marching cubes
# ---------------------------------------------------------------------------
class Mesh:
    """Triangle soup as produced by MarchingCubes::run, plus optional side
    outputs.  soup is the raw 28-byte vertex_voxel records (N, 28) uint8."""

    def __init__(self, soup=None, normals=None, vi2vox=None, ver_voxel=None, tri_cube=None,
                 counts=None):
        self.soup = soup
        self.normals = normals
        self.vi2vox = vi2vox
        self.ver_voxel = ver_voxel
        self.tri_cube = tri_cube
        self.counts = counts or {}

    @property
    def num_vertices(self):
        return int(self.counts.get("vertices", 0))

    @property
    def num_triangles(self):
        return int(self.counts.get("triangles", 0))

    def _words(self):
        return self.soup.view(torch.int32).view(-1, 7)

    @property
    def positions(self):
        return self.soup.view(torch.float32).view(-1, 7)[:, 0:3]

    @property
    def vox_pos(self):
        return self._words()[:, 3:6]

    @property
    def tsdf(self):
        return self.soup.view(torch.int16).view(-1, 14)[:, 12]

    @property
    def w(self):
        return self.soup.view(torch.int16).view(-1, 14)[:, 13]


def _alloc_outputs(n, nvox, device, soup, normals, vi2vox, ver_voxel, tri_cube):
    out = {}
    out["soup"] = torch.empty((n, VERTEX_VOXEL_BYTES), dtype=torch.uint8, device=device) if soup else None
    out["normals"] = torch.empty((n, 3), dtype=torch.float32, device=device) if normals else None
    out["vi2vox"] = torch.empty((n, 3), dtype=torch.int32, device=device) if vi2vox else None
    out["ver_voxel"] = torch.empty((nvox,), dtype=torch.int16, device=device) if ver_voxel else None
    out["tri_cube"] = torch.empty((n // 3,), dtype=torch.int64, device=device) if tri_cube else None
    return out


def _mesh_out(o, cap):
    return _capi.MeshOut(
        o["soup"].data_ptr() if o["soup"] is not None else None,
        o["normals"].data_ptr() if o["normals"] is not None else None,
        o["vi2vox"].data_ptr() if o["vi2vox"] is not None else None,
        o["ver_voxel"].data_ptr() if o["ver_voxel"] is not None else None,
        o["tri_cube"].data_ptr() if o["tri_cube"] is not None else None,
        int(cap))


def counts(ctx):
    c = _capi.MeshCounts()
    st = _lib.mcg_mc_counts(ctx.handle, ctypes.byref(c))
    if st not in (MCG_OK, MCG_ERR_CAPACITY):
        ctx.check(st, "mcg_mc_counts")
    return {"occupied": c.occupied, "triangles": c.triangles, "vertices": c.vertices,
            "active_bricks": c.active_bricks, "status": c.status}


def extract(volume, cell, *, soup=True, normals=True, vi2vox=False, ver_voxel=False, tri_cube=False,
            ctx=None, stream=None) -> Mesh:
    """Marching cubes over a (nz, ny, nx, 2) volume; outputs sized exactly.

    Runs the count phase, reads the totals (one host synchronisation, as the
    reference's getOccupiedVoxels / computeOffsetsAndTotalVertexes do), then
    generates into exactly-sized buffers."""
    ctx = ctx or default_context(volume.device.index)
    cv = _cvol(volume, cell)
    s = _stream(stream)
    ctx.check(_lib.mcg_mc_classify(ctx.handle, ctypes.byref(cv), s), "mcg_mc_classify")
    c = counts(ctx)
    n = c["vertices"]
    nz, ny, nx, _ = volume.shape
    o = _alloc_outputs(n, nx * ny * nz, volume.device, soup, normals, vi2vox, ver_voxel, tri_cube)
    mo = _mesh_out(o, n)
    ctx.check(_lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "mcg_mc_generate")
    return Mesh(o["soup"], o["normals"], o["vi2vox"], o["ver_voxel"], o["tri_cube"], c)


class IndexedMesh:
    """Indexed mesh: vertices shared between triangles (one per crossed grid
    edge), triangles as (T, 3) int32 vertex indices in the soup's order and
    winding."""

    def __init__(self, positions=None, normals=None, vi2vox=None, vertex_edge=None, triangles=None, tri_cube=None,
                 counts=None):
        self.positions = positions
        self.normals = normals
        self.vi2vox = vi2vox
        self.vertex_edge = vertex_edge
        self.triangles = triangles
        self.tri_cube = tri_cube
        self.counts = counts or {}

    @property
    def num_vertices(self):
        return int(self.counts.get("vertices", 0))

    @property
    def num_triangles(self):
        return int(self.counts.get("triangles", 0))


def _indexed_out(o, capv, capt):
    def ptr(k):
        return o[k].data_ptr() if o.get(k) is not None else None
    return _capi.IndexedOut(ptr("positions"), ptr("normals"), ptr("vi2vox"), ptr("vertex_edge"), ptr("triangles"),
                            ptr("tri_cube"), int(capv), int(capt))


def extract_indexed(volume, cell, *, normals=True, vi2vox=False, vertex_edge=False, tri_cube=False, ctx=None,
                    stream=None) -> IndexedMesh:
    """Indexed marching cubes: count phase, one host synchronisation for the
    sizes, then vertices and triangles into exactly-sized buffers."""
    ctx = ctx or default_context(volume.device.index)
    cv = _cvol(volume, cell)
    s = _stream(stream)
    ctx.check(_lib.mcg_mc_classify_indexed(ctx.handle, ctypes.byref(cv), s), "mcg_mc_classify_indexed")
    c = counts(ctx)
    nv, nt = c["vertices"], c["triangles"]
    dev = volume.device
    o = {"positions": torch.empty((nv, 3), dtype=torch.float32, device=dev),
         "normals": torch.empty((nv, 3), dtype=torch.float32, device=dev) if normals else None,
         "vi2vox": torch.empty((nv, 3), dtype=torch.int32, device=dev) if vi2vox else None,
         "vertex_edge": torch.empty((nv,), dtype=torch.int64, device=dev) if vertex_edge else None,
         "triangles": torch.empty((nt, 3), dtype=torch.int32, device=dev),
         "tri_cube": torch.empty((nt,), dtype=torch.int64, device=dev) if tri_cube else None}
    io = _indexed_out(o, nv, nt)
    ctx.check(_lib.mcg_mc_generate_indexed(ctx.handle, ctypes.byref(cv), ctypes.byref(io), s),
              "mcg_mc_generate_indexed")
    return IndexedMesh(o["positions"], o["normals"], o["vi2vox"], o["vertex_edge"], o["triangles"], o["tri_cube"], c)


def extract_indexed_into(volume, cell, outputs: dict, capacity_vertices, capacity_triangles, ctx=None, stream=None):
    """Asynchronous indexed extraction into preallocated buffers (keys as
    IndexedMesh's attributes); counts(ctx) afterwards gives the sizes."""
    ctx = ctx or default_context(volume.device.index)
    cv = _cvol(volume, cell)
    io = _indexed_out(outputs, capacity_vertices, capacity_triangles)
    ctx.check(_lib.mcg_mc_extract_indexed(ctx.handle, ctypes.byref(cv), ctypes.byref(io), _stream(stream)),
              "mcg_mc_extract_indexed")
    return ctx


def extract_slab(volume, cell, z0, z1, *, soup=True, normals=True, vi2vox=False, tri_cube=False, ctx=None,
                 stream=None) -> Mesh:
    """Marching cubes over the cubes with z0 <= z < z1 (z0 a multiple of 8):
    the part of extract(volume) those cubes emit, in the same order, so the
    slabs of consecutive ranges concatenate to the whole soup."""
    ctx = ctx or default_context(volume.device.index)
    cv = _cvol(volume, cell)
    s = _stream(stream)
    ctx.check(_lib.mcg_mc_classify_slab(ctx.handle, ctypes.byref(cv), int(z0), int(z1), s), "mcg_mc_classify_slab")
    c = counts(ctx)
    n = c["vertices"]
    nz, ny, nx, _ = volume.shape
    o = _alloc_outputs(n, nx * ny * nz, volume.device, soup, normals, vi2vox, False, tri_cube)
    mo = _mesh_out(o, n)
    ctx.check(_lib.mcg_mc_generate(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), s), "mcg_mc_generate")
    return Mesh(o["soup"], o["normals"], o["vi2vox"], None, o["tri_cube"], c)


def extract_into(volume, cell, outputs: dict, capacity, ctx=None, stream=None):
    """Asynchronous extraction into preallocated buffers (no host sync).

    outputs: dict with any of soup/normals/vi2vox/ver_voxel/tri_cube tensors.
    Call counts(ctx) afterwards for the totals and the capacity status."""
    ctx = ctx or default_context(volume.device.index)
    cv = _cvol(volume, cell)
    o = {k: outputs.get(k) for k in ("soup", "normals", "vi2vox", "ver_voxel", "tri_cube")}
    mo = _mesh_out(o, capacity)
    ctx.check(_lib.mcg_mc_extract(ctx.handle, ctypes.byref(cv), ctypes.byref(mo), _stream(stream)),
              "mcg_mc_extract")
    return ctx


class ExtractStream:
    """Extraction of a sequence of host volumes (a fusion run's frames, a
    directory of volumes) with the host link kept busy in both directions:
    volume i+1 is copied to the device while volume i is extracted and its
    soup + normals are copied back.  Two contexts, two device volumes and
    two output sets alternate; copies in each direction have their own
    stream.  Host buffers should be pinned (page-locked) for the copies to
    overlap."""

    def __init__(self, shape, cell, capacity, device=None, normals=True):
        nz, ny, nx = (int(x) for x in shape)
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self.cell = float(cell)
        self.capacity = int(capacity)
        self.ctx = [Context(self.device.index), Context(self.device.index)]
        self.vol = [torch.empty((nz, ny, nx, 2), dtype=torch.int16, device=self.device) for _ in range(2)]
        self.out = [{"soup": torch.empty((self.capacity, VERTEX_VOXEL_BYTES), dtype=torch.uint8, device=self.device),
                     "normals": torch.empty((self.capacity, 3), dtype=torch.float32, device=self.device)
                     if normals else None} for _ in range(2)]
        self.s_in = torch.cuda.Stream(self.device)
        self.s_out = torch.cuda.Stream(self.device)
        self.s_run = [torch.cuda.Stream(self.device), torch.cuda.Stream(self.device)]

    def run(self, host_volumes, host_outputs):
        """host_volumes: (nz, ny, nx, 2) int16 host tensors; host_outputs:
        dicts with "soup" ((capacity, 28) uint8) and "normals" ((capacity, 3)
        float32) host tensors, one per volume (they may repeat once their
        copy has been consumed).  Returns the counts of every volume (status
        MCG_ERR_CAPACITY when a soup was cut at the capacity)."""
        ev_in = [torch.cuda.Event(), torch.cuda.Event()]
        ev_run = [torch.cuda.Event(), torch.cuda.Event()]
        ev_out = [torch.cuda.Event(), torch.cuda.Event()]
        used = [False, False]
        results = [None] * len(host_volumes)
        pending = [None, None]  # volume index last extracted with each buffer set

        def collect(b):
            if pending[b] is not None:
                results[pending[b]] = counts(self.ctx[b])
                pending[b] = None

        for i, hv in enumerate(host_volumes):
            b = i & 1
            if used[b]:  # the buffers of volume i - 2: extraction read, outputs copied out
                self.s_in.wait_event(ev_run[b])
            with torch.cuda.stream(self.s_in):
                self.vol[b].copy_(hv, non_blocking=True)
            ev_in[b].record(self.s_in)
            collect(b)
            self.s_run[b].wait_event(ev_in[b])
            if used[b]:
                self.s_run[b].wait_event(ev_out[b])
            extract_into(self.vol[b], self.cell, self.out[b], self.capacity, ctx=self.ctx[b],
                         stream=self.s_run[b])
            ev_run[b].record(self.s_run[b])
            pending[b] = i
            self.s_out.wait_event(ev_run[b])
            ho = host_outputs[i]
            with torch.cuda.stream(self.s_out):
                for k in ("soup", "normals"):
                    if self.out[b][k] is not None and ho.get(k) is not None:
                        ho[k].copy_(self.out[b][k], non_blocking=True)
            ev_out[b].record(self.s_out)
            used[b] = True
        self.s_out.synchronize()
        for b in (0, 1):
            collect(b)
        return results


def extract_batched(volumes, cells, *, soup=True, normals=True, vi2vox=False, ver_voxel=False, tri_cube=False,
                    ctx=None, stream=None):
    """Marching cubes over many volumes (same voxel type, any sizes) with one
    launch per pass; returns one Mesh per volume, identical to extract() of
    that volume."""
    if not volumes:
        return []
    if not isinstance(cells, (list, tuple)):
        cells = [cells] * len(volumes)
    ctx = ctx or default_context(volumes[0].device.index)
    n = len(volumes)
    cvs = (_capi.Volume * n)(*[_cvol(v, c) for v, c in zip(volumes, cells)])
    s = _stream(stream)
    ctx.check(_lib.mcg_mc_classify_batched(ctx.handle, cvs, n, s), "mcg_mc_classify_batched")
    cnt = (_capi.MeshCounts * n)()
    st = _lib.mcg_mc_counts_batched(ctx.handle, cnt, n)
    if st not in (MCG_OK, MCG_ERR_CAPACITY):
        ctx.check(st, "mcg_mc_counts_batched")
    allocs, outs = [], (_capi.MeshOut * n)()
    for i, v in enumerate(volumes):
        nz, ny, nx, _ = v.shape
        o = _alloc_outputs(cnt[i].vertices, nx * ny * nz, v.device, soup, normals, vi2vox, ver_voxel, tri_cube)
        allocs.append(o)
        outs[i] = _mesh_out(o, cnt[i].vertices)
    ctx.check(_lib.mcg_mc_generate_batched(ctx.handle, cvs, outs, n, s), "mcg_mc_generate_batched")
    meshes = []
    for i, o in enumerate(allocs):
        c = {"occupied": cnt[i].occupied, "triangles": cnt[i].triangles, "vertices": cnt[i].vertices,
             "active_bricks": 0, "status": 0}
        meshes.append(Mesh(o["soup"], o["normals"], o["vi2vox"], o["ver_voxel"], o["tri_cube"], c))
    return meshes


def extract_batched_into(volumes, cells, outputs, capacities, ctx=None, stream=None):
    """Asynchronous batched extraction into preallocated buffers (no host
    synchronisation); outputs[i] is a dict like extract_into's."""
    if not isinstance(cells, (list, tuple)):
        cells = [cells] * len(volumes)
    ctx = ctx or default_context(volumes[0].device.index)
    n = len(volumes)
    cvs = (_capi.Volume * n)(*[_cvol(v, c) for v, c in zip(volumes, cells)])
    outs = (_capi.MeshOut * n)()
    for i in range(n):
        o = {k: outputs[i].get(k) for k in ("soup", "normals", "vi2vox", "ver_voxel", "tri_cube")}
        outs[i] = _mesh_out(o, capacities[i])
    ctx.check(_lib.mcg_mc_extract_batched(ctx.handle, cvs, outs, n, _stream(stream)), "mcg_mc_extract_batched")
    return ctx


def counts_batched(ctx, n):
    cnt = (_capi.MeshCounts * n)()
    st = _lib.mcg_mc_counts_batched(ctx.handle, cnt, n)
    if st not in (MCG_OK, MCG_ERR_CAPACITY):
        ctx.check(st, "mcg_mc_counts_batched")
    return [{"occupied": c.occupied, "triangles": c.triangles, "vertices": c.vertices, "status": c.status}
            for c in cnt]


class MarchingCubes:
    """cu_marching_cubes_v1.h:28-65.  run() returns the triangle soup; if the
    caller's buffer is empty it is sized from the count phase."""

    POINTS_PER_TRIANGLE = 3
    DEFAULT_TRIANGLES_BUFFER_SIZE = DEFAULT_TRIANGLES_BUFFER_SIZE

    def __init__(self, ctx=None):
        self.ctx = ctx

    def run(self, tsdf: Voxel, normals=True, vi2vox=True, ver_voxel=True, stream=None) -> Mesh:
        return extract(tsdf.data, tsdf.grid_s, soup=True, normals=normals, vi2vox=vi2vox,
                       ver_voxel=ver_voxel, tri_cube=False, ctx=self.ctx, stream=stream)


def extract_surface_normals(volume, cell, soup, ctx=None, stream=None):
    """d_voxel_extract_surface_normals (kf.cu:3236-3242) over vertex records."""
    ctx = ctx or default_context(volume.device.index)
    cv = _cvol(volume, cell)
    n = soup.shape[0]
    out = torch.empty((n, 3), dtype=torch.float32, device=volume.device)
    ctx.check(_lib.mcg_mc_normals(ctx.handle, ctypes.byref(cv), _ptr(soup), n, _ptr(out), _stream(stream)),
              "mcg_mc_normals")
    return out


# ---------------------------------------------------------------------------
# cameras, depth maps, integrate
# ---------------------------------------------------------------------------
def intrinsic(fx, fy, cx, cy):
    k = _capi.Intrinsic()
    k.fx, k.fy, k.cx, k.cy = float(fx), float(fy), float(cx), float(cy)
    return k


def extrinsic(R, t):
    """camera -> global pose; R is a 3x3 rotation (row-major nested list or
    array), stored column-major as the reference's float33."""
    import numpy as np
    R = np.asarray(R, dtype=np.float32).reshape(3, 3)
    e = _capi.Extrinsic()
    cols = R.T.reshape(-1)  # column 0 first
    for i in range(9):
        e.r[i] = float(cols[i])
    for i in range(3):
        e.t[i] = float(np.asarray(t, dtype=np.float32).reshape(3)[i])
    return e


def depth_to_maps(depth_mm, k, depth_min=KINECT_DEPTH_MIN, depth_max=KINECT_DEPTH_MAX, meter=True,
                  vertex=True, normal=True, ctx=None, stream=None, out_meter=None, out_vertex=None,
                  out_normal=None):
    """uint16-mm depth (h, w) -> metre (h, w), vertex (h, w, 3), normal (h, w, 3).
    out_* may supply preallocated outputs (e.g. inside a CUDA graph capture)."""
    if depth_mm.dtype not in (torch.int16, torch.uint16) or not depth_mm.is_cuda or depth_mm.dim() != 2:
        raise ValueError("depth_mm must be a (h, w) 16-bit CUDA tensor")
    depth_mm = depth_mm.contiguous()
    ctx = ctx or default_context(depth_mm.device.index)
    h, w = depth_mm.shape
    dev = depth_mm.device
    m = out_meter if out_meter is not None else (
        torch.empty((h, w), dtype=torch.float32, device=dev) if meter else None)
    v = out_vertex if out_vertex is not None else (
        torch.empty((h, w, 3), dtype=torch.float32, device=dev) if vertex else None)
    n = out_normal if out_normal is not None else (
        torch.empty((h, w, 3), dtype=torch.float32, device=dev) if normal else None)
    ctx.check(_lib.mcg_depth_to_maps(ctx.handle, ctypes.byref(k), w, h, _ptr(depth_mm), float(depth_min),
                                     float(depth_max), _ptr(m), _ptr(v), _ptr(n), _stream(stream)),
              "mcg_depth_to_maps")
    return m, v, n


def meter_to_vertex(meter, k, ctx=None, stream=None):
    meter = meter.contiguous()
    ctx = ctx or default_context(meter.device.index)
    h, w = meter.shape
    v = torch.empty((h, w, 3), dtype=torch.float32, device=meter.device)
    ctx.check(_lib.mcg_meter_to_vertex(ctx.handle, ctypes.byref(k), w, h, _ptr(meter), _ptr(v), _stream(stream)),
              "mcg_meter_to_vertex")
    return v


def vertex_to_normal(vertex, ctx=None, stream=None):
    vertex = vertex.contiguous()
    ctx = ctx or default_context(vertex.device.index)
    h, w, _ = vertex.shape
    n = torch.empty_like(vertex)
    ctx.check(_lib.mcg_vertex_to_normal(ctx.handle, w, h, _ptr(vertex), _ptr(n), _stream(stream)),
              "mcg_vertex_to_normal")
    return n


def volumetric_integration(v: Voxel, k, e, depth_m, normals=None, is_dynamic=False, ctx=None, stream=None):
    """_cu_voxel_volumetric_integration (kf.cu:534-549): fuse one depth frame
    (metres, (h, w) float32 CUDA tensor) into v in place."""
    vt = _check_volume(v.data)
    depth_m = depth_m.contiguous()
    if normals is not None:
        normals = normals.contiguous()
    ctx = ctx or default_context(v.data.device.index)
    h, w = depth_m.shape
    nx, ny, nz = v.size
    ctx.check(_lib.mcg_integrate(ctx.handle, _ptr(v.data), vt, nx, ny, nz, v.min_t, v.max_t, v.grid_s,
                                 ctypes.byref(k), ctypes.byref(e), w, h, _ptr(depth_m), _ptr(normals),
                                 1 if is_dynamic else 0, _stream(stream)),
              "mcg_integrate")


def raycast(v: Voxel, k, e, w, h, normals=True, out_depth=None, out_normal=None, ctx=None, stream=None):
    """_cu_voxel_extract_depth_and_normal_map (kf.cu:786-986): depth (h, w)
    metres and camera-frame normals (h, w, 3) of a short2 volume seen by
    camera (k, e).  out_* may supply preallocated outputs."""
    if v.data.dtype != torch.int16:
        raise TypeError("ray casting reads short2 (int16) volumes")
    _check_volume(v.data)
    ctx = ctx or default_context(v.data.device.index)
    nx, ny, nz = v.size
    dev = v.data.device
    d = out_depth if out_depth is not None else torch.empty((h, w), dtype=torch.float32, device=dev)
    n = out_normal if out_normal is not None else (
        torch.empty((h, w, 3), dtype=torch.float32, device=dev) if normals else None)
    ctx.check(_lib.mcg_raycast(ctx.handle, _ptr(v.data), nx, ny, nz, v.grid_s, ctypes.byref(k), ctypes.byref(e), w, h,
                               _ptr(d), _ptr(n), _stream(stream)), "mcg_raycast")
    return d, n


def extrinsic_tensor(R, t, device=None):
    """Pose as a 12-float device tensor (rotation column-major, then t) for
    volumetric_integration_device_pose."""
    import numpy as np
    e = extrinsic(R, t)
    host = torch.tensor(list(e.r) + list(e.t), dtype=torch.float32)
    return host.to(device or torch.device("cuda", torch.cuda.current_device()))


def volumetric_integration_device_pose(v: Voxel, k, pose_dev, depth_m, normals=None, is_dynamic=False, ctx=None,
                                       stream=None):
    """volumetric_integration with the pose read from a device tensor (12
    floats), so a captured CUDA graph can be replayed with new poses."""
    vt = _check_volume(v.data)
    if pose_dev.dtype != torch.float32 or pose_dev.numel() != 12 or not pose_dev.is_cuda:
        raise ValueError("pose_dev must be 12 float32 values on the device")
    ctx = ctx or default_context(v.data.device.index)
    h, w = depth_m.shape
    nx, ny, nz = v.size
    ctx.check(_lib.mcg_integrate_device_pose(ctx.handle, _ptr(v.data), vt, nx, ny, nz, v.min_t, v.max_t, v.grid_s,
                                             ctypes.byref(k), _ptr(pose_dev), w, h, _ptr(depth_m), _ptr(normals),
                                             1 if is_dynamic else 0, _stream(stream)),
              "mcg_integrate_device_pose")


# ---------------------------------------------------------------------------
# adjoints: soup positions -> voxel values -> depth pixels
# ---------------------------------------------------------------------------
def mc_backward(volume, cell, grad_pos, grad_f=None, *, reclassify=True, ctx=None, stream=None):
    """dL/df per voxel, (nz, ny, nx) float32, for dL/dP of the soup vertices
    of extract(volume, cell) in the same order (grad_pos (n, 3) float32).
    f is the tsdf of a float32 volume, tsdf/32766 of an int16 one.  grad_f,
    if given, is accumulated into.  reclassify=False reuses the count phase
    the last extraction on ctx ran for this volume (the volume must be
    unchanged since)."""
    ctx = ctx or default_context(volume.device.index)
    cv = _cvol(volume, cell)
    s = _stream(stream)
    nz, ny, nx, _ = volume.shape
    if grad_f is None:
        grad_f = torch.zeros((nz, ny, nx), dtype=torch.float32, device=volume.device)
    elif grad_f.dtype != torch.float32 or grad_f.numel() != nx * ny * nz or not grad_f.is_contiguous():
        raise ValueError("grad_f must be a contiguous float32 tensor of nz*ny*nx values")
    grad_pos = grad_pos.to(torch.float32).contiguous()
    if grad_pos.dim() != 2 or grad_pos.shape[1] != 3:
        raise ValueError("grad_pos must be (n, 3)")
    if reclassify:
        ctx.check(_lib.mcg_mc_classify(ctx.handle, ctypes.byref(cv), s), "mcg_mc_classify")
    ctx.check(_lib.mcg_mc_backward(ctx.handle, ctypes.byref(cv), _ptr(grad_pos), grad_pos.shape[0], _ptr(grad_f),
                                   s), "mcg_mc_backward")
    return grad_f


def _poses_tensor(poses, device):
    if isinstance(poses, torch.Tensor):
        p = poses.to(device=device, dtype=torch.float32).reshape(-1, 12).contiguous()
    else:
        p = torch.stack([extrinsic_tensor(R, t, device) for R, t in poses]).contiguous()
    return p


def integrate_backward(shape, min_t, max_t, grid_s, k, poses, depth, grad_f, grad_w=None, vol0=None, normals=None,
                       is_dynamic=False, grad_depth=None, want_grad_vol0=False, ctx=None, stream=None):
    """Adjoint of integrating depth frames (K, h, w) into a float32 volume of
    shape (nz, ny, nx) with poses (K, 12) (see integrate_frames).  Returns
    (grad_depth, grad_f0, grad_w0); the last two are None unless
    want_grad_vol0.  Pixel choices, truncation and clamping are held fixed;
    normal maps are constants."""
    nz, ny, nx = shape
    dev = depth.device
    ctx = ctx or default_context(dev.index)
    depth = depth.to(torch.float32).contiguous()
    nf, h, w = depth.shape
    pt = _poses_tensor(poses, dev)
    if pt.shape[0] != nf:
        raise ValueError("one pose per depth frame")
    if grad_depth is None:
        grad_depth = torch.zeros_like(depth)
    gf = grad_f.to(torch.float32).contiguous()
    gw = grad_w.to(torch.float32).contiguous() if grad_w is not None else None
    if gf.numel() != nx * ny * nz or (gw is not None and gw.numel() != nx * ny * nz):
        raise ValueError("grad_f / grad_w must hold one value per voxel")
    if vol0 is not None:
        if vol0.dtype != torch.float32 or tuple(vol0.shape) != (nz, ny, nx, 2) or not vol0.is_contiguous():
            raise ValueError("vol0 must be a contiguous float32 (nz, ny, nx, 2) tensor")
    nrm = normals.to(torch.float32).contiguous() if normals is not None else None
    gf0 = torch.empty((nz, ny, nx), dtype=torch.float32, device=dev) if want_grad_vol0 else None
    gw0 = torch.empty((nz, ny, nx), dtype=torch.float32, device=dev) if want_grad_vol0 else None
    ctx.check(_lib.mcg_integrate_backward(ctx.handle, _ptr(vol0), nx, ny, nz, min_t, max_t, grid_s, ctypes.byref(k),
                                          nf, _ptr(pt), w, h, _ptr(depth), _ptr(nrm), 1 if is_dynamic else 0,
                                          _ptr(gf), _ptr(gw), _ptr(grad_depth), _ptr(gf0), _ptr(gw0),
                                          _stream(stream)),
              "mcg_integrate_backward")
    return grad_depth, gf0, gw0


class MarchingCubesFunction(torch.autograd.Function):
    """volume (nz, ny, nx, 2) float32 -> soup positions (n, 3); the gradient
    flows into the tsdf channel (the weight channel only selects cubes)."""

    @staticmethod
    def forward(fctx, volume, cell):
        mesh = extract(volume, cell, soup=True, normals=False)
        pos = mesh.positions.contiguous() if mesh.num_vertices else torch.zeros(
            (0, 3), dtype=torch.float32, device=volume.device)
        fctx.save_for_backward(volume)
        fctx.cell = float(cell)
        return pos

    @staticmethod
    def backward(fctx, grad_pos):
        (volume,) = fctx.saved_tensors
        if not fctx.needs_input_grad[0]:
            return None, None
        gv = torch.zeros_like(volume)
        if grad_pos.shape[0]:
            gf = mc_backward(volume, fctx.cell, grad_pos)
            gv[..., 0] = gf
        return gv, None


def mesh_positions(volume, cell):
    """Differentiable soup positions of a float32 volume."""
    if volume.dtype != torch.float32:
        raise TypeError("the differentiable path takes float32 (float2) volumes")
    return MarchingCubesFunction.apply(volume, cell)


class IntegrateFunction(torch.autograd.Function):
    """depth frames (K, h, w) [+ initial volume] -> float32 volume
    (nz, ny, nx, 2) after integrating every frame in order."""

    @staticmethod
    def forward(fctx, depth, vol0, poses, shape, min_t, max_t, grid_s, k, normals, is_dynamic):
        nz, ny, nx = shape
        dev = depth.device
        depth_c = depth.to(torch.float32).contiguous()
        pt = _poses_tensor(poses, dev)
        if vol0 is not None:
            vol = vol0.detach().clone()
        else:
            vol = torch.empty((nz, ny, nx, 2), dtype=torch.float32, device=dev)
            voxel_init(vol)
        v = Voxel(vol, min_t, max_t, grid_s)
        nrm = normals.to(torch.float32).contiguous() if normals is not None else None
        for f in range(depth_c.shape[0]):
            volumetric_integration_device_pose(v, k, pt[f], depth_c[f], None if nrm is None else nrm[f],
                                               is_dynamic)
        fctx.save_for_backward(depth_c, pt, vol0 if vol0 is not None else None, nrm)
        fctx.params = (tuple(shape), min_t, max_t, grid_s, k, is_dynamic)
        return vol

    @staticmethod
    def backward(fctx, grad_vol):
        depth, pt, vol0, nrm = fctx.saved_tensors
        shape, min_t, max_t, grid_s, k, is_dynamic = fctx.params
        grad_vol = grad_vol.contiguous()
        want0 = vol0 is not None and fctx.needs_input_grad[1]
        gd, gf0, gw0 = integrate_backward(shape, min_t, max_t, grid_s, k, pt, depth, grad_vol[..., 0], grad_vol[..., 1],
                                          vol0=vol0.detach().contiguous() if vol0 is not None else None,
                                          normals=nrm, is_dynamic=is_dynamic, want_grad_vol0=want0)
        g0 = torch.stack([gf0, gw0], dim=-1) if want0 else None
        return (gd if fctx.needs_input_grad[0] else None), g0, None, None, None, None, None, None, None, None


def integrate_frames(depth, poses, shape, min_t, max_t, grid_s, k, vol0=None, normals=None, is_dynamic=False):
    """Differentiable fusion of depth frames (K, h, w metres, z-depth) with
    camera -> global poses (K, 12 device tensor, or a list of (R, t)) into a
    float32 volume (nz, ny, nx, 2), starting from vol0 or the initial state."""
    return IntegrateFunction.apply(depth, vol0, poses, tuple(shape), float(min_t), float(max_t), float(grid_s), k,
                                   normals, bool(is_dynamic))


# ---------------------------------------------------------------------------
# RLE volume I/O (kf.cu:1303-1600)
# ---------------------------------------------------------------------------
def _image_out(cap, fill):
    """Runs fill(pointer, capacity, size_ref) into a fresh bytearray of cap
    bytes and returns the bytearray cut to the written size (in place, no
    copy; ctypes.string_at would take a 32-bit length and truncate images of
    2 GiB and more)."""
    buf = bytearray(cap)
    view = (ctypes.c_uint8 * cap).from_buffer(buf)
    size = ctypes.c_int64(0)
    try:
        st = fill(ctypes.c_void_p(ctypes.addressof(view)), cap, ctypes.byref(size))
    finally:
        del view
    del buf[size.value:]
    return st, buf


def _image_in(image):
    """(pointer, length, keep-alive) of a bytes-like file image."""
    import numpy as np
    arr = np.frombuffer(image, dtype=np.uint8)
    return arr.ctypes.data_as(ctypes.c_void_p), arr.size, arr


def rle_encode(v: Voxel, lossless=False, out=None, ctx=None, stream=None) -> memoryview:
    """Encode a short2 volume into the reference's RLE file image (on the
    GPU).  out: optional writable buffer reused across calls; the result is a
    memoryview of the written bytes (of `out`, or of a new buffer sized
    exactly)."""
    import numpy as np
    if v.data.dtype != torch.int16:
        raise TypeError("RLE volumes are short2 (int16) volumes")
    ctx = ctx or default_context(v.data.device.index)
    nx, ny, nz = v.size
    size = ctypes.c_int64(0)

    def call(ptr, cap):
        return _lib.mcg_rle_encode(ctx.handle, _ptr(v.data), nx, ny, nz, v.min_t, v.max_t, v.grid_s,
                                   1 if lossless else 0, ptr, cap, ctypes.byref(size), _stream(stream))

    if out is None:
        ctx.check(call(None, 0), "mcg_rle_encode")  # exact size first
        buf = np.empty(size.value, np.uint8)
    else:
        buf = np.frombuffer(out, dtype=np.uint8)
        if buf.flags.writeable is False:
            raise ValueError("out must be writable")
    ctx.check(call(buf.ctypes.data_as(ctypes.c_void_p), buf.size), "mcg_rle_encode")
    return memoryview(buf)[: size.value]


def rle_header(image):
    dims = (ctypes.c_int32 * 3)()
    params = (ctypes.c_float * 3)()
    p, n, _keep = _image_in(image)
    st = _lib.mcg_rle_header(p, n, dims, params)
    if st != MCG_OK:
        raise MCGError(st, "mcg_rle_header")
    return (dims[0], dims[1], dims[2]), (params[0], params[1], params[2])


def rle_decode(image, device=None, ctx=None, stream=None) -> Voxel:
    (nx, ny, nz), (min_t, max_t, grid_s) = rle_header(image)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    data = torch.empty((nz, ny, nx, 2), dtype=torch.int16, device=device)
    ctx = ctx or default_context(data.device.index)
    p, n, _keep = _image_in(image)
    ctx.check(_lib.mcg_rle_decode(ctx.handle, p, n, _ptr(data), nx * ny * nz, _stream(stream)), "mcg_rle_decode")
    return Voxel(data, min_t, max_t, grid_s)


def rle_encode_host(vol, min_t, max_t, grid_s, lossless=False) -> bytearray:
    """Encode a host (numpy) short2 volume (nz, ny, nx, 2) int16; no GPU needed."""
    import numpy as np
    vol = np.ascontiguousarray(vol, dtype=np.int16)
    if vol.ndim != 4 or vol.shape[3] != 2:
        raise ValueError("volume must be (nz, ny, nx, 2)")
    nz, ny, nx, _ = vol.shape
    st, img = _image_out(_lib.mcg_rle_bound(nx, ny, nz), lambda p, cap, size: _lib.mcg_rle_encode_host(
        vol.ctypes.data_as(ctypes.c_void_p), nx, ny, nz, float(min_t), float(max_t), float(grid_s),
        1 if lossless else 0, p, cap, size))
    if st != MCG_OK:
        raise MCGError(st, "mcg_rle_encode_host")
    return img


def rle_decode_host(image):
    """Decode a file image into a host numpy volume; returns (vol, (min_t, max_t, grid_s))."""
    import numpy as np
    (nx, ny, nz), params = rle_header(image)
    vol = np.empty((nz, ny, nx, 2), np.int16)
    p, n, _keep = _image_in(image)
    st = _lib.mcg_rle_decode_host(p, n, vol.ctypes.data_as(ctypes.c_void_p), nx * ny * nz)
    if st != MCG_OK:
        raise MCGError(st, "mcg_rle_decode_host")
    return vol, params


def run_length_encode(v: Voxel, file_name, lossless=False):
    """cu_voxel_run_length_encode (kf.cu:1451-1478), whole-volume form."""
    img = rle_encode(v, lossless)
    with open(file_name, "wb") as f:
        f.write(img)


def run_length_decode(file_name, device=None, ctx=None, stream=None) -> Voxel:
    """cu_voxel_run_length_decode (kf.cu:1533-1563), whole-volume form: the
    file streams to the GPU in pieces and is expanded there."""
    try:
        with open(file_name, "rb") as f:
            head = f.read(40)
    except OSError as ex:
        raise MCGError(MCG_ERR_IO, "mcg_rle_decode_file: %s" % ex)
    (nx, ny, nz), _ = rle_header(head)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    data = torch.empty((nz, ny, nx, 2), dtype=torch.int16, device=device)
    ctx = ctx or default_context(data.device.index)
    dims = (ctypes.c_int32 * 3)()
    params = (ctypes.c_float * 3)()
    ctx.check(_lib.mcg_rle_decode_file(ctx.handle, os.fsencode(file_name), _ptr(data), nx * ny * nz, dims, params,
                                       _stream(stream)), "mcg_rle_decode_file")
    return Voxel(data, params[0], params[1], params[2])


# ---------------------------------------------------------------------------
# text-record volume loader (kf.cu:3289-3361)
# ---------------------------------------------------------------------------
TEXT_TAIL_BYTES = 11_000_000_000   # kf.cu:3316 seekg(-11000000000, end)
TEXT_ORIGIN = (512, 512, 0)        # kf.cu:3314 xs, ys, zs
TEXT_GRID_S = 0.003                # kf.cu:3271 local_volume.grid_s


def load_text_records(source, dim, origin=TEXT_ORIGIN, tail_bytes=TEXT_TAIL_BYTES, out=None, grid_s=TEXT_GRID_S,
                      stats=None, device=None, ctx=None, stream=None) -> Voxel:
    """The volume loader of cu_voxel_rlc_to_mesh: "x y z sdf weight" text
    records inside [origin, origin + dim)^3 fill a dim^3 short2 volume in
    arrival order (z fastest, then y, then x), parsed on the GPU.

    source: a path (the last tail_bytes of the file, the reference's seek and
    line skip; tail_bytes=None reads it whole), host bytes (bytes, bytearray,
    memoryview, numpy uint8, CPU uint8 tensor) or a CUDA uint8 tensor.
    out: optional (dim, dim, dim, 2) int16 CUDA tensor to fill.  stats: an
    optional dict receiving the mcg_text_info fields.  Raises MCGError with
    MCG_ERR_FORMAT where the reference's loop would never end."""
    import numpy as np
    dim = int(dim)
    if out is None:
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        out = torch.empty((dim, dim, dim, 2), dtype=torch.int16, device=device)
    elif out.dtype != torch.int16 or tuple(out.shape) != (dim, dim, dim, 2) or not out.is_contiguous() \
            or not out.is_cuda:
        raise ValueError("out must be a contiguous (dim, dim, dim, 2) int16 CUDA tensor")
    ctx = ctx or default_context(out.device.index)
    org = (ctypes.c_int32 * 3)(*(int(o) for o in origin))
    info = _capi.TextInfo()
    if isinstance(source, (str, os.PathLike)):
        tail = 0 if tail_bytes is None else int(tail_bytes)
        st = _lib.mcg_text_records_load_file(ctx.handle, os.fsencode(source), tail, dim, org, _ptr(out),
                                             ctypes.byref(info), _stream(stream))
        what = "mcg_text_records_load_file"
    elif isinstance(source, torch.Tensor) and source.is_cuda:
        if source.dtype != torch.uint8 or not source.is_contiguous():
            raise ValueError("device text must be a contiguous uint8 tensor")
        st = _lib.mcg_text_records_parse(ctx.handle, _ptr(source), source.numel(), dim, org, _ptr(out),
                                         ctypes.byref(info), _stream(stream))
        what = "mcg_text_records_parse"
    else:
        if isinstance(source, torch.Tensor):
            source = source.numpy()
        arr = np.frombuffer(source, dtype=np.uint8) if not isinstance(source, np.ndarray) else source
        if arr.dtype != np.uint8 or not arr.flags.c_contiguous:
            raise ValueError("host text must be contiguous bytes")
        st = _lib.mcg_text_records_load(ctx.handle, arr.ctypes.data_as(ctypes.c_void_p), arr.size, dim, org,
                                        _ptr(out), ctypes.byref(info), _stream(stream))
        what = "mcg_text_records_load"
    if stats is not None:
        stats.update({k: getattr(info, k) for k, _ in _capi.TextInfo._fields_ if k != "reserved"})
    ctx.check(st, what)
    return Voxel(out, 0.0, 0.0, float(grid_s))


# ---------------------------------------------------------------------------
# mesh writers (kf.cu:3394-3424 PLY, 3625-3726 OBJ), built on the GPU
# ---------------------------------------------------------------------------
def _mesh_args(mesh: Mesh, n):
    n = mesh.num_vertices if n is None else int(n)
    if mesh.soup is None or mesh.normals is None:
        raise ValueError("the writers need the soup and its normals")
    if n > mesh.soup.shape[0] or n > mesh.normals.shape[0]:
        raise ValueError("n exceeds the soup")
    return n


def mesh_ply(mesh: Mesh, n=None, ctx=None, stream=None) -> bytes:
    """The reference's binary PLY image of the soup (header, positions +
    normals, faces (3i, 3i+1, 3i+2))."""
    import numpy as np
    n = _mesh_args(mesh, n)
    ctx = ctx or default_context(mesh.soup.device.index)
    size = ctypes.c_int64(0)
    ctx.check(_lib.mcg_mesh_ply(ctx.handle, _ptr(mesh.soup), _ptr(mesh.normals), n, None, 0, ctypes.byref(size),
                                _stream(stream)), "mcg_mesh_ply")
    out = np.empty(size.value, np.uint8)
    ctx.check(_lib.mcg_mesh_ply(ctx.handle, _ptr(mesh.soup), _ptr(mesh.normals), n,
                                out.ctypes.data_as(ctypes.c_void_p), out.size, ctypes.byref(size), _stream(stream)),
              "mcg_mesh_ply")
    return out.tobytes()


def mesh_obj(mesh: Mesh, n=None, ctx=None, stream=None):
    """(OBJ text, qi_volume text) of the soup with the reference's vertex
    merge by "%.4f" keys, as bytes."""
    import numpy as np
    n = _mesh_args(mesh, n)
    ctx = ctx or default_context(mesh.soup.device.index)
    os_, qs = ctypes.c_int64(0), ctypes.c_int64(0)
    ctx.check(_lib.mcg_mesh_obj(ctx.handle, _ptr(mesh.soup), _ptr(mesh.normals), n, None, 0, ctypes.byref(os_),
                                None, 0, ctypes.byref(qs), _stream(stream)), "mcg_mesh_obj")
    obj = np.empty(max(os_.value, 1), np.uint8)
    qi = np.empty(max(qs.value, 1), np.uint8)
    ctx.check(_lib.mcg_mesh_obj(ctx.handle, _ptr(mesh.soup), _ptr(mesh.normals), n,
                                obj.ctypes.data_as(ctypes.c_void_p), obj.size, ctypes.byref(os_),
                                qi.ctypes.data_as(ctypes.c_void_p), qi.size, ctypes.byref(qs), _stream(stream)),
              "mcg_mesh_obj")
    return obj[:os_.value].tobytes(), qi[:qs.value].tobytes()


def mesh_write(mesh: Mesh, path, qi_path=None, n=None, ctx=None, stream=None):
    """Write the soup as path (".ply" or ".obj"), and qi_path for OBJ."""
    n = _mesh_args(mesh, n)
    ctx = ctx or default_context(mesh.soup.device.index)
    ctx.check(_lib.mcg_mesh_write(ctx.handle, _ptr(mesh.soup), _ptr(mesh.normals), n, os.fsencode(path),
                                  os.fsencode(qi_path) if qi_path else None, _stream(stream)), "mcg_mesh_write")


# ---------------------------------------------------------------------------
# depth pyramid and ICP (kf.cu:66-80, 226-261, 988-1301)
# ---------------------------------------------------------------------------
import math as _math

ICP_DT = 0.10                                   # kf.cu:1966 (100 mm)
ICP_NT = float(_math.cos(_math.radians(20.0)))  # kf.cu:1967
ICP_RT = _math.radians(20.0)                    # kf.cu:1968
ICP_TT = 0.10                                   # kf.cu:1969
ICP_IT_MAX = (15, 11, 8)                        # kf.cu:1970, per level (0 = full size)
PYRAMID_SIGMA = 0.06                            # kf.cu:2117


def icp_params(it_max, bilinear=False, dt=ICP_DT, nt=ICP_NT, rt=ICP_RT, tt=ICP_TT):
    p = _capi.IcpParams()
    p.nt, p.dt, p.rt, p.tt = float(nt), float(dt), float(rt), float(tt)
    p.it_max = int(it_max)
    p.bilinear = 1 if bilinear else 0
    return p


def intrinsic_pyramid_down(k):
    """float_camera_intrinsic_pyramid_down (cu_geometry_functions.h:218-225): fc / 2, cc / 2."""
    return intrinsic(k.fx / 2.0, k.fy / 2.0, k.cx / 2.0, k.cy / 2.0)


def float_data_to_mask(data, mask=None, ctx=None, stream=None):
    """d_float_data_to_mask: 0xff where data != 0 (uint8 tensor)."""
    mask = torch.empty(data.shape, dtype=torch.uint8, device=data.device) if mask is None else mask
    ctx = ctx or default_context(data.device.index)
    ctx.check(_lib.mcg_depth_mask(ctx.handle, data.numel(), _ptr(data), _ptr(mask), 1, _stream(stream)),
              "mcg_depth_mask")
    return mask


def float_mask_to_data(mask, data, ctx=None, stream=None):
    """d_float_mask_to_data: data = 0 where mask == 0 (in place)."""
    ctx = ctx or default_context(data.device.index)
    ctx.check(_lib.mcg_depth_mask(ctx.handle, data.numel(), _ptr(data), _ptr(mask), 0, _stream(stream)),
              "mcg_depth_mask")
    return data


def pyramid_down(src, mask, dst_shape=None, sigma=PYRAMID_SIGMA, ctx=None, stream=None):
    """d_pyramid_down (kf.cu:226-261): (dst, dst_mask) of half size (or
    dst_shape = (h, w)); dst is zero where dst_mask is 0."""
    sh, sw = src.shape
    dh, dw = dst_shape if dst_shape is not None else (sh >> 1, sw >> 1)
    dst = torch.zeros((dh, dw), dtype=torch.float32, device=src.device)
    dmask = torch.empty((dh, dw), dtype=torch.uint8, device=src.device)
    ctx = ctx or default_context(src.device.index)
    ctx.check(_lib.mcg_pyramid_down(ctx.handle, sw, sh, dw, dh, _ptr(src), _ptr(mask), _ptr(dst), _ptr(dmask),
                                    float(sigma), _stream(stream)), "mcg_pyramid_down")
    return dst, dmask


def _maps(v1, n1, v2, n2):
    for m in (v1, n1, v2, n2):
        if m.dtype != torch.float32 or m.dim() != 3 or m.shape[2] != 3 or not m.is_contiguous():
            raise ValueError("vertex / normal maps are contiguous (h, w, 3) float32 tensors")
    if v1.shape != n1.shape or v2.shape != n2.shape:
        raise ValueError("vertex and normal maps of a frame have one shape")
    return v1.shape[1], v1.shape[0], v2.shape[1], v2.shape[0]


def icp_correspond(params, k2, pose, v1, n1, v2, n2, ctx=None, stream=None):
    """One correspondence pass at `pose` (steps 1/4, 2, 3): dict of v21
    (h1, w1, 3), A (6, h1*w1), b (h1*w1,), inlier (h1, w1) uint8."""
    w1, h1, w2, h2 = _maps(v1, n1, v2, n2)
    dev = v1.device
    out = {"v21": torch.empty((h1, w1, 3), dtype=torch.float32, device=dev),
           "A": torch.empty((6, h1 * w1), dtype=torch.float32, device=dev),
           "b": torch.empty(h1 * w1, dtype=torch.float32, device=dev),
           "inlier": torch.empty((h1, w1), dtype=torch.uint8, device=dev)}
    ctx = ctx or default_context(dev.index)
    ctx.check(_lib.mcg_icp_correspond(ctx.handle, ctypes.byref(params), ctypes.byref(k2), ctypes.byref(pose), w1, h1,
                                      w2, h2, _ptr(v1), _ptr(n1), _ptr(v2), _ptr(n2), _ptr(out["v21"]),
                                      _ptr(out["A"]), _ptr(out["b"]), _ptr(out["inlier"]), _stream(stream)),
              "mcg_icp_correspond")
    return out


def icp(params, k2, pose, v1, n1, v2, n2, inlier=None, ctx=None, stream=None):
    """_cu_icp_projective_3d: align map 2 (v2, n2) to map 1 starting from
    `pose` (an Extrinsic mapping map-2 points into map 1's frame).  Returns
    (ok, pose, iterations); the returned pose and `inlier` are updated only
    when ok."""
    w1, h1, w2, h2 = _maps(v1, n1, v2, n2)
    out = _capi.Extrinsic()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(pose), ctypes.sizeof(out))
    ok, iters = ctypes.c_int32(0), ctypes.c_int32(0)
    ctx = ctx or default_context(v1.device.index)
    ctx.check(_lib.mcg_icp(ctx.handle, ctypes.byref(params), ctypes.byref(k2), ctypes.byref(out), w1, h1, w2, h2,
                           _ptr(v1), _ptr(n1), _ptr(v2), _ptr(n2), _ptr(inlier), ctypes.byref(ok), ctypes.byref(iters),
                           _stream(stream)), "mcg_icp")
    return bool(ok.value), out, int(iters.value)


def icp_pyramid(k0, pose, maps1, maps2, it_max=ICP_IT_MAX, bilinear=False, inlier=None, ctx=None, stream=None):
    """The fusion loop's tracking (kf.cu:2213-2218): ICP from the coarsest
    level to the finest, each level starting from the pose of the one
    before; stops at the first level that fails.  maps1 / maps2: lists of
    (vertex, normal) per level, level 0 the full size; k0 the level-0
    intrinsic (halved per level); the inlier map is that of level 0."""
    ks = [k0]
    for _ in range(1, len(maps1)):
        ks.append(intrinsic_pyramid_down(ks[-1]))
    ok, iters = True, []
    for lv in range(len(maps1) - 1, -1, -1):
        p = icp_params(it_max[lv], bilinear)
        ok, pose, it = icp(p, ks[lv], pose, maps1[lv][0], maps1[lv][1], maps2[lv][0], maps2[lv][1],
                           inlier=inlier if lv == 0 else None, ctx=ctx, stream=stream)
        iters.append(it)
        if not ok:
            break
    return ok, pose, iters[::-1]
