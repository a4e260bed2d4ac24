"""Python bindings of the CPU oracle (oracle.c).  TEST INFRASTRUCTURE ONLY.

Used by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
leg as the checker.  Parity status: unpinned by reference tests (the
reference has none); see oracle.h.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

VOXEL_SHORT2 = 0
VOXEL_FLOAT2 = 1


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


class Intrinsic(ctypes.Structure):
    _fields_ = [("fx", ctypes.c_float), ("fy", ctypes.c_float), ("cx", ctypes.c_float),
                ("cy", ctypes.c_float), ("dc", ctypes.c_float * 5)]


class Extrinsic(ctypes.Structure):
    _fields_ = [("r", ctypes.c_float * 9), ("t", ctypes.c_float * 3)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, i64, f32, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_double
        sig = {
            "orc_mc_classify": (None, [vp, i32, i32, i32, i32, vp, vp]),
            "orc_mc_count": (None, [vp, i32, i32, i32, i32, vp, vp, i32]),
            "orc_mc_extract": (i64, [vp, i32, i32, i32, i32, f32, vp, vp, vp, vp, vp, i64, i32]),
            "orc_mc_extract_f64": (i64, [vp, i32, i32, i32, i32, f64, vp, vp, i64]),
            "orc_surface_normal": (None, [vp, i32, i32, i32, i32, f32, vp, vp]),
            "orc_voxel_init": (None, [vp, i64]),
            "orc_depth_to_meter": (None, [vp, i64, f32, f32, vp]),
            "orc_meter_to_vertex": (None, [vp, i32, i32, vp, vp]),
            "orc_vertex_to_normal": (None, [i32, i32, vp, vp]),
            "orc_depth_scale": (None, [vp, i32, i32, vp, vp]),
            "orc_integrate": (None, [vp, i32, i32, i32, i32, f32, f32, f32, vp, vp, i32, i32, vp, vp, i32, i32]),
            "orc_rle_encode_slice": (i64, [vp, i64, i32, vp]),
            "orc_rle_decode_slice": (i64, [vp, i64, vp, i64]),
            "orc_rle_encode_volume": (i64, [vp, i32, i32, i32, f32, f32, f32, i32, vp, i64]),
            "orc_rle_decode_volume": (i32, [vp, i64, vp, i64, vp, vp]),
            "orc_max_threads": (i32, []),
            "orc_mc_edges": (i64, [vp, i32, i32, i32, i32, vp, vp, i64]),
            "orc_raycast": (i32, [vp, i32, i32, i32, f32, vp, vp, i32, i32, vp, vp, i32]),
            "orc_mc_edge_vertices": (None, [vp, i32, i32, i32, i32, f32, vp, i64, vp, vp, vp]),
            "orc_mc_backward_f64": (i64, [vp, i32, i32, i32, i32, f64, vp, i64, vp]),
            "orc_integrate_seq_f64": (None, [vp, i32, i32, i32, f32, f32, f32, vp, i32, vp, i32, i32, vp, vp, i32,
                                             vp, vp, vp, i32]),
            "orc_integrate_seq_backward_f64": (None, [vp, i32, i32, i32, f32, f32, f32, vp, i32, vp, i32, i32, vp, vp,
                                                      i32, vp, vp, vp, vp, vp, i32]),
            "orc_text_load": (i32, [ctypes.c_char_p, i64, i32, i32, i32, i32, vp, vp]),
            "orc_text_load_file": (i32, [ctypes.c_char_p, i64, i32, i32, i32, i32, vp, vp]),
            "orc_mesh_ply": (i64, [vp, vp, i64, vp, i64]),
            "orc_float_data_to_mask": (None, [i64, vp, vp]),
            "orc_float_mask_to_data": (None, [i64, vp, vp]),
            "orc_pyramid_down": (None, [i32, i32, i32, i32, vp, vp, vp, vp, f32]),
            "orc_icp_correspond": (None, [i32, f32, f32, vp, vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp,
                                          vp]),
            "orc_icp_normal_equations": (None, [i64, vp, vp, vp, vp]),
            "orc_icp_solve": (i32, [vp, vp, vp, vp]),
            "orc_so3_exp": (None, [vp, vp]),
            "orc_icp": (i32, [i32, f32, f32, f32, f32, i32, vp, vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp,
                              vp, vp]),
            "orc_mesh_obj": (None, [vp, vp, i64, vp, i64, vp, i64, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _vol(vol):
    vol = np.ascontiguousarray(vol)
    if vol.ndim != 4 or vol.shape[3] != 2:
        raise ValueError("volume must be (nz, ny, nx, 2)")
    if vol.dtype == np.int16:
        vt = VOXEL_SHORT2
    elif vol.dtype == np.float32:
        vt = VOXEL_FLOAT2
    else:
        raise TypeError(vol.dtype)
    nz, ny, nx, _ = vol.shape
    return vol, vt, nx, ny, nz


def max_threads():
    return lib().orc_max_threads()


def mc_classify(vol):
    vol, vt, nx, ny, nz = _vol(vol)
    shape = (max(nz - 1, 0), max(ny - 1, 0), max(nx - 1, 0))
    ci = np.zeros(shape, np.uint8)
    nv = np.zeros(shape, np.uint8)
    lib().orc_mc_classify(_p(vol), vt, nx, ny, nz, _p(ci), _p(nv))
    return ci, nv


def mc_count(vol, nthreads=0):
    vol, vt, nx, ny, nz = _vol(vol)
    o = np.zeros(1, np.int64)
    t = np.zeros(1, np.int64)
    lib().orc_mc_count(_p(vol), vt, nx, ny, nz, _p(o), _p(t), nthreads)
    return int(o[0]), int(t[0])


VERTEX_DTYPE = np.dtype([("pos", "<f4", (3,)), ("vox", "<i4", (3,)), ("tsdf", "<i2"), ("w", "<i2")])
assert VERTEX_DTYPE.itemsize == 28


def mc_extract(vol, cell, normals=True, vi2vox=True, ver_voxel=True, tri_cube=True, nthreads=0):
    """FP32 mirror; canonical order (cube linear id, table slot)."""
    vol, vt, nx, ny, nz = _vol(vol)
    _, ntri = mc_count(vol, nthreads)
    n = 3 * ntri
    soup = np.zeros(n, VERTEX_DTYPE)
    nrm = np.zeros((n, 3), np.float32) if normals else None
    v2v = np.zeros((n, 3), np.int32) if vi2vox else None
    vv = np.zeros(nx * ny * nz, np.int16) if ver_voxel else None
    tc = np.zeros(ntri, np.int64) if tri_cube else None
    total = lib().orc_mc_extract(_p(vol), vt, nx, ny, nz, float(cell), _p(soup), _p(nrm), _p(v2v), _p(vv),
                                 _p(tc), n, nthreads)
    assert total == n
    return {"soup": soup, "normals": nrm, "vi2vox": v2v, "ver_voxel": vv, "tri_cube": tc}


def mc_extract_f64(vol, cell):
    vol, vt, nx, ny, nz = _vol(vol)
    _, ntri = mc_count(vol)
    n = 3 * ntri
    pos = np.zeros((n, 3), np.float64)
    nrm = np.zeros((n, 3), np.float64)
    lib().orc_mc_extract_f64(_p(vol), vt, nx, ny, nz, float(cell), _p(pos), _p(nrm), n)
    return pos, nrm


def surface_normal(vol, cell, p):
    vol, vt, nx, ny, nz = _vol(vol)
    p = np.asarray(p, np.float32)
    n = np.zeros(3, np.float32)
    lib().orc_surface_normal(_p(vol), vt, nx, ny, nz, float(cell), _p(p), _p(n))
    return n


def voxel_init(n_voxels):
    v = np.zeros((n_voxels, 2), np.int16)
    lib().orc_voxel_init(_p(v), n_voxels)
    return v


def intrinsic(fx, fy, cx, cy):
    k = Intrinsic()
    k.fx, k.fy, k.cx, k.cy = fx, fy, cx, cy
    return k


def extrinsic(R, t):
    R = np.asarray(R, np.float32).reshape(3, 3)
    e = Extrinsic()
    cols = R.T.reshape(-1)
    for i in range(9):
        e.r[i] = float(cols[i])
    t = np.asarray(t, np.float32).reshape(3)
    for i in range(3):
        e.t[i] = float(t[i])
    return e


def depth_to_meter(depth_mm, dmin=0.0, dmax=2.0):
    d = np.ascontiguousarray(depth_mm, np.uint16)
    m = np.zeros(d.shape, np.float32)
    lib().orc_depth_to_meter(_p(d), d.size, dmin, dmax, _p(m))
    return m


def meter_to_vertex(k, meter):
    meter = np.ascontiguousarray(meter, np.float32)
    h, w = meter.shape
    v = np.zeros((h, w, 3), np.float32)
    lib().orc_meter_to_vertex(ctypes.byref(k), w, h, _p(meter), _p(v))
    return v


def vertex_to_normal(vertex):
    vertex = np.ascontiguousarray(vertex, np.float32)
    h, w, _ = vertex.shape
    n = np.zeros_like(vertex)
    lib().orc_vertex_to_normal(w, h, _p(vertex), _p(n))
    return n


def depth_scale(k, depth):
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    out = np.zeros_like(depth)
    lib().orc_depth_scale(ctypes.byref(k), w, h, _p(depth), _p(out))
    return out


def integrate(vol, min_t, max_t, grid_s, k, e, depth_m, normals=None, is_dynamic=False, nthreads=0):
    """In place on a contiguous numpy volume."""
    if not vol.flags.c_contiguous:
        raise ValueError("volume must be contiguous")
    _, vt, nx, ny, nz = _vol(vol)
    depth_m = np.ascontiguousarray(depth_m, np.float32)
    h, w = depth_m.shape
    if normals is not None:
        normals = np.ascontiguousarray(normals, np.float32)
    lib().orc_integrate(_p(vol), vt, nx, ny, nz, min_t, max_t, grid_s, ctypes.byref(k), ctypes.byref(e), w, h,
                        _p(depth_m), _p(normals), 1 if is_dynamic else 0, nthreads)


def rle_encode_slice(vox, lossless=False):
    vox = np.ascontiguousarray(vox, np.int16).reshape(-1, 2)
    buf = np.zeros(6 * len(vox) + 16, np.uint8)
    n = lib().orc_rle_encode_slice(_p(vox), len(vox), 1 if lossless else 0, _p(buf))
    return buf[:n].tobytes()


def rle_decode_slice(data: bytes, n_voxels):
    buf = np.frombuffer(data, np.uint8).copy()
    out = np.zeros((n_voxels, 2), np.int16)
    r = lib().orc_rle_decode_slice(_p(buf), len(buf), _p(out), n_voxels)
    if r < 0:
        raise ValueError("malformed RLE slice")
    return out


def rle_encode_volume(vol, min_t, max_t, grid_s, lossless=False):
    vol, vt, nx, ny, nz = _vol(vol)
    assert vt == VOXEL_SHORT2
    cap = 40 + nz * (4 + 6 * nx * ny)
    buf = np.zeros(cap, np.uint8)
    n = lib().orc_rle_encode_volume(_p(vol), nx, ny, nz, min_t, max_t, grid_s, 1 if lossless else 0, _p(buf), cap)
    if n < 0:
        raise RuntimeError("encode failed")
    return buf[:n].tobytes()


def rle_decode_volume(img: bytes):
    buf = np.frombuffer(img, np.uint8).copy()
    dims = np.zeros(3, np.int32)
    params = np.zeros(3, np.float32)
    r = lib().orc_rle_decode_volume(_p(buf), len(buf), None, 0, _p(dims), _p(params))
    if r != 0:
        raise ValueError("bad header (%d)" % r)
    nx, ny, nz = (int(d) for d in dims)
    vol = np.zeros((nz, ny, nx, 2), np.int16)
    r = lib().orc_rle_decode_volume(_p(buf), len(buf), _p(vol), vol.size // 2, _p(dims), _p(params))
    if r != 0:
        raise ValueError("malformed RLE volume (%d)" % r)
    return vol, tuple(float(p) for p in params)


# ---------------------------------------------------------------------------
# adjoints (binary64; discrete choices from the FP32 mirror, held fixed)
# ---------------------------------------------------------------------------
def mc_edges(vol):
    """(va, vb): linear voxel indices of each soup vertex's edge corners,
    canonical order."""
    vol, vt, nx, ny, nz = _vol(vol)
    _, ntri = mc_count(vol)
    n = 3 * ntri
    va = np.zeros(n, np.int64)
    vb = np.zeros(n, np.int64)
    lib().orc_mc_edges(_p(vol), vt, nx, ny, nz, _p(va), _p(vb), n)
    return va, vb


def mc_positions_f64(F, va, vb, shape, cell):
    """Soup positions from per-voxel values F (any float array of nz*ny*nx)
    on a fixed topology (va, vb)."""
    nz, ny, nx = shape
    F = np.asarray(F, np.float64).reshape(-1)

    def xyz(li):
        return np.stack([li % nx, (li // nx) % ny, li // (nx * ny)], axis=1).astype(np.float64)

    pa = (xyz(va) + 0.5) * cell
    pb = (xyz(vb) + 0.5) * cell
    fa, fb = F[va], F[vb]
    t = -fa / (fb - fa + 1e-15)
    return pa + t[:, None] * (pb - pa)


def mc_backward_f64(vol, cell, grad_pos):
    """dL/df per voxel (nz, ny, nx) for dL/dP in canonical order."""
    vol, vt, nx, ny, nz = _vol(vol)
    g = np.ascontiguousarray(grad_pos, np.float64).reshape(-1, 3)
    out = np.zeros((nz, ny, nx), np.float64)
    lib().orc_mc_backward_f64(_p(vol), vt, nx, ny, nz, float(cell), _p(g), len(g), _p(out))
    return out


def _poses(poses):
    arr = (Extrinsic * len(poses))()
    for i, e in enumerate(poses):
        arr[i] = e
    return arr


def integrate_seq_f64(shape, min_t, max_t, grid_s, k, poses, depth, vol0=None, normals=None, is_dynamic=False,
                      nthreads=0):
    """n_frames integrate steps in binary64 on a float2 volume of shape
    (nz, ny, nx).  Returns (F, W, signature)."""
    nz, ny, nx = shape
    depth = np.ascontiguousarray(depth, np.float64)
    nf, h, w = depth.shape
    if vol0 is not None:
        vol0 = np.ascontiguousarray(vol0, np.float32)
    if normals is not None:
        normals = np.ascontiguousarray(normals, np.float32)
    F = np.zeros(shape, np.float64)
    W = np.zeros(shape, np.float64)
    sig = np.zeros(1, np.uint64)
    lib().orc_integrate_seq_f64(_p(vol0), nx, ny, nz, min_t, max_t, grid_s, ctypes.byref(k), nf, _poses(poses),
                                w, h, _p(depth), _p(normals), 1 if is_dynamic else 0, _p(F), _p(W), _p(sig),
                                nthreads)
    return F, W, int(sig[0])


def integrate_seq_backward_f64(shape, min_t, max_t, grid_s, k, poses, depth, grad_f, grad_w=None, vol0=None,
                               normals=None, is_dynamic=False, nthreads=0):
    """Adjoint of integrate_seq_f64: (dL/ddepth, dL/dF0, dL/dW0)."""
    nz, ny, nx = shape
    depth = np.ascontiguousarray(depth, np.float64)
    nf, h, w = depth.shape
    if vol0 is not None:
        vol0 = np.ascontiguousarray(vol0, np.float32)
    if normals is not None:
        normals = np.ascontiguousarray(normals, np.float32)
    gf = np.ascontiguousarray(grad_f, np.float64)
    gw = None if grad_w is None else np.ascontiguousarray(grad_w, np.float64)
    gd = np.zeros_like(depth)
    gF0 = np.zeros(shape, np.float64)
    gW0 = np.zeros(shape, np.float64)
    lib().orc_integrate_seq_backward_f64(_p(vol0), nx, ny, nz, min_t, max_t, grid_s, ctypes.byref(k), nf,
                                         _poses(poses), w, h, _p(depth), _p(normals), 1 if is_dynamic else 0,
                                         _p(gf), _p(gw), _p(gd), _p(gF0), _p(gW0), nthreads)
    return gd, gF0, gW0


# ---------------------------------------------------------------------------
# indexed mesh
# ---------------------------------------------------------------------------
def edge_keys(va, vb, nx, ny):
    """Soup vertex edges (va, vb) -> 3 * linear index of the lower voxel + axis."""
    lo = np.minimum(va, vb)
    d = np.abs(vb - va)
    axis = np.where(d == 1, 0, np.where(d == nx, 1, 2))
    return 3 * lo + axis


def mc_indexed(vol):
    """Indexed topology of the soup: (keys of the unique vertices sorted,
    triangles (T, 3) as edge keys in canonical soup order)."""
    v, vt, nx, ny, nz = _vol(vol)
    va, vb = mc_edges(v)
    k = edge_keys(va, vb, nx, ny)
    return np.unique(k), k.reshape(-1, 3)


def mc_edge_vertices(vol, cell, keys):
    vol, vt, nx, ny, nz = _vol(vol)
    keys = np.ascontiguousarray(keys, np.int64)
    n = len(keys)
    pos = np.zeros((n, 3), np.float32)
    nrm = np.zeros((n, 3), np.float32)
    v2v = np.zeros((n, 3), np.int32)
    lib().orc_mc_edge_vertices(_p(vol), vt, nx, ny, nz, float(cell), _p(keys), n, _p(pos), _p(nrm), _p(v2v))
    return pos, nrm, v2v


# ---------------------------------------------------------------------------
# ray casting (kf.cu:551-659, 786-986)
# ---------------------------------------------------------------------------
def raycast(vol, grid_s, k, e, w, h, normals=True, nthreads=0):
    """(depth (h, w) metres, normal (h, w, 3) or None) of a short2 volume seen
    by camera (k, e); None if the camera matrix is singular."""
    vol = np.ascontiguousarray(vol)
    if vol.dtype != np.int16:
        raise TypeError("ray casting reads short2 volumes")
    nz, ny, nx, _ = vol.shape
    depth = np.zeros((h, w), np.float32)
    nrm = np.zeros((h, w, 3), np.float32) if normals else None
    ok = lib().orc_raycast(_p(vol), nx, ny, nz, float(grid_s), ctypes.byref(k), ctypes.byref(e), w, h, _p(depth),
                           _p(nrm), nthreads)
    return (depth, nrm) if ok else None


# ---------------------------------------------------------------------------
# text-record volume loader (kf.cu:3289-3361), libstdc++ extraction rules
# ---------------------------------------------------------------------------
REFERENCE_TAIL_BYTES = 11_000_000_000  # kf.cu:3316 seekg(-11000000000, end)


def text_load(text, dim, origin=(512, 512, 0)):
    """Load records from a text in memory: (volume (dim, dim, dim, 2) int16,
    {"stored", "iterations", "status"}); status 1 = the reference's loop
    would not end (a failed extraction outside the window)."""
    text = bytes(text)
    vol = np.empty((dim, dim, dim, 2), np.int16)
    st = np.zeros(3, np.int64)
    lib().orc_text_load(text, len(text), int(dim), int(origin[0]), int(origin[1]), int(origin[2]), _p(vol), _p(st))
    return vol, {"stored": int(st[0]), "iterations": int(st[1]), "status": int(st[2])}


def text_load_file(path, dim, origin=(512, 512, 0), tail_bytes=REFERENCE_TAIL_BYTES):
    """Load records from the last tail_bytes of a file (seek, skip the cut
    line, then the loop of text_load)."""
    vol = np.empty((dim, dim, dim, 2), np.int16)
    st = np.zeros(3, np.int64)
    r = lib().orc_text_load_file(os.fsencode(path), int(tail_bytes), int(dim), int(origin[0]), int(origin[1]),
                                 int(origin[2]), _p(vol), _p(st))
    if r != 0:
        raise OSError("cannot open %s" % path)
    return vol, {"stored": int(st[0]), "iterations": int(st[1]), "status": int(st[2])}


# ---------------------------------------------------------------------------
# mesh writers (kf.cu:3394-3424 PLY, 3625-3726 OBJ), glibc formatting
# ---------------------------------------------------------------------------
def mesh_ply(soup, normals):
    """Binary PLY image (bytes) of a soup: soup (n, 28) uint8 vertex_voxel
    records, normals (n, 3) float32."""
    soup = np.ascontiguousarray(soup, np.uint8).reshape(-1, 28)
    normals = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    n = len(soup)
    size = lib().orc_mesh_ply(_p(soup), _p(normals), n, None, 0)
    out = np.empty(size, np.uint8)
    lib().orc_mesh_ply(_p(soup), _p(normals), n, _p(out), size)
    return out.tobytes()


def mesh_obj(soup, normals):
    """(OBJ image, qi_volume image) of a soup, as bytes."""
    soup = np.ascontiguousarray(soup, np.uint8).reshape(-1, 28)
    normals = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    n = len(soup)
    sizes = np.zeros(2, np.int64)
    lib().orc_mesh_obj(_p(soup), _p(normals), n, None, 0, None, 0, _p(sizes))
    obj = np.empty(sizes[0], np.uint8)
    qi = np.empty(sizes[1], np.uint8)
    lib().orc_mesh_obj(_p(soup), _p(normals), n, _p(obj), int(sizes[0]), _p(qi), int(sizes[1]), _p(sizes))
    return obj.tobytes(), qi.tobytes()


# ---------------------------------------------------------------------------
# depth pyramid and ICP (kf.cu:66-80, 226-261, 988-1301)
# ---------------------------------------------------------------------------
def float_data_to_mask(data):
    data = np.ascontiguousarray(data, np.float32)
    mask = np.empty(data.shape, np.uint8)
    lib().orc_float_data_to_mask(data.size, _p(data), _p(mask))
    return mask


def float_mask_to_data(mask, data):
    data = np.array(data, np.float32, copy=True)
    mask = np.ascontiguousarray(mask, np.uint8)
    lib().orc_float_mask_to_data(data.size, _p(mask), _p(data))
    return data


def pyramid_down(src, mask, dst_shape, sigma=0.06):
    """(dst, dst_mask) of kf.cu:226-261; src / mask (h, w); dst left 0
    where the mask is 0 (the reference leaves it unwritten)."""
    src = np.ascontiguousarray(src, np.float32)
    mask = np.ascontiguousarray(mask, np.uint8)
    sh, sw = src.shape
    dh, dw = dst_shape
    dst = np.zeros((dh, dw), np.float32)
    dmask = np.zeros((dh, dw), np.uint8)
    lib().orc_pyramid_down(sw, sh, dw, dh, _p(src), _p(mask), _p(dst), _p(dmask), float(sigma))
    return dst, dmask


def _k4(k):
    return np.array([k.fx, k.fy, k.cx, k.cy], np.float32)


def _pose(e):
    return np.array(list(e.r), np.float32), np.array(list(e.t), np.float32)


def icp_correspond(nt, dt, k, e, v1, n1, v2, n2, bilinear=False):
    """One correspondence pass: (v21 (h1, w1, 3), A (6, n), b (n), inlier (h1, w1))."""
    v1, n1, v2, n2 = (np.ascontiguousarray(a, np.float32) for a in (v1, n1, v2, n2))
    h1, w1 = v1.shape[:2]
    h2, w2 = v2.shape[:2]
    r, t = _pose(e)
    v21 = np.zeros((h1, w1, 3), np.float32)
    A = np.zeros((6, h1 * w1), np.float32)
    b = np.zeros(h1 * w1, np.float32)
    inl = np.zeros((h1, w1), np.uint8)
    lib().orc_icp_correspond(1 if bilinear else 0, float(nt), float(dt), _p(_k4(k)), _p(r), _p(t), w1, h1, w2, h2,
                             _p(v1), _p(n1), _p(v2), _p(n2), _p(v21), _p(A), _p(b), _p(inl))
    return v21, A, b, inl


def icp(nt, dt, rt, tt, it_max, k, e, v1, n1, v2, n2, bilinear=False):
    """_cu_icp_projective_3d: (ok, (r, t) updated pose, iterations, inlier map)."""
    v1, n1, v2, n2 = (np.ascontiguousarray(a, np.float32) for a in (v1, n1, v2, n2))
    h1, w1 = v1.shape[:2]
    h2, w2 = v2.shape[:2]
    r, t = _pose(e)
    n = h1 * w1
    v21 = np.zeros(3 * n, np.float32)
    A = np.zeros(6 * n, np.float32)
    b = np.zeros(n, np.float32)
    inl = np.zeros((h1, w1), np.uint8)
    iters = np.zeros(1, np.int32)
    ok = lib().orc_icp(1 if bilinear else 0, float(nt), float(dt), float(rt), float(tt), int(it_max), _p(_k4(k)),
                       _p(r), _p(t), w1, h1, w2, h2, _p(v1), _p(n1), _p(v2), _p(n2), _p(inl), _p(v21), _p(A), _p(b),
                       _p(iters))
    return bool(ok), (r, t), int(iters[0]), inl
