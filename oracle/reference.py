"""Python bindings of the reference's own source compiled for the host
(oracle/ref/build_ref.py -> oracle/_ref/libref_*.so).  TEST INFRASTRUCTURE
ONLY: the checker of the oracle.  Available only where the reference tree is
(REFERENCE_ROOT, default /root/reference); `available()` is False elsewhere
and the tests that use it skip.
"""
import ctypes
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
_libs = {}
_built = None


def _recipe():
    spec = importlib.util.spec_from_file_location("_mcg_build_ref", os.path.join(HERE, "ref", "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def build():
    """Builds the libraries once per process; None when the reference tree is absent."""
    global _built
    if _built is None:
        _built = _recipe().build() or []
    return _built


def available():
    return bool(build())


def lib(unit, fma=False):
    key = (unit, fma)
    if key not in _libs:
        if not available():
            raise RuntimeError("the reference tree is not available here")
        L = ctypes.CDLL(os.path.join(REF_DIR, "libref_%s%s.so" % (unit, "_fma" if fma else "")))
        vp, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float
        sig = {
            "ref_mc_cube_index": (None, [vp, i32, i32, i32, vp]),
            "ref_mc_count": (i64, [vp, i32, i32, i32, vp]),
            "ref_mc_extract": (i64, [vp, i32, i32, i32, f32, vp, vp, vp, vp, i64]),
            "ref_surface_normals": (None, [vp, i32, i32, i32, f32, vp, i64, vp]),
            "ref_depth_to_meter": (None, [vp, i64, vp]),
            "ref_meter_to_vertex": (None, [vp, i32, i32, vp, vp]),
            "ref_vertex_to_normal": (None, [i32, i32, vp, vp]),
            "ref_voxel_init": (None, [vp, i32, i32, i32]),
            "ref_integrate": (None, [vp, i32, i32, i32, f32, f32, f32, vp, vp, i32, i32, vp, vp, i32]),
            "ref_rle_encode_slice": (i64, [vp, i64, vp]),
            "ref_rle_decode_slice": (None, [vp, vp, i64]),
        }
        for name, (res, args) in sig.items():
            if hasattr(L, name):
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
        _libs[key] = L
    return _libs[key]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _vol(vol):
    vol = np.ascontiguousarray(vol)
    assert vol.dtype == np.int16 and vol.shape[-1] == 2
    nz, ny, nx = vol.shape[:3]
    return vol, nx, ny, nz


VERTEX_DTYPE = np.dtype([("pos", "<f4", (3,)), ("vox", "<i4", (3,)), ("tsdf", "<i2"), ("w", "<i2")])


def mc_cube_index(vol, fma=False):
    vol, nx, ny, nz = _vol(vol)
    ci = np.zeros((nz - 1, ny - 1, nx - 1), np.uint8)
    lib("live", fma).ref_mc_cube_index(_p(vol), nx, ny, nz, _p(ci))
    return ci


def mc_count(vol):
    vol, nx, ny, nz = _vol(vol)
    occ = ctypes.c_longlong(0)
    nv = lib("live").ref_mc_count(_p(vol), nx, ny, nz, ctypes.byref(occ))
    return occ.value, nv // 3


def mc_extract(vol, cell, fma=False):
    """MarchingCubes::run + the normals of its driver, triangles in linear
    cube order (the oracle's canonical order)."""
    vol, nx, ny, nz = _vol(vol)
    _, ntri = mc_count(vol)
    n = 3 * ntri
    soup = np.zeros(max(n, 1), VERTEX_DTYPE)
    v2v = np.zeros((max(n, 1), 3), np.int32)
    vv = np.zeros(nx * ny * nz, np.int16)
    nrm = np.zeros((max(n, 1), 3), np.float32)
    got = lib("live", fma).ref_mc_extract(_p(vol), nx, ny, nz, float(cell), _p(soup), _p(v2v), _p(vv), _p(nrm), n)
    assert got == n, (got, n)
    return {"soup": soup[:n], "vi2vox": v2v[:n], "ver_voxel": vv, "normals": nrm[:n]}


def surface_normals(vol, cell, verts, fma=False):
    vol, nx, ny, nz = _vol(vol)
    verts = np.ascontiguousarray(verts)
    out = np.zeros((len(verts), 3), np.float32)
    lib("live", fma).ref_surface_normals(_p(vol), nx, ny, nz, float(cell), _p(verts), len(verts), _p(out))
    return out


def depth_to_meter(depth_u16, fma=False):
    d = np.ascontiguousarray(depth_u16).view(np.int16)
    out = np.zeros(d.shape, np.float32)
    lib("dead", fma).ref_depth_to_meter(_p(d), d.size, _p(out))
    return out


def meter_to_vertex(k, meter, fma=False):
    meter = np.ascontiguousarray(meter, dtype=np.float32)
    h, w = meter.shape
    out = np.zeros((h, w, 3), np.float32)
    lib("dead", fma).ref_meter_to_vertex(ctypes.byref(k), w, h, _p(meter), _p(out))
    return out


def vertex_to_normal(vertex, fma=False):
    vertex = np.ascontiguousarray(vertex, dtype=np.float32)
    h, w = vertex.shape[:2]
    out = np.zeros((h, w, 3), np.float32)
    lib("dead", fma).ref_vertex_to_normal(w, h, _p(vertex), _p(out))
    return out


def voxel_init(shape):
    nz, ny, nx = shape
    vol = np.full((nz, ny, nx, 2), 7, np.int16)
    lib("dead").ref_voxel_init(_p(vol), nx, ny, nz)
    return vol


def integrate(vol, min_t, max_t, grid_s, k, e, meter, normals=None, is_dynamic=False, fma=False):
    """In place on vol (int16 (nz, ny, nx, 2)); k, e: oracle.Intrinsic /
    oracle.Extrinsic (the reference's camera structs, same layout)."""
    assert vol.flags.c_contiguous and vol.dtype == np.int16
    nz, ny, nx = vol.shape[:3]
    meter = np.ascontiguousarray(meter, dtype=np.float32)
    h, w = meter.shape
    nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32)
    lib("dead", fma).ref_integrate(_p(vol), nx, ny, nz, float(min_t), float(max_t), float(grid_s),
                                   ctypes.byref(k), ctypes.byref(e), w, h, _p(meter), _p(nrm),
                                   1 if is_dynamic else 0)


def rle_encode_slice(vox):
    vox = np.ascontiguousarray(vox, dtype=np.int16).reshape(-1, 2)
    buf = np.zeros(6 * len(vox) + 16, np.uint8)
    n = lib("dead").ref_rle_encode_slice(_p(vox), len(vox), _p(buf))
    return buf[:n].tobytes()


def rle_decode_slice(data, n_voxels):
    buf = np.frombuffer(data, np.uint8).copy()
    out = np.zeros((n_voxels, 2), np.int16)
    lib("dead").ref_rle_decode_slice(_p(buf), _p(out), n_voxels)
    return out
