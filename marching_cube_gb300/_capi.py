"""ctypes declarations of the C ABI in include/mcg.h.

The shared library is the product: if it is missing this module raises at
import time -- there is no Python or CPU fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmcg.so")

c_void_p = ctypes.c_void_p
c_int = ctypes.c_int
c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_float = ctypes.c_float


class Volume(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("nx", c_int32), ("ny", c_int32), ("nz", c_int32),
                ("voxel_type", c_int32), ("cell", c_float)]


class MeshOut(ctypes.Structure):
    _fields_ = [("soup", c_void_p), ("soup_normals", c_void_p), ("vi2vox", c_void_p),
                ("ver_voxel", c_void_p), ("tri_cube", c_void_p), ("capacity_vertices", c_int64)]


class IndexedOut(ctypes.Structure):
    _fields_ = [("positions", c_void_p), ("normals", c_void_p), ("vi2vox", c_void_p), ("vertex_edge", c_void_p),
                ("triangles", c_void_p), ("tri_cube", c_void_p), ("capacity_vertices", c_int64),
                ("capacity_triangles", c_int64)]


class MeshCounts(ctypes.Structure):
    _fields_ = [("occupied", c_int64), ("triangles", c_int64), ("vertices", c_int64),
                ("active_bricks", c_int64), ("status", c_int32), ("reserved", c_int32)]


class McConfig(ctypes.Structure):
    _fields_ = [("fused", c_int32), ("classify_shape", c_int32), ("gen_fixed_rounds", c_int32),
                ("reserved", c_int32)]


class TextInfo(ctypes.Structure):
    _fields_ = [("bytes", c_int64), ("numbers", c_int64), ("records", c_int64), ("stored", c_int64),
                ("fail_offset", c_int64), ("filled_rest", c_int32), ("reserved", c_int32)]


class IcpParams(ctypes.Structure):
    _fields_ = [("nt", c_float), ("dt", c_float), ("rt", c_float), ("tt", c_float), ("it_max", c_int32),
                ("bilinear", c_int32)]


class Intrinsic(ctypes.Structure):
    _fields_ = [("fx", c_float), ("fy", c_float), ("cx", c_float), ("cy", c_float),
                ("dc", c_float * 5)]


class Extrinsic(ctypes.Structure):
    _fields_ = [("r", c_float * 9), ("t", c_float * 3)]


# name -> (restype, argtypes)
SIGNATURES = {
    "mcg_status_string": (ctypes.c_char_p, [c_int]),
    "mcg_version": (c_int, []),
    "mcg_create": (c_int, [ctypes.POINTER(c_void_p), c_int]),
    "mcg_destroy": (c_int, [c_void_p]),
    "mcg_last_cuda_error": (c_int, [c_void_p]),
    "mcg_voxel_init": (c_int, [c_void_p, c_void_p, c_int32, c_int64, c_void_p]),
    "mcg_mc_classify": (c_int, [c_void_p, ctypes.POINTER(Volume), c_void_p]),
    "mcg_mc_counts": (c_int, [c_void_p, ctypes.POINTER(MeshCounts)]),
    "mcg_set_kernel_timing": (c_int, [c_void_p, c_int32]),
    "mcg_mc_count_kernel_ms": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "mcg_mc_generate": (c_int, [c_void_p, ctypes.POINTER(Volume), ctypes.POINTER(MeshOut), c_void_p]),
    "mcg_mc_classify_indexed": (c_int, [c_void_p, ctypes.POINTER(Volume), c_void_p]),
    "mcg_mc_generate_indexed": (c_int, [c_void_p, ctypes.POINTER(Volume), ctypes.POINTER(IndexedOut), c_void_p]),
    "mcg_mc_extract_indexed": (c_int, [c_void_p, ctypes.POINTER(Volume), ctypes.POINTER(IndexedOut), c_void_p]),
    "mcg_mc_classify_slab": (c_int, [c_void_p, ctypes.POINTER(Volume), c_int32, c_int32, c_void_p]),
    "mcg_mc_get_config": (c_int, [c_void_p, ctypes.POINTER(McConfig)]),
    "mcg_mc_set_config": (c_int, [c_void_p, ctypes.POINTER(McConfig)]),
    "mcg_mc_extract_slab": (c_int, [c_void_p, ctypes.POINTER(Volume), c_int32, c_int32, ctypes.POINTER(MeshOut),
                                    c_void_p]),
    "mcg_mc_extract": (c_int, [c_void_p, ctypes.POINTER(Volume), ctypes.POINTER(MeshOut), c_void_p]),
    "mcg_mc_classify_batched": (c_int, [c_void_p, ctypes.POINTER(Volume), c_int32, c_void_p]),
    "mcg_mc_counts_batched": (c_int, [c_void_p, ctypes.POINTER(MeshCounts), c_int32]),
    "mcg_mc_generate_batched": (c_int, [c_void_p, ctypes.POINTER(Volume), ctypes.POINTER(MeshOut), c_int32,
                                        c_void_p]),
    "mcg_mc_extract_batched": (c_int, [c_void_p, ctypes.POINTER(Volume), ctypes.POINTER(MeshOut), c_int32,
                                       c_void_p]),
    "mcg_mc_extract_noalloc": (c_int, [ctypes.POINTER(Volume), ctypes.POINTER(MeshOut),
                                       ctypes.POINTER(MeshCounts), c_void_p]),
    "mcg_mc_backward": (c_int, [c_void_p, ctypes.POINTER(Volume), c_void_p, c_int64, c_void_p, c_void_p]),
    "mcg_mc_normals": (c_int, [c_void_p, ctypes.POINTER(Volume), c_void_p, c_int64, c_void_p, c_void_p]),
    "mcg_depth_to_maps": (c_int, [c_void_p, ctypes.POINTER(Intrinsic), c_int32, c_int32, c_void_p,
                                  c_float, c_float, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mcg_meter_to_vertex": (c_int, [c_void_p, ctypes.POINTER(Intrinsic), c_int32, c_int32,
                                    c_void_p, c_void_p, c_void_p]),
    "mcg_vertex_to_normal": (c_int, [c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "mcg_integrate": (c_int, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_int32, c_float, c_float,
                              c_float, ctypes.POINTER(Intrinsic), ctypes.POINTER(Extrinsic), c_int32,
                              c_int32, c_void_p, c_void_p, c_int32, c_void_p]),
    "mcg_raycast": (c_int, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_float, ctypes.POINTER(Intrinsic),
                            ctypes.POINTER(Extrinsic), c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "mcg_integrate_backward": (c_int, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_float, c_float, c_float,
                                       ctypes.POINTER(Intrinsic), c_int32, c_void_p, c_int32, c_int32, c_void_p,
                                       c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                       c_void_p]),
    "mcg_integrate_device_pose": (c_int, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_int32, c_float, c_float,
                                          c_float, ctypes.POINTER(Intrinsic), c_void_p, c_int32, c_int32, c_void_p,
                                          c_void_p, c_int32, c_void_p]),
    "mcg_rle_bound": (c_int64, [c_int32, c_int32, c_int32]),
    "mcg_rle_encode": (c_int, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_float, c_float, c_float,
                               c_int32, c_void_p, c_int64, ctypes.POINTER(c_int64), c_void_p]),
    "mcg_rle_encode_host": (c_int, [c_void_p, c_int32, c_int32, c_int32, c_float, c_float, c_float, c_int32,
                                    c_void_p, c_int64, ctypes.POINTER(c_int64)]),
    "mcg_rle_decode_host": (c_int, [c_void_p, c_int64, c_void_p, c_int64]),
    "mcg_rle_header": (c_int, [c_void_p, c_int64, ctypes.POINTER(c_int32), ctypes.POINTER(c_float)]),
    "mcg_rle_decode": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_void_p]),
    "mcg_rle_decode_file": (c_int, [c_void_p, ctypes.c_char_p, c_void_p, c_int64, ctypes.POINTER(c_int32),
                                    ctypes.POINTER(c_float), c_void_p]),
    "mcg_mesh_ply": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_int64, ctypes.POINTER(c_int64),
                             c_void_p]),
    "mcg_mesh_obj": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_int64, ctypes.POINTER(c_int64),
                             c_void_p, c_int64, ctypes.POINTER(c_int64), c_void_p]),
    "mcg_mesh_write": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, ctypes.c_char_p, ctypes.c_char_p, c_void_p]),
    "mcg_pyramid_down": (c_int, [c_void_p, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_float, c_void_p]),
    "mcg_depth_mask": (c_int, [c_void_p, c_int64, c_void_p, c_void_p, c_int32, c_void_p]),
    "mcg_icp_correspond": (c_int, [c_void_p, ctypes.POINTER(IcpParams), ctypes.POINTER(Intrinsic),
                                   ctypes.POINTER(Extrinsic), c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mcg_icp": (c_int, [c_void_p, ctypes.POINTER(IcpParams), ctypes.POINTER(Intrinsic), ctypes.POINTER(Extrinsic),
                        c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                        ctypes.POINTER(c_int32), ctypes.POINTER(c_int32), c_void_p]),
    "mcg_text_records_parse": (c_int, [c_void_p, c_void_p, c_int64, c_int32, ctypes.POINTER(c_int32), c_void_p,
                                       ctypes.POINTER(TextInfo), c_void_p]),
    "mcg_text_records_load": (c_int, [c_void_p, c_void_p, c_int64, c_int32, ctypes.POINTER(c_int32), c_void_p,
                                      ctypes.POINTER(TextInfo), c_void_p]),
    "mcg_text_records_load_file": (c_int, [c_void_p, ctypes.c_char_p, c_int64, c_int32, ctypes.POINTER(c_int32),
                                           c_void_p, ctypes.POINTER(TextInfo), c_void_p]),
}


def load(path=LIB_PATH):
    if not os.path.exists(path):
        raise ImportError(
            "libmcg.so is not built (%s); run `python marching_cube_gb300/_build.py` "
            "(or __graft_entry__.build())" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
