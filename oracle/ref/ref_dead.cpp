// Harness around the reference's KinectFusion code that sits inside #if 0
// (cu_kinect_fusion_v1.cu:43-3137), compiled for the host by
// oracle/ref/build_ref.py.  TEST INFRASTRUCTURE ONLY: a second checker of
// the oracle, built from the reference's own source.
//
// Included from the reference (by line range, see build_ref.py):
//   cu_kinect_fusion_v1.h:30-46     depth range, DEVICE_OPENNI, CU_VOXEL_* constants
//   cu_kinect_fusion_v1.h:152-171   d_pack_tsdf / d_unpack_tsdf / d_pack_weight /
//                                   d_unpack_weight (the self-consistent pair)
//   structure.h:20-39               cu_voxel, vertex_voxel, cu_voxel_access_*
//   cu_kinect_fusion_v1.cu:95-151   d_kinect_depth_to_meter, d_img_meter_to_vertex,
//                                   d_img_vertex_to_normal
//   cu_kinect_fusion_v1.cu:364-379  d_voxel_initialize
//   cu_kinect_fusion_v1.cu:416-532  d_voxel_volumetric_depth_scaling,
//                                   d_voxel_volumetric_integration
//   cu_kinect_fusion_v1.cu:1362-1447 cu_voxel_rle, run-length encode / decode of a slice
// and, whole, cu_vector_functions.h and cu_geometry_functions.h.
//
// Stand-ins (the pieces the reference leaves undefined or dead):
//  * the voxel is the live 4-byte cu_voxel_t of structure.h:14-18; the dead
//    code also writes and reads a colour member, which here is a placeholder
//    with no storage (colour is not part of the live voxel, and the
//    integrate harness passes a black colour image, for which the colour
//    update is skipped, cu_kinect_fusion_v1.cu:505);
//  * the validity helpers come from a library the reference does not ship;
//    they are fixed as the oracle fixes them: invalid metre = 0, invalid
//    vertex = invalid normal = (0, 0, 0).
#include "cu_vector_functions.h"
#include "cu_geometry_functions.h"

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;

struct ref_color_sink {
    static inline unsigned char x = 0, y = 0, z = 0;
    ref_color_sink() = default;
    ref_color_sink(uchar3) {}
};

typedef struct _CU_VOXEL_T {
    short tsdf;
    ushort w;
    [[no_unique_address]] ref_color_sink color;
} cu_voxel_t;
static_assert(sizeof(cu_voxel_t) == 4, "the live 4-byte voxel");

#include "st_volume.inc"
#include "kfh_consts.inc"
#include "kfh_pack.inc"

inline bool is_meter_valid(float m) { return m != 0.0f; }
inline bool is_vertex_valid(const float3 &v) { return !(v.x == 0.0f && v.y == 0.0f && v.z == 0.0f); }
inline bool is_normal_valid(const float3 &n) { return !(n.x == 0.0f && n.y == 0.0f && n.z == 0.0f); }
inline void set_vertex_invalid(float3 &v) { v = make_float3(0.0f, 0.0f, 0.0f); }
inline void set_normal_invalid(float3 &n) { n = make_float3(0.0f, 0.0f, 0.0f); }

#include "kf_depth_maps.inc"
#include "kf_voxel_init.inc"
#include "kf_integrate.inc"
#include "kf_rle.inc"

#include <vector>

namespace {

// one 2-D launch of BX x BY blocks over an (nx, ny) grid of threads, run one
// thread at a time
template <class F>
void run_2d(int nx, int ny, F &&body) {
    const int BXS = CU_BLOCK_X, BYS = CU_BLOCK_Y;
    blockDim = dim3(BXS, BYS, 1);
    for (int by = 0; by < (ny + BYS - 1) / BYS; ++by)
        for (int bx = 0; bx < (nx + BXS - 1) / BXS; ++bx)
            for (int ty = 0; ty < BYS; ++ty)
                for (int tx = 0; tx < BXS; ++tx) {
                    blockIdx = make_uint3(bx, by, 0);
                    threadIdx = make_uint3(tx, ty, 0);
                    body();
                }
}

}  // namespace

extern "C" {

// d_kinect_depth_to_meter over n pixels; depth holds the uint16 millimetre
// bits, read as the reference's short
void ref_depth_to_meter(const short *depth, long long n, float *meter) {
    blockDim = dim3(256, 1, 1);
    for (long long i = 0; i < n; ++i) {
        blockIdx = make_uint3((unsigned)(i / 256), 0, 0);
        threadIdx = make_uint3((unsigned)(i % 256), 0, 0);
        d_kinect_depth_to_meter((int)n, nullptr, const_cast<short *>(depth), meter);
    }
}

void ref_meter_to_vertex(const float_camera_intrinsic *k, int w, int h, const float *meter, float3 *vertex) {
    run_2d(w, h, [&] { d_img_meter_to_vertex(*k, make_int2(w, h), const_cast<float *>(meter), vertex); });
}

void ref_vertex_to_normal(int w, int h, const float3 *vertex, float3 *normal) {
    run_2d(w, h, [&] { d_img_vertex_to_normal(make_int2(w, h), const_cast<float3 *>(vertex), normal); });
}

void ref_voxel_init(cu_voxel_t *data, int nx, int ny, int nz) {
    cu_voxel v;
    v.size = make_int3(nx, ny, nz);
    v.size_xy = nx * ny;
    v.min_t = v.max_t = v.grid_s = 0.0f;
    v.data = data;
    run_2d(ny, nz, [&] { d_voxel_initialize(v); });
}

// _cu_voxel_volumetric_integration (cu_kinect_fusion_v1.cu:534-549):
// depth scaling, then the integration over every (y, z) column
void ref_integrate(cu_voxel_t *data, int nx, int ny, int nz, float min_t, float max_t, float grid_s,
                   const float_camera_intrinsic *ci, const float_camera_extrinsic *ce, int w, int h,
                   const float *meter, const float3 *normals, int is_dynamic) {
    cu_voxel v;
    v.size = make_int3(nx, ny, nz);
    v.size_xy = nx * ny;
    v.min_t = min_t;
    v.max_t = max_t;
    v.grid_s = grid_s;
    v.data = data;
    const int2 size = make_int2(w, h);
    std::vector<float> scaled((size_t)w * h);
    std::vector<uchar3> black((size_t)w * h, make_uchar3(0, 0, 0));
    run_2d(w, h, [&] {
        d_voxel_volumetric_depth_scaling(*ci, size, const_cast<float *>(meter), scaled.data());
    });
    run_2d(ny, nz, [&] {
        d_voxel_volumetric_integration(v, *ci, *ce, size, scaled.data(), const_cast<float3 *>(normals),
                                       black.data(), is_dynamic != 0);
    });
}

// cu_voxel_run_length_encode_slice over [data, data + n); returns the bytes
// written to buffer (at most 6 per voxel)
long long ref_rle_encode_slice(const cu_voxel_t *data, long long n, char *buffer) {
    uint size = 0;
    cu_voxel_run_length_encode_slice(buffer, &size, const_cast<cu_voxel_t *>(data),
                                     const_cast<cu_voxel_t *>(data) + n);
    return (long long)size;
}

void ref_rle_decode_slice(const char *buffer, cu_voxel_t *data, long long n) {
    cu_voxel_run_length_decode_slice(const_cast<char *>(buffer), data, data + n);
}

}  // extern "C"
