// KinectFusion-side kernels on sm_103a: voxel init, depth -> metre / vertex /
// normal maps, and the projective TSDF integrate step.
//
// Replaces (cu_kinect_fusion_v1.cu, all inside the reference's `#if 0`):
//   d_voxel_initialize            (:364-379)  -> voxel_init_kernel
//   d_kinect_depth_to_meter       (:99-113)   \
//   d_img_meter_to_vertex         (:116-127)   > depth_maps_kernel (fused)
//   d_img_vertex_to_normal        (:130-151)  /
//   d_voxel_volumetric_depth_scaling (:416-425) -> depth_scale_kernel
//   d_voxel_volumetric_integration (:427-532) -> integrate_kernel
//
// The reference walks x inside each thread (one thread per (y, z) row), so
// consecutive threads touch voxels a row apart.  Here consecutive threads own
// consecutive groups of 4 voxels along x and move them with one 16-byte load
// and store, and only when at least one of the 4 is updated.
//
// Arithmetic: the reference's expressions in IEEE binary32, source order, no
// contraction (--fmad=false), __float2int_rn for the pixel coordinates.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "mcg_internal.h"
#include "unpack.h"

namespace mcg {
namespace {

// ---- voxel init -------------------------------------------------------------
__global__ void voxel_init_kernel(uint4 *__restrict__ v4, long long n4, unsigned int word0,
                                  unsigned int word1, int words_per_voxel) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    uint4 val;
    if (words_per_voxel == 1) val = make_uint4(word0, word0, word0, word0);
    else val = make_uint4(word0, word1, word0, word1);
    for (long long k = i; k < n4; k += stride) v4[k] = val;
}

__global__ void voxel_init_tail_kernel(unsigned int *__restrict__ w, long long first_word,
                                       long long n_words, unsigned int word0, unsigned int word1,
                                       int words_per_voxel) {
    const long long i = first_word + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_words) return;
    w[i] = (words_per_voxel == 1 || (i & 1) == 0) ? word0 : word1;
}

// ---- depth maps ---------------------------------------------------------------
struct Intr {
    float fx, fy, cx, cy;
};

// d_kinect_depth_to_meter, OpenNI branch (:105, :112): invalid -> 0
__device__ __forceinline__ float meter_of(uint16_t d, float dmin, float dmax) {
    float m = (float)d / 1000.0f;
    if (m < dmin || m > dmax) m = 0.0f;
    return m;
}

// float_camera_intrinsic_unproject_3 (cu_geometry_functions.h:237-246)
__device__ __forceinline__ float3 unproject(const Intr &k, int j, int i, float m) {
    if (m == 0.0f) return make_float3(0.f, 0.f, 0.f);
    const float px = ((float)j - k.cx) / k.fx;
    const float py = ((float)i - k.cy) / k.fy;
    return make_float3(px * m, py * m, m);
}

__device__ __forceinline__ bool vvalid(float3 v) { return !(v.x == 0.f && v.y == 0.f && v.z == 0.f); }

// float3_unit (cu_vector_functions.h:258-264)
__device__ __forceinline__ float3 unit3(float3 n) {
    const float norm = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    if (norm > FLT_EPSILON || norm < -FLT_EPSILON) {
        n.x = n.x / norm;
        n.y = n.y / norm;
        n.z = n.z / norm;
    }
    return n;
}

// d_img_vertex_to_normal (:130-151) for one pixel given its three vertices
__device__ __forceinline__ float3 normal_of(float3 vc, float3 vx, float3 vy) {
    if (!(vvalid(vc) && vvalid(vx) && vvalid(vy))) return make_float3(0.f, 0.f, 0.f);
    const float3 tx = make_float3(vx.x - vc.x, vx.y - vc.y, vx.z - vc.z);
    const float3 ty = make_float3(vc.x - vy.x, vc.y - vy.y, vc.z - vy.z);
    float3 n;
    n.x = tx.y * ty.z - tx.z * ty.y;
    n.y = tx.z * ty.x - tx.x * ty.z;
    n.z = tx.x * ty.y - tx.y * ty.x;
    return unit3(n);
}

// one thread per pixel; the right and lower neighbours' vertices are
// recomputed from depth instead of being exchanged
__global__ void depth_maps_kernel(Intr k, int w, int h, const uint16_t *__restrict__ depth,
                                  float dmin, float dmax, float *__restrict__ meter,
                                  float3 *__restrict__ vertex, float3 *__restrict__ normal) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= h || j >= w) return;
    const long long idx = (long long)i * w + j;
    const float m = meter_of(depth[idx], dmin, dmax);
    const float3 vc = unproject(k, j, i, m);
    if (meter) meter[idx] = m;
    if (vertex) vertex[idx] = vc;
    if (normal) {
        float3 n = make_float3(0.f, 0.f, 0.f);
        if (i < h - 1 && j < w - 1) {
            const float3 vx = unproject(k, j + 1, i, meter_of(depth[idx + 1], dmin, dmax));
            const float3 vy = unproject(k, j, i + 1, meter_of(depth[idx + w], dmin, dmax));
            n = normal_of(vc, vx, vy);
        }
        normal[idx] = n;
    }
}

__global__ void meter_to_vertex_kernel(Intr k, int w, int h, const float *__restrict__ meter,
                                       float3 *__restrict__ vertex) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= h || j >= w) return;
    const long long idx = (long long)i * w + j;
    vertex[idx] = unproject(k, j, i, meter[idx]);
}

__global__ void vertex_to_normal_kernel(int w, int h, const float3 *__restrict__ vertex,
                                        float3 *__restrict__ normal) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= h || j >= w) return;
    const long long idx = (long long)i * w + j;
    float3 n = make_float3(0.f, 0.f, 0.f);
    if (i < h - 1 && j < w - 1) n = normal_of(vertex[idx], vertex[idx + 1], vertex[idx + w]);
    normal[idx] = n;
}

// ---- integrate ------------------------------------------------------------------
// d_voxel_volumetric_depth_scaling (:416-425): z-depth -> distance along the ray
// Also the largest ray-length depth of the frame into *zmax (as float bits,
// atomic max; *zmax is zero before the launch): +inf when any value is not a
// finite number, so that the row culling below then culls nothing by depth.
__global__ void depth_scale_kernel(Intr k, int w, int h, const float *__restrict__ depth,
                                   float *__restrict__ scaled, unsigned int *__restrict__ zmax) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    unsigned int zb = 0;
    if (x < w && y < h) {
        const float px = ((float)x - k.cx) / k.fx;
        const float py = ((float)y - k.cy) / k.fy;
        const long long i = (long long)y * w + x;
        const float d = depth[i] * sqrtf(px * px + py * py + 1.0f);
        scaled[i] = d;
        zb = isfinite(d) ? __float_as_uint(fmaxf(d, 0.0f)) : 0x7f800000u;
    }
    zb = __reduce_max_sync(0xffffffffu, zb);
    if ((threadIdx.x + threadIdx.y * blockDim.x) % 32 == 0 && zb) atomicMax(zmax, zb);
}

struct IntegParams {
    int nx, ny, nz;
    float min_t, max_t, grid_s;
    Intr k;
    float r[9], t[3];
    int w, h;
    const float *ds;        // ray-length depth
    const float3 *normals;  // optional normal map
    const float *ray_x;     // accumulated x coordinate per voxel column
    const float *pose_dev;  // if set: r[9], t[3] read from device memory (graph replay)
    int is_dynamic;
    const int2 *rows;       // per (y, z) row: the voxels x0 .. x1 that can be updated (x1 < x0: none)
};

// pose from device memory into the block's copy of the parameters
__device__ __forceinline__ void load_pose(IntegParams &p) {
    __shared__ float pose[12];
    if (p.pose_dev) {
        if (threadIdx.x < 12) pose[threadIdx.x] = p.pose_dev[threadIdx.x];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 9; ++i) p.r[i] = pose[i];
#pragma unroll
        for (int i = 0; i < 3; ++i) p.t[i] = pose[9 + i];
    }
}

// d_pack_tsdf / d_pack_weight / d_unpack_weight (cu_kinect_fusion_v1.h:152-171)
__device__ __forceinline__ short pack_tsdf(float f) { return (short)(int)(f * (float)kMaxTsdf); }
__device__ __forceinline__ unsigned short pack_weight(float w) {
    w = (w < kUbW) ? w / kUbW : 1.0f;
    return (unsigned short)(w * (float)kMaxW + 0.5f);
}
__device__ __forceinline__ float unpack_weight(unsigned short w) { return (float)w / (float)kMaxW * kUbW; }

// One observation of a voxel: truncated sdf, weight before the dynamic term,
// ray-length depth at the pixel, ds/dz (0 where the sdf is clamped at 1),
// the pixel's ray scale and the pixel index.
struct Obs {
    float s, w0, z, dsdz, c;
    long long pix;
};

// Per-voxel part of :442-529 up to the update.  Returns false when the voxel
// is not updated.  zat(u, v, pix, c) gives the ray-length depth at the pixel
// (and its ray scale c).
template <class ZAt>
__device__ __forceinline__ bool observe_core(const float *r, const float *t, const Intr &k, int w, int h,
                                             float min_t, float max_t, const float3 *normals, ZAt zat,
                                             float px, float py, float pz, Obs &o) {
    // float_camera_extrinsic_backward (cu_geometry_functions.h:125-129), matrix33_tv
    const float v0 = px - t[0], v1 = py - t[1], v2 = pz - t[2];
    const float q0 = r[0] * v0 + r[1] * v1 + r[2] * v2;
    const float q1 = r[3] * v0 + r[4] * v1 + r[5] * v2;
    const float q2 = r[6] * v0 + r[7] * v1 + r[8] * v2;
    if (q2 < FLT_MIN) return false;
    // float_camera_intrinsic_project_3 (cu_geometry_functions.h:232-235)
    const float uf = k.fx * (q0 / q2) + k.cx;
    const float vf = k.fy * (q1 / q2) + k.cy;
    const int u = __float2int_rn(uf), v = __float2int_rn(vf);
    if (u < 0 || v < 0 || u >= (w - 2) || v >= (h - 2)) return false;
    const long long pix = (long long)v * w + u;
    float c = 1.0f;
    const float z_val = zat(u, v, pix, c);
    if (!(z_val > FLT_MIN)) return false;
    const float qn = sqrtf(q0 * q0 + q1 * q1 + q2 * q2);
    float s = z_val - qn;
    if (!(s >= -min_t)) return false;
    float dsdz;
    if (s > 0.0f) {
        s = s / max_t;
        dsdz = 1.0f / max_t;
        if (s > 1.0f) {
            s = 1.0f;
            dsdz = 0.0f;
        }
    } else {
        s = s / min_t;
        dsdz = 1.0f / min_t;
    }
    float wgt = 1.0f;
    if (normals) {
        const float3 n = normals[pix];
        if (!vvalid(n)) return false;
        wgt = -(n.x * (q0 / qn) + n.y * (q1 / qn) + n.z * (q2 / qn));
        if (wgt < FLT_MIN) return false;
    }
    o.w0 = wgt / z_val;
    o.s = s;
    o.z = z_val;
    o.dsdz = dsdz;
    o.c = c;
    o.pix = pix;
    return true;
}

__device__ __forceinline__ bool observe(const IntegParams &p, float px, float py, float pz,
                                        float &sdf, float &weight) {
    Obs o;
    const float *ds = p.ds;
    if (!observe_core(p.r, p.t, p.k, p.w, p.h, p.min_t, p.max_t, p.normals,
                      [ds](int, int, long long pix, float &) { return ds[pix]; }, px, py, pz, o))
        return false;
    sdf = o.s;
    weight = o.w0;
    return true;
}

// :509-529 weighted running average (FP32 path)
__device__ __forceinline__ void fuse_core(int is_dynamic, float sdf, float weight, float sdf1, float w1,
                                          float &sdf2, float &w2) {
    if (is_dynamic) {
        const float d = fabsf(sdf - sdf1);
        weight = weight * (1.0f + d * d * 10.0f);
    }
    w2 = w1 + weight;
    sdf2 = (w1 * sdf1 + weight * sdf) / w2;
}

__device__ __forceinline__ void fuse(const IntegParams &p, float sdf, float weight, float sdf1,
                                     float w1, float &sdf2, float &w2) {
    fuse_core(p.is_dynamic, sdf, weight, sdf1, w1, sdf2, w2);
}

// Row culling.  Along a voxel row (fixed y, z) the camera-frame point is
// linear in the row's x coordinate X: q(X) = q(0) + X (r0, r3, r6).  A voxel
// can be updated only if q_z > 0, its pixel lies inside the image (u in
// [0, w-3], v in [0, h-3] after rounding) and q_z <= |q| <= zmax + min_t
// (otherwise its sdf is below -min_t for every pixel).  With q_z > 0 each
// image bound is a linear inequality in X (fx q_x + (cx - u_bound) q_z
// against 0), so the row's candidates form one interval of X.  The bounds
// are widened by one pixel and each inequality by an absolute 1e-3, which
// covers the binary32 error of evaluating them, and the interval by two
// voxels beyond its ends, which covers the accumulated x coordinates
// (p.x += grid_s, :434-444); the exact per-voxel tests still decide.
__global__ void __launch_bounds__(256) integrate_rows_kernel(IntegParams p, const unsigned int *__restrict__ zmax,
                                                             int2 *__restrict__ rows) {
    load_pose(p);
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (long long)p.ny * p.nz) return;
    const int y = (int)(row % p.ny), z = (int)(row / p.ny);
    const float py = (float)y * p.grid_s, pz = (float)z * p.grid_s;
    const float v1 = py - p.t[1], v2 = pz - p.t[2];
    float A[3], B[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        A[k] = p.r[3 * k] * (-p.t[0]) + p.r[3 * k + 1] * v1 + p.r[3 * k + 2] * v2;
        B[k] = p.r[3 * k];
    }
    const float zb = __uint_as_float(*zmax);
    const float zlim = zb + p.min_t;
    const float m = 1.0f;
    const float xmax = (float)p.nx * p.grid_s + fabsf(p.grid_s);
    // constraints a + b X >= -d_c, d_c 1e-5 of the constraint's terms' size
    // (two orders above the binary32 error of evaluating them) plus 1e-3
    float a[6], b[6], sz[6];
    const float ul = p.k.cx + 1.0f + m, uh = (float)p.w - 2.0f + m - p.k.cx;
    const float vl = p.k.cy + 1.0f + m, vh = (float)p.h - 2.0f + m - p.k.cy;
    const float s0 = fabsf(p.r[0] * p.t[0]) + fabsf(p.r[1] * v1) + fabsf(p.r[2] * v2) + fabsf(B[0]) * xmax;
    const float s1 = fabsf(p.r[3] * p.t[0]) + fabsf(p.r[4] * v1) + fabsf(p.r[5] * v2) + fabsf(B[1]) * xmax;
    const float s2 = fabsf(p.r[6] * p.t[0]) + fabsf(p.r[7] * v1) + fabsf(p.r[8] * v2) + fabsf(B[2]) * xmax;
    a[0] = A[2]; b[0] = B[2]; sz[0] = s2;                                                    // q_z >= 0
    a[1] = p.k.fx * A[0] + ul * A[2]; b[1] = p.k.fx * B[0] + ul * B[2];                      // u >= -1 - m
    sz[1] = fabsf(p.k.fx) * s0 + fabsf(ul) * s2;
    a[2] = uh * A[2] - p.k.fx * A[0]; b[2] = uh * B[2] - p.k.fx * B[0];                      // u <= w - 2 + m
    sz[2] = fabsf(uh) * s2 + fabsf(p.k.fx) * s0;
    a[3] = p.k.fy * A[1] + vl * A[2]; b[3] = p.k.fy * B[1] + vl * B[2];                      // v >= -1 - m
    sz[3] = fabsf(p.k.fy) * s1 + fabsf(vl) * s2;
    a[4] = vh * A[2] - p.k.fy * A[1]; b[4] = vh * B[2] - p.k.fy * B[1];                      // v <= h - 2 + m
    sz[4] = fabsf(vh) * s2 + fabsf(p.k.fy) * s1;
    const int nc = isfinite(zlim) ? 6 : 5;
    a[5] = zlim - A[2]; b[5] = -B[2]; sz[5] = fabsf(zlim) + s2;                              // q_z <= zmax + min_t
    float lo = -INFINITY, hi = INFINITY;
    bool empty = false;
    for (int c = 0; c < nc; ++c) {
        const float d = 1e-5f * sz[c] + 1e-3f;
        const float t = (-d - a[c]);
        if (b[c] > 0.0f) lo = fmaxf(lo, t / b[c]);
        else if (b[c] < 0.0f) hi = fminf(hi, t / b[c]);
        else if (a[c] < -d) empty = true;
    }
    int x0 = 0, x1 = -1;
    if (!empty && !(lo > hi)) {
        const float g = p.grid_s;
        const float fl = floorf(lo / g) - 2.0f, fh = ceilf(hi / g) + 2.0f;
        x0 = fl <= 0.0f ? 0 : (fl >= (float)p.nx ? p.nx : (int)fl);
        x1 = fh >= (float)(p.nx - 1) ? p.nx - 1 : (fh < 0.0f ? -1 : (int)fh);
    }
    rows[row] = make_int2(x0, x1);
}

// short2 volume, 4 voxels per thread; vec = 16-byte path usable
__global__ void __launch_bounds__(256) integrate_short2_kernel(IntegParams p, short2 *__restrict__ vol, int vec) {
    load_pose(p);
    const int groups = (p.nx + 3) >> 2;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)p.ny * p.nz;
    if (gid >= (long long)groups * rows) return;
    const int g = (int)(gid % groups);
    const long long row = gid / groups;
    const int y = (int)(row % p.ny), z = (int)(row / p.ny);
    const float py = (float)y * p.grid_s, pz = (float)z * p.grid_s;
    const int x0 = g * 4;
    const int2 span = p.rows[row];
    if (x0 + 3 < span.x || x0 > span.y) return;
    float sdf[4], wt[4];
    unsigned int upd = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int x = x0 + i;
        if (x < p.nx && observe(p, p.ray_x[x], py, pz, sdf[i], wt[i])) upd |= 1u << i;
    }
    if (!upd) return;
    short2 *row_ptr = vol + row * p.nx;
    short2 cur[4];
    if (vec) {
        const uint4 raw = *reinterpret_cast<const uint4 *>(row_ptr + x0);
        cur[0] = *reinterpret_cast<const short2 *>(&raw.x);
        cur[1] = *reinterpret_cast<const short2 *>(&raw.y);
        cur[2] = *reinterpret_cast<const short2 *>(&raw.z);
        cur[3] = *reinterpret_cast<const short2 *>(&raw.w);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (upd & (1u << i)) cur[i] = row_ptr[x0 + i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (!(upd & (1u << i))) continue;
        const float sdf1 = mcg_unpack_tsdf(cur[i].x);  // (float)tsdf / 32766, exact
        const float w1 = unpack_weight((unsigned short)cur[i].y);
        float s2, w2;
        fuse(p, sdf[i], wt[i], sdf1, w1, s2, w2);
        cur[i].x = pack_tsdf(s2);
        cur[i].y = (short)pack_weight(w2);
    }
    if (vec) {
        uint4 raw;
        raw.x = *reinterpret_cast<const unsigned int *>(&cur[0]);
        raw.y = *reinterpret_cast<const unsigned int *>(&cur[1]);
        raw.z = *reinterpret_cast<const unsigned int *>(&cur[2]);
        raw.w = *reinterpret_cast<const unsigned int *>(&cur[3]);
        *reinterpret_cast<uint4 *>(row_ptr + x0) = raw;
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (upd & (1u << i)) row_ptr[x0 + i] = cur[i];
    }
}

// float2 volume (FP32 tsdf and weight, no packing), 2 voxels per thread
__global__ void __launch_bounds__(256) integrate_float2_kernel(IntegParams p, float2 *__restrict__ vol, int vec) {
    load_pose(p);
    const int groups = (p.nx + 1) >> 1;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)p.ny * p.nz;
    if (gid >= (long long)groups * rows) return;
    const int g = (int)(gid % groups);
    const long long row = gid / groups;
    const int y = (int)(row % p.ny), z = (int)(row / p.ny);
    const float py = (float)y * p.grid_s, pz = (float)z * p.grid_s;
    const int x0 = g * 2;
    const int2 span = p.rows[row];
    if (x0 + 1 < span.x || x0 > span.y) return;
    float sdf[2], wt[2];
    unsigned int upd = 0;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int x = x0 + i;
        if (x < p.nx && observe(p, p.ray_x[x], py, pz, sdf[i], wt[i])) upd |= 1u << i;
    }
    if (!upd) return;
    float2 *row_ptr = vol + row * p.nx;
    float2 cur[2];
    if (vec) {
        const float4 raw = *reinterpret_cast<const float4 *>(row_ptr + x0);
        cur[0] = make_float2(raw.x, raw.y);
        cur[1] = make_float2(raw.z, raw.w);
    } else {
#pragma unroll
        for (int i = 0; i < 2; ++i)
            if (upd & (1u << i)) cur[i] = row_ptr[x0 + i];
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        if (!(upd & (1u << i))) continue;
        float s2, w2;
        fuse(p, sdf[i], wt[i], cur[i].x, cur[i].y, s2, w2);
        cur[i] = make_float2(s2, w2);
    }
    if (vec) {
        *reinterpret_cast<float4 *>(row_ptr + x0) = make_float4(cur[0].x, cur[0].y, cur[1].x, cur[1].y);
    } else {
#pragma unroll
        for (int i = 0; i < 2; ++i)
            if (upd & (1u << i)) row_ptr[x0 + i] = cur[i];
    }
}

// ---- integrate adjoint ----------------------------------------------------------
// Reverse of a sequence of float2 integrate steps (no counterpart in the
// reference).  Per voxel, step k (observation s, weight w) maps
//   W' = W + w,  F' = (W F + w s) / W'
// so, holding the discrete choices (pixel, truncation, clamp) fixed,
//   dF'/dF = W/W',  dF'/dW = (F - F')/W',  dF'/ds = w/W',  dF'/dw = (s - F')/W'
// and s = (c d - |q|)/m (m = max_t or min_t, ds/dz = 0 where clamped),
// w = wgt / (c d) (dw/dd = -w c / z) with d the pixel's z-depth and c its
// ray scale.  The dynamic term multiplies w by 1 + 10 (s - F)^2.  Normal maps
// are held constant.
constexpr int BW_SEG = 16;                    // frames whose (F, W) one thread keeps while reversing
constexpr int BW_MAX_FRAMES = BW_SEG * 32;    // frames per call (checkpoint every BW_SEG)

struct IntegBwParams {
    int nx, ny, nz;
    float min_t, max_t, grid_s;
    Intr k;
    int w, h, n_frames;
    const float *poses;    // n_frames x (r[9] column-major, t[3])
    const float *depth;    // n_frames x h x w metres (z-depth)
    const float3 *normals; // n_frames x h x w, or null
    const float *ray_x;
    int is_dynamic;
    const float2 *vol0;    // volume before the first frame, or null: (-1, 0)
    const float *grad_f;   // dL/dF after the last frame
    const float *grad_w;   // dL/dW after the last frame, or null: 0
    float *grad_depth;     // n_frames x h x w, accumulated
    float *grad_f0;        // dL/dF before the first frame, or null
    float *grad_w0;
};

__device__ __forceinline__ bool bw_observe(const IntegBwParams &p, const float *pose, int f, float px,
                                           float py, float pz, Obs &o) {
    const long long plane = (long long)p.w * p.h;
    const float *dep = p.depth + f * plane;
    const Intr k = p.k;
    return observe_core(pose, pose + 9, k, p.w, p.h, p.min_t, p.max_t, p.normals ? p.normals + f * plane : nullptr,
                        [dep, k](int u, int v, long long pix, float &c) {
                            // d_voxel_volumetric_depth_scaling (:416-425) for one pixel
                            const float cx = ((float)u - k.cx) / k.fx;
                            const float cy = ((float)v - k.cy) / k.fy;
                            c = sqrtf(cx * cx + cy * cy + 1.0f);
                            return dep[pix] * c;
                        },
                        px, py, pz, o);
}

__global__ void __launch_bounds__(128) integrate_backward_kernel(IntegBwParams p) {
    extern __shared__ float s_pose[];
    for (int i = threadIdx.x; i < p.n_frames * 12; i += blockDim.x) s_pose[i] = p.poses[i];
    __syncthreads();
    const long long n = (long long)p.nx * p.ny * p.nz;
    const int nseg = (p.n_frames + BW_SEG - 1) / BW_SEG;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float gF = p.grad_f[i];
        float gW = p.grad_w ? p.grad_w[i] : 0.0f;
        if (gF != 0.0f || gW != 0.0f) {
            const int x = (int)(i % p.nx);
            const long long row = i / p.nx;
            const int y = (int)(row % p.ny), z = (int)(row / p.ny);
            const float px = p.ray_x[x], py = (float)y * p.grid_s, pz = (float)z * p.grid_s;
            float F = p.vol0 ? p.vol0[i].x : -1.0f;
            float W = p.vol0 ? p.vol0[i].y : 0.0f;
            // forward sweep: (F, W) at the start of every segment
            float ckF[BW_MAX_FRAMES / BW_SEG], ckW[BW_MAX_FRAMES / BW_SEG];
            for (int f = 0; f < p.n_frames; ++f) {
                if (f % BW_SEG == 0) {
                    ckF[f / BW_SEG] = F;
                    ckW[f / BW_SEG] = W;
                }
                Obs o;
                if (bw_observe(p, s_pose + 12 * f, f, px, py, pz, o)) fuse_core(p.is_dynamic, o.s, o.w0, F, W, F, W);
            }
            for (int sg = nseg - 1; sg >= 0; --sg) {
                const int f0 = sg * BW_SEG;
                const int f1 = min(p.n_frames, f0 + BW_SEG);
                float sF[BW_SEG], sW[BW_SEG];
                float cF = ckF[sg], cW = ckW[sg];
                for (int f = f0; f < f1; ++f) {
                    sF[f - f0] = cF;
                    sW[f - f0] = cW;
                    Obs o;
                    if (bw_observe(p, s_pose + 12 * f, f, px, py, pz, o))
                        fuse_core(p.is_dynamic, o.s, o.w0, cF, cW, cF, cW);
                }
                for (int f = f1 - 1; f >= f0; --f) {
                    Obs o;
                    if (!bw_observe(p, s_pose + 12 * f, f, px, py, pz, o)) continue;
                    const float Fp = sF[f - f0], Wp = sW[f - f0];
                    float wv = o.w0, mult = 1.0f, d = 0.0f;
                    if (p.is_dynamic) {
                        d = o.s - Fp;
                        mult = 1.0f + d * d * 10.0f;
                        wv = wv * mult;
                    }
                    const float Wn = Wp + wv;
                    const float Fn = (Wp * Fp + wv * o.s) / Wn;
                    float gs = gF * wv / Wn;
                    const float gw = gF * (o.s - Fn) / Wn + gW;
                    float gFp = gF * Wp / Wn;
                    const float gWp = gF * (Fp - Fn) / Wn + gW;
                    float gw0 = gw;
                    if (p.is_dynamic) {
                        const float t = gw * o.w0 * 20.0f * d;
                        gs += t;
                        gFp -= t;
                        gw0 = gw * mult;
                    }
                    const float gz = gs * o.dsdz - gw0 * o.w0 / o.z;
                    atomicAdd(p.grad_depth + f * (long long)p.w * p.h + o.pix, gz * o.c);
                    gF = gFp;
                    gW = gWp;
                }
            }
        }
        if (p.grad_f0) p.grad_f0[i] = gF;
        if (p.grad_w0) p.grad_w0[i] = gW;
    }
}

Intr intr_of(const mcg_intrinsic *k) { return Intr{k->fx, k->fy, k->cx, k->cy}; }

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" {

mcg_status mcg_voxel_init(mcg_context *ctx, void *vol, int32_t voxel_type, int64_t n_voxels,
                          mcg_stream_t stream) {
    if (!ctx || (n_voxels > 0 && !vol) || n_voxels < 0) return MCG_ERR_INVALID_ARG;
    if (voxel_type != MCG_VOXEL_SHORT2 && voxel_type != MCG_VOXEL_FLOAT2) return MCG_ERR_INVALID_ARG;
    if (n_voxels == 0) return MCG_OK;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int w0, w1;
    int wpv;
    if (voxel_type == MCG_VOXEL_SHORT2) {
        // {tsdf = -32766, w = 0}
        w0 = (unsigned int)(unsigned short)(short)(-kMaxTsdf);
        w1 = 0;
        wpv = 1;
    } else {
        const float m1 = -1.0f;
        w0 = *reinterpret_cast<const unsigned int *>(&m1);
        w1 = 0;
        wpv = 2;
    }
    const long long n_words = (long long)n_voxels * wpv;
    long long n4 = 0;
    if (((uintptr_t)vol & 15) == 0) n4 = n_words / 4;
    if (n4 > 0) {
        long long grid = (n4 + 255) / 256;
        const long long cap = (long long)ctx->num_sms * 16;
        if (grid > cap) grid = cap;
        voxel_init_kernel<<<(int)grid, 256, 0, s>>>((uint4 *)vol, n4, w0, w1, wpv);
    }
    const long long first = n4 * 4;
    if (first < n_words) {
        const long long rem = n_words - first;
        voxel_init_tail_kernel<<<(unsigned int)((rem + 255) / 256), 256, 0, s>>>(
            (unsigned int *)vol, first, n_words, w0, w1, wpv);
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

mcg_status mcg_depth_to_maps(mcg_context *ctx, const mcg_intrinsic *k, int32_t w, int32_t h,
                             const uint16_t *depth_mm, float depth_min, float depth_max,
                             float *meter, float *vertex, float *normal, mcg_stream_t stream) {
    if (!ctx || !k || !depth_mm || w <= 0 || h <= 0) return MCG_ERR_INVALID_ARG;
    if (!meter && !vertex && !normal) return MCG_OK;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const dim3 block(32, 8), grid((w + 31) / 32, (h + 7) / 8);
    depth_maps_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(intr_of(k), w, h, depth_mm, depth_min,
                                                                depth_max, meter, (float3 *)vertex,
                                                                (float3 *)normal);
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

mcg_status mcg_meter_to_vertex(mcg_context *ctx, const mcg_intrinsic *k, int32_t w, int32_t h,
                               const float *meter, float *vertex, mcg_stream_t stream) {
    if (!ctx || !k || !meter || !vertex || w <= 0 || h <= 0) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const dim3 block(32, 8), grid((w + 31) / 32, (h + 7) / 8);
    meter_to_vertex_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(intr_of(k), w, h, meter, (float3 *)vertex);
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

mcg_status mcg_vertex_to_normal(mcg_context *ctx, int32_t w, int32_t h, const float *vertex,
                                float *normal, mcg_stream_t stream) {
    if (!ctx || !vertex || !normal || w <= 0 || h <= 0) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const dim3 block(32, 8), grid((w + 31) / 32, (h + 7) / 8);
    vertex_to_normal_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(w, h, (const float3 *)vertex, (float3 *)normal);
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

// x coordinate table, accumulated exactly as :434/:444 do
// x coordinate of voxel column x as kf.cu:434-444 accumulates it: p.x starts
// at 0 and grows by grid_s per voxel, in FP32, one addition after another
__global__ void ray_x_kernel(float *__restrict__ out, int nx, float g) {
    float px = -g;
    for (int x = 0; x < nx; ++x) {
        px = __fadd_rn(px, g);
        out[x] = px;
    }
}

// the context's table for (nx, grid_s), built by one thread on stream s the
// first time (and waited for); inside a stream capture a missing table is MCG_ERR_STATE (an
// earlier call with this volume shape outside the capture builds it)
static mcg_status ray_x_table(mcg_context *ctx, int32_t nx, float grid_s, cudaStream_t s, const float **out) {
    for (const auto &r : ctx->ray_x)
        if (r.nx == nx && __builtin_memcmp(&r.g, &grid_s, sizeof(float)) == 0) {
            *out = r.d;
            return MCG_OK;
        }
    if (mcg_capturing(s)) return MCG_ERR_STATE;
    float *d = nullptr;
    if (cudaMalloc((void **)&d, sizeof(float) * (size_t)nx) != cudaSuccess)
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    ray_x_kernel<<<1, 1, 0, s>>>(d, nx, grid_s);
    // once per shape: complete before a call on another stream can use it
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(d);
        return mcg_cuda_fail(ctx, e);
    }
    ctx->ray_x.push_back({nx, grid_s, d});
    *out = d;
    return MCG_OK;
}

static mcg_status integrate_impl(mcg_context *ctx, void *vol, int32_t voxel_type, int32_t nx, int32_t ny,
                                 int32_t nz, float min_t, float max_t, float grid_s, const mcg_intrinsic *k,
                                 const mcg_extrinsic *ext, const float *pose_dev, int32_t w, int32_t h,
                                 const float *depth_m, const float *normals, int32_t is_dynamic,
                                 mcg_stream_t stream) {
    if (!ctx || !vol || !k || (!ext && !pose_dev) || !depth_m || nx <= 0 || ny <= 0 || nz <= 0 || w <= 0 || h <= 0)
        return MCG_ERR_INVALID_ARG;
    if (voxel_type != MCG_VOXEL_SHORT2 && voxel_type != MCG_VOXEL_FLOAT2) return MCG_ERR_INVALID_ARG;
    if (!(min_t > 0.0f) || !(max_t > 0.0f) || !(grid_s > 0.0f)) return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const long long rows = (long long)ny * nz;
    // inside a stream capture nothing may be allocated: an earlier call of
    // the same shapes outside the capture has sized every buffer
    if (mcg_capturing(s) && (ctx->depth_scaled_cap < (size_t)w * h || ctx->integ_rows_cap < (size_t)rows ||
                             ctx->integ_zmax_cap < 1))
        return MCG_ERR_STATE;
    if (!ensure(&ctx->depth_scaled, &ctx->depth_scaled_cap, (size_t)w * h))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    const float *ray_x = nullptr;
    {
        const mcg_status st = ray_x_table(ctx, nx, grid_s, s, &ray_x);
        if (st != MCG_OK) return st;
    }
    IntegParams p;
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.min_t = min_t; p.max_t = max_t; p.grid_s = grid_s;
    p.k = intr_of(k);
    for (int i = 0; i < 9; ++i) p.r[i] = ext ? ext->r[i] : 0.0f;
    for (int i = 0; i < 3; ++i) p.t[i] = ext ? ext->t[i] : 0.0f;
    p.pose_dev = ext ? nullptr : pose_dev;
    p.w = w; p.h = h;
    p.ds = ctx->depth_scaled;
    p.normals = (const float3 *)normals;
    p.ray_x = ray_x;
    p.is_dynamic = is_dynamic ? 1 : 0;
    if (!ensure(&ctx->integ_rows, &ctx->integ_rows_cap, (size_t)rows) ||
        !ensure(&ctx->integ_zmax, &ctx->integ_zmax_cap, (size_t)1))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    p.rows = ctx->integ_rows;
    e = cudaMemsetAsync(ctx->integ_zmax, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const dim3 b2(32, 8), g2((w + 31) / 32, (h + 7) / 8);
    depth_scale_kernel<<<g2, b2, 0, s>>>(p.k, w, h, depth_m, ctx->depth_scaled, ctx->integ_zmax);
    integrate_rows_kernel<<<(unsigned int)((rows + 255) / 256), 256, 0, s>>>(p, ctx->integ_zmax, ctx->integ_rows);
    if (voxel_type == MCG_VOXEL_SHORT2) {
        const int vec = (nx % 4 == 0) && (((uintptr_t)vol & 15) == 0);
        const long long threads = (long long)((nx + 3) / 4) * rows;
        integrate_short2_kernel<<<(unsigned int)((threads + 255) / 256), 256, 0, s>>>(p, (short2 *)vol, vec);
    } else {
        const int vec = (nx % 2 == 0) && (((uintptr_t)vol & 15) == 0);
        const long long threads = (long long)((nx + 1) / 2) * rows;
        integrate_float2_kernel<<<(unsigned int)((threads + 255) / 256), 256, 0, s>>>(p, (float2 *)vol, vec);
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

mcg_status mcg_integrate(mcg_context *ctx, void *vol, int32_t voxel_type, int32_t nx, int32_t ny,
                         int32_t nz, float min_t, float max_t, float grid_s,
                         const mcg_intrinsic *k, const mcg_extrinsic *ext, int32_t w, int32_t h,
                         const float *depth_m, const float *normals, int32_t is_dynamic,
                         mcg_stream_t stream) {
    if (!ext) return MCG_ERR_INVALID_ARG;
    return integrate_impl(ctx, vol, voxel_type, nx, ny, nz, min_t, max_t, grid_s, k, ext, nullptr, w, h, depth_m,
                          normals, is_dynamic, stream);
}

mcg_status mcg_integrate_device_pose(mcg_context *ctx, void *vol, int32_t voxel_type, int32_t nx, int32_t ny,
                                     int32_t nz, float min_t, float max_t, float grid_s, const mcg_intrinsic *k,
                                     const float *pose_dev, int32_t w, int32_t h, const float *depth_m,
                                     const float *normals, int32_t is_dynamic, mcg_stream_t stream) {
    if (!pose_dev) return MCG_ERR_INVALID_ARG;
    return integrate_impl(ctx, vol, voxel_type, nx, ny, nz, min_t, max_t, grid_s, k, nullptr, pose_dev, w, h,
                          depth_m, normals, is_dynamic, stream);
}


mcg_status mcg_integrate_backward(mcg_context *ctx, const void *vol0, int32_t nx, int32_t ny, int32_t nz,
                                  float min_t, float max_t, float grid_s, const mcg_intrinsic *k, int32_t n_frames,
                                  const float *poses_dev, int32_t w, int32_t h, const float *depth_m,
                                  const float *normals, int32_t is_dynamic, const float *grad_f,
                                  const float *grad_w, float *grad_depth, float *grad_f0, float *grad_w0,
                                  mcg_stream_t stream) {
    if (!ctx || !k || !poses_dev || !depth_m || !grad_f || !grad_depth || nx <= 0 || ny <= 0 || nz <= 0 ||
        w <= 0 || h <= 0 || n_frames <= 0)
        return MCG_ERR_INVALID_ARG;
    if (!(min_t > 0.0f) || !(max_t > 0.0f) || !(grid_s > 0.0f)) return MCG_ERR_INVALID_ARG;
    if (n_frames > BW_MAX_FRAMES) return MCG_ERR_TOO_LARGE;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const float *ray_x = nullptr;
    const mcg_status st = ray_x_table(ctx, nx, grid_s, s, &ray_x);
    if (st != MCG_OK) return st;
    IntegBwParams p;
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.min_t = min_t; p.max_t = max_t; p.grid_s = grid_s;
    p.k = intr_of(k);
    p.w = w; p.h = h; p.n_frames = n_frames;
    p.poses = poses_dev;
    p.depth = depth_m;
    p.normals = (const float3 *)normals;
    p.ray_x = ray_x;
    p.is_dynamic = is_dynamic ? 1 : 0;
    p.vol0 = (const float2 *)vol0;
    p.grad_f = grad_f;
    p.grad_w = grad_w;
    p.grad_depth = grad_depth;
    p.grad_f0 = grad_f0;
    p.grad_w0 = grad_w0;
    const long long n = (long long)nx * ny * nz;
    long long grid = (n + 127) / 128;
    const long long cap = (long long)ctx->num_sms * 16;
    if (grid > cap) grid = cap;
    integrate_backward_kernel<<<(unsigned int)grid, 128, sizeof(float) * 12 * n_frames, s>>>(p);
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

}  // extern "C"
