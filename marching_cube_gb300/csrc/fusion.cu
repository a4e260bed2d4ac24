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
__global__ void depth_scale_kernel(Intr k, int w, int h, const float *__restrict__ depth,
                                   float *__restrict__ scaled) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float px = ((float)x - k.cx) / k.fx;
    const float py = ((float)y - k.cy) / k.fy;
    const long long i = (long long)y * w + x;
    scaled[i] = depth[i] * sqrtf(px * px + py * py + 1.0f);
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

// Per-voxel part of :442-529 up to the update.  Returns false when the voxel
// is not updated; otherwise the new observation (sdf, weight before the
// dynamic term).
__device__ __forceinline__ bool observe(const IntegParams &p, float px, float py, float pz,
                                        float &sdf, float &weight) {
    // float_camera_extrinsic_backward (cu_geometry_functions.h:125-129), matrix33_tv
    const float v0 = px - p.t[0], v1 = py - p.t[1], v2 = pz - p.t[2];
    const float q0 = p.r[0] * v0 + p.r[1] * v1 + p.r[2] * v2;
    const float q1 = p.r[3] * v0 + p.r[4] * v1 + p.r[5] * v2;
    const float q2 = p.r[6] * v0 + p.r[7] * v1 + p.r[8] * v2;
    if (q2 < FLT_MIN) return false;
    // float_camera_intrinsic_project_3 (cu_geometry_functions.h:232-235)
    const float uf = p.k.fx * (q0 / q2) + p.k.cx;
    const float vf = p.k.fy * (q1 / q2) + p.k.cy;
    const int u = __float2int_rn(uf), v = __float2int_rn(vf);
    if (u < 0 || v < 0 || u >= (p.w - 2) || v >= (p.h - 2)) return false;
    const long long pix = (long long)v * p.w + u;
    const float z_val = p.ds[pix];
    if (!(z_val > FLT_MIN)) return false;
    const float qn = sqrtf(q0 * q0 + q1 * q1 + q2 * q2);
    float s = z_val - qn;
    if (!(s >= -p.min_t)) return false;
    if (s > 0.0f) {
        s = s / p.max_t;
        if (s > 1.0f) s = 1.0f;
    } else {
        s = s / p.min_t;
    }
    float wgt = 1.0f;
    if (p.normals) {
        const float3 n = p.normals[pix];
        if (!vvalid(n)) return false;
        wgt = -(n.x * (q0 / qn) + n.y * (q1 / qn) + n.z * (q2 / qn));
        if (wgt < FLT_MIN) return false;
    }
    weight = wgt / z_val;
    sdf = s;
    return true;
}

__device__ __forceinline__ void fuse(const IntegParams &p, float sdf, float weight, float sdf1,
                                     float w1, float &sdf2, float &w2) {
    if (p.is_dynamic) {
        const float d = fabsf(sdf - sdf1);
        weight = weight * (1.0f + d * d * 10.0f);
    }
    w2 = w1 + weight;
    sdf2 = (w1 * sdf1 + weight * sdf) / w2;
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
    if (!ensure(&ctx->depth_scaled, &ctx->depth_scaled_cap, (size_t)w * h))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    // x coordinate table, accumulated exactly as :434/:444 do
    if (ctx->ray_x_n != nx || ctx->ray_x_g != grid_s || !ctx->ray_x) {
        if (!ensure(&ctx->ray_x, &ctx->ray_x_cap, (size_t)nx)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        if (ctx->h_ray_x_cap < (size_t)nx) {
            if (ctx->h_ray_x) cudaFreeHost(ctx->h_ray_x);
            ctx->h_ray_x = nullptr;
            ctx->h_ray_x_cap = 0;
            if (cudaMallocHost((void **)&ctx->h_ray_x, sizeof(float) * nx) != cudaSuccess)
                return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
            ctx->h_ray_x_cap = nx;
        }
        // the pinned table may still be in flight from an earlier call
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        volatile float px = -grid_s;
        for (int x = 0; x < nx; ++x) {
            px = px + grid_s;
            ctx->h_ray_x[x] = px;
        }
        e = cudaMemcpyAsync(ctx->ray_x, ctx->h_ray_x, sizeof(float) * nx, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        ctx->ray_x_n = nx;
        ctx->ray_x_g = grid_s;
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
    p.ray_x = ctx->ray_x;
    p.is_dynamic = is_dynamic ? 1 : 0;
    const dim3 b2(32, 8), g2((w + 31) / 32, (h + 7) / 8);
    depth_scale_kernel<<<g2, b2, 0, s>>>(p.k, w, h, depth_m, ctx->depth_scaled);
    const long long rows = (long long)ny * nz;
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

}  // extern "C"
