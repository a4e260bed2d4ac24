// Ray casting of a short2 TSDF volume into depth and normal maps on sm_103a.
//
// Replaces d_voxel_extract_depth_and_normal_map and its host set-up
// (cu_kinect_fusion_v1.cu:786-986, with the trilinear sampler :551-657 and
// the surface normal :3146-3233).  One thread per pixel marches its ray as
// the reference does: entry and exit over the six faces of the volume shrunk
// by one voxel, steps of 1 voxel, backing off and stepping 0.25 inside the
// truncation band, the zero crossing placed by linear interpolation of the
// last two samples (eq. 15), a back-face crossing ends the ray.
//
// The camera set-up (K, M = K R^T, M^-1, camera centre) is computed on the
// device by one thread per CTA in the reference's binary32 operation order,
// so host compilers' contraction rules play no part in the results.  A
// singular M writes nothing, as the reference launches nothing then.
//
// Arithmetic: the reference's expressions in IEEE binary32, source order, no
// contraction (--fmad=false).
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "mc_common.cuh"

namespace mcg {
namespace {

struct RayCamera {
    float IM[3][3];  // (K R^T)^-1, columns IM[j]
    float cc[3];     // camera centre in voxel units
    int ok;
};

struct RayParams {
    const short2 *vol;
    int nx, ny, nz;
    float grid_s;
    float fx, fy, cx, cy;
    float r[9], t[3];  // camera -> global, rotation column-major
    int w, h;
    float *depth;
    float *normal;
};

// _cu_voxel_extract_depth_and_normal_map (:965-986): K (cu_geometry_functions.h:248-255),
// matrix33_mt, float33_inv (cu_vector_functions.h:555-575), float3_div_c
__device__ void ray_camera(const RayParams &p, RayCamera &c) {
    const float K[3][3] = {{p.fx, 0.0f, 0.0f}, {0.0f, p.fy, 0.0f}, {p.cx, p.cy, 1.0f}};
    float M[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            M[j][i] = K[0][i] * p.r[j] + K[1][i] * p.r[3 + j] + K[2][i] * p.r[6 + j];
    const float A = M[2][2] * M[1][1] - M[2][1] * M[1][2];
    const float B = M[0][2] * M[2][1] - M[0][1] * M[2][2];
    const float C = M[0][1] * M[1][2] - M[0][2] * M[1][1];
    const float det = M[0][0] * A + M[1][0] * B + M[2][0] * C;
    c.ok = !(det > -FLT_EPSILON && det < FLT_EPSILON);
    float I[3][3];
    I[0][0] = A;
    I[0][1] = B;
    I[0][2] = C;
    I[1][0] = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    I[1][1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
    I[1][2] = M[0][2] * M[1][0] - M[0][0] * M[1][2];
    I[2][0] = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    I[2][1] = M[0][1] * M[2][0] - M[0][0] * M[2][1];
    I[2][2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) c.IM[j][i] = I[j][i] / det;
#pragma unroll
    for (int i = 0; i < 3; ++i) c.cc[i] = p.t[i] / p.grid_s;
}

// d_voxel_extract_trilinear_interpolated_sdf (:551-657): samples in the order
// V000, V100, V010, V001, V101, V011, V110, V111; the first +-32766 met
// returns +-1; float_interpolation_trilinear (cu_math_functions.h:107-111)
__device__ __forceinline__ float trilinear_sdf(const short2 *__restrict__ vol, int nx, int ny, float px, float py,
                                               float pz) {
    const int ix = (int)px, iy = (int)py, iz = (int)pz;
    const float x = px - (float)ix, y = py - (float)iy, z = pz - (float)iz;
    const long long sx = 1, sy = nx, sz = (long long)nx * ny;
    const long long base = iz * sz + (long long)iy * sy + ix;
    const long long off[8] = {0, sx, sy, sz, sx + sz, sy + sz, sx + sy, sx + sy + sz};
    float s[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const short t = __ldg(&vol[base + off[k]].x);
        if (t == (short)kMaxTsdf) return 1.0f;
        if (t == (short)-kMaxTsdf) return -1.0f;
        s[k] = mcg_unpack_tsdf(t);
    }
    const float a = 1.0f - x, b = 1.0f - y, c = 1.0f - z;
    return s[0] * a * b * c + s[1] * x * b * c + s[2] * a * y * c + s[3] * a * b * z + s[4] * x * b * z +
           s[5] * a * y * z + s[6] * x * y * c + s[7] * x * y * z;
}

__global__ void __launch_bounds__(256) raycast_kernel(RayParams p) {
    __shared__ RayCamera cam;
    if (threadIdx.x == 0 && threadIdx.y == 0) ray_camera(p, cam);
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.w || y >= p.h || !cam.ok) return;
    const long long idx = (long long)y * p.w + x;
    p.depth[idx] = 0.0f;
    if (p.normal) {
        p.normal[3 * idx] = 0.0f;
        p.normal[3 * idx + 1] = 0.0f;
        p.normal[3 * idx + 2] = 0.0f;
    }
    const float margin = 1.0f;
    const float hi[3] = {(float)p.nx - margin, (float)p.ny - margin, (float)p.nz - margin};
    const float dt_max = 1.0f, dt_min = 0.25f;
    float dt = dt_max;
    bool dt_status = false;
    const float fx = (float)x, fy = (float)y;
    // float33_mv_2 (cu_vector_functions.h:623-626), then float3_unit
    float rd[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) rd[i] = cam.IM[0][i] * fx + cam.IM[1][i] * fy + cam.IM[2][i];
    {
        const float norm = sqrtf(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]);
        if (norm > FLT_EPSILON || norm < -FLT_EPSILON) {
#pragma unroll
            for (int i = 0; i < 3; ++i) rd[i] = rd[i] / norm;
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
        if (rd[i] == 0.0f) rd[i] = (float)1e-15;
    const float *cc = cam.cc;
    // entry and exit over the faces c = margin and c = c_max of each axis
    float t_min = FLT_MAX, t_max = 0.0f;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        const int a1 = ax == 0 ? 1 : 0, a2 = ax == 2 ? 1 : 2;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const float t = ((side == 0 ? margin : hi[ax]) - cc[ax]) / rd[ax];
            if (t > 0.0f) {
                const float u1 = rd[a1] * t + cc[a1];
                const float u2 = rd[a2] * t + cc[a2];
                if (u1 > margin && u1 < hi[a1] && u2 > margin && u2 < hi[a2]) {
                    if (t < t_min) t_min = t;
                    if (t > t_max) t_max = t;
                }
            }
        }
    }
    if (t_min == FLT_MAX && t_max == 0.0f) return;
    if (t_min == t_max) t_min = dt * margin;
    // the reference's march cannot run longer than this; the bound only guards
    // inputs (non-finite poses) on which it would not end
    const float span = t_max - t_min;
    const long long cap = span < 1.0e7f ? (long long)(span * 8.0f) + 4096 : 0;
    float t1 = 0.0f, sdf1 = 1.0f;
    long long steps = 0;
    for (float t = t_min; t < t_max && steps < cap; t += dt, ++steps) {
        const float px = rd[0] * t + cc[0], py = rd[1] * t + cc[1], pz = rd[2] * t + cc[2];
        if (px < 0.0f || py < 0.0f || pz < 0.0f || px >= hi[0] || py >= hi[1] || pz >= hi[2]) continue;
        const float sdf = trilinear_sdf(p.vol, p.nx, p.ny, px, py, pz);
        if (sdf < 0.0f && sdf > -1.0f && sdf1 >= 0.0f && sdf1 < 1.0f) {
            const float t2 = t1 - dt * sdf1 / (sdf - sdf1);  // eq. (15)
            const float n0 = rd[0] * t2, n1 = rd[1] * t2, n2 = rd[2] * t2;
            const float q0 = n0 + cc[0], q1 = n1 + cc[1], q2 = n2 + cc[2];
            // float_camera_intrinsic_unproject_2 (cu_geometry_functions.h:237-240)
            const float ux = (fx - p.cx) / p.fx, uy = (fy - p.cy) / p.fy;
            p.depth[idx] = sqrtf(n0 * n0 + n1 * n1 + n2 * n2) / sqrtf(ux * ux + uy * uy + 1.0f) * p.grid_s;
            if (p.normal) {
                // the surface normal at the hit (grid units), then float33_tv: R^T n
                const float3 sn = normal_global<MCG_VOXEL_SHORT2>(p.vol, p.nx, p.ny, p.nz, 1.0f, q0, q1, q2);
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    p.normal[3 * idx + i] = p.r[3 * i] * sn.x + p.r[3 * i + 1] * sn.y + p.r[3 * i + 2] * sn.z;
            }
            break;
        } else if (sdf1 <= 0.0f && sdf1 > -1.0f && sdf >= 0.0f && sdf < 1.0f) {
            break;  // back face
        }
        if (sdf > -1.0f && sdf < 1.0f) {
            if (!dt_status) {
                t -= dt;
                dt_status = true;
                dt = dt_min;
                continue;
            }
        } else if (dt_status) {
            dt_status = false;
            dt = dt_max;
        }
        t1 = t;
        sdf1 = sdf;
    }
}

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" mcg_status mcg_raycast(mcg_context *ctx, const void *vol, int32_t nx, int32_t ny, int32_t nz,
                                  float grid_s, const mcg_intrinsic *k, const mcg_extrinsic *e, int32_t w, int32_t h,
                                  float *depth, float *normal, mcg_stream_t stream) {
    if (!ctx || !vol || !k || !e || !depth || nx < 2 || ny < 2 || nz < 2 || w <= 0 || h <= 0) return MCG_ERR_INVALID_ARG;
    if (!(grid_s > 0.0f)) return MCG_ERR_INVALID_ARG;
    cudaError_t err = cudaSetDevice(ctx->device);
    if (err != cudaSuccess) return mcg_cuda_fail(ctx, err);
    RayParams p;
    p.vol = static_cast<const short2 *>(vol);
    p.nx = nx;
    p.ny = ny;
    p.nz = nz;
    p.grid_s = grid_s;
    p.fx = k->fx;
    p.fy = k->fy;
    p.cx = k->cx;
    p.cy = k->cy;
    for (int i = 0; i < 9; ++i) p.r[i] = e->r[i];
    for (int i = 0; i < 3; ++i) p.t[i] = e->t[i];
    p.w = w;
    p.h = h;
    p.depth = depth;
    p.normal = normal;
    const dim3 block(16, 16), grid((w + 15) / 16, (h + 15) / 16);
    raycast_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(p);
    err = cudaGetLastError();
    return err == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, err);
}
