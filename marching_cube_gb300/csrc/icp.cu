// Depth pyramid and projective point-to-plane ICP on sm_103a
// (cu_kinect_fusion_v1.cu:66-80, 226-261, 988-1301).
//
// The reference runs, per ICP iteration, a correspondence kernel, a kernel
// writing the 6 columns of A and b, then 27 pairs of nppsMul_32f +
// thrust::inclusive_scan for the normal equations, copies them to the host
// and solves there.  Here one iteration is two launches on the stream and
// no host round trip:
//   icp_reduce  per pixel: the correspondence (nearest pixel, step 1, or
//               bilinear, step 4), the row of A and b (step 2), the inlier
//               flag (step 3); the 27 products A_i A_j and A_i b are formed
//               in binary32 as nppsMul_32f forms them and summed in binary64
//               per CTA (fixed order);
//   icp_solve   one warp: the per-CTA sums in a fixed order, then Cholesky,
//               the determinant and 1-norm condition tests, the increment,
//               its bounds, exp([w]x) (Rodrigues), compose and the stopping
//               rule of kf.cu:1177-1262, and the loop state on the device.
// All it_max iterations are enqueued at once; once the loop has ended the
// remaining launches return at their first instruction.  The host reads the
// loop state once, after the last launch.  Per-pixel arithmetic is the
// reference's binary32 in source order (--fmad=false).
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "mcg_internal.h"

namespace mcg {
namespace {

constexpr int IC_THREADS = 256;

struct IcpState {
    float r[9], t[3];  // pose_rel: rotation column-major, translation
    double md;         // mahalanobis distance of the last step
    int it;            // iterations left (the reference's `it`)
    int rt;            // result so far
    int done;          // the loop has ended
    int iters;         // iterations run
};

struct IcpArgs {
    float nt, dt;
    float fx, fy, cx, cy;
    int w1, h1, w2, h2;
    const float3 *v1, *n1, *v2, *n2;
};

__device__ __forceinline__ bool ic_nz(float3 n) { return n.x != 0.0f || n.y != 0.0f || n.z != 0.0f; }
__device__ __forceinline__ float3 ic_rot(const float *r, float3 p) {  // float33_mv
    return make_float3(r[0] * p.x + r[3] * p.y + r[6] * p.z, r[1] * p.x + r[4] * p.y + r[7] * p.z,
                       r[2] * p.x + r[5] * p.y + r[8] * p.z);
}
__device__ __forceinline__ float3 ic_fwd(const float *r, const float *t, float3 p) {  // extrinsic_forward
    const float3 q = ic_rot(r, p);
    return make_float3(q.x + t[0], q.y + t[1], q.z + t[2]);
}
__device__ __forceinline__ float3 ic_bwd(const float *r, const float *t, float3 p) {  // extrinsic_backward
    const float dx = p.x - t[0], dy = p.y - t[1], dz = p.z - t[2];
    return make_float3(r[0] * dx + r[1] * dy + r[2] * dz, r[3] * dx + r[4] * dy + r[5] * dz,
                       r[6] * dx + r[7] * dy + r[8] * dz);
}
__device__ __forceinline__ float ic_dist(float3 a, float3 b) {  // float3_distance
    float d = a.x - b.x, s = d * d;
    d = a.y - b.y;
    s += d * d;
    d = a.z - b.z;
    s += d * d;
    return sqrtf(s);
}
__device__ __forceinline__ float3 ic_bilerp(const float3 *v, float x, float y) {  // vector3_interpolation_bilinear
    const float a = 1.0f - x, b = 1.0f - y;
    const float ab = a * b, xb = x * b, ay = a * y, xy = x * y;
    return make_float3(v[0].x * ab + v[1].x * xb + v[2].x * ay + v[3].x * xy,
                       v[0].y * ab + v[1].y * xb + v[2].y * ay + v[3].y * xy,
                       v[0].z * ab + v[1].z * xb + v[2].z * ay + v[3].z * xy);
}

// steps 1 / 4 for pixel idx of map 1: the transformed match in *out
template <bool BILINEAR>
__device__ __forceinline__ bool ic_match(const IcpArgs &a, const float *r, const float *t, long long idx,
                                         float3 *v1o, float3 *n1o, float3 *out) {
    const float3 p1 = a.v1[idx], m1 = a.n1[idx];
    *v1o = p1;
    *n1o = m1;
    if (!ic_nz(m1)) return false;
    const float3 p3 = ic_bwd(r, t, p1);
    const float px = a.fx * (p3.x / p3.z) + a.cx, py = a.fy * (p3.y / p3.z) + a.cy;
    if (!BILINEAR) {
        const int ix = __float2int_rn(px), iy = __float2int_rn(py);
        if (ix < 0 || iy < 0 || ix >= a.w2 || iy >= a.h2) return false;
        const long long j = (long long)iy * a.w2 + ix;
        float3 m2 = a.n2[j];
        if (!ic_nz(m2)) return false;
        m2 = ic_rot(r, m2);
        if (!(m1.x * m2.x + m1.y * m2.y + m1.z * m2.z > a.nt)) return false;
        const float3 p2 = ic_fwd(r, t, a.v2[j]);
        if (!(ic_dist(p1, p2) < a.dt)) return false;
        *out = p2;
        return true;
    } else {
        const int ix = (int)px, iy = (int)py;
        if (ix < 0 || iy < 0 || ix >= a.w2 - 1 || iy >= a.h2 - 1) return false;
        const long long j = (long long)iy * a.w2 + ix;
        float3 nn[4] = {a.n2[j], a.n2[j + 1], a.n2[j + a.w2], a.n2[j + a.w2 + 1]};
        if (!(ic_nz(nn[0]) && ic_nz(nn[1]) && ic_nz(nn[2]) && ic_nz(nn[3]))) return false;
        const float du = px - ix, dv = py - iy;
        const float3 m2 = ic_rot(r, ic_bilerp(nn, du, dv));
        if (!(m1.x * m2.x + m1.y * m2.y + m1.z * m2.z > a.nt)) return false;
        nn[0] = a.v2[j];
        nn[1] = a.v2[j + 1];
        nn[2] = a.v2[j + a.w2];
        nn[3] = a.v2[j + a.w2 + 1];
        const float3 p2 = ic_fwd(r, t, ic_bilerp(nn, du, dv));
        if (!(ic_dist(p1, p2) < a.dt)) return false;
        *out = p2;
        return true;
    }
}

// step 2: the row of A and b of a match
__device__ __forceinline__ void ic_row(float3 p1, float3 m1, float3 o, float A[6], float *b) {
    A[0] = m1.z * o.y - m1.y * o.z;
    A[1] = m1.x * o.z - m1.z * o.x;
    A[2] = m1.y * o.x - m1.x * o.y;
    A[3] = m1.x;
    A[4] = m1.y;
    A[5] = m1.z;
    *b = m1.x * p1.x + m1.y * p1.y + m1.z * p1.z - m1.x * o.x - m1.y * o.y - m1.z * o.z;
}

// one correspondence pass with all per-pixel outputs (for checking and for
// callers that want the rows): v21 (x = FLT_MAX and y = z = 0 when none),
// A column-major (n rows per column), b, inlier flags
template <bool BILINEAR>
__global__ void __launch_bounds__(IC_THREADS) icp_correspond_kernel(IcpArgs a, const float *__restrict__ pose,
                                                                    float3 *__restrict__ v21, float *__restrict__ A,
                                                                    float *__restrict__ bv, uint8_t *__restrict__ inl) {
    const long long n = (long long)a.w1 * a.h1;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        float3 p1, m1, o = make_float3(FLT_MAX, 0.0f, 0.0f);
        const bool found = ic_match<BILINEAR>(a, pose, pose + 9, idx, &p1, &m1, &o);
        if (v21) v21[idx] = found ? o : make_float3(FLT_MAX, 0.0f, 0.0f);
        if (inl) inl[idx] = found ? 0xff : 0;
        if (A) {
            float row[6] = {0, 0, 0, 0, 0, 0}, b = 0.0f;
            if (found) ic_row(p1, m1, o, row, &b);
#pragma unroll
            for (int c = 0; c < 6; ++c) A[c * n + idx] = row[c];
            bv[idx] = b;
        }
    }
}

// the 27 sums of one iteration: 21 of A_i A_j (i <= j, row-major upper
// triangle), 6 of A_i b
template <bool BILINEAR>
__global__ void __launch_bounds__(IC_THREADS) icp_reduce(IcpArgs a, const IcpState *__restrict__ st,
                                                         double *__restrict__ partial, uint8_t *__restrict__ inl) {
    __shared__ double s_red[IC_THREADS / 32][27];
    __shared__ float s_pose[12];
    if (st->done) return;
    if (threadIdx.x < 12) s_pose[threadIdx.x] = threadIdx.x < 9 ? st->r[threadIdx.x] : st->t[threadIdx.x - 9];
    __syncthreads();
    double acc[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) acc[k] = 0.0;
    const long long n = (long long)a.w1 * a.h1;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        float3 p1, m1, o;
        const bool found = ic_match<BILINEAR>(a, s_pose, s_pose + 9, idx, &p1, &m1, &o);
        if (inl) inl[idx] = found ? 0xff : 0;
        if (found) {
            float row[6], b;
            ic_row(p1, m1, o, row, &b);
            int k = 0;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
#pragma unroll
                for (int j = i; j < 6; ++j) acc[k++] += (double)(row[i] * row[j]);
            }
#pragma unroll
            for (int i = 0; i < 6; ++i) acc[21 + i] += (double)(row[i] * b);
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 27; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_down_sync(0xffffffffu, v, o2);
        if (lane == 0) s_red[wid][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 27) {
        double v = 0.0;
        for (int w = 0; w < IC_THREADS / 32; ++w) v += s_red[w][threadIdx.x];
        partial[(long long)blockIdx.x * 27 + threadIdx.x] = v;
    }
}

// Cholesky solve with the reference's tests; returns false to stop the loop
__device__ bool ic_solve(const double *ata21, const double *atb, double *x, double *md) {
    double M[6][6], L[6][6];
    int k = 0, count = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) M[i][j] = M[j][i] = ata21[k++];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < i; ++j)
            if (M[i][j] != 0.0) ++count;
    if (count == 0) return false;  // empty
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) L[i][j] = 0.0;
    for (int j = 0; j < 6; ++j) {
        double d = M[j][j];
        for (int p = 0; p < j; ++p) d -= L[j][p] * L[j][p];
        if (!(d > 0.0)) return false;  // not positive definite
        L[j][j] = sqrt(d);
        for (int i = j + 1; i < 6; ++i) {
            double s = M[i][j];
            for (int p = 0; p < j; ++p) s -= L[i][p] * L[j][p];
            L[i][j] = s / L[j][j];
        }
    }
    double det = 1.0;
    for (int i = 0; i < 6; ++i) det *= L[i][i] * L[i][i];
    if (!(fabs(det) > 1e-15)) return false;  // null space
    double anorm = 0.0, inorm = 0.0;
    for (int j = 0; j < 6; ++j) {
        double c = 0.0;
        for (int i = 0; i < 6; ++i) c += fabs(M[i][j]);
        anorm = c > anorm ? c : anorm;
    }
    for (int j = 0; j < 6; ++j) {  // column j of the inverse
        double y[6], z[6];
        for (int i = 0; i < 6; ++i) {
            double s = i == j ? 1.0 : 0.0;
            for (int p = 0; p < i; ++p) s -= L[i][p] * y[p];
            y[i] = s / L[i][i];
        }
        for (int i = 5; i >= 0; --i) {
            double s = y[i];
            for (int p = i + 1; p < 6; ++p) s -= L[p][i] * z[p];
            z[i] = s / L[i][i];
        }
        double c = 0.0;
        for (int i = 0; i < 6; ++i) c += fabs(z[i]);
        inorm = c > inorm ? c : inorm;
    }
    if (!(1.0 / (anorm * inorm) > 5e-5)) return false;  // ill-conditioned
    double y[6];
    for (int i = 0; i < 6; ++i) {
        double s = atb[i];
        for (int p = 0; p < i; ++p) s -= L[i][p] * y[p];
        y[i] = s / L[i][i];
    }
    for (int i = 5; i >= 0; --i) {
        double s = y[i];
        for (int p = i + 1; p < 6; ++p) s -= L[p][i] * x[p];
        x[i] = s / L[i][i];
    }
    double m = 0.0;
    for (int i = 0; i < 6; ++i) m += atb[i] * x[i];
    *md = m;
    return true;
}

__global__ void icp_solve(IcpState *__restrict__ st, const double *__restrict__ partial, int nblocks, float rtb,
                          float ttb) {
    __shared__ double s_sum[27];
    if (st->done) return;
    if (threadIdx.x < 27) {
        double v = 0.0;
        for (int b = 0; b < nblocks; ++b) v += partial[(long long)b * 27 + threadIdx.x];
        s_sum[threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    st->iters += 1;
    double x[6], md = 0.0;
    bool rt = ic_solve(s_sum, s_sum + 21, x, &md);
    if (rt) {
        if (fabs(x[0]) > rtb || fabs(x[1]) > rtb || fabs(x[2]) > rtb || fabs(x[3]) > ttb || fabs(x[4]) > ttb ||
            fabs(x[5]) > ttb) {
            rt = false;  // out of bound
        } else {
            // exp([w]x) by Rodrigues' formula, column-major
            const double th2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2], th = sqrt(th2);
            const double ca = th < 1e-12 ? 1.0 : sin(th) / th, cb = th < 1e-12 ? 0.5 : (1.0 - cos(th)) / th2;
            const double K[3][3] = {{0.0, -x[2], x[1]}, {x[2], 0.0, -x[0]}, {-x[1], x[0], 0.0}};
            float ri[9];
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    double kk = 0.0;
                    for (int p = 0; p < 3; ++p) kk += K[r][p] * K[p][c];
                    ri[3 * c + r] = (float)((r == c ? 1.0 : 0.0) + ca * K[r][c] + cb * kk);
                }
            const float ti[3] = {(float)x[3], (float)x[4], (float)x[5]};
            // float_camera_extrinsic_compose(pose, inc): R = Ri R, t = Ri t + ti (binary32)
            float nr[9], nt[3];
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r)
                    nr[3 * c + r] = ri[r] * st->r[3 * c] + ri[3 + r] * st->r[3 * c + 1] + ri[6 + r] * st->r[3 * c + 2];
            for (int r = 0; r < 3; ++r) nt[r] = ri[r] * st->t[0] + ri[3 + r] * st->t[1] + ri[6 + r] * st->t[2];
            for (int r = 0; r < 3; ++r) nt[r] = nt[r] + ti[r];
            for (int i = 0; i < 9; ++i) st->r[i] = nr[i];
            for (int i = 0; i < 3; ++i) st->t[i] = nt[i];
            if (md > st->md || md < 1e-5) st->it = 1;
            st->md = md;
        }
    }
    st->rt = rt ? 1 : 0;
    st->it -= 1;
    if (st->it == 0 || !rt) st->done = 1;
}

// kf.cu:226-261
__global__ void pyramid_down_kernel(int sw, int sh, int dw, int dh, const float *__restrict__ s,
                                    const uint8_t *__restrict__ sm, float *__restrict__ d, uint8_t *__restrict__ dm,
                                    float sigma) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    const int D = 5, H = D >> 1;
    int si = (y << 1) * sw + (x << 1);
    const int di = y * dw + x;
    dm[di] = 0;
    if (!sm[si]) return;
    const float center = s[si];
    const int tx = min((x << 1) - H + D, sw - 1), ty = min((y << 1) - H + D, sh - 1);
    float sum = 0.0f;
    int count = 0;
    for (int cy = max(0, (y << 1) - H); cy < ty; ++cy)
        for (int cx = max(0, (x << 1) - H); cx < tx; ++cx) {
            si = cy * sw + cx;
            if (sm[si]) {
                const float val = s[si];
                if (fabsf(val - center) < sigma) {
                    sum += val;
                    ++count;
                }
            }
        }
    if (count) {
        d[di] = sum / count;
        dm[di] = 0xff;
    }
}

// kf.cu:66-72 (to_mask = 1), 74-80 (to_mask = 0)
__global__ void mask_kernel(long long n, int to_mask, float *__restrict__ data, uint8_t *__restrict__ mask) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (to_mask)
            mask[i] = data[i] != 0.0f ? 0xff : 0;
        else if (mask[i] == 0)
            data[i] = 0.0f;
    }
}

IcpArgs make_args(const mcg_icp_params *p, const mcg_intrinsic *k, int w1, int h1, int w2, int h2, const float *v1,
                  const float *n1, const float *v2, const float *n2) {
    IcpArgs a;
    a.nt = p->nt;
    a.dt = p->dt;
    a.fx = k->fx;
    a.fy = k->fy;
    a.cx = k->cx;
    a.cy = k->cy;
    a.w1 = w1;
    a.h1 = h1;
    a.w2 = w2;
    a.h2 = h2;
    a.v1 = reinterpret_cast<const float3 *>(v1);
    a.n1 = reinterpret_cast<const float3 *>(n1);
    a.v2 = reinterpret_cast<const float3 *>(v2);
    a.n2 = reinterpret_cast<const float3 *>(n2);
    return a;
}

bool icp_args_ok(const mcg_icp_params *p, const mcg_intrinsic *k, int w1, int h1, int w2, int h2, const void *v1,
                 const void *n1, const void *v2, const void *n2) {
    return p && k && v1 && n1 && v2 && n2 && w1 > 0 && h1 > 0 && w2 > 0 && h2 > 0 && p->it_max > 0;
}

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" mcg_status mcg_pyramid_down(mcg_context *ctx, int32_t sw, int32_t sh, int32_t dw, int32_t dh,
                                       const float *src, const uint8_t *src_mask, float *dst, uint8_t *dst_mask,
                                       float sigma, mcg_stream_t stream) {
    if (!ctx || !src || !src_mask || !dst || !dst_mask || sw <= 0 || sh <= 0 || dw <= 0 || dh <= 0 ||
        2 * (dw - 1) >= sw || 2 * (dh - 1) >= sh)
        return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const dim3 block(16, 16), grid((dw + 15) / 16, (dh + 15) / 16);
    pyramid_down_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(sw, sh, dw, dh, src, src_mask, dst, dst_mask, sigma);
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

extern "C" mcg_status mcg_depth_mask(mcg_context *ctx, int64_t n, float *data, uint8_t *mask, int32_t to_mask,
                                     mcg_stream_t stream) {
    if (!ctx || !data || !mask || n < 0) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    if (n == 0) return MCG_OK;
    const int blocks = (int)std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * 8);
    mask_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(n, to_mask ? 1 : 0, data, mask);
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

extern "C" mcg_status mcg_icp_correspond(mcg_context *ctx, const mcg_icp_params *p, const mcg_intrinsic *k2,
                                         const mcg_extrinsic *pose_rel, int32_t w1, int32_t h1, int32_t w2, int32_t h2,
                                         const float *v1, const float *n1, const float *v2, const float *n2,
                                         float *v21, float *A, float *b, uint8_t *inlier, mcg_stream_t stream) {
    if (!ctx || !pose_rel || !icp_args_ok(p, k2, w1, h1, w2, h2, v1, n1, v2, n2) || (A && !b) || (!A && b))
        return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const cudaStream_t s = (cudaStream_t)stream;
    if (!ensure(&ctx->icp_pose, &ctx->icp_pose_cap, 12)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    float hp[12];
    for (int i = 0; i < 9; ++i) hp[i] = pose_rel->r[i];
    for (int i = 0; i < 3; ++i) hp[9 + i] = pose_rel->t[i];
    if ((e = cudaMemcpyAsync(ctx->icp_pose, hp, sizeof(hp), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    const IcpArgs a = make_args(p, k2, w1, h1, w2, h2, v1, n1, v2, n2);
    const long long n = (long long)w1 * h1;
    const int blocks = (int)std::min<long long>((n + IC_THREADS - 1) / IC_THREADS, (long long)ctx->num_sms * 8);
    if (p->bilinear)
        icp_correspond_kernel<true><<<blocks, IC_THREADS, 0, s>>>(a, ctx->icp_pose, reinterpret_cast<float3 *>(v21), A,
                                                                   b, inlier);
    else
        icp_correspond_kernel<false><<<blocks, IC_THREADS, 0, s>>>(a, ctx->icp_pose, reinterpret_cast<float3 *>(v21),
                                                                    A, b, inlier);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)  // hp is on the stack
        return mcg_cuda_fail(ctx, e);
    return MCG_OK;
}

extern "C" mcg_status mcg_icp(mcg_context *ctx, const mcg_icp_params *p, const mcg_intrinsic *k2,
                              mcg_extrinsic *pose_rel, int32_t w1, int32_t h1, int32_t w2, int32_t h2, const float *v1,
                              const float *n1, const float *v2, const float *n2, uint8_t *inlier, int32_t *ok,
                              int32_t *iterations, mcg_stream_t stream) {
    if (!ctx || !pose_rel || !ok || !icp_args_ok(p, k2, w1, h1, w2, h2, v1, n1, v2, n2)) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const cudaStream_t s = (cudaStream_t)stream;
    const int nblocks = ctx->num_sms * 2;
    if (!ensure(&ctx->icp_state, &ctx->icp_state_cap, sizeof(IcpState)) ||
        !ensure(&ctx->icp_partial, &ctx->icp_partial_cap, (size_t)nblocks * 27))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    if (!ctx->h_icp_state && cudaMallocHost((void **)&ctx->h_icp_state, sizeof(IcpState)) != cudaSuccess) {
        ctx->h_icp_state = nullptr;
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    }
    IcpState *hs = reinterpret_cast<IcpState *>(ctx->h_icp_state);
    IcpState *ds = reinterpret_cast<IcpState *>(ctx->icp_state);
    for (int i = 0; i < 9; ++i) hs->r[i] = pose_rel->r[i];
    for (int i = 0; i < 3; ++i) hs->t[i] = pose_rel->t[i];
    hs->md = (double)FLT_MAX;
    hs->it = p->it_max;
    hs->rt = 1;
    hs->done = 0;
    hs->iters = 0;
    if ((e = cudaMemcpyAsync(ds, hs, sizeof(IcpState), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    // the flags of every pass go to scratch; the caller's map receives the
    // last pass's flags only when the loop succeeds (kf.cu:1285-1292)
    const long long npx = (long long)w1 * h1;
    uint8_t *flags = nullptr;
    if (inlier) {
        if (!ensure(&ctx->icp_inlier, &ctx->icp_inlier_cap, (size_t)npx))
            return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        flags = ctx->icp_inlier;
    }
    const IcpArgs a = make_args(p, k2, w1, h1, w2, h2, v1, n1, v2, n2);
    for (int it = 0; it < p->it_max; ++it) {
        if (p->bilinear)
            icp_reduce<true><<<nblocks, IC_THREADS, 0, s>>>(a, ds, ctx->icp_partial, flags);
        else
            icp_reduce<false><<<nblocks, IC_THREADS, 0, s>>>(a, ds, ctx->icp_partial, flags);
        icp_solve<<<1, 32, 0, s>>>(ds, ctx->icp_partial, nblocks, p->rt, p->tt);
    }
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(hs, ds, sizeof(IcpState), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    *ok = hs->rt;
    if (iterations) *iterations = hs->iters;
    if (hs->rt) {
        for (int i = 0; i < 9; ++i) pose_rel->r[i] = hs->r[i];
        for (int i = 0; i < 3; ++i) pose_rel->t[i] = hs->t[i];
        if (inlier && (e = cudaMemcpyAsync(inlier, flags, (size_t)npx, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return mcg_cuda_fail(ctx, e);
    }
    return MCG_OK;
}
