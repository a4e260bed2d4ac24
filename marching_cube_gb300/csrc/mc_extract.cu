// Marching-cubes extraction on sm_103a.
//
// Replaces the reference pipeline (cu_marching_cubes_v1.cu):
//   getOccupiedVoxelsKernel (:97-206)   -> mc_classify_kernel
//   thrust::exclusive_scan   (:208-225) -> mc_scan_kernel
//   trianglesGeneratorKernel (:228-396) -> mc_generate_kernel (+ fused normals,
//                                          cu_kinect_fusion_v1.cu:3146-3242)
//
// Work is organised in bricks of 32x8x8 cubes.  Pass 1 reads the whole volume
// once (brick + 1-voxel halo staged in shared memory), counts triangles and
// occupied cubes per brick.  A single-CTA scan turns brick counts into 64-bit
// soup offsets and a list of active bricks in brick order.  Pass 2 revisits
// only active bricks (brick + halo of -1/+2 voxels for the side outputs and
// normals), re-derives cube indices, scans emitted vertices inside the brick
// and writes one soup vertex per thread through a per-warp shared-memory
// stage so every global store is a full coalesced line.
//
// Output order is deterministic: bricks in (bz, by, bx) order, cubes in
// (z, y, x) order inside a brick, then the table slot -- the reference's
// order is non-deterministic (one atomicAdd per warp, :145).
//
// Arithmetic follows the reference's expressions in IEEE binary32, source
// order, no contraction (the library is built with --fmad=false).
#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_tables.h"
#include "mcg_internal.h"

namespace mcg {
namespace {

constexpr int BX = 32, BY = 8, BZ = 8;
constexpr int BRICK_CUBES = BX * BY * BZ;  // 2048
constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
static_assert(BX == 32 && BY == WARPS, "thread (lane, warp) maps to cube (x, y)");

// generate tile: voxels [x0-1, x0+BX+2) etc.
constexpr int TX = BX + 3, TY = BY + 3, TZ = BZ + 3;
constexpr int TILE = TX * TY * TZ;
// classify tile: voxels [x0, x0+BX+1)
constexpr int CX1 = BX + 1, CY1 = BY + 1, CZ1 = BZ + 1;
constexpr int CTILE = CX1 * CY1 * CZ1;

// corner offsets (cu_marching_cubes_v1.cu:74-81) and edge corner pairs in
// vertex_interp argument order (:304-315)
// corner c: x = {0,1,1,0,0,1,1,0}, y = {0,0,1,1,0,0,1,1}, z = {0,0,0,0,1,1,1,1}
__device__ __forceinline__ int c_cx(int c) { return (c ^ (c >> 1)) & 1; }
__device__ __forceinline__ int c_cy(int c) { return (c >> 1) & 1; }
__device__ __forceinline__ int c_cz(int c) { return c >> 2; }
// edge e: first corner {0..7,0,1,2,3}, second {1,2,3,0,5,6,7,4,4,5,6,7}
__device__ __forceinline__ int c_ea(int e) { return e < 8 ? e : e - 8; }
__device__ __forceinline__ int c_eb(int e) { return e < 8 ? (e & 4) | ((e + 1) & 3) : e - 4; }
__constant__ signed char c_tri[256][16];
__constant__ unsigned char c_nverts[256];

// ---- voxel traits -----------------------------------------------------------
template <int VT>
struct Vox;

template <>
struct Vox<MCG_VOXEL_SHORT2> {
    using T = short2;  // {tsdf, w}: w is a ushort, only ==0 is tested
    static __device__ __forceinline__ T fill() { return make_short2(0, 0); }
    static __device__ __forceinline__ bool neg(T v) { return v.x < 0; }
    static __device__ __forceinline__ bool w0(T v) { return v.y == 0; }
    // d_unpack_tsdf (cu_kinect_fusion_v1.h:253-256)
    static __device__ __forceinline__ float f(T v) { return (float)v.x / (float)kMaxTsdf; }
    static __device__ __forceinline__ bool sentinel(T v) { return v.x == kMaxTsdf || v.x == -kMaxTsdf; }
    static __device__ __forceinline__ short tsdf(T v) { return v.x; }
    static __device__ __forceinline__ short wt(T v) { return v.y; }
};

template <>
struct Vox<MCG_VOXEL_FLOAT2> {
    using T = float2;
    static __device__ __forceinline__ T fill() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ bool neg(T v) { return v.x < 0.f; }
    static __device__ __forceinline__ bool w0(T v) { return v.y == 0.f; }
    static __device__ __forceinline__ float f(T v) { return v.x; }
    static __device__ __forceinline__ bool sentinel(T) { return false; }
    static __device__ __forceinline__ short tsdf(T) { return 0; }
    static __device__ __forceinline__ short wt(T) { return 0; }
};

__device__ __forceinline__ long long lin3(int nx, int ny, int x, int y, int z) {
    return ((long long)z * ny + y) * nx + x;
}

// ---- pass 1: classify ------------------------------------------------------
template <int VT>
__global__ void __launch_bounds__(THREADS)
    mc_classify_kernel(const typename Vox<VT>::T *__restrict__ vol, int nx, int ny, int nz,
                       int nbx, int nby, long long nbricks, uint32_t *__restrict__ brick_tris,
                       uint32_t *__restrict__ brick_occ) {
    using V = Vox<VT>;
    __shared__ unsigned char s_ntri[256];
    __shared__ unsigned char s_flag[CTILE];
    __shared__ unsigned int s_red[2][WARPS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // triangles per case; cases 0 and 255 emit nothing (:136)
    s_ntri[tid] = (tid == 0 || tid == 255) ? 0 : c_nverts[tid] / 3;

    for (long long b = blockIdx.x; b < nbricks; b += gridDim.x) {
        const int bx = (int)(b % nbx);
        const long long r = b / nbx;
        const int by = (int)(r % nby), bz = (int)(r / nby);
        const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;
        __syncthreads();  // s_flag reuse
        // flags: bit0 = tsdf < 0, bit1 = weight == 0 (outside volume counts as w == 0)
        for (int i = tid; i < CTILE; i += THREADS) {
            const int lx = i % CX1, t = i / CX1, ly = t % CY1, lz = t / CY1;
            const int gx = x0 + lx, gy = y0 + ly, gz = z0 + lz;
            unsigned char fl = 2;
            if (gx < nx && gy < ny && gz < nz) {
                const typename V::T v = vol[lin3(nx, ny, gx, gy, gz)];
                fl = (unsigned char)(V::neg(v) | (V::w0(v) << 1));
            }
            s_flag[i] = fl;
        }
        __syncthreads();
        unsigned int tri = 0, occ = 0;
        const int cx = lane, cy = warp;
        if (x0 + cx < nx - 1 && y0 + cy < ny - 1) {
            const unsigned char *p = s_flag + cy * CX1 + cx;
            // rolling pair of voxel planes along z
            unsigned int a0 = p[0], a1 = p[1], a2 = p[CX1 + 1], a3 = p[CX1];
            const int zend = min(BZ, nz - 1 - z0);
            for (int cz = 0; cz < zend; ++cz) {
                const unsigned char *q = p + (cz + 1) * (CX1 * CY1);
                const unsigned int b0 = q[0], b1 = q[1], b2 = q[CX1 + 1], b3 = q[CX1];
                const unsigned int any = a0 | a1 | a2 | a3 | b0 | b1 | b2 | b3;
                if (!(any & 2)) {
                    const unsigned int ci = (a0 & 1) | ((a1 & 1) << 1) | ((a2 & 1) << 2) |
                                            ((a3 & 1) << 3) | ((b0 & 1) << 4) | ((b1 & 1) << 5) |
                                            ((b2 & 1) << 6) | ((b3 & 1) << 7);
                    const unsigned int nt = s_ntri[ci];
                    tri += nt;
                    occ += nt > 0;
                }
                a0 = b0; a1 = b1; a2 = b2; a3 = b3;
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            tri += __shfl_xor_sync(0xffffffffu, tri, o);
            occ += __shfl_xor_sync(0xffffffffu, occ, o);
        }
        if (lane == 0) { s_red[0][warp] = tri; s_red[1][warp] = occ; }
        __syncthreads();
        if (tid == 0) {
            unsigned int t = 0, o = 0;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) { t += s_red[0][w]; o += s_red[1][w]; }
            brick_tris[b] = t;
            brick_occ[b] = o;
        }
    }
}

// ---- scan: brick counts -> soup offsets + active brick list ---------------------
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER = 8;

__global__ void __launch_bounds__(SCAN_THREADS)
    mc_scan_kernel(const uint32_t *__restrict__ brick_tris, const uint32_t *__restrict__ brick_occ,
                   long long nb, unsigned long long *__restrict__ brick_vofs,
                   uint32_t *__restrict__ active, MeshTotals *__restrict__ totals) {
    __shared__ unsigned long long s_wv[32];
    __shared__ unsigned int s_wa[32];
    __shared__ unsigned long long s_occ[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long carry_v = 0, occ_sum = 0;
    unsigned int carry_a = 0;
    for (long long base = 0; base < nb; base += (long long)SCAN_THREADS * SCAN_PER) {
        const long long i0 = base + (long long)tid * SCAN_PER;
        uint32_t t[SCAN_PER];
        unsigned long long lv = 0;
        unsigned int la = 0;
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) {
            const long long i = i0 + k;
            t[k] = i < nb ? brick_tris[i] : 0u;
            occ_sum += i < nb ? brick_occ[i] : 0u;
            lv += t[k];
            la += t[k] != 0;
        }
        // warp inclusive scans
        unsigned long long iv = lv;
        unsigned int ia = la;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long nv = __shfl_up_sync(0xffffffffu, iv, o);
            const unsigned int na = __shfl_up_sync(0xffffffffu, ia, o);
            if (lane >= o) { iv += nv; ia += na; }
        }
        if (lane == 31) { s_wv[warp] = iv; s_wa[warp] = ia; }
        __syncthreads();
        if (warp == 0) {
            unsigned long long wv = s_wv[lane];
            unsigned int wa = s_wa[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long nv = __shfl_up_sync(0xffffffffu, wv, o);
                const unsigned int na = __shfl_up_sync(0xffffffffu, wa, o);
                if (lane >= o) { wv += nv; wa += na; }
            }
            s_wv[lane] = wv;  // inclusive over warps
            s_wa[lane] = wa;
        }
        __syncthreads();
        unsigned long long ev = carry_v + (warp ? s_wv[warp - 1] : 0ull) + (iv - lv);
        unsigned int ea = carry_a + (warp ? s_wa[warp - 1] : 0u) + (ia - la);
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) {
            const long long i = i0 + k;
            if (i < nb) {
                brick_vofs[i] = 3ull * ev;
                if (t[k]) active[ea++] = (uint32_t)i;
            }
            ev += t[k];
        }
        carry_v += s_wv[31];
        carry_a += s_wa[31];
        __syncthreads();
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) occ_sum += __shfl_xor_sync(0xffffffffu, occ_sum, o);
    if (lane == 0) s_occ[warp] = occ_sum;
    __syncthreads();
    if (tid == 0) {
        unsigned long long o = 0;
        for (int w = 0; w < SCAN_THREADS / 32; ++w) o += s_occ[w];
        totals->occupied = o;
        totals->triangles = carry_v;
        totals->vertices = 3ull * carry_v;
        totals->active_bricks = carry_a;
        totals->pad = 0;
    }
}

// ---- normals (cu_kinect_fusion_v1.cu:3146-3225) -----------------------------------
// cu_math_functions.h:99-103
__device__ __forceinline__ float bilinear(float v0, float v1, float v2, float v3, float x, float y) {
    const float a = 1.0f - x, b = 1.0f - y;
    return v0 * a * b + v1 * x * b + v2 * a * y + v3 * x * y;
}

// s[] in the reference's sdfs[] slot order; t = fractional position
__device__ __forceinline__ float3 normal_from_samples(const float s[8], float tx, float ty, float tz) {
    float3 n;
    float s1 = bilinear(s[0], s[2], s[3], s[5], ty, tz);
    float s2 = bilinear(s[1], s[6], s[4], s[7], ty, tz);
    n.x = s2 - s1;
    s1 = bilinear(s[0], s[1], s[3], s[4], tx, tz);
    s2 = bilinear(s[2], s[6], s[5], s[7], tx, tz);
    n.y = s2 - s1;
    s1 = bilinear(s[0], s[1], s[2], s[6], tx, ty);
    s2 = bilinear(s[3], s[4], s[5], s[7], tx, ty);
    n.z = s2 - s1;
    // float3_unit (cu_vector_functions.h:258-264)
    const float norm = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    if (norm > 1.192092896e-07f || norm < -1.192092896e-07f) {
        n.x = n.x / norm;
        n.y = n.y / norm;
        n.z = n.z / norm;
    }
    return n;
}

// Sample order V000, V100, V110, V010, V001, V101, V111, V011 -> sdfs slot
// (0, 1, 6, 2, 3, 4, 7, 5); compile-time so the samples stay in registers
template <int K>
struct NSlot {
    static constexpr int v = K == 0 ? 0 : K == 1 ? 1 : K == 2 ? 6 : K == 3 ? 2 : K == 4 ? 3 : K == 5 ? 4 : K == 6 ? 7 : 5;
};
__device__ __forceinline__ void put_slot(float s[8], int k, float v) {
    switch (k) {
        case 0: s[NSlot<0>::v] = v; break;
        case 1: s[NSlot<1>::v] = v; break;
        case 2: s[NSlot<2>::v] = v; break;
        case 3: s[NSlot<3>::v] = v; break;
        case 4: s[NSlot<4>::v] = v; break;
        case 5: s[NSlot<5>::v] = v; break;
        case 6: s[NSlot<6>::v] = v; break;
        default: s[NSlot<7>::v] = v; break;
    }
}

// Normal at p through global memory, with the reference's linear addressing
// from the start of slice p_i.z; any sample outside [0, N) (the reference
// reads outside its allocation there) gives the zero normal.
template <int VT>
__device__ float3 normal_global(const typename Vox<VT>::T *__restrict__ vol, int nx, int ny, int nz,
                                float cell, float px, float py, float pz) {
    using V = Vox<VT>;
    const float fx = px / cell, fy = py / cell, fz = pz / cell;
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const long long xy = (long long)nx * ny, N = xy * nz;
    const long long base = (long long)iz * xy + (long long)iy * nx + ix;
    const long long off[8] = {0, 1, 1 + (long long)nx, nx, xy, xy + 1, xy + 1 + nx, xy + nx};
    float s[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const long long a = base + off[k];
        if (a < 0 || a >= N) return make_float3(0.f, 0.f, 0.f);
        const typename V::T v = vol[a];
        if (V::sentinel(v)) return make_float3(0.f, 0.f, 0.f);
        put_slot(s, k, V::f(v));
    }
    return normal_from_samples(s, fx - (float)ix, fy - (float)iy, fz - (float)iz);
}

// ---- pass 2: generate ------------------------------------------------------
struct GenParams {
    const void *vol;
    int nx, ny, nz;
    float cell;
    int nbx, nby;
    const uint32_t *active;
    const unsigned long long *brick_vofs;
    const MeshTotals *totals;
    mcg_vertex_voxel *soup;
    float *normals;
    int32_t *vi2vox;
    int16_t *ver_voxel;
    int64_t *tri_cube;
    long long cap;
};

template <int VT>
struct GenSmem {
    typename Vox<VT>::T tile[TILE];
    signed char tri[256][16];
    unsigned char nv[256];
    unsigned char ci[BRICK_CUBES];
    unsigned short off[BRICK_CUBES];
    unsigned int stage[WARPS][32 * 7];
    unsigned int wsum[BZ][WARPS];
    unsigned int total;
};

__device__ __forceinline__ int tidx(int lx, int ly, int lz) { return (lz * TY + ly) * TX + lx; }

template <int VT>
__global__ void __launch_bounds__(THREADS) mc_generate_kernel(GenParams p) {
    using V = Vox<VT>;
    using T = typename V::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GenSmem<VT> &S = *reinterpret_cast<GenSmem<VT> *>(smem_raw);
    const T *__restrict__ vol = static_cast<const T *>(p.vol);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const long long N = (long long)nx * ny * nz;
    const float cell = p.cell;

    for (int i = tid; i < 256 * 16; i += THREADS) (&S.tri[0][0])[i] = (&c_tri[0][0])[i];
    S.nv[tid] = (tid == 0 || tid == 255) ? 0 : c_nverts[tid];

    const unsigned int nactive = p.totals->active_bricks;
    for (unsigned int w = blockIdx.x; w < nactive; w += gridDim.x) {
        const long long b = p.active[w];
        const unsigned long long vbase = p.brick_vofs[b];
        const int bx = (int)(b % p.nbx);
        const long long r = b / p.nbx;
        const int by = (int)(r % p.nby), bz = (int)(r / p.nby);
        const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;
        __syncthreads();  // previous brick finished with the tile
        for (int i = tid; i < TILE; i += THREADS) {
            const int lx = i % TX, t = i / TX, ly = t % TY, lz = t / TY;
            const int gx = x0 - 1 + lx, gy = y0 - 1 + ly, gz = z0 - 1 + lz;
            T v = V::fill();
            if (gx >= 0 && gy >= 0 && gz >= 0 && gx < nx && gy < ny && gz < nz)
                v = vol[lin3(nx, ny, gx, gy, gz)];
            S.tile[i] = v;
        }
        __syncthreads();

        // classify the brick's cubes; thread (lane, warp) owns column (x, y)
        unsigned int nvs[BZ];
        const int cx = lane, cy = warp;
        const bool col_ok = (x0 + cx < nx - 1) && (y0 + cy < ny - 1);
#pragma unroll
        for (int cz = 0; cz < BZ; ++cz) {
            unsigned int ci = 0;
            if (col_ok && z0 + cz < nz - 1) {
                bool dead = false;
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const T v = S.tile[tidx(cx + 1 + c_cx(c), cy + 1 + c_cy(c), cz + 1 + c_cz(c))];
                    dead |= V::w0(v);
                    ci |= (unsigned int)V::neg(v) << c;
                }
                if (dead) ci = 0;
            }
            const int idx = (cz * BY + cy) * BX + cx;
            S.ci[idx] = (unsigned char)ci;
            nvs[cz] = S.nv[ci];
        }
        // exclusive scan in (z, y, x) order: warp scans per z-row, then rows x warps
        unsigned int incl[BZ];
#pragma unroll
        for (int cz = 0; cz < BZ; ++cz) {
            unsigned int x = nvs[cz];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            incl[cz] = x;
            if (lane == 31) S.wsum[cz][warp] = x;
        }
        __syncthreads();
        if (warp == 0) {
            // 64 (row, warp) sums in row-major order, 2 per lane
            const unsigned int a = (&S.wsum[0][0])[2 * lane], c = (&S.wsum[0][0])[2 * lane + 1];
            unsigned int x = a + c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            const unsigned int ex = x - a - c;
            (&S.wsum[0][0])[2 * lane] = ex;
            (&S.wsum[0][0])[2 * lane + 1] = ex + a;
            if (lane == 31) S.total = x;
        }
        __syncthreads();
#pragma unroll
        for (int cz = 0; cz < BZ; ++cz) {
            const int idx = (cz * BY + cy) * BX + cx;
            S.off[idx] = (unsigned short)(S.wsum[cz][warp] + incl[cz] - nvs[cz]);
        }
        __syncthreads();
        const unsigned int T_brick = S.total;

        // emission: one soup vertex per thread, warps take 32 consecutive vertices
        for (unsigned int v0 = warp * 32; v0 < T_brick; v0 += THREADS) {
            const unsigned int v = v0 + lane;
            const bool valid = v < T_brick;
            float P[3] = {0.f, 0.f, 0.f};
            int vox[3] = {0, 0, 0};
            short vt = 0, vw = 0;
            float3 nrm = make_float3(0.f, 0.f, 0.f);
            long long cube_lin = 0;
            int kslot = 1;
            if (valid) {
                // owning cube: last c with off[c] <= v
                int lo = 0, hi = BRICK_CUBES - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (S.off[mid] <= v) lo = mid; else hi = mid - 1;
                }
                const int c = lo;
                const int lcx = c & (BX - 1), lcy = (c / BX) & (BY - 1), lcz = c / (BX * BY);
                const unsigned int ci = S.ci[c];
                const unsigned int s = v - S.off[c];
                const unsigned int j = s / 3, k = s - 3 * j;
                kslot = (int)k;
                // output slot k of triangle j takes edge tri[3j+2-k] (:322-333)
                const int e = S.tri[ci][3 * j + 2 - k];
                const int a = c_ea(e), bb = c_eb(e);
                const int gx = x0 + lcx, gy = y0 + lcy, gz = z0 + lcz;
                cube_lin = lin3(nx, ny, gx, gy, gz);
                const float f0 = V::f(S.tile[tidx(lcx + 1 + c_cx(a), lcy + 1 + c_cy(a), lcz + 1 + c_cz(a))]);
                const float f1 = V::f(S.tile[tidx(lcx + 1 + c_cx(bb), lcy + 1 + c_cy(bb), lcz + 1 + c_cz(bb))]);
                // getNodeCoo (:243-254) and vertex_interp (:256-264)
                const float t = (0.0f - f0) / (f1 - f0 + 1e-15f);
                const int ga[3] = {gx + c_cx(a), gy + c_cy(a), gz + c_cz(a)};
                const int gb[3] = {gx + c_cx(bb), gy + c_cy(bb), gz + c_cz(bb)};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float p0 = ((float)ga[d] + 0.5f) * cell;
                    const float p1 = ((float)gb[d] + 0.5f) * cell;
                    P[d] = p0 + t * (p1 - p0);
                }
                // store_point (:336-367): voxel of the vertex, its tsdf / w
                const int dims[3] = {nx, ny, nz};
                const int org[3] = {x0 - 1, y0 - 1, z0 - 1};
                // tile path only when the voxel is inside the volume and the tile
                const int tdim[3] = {TX, TY, TZ};
                bool inside = true;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    vox[d] = (int)floorf(P[d] / cell - 0.5f);
                    inside &= vox[d] >= 0 && vox[d] < dims[d] && vox[d] - org[d] >= 0 && vox[d] - org[d] < tdim[d];
                }
                const long long li = lin3(nx, ny, vox[0], vox[1], vox[2]);
                if (inside) {
                    const T vv = S.tile[tidx(vox[0] - org[0], vox[1] - org[1], vox[2] - org[2])];
                    vt = V::tsdf(vv);
                    vw = V::wt(vv);
                } else if (li >= 0 && li < N) {
                    const T vv = vol[li];
                    vt = V::tsdf(vv);
                    vw = V::wt(vv);
                }
                if (p.ver_voxel && li >= 0 && li < N && vbase + v < (unsigned long long)p.cap)
                    p.ver_voxel[li] = vt;
                if (p.normals) {
                    const float fx = P[0] / cell, fy = P[1] / cell, fz = P[2] / cell;
                    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
                    const int lx = ix - org[0], ly = iy - org[1], lz = iz - org[2];
                    if (ix + 1 < nx && iy + 1 < ny && iz + 1 < nz && lx >= 0 && ly >= 0 && lz >= 0 &&
                        lx + 1 < TX && ly + 1 < TY && lz + 1 < TZ) {
                        const T smp[8] = {S.tile[tidx(lx, ly, lz)],         S.tile[tidx(lx + 1, ly, lz)],
                                          S.tile[tidx(lx + 1, ly + 1, lz)], S.tile[tidx(lx, ly + 1, lz)],
                                          S.tile[tidx(lx, ly, lz + 1)],     S.tile[tidx(lx + 1, ly, lz + 1)],
                                          S.tile[tidx(lx + 1, ly + 1, lz + 1)], S.tile[tidx(lx, ly + 1, lz + 1)]};
                        bool sent = false;
                        float sd[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            sent |= V::sentinel(smp[q]);
                            put_slot(sd, q, V::f(smp[q]));
                        }
                        if (!sent) nrm = normal_from_samples(sd, fx - (float)ix, fy - (float)iy, fz - (float)iz);
                    } else {
                        nrm = normal_global<VT>(vol, nx, ny, nz, cell, P[0], P[1], P[2]);
                    }
                }
            }
            // ---- coalesced stores through the warp stage ----
            const unsigned long long g0 = vbase + v0;  // first record of this warp
            const long long room = p.cap - (long long)g0;
            const int nrec = (int)min((long long)min(32u, T_brick - v0), room > 0 ? room : 0ll);
            unsigned int *st = S.stage[warp];
            if (p.soup) {
                st[lane * 7 + 0] = __float_as_uint(P[0]);
                st[lane * 7 + 1] = __float_as_uint(P[1]);
                st[lane * 7 + 2] = __float_as_uint(P[2]);
                st[lane * 7 + 3] = (unsigned int)vox[0];
                st[lane * 7 + 4] = (unsigned int)vox[1];
                st[lane * 7 + 5] = (unsigned int)vox[2];
                st[lane * 7 + 6] = (unsigned int)(unsigned short)vt | ((unsigned int)(unsigned short)vw << 16);
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(p.soup) + g0 * 7;
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 7) dst[word] = st[word];
                }
                __syncwarp();
            }
            if (p.normals) {
                st[lane * 3 + 0] = __float_as_uint(nrm.x);
                st[lane * 3 + 1] = __float_as_uint(nrm.y);
                st[lane * 3 + 2] = __float_as_uint(nrm.z);
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(p.normals) + g0 * 3;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 3) dst[word] = st[word];
                }
                __syncwarp();
            }
            if (p.vi2vox) {
                st[lane * 3 + 0] = (unsigned int)vox[0];
                st[lane * 3 + 1] = (unsigned int)vox[1];
                st[lane * 3 + 2] = (unsigned int)vox[2];
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(p.vi2vox) + g0 * 3;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 3) dst[word] = st[word];
                }
                __syncwarp();
            }
            // a triangle's cube id is written only when the whole triangle fits
            if (p.tri_cube && valid && kslot == 0 && (long long)(g0 + lane) + 2 < p.cap)
                p.tri_cube[(g0 + lane) / 3] = cube_lin;
        }
    }
}

// normals for arbitrary vertex records (d_voxel_extract_surface_normals)
template <int VT>
__global__ void mc_normals_kernel(const typename Vox<VT>::T *__restrict__ vol, int nx, int ny, int nz,
                                  float cell, const mcg_vertex_voxel *__restrict__ verts, long long n,
                                  float *__restrict__ normals) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const mcg_vertex_voxel r = verts[i];
    const float3 nn = normal_global<VT>(vol, nx, ny, nz, cell, r.x, r.y, r.z);
    normals[3 * i] = nn.x;
    normals[3 * i + 1] = nn.y;
    normals[3 * i + 2] = nn.z;
}

bool g_tables_ready[64] = {false};

cudaError_t upload_tables(int device) {
    if (device >= 0 && device < 64 && g_tables_ready[device]) return cudaSuccess;
    cudaError_t e = cudaMemcpyToSymbol(c_tri, mcg_tri_table, sizeof(mcg_tri_table));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_nverts, mcg_num_verts, sizeof(mcg_num_verts));
    if (e == cudaSuccess && device >= 0 && device < 64) g_tables_ready[device] = true;
    return e;
}

struct Geometry {
    int nbx, nby, nbz;
    long long nbricks;
};

Geometry geometry(int nx, int ny, int nz) {
    Geometry g;
    // cubes exist for x < nx-1 etc.
    g.nbx = (nx - 1 + BX - 1) / BX;
    g.nby = (ny - 1 + BY - 1) / BY;
    g.nbz = (nz - 1 + BZ - 1) / BZ;
    g.nbricks = (long long)g.nbx * g.nby * g.nbz;
    return g;
}

bool vol_ok(const mcg_volume *v) {
    if (!v || !v->data) return false;
    if (v->nx < 2 || v->ny < 2 || v->nz < 2) return false;
    if (v->voxel_type != MCG_VOXEL_SHORT2 && v->voxel_type != MCG_VOXEL_FLOAT2) return false;
    if (!(v->cell > 0.0f)) return false;
    // brick coordinates are 32-bit
    if ((long long)v->nx * v->ny * v->nz > (1ll << 40)) return false;
    return true;
}

template <int VT>
size_t gen_smem() { return sizeof(GenSmem<VT>); }

template <int VT>
int gen_grid(mcg_context *ctx, long long nbricks) {
    static int occ[2] = {0, 0};
    int &o = occ[VT];
    if (!o) {
        cudaFuncSetAttribute(mc_generate_kernel<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gen_smem<VT>());
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, mc_generate_kernel<VT>, THREADS,
                                                          gen_smem<VT>()) != cudaSuccess || o < 1)
            o = 1;
    }
    long long g = (long long)ctx->num_sms * o;
    if (g > nbricks) g = nbricks;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace mcg

using namespace mcg;

mcg_status mcg_mc_classify(mcg_context *ctx, const mcg_volume *vol, mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol)) return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = upload_tables(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const Geometry g = geometry(vol->nx, vol->ny, vol->nz);
    if (!ensure(&ctx->brick_tris, &ctx->brick_tris_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->brick_occ, &ctx->brick_occ_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->brick_vofs, &ctx->brick_vofs_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->active, &ctx->active_cap, (size_t)g.nbricks))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    long long grid = (long long)ctx->num_sms * 8;
    if (grid > g.nbricks) grid = g.nbricks;
    if (vol->voxel_type == MCG_VOXEL_SHORT2)
        mc_classify_kernel<MCG_VOXEL_SHORT2><<<(int)grid, THREADS, 0, s>>>(
            (const short2 *)vol->data, vol->nx, vol->ny, vol->nz, g.nbx, g.nby, g.nbricks,
            ctx->brick_tris, ctx->brick_occ);
    else
        mc_classify_kernel<MCG_VOXEL_FLOAT2><<<(int)grid, THREADS, 0, s>>>(
            (const float2 *)vol->data, vol->nx, vol->ny, vol->nz, g.nbx, g.nby, g.nbricks,
            ctx->brick_tris, ctx->brick_occ);
    mc_scan_kernel<<<1, SCAN_THREADS, 0, s>>>(ctx->brick_tris, ctx->brick_occ, g.nbricks,
                                              ctx->brick_vofs, ctx->active, ctx->d_totals);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->counts_ready, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    ctx->counts_pending = true;
    ctx->classified = true;
    ctx->cls_data = vol->data;
    ctx->cls_nx = vol->nx;
    ctx->cls_ny = vol->ny;
    ctx->cls_nz = vol->nz;
    ctx->cls_vtype = vol->voxel_type;
    ctx->last_capacity = -1;
    return MCG_OK;
}

mcg_status mcg_mc_counts(mcg_context *ctx, mcg_mesh_counts *out) {
    if (!ctx || !out) return MCG_ERR_INVALID_ARG;
    if (!ctx->classified) return MCG_ERR_STATE;
    if (ctx->counts_pending) {
        cudaError_t e = cudaEventSynchronize(ctx->counts_ready);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        ctx->counts_pending = false;
    }
    out->occupied = (int64_t)ctx->h_totals->occupied;
    out->triangles = (int64_t)ctx->h_totals->triangles;
    out->vertices = (int64_t)ctx->h_totals->vertices;
    out->active_bricks = (int64_t)ctx->h_totals->active_bricks;
    out->status = (ctx->last_capacity >= 0 && out->vertices > ctx->last_capacity) ? MCG_ERR_CAPACITY : MCG_OK;
    out->reserved = 0;
    return (mcg_status)out->status;
}

mcg_status mcg_mc_generate(mcg_context *ctx, const mcg_volume *vol, const mcg_mesh_out *out,
                           mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol) || !out || out->capacity_vertices < 0) return MCG_ERR_INVALID_ARG;
    if (!ctx->classified || ctx->cls_data != vol->data || ctx->cls_nx != vol->nx ||
        ctx->cls_ny != vol->ny || ctx->cls_nz != vol->nz || ctx->cls_vtype != vol->voxel_type)
        return MCG_ERR_STATE;
    if (out->capacity_vertices > 0 && !out->soup && !out->soup_normals && !out->vi2vox &&
        !out->ver_voxel && !out->tri_cube)
        return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const Geometry g = geometry(vol->nx, vol->ny, vol->nz);
    if (out->ver_voxel) {
        e = cudaMemsetAsync(out->ver_voxel, 0, sizeof(int16_t) * (size_t)vol->nx * vol->ny * vol->nz, s);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    }
    GenParams p;
    p.vol = vol->data;
    p.nx = vol->nx;
    p.ny = vol->ny;
    p.nz = vol->nz;
    p.cell = vol->cell;
    p.nbx = g.nbx;
    p.nby = g.nby;
    p.active = ctx->active;
    p.brick_vofs = ctx->brick_vofs;
    p.totals = ctx->d_totals;
    p.soup = out->soup;
    p.normals = out->soup_normals;
    p.vi2vox = out->vi2vox;
    p.ver_voxel = out->ver_voxel;
    p.tri_cube = out->tri_cube;
    p.cap = out->capacity_vertices;
    if (vol->voxel_type == MCG_VOXEL_SHORT2) {
        const int grid = gen_grid<MCG_VOXEL_SHORT2>(ctx, g.nbricks);
        mc_generate_kernel<MCG_VOXEL_SHORT2><<<grid, THREADS, gen_smem<MCG_VOXEL_SHORT2>(), s>>>(p);
    } else {
        const int grid = gen_grid<MCG_VOXEL_FLOAT2>(ctx, g.nbricks);
        mc_generate_kernel<MCG_VOXEL_FLOAT2><<<grid, THREADS, gen_smem<MCG_VOXEL_FLOAT2>(), s>>>(p);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(ctx->counts_ready, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    ctx->counts_pending = true;
    ctx->last_capacity = out->capacity_vertices;
    return MCG_OK;
}

mcg_status mcg_mc_extract(mcg_context *ctx, const mcg_volume *vol, const mcg_mesh_out *out,
                          mcg_stream_t stream) {
    mcg_status st = mcg_mc_classify(ctx, vol, stream);
    if (st != MCG_OK) return st;
    return mcg_mc_generate(ctx, vol, out, stream);
}

mcg_status mcg_mc_normals(mcg_context *ctx, const mcg_volume *vol, const mcg_vertex_voxel *verts,
                          int64_t n, float *normals, mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol) || n < 0 || (n > 0 && (!verts || !normals))) return MCG_ERR_INVALID_ARG;
    if (n == 0) return MCG_OK;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const int bs = 256;
    const long long grid = (n + bs - 1) / bs;
    if (vol->voxel_type == MCG_VOXEL_SHORT2)
        mc_normals_kernel<MCG_VOXEL_SHORT2><<<(unsigned int)grid, bs, 0, (cudaStream_t)stream>>>(
            (const short2 *)vol->data, vol->nx, vol->ny, vol->nz, vol->cell, verts, n, normals);
    else
        mc_normals_kernel<MCG_VOXEL_FLOAT2><<<(unsigned int)grid, bs, 0, (cudaStream_t)stream>>>(
            (const float2 *)vol->data, vol->nx, vol->ny, vol->nz, vol->cell, verts, n, normals);
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

// ---- extraction without any allocation ------------------------------------------
// For callers that cannot allocate device memory: the scratch of the three
// passes lives in one file-scope device array of fixed size, reserved when
// the library is loaded onto a device and held until the process exits.
namespace mcg {
namespace {

constexpr long long kNoAllocBricks = MCG_NOALLOC_MAX_BRICKS;
constexpr size_t kNoAllocTrisOff = 0;
constexpr size_t kNoAllocOccOff = kNoAllocTrisOff + sizeof(uint32_t) * kNoAllocBricks;
constexpr size_t kNoAllocVofsOff = kNoAllocOccOff + sizeof(uint32_t) * kNoAllocBricks;
constexpr size_t kNoAllocActiveOff = kNoAllocVofsOff + sizeof(unsigned long long) * kNoAllocBricks;
constexpr size_t kNoAllocTotalsOff = kNoAllocActiveOff + sizeof(uint32_t) * kNoAllocBricks;
constexpr size_t kNoAllocBytes = kNoAllocTotalsOff + 256;
static_assert(kNoAllocVofsOff % 8 == 0 && kNoAllocTotalsOff % 8 == 0, "scratch alignment");
static_assert(kNoAllocBytes == MCG_NOALLOC_SCRATCH_BYTES, "scratch size stated in mcg.h");

// brick counts, soup offsets, active-brick list and totals of one call
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// device address of g_noalloc_scratch per device, taken once with that device current
unsigned char *g_noalloc_addr[64] = {nullptr};

}  // namespace
}  // namespace mcg

extern "C" mcg_status mcg_mc_extract_noalloc(const mcg_volume *vol, const mcg_mesh_out *out,
                                             mcg_mesh_counts *counts, mcg_stream_t stream) {
    using namespace mcg;
    if (!vol_ok(vol) || !out || !counts || out->capacity_vertices < 0) return MCG_ERR_INVALID_ARG;
    const Geometry g = geometry(vol->nx, vol->ny, vol->nz);
    if (g.nbricks > kNoAllocBricks) return MCG_ERR_TOO_LARGE;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return MCG_ERR_CUDA;
    // set-up, once per device: the host-side symbol is only a stand-in, the
    // kernels need the device address of the array
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) { cudaGetLastError(); return MCG_ERR_CUDA; }
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    e = upload_tables(dev);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    unsigned char *base = g_noalloc_addr[dev];
    uint32_t *tris = reinterpret_cast<uint32_t *>(base + kNoAllocTrisOff);
    uint32_t *occ = reinterpret_cast<uint32_t *>(base + kNoAllocOccOff);
    unsigned long long *vofs = reinterpret_cast<unsigned long long *>(base + kNoAllocVofsOff);
    uint32_t *active = reinterpret_cast<uint32_t *>(base + kNoAllocActiveOff);
    MeshTotals *totals = reinterpret_cast<MeshTotals *>(base + kNoAllocTotalsOff);
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    cudaStream_t s = (cudaStream_t)stream;
    // every scratch entry read later is written first by these launches, so
    // nothing carried over from an earlier call is used
    long long cgrid = (long long)sms * 8;
    if (cgrid > g.nbricks) cgrid = g.nbricks;
    if (vol->voxel_type == MCG_VOXEL_SHORT2)
        mc_classify_kernel<MCG_VOXEL_SHORT2><<<(int)cgrid, THREADS, 0, s>>>(
            (const short2 *)vol->data, vol->nx, vol->ny, vol->nz, g.nbx, g.nby, g.nbricks, tris, occ);
    else
        mc_classify_kernel<MCG_VOXEL_FLOAT2><<<(int)cgrid, THREADS, 0, s>>>(
            (const float2 *)vol->data, vol->nx, vol->ny, vol->nz, g.nbx, g.nby, g.nbricks, tris, occ);
    mc_scan_kernel<<<1, SCAN_THREADS, 0, s>>>(tris, occ, g.nbricks, vofs, active, totals);
    if (out->ver_voxel) {
        e = cudaMemsetAsync(out->ver_voxel, 0, sizeof(int16_t) * (size_t)vol->nx * vol->ny * vol->nz, s);
        if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    }
    GenParams p;
    p.vol = vol->data;
    p.nx = vol->nx;
    p.ny = vol->ny;
    p.nz = vol->nz;
    p.cell = vol->cell;
    p.nbx = g.nbx;
    p.nby = g.nby;
    p.active = active;
    p.brick_vofs = vofs;
    p.totals = totals;
    p.soup = out->soup;
    p.normals = out->soup_normals;
    p.vi2vox = out->vi2vox;
    p.ver_voxel = out->ver_voxel;
    p.tri_cube = out->tri_cube;
    p.cap = out->capacity_vertices;
    int occb = 1;
    if (vol->voxel_type == MCG_VOXEL_SHORT2) {
        cudaFuncSetAttribute(mc_generate_kernel<MCG_VOXEL_SHORT2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gen_smem<MCG_VOXEL_SHORT2>());
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occb, mc_generate_kernel<MCG_VOXEL_SHORT2>, THREADS,
                                                          gen_smem<MCG_VOXEL_SHORT2>()) != cudaSuccess || occb < 1)
            occb = 1;
        long long grid = (long long)sms * occb;
        if (grid > g.nbricks) grid = g.nbricks;
        mc_generate_kernel<MCG_VOXEL_SHORT2><<<(int)grid, THREADS, gen_smem<MCG_VOXEL_SHORT2>(), s>>>(p);
    } else {
        cudaFuncSetAttribute(mc_generate_kernel<MCG_VOXEL_FLOAT2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gen_smem<MCG_VOXEL_FLOAT2>());
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occb, mc_generate_kernel<MCG_VOXEL_FLOAT2>, THREADS,
                                                          gen_smem<MCG_VOXEL_FLOAT2>()) != cudaSuccess || occb < 1)
            occb = 1;
        long long grid = (long long)sms * occb;
        if (grid > g.nbricks) grid = g.nbricks;
        mc_generate_kernel<MCG_VOXEL_FLOAT2><<<(int)grid, THREADS, gen_smem<MCG_VOXEL_FLOAT2>(), s>>>(p);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return MCG_ERR_CUDA;
    // counts: copy the totals out of the array into a host variable and wait
    MeshTotals t;
    e = cudaMemcpyAsync(&t, totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    counts->occupied = (int64_t)t.occupied;
    counts->triangles = (int64_t)t.triangles;
    counts->vertices = (int64_t)t.vertices;
    counts->active_bricks = (int64_t)t.active_bricks;
    counts->status = counts->vertices > out->capacity_vertices ? MCG_ERR_CAPACITY : MCG_OK;
    counts->reserved = 0;
    return (mcg_status)counts->status;
}
