// Device and host helpers shared by the marching-cubes translation units
// (mc_extract.cu: soup extraction and its adjoint; mc_indexed.cu: indexed
// extraction).  Everything is in an anonymous namespace, so each unit has its
// own copy of the device tables and uploads them itself.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MCG_TABLES_DEVICE  // the tables also as device data initialised with the module
#include "mc_tables.h"
#include "mcg_internal.h"
#include "tma.cuh"
#include "unpack.h"

namespace mcg {
namespace {

// bricks of 32x8x8 cubes
constexpr int BX = 32, BY = 8, BZ = 8;
constexpr int BRICK_CUBES = BX * BY * BZ;  // 2048
constexpr int CHUNK = 256;                 // bricks per scan chunk
// per-chunk sums written by the count pass: triangles, active bricks,
// occupied cubes, then heavy bricks by class.  A brick is heavy when it has
// more than HEAVY_TRIS triangles (more than one pass of a 256-thread CTA over
// its soup vertices); class k holds the bricks with more than
// HEAVY_TRIS << (NHEAVY - 1 - k) triangles not in a lower class, so class 0
// is the heaviest.  The active list holds the classes in order, then the
// light bricks: the longest bricks start first and the tail stays short.
constexpr int NHEAVY = 4;
constexpr int CHUNK_FIELDS = 3 + NHEAVY;
constexpr unsigned int HEAVY_TRIS = 85;
__host__ __device__ __forceinline__ int heavy_class(unsigned int t) {
    for (int k = 0; k < NHEAVY; ++k)
        if (t > (HEAVY_TRIS << (NHEAVY - 1 - k))) return k;
    return -1;
}

__host__ __device__ constexpr int pad128(int bytes) { return (bytes + 127) / 128 * 128; }

// corner c: x = {0,1,1,0,0,1,1,0}, y = {0,0,1,1,0,0,1,1}, z = {0,0,0,0,1,1,1,1}
// (corner order of cu_marching_cubes_v1.cu:74-81)
__device__ __forceinline__ int c_cx(int c) { return (c ^ (c >> 1)) & 1; }
__device__ __forceinline__ int c_cy(int c) { return (c >> 1) & 1; }
__device__ __forceinline__ int c_cz(int c) { return c >> 2; }
// edge e: first corner {0..7,0,1,2,3}, second {1,2,3,0,5,6,7,4,4,5,6,7}
// (vertex_interp argument order, :304-315)
__device__ __forceinline__ int c_ea(int e) { return e < 8 ? e : e - 8; }
__device__ __forceinline__ int c_eb(int e) { return e < 8 ? (e & 4) | ((e + 1) & 3) : e - 4; }
// The triangle table and the vertex count of each cube case are global
// memory initialised with the module (mcg_tri_table_dev, mcg_num_verts_dev
// in mc_tables.h), so nothing is uploaded and a device reset reloads them.
// Kernels copy them into shared memory at start: the triangle table with one
// 16-byte load per thread (from constant memory the lanes of a load that
// read different words are served one after another, which made that copy
// take most of a short kernel's time).
#define g_tri mcg_tri_table_dev
#define g_nverts mcg_num_verts_dev

// dst[256][16] (16-byte aligned shared memory) <- g_tri, by threads tid of nt
__device__ __forceinline__ void load_tri_table(signed char (*dst)[16], int tid, int nt) {
    const uint4 *src = reinterpret_cast<const uint4 *>(&g_tri[0][0]);
    uint4 *d = reinterpret_cast<uint4 *>(&dst[0][0]);
    for (int i = tid; i < 256; i += nt) d[i] = src[i];
}

// ---- voxel traits -----------------------------------------------------------
template <int VT>
struct Vox;

template <>
struct Vox<MCG_VOXEL_SHORT2> {
    using T = short2;  // {tsdf, w}: w is a ushort, only ==0 is tested
    static constexpr int bytes = 4;
    static __device__ __forceinline__ T fill() { return make_short2(0, 0); }
    static __device__ __forceinline__ bool neg(T v) { return v.x < 0; }
    static __device__ __forceinline__ bool w0(T v) { return v.y == 0; }
    // d_unpack_tsdf (cu_kinect_fusion_v1.h:253-256), division-free and exact
    static __device__ __forceinline__ float f(T v) { return mcg_unpack_tsdf(v.x); }
    static __device__ __forceinline__ bool sentinel(T v) { return v.x == kMaxTsdf || v.x == -kMaxTsdf; }
    static __device__ __forceinline__ short tsdf(T v) { return v.x; }
    static __device__ __forceinline__ short wt(T v) { return v.y; }
};

template <>
struct Vox<MCG_VOXEL_FLOAT2> {
    using T = float2;
    static constexpr int bytes = 8;
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

struct BrickPos {
    int x0, y0, z0;
};

__device__ __forceinline__ BrickPos brick_pos(long long b, int nbx, int nby) {
    BrickPos p;
    const long long r = b / nbx;
    p.x0 = (int)(b % nbx) * BX;
    p.y0 = (int)(r % nby) * BY;
    p.z0 = (int)(r / nby) * BZ;
    return p;
}

// brick b of a slab whose first brick layer starts at voxel z = zbase
__device__ __forceinline__ BrickPos slab_pos(long long b, int nbx, int nby, int zbase) {
    BrickPos p = brick_pos(b, nbx, nby);
    p.z0 += zbase;
    return p;
}

// Fill of a (DX, DY, DZ) tile whose origin is (ox, oy, oz) for volumes TMA
// cannot describe (rows not a multiple of 16 bytes, or a misaligned base),
// zero outside the volume like the TMA fill.  Each thread writes whole
// 16-byte words of tile rows: the voxels of a tile word lie in at most two
// aligned 16-byte words of the volume, which are loaded whole and shifted
// into place; the volume's first and last words, partly outside its
// allocation, are read voxel by voxel.  Rows outside the volume and voxels
// with x outside [0, nx) are zero.  The stores are plain shared-memory
// stores (WAIT is kept for the callers' cp.async bookkeeping); the caller's
// barrier publishes the tile.
template <int VT>
__device__ __forceinline__ uint4 vol_word(const uint4 *__restrict__ gbase, const typename Vox<VT>::T *__restrict__ vol,
                                          long long k, long long klo, long long khi, int b0, long long N) {
    constexpr int B = Vox<VT>::bytes, VPW = 16 / B;
    if (k >= klo && k <= khi) return __ldg(gbase + k);
    // partly (or wholly) outside the volume: voxel by voxel
    unsigned int u[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int j = 0; j < VPW; ++j) {
        const long long L = k * VPW + j - b0;
        if (L >= 0 && L < N) {
            const unsigned int *src = reinterpret_cast<const unsigned int *>(vol + L);
#pragma unroll
            for (int q = 0; q < B / 4; ++q) u[j * (B / 4) + q] = src[q];
        }
    }
    return make_uint4(u[0], u[1], u[2], u[3]);
}

template <int VT, int DX, int DY, int DZ, bool WAIT = true>
__device__ __forceinline__ void fill_tile(typename Vox<VT>::T *tile, const typename Vox<VT>::T *__restrict__ vol,
                                          int nx, int ny, int nz, int ox, int oy, int oz) {
    constexpr int B = Vox<VT>::bytes, VPW = 16 / B, WPR = DX / VPW, NWORDS = WPR * DY * DZ, UPV = B / 4;
    static_assert(DX % VPW == 0, "tile rows hold whole 16-byte words");
    const long long N = (long long)nx * ny * nz;
    // voxel offsets below are counted from the 16-byte boundary at or below vol
    const int b0 = (int)((reinterpret_cast<uintptr_t>(vol) & 15u) / B);
    const uint4 *gbase = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(vol) & ~(uintptr_t)15);
    const long long klo = b0 > 0 ? 1 : 0, khi = (b0 + N) / VPW - 1;  // words wholly inside the volume
    uint4 *dst = reinterpret_cast<uint4 *>(tile);
    for (int i = threadIdx.x; i < NWORDS; i += blockDim.x) {
        const int w = i % WPR, r = i / WPR, ly = r % DY, lz = r / DY;
        const int gy = oy + ly, gz = oz + lz, gx0 = ox + w * VPW;
        uint4 out = make_uint4(0u, 0u, 0u, 0u);
        if (gy >= 0 && gy < ny && gz >= 0 && gz < nz && gx0 + VPW > 0 && gx0 < nx) {
            const long long A = ((long long)gz * ny + gy) * nx + gx0 + b0;
            const long long k0 = A >> (VPW == 4 ? 2 : 1);  // floor, also below the base
            const int m = (int)(A & (VPW - 1));
            const uint4 a = vol_word<VT>(gbase, vol, k0, klo, khi, b0, N);
            const uint4 c = m ? vol_word<VT>(gbase, vol, k0 + 1, klo, khi, b0, N) : make_uint4(0u, 0u, 0u, 0u);
            // the 4 words starting at word m * UPV of the window (a, c)
            switch (m * UPV) {
                case 0: out = a; break;
                case 1: out = make_uint4(a.y, a.z, a.w, c.x); break;
                case 2: out = make_uint4(a.z, a.w, c.x, c.y); break;
                default: out = make_uint4(a.w, c.x, c.y, c.z); break;
            }
            if (gx0 < 0 || gx0 + VPW > nx) {
                unsigned int u[4] = {out.x, out.y, out.z, out.w};
#pragma unroll
                for (int j = 0; j < VPW; ++j)
                    if (gx0 + j < 0 || gx0 + j >= nx) {
#pragma unroll
                        for (int q = 0; q < UPV; ++q) u[j * UPV + q] = 0u;
                    }
                out = make_uint4(u[0], u[1], u[2], u[3]);
            }
        }
        dst[i] = out;
    }
    (void)WAIT;
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

// Sign masks of the four voxel rows around one cube row and the occupied
// cubes of that row (bit x).
struct CubeRow {
    unsigned long long a, b, c, d;  // neg masks of rows (y,z), (y+1,z), (y,z+1), (y+1,z+1)
    unsigned int occ;
};

// ---- host helpers -------------------------------------------------------------
struct Geometry {
    int nbx, nby, nbz;
    long long nbricks;
    int zbase, zlim;  // brick layer 0 starts at voxel z = zbase; cubes exist for z < zlim
};

Geometry geometry(int nx, int ny, int nz) {
    Geometry g;
    // cubes exist for x < nx-1 etc.
    g.nbx = (nx - 1 + BX - 1) / BX;
    g.nby = (ny - 1 + BY - 1) / BY;
    g.nbz = (nz - 1 + BZ - 1) / BZ;
    g.nbricks = (long long)g.nbx * g.nby * g.nbz;
    g.zbase = 0;
    g.zlim = nz - 1;
    return g;
}

// the cubes with z0 <= z < z1 (z0 a multiple of the brick depth)
Geometry geometry_slab(int nx, int ny, int z0, int z1) {
    Geometry g;
    g.nbx = (nx - 1 + BX - 1) / BX;
    g.nby = (ny - 1 + BY - 1) / BY;
    g.nbz = (z1 - z0 + BZ - 1) / BZ;
    g.nbricks = (long long)g.nbx * g.nby * g.nbz;
    g.zbase = z0;
    g.zlim = z1;
    return g;
}

bool vol_ok(const mcg_volume *v) {
    if (!v || !v->data) return false;
    if (v->nx < 2 || v->ny < 2 || v->nz < 2) return false;
    if (v->voxel_type != MCG_VOXEL_SHORT2 && v->voxel_type != MCG_VOXEL_FLOAT2) return false;
    if (!(v->cell > 0.0f)) return false;
    // voxels are read whole: the data is aligned to the voxel size
    if (reinterpret_cast<uintptr_t>(v->data) % (v->voxel_type == MCG_VOXEL_SHORT2 ? 4u : 8u)) return false;
    // brick ids are 32-bit in the active list
    if (geometry(v->nx, v->ny, v->nz).nbricks >= (1ll << 32)) return false;
    return true;
}

template <class K>
int occupancy(K kernel, int threads, size_t smem) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int o = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kernel, threads, smem) != cudaSuccess || o < 1) {
        cudaGetLastError();
        o = 1;
    }
    return o;
}

}  // namespace
}  // namespace mcg
