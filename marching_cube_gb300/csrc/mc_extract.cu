// Marching-cubes extraction on sm_103a.
//
// Replaces the reference pipeline (cu_marching_cubes_v1.cu):
//   getOccupiedVoxelsKernel (:97-206)   -> mc_classify_kernel
//   thrust::exclusive_scan   (:208-225) -> mc_scan_kernel
//   trianglesGeneratorKernel (:228-396) -> mc_generate_kernel (+ fused normals,
//                                          cu_kinect_fusion_v1.cu:3146-3242)
//
// Work is organised in bricks of 32x8x8 cubes.
//
// Pass 1 (classify) streams the whole volume once.  Persistent CTAs, four per
// SM with one tile stage each, take work items (groups of 4 bricks adjacent
// in x, 2 for float2) from a counter; each item's voxels (132x9x9: the bricks
// plus the voxels the last cube column and the y / z halo need) arrive by
// TMA (cp.async.bulk.tensor.3d, completion on an mbarrier that one thread
// polls with a time bound).  A tile whose in-volume voxels all have one sign
// is settled by one OR/AND pass; otherwise threads turn its rows into two bit
// masks per 33 voxels (tsdf < 0, weight == 0) from 16-byte shared-memory
// loads, and a cube row of 32 cubes is classified with a handful of 64-bit
// AND/OR operations on four row masks and __popc, so only occupied cubes (a
// few per mille of a fusion volume) ever look up a table.  Output: triangle
// counts per brick and per-chunk sums.
//
// A multi-CTA scan (one CTA per chunk of 256 bricks) turns brick counts into
// 64-bit soup offsets and a list of active bricks (heaviest classes first).
//
// Pass 2 (generate) visits only active bricks, with a 2-stage TMA prefetch
// of the brick + halo (36x10x10 voxels).  The same masks give a compact list
// of occupied cubes with their vertex offsets; each thread then emits one
// soup vertex (its cube and edge through a vertex map, or a binary search
// over the list), computes the fused normal from the tile, and the 28-byte
// records go out through a per-warp shared-memory stage as full coalesced
// lines.  The three launches chain with programmatic dependent launch.
//
// When TMA cannot describe the volume (x row not a multiple of 16 bytes or an
// unaligned base) the same kernels fill the tiles by 16-byte words of the
// volume shifted into place (fill_tile).
//
// Output order is deterministic: bricks in (bz, by, bx) order, cubes in
// (z, y, x) order inside a brick, then the table slot -- the reference's
// order is non-deterministic (one atomicAdd per warp, :145).
//
// Arithmetic follows the reference's expressions in IEEE binary32, source
// order, no contraction (the library is built with --fmad=false).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <utility>

#include "mc_common.cuh"

namespace mcg {
namespace {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int ROWS = (BY + 1) * (BZ + 1);  // voxel rows feeding one brick: 81
constexpr int CUBE_ROWS = BY * BZ;         // 64

// classify tile: voxels [x0, x0+36) x [y0, y0+9) x [z0, z0+9)
constexpr int CTX = 36, CTY = BY + 1, CTZ = BZ + 1;
constexpr int CTILE = CTX * CTY * CTZ;
// generate tile: voxels [x0, x0+36) x [y0, y0+10) x [z0, z0+10) -- every
// corner and normal sample of the brick's cubes; the rare side-output reads
// of voxel x0-1 / y0-1 / z0-1 go to global memory
constexpr int TXO = 0, TYO = 0, TZO = 0;
constexpr int TX = BX + 4, TY = BY + 2, TZ = BZ + 2;
constexpr int GTILE = TX * TY * TZ;
constexpr int GSTAGES = 2;
// tile stages and minimum resident CTAs per SM of the single-volume generate
// launch.  One stage measured faster than two at 4 CTAs/SM (a brick's work
// hides most of its next tile's load, and the smaller footprint lets the next
// launch's count CTAs start beside the drained ones); 5 CTAs/SM spill.
#ifndef MCG_GEN_STAGES
#define MCG_GEN_STAGES 1
#endif
#ifndef MCG_GEN_MINB
#define MCG_GEN_MINB 4
#endif
constexpr int GEN_STAGES = MCG_GEN_STAGES;
constexpr int GEN_MINB = MCG_GEN_MINB;

// Row masks: bit k of neg / dead = voxel (x0 + k) of a 33-voxel row is
// negative / has weight 0, k = 0..32.  One thread builds one row from 16-byte
// shared-memory loads of its first 32 voxels (`row` 16-byte aligned) and the
// 33rd voxel `last`: about 4 integer operations per voxel instead of a warp
// vote per row.  The two-argument form takes the 33rd voxel from the row.
template <int VT>
struct RowMask;

template <>
struct RowMask<MCG_VOXEL_SHORT2> {
    static __device__ __forceinline__ void build(const short2 *row, short2 last, unsigned long long &neg,
                                                 unsigned long long &dead) {
        const uint4 *q = reinterpret_cast<const uint4 *>(row);
        unsigned int n = 0, d = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint4 v = q[k];
            const unsigned int w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                n |= ((w[j] >> 15) & 1u) << (4 * k + j);     // tsdf (low half) < 0
                d |= (unsigned int)(w[j] < 0x10000u) << (4 * k + j);  // w (high half) == 0
            }
        }
        neg = (unsigned long long)n | ((unsigned long long)(last.x < 0) << 32);
        dead = (unsigned long long)d | ((unsigned long long)(last.y == 0) << 32);
    }
    static __device__ __forceinline__ void build(const short2 *row, unsigned long long &neg,
                                                 unsigned long long &dead) {
        build(row, row[32], neg, dead);
    }
};

template <>
struct RowMask<MCG_VOXEL_FLOAT2> {
    static __device__ __forceinline__ void build(const float2 *row, float2 last, unsigned long long &neg,
                                                 unsigned long long &dead) {
        const float4 *q = reinterpret_cast<const float4 *>(row);
        unsigned int n = 0, d = 0;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const float4 v = q[k];
            n |= (unsigned int)(v.x < 0.f) << (2 * k);
            n |= (unsigned int)(v.z < 0.f) << (2 * k + 1);
            d |= (unsigned int)(v.y == 0.f) << (2 * k);
            d |= (unsigned int)(v.w == 0.f) << (2 * k + 1);
        }
        neg = (unsigned long long)n | ((unsigned long long)(last.x < 0.f) << 32);
        dead = (unsigned long long)d | ((unsigned long long)(last.y == 0.f) << 32);
    }
    static __device__ __forceinline__ void build(const float2 *row, unsigned long long &neg,
                                                 unsigned long long &dead) {
        build(row, row[32], neg, dead);
    }
};

// Occupied-cube mask of cube row (cy, cz) of a brick: bit x set iff cube x
// has a sign change and no weight-0 corner (cu_marching_cubes_v1.cu:74-91,
// :136 -- every case other than 0 and 255 emits triangles).

__device__ __forceinline__ CubeRow cube_row(const unsigned long long *neg, const unsigned long long *dead, int cy,
                                            int cz, unsigned int valid) {
    CubeRow r;
    const int r00 = cz * (BY + 1) + cy, r01 = r00 + 1, r10 = r00 + (BY + 1), r11 = r10 + 1;
    r.a = neg[r00];
    r.b = neg[r01];
    r.c = neg[r10];
    r.d = neg[r11];
    const unsigned long long all = r.a & (r.a >> 1) & r.b & (r.b >> 1) & r.c & (r.c >> 1) & r.d & (r.d >> 1);
    const unsigned long long any = r.a | (r.a >> 1) | r.b | (r.b >> 1) | r.c | (r.c >> 1) | r.d | (r.d >> 1);
    const unsigned long long da = dead[r00], db = dead[r01], dc = dead[r10], dd = dead[r11];
    const unsigned long long dz = da | (da >> 1) | db | (db >> 1) | dc | (dc >> 1) | dd | (dd >> 1);
    r.occ = (unsigned int)(any & ~all & ~dz) & valid;
    return r;
}

// cube index of cube x of a row (bit i = corner i negative)
__device__ __forceinline__ unsigned int cube_index(const CubeRow &r, int x) {
    return (unsigned int)(((r.a >> x) & 1) | (((r.a >> (x + 1)) & 1) << 1) | (((r.b >> (x + 1)) & 1) << 2) |
                          (((r.b >> x) & 1) << 3) | (((r.c >> x) & 1) << 4) | (((r.c >> (x + 1)) & 1) << 5) |
                          (((r.d >> (x + 1)) & 1) << 6) | (((r.d >> x) & 1) << 7));
}

__device__ __forceinline__ unsigned int valid_mask(int x0, int nx) {
    const int nvalid = nx - 1 - x0;  // cubes exist for x < nx - 1
    return nvalid >= 32 ? 0xffffffffu : (nvalid <= 0 ? 0u : ((1u << nvalid) - 1u));
}

// ---- pass 1: classify ------------------------------------------------------
constexpr int CTHREADS = 128;

// True when the tile holds both negative and non-negative voxels.  Most
// bricks of a fusion volume lie wholly on one side of the surface (or in
// unobserved space, all -32766), and no cube of such a brick changes sign, so
// one OR / AND pass over the tile's sign bits settles them before any mask
// work.  Called by every thread; contains a barrier.
template <int VT, int NVOX = CTILE, class Smem>
__device__ __forceinline__ bool tile_mixed(Smem &S, const typename Vox<VT>::T *tile) {
    static_assert(NVOX * Vox<VT>::bytes % 16 == 0, "tile is a whole number of 16-byte words");
    constexpr int NQ = NVOX * Vox<VT>::bytes / 16;
    const uint4 *q = reinterpret_cast<const uint4 *>(tile);
    unsigned int neg_any = 0, pos_any = 0;
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) {
        const uint4 v = q[i];
        if (VT == MCG_VOXEL_SHORT2) {
            // bit 15 of each word is the tsdf sign
            neg_any |= v.x | v.y | v.z | v.w;
            pos_any |= ~(v.x & v.y & v.z & v.w);
        } else {
            // x and z are the tsdf of two voxels; -0.0f is not negative
            const bool n0 = __uint_as_float(v.x) < 0.f, n1 = __uint_as_float(v.z) < 0.f;
            neg_any |= (unsigned int)(n0 | n1) << 15;
            pos_any |= (unsigned int)(!n0 | !n1) << 15;
        }
    }
    neg_any = __reduce_or_sync(0xffffffffu, neg_any & 0x8000u);
    pos_any = __reduce_or_sync(0xffffffffu, pos_any & 0x8000u);
    if ((threadIdx.x & 31) == 0) S.mix[threadIdx.x >> 5] = (neg_any ? 1u : 0u) | (pos_any ? 2u : 0u);
    __syncthreads();
    unsigned int m = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m |= S.mix[w];
    return m == 3u;
}

// Pass-1 work on one brick tile: row masks, cube rows, per-warp sums into
// S.red (read after the caller's next __syncthreads).  Called by every
// thread of the CTA.
template <int VT, class Smem>
__device__ __forceinline__ void classify_brick(Smem &S, const typename Vox<VT>::T *tile, int nx, int ny, int nz,
                                               BrickPos bp) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < ROWS) RowMask<VT>::build(tile + tid * CTX, S.neg[tid], S.dead[tid]);
        __syncthreads();
        if (tid < CUBE_ROWS) {
            const int cy = tid & (BY - 1), cz = tid / BY;
            unsigned int tri = 0, occ = 0;
            if (bp.y0 + cy < ny - 1 && bp.z0 + cz < nz - 1) {
                const CubeRow cr = cube_row(S.neg, S.dead, cy, cz, valid_mask(bp.x0, nx));
                occ = __popc(cr.occ);
                unsigned int m = cr.occ;
                while (m) {
                    const int x = __ffs(m) - 1;
                    m &= m - 1;
                    tri += S.ntri[cube_index(cr, x)];
                }
            }
            tri = __reduce_add_sync(0xffffffffu, tri);
            occ = __reduce_add_sync(0xffffffffu, occ);
            if (lane == 0) {
                S.red[warp][0] = tri;
                S.red[warp][1] = occ;
            }
        }
}

// next work item of the launch for this CTA (dynamic: CTAs take items in
// order from a counter, so a CTA that drew cheap items takes more), -1 when
// done; launches have fewer than 2^31 items
__device__ __forceinline__ int next_item(unsigned int *ticket, int n) {
    const unsigned int t = atomicAdd(ticket, 1u);
    return t < (unsigned int)n ? (int)t : -1;
}

// the same over a 64-bit count
__device__ __forceinline__ long long next_brick(unsigned int *ticket, long long n) {
    const unsigned int t = atomicAdd(ticket, 1u);
    return (long long)t < n ? (long long)t : -1ll;
}

// Single-volume classify: one work item is a group of G bricks adjacent in x.
// Its voxels arrive by two TMA boxes on one mbarrier: the bricks' own
// 32 G x 9 x 9 voxels (rows of 512 bytes at the preferred G), and a box
// 16 bytes wide at voxel column x0 + 32 G for the 33rd voxel of the last
// brick's rows.  A halo of 4 voxels on every row of the main box would add a
// partial line to each row request: on GB300 a 68-voxel box streams a 512^3
// short2 volume at about 5.7 TB/s, a 64-voxel box at 6.3 and a 128-voxel box
// at 7.0.
template <int G, int XH>
struct ClsGeom {
    static constexpr int TXW = BX * G + XH;  // main box width in voxels (XH: in-box halo, 0 or 4)
    static constexpr int TILE = TXW * CTY * CTZ;
};

// halo box: the first 16 bytes of each of the ROWS rows right of the main box
template <int VT>
struct ClsHalo {
    static constexpr int HW = 16 / Vox<VT>::bytes;  // voxels per halo row
    static constexpr int N = HW * ROWS;
};

template <int VT, int G, int XH, int CSTAGES, int NT>
struct ClsSmemG {
    static constexpr int STAGE_BYTES = pad128(ClsGeom<G, XH>::TILE * Vox<VT>::bytes);
    static constexpr int HALO_BYTES = XH ? 0 : pad128(ClsHalo<VT>::N * Vox<VT>::bytes);
    unsigned char tiles[CSTAGES][STAGE_BYTES];
    unsigned char halo[CSTAGES][HALO_BYTES];
    unsigned long long neg[G * ROWS], dead[G * ROWS];  // [brick h of the group][row]
    uint64_t bars[CSTAGES];
    int4 sorg[CSTAGES];  // stage's item: {x0, y0, z0, first brick x}; x0 < 0 when none
    unsigned int red[NT / 32][2];
    unsigned int mix[NT / 32];
    unsigned char ntri[256];
    int abort;
};

// True when the voxels of the item that lie inside the volume (tile and halo
// column) hold both negative and non-negative values.  Rows, columns and the
// halo outside the volume arrive zero-filled and are left out, so the border
// items of an all-negative volume stay on the one-pass path.  Called by every
// thread; contains a barrier.
template <int VT, int G, int XH, int NT, class Smem>
__device__ __forceinline__ bool item_mixed(Smem &S, const typename Vox<VT>::T *tile, const typename Vox<VT>::T *hal,
                                           int nx, int ny, int nz, int x0, int y0, int z0) {
    using V = Vox<VT>;
    constexpr int WPR = ClsGeom<G, XH>::TXW * V::bytes / 16;  // 16-byte words per row
    constexpr int VPW = 16 / V::bytes;                   // voxels per word
    const uint4 *q = reinterpret_cast<const uint4 *>(tile);
    const int ry = ny - y0, rz = nz - z0, rx = nx - x0;  // inside: ly < ry, lz < rz, lx < rx
    unsigned int neg_any = 0, pos_any = 0;
    for (int i = threadIdx.x; i < WPR * ROWS; i += NT) {
        const int r = i / WPR, lx = (i - r * WPR) * VPW;
        const int lz = r / CTY, ly = r - lz * CTY;
        if (ly >= ry || lz >= rz || lx >= rx) continue;
        const uint4 v = q[i];
        if (VT == MCG_VOXEL_SHORT2) {
            // bit 15 of each word is the tsdf sign
            neg_any |= v.x | v.y | v.z | v.w;
            pos_any |= ~(v.x & v.y & v.z & v.w);
        } else {
            // x and z are the tsdf of two voxels; -0.0f is not negative
            const bool n0 = __uint_as_float(v.x) < 0.f, n1 = __uint_as_float(v.z) < 0.f;
            neg_any |= (unsigned int)(n0 | n1) << 15;
            pos_any |= (unsigned int)(!n0 | !n1) << 15;
        }
    }
    if (XH == 0 && threadIdx.x < ROWS && ClsGeom<G, XH>::TXW < rx) {
        const int r = threadIdx.x, lz = r / CTY, ly = r - lz * CTY;
        if (ly < ry && lz < rz) {
            if (V::neg(hal[r * ClsHalo<VT>::HW])) neg_any |= 0x8000u;
            else pos_any |= 0x8000u;
        }
    }
    neg_any = __reduce_or_sync(0xffffffffu, neg_any & 0x8000u);
    pos_any = __reduce_or_sync(0xffffffffu, pos_any & 0x8000u);
    if ((threadIdx.x & 31) == 0) S.mix[threadIdx.x >> 5] = (neg_any ? 1u : 0u) | (pos_any ? 2u : 0u);
    __syncthreads();
    unsigned int m = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) m |= S.mix[w];
    return m == 3u;
}

// Persistent CTAs of NT threads take work items from a counter into a ring
// of CSTAGES tile stages (one thread issues the loads and polls the
// barriers with a time bound).
template <int VT, bool TMA, int G, int XH, int CSTAGES, int NT>
__global__ void __launch_bounds__(NT)
    mc_classify_kernel(const __grid_constant__ CUtensorMap map, const __grid_constant__ CUtensorMap hmap,
                       const typename Vox<VT>::T *__restrict__ vol, int nx, int ny, int nz, int nbx, int nby,
                       int nitems, int ngx, int zbase, int zlim, uint32_t *__restrict__ brick_tris,
                       uint32_t *__restrict__ chunk, unsigned int *__restrict__ flags,
                       unsigned int *__restrict__ ticket) {
    static_assert(NT >= G * CUBE_ROWS && NT >= ROWS && NT % 32 == 0, "one thread per cube row and per halo row");
    using V = Vox<VT>;
    using T = typename V::T;
    using Geo = ClsGeom<G, XH>;
    using H = ClsHalo<VT>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    ClsSmemG<VT, G, XH, CSTAGES, NT> &S = *reinterpret_cast<ClsSmemG<VT, G, XH, CSTAGES, NT> *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = tid; c < 256; c += NT) S.ntri[c] = (c == 0 || c == 255) ? 0 : g_nverts[c] / 3;
    // everything above touches only shared and constant memory: the launch may
    // overlap the kernel before it, whose writes (the volume, the counters) are
    // waited for here
    pdl_wait();
    // stage st's item (drawn by thread 0, which alone divides): origin into
    // S.sorg[st] and, with TMA, its loads -- the halo box only when column
    // x0 + TXW is inside the volume (its voxel is used by no cube otherwise)
    auto stage_item = [&](int st, int it) {
        if (it < 0) {
            S.sorg[st] = make_int4(-1, 0, 0, 0);
            return;
        }
        const unsigned int r = (unsigned int)it / (unsigned int)ngx;
        const int bx0 = (int)((unsigned int)it - r * (unsigned int)ngx) * G;
        const int y0 = (int)(r % (unsigned int)nby) * BY, z0 = (int)(r / (unsigned int)nby) * BZ + zbase;
        const int x0 = bx0 * BX;
        S.sorg[st] = make_int4(x0, y0, z0, bx0);
        if (TMA) {
            const bool halo = XH == 0 && x0 + Geo::TXW < nx;
            mbar_arrive_expect_tx(&S.bars[st], (Geo::TILE + (halo ? H::N : 0)) * V::bytes);
            tma_load_3d(S.tiles[st], &map, &S.bars[st], x0, y0, z0);
            if (halo) tma_load_3d(S.halo[st], &hmap, &S.bars[st], x0 + Geo::TXW, y0, z0);
        }
    };
    // Thread 0 draws the ticket of the next refill one iteration ahead and
    // reads it only at that refill: the counter is contended by every CTA, and
    // a use right after the atomic would hold warp 0 -- and with it the whole
    // CTA at the next barrier -- for the round trip.  The first stages take
    // CSTAGES consecutive tickets with one atomic.
    unsigned int ptk = 0xffffffffu;
    if (tid == 0) {
        S.abort = 0;
        if (TMA) {
            for (int s = 0; s < CSTAGES; ++s) mbar_init(&S.bars[s], 1);
            fence_barrier_init();
            const unsigned int t0 = atomicAdd(ticket, (unsigned int)CSTAGES);
            for (int s = 0; s < CSTAGES; ++s) stage_item(s, t0 + s < (unsigned int)nitems ? (int)(t0 + s) : -1);
            if (t0 + CSTAGES < (unsigned int)nitems) ptk = atomicAdd(ticket, 1u);
        }
    }
    __syncthreads();
    for (int i = 0;; ++i) {
        const int s = TMA ? i % CSTAGES : 0;
        if (!TMA) {
            if (tid == 0) stage_item(0, next_item(ticket, nitems));
            __syncthreads();
        }
        const int4 org = S.sorg[s];
        if (org.x < 0) break;  // uniform: every thread reads the same entry
        const int x0 = org.x, y0 = org.y, z0 = org.z, bx0 = org.w;
        T *tile = reinterpret_cast<T *>(S.tiles[s]);
        T *hal = XH ? nullptr : reinterpret_cast<T *>(S.halo[s]);
        if (TMA) {
            // one thread polls the barrier; the others wait at __syncthreads
            if (tid == 0 && !mbar_wait(&S.bars[s], (uint32_t)((i / CSTAGES) & 1))) S.abort = 1;
        } else {
            fill_tile<VT, Geo::TXW, CTY, CTZ>(tile, vol, nx, ny, nz, x0, y0, z0);
            if (XH == 0 && tid < ROWS) {
                const int gx = x0 + Geo::TXW, gy = y0 + tid % CTY, gz = z0 + tid / CTY;
                hal[tid * H::HW] = (gx < nx && gy < ny && gz < nz) ? vol[lin3(nx, ny, gx, gy, gz)] : V::fill();
            }
        }
        __syncthreads();
        if (S.abort) break;
        const bool mixed = item_mixed<VT, G, XH, NT>(S, tile, hal, nx, ny, nz, x0, y0, z0);
        if (mixed) {
            // row masks: 33 bits of row r starting at voxel x0 + 32 h; the 33rd
            // voxel of the last brick's rows is the halo column's
            const bool has_halo = x0 + Geo::TXW < nx;
            for (int m = tid; m < G * ROWS; m += NT) {
                const int h = m / ROWS, r = m - h * ROWS;
                const T *row = tile + r * Geo::TXW + h * BX;
                const T last = (XH || h < G - 1) ? row[BX] : (has_halo ? hal[r * H::HW] : V::fill());
                RowMask<VT>::build(row, last, S.neg[m], S.dead[m]);
            }
            __syncthreads();
        }
        // the tile has been read for the last time: refill its stage now, so the
        // load overlaps the cube rows below
        if (TMA && tid == 0) {
            const int it = ptk < (unsigned int)nitems ? (int)ptk : -1;
            stage_item(s, it);
            if (it >= 0) ptk = atomicAdd(ticket, 1u);
        }
        if (mixed) {
            if (tid < G * CUBE_ROWS) {
                // 64 cube rows per brick = two whole warps per brick
                const int h = tid / CUBE_ROWS, c = tid - h * CUBE_ROWS;
                const int cy = c & (BY - 1), cz = c / BY;
                unsigned int tri = 0, occ = 0;
                if (bx0 + h < nbx && y0 + cy < ny - 1 && z0 + cz < zlim) {
                    const CubeRow cr = cube_row(S.neg + h * ROWS, S.dead + h * ROWS, cy, cz,
                                                valid_mask(x0 + h * BX, nx));
                    occ = __popc(cr.occ);
                    unsigned int mm = cr.occ;
                    while (mm) {
                        const int x = __ffs(mm) - 1;
                        mm &= mm - 1;
                        tri += S.ntri[cube_index(cr, x)];
                    }
                }
                tri = __reduce_add_sync(0xffffffffu, tri);
                occ = __reduce_add_sync(0xffffffffu, occ);
                if (lane == 0) {
                    S.red[warp][0] = tri;
                    S.red[warp][1] = occ;
                }
            }
            __syncthreads();  // red[] complete
        }
        if (tid < G && bx0 + tid < nbx) {
            const int h = tid;
            unsigned int t = 0, o = 0;
            if (mixed) {
                t = S.red[2 * h][0] + S.red[2 * h + 1][0];
                o = S.red[2 * h][1] + S.red[2 * h + 1][1];
            }
            const long long b = ((long long)((z0 - zbase) / BZ) * nby + y0 / BY) * nbx + bx0 + h;
            brick_tris[b] = t;
            // per-chunk (CHUNK consecutive bricks) sums feed the scan
            if (t) {
                uint32_t *c = chunk + (b / CHUNK) * CHUNK_FIELDS;
                atomicAdd(c + 0, t);
                atomicAdd(c + 1, 1u);
                atomicAdd(c + 2, o);
                const int hc = heavy_class(t);
                if (hc >= 0) atomicAdd(c + 3 + hc, 1u);
            }
        }
        // with one stage, the entry read at the top is the one just rewritten
        if (!TMA || CSTAGES == 1) __syncthreads();
    }
    pdl_trigger();  // no more work: the scan may start its launch
    if (S.abort && tid == 0) {
        atomicOr(flags, 1u);
        // give loads still in flight a bounded chance to land before exit
        for (int s = 0; s < CSTAGES; ++s) mbar_wait(&S.bars[s], 0, 100000000ull);
    }
}

// ---- batched extraction: shared definitions ----------------------------------------
// Bricks of all volumes of a batch form one index space: volume v owns bricks
// [brick_base, brick_base + nbricks).  A brick's volume is found by binary
// search over the descriptor table; tiles come by TMA through the volume's
// own tensor map (global memory) when TMA can describe it, by 16-byte words
// shifted into place otherwise (fill_tile).  Soup offsets come from one scan over all
// bricks; a volume's soup starts at the offset of its first brick, i.e. 3x
// the triangles of the volumes before it.
struct VolDesc {
    const void *data;
    int nx, ny, nz;
    float cell;
    int nbx, nby;
    int tma;
    int pad;
    long long brick_base;
    long long nbricks;
    mcg_vertex_voxel *soup;
    float *normals;
    int32_t *vi2vox;
    int16_t *ver_voxel;
    int64_t *tri_cube;
    long long cap;
};

__device__ __forceinline__ int find_volume(const VolDesc *__restrict__ vols, int nvol, long long b) {
    int lo = 0, hi = nvol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (vols[mid].brick_base <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// An active-list entry of a batch as the batch's scan writes it for the
// generate launch: volume, brick origin and soup offset inside the volume's
// soup, so the thread that stages the brick does no search.
struct BatchBrick {
    unsigned long long vbase;
    int v, x0, y0, z0;
    int pad[2];
};
static_assert(sizeof(BatchBrick) == 32, "two 16-byte copies");

// ---- scan: brick counts -> soup offsets + active brick list ---------------------
// One CTA per chunk of CHUNK consecutive bricks.  Classify has accumulated
// each chunk's triangles, active bricks, occupied cubes and heavy bricks by
// class; a CTA adds up the chunks before its own for its base offsets, scans
// its bricks, and writes 64-bit soup offsets and its part of the active-brick
// list: heavy classes first (heaviest first), then the light bricks, each in
// brick order, with each entry's soup offset beside it (list_vofs, when
// given).  CTA 0 also writes the totals, to `host` as well when given (a
// mapped host copy).  The last CTA to have read the chunk sums zeroes them for
// the next count phase.  Over a batch (BATCH) it also writes each active
// entry's BatchBrick: the brick's volume, origin and offset in that volume's
// soup, from the per-volume triangle sums of the count launch.
struct ScanBatch {
    const VolDesc *vols;
    int nvol;
    const unsigned long long *vol_sums;  // {triangles, occupied cubes} per volume
    BatchBrick *list;                    // one entry per active-list entry
    unsigned long long *host_vol_sums;   // mapped host copy of vol_sums (written by CTA 0), or null
};

template <bool BATCH>
__global__ void __launch_bounds__(CHUNK)
    mc_scan_kernel(const uint32_t *__restrict__ brick_tris, uint32_t *__restrict__ chunk, long long nb,
                   unsigned long long *__restrict__ brick_vofs, uint32_t *__restrict__ active,
                   unsigned long long *__restrict__ list_vofs, MeshTotals *__restrict__ totals,
                   MeshTotals *__restrict__ host, ScanBatch bt) {
    // acc: [0] base tris, [1] base active, [2, 2+NH) base heavy per class,
    // [2+NH] all tris, [3+NH] all active, [4+NH] all occupied, [5+NH, 5+2NH) all heavy
    constexpr int NH = NHEAVY, NACC = 5 + 2 * NH, NF = NH + 2;  // scanned per brick: tris, classes, light
    __shared__ unsigned long long s_part[NACC][CHUNK / 32];
    __shared__ unsigned long long s_base_v;
    __shared__ unsigned int s_base[NH + 1];  // list offset of this chunk's first brick of each class / light
    __shared__ bool s_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long j = blockIdx.x;
    const long long nchunks = (nb + CHUNK - 1) / CHUNK;
    pdl_wait();     // the count launch's sums and counts
    pdl_trigger();  // the generate launch may start its prologue
    unsigned long long acc[NACC];
#pragma unroll
    for (int k = 0; k < NACC; ++k) acc[k] = 0;
    for (long long i = tid; i < nchunks; i += CHUNK) {
        const uint32_t *c = chunk + i * CHUNK_FIELDS;
        const unsigned long long cv = c[0], ca = c[1];
        if (i < j) {
            acc[0] += cv;
            acc[1] += ca;
#pragma unroll
            for (int k = 0; k < NH; ++k) acc[2 + k] += c[3 + k];
        }
        acc[2 + NH] += cv;
        acc[3 + NH] += ca;
        acc[4 + NH] += c[2];
#pragma unroll
        for (int k = 0; k < NH; ++k) acc[5 + NH + k] += c[3 + k];
    }
#pragma unroll
    for (int k = 0; k < NACC; ++k) {
#pragma unroll
        for (int o = 16; o; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if (lane == 0) s_part[k][warp] = acc[k];
    }
    __syncthreads();  // this CTA's reads of the chunk sums are done
    if (tid == 0) {
        // the count launch's flags, read before this CTA counts itself done
        // (the last CTA may clear them after that)
        const unsigned int fl = j == 0 ? *(volatile unsigned int *)&totals->flags : 0u;
        __threadfence();
        s_last = atomicAdd(&totals->scan_done, 1u) == gridDim.x - 1;
        unsigned long long r[NACC];
        for (int k = 0; k < NACC; ++k) {
            r[k] = 0;
            for (int w = 0; w < CHUNK / 32; ++w) r[k] += s_part[k][w];
        }
        s_base_v = r[0];
        unsigned long long start = 0, heavy_before = 0;  // list start of the class; heavy bricks of earlier chunks
        for (int k = 0; k < NH; ++k) {
            s_base[k] = (unsigned int)(start + r[2 + k]);
            start += r[5 + NH + k];
            heavy_before += r[2 + k];
        }
        s_base[NH] = (unsigned int)(start + (r[1] - heavy_before));
        if (j == 0) {
            totals->occupied = r[4 + NH];
            totals->triangles = r[2 + NH];
            totals->vertices = 3ull * r[2 + NH];
            totals->active_bricks = (unsigned int)r[3 + NH];
            if (host) {
                host->occupied = r[4 + NH];
                host->triangles = r[2 + NH];
                host->vertices = 3ull * r[2 + NH];
                host->active_bricks = (unsigned int)r[3 + NH];
                host->flags = fl;
                __threadfence_system();
            }
        }
    }
    __syncthreads();
    if (BATCH && j == 0 && bt.host_vol_sums) {
        for (int i = tid; i < 2 * bt.nvol; i += CHUNK) bt.host_vol_sums[i] = bt.vol_sums[i];
        __threadfence_system();
    }
    // BATCH: the soup start of each volume this chunk's bricks lie in (at
    // most CHUNK volumes, each owning at least one brick): 3x the triangles
    // of the volumes before it
    __shared__ unsigned long long s_vpre[BATCH ? CHUNK : 1];
    int vmin = 0;
    if (BATCH) {
        const long long first = j * CHUNK, last = (first + CHUNK < nb ? first + CHUNK : nb) - 1;
        vmin = find_volume(bt.vols, bt.nvol, first);
        const int vmax = find_volume(bt.vols, bt.nvol, last);
        unsigned long long pre = 0;
        for (int u = tid; u < vmin; u += CHUNK) pre += bt.vol_sums[2 * u];
#pragma unroll
        for (int o = 16; o; o >>= 1) pre += __shfl_xor_sync(0xffffffffu, pre, o);
        if (lane == 0) s_part[0][warp] = pre;  // thread 0 read s_part before the barrier above
        __syncthreads();
        if (tid == 0) {
            unsigned long long r = 0;
            for (int w = 0; w < CHUNK / 32; ++w) r += s_part[0][w];
            for (int v = vmin; v <= vmax; ++v) {
                s_vpre[v - vmin] = 3ull * r;
                r += bt.vol_sums[2 * v];
            }
        }
        __syncthreads();
    }
    const unsigned long long base_v = s_base_v;
    const long long b = j * CHUNK + tid;
    const unsigned int t = b < nb ? brick_tris[b] : 0u;
    const int cls = t == 0 ? -1 : (heavy_class(t) >= 0 ? heavy_class(t) : NH);  // NH: light
    unsigned int f[NF], x[NF];
    f[0] = t;
#pragma unroll
    for (int k = 0; k <= NH; ++k) f[1 + k] = cls == k ? 1u : 0u;
#pragma unroll
    for (int k = 0; k < NF; ++k) x[k] = f[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            const unsigned int u = __shfl_up_sync(0xffffffffu, x[k], o);
            if (lane >= o) x[k] += u;
        }
    }
    __shared__ unsigned int s_w[NF][CHUNK / 32];
    if (lane == 31) {
#pragma unroll
        for (int k = 0; k < NF; ++k) s_w[k][warp] = x[k];
    }
    __syncthreads();
    unsigned int wp[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        wp[k] = 0;
        for (int w = 0; w < warp; ++w) wp[k] += s_w[k][w];
    }
    if (b < nb) {
        const unsigned long long v = 3ull * (base_v + wp[0] + x[0] - t);
        brick_vofs[b] = v;
#pragma unroll
        for (int k = 0; k <= NH; ++k)
            if (f[1 + k]) {
                const unsigned int w = s_base[k] + wp[1 + k] + x[1 + k] - 1;
                active[w] = (uint32_t)b;
                if (list_vofs) list_vofs[w] = v;
                if (BATCH) {
                    const int vb = find_volume(bt.vols, bt.nvol, b);
                    const VolDesc &d = bt.vols[vb];
                    const BrickPos bp = brick_pos(b - d.brick_base, d.nbx, d.nby);
                    BatchBrick r;
                    r.vbase = v - s_vpre[vb - vmin];
                    r.v = vb;
                    r.x0 = bp.x0;
                    r.y0 = bp.y0;
                    r.z0 = bp.z0;
                    r.pad[0] = r.pad[1] = 0;
                    bt.list[w] = r;
                }
            }
    }
    if (s_last) {  // every CTA has read the chunk sums (and CTA 0 the flags)
        for (long long i = tid; i < nchunks * CHUNK_FIELDS; i += CHUNK) chunk[i] = 0;
        if (tid == 0) {
            totals->scan_done = 0;
            if (BATCH) totals->gen_ticket = 0;  // the batch's generate launch draws from it
            if (host) {  // the flags live on in the host copy
                totals->flags = 0;
                totals->cls_ticket = 0;
            }
        }
    }
}

// ---- pass 2: generate ------------------------------------------------------
struct GenParams {
    const void *vol;
    int nx, ny, nz;
    float cell;
    int nbx, nby;
    int zbase, zlim;  // z of brick layer 0; cubes exist for z < zlim
    const uint32_t *active;
    const unsigned long long *brick_vofs;
    const unsigned long long *list_vofs;  // soup offset of each active-list entry
    MeshTotals *totals;
    MeshTotals *host;  // mapped host copy of the totals (flags written at exit), or null
    unsigned int fixed_rounds;  // first bricks of each CTA taken in fixed serpentine rounds
    mcg_vertex_voxel *soup;
    float *normals;
    int32_t *vi2vox;
    int16_t *ver_voxel;
    int64_t *tri_cube;
    long long cap;
    // adjoint (MODE 1): dL/dP per soup vertex in, dL/df per voxel accumulated
    const float *grad_pos;
    float *grad_f;
    long long n_grad;
};

template <int VT, int NST = GSTAGES>
struct GenSmem {
    static constexpr int STAGE_BYTES = pad128(GTILE * Vox<VT>::bytes);
    unsigned char tiles[NST][STAGE_BYTES];
    unsigned long long neg[ROWS], dead[ROWS];
    uint64_t bars[NST];
    unsigned int stage[WARPS][32 * 7];
    unsigned short occ_cube[BRICK_CUBES];  // local cube index (z*8 + y)*32 + x, in that order
    unsigned short occ_off[BRICK_CUBES];   // exclusive soup-vertex offset inside the brick
    unsigned char occ_ci[BRICK_CUBES];
    alignas(16) signed char tri[256][16];  // read a row at a time as 16 bytes
    unsigned char nv[256];
    unsigned short vmap[BRICK_CUBES];      // soup vertex -> local cube << 4 | edge, when the brick has <= 2048
    long long sbrick[NST];                 // brick id, soup offset and origin of each stage's tile
    unsigned long long svbase[NST];
    int4 spos[NST];
    unsigned long long pipe_v;  // refill pipeline (thread 0): the brick staged at the next
    unsigned int pipe_b;        // refill and its soup offset; pipe_b ~0u = none
    unsigned int wsum[2][2];
    unsigned int nocc, total;
    int abort;
};

__device__ __forceinline__ int tidx(int lx, int ly, int lz) { return (lz * TY + ly) * TX + lx; }

// Output arrays of one volume (device pointers, any may be null).
struct GenOut {
    mcg_vertex_voxel *soup;
    float *normals;
    int32_t *vi2vox;
    int16_t *ver_voxel;
    int64_t *tri_cube;
    long long cap;
    int zlim;  // cubes exist for z < zlim (nz - 1, or the end of a slab)
};

// All per-brick work of pass 2 once the brick's tile is in shared memory:
// occupied-cube list with vertex offsets, then one soup vertex per thread.
// Called by every thread of the CTA (contains __syncthreads).
// Occupied-cube list of a brick whose tile is in shared memory: S.occ_cube /
// occ_ci / occ_off in (z, y, x) order, S.nocc entries, S.total soup
// vertices, and S.vmap (each vertex's cube and edge) when the brick has at
// most 2048 of them.  Called by
// every thread (contains __syncthreads); the list is valid after return.
template <int VT, class Smem>
__device__ __forceinline__ void occupied_list(Smem &S, const typename Vox<VT>::T *tile, int nx, int ny, int zlim,
                                              int x0, int y0, int z0) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
        // occupied cubes of the brick, from row masks (voxel rows y0..y0+8, z0..z0+8)
        if (tid < ROWS) {
            const int ry = tid % (BY + 1), rz = tid / (BY + 1);
            RowMask<VT>::build(tile + tidx(TXO, ry + TYO, rz + TZO), S.neg[tid], S.dead[tid]);
        }
        __syncthreads();
        CubeRow cr;
        cr.occ = 0;
        unsigned int cnt = 0, vsum = 0;
        if (tid < CUBE_ROWS) {
            const int cy = tid & (BY - 1), cz = tid / BY;
            if (y0 + cy < ny - 1 && z0 + cz < zlim) cr = cube_row(S.neg, S.dead, cy, cz, valid_mask(x0, nx));
            cnt = __popc(cr.occ);
            unsigned int m = cr.occ;
            while (m) {
                const int x = __ffs(m) - 1;
                m &= m - 1;
                vsum += S.nv[cube_index(cr, x)];
            }
            // exclusive scans over the 64 cube rows (row = tid, (z, y) order)
            unsigned int ic = cnt, iv = vsum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int a = __shfl_up_sync(0xffffffffu, ic, o);
                const unsigned int c = __shfl_up_sync(0xffffffffu, iv, o);
                if (lane >= o) { ic += a; iv += c; }
            }
            if (lane == 31) { S.wsum[warp][0] = ic; S.wsum[warp][1] = iv; }
            cnt = ic - cnt;  // now exclusive
            vsum = iv - vsum;
        }
        __syncthreads();
        if (tid < CUBE_ROWS) {
            if (warp == 1) { cnt += S.wsum[0][0]; vsum += S.wsum[0][1]; }
            const int cy = tid & (BY - 1), cz = tid / BY;
            unsigned int m = cr.occ;
            while (m) {
                const int x = __ffs(m) - 1;
                m &= m - 1;
                const unsigned int ci = cube_index(cr, x);
                S.occ_cube[cnt] = (unsigned short)((cz * BY + cy) * BX + x);
                S.occ_ci[cnt] = (unsigned char)ci;
                S.occ_off[cnt] = (unsigned short)vsum;
                ++cnt;
                vsum += S.nv[ci];
            }
            if (tid == 0) {
                S.nocc = S.wsum[0][0] + S.wsum[1][0];
                S.total = S.wsum[0][1] + S.wsum[1][1];
            }
        }
        __syncthreads();
        // vertex -> (cube, edge) map, one occupied cube per thread (a row per
        // thread would serialise up to 32 x 15 writes): entry = local cube
        // index << 4 | edge, the edge of output slot k of triangle j being
        // tri[3j + 2 - k] (cu_marching_cubes_v1.cu:322-333); cube offsets are
        // multiples of 3, so a vertex's slot is its index mod 3
        if (S.total <= BRICK_CUBES) {
            const unsigned int nocc = S.nocc;
            for (unsigned int i = tid; i < nocc; i += THREADS) {
                const unsigned int off = S.occ_off[i], ci = S.occ_ci[i], nvc = S.nv[ci];
                const unsigned int cbits = (unsigned int)S.occ_cube[i] << 4;
                const uint4 row = *reinterpret_cast<const uint4 *>(S.tri[ci]);
                for (unsigned int q = 0; q < nvc; ++q) {
                    const unsigned int j = q / 3, k = q - 3 * j, slot = 3 * j + 2 - k;
                    const unsigned int word = slot < 4 ? row.x : slot < 8 ? row.y : slot < 12 ? row.z : row.w;
                    const unsigned int e = (word >> (8 * (slot & 3))) & 0xffu;
                    S.vmap[off + q] = (unsigned short)(cbits | e);
                }
            }
            __syncthreads();
        }
}

template <int VT, class Smem>
__device__ __forceinline__ void generate_brick(Smem &S, const typename Vox<VT>::T *tile,
                                               const typename Vox<VT>::T *__restrict__ vol, int nx, int ny,
                                               int nz, float cell, int x0, int y0, int z0,
                                               unsigned long long vbase, const GenOut &o) {
    using V = Vox<VT>;
    using T = typename V::T;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long N = (long long)nx * ny * nz;

        occupied_list<VT>(S, tile, nx, ny, o.zlim, x0, y0, z0);
        const unsigned int nocc = S.nocc, T_brick = S.total;
        const bool use_map = T_brick <= BRICK_CUBES;

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
                // owning cube and edge: the map, or the last list entry with off <= v
                int c, e;
                if (use_map) {
                    const unsigned int w = S.vmap[v];
                    c = (int)(w >> 4);
                    e = (int)(w & 15u);
                    kslot = (int)(v % 3u);
                } else {
                    int lo = 0, hi = (int)nocc - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (S.occ_off[mid] <= v) lo = mid; else hi = mid - 1;
                    }
                    c = S.occ_cube[lo];
                    const unsigned int ci = S.occ_ci[lo];
                    const unsigned int sl = v - S.occ_off[lo];
                    const unsigned int j = sl / 3, k = sl - 3 * j;
                    kslot = (int)k;
                    // output slot k of triangle j takes edge tri[3j+2-k] (:322-333)
                    e = S.tri[ci][3 * j + 2 - k];
                }
                const int lcx = c & (BX - 1), lcy = (c / BX) & (BY - 1), lcz = c / (BX * BY);
                const int a = c_ea(e), bb = c_eb(e);
                const int gx = x0 + lcx, gy = y0 + lcy, gz = z0 + lcz;
                if (o.tri_cube) cube_lin = lin3(nx, ny, gx, gy, gz);
                const float f0 =
                    V::f(tile[tidx(lcx + TXO + c_cx(a), lcy + TYO + c_cy(a), lcz + TZO + c_cz(a))]);
                const float f1 =
                    V::f(tile[tidx(lcx + TXO + c_cx(bb), lcy + TYO + c_cy(bb), lcz + TZO + c_cz(bb))]);
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
                const int org[3] = {x0 - TXO, y0 - TYO, z0 - TZO};
                const int tdim[3] = {TX, TY, TZ};
                // P / cell serves both the voxel (:344-350) and the normal sample (kf.cu:3241)
                const float pf[3] = {P[0] / cell, P[1] / cell, P[2] / cell};
                bool inside = true;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    vox[d] = (int)floorf(pf[d] - 0.5f);
                    inside &= vox[d] >= 0 && vox[d] < dims[d] && vox[d] - org[d] >= 0 && vox[d] - org[d] < tdim[d];
                }
                if (inside) {
                    const T vv = tile[tidx(vox[0] - org[0], vox[1] - org[1], vox[2] - org[2])];
                    vt = V::tsdf(vv);
                    vw = V::wt(vv);
                }
                if (!inside || o.ver_voxel) {
                    const long long li = lin3(nx, ny, vox[0], vox[1], vox[2]);
                    if (!inside && li >= 0 && li < N) {
                        const T vv = vol[li];
                        vt = V::tsdf(vv);
                        vw = V::wt(vv);
                    }
                    if (o.ver_voxel && li >= 0 && li < N && vbase + v < (unsigned long long)o.cap)
                        o.ver_voxel[li] = vt;
                }
                if (o.normals) {
                    const float fx = pf[0], fy = pf[1], fz = pf[2];
                    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
                    const int lx = ix - org[0], ly = iy - org[1], lz = iz - org[2];
                    if (ix + 1 < nx && iy + 1 < ny && iz + 1 < nz && lx >= 0 && ly >= 0 && lz >= 0 &&
                        lx + 1 < TX && ly + 1 < TY && lz + 1 < TZ) {
                        const T smp[8] = {tile[tidx(lx, ly, lz)],         tile[tidx(lx + 1, ly, lz)],
                                          tile[tidx(lx + 1, ly + 1, lz)], tile[tidx(lx, ly + 1, lz)],
                                          tile[tidx(lx, ly, lz + 1)],     tile[tidx(lx + 1, ly, lz + 1)],
                                          tile[tidx(lx + 1, ly + 1, lz + 1)], tile[tidx(lx, ly + 1, lz + 1)]};
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
            const long long room = o.cap - (long long)g0;
            const int nrec = (int)min((long long)min(32u, T_brick - v0), room > 0 ? room : 0ll);
            unsigned int *st = S.stage[warp];
            if (o.soup) {
                st[lane * 7 + 0] = __float_as_uint(P[0]);
                st[lane * 7 + 1] = __float_as_uint(P[1]);
                st[lane * 7 + 2] = __float_as_uint(P[2]);
                st[lane * 7 + 3] = (unsigned int)vox[0];
                st[lane * 7 + 4] = (unsigned int)vox[1];
                st[lane * 7 + 5] = (unsigned int)vox[2];
                st[lane * 7 + 6] = (unsigned int)(unsigned short)vt | ((unsigned int)(unsigned short)vw << 16);
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(o.soup) + g0 * 7;
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 7) dst[word] = st[word];
                }
                __syncwarp();
            }
            if (o.normals) {
                st[lane * 3 + 0] = __float_as_uint(nrm.x);
                st[lane * 3 + 1] = __float_as_uint(nrm.y);
                st[lane * 3 + 2] = __float_as_uint(nrm.z);
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(o.normals) + g0 * 3;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 3) dst[word] = st[word];
                }
                __syncwarp();
            }
            if (o.vi2vox) {
                st[lane * 3 + 0] = (unsigned int)vox[0];
                st[lane * 3 + 1] = (unsigned int)vox[1];
                st[lane * 3 + 2] = (unsigned int)vox[2];
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(o.vi2vox) + g0 * 3;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 3) dst[word] = st[word];
                }
                __syncwarp();
            }
            // a triangle's cube id is written only when the whole triangle fits
            if (o.tri_cube && valid && kslot == 0 && (long long)(g0 + lane) + 2 < o.cap)
                o.tri_cube[(g0 + lane) / 3] = cube_lin;
        }
}

// Adjoint of the soup positions with respect to the voxel values, for one
// brick whose tile is in shared memory.  Soup vertex v of the brick lies on
// edge (a, b) of its cube: P = p_a + t (p_b - p_a), t = -f_a / D,
// D = f_b - f_a + 1e-15 (cu_marching_cubes_v1.cu:256-264), so
//   dL/df_a += (dL/dP . (p_b - p_a)) * -(f_b + 1e-15) / D^2
//   dL/df_b += (dL/dP . (p_b - p_a)) *  f_a / D^2
// accumulated in FP32 with atomics (a voxel is shared by up to 6 edges).
// Called by every thread (contains __syncthreads).
template <int VT, class Smem>
__device__ __forceinline__ void backward_brick(Smem &S, const typename Vox<VT>::T *tile, int nx, int ny,
                                               int nz, int zlim, float cell, int x0, int y0, int z0,
                                               unsigned long long vbase,
                                               const float *__restrict__ grad_pos, float *__restrict__ grad_f,
                                               long long n_grad) {
    using V = Vox<VT>;
    const int tid = threadIdx.x;
    occupied_list<VT>(S, tile, nx, ny, zlim, x0, y0, z0);
    const unsigned int nocc = S.nocc, T_brick = S.total;
    const bool use_map = T_brick <= BRICK_CUBES;
    for (unsigned int v = tid; v < T_brick; v += THREADS) {
        const unsigned long long gv = vbase + v;
        if ((long long)gv >= n_grad) break;
        int c, e;
        if (use_map) {
            const unsigned int w = S.vmap[v];
            c = (int)(w >> 4);
            e = (int)(w & 15u);
        } else {
            int lo = 0, hi = (int)nocc - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (S.occ_off[mid] <= v) lo = mid; else hi = mid - 1;
            }
            c = S.occ_cube[lo];
            const unsigned int ci = S.occ_ci[lo];
            const unsigned int sl = v - S.occ_off[lo];
            const unsigned int j = sl / 3, k = sl - 3 * j;
            e = S.tri[ci][3 * j + 2 - k];
        }
        const int lcx = c & (BX - 1), lcy = (c / BX) & (BY - 1), lcz = c / (BX * BY);
        const int a = c_ea(e), bb = c_eb(e);
        const float f0 = V::f(tile[tidx(lcx + TXO + c_cx(a), lcy + TYO + c_cy(a), lcz + TZO + c_cz(a))]);
        const float f1 = V::f(tile[tidx(lcx + TXO + c_cx(bb), lcy + TYO + c_cy(bb), lcz + TZO + c_cz(bb))]);
        const int gx = x0 + lcx, gy = y0 + lcy, gz = z0 + lcz;
        const int ga[3] = {gx + c_cx(a), gy + c_cy(a), gz + c_cz(a)};
        const int gb[3] = {gx + c_cx(bb), gy + c_cy(bb), gz + c_cz(bb)};
        float g = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float p0 = ((float)ga[d] + 0.5f) * cell;
            const float p1 = ((float)gb[d] + 0.5f) * cell;
            g += grad_pos[3 * gv + d] * (p1 - p0);
        }
        const float D = f1 - f0 + 1e-15f;
        const float inv = 1.0f / (D * D);
        atomicAdd(&grad_f[lin3(nx, ny, ga[0], ga[1], ga[2])], g * (-(f1 + 1e-15f) * inv));
        atomicAdd(&grad_f[lin3(nx, ny, gb[0], gb[1], gb[2])], g * (f0 * inv));
    }
}

template <int VT, bool TMA, int MODE>
__global__ void __launch_bounds__(THREADS, GEN_MINB) mc_generate_kernel(const __grid_constant__ CUtensorMap map, GenParams p) {
    using V = Vox<VT>;
    using T = typename V::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    GenSmem<VT, GEN_STAGES> &S = *reinterpret_cast<GenSmem<VT, GEN_STAGES> *>(smem_raw);
    const T *__restrict__ vol = static_cast<const T *>(p.vol);
    const int tid = threadIdx.x;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const float cell = p.cell;

    load_tri_table(S.tri, tid, THREADS);
    S.nv[tid] = (tid == 0 || tid == 255) ? 0 : g_nverts[tid];
    if (tid == 0) {
        S.abort = 0;
        if (TMA) {
            for (int s = 0; s < GEN_STAGES; ++s) mbar_init(&S.bars[s], 1);
            fence_barrier_init();
        }
    }
    __syncthreads();
    pdl_wait();  // the scan's list, offsets and totals
    const unsigned int nactive = p.totals->active_bricks;
    unsigned int *ticket = &p.totals->gen_ticket;
    // stage st <- brick b (soup offset v): thread 0 records the brick, its
    // offset and origin for the CTA and starts the tile load
    auto stage_brick = [&](int st, long long b, unsigned long long v) {
        S.sbrick[st] = b;
        if (b < 0) return;
        S.svbase[st] = v;
        const BrickPos bp = slab_pos(b, p.nbx, p.nby, p.zbase);
        S.spos[st] = make_int4(bp.x0, bp.y0, bp.z0, 0);
        mbar_arrive_expect_tx(&S.bars[st], GTILE * V::bytes);
        tma_load_3d(S.tiles[st], &map, &S.bars[st], bp.x0 - TXO, bp.y0 - TYO, bp.z0 - TZO);
    };
    // The first GEN_STAGES + 1 bricks of each CTA are fixed: round r gives list
    // entry r * grid + c to CTA c, c counted backwards in odd rounds, so the
    // heaviest bricks at the head of the list spread over all CTAs with the
    // heaviest and lightest of adjacent rounds paired.  Later bricks come from
    // the counter, past those rounds.
    //
    // Thread 0's refill pipeline: the ticket for a refill is drawn at the top
    // of the brick before, and its list entry and soup offset are copied
    // (asynchronously, into shared memory) at that brick's end, to be staged
    // at the end of the next brick.  Each result is used a whole brick after
    // it was asked for, so no refill waits on the contended counter or on
    // global memory (a wait in warp 0 would hold the whole CTA at its next
    // barrier).
    const unsigned int grid = gridDim.x, c = blockIdx.x;
    const unsigned int nfix = p.fixed_rounds;
    const unsigned int tbase = nfix * grid;  // list entry of ticket 0
    // list entry of this CTA's k-th brick: fixed rounds first, then the counter
    auto next_entry = [&](unsigned int k) {
        return k < nfix ? k * grid + ((k & 1) ? grid - 1 - c : c) : tbase + atomicAdd(ticket, 1u);
    };
    unsigned int ptk = 0xffffffffu;  // list entry of the ticket drawn at the top of this brick
    unsigned int kdraw = GEN_STAGES + 1;  // entries assigned so far (thread 0)
    if (TMA && tid == 0) {
        unsigned int wr[GEN_STAGES + 1];
#pragma unroll
        for (unsigned int r = 0; r <= GEN_STAGES; ++r) wr[r] = next_entry(r);
#pragma unroll
        for (int r = 0; r < GEN_STAGES; ++r) {
            const unsigned int w = wr[r];
            stage_brick(r, w < nactive ? (long long)p.active[w] : -1ll, w < nactive ? p.list_vofs[w] : 0ull);
        }
        const unsigned int w = wr[GEN_STAGES];
        S.pipe_b = 0xffffffffu;
        if (w < nactive) {
            cp_async_4(&S.pipe_b, p.active + w);
            cp_async_8(&S.pipe_v, p.list_vofs + w);
        }
        if (w < nactive) ptk = 0;  // not ~0u: draw tickets at the tops of the bricks
    }
    if (TMA) __syncthreads();
    for (int it = 0;; ++it) {
        const int s = TMA ? it % GEN_STAGES : 0;
        const T *tile = reinterpret_cast<const T *>(S.tiles[s]);
        long long b;
        unsigned long long vbase;
        BrickPos bp;
        if (TMA) {
            b = S.sbrick[s];
            if (b < 0) break;  // uniform
            if (tid == 0) {
                // the ticket of the refill after the next one (used at this brick's end)
                if (ptk != 0xffffffffu) ptk = next_entry(kdraw++);
                if (!mbar_wait(&S.bars[s], (uint32_t)((it / GEN_STAGES) & 1))) S.abort = 1;
            }
            __syncthreads();
            if (S.abort) break;
            vbase = S.svbase[s];
            const int4 sp = S.spos[s];
            bp.x0 = sp.x;
            bp.y0 = sp.y;
            bp.z0 = sp.z;
        } else {
            if (tid == 0) {
                const long long w = next_brick(ticket, nactive);
                S.sbrick[0] = w >= 0 ? (long long)p.active[w] : -1ll;
            }
            __syncthreads();
            b = S.sbrick[0];
            if (b < 0) break;
            vbase = p.brick_vofs[b];
            bp = slab_pos(b, p.nbx, p.nby, p.zbase);
            fill_tile<VT, TX, TY, TZ>(reinterpret_cast<T *>(S.tiles[s]), vol, nx, ny, nz, bp.x0 - TXO,
                                      bp.y0 - TYO, bp.z0 - TZO);
            __syncthreads();
        }
        if (MODE == 0) {
            GenOut o;
            o.soup = p.soup;
            o.normals = p.normals;
            o.vi2vox = p.vi2vox;
            o.ver_voxel = p.ver_voxel;
            o.tri_cube = p.tri_cube;
            o.cap = p.cap;
            o.zlim = p.zlim;
            generate_brick<VT>(S, tile, vol, nx, ny, nz, cell, bp.x0, bp.y0, bp.z0, vbase, o);
        } else {
            backward_brick<VT>(S, tile, nx, ny, nz, p.zlim, cell, bp.x0, bp.y0, bp.z0, vbase, p.grad_pos,
                               p.grad_f, p.n_grad);
        }
        __syncthreads();  // tile s, the list and the stage are free again
        if (TMA && tid == 0) {
            cp_async_wait_all();
            const unsigned int pb = S.pipe_b;
            stage_brick(s, pb == 0xffffffffu ? -1ll : (long long)pb, S.pipe_v);
            S.pipe_b = 0xffffffffu;
            if (ptk < nactive) {
                cp_async_4(&S.pipe_b, p.active + ptk);
                cp_async_8(&S.pipe_v, p.list_vofs + ptk);
            } else {
                ptk = 0xffffffffu;  // the list is exhausted: draw no more tickets
            }
        }
        // S.sbrick[s] is next read at the top of iteration it + GEN_STAGES, after the
        // barriers of iteration it + 1 (with one stage: after this barrier)
        if (GEN_STAGES == 1) __syncthreads();
    }
    if (S.abort && tid == 0) {
        atomicOr(&p.totals->flags, 1u);
        for (int s = 0; s < GEN_STAGES; ++s) mbar_wait(&S.bars[s], 0, 100000000ull);
    }
    // the last CTA out resets the work counter for the next launch over the
    // same list and reports the flags to the host copy
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&p.totals->gen_exit, 1u) == gridDim.x - 1) {
            p.totals->gen_ticket = 0;
            p.totals->gen_exit = 0;
            if (p.host) {  // onto the count phase's flags in the host copy
                p.host->flags |= *(volatile unsigned int *)&p.totals->flags;
                p.totals->flags = 0;
                __threadfence_system();
            }
        }
    }
}


// ---- fused extraction: count, offsets and generation in one persistent launch ----
// The count pass already holds every brick's voxels in shared memory and has
// classified its cubes; the fused kernel generates a work item's triangles
// right there, instead of a scan launch and a generate launch that fetch the
// active bricks again and rebuild their occupied-cube lists.  A work item is
// FG bricks adjacent in x; its tile holds their voxels plus one voxel column
// and one row / plane of y / z halo beyond what the cubes need, because the
// normals sample one voxel further (cu_kinect_fusion_v1.cu:3152-3194).
//
// Soup offsets come from a decoupled look-back over the items in ticket
// order, at two levels.  An item publishes its triangle count as soon as it
// is classified.  Items form groups of FGROUP; the last item of a group sums
// the group's counts and publishes that aggregate, then looks back over the
// groups before it and publishes the group's inclusive prefix.  An item that
// emits triangles sums the counts before it in its own group and looks back
// over the groups before: a warp reads the states of 32 groups at once, the
// nearest inclusive prefix ends the walk and the aggregates after it are
// added.  Items are drawn in order by running CTAs, and neither a count nor
// an aggregate waits for anything but earlier items, so every wait ends
// (each is bounded by %globaltimer all the same).  The output order is the
// one of the two-launch path: bricks in (bz, by, bx) order, cubes in (z, y, x)
// order inside a brick, table slot order inside a cube.
// Item geometry for FG bricks per item (4: 132-voxel tiles, 256 threads;
// 2: 68-voxel tiles, 128 threads): one thread per cube row of the item.
constexpr int FTY = BY + 2, FTZ = BZ + 2;    // 10 x 10 rows
constexpr int FGROUP = 32;                   // items per look-back group
template <int FG>
struct FGeo {
    static constexpr int TX = BX * FG + 4;   // voxels in x
    static constexpr int TILE = TX * FTY * FTZ;
    static constexpr int NT = FG * CUBE_ROWS; // threads = cube rows per item
    static constexpr int NWARP = NT / 32;
};

template <int VT, int FG>
struct FusedSmem {
    static constexpr int NT = FGeo<FG>::NT, WARPS = FGeo<FG>::NWARP, FROWS = NT;
    static constexpr int TILE_BYTES = pad128(FGeo<FG>::TILE * Vox<VT>::bytes);
    unsigned char tile[TILE_BYTES];
    unsigned long long neg[FG * ROWS];           // row masks of the item's bricks, [brick][row]
    union {
        unsigned long long dead[FG * ROWS];      // classification only
        unsigned int stage[WARPS][32 * 7];       // emission only: per-warp store staging
    };
    unsigned int rowocc[FROWS];                  // occupied cubes of each cube row (bit x)
    unsigned int rownib[FROWS][4];               // soup vertices of each cube of the row, 4 bits each
    unsigned int rowoff[FROWS + 1];              // exclusive vertex offset of each row in the item; [FROWS]: total
    alignas(16) signed char tri[256][16];
    unsigned char nv[256];
    uint64_t bar;
    int4 sorg;                                   // item origin {x0, y0, z0, first brick x}; x0 < 0: none
    int sitem;                                   // item number
    unsigned long long base;                     // soup offset (vertices) of the item
    unsigned int wsum[WARPS];
    unsigned int red[WARPS];
    unsigned int mix[WARPS];
    int abort;
};

struct FusedParams {
    const void *vol;
    int nx, ny, nz;
    float cell;
    int nbx, nby;
    int nitems, ngx, zlim;
    unsigned long long *item;   // per item: epoch << 32 | (triangles + 1)
    unsigned long long *group;  // per group of FGROUP items: group_word(epoch, kind, value)
    unsigned int epoch;         // 1 .. 2^22 - 1
    MeshTotals *totals;
    MeshTotals *host;           // mapped host copy, or null
    GenOut out;
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Triangle count of item j of this launch, waiting (bounded) until it is
// published; false on timeout.
__device__ __forceinline__ bool item_count(const FusedParams &p, int j, unsigned int &tris) {
    const unsigned long long *q = p.item + j;
    unsigned long long v = ld_relaxed_u64(q);
    if ((unsigned int)(v >> 32) != p.epoch) {
        const unsigned long long t0 = globaltimer_ns();
        do {
            if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
            v = ld_relaxed_u64(q);
        } while ((unsigned int)(v >> 32) != p.epoch);
    }
    tris = (unsigned int)v - 1u;
    return true;
}

// Group state word: epoch << 42 | kind << 40 | value, kind 1 = the group's
// triangle total (aggregate), 2 = the inclusive prefix through the group.
constexpr int FX_EPOCH_BITS = 22;
constexpr unsigned long long FX_VALUE_MASK = (1ull << 40) - 1ull;
__device__ __forceinline__ unsigned long long group_word(unsigned int epoch, unsigned int kind,
                                                         unsigned long long value) {
    return ((unsigned long long)epoch << 42) | ((unsigned long long)kind << 40) | (value & FX_VALUE_MASK);
}

// State of group h once it holds at least its aggregate (bounded wait);
// false on timeout.
__device__ __forceinline__ bool group_state(const FusedParams &p, int h, unsigned int &kind,
                                            unsigned long long &value) {
    const unsigned long long *q = p.group + h;
    unsigned long long v = ld_relaxed_u64(q);
    if ((unsigned int)(v >> 42) != p.epoch) {
        const unsigned long long t0 = globaltimer_ns();
        do {
            if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
            v = ld_relaxed_u64(q);
        } while ((unsigned int)(v >> 42) != p.epoch);
    }
    kind = (unsigned int)(v >> 40) & 3u;
    value = v & FX_VALUE_MASK;
    return true;
}

// Triangles of all groups before group g (called by one whole warp): windows
// of 32 groups, one per lane; the nearest group holding an inclusive prefix
// ends the walk, the aggregates of the groups after it are added.  False on
// a timeout.
__device__ bool groups_before(const FusedParams &p, int g, unsigned long long &sum) {
    const int lane = threadIdx.x & 31;
    bool ok = true;
    sum = 0;
    for (int h = g - 1; h >= 0; h -= 32) {
        const int hh = h - lane;
        unsigned int kind = 2;  // before group 0: an inclusive prefix of 0
        unsigned long long val = 0;
        if (hh >= 0) ok = group_state(p, hh, kind, val) && ok;
        const unsigned int pref = __ballot_sync(0xffffffffu, kind == 2u || !ok);
        unsigned long long a = (pref == 0u || lane <= __ffs(pref) - 1) ? val : 0ull;
#pragma unroll
        for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        sum += a;
        if (pref) break;
    }
    return __all_sync(0xffffffffu, ok);
}

// Triangles of the items of `it`'s group that come before it (one whole warp).
__device__ bool items_before(const FusedParams &p, int it, unsigned long long &sum) {
    const int lane = threadIdx.x & 31;
    const int first = (it / FGROUP) * FGROUP;
    bool ok = true;
    unsigned long long v = 0;
    if (lane < it - first) {
        unsigned int t = 0;
        ok = item_count(p, first + lane, t);
        v = t;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    sum = v;
    return __all_sync(0xffffffffu, ok);
}

// True when the item's voxels hold both signs; contains a barrier.  An item
// whose classification region (voxel rows y0 .. y0+8 of planes z0 .. z0+8,
// all 132 columns) lies inside the volume tests every 16-byte word of its
// tile in one contiguous sweep -- the extra row and plane the normals need
// can only turn a one-signed item into a "mixed" one, which costs the full
// classification but changes no count.  Items at the volume's end test only
// their words inside the volume (rows and columns beyond it arrive
// zero-filled and would make an all-negative border item mixed).
template <int VT, int FG, class Smem>
__device__ __forceinline__ bool fused_mixed(Smem &S, const typename Vox<VT>::T *tile, int nx, int ny, int nz,
                                            int x0, int y0, int z0) {
    using V = Vox<VT>;
    constexpr int FTX = FGeo<FG>::TX, THREADS = FGeo<FG>::NT, WARPS = FGeo<FG>::NWARP;
    constexpr int WPR = FTX * V::bytes / 16;  // 16-byte words per row
    constexpr int VPW = 16 / V::bytes;
    constexpr int NW = FGeo<FG>::TILE * V::bytes / 16;
    const uint4 *q = reinterpret_cast<const uint4 *>(tile);
    unsigned int neg_any = 0, pos_any = 0;
    auto acc = [&](const uint4 v) {
        if (VT == MCG_VOXEL_SHORT2) {
            // bit 15 of each word is the tsdf sign
            neg_any |= v.x | v.y | v.z | v.w;
            pos_any |= ~(v.x & v.y & v.z & v.w);
        } else {
            // x and z are the tsdf of two voxels; -0.0f is not negative
            const bool n0 = __uint_as_float(v.x) < 0.f, n1 = __uint_as_float(v.z) < 0.f;
            neg_any |= (unsigned int)(n0 | n1) << 15;
            pos_any |= (unsigned int)(!n0 | !n1) << 15;
        }
    };
    if (x0 + FTX <= nx && y0 + CTY <= ny && z0 + CTZ <= nz) {
        int i = threadIdx.x;
        for (; i + THREADS < NW; i += 2 * THREADS) {
            const uint4 a = q[i], b = q[i + THREADS];
            acc(a);
            acc(b);
        }
        if (i < NW) acc(q[i]);
    } else {
        const int ry = ny - y0, rz = nz - z0, rx = nx - x0;
        for (int i = threadIdx.x; i < WPR * ROWS; i += THREADS) {
            const int r = i / WPR, w = i - r * WPR, lx = w * VPW;
            const int lz = r / CTY, ly = r - lz * CTY;  // rows 0..8 of planes 0..8
            if (ly >= ry || lz >= rz || lx >= rx) continue;
            acc(q[(lz * FTY + ly) * WPR + w]);
        }
    }
    neg_any = __reduce_or_sync(0xffffffffu, neg_any & 0x8000u);
    pos_any = __reduce_or_sync(0xffffffffu, pos_any & 0x8000u);
    if ((threadIdx.x & 31) == 0) S.mix[threadIdx.x >> 5] = (neg_any ? 1u : 0u) | (pos_any ? 2u : 0u);
    __syncthreads();
    unsigned int m = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) m |= S.mix[w];
    return m == 3u;
}

template <int FG>
__device__ __forceinline__ int ftidx(int lx, int ly, int lz) { return (lz * FTY + ly) * FGeo<FG>::TX + lx; }

template <int VT, int FG, int MINB>
__global__ void __launch_bounds__(FGeo<FG>::NT, MINB) mc_fused_kernel(const __grid_constant__ CUtensorMap map,
                                                                        FusedParams p) {
    using V = Vox<VT>;
    using T = typename V::T;
    constexpr int FTX = FGeo<FG>::TX, FTILE = FGeo<FG>::TILE, THREADS = FGeo<FG>::NT, WARPS = FGeo<FG>::NWARP;
    constexpr int FROWS = THREADS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    FusedSmem<VT, FG> &S = *reinterpret_cast<FusedSmem<VT, FG> *>(smem_raw);
    const T *__restrict__ vol = static_cast<const T *>(p.vol);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const float cell = p.cell;
    const GenOut &o = p.out;
    const long long N = (long long)nx * ny * nz;
    load_tri_table(S.tri, tid, THREADS);
    for (int c = tid; c < 256; c += THREADS) S.nv[c] = (c == 0 || c == 255) ? 0 : g_nverts[c];
    pdl_wait();  // the launch before (a writer of the volume or of the counters)
    unsigned int *ticket = &p.totals->cls_ticket;
    // thread 0: item -> origin and TMA load of its tile
    auto stage_item = [&](int it) {
        S.sitem = it;
        if (it < 0) {
            S.sorg = make_int4(-1, 0, 0, 0);
            return;
        }
        const unsigned int r = (unsigned int)it / (unsigned int)p.ngx;
        const int bx0 = (int)((unsigned int)it - r * (unsigned int)p.ngx) * FG;
        const int y0 = (int)(r % (unsigned int)p.nby) * BY, z0 = (int)(r / (unsigned int)p.nby) * BZ;
        const int x0 = bx0 * BX;
        S.sorg = make_int4(x0, y0, z0, bx0);
        mbar_arrive_expect_tx(&S.bar, FTILE * V::bytes);
        tma_load_3d(S.tile, &map, &S.bar, x0, y0, z0);
    };
    // Thread 0 draws the next item only when its tile can be loaded: a CTA
    // never holds an item it has not started, so an item's count is
    // published a tile load and a classification after it was drawn, never
    // after another item's look-back or emission (which could chain waits
    // across CTAs).
    auto refill = [&]() {
        const unsigned int t = atomicAdd(ticket, 1u);
        stage_item(t < (unsigned int)p.nitems ? (int)t : -1);
    };
    if (tid == 0) {
        S.abort = 0;
        mbar_init(&S.bar, 1);
        fence_barrier_init();
        refill();
    }
    __syncthreads();
    const T *tile = reinterpret_cast<const T *>(S.tile);
    // thread 0: this CTA's contributions to the totals
    unsigned long long my_occ = 0, my_tris = 0;
    unsigned int my_active = 0;
    for (int i = 0;; ++i) {
        const int4 org = S.sorg;
        const int it = S.sitem;
        if (org.x < 0) break;  // uniform
        const int x0 = org.x, y0 = org.y, z0 = org.z, bx0 = org.w;
        if (tid == 0 && !mbar_wait(&S.bar, (uint32_t)(i & 1))) S.abort = 1;
        __syncthreads();
        if (S.abort) break;
        const bool mixed = fused_mixed<VT, FG>(S, tile, nx, ny, nz, x0, y0, z0);
        unsigned int item_v = 0;  // soup vertices of the item
        if (mixed) {
            // row masks of the FG bricks (voxel rows y0..y0+8, z0..z0+8)
            for (int m = tid; m < FG * ROWS; m += THREADS) {
                const int h = m / ROWS, r = m - h * ROWS, rz = r / CTY, ry = r - rz * CTY;
                const T *row = tile + ftidx<FG>(h * BX, ry, rz);
                RowMask<VT>::build(row, row[BX], S.neg[m], S.dead[m]);
            }
            __syncthreads();
            // one cube row per thread: occupancy, vertices per cube, row total
            const int h = tid / CUBE_ROWS, c = tid - h * CUBE_ROWS, cy = c & (BY - 1), cz = c / BY;
            unsigned int occ = 0, rv = 0, nib[4] = {0u, 0u, 0u, 0u};
            if (bx0 + h < p.nbx && y0 + cy < ny - 1 && z0 + cz < p.zlim) {
                const CubeRow cr =
                    cube_row(S.neg + h * ROWS, S.dead + h * ROWS, cy, cz, valid_mask(x0 + h * BX, nx));
                occ = cr.occ;
                unsigned int mm = occ;
                while (mm) {
                    const int x = __ffs(mm) - 1;
                    mm &= mm - 1;
                    const unsigned int n = S.nv[cube_index(cr, x)];
                    nib[x >> 3] |= n << ((x & 7) * 4);
                    rv += n;
                }
            }
            S.rowocc[tid] = occ;
#pragma unroll
            for (int k = 0; k < 4; ++k) S.rownib[tid][k] = nib[k];
            // exclusive scan of the row totals over the item (rows in soup order)
            unsigned int incl = rv;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned int u = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += u;
            }
            const unsigned int wocc = __reduce_add_sync(0xffffffffu, (unsigned int)__popc(occ));
            if (lane == 31) S.wsum[warp] = incl;
            if (lane == 0) S.red[warp] = wocc;
            __syncthreads();
            unsigned int before = 0;
            for (int w = 0; w < warp; ++w) before += S.wsum[w];
            S.rowoff[tid] = before + incl - rv;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) item_v += S.wsum[w];
            if (tid == 0) {
                // totals: occupied cubes, triangles, bricks with triangles (two warps per brick)
                unsigned int o8 = 0, act = 0;
                for (int w = 0; w < WARPS; ++w) o8 += S.red[w];
                for (int b = 0; b < FG; ++b) act += (S.wsum[2 * b] + S.wsum[2 * b + 1]) ? 1u : 0u;
                my_occ += o8;
                my_tris += item_v / 3u;
                my_active += act;
            }
        }
        const bool emit = item_v != 0;
        // publish the item's count; the last item of each group also publishes
        // the group's aggregate and, once it has looked back, its inclusive
        // prefix; items that emit look back for their soup offset
        if (warp == 0) {
            const unsigned int tris = item_v / 3u;
            if (lane == 0)
                st_relaxed_u64(p.item + it, ((unsigned long long)p.epoch << 32) | (unsigned long long)(tris + 1u));
            const int g = it / FGROUP;
            const bool last = (it % FGROUP == FGROUP - 1) || it == p.nitems - 1;
            if (emit || last) {
                unsigned long long in_group = 0, before = 0;
                bool ok = items_before(p, it, in_group);
                if (last && lane == 0) st_relaxed_u64(p.group + g, group_word(p.epoch, 1u, in_group + tris));
                ok = groups_before(p, g, before) && ok;
                if (lane == 0) {
                    if (!ok) S.abort = 1;
                    S.base = 3ull * (before + in_group);
                    if (ok && last) st_relaxed_u64(p.group + g, group_word(p.epoch, 2u, before + in_group + tris));
                }
            }
        }
        if (!emit) {
            // nothing to generate: no thread reads the tile any more, refill it now
            if (tid == 0) refill();
            __syncthreads();  // the next item is staged
            continue;
        }
        __syncthreads();  // S.base, the row tables and S.abort
        if (S.abort) break;
        // ---- emission: warps take 32 consecutive soup vertices of the item ----
        const unsigned long long vbase = S.base;
        for (unsigned int v0 = warp * 32; v0 < item_v; v0 += THREADS) {
            const unsigned int v = v0 + lane;
            const bool valid = v < item_v;
            // row of the chunk's first vertex (the same search in every lane)
            int r0 = 0;
            {
                int hi = FROWS - 1;
                while (r0 < hi) {
                    const int mid = (r0 + hi + 1) >> 1;
                    if (S.rowoff[mid] <= v0) r0 = mid; else hi = mid - 1;
                }
            }
            float P[3] = {0.f, 0.f, 0.f};
            int vox[3] = {0, 0, 0};
            short vt = 0, vw = 0;
            float3 nrm = make_float3(0.f, 0.f, 0.f);
            long long cube_lin = 0;
            int kslot = 1;
            if (valid) {
                // the cube row holding vertex v: the last row starting at or
                // before it, scanned forward from the row of the chunk's first
                // vertex (32 consecutive vertices span a few rows)
                int r = r0;
                while (r + 1 < FROWS && S.rowoff[r + 1] <= v) ++r;
                unsigned int j = v - S.rowoff[r];
                // the cube of the row and the vertex's slot in it
                unsigned int mm = S.rowocc[r];
                int x = 0;
                for (;;) {
                    x = __ffs(mm) - 1;
                    const unsigned int n = (S.rownib[r][x >> 3] >> ((x & 7) * 4)) & 15u;
                    if (j < n) break;
                    j -= n;
                    mm &= mm - 1;
                }
                const int h = r / CUBE_ROWS, c = r - h * CUBE_ROWS, cy = c & (BY - 1), cz = c / BY;
                // sign masks only (the weight masks share their storage with the stage)
                const CubeRow cr = cube_row(S.neg + h * ROWS, S.neg + h * ROWS, cy, cz, 0xffffffffu);
                const unsigned int ci = cube_index(cr, x);
                const unsigned int tj = j / 3, k = j - 3 * tj;
                kslot = (int)k;
                // output slot k of triangle tj takes edge tri[3 tj + 2 - k] (:322-333)
                const int e = S.tri[ci][3 * tj + 2 - k];
                const int lcx = h * BX + x, lcy = cy, lcz = cz;  // cube in tile coordinates
                const int a = c_ea(e), bb = c_eb(e);
                const int gx = x0 + lcx, gy = y0 + lcy, gz = z0 + lcz;
                if (o.tri_cube) cube_lin = lin3(nx, ny, gx, gy, gz);
                const float f0 = V::f(tile[ftidx<FG>(lcx + c_cx(a), lcy + c_cy(a), lcz + c_cz(a))]);
                const float f1 = V::f(tile[ftidx<FG>(lcx + c_cx(bb), lcy + c_cy(bb), lcz + c_cz(bb))]);
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
                const int orgv[3] = {x0, y0, z0};
                const int tdim[3] = {FTX, FTY, FTZ};
                const float pf[3] = {P[0] / cell, P[1] / cell, P[2] / cell};
                bool inside = true;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    vox[d] = (int)floorf(pf[d] - 0.5f);
                    inside &= vox[d] >= 0 && vox[d] < dims[d] && vox[d] - orgv[d] >= 0 && vox[d] - orgv[d] < tdim[d];
                }
                if (inside) {
                    const T vv = tile[ftidx<FG>(vox[0] - x0, vox[1] - y0, vox[2] - z0)];
                    vt = V::tsdf(vv);
                    vw = V::wt(vv);
                }
                if (!inside || o.ver_voxel) {
                    const long long li = lin3(nx, ny, vox[0], vox[1], vox[2]);
                    if (!inside && li >= 0 && li < N) {
                        const T vv = vol[li];
                        vt = V::tsdf(vv);
                        vw = V::wt(vv);
                    }
                    if (o.ver_voxel && li >= 0 && li < N && vbase + v < (unsigned long long)o.cap)
                        o.ver_voxel[li] = vt;
                }
                if (o.normals) {
                    const float fx = pf[0], fy = pf[1], fz = pf[2];
                    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
                    const int lx = ix - x0, ly = iy - y0, lz = iz - z0;
                    if (ix + 1 < nx && iy + 1 < ny && iz + 1 < nz && lx >= 0 && ly >= 0 && lz >= 0 &&
                        lx + 1 < FTX && ly + 1 < FTY && lz + 1 < FTZ) {
                        const T smp[8] = {tile[ftidx<FG>(lx, ly, lz)],         tile[ftidx<FG>(lx + 1, ly, lz)],
                                          tile[ftidx<FG>(lx + 1, ly + 1, lz)], tile[ftidx<FG>(lx, ly + 1, lz)],
                                          tile[ftidx<FG>(lx, ly, lz + 1)],     tile[ftidx<FG>(lx + 1, ly, lz + 1)],
                                          tile[ftidx<FG>(lx + 1, ly + 1, lz + 1)], tile[ftidx<FG>(lx, ly + 1, lz + 1)]};
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
            const unsigned long long g0 = vbase + v0;
            const long long room = o.cap - (long long)g0;
            const int nrec = (int)min((long long)min(32u, item_v - v0), room > 0 ? room : 0ll);
            unsigned int *st = S.stage[warp];
            if (o.soup) {
                st[lane * 7 + 0] = __float_as_uint(P[0]);
                st[lane * 7 + 1] = __float_as_uint(P[1]);
                st[lane * 7 + 2] = __float_as_uint(P[2]);
                st[lane * 7 + 3] = (unsigned int)vox[0];
                st[lane * 7 + 4] = (unsigned int)vox[1];
                st[lane * 7 + 5] = (unsigned int)vox[2];
                st[lane * 7 + 6] = (unsigned int)(unsigned short)vt | ((unsigned int)(unsigned short)vw << 16);
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(o.soup) + g0 * 7;
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 7) dst[word] = st[word];
                }
                __syncwarp();
            }
            if (o.normals) {
                st[lane * 3 + 0] = __float_as_uint(nrm.x);
                st[lane * 3 + 1] = __float_as_uint(nrm.y);
                st[lane * 3 + 2] = __float_as_uint(nrm.z);
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(o.normals) + g0 * 3;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 3) dst[word] = st[word];
                }
                __syncwarp();
            }
            if (o.vi2vox) {
                st[lane * 3 + 0] = (unsigned int)vox[0];
                st[lane * 3 + 1] = (unsigned int)vox[1];
                st[lane * 3 + 2] = (unsigned int)vox[2];
                __syncwarp();
                unsigned int *dst = reinterpret_cast<unsigned int *>(o.vi2vox) + g0 * 3;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int word = q * 32 + lane;
                    if (word < nrec * 3) dst[word] = st[word];
                }
                __syncwarp();
            }
            // a triangle's cube id is written only when the whole triangle fits
            if (o.tri_cube && valid && kslot == 0 && (long long)(g0 + lane) + 2 < o.cap)
                o.tri_cube[(g0 + lane) / 3] = cube_lin;
        }
        __syncthreads();  // the tile, the row tables and the stages are free again
        if (tid == 0) refill();
        __syncthreads();  // the next item is staged
    }
    pdl_trigger();
    if (tid == 0) {
        if (S.abort) {
            atomicOr(&p.totals->flags, 1u);
            mbar_wait(&S.bar, 0, 100000000ull);  // give a load still in flight a bounded chance to land
        }
        if (my_tris) atomicAdd(&p.totals->triangles, my_tris);
        if (my_occ) atomicAdd(&p.totals->occupied, my_occ);
        if (my_active) atomicAdd(&p.totals->active_bricks, my_active);
        __threadfence();
        // the last CTA out completes the totals, hands them (and the flags) to
        // the mapped host copy, and leaves the counters clear for the next launch
        if (atomicAdd(&p.totals->gen_exit, 1u) == gridDim.x - 1) {
            MeshTotals *t = p.totals;
            volatile MeshTotals *vt = t;
            const unsigned long long tris = vt->triangles;
            t->vertices = 3ull * tris;
            t->cls_ticket = 0;
            t->gen_exit = 0;
            if (p.host) {
                p.host->occupied = vt->occupied;
                p.host->triangles = tris;
                p.host->vertices = 3ull * tris;
                p.host->active_bricks = vt->active_bricks;
                p.host->flags = vt->flags;
                __threadfence_system();
                t->occupied = 0;
                t->triangles = 0;
                t->vertices = 0;
                t->active_bricks = 0;
                t->flags = 0;
            }
        }
    }
}

// ---- batched extraction: count and generate launches -------------------------------
template <int VT>
struct ClsSmemMulti {
    static constexpr int STAGE_BYTES = pad128(CTILE * Vox<VT>::bytes);
    unsigned char tiles[2][STAGE_BYTES];
    unsigned long long neg[ROWS], dead[ROWS];
    uint64_t bars[2];
    unsigned int red[2][2];
    unsigned int mix[CTHREADS / 32];
    unsigned char ntri[256];
    int svol[2];
    int stma[2];
    int4 spos[2];  // origin of each stage's brick
    long long sb[2];  // brick of each stage, -1: none
    int4 nxt;      // the brick refilled at the end of this iteration: {volume, TMA, origin x, y}
    int nxt_z;
    long long nxt_b;  // its brick id, or -1
    int abort;
};

// volume of the bricks [base, end) that thread 0 resolved last: a CTA's
// bricks are a fixed stride apart, so most lie in the same volume as the one
// before and skip the search
struct VolCache {
    int v = -1;
    long long base = 0, end = 0;
};

__device__ __forceinline__ int cached_volume(VolCache &c, const VolDesc *__restrict__ vols, int nvol, long long b) {
    if (c.v < 0 || b < c.base || b >= c.end) {
        c.v = find_volume(vols, nvol, b);
        c.base = vols[c.v].brick_base;
        c.end = c.base + vols[c.v].nbricks;
    }
    return c.v;
}

template <int VT>
__device__ __forceinline__ void issue_cls_tile(ClsSmemMulti<VT> &S, int s, const VolDesc *__restrict__ vols, int nvol,
                                               const CUtensorMap *maps, long long b, VolCache &vc) {
    const int v = cached_volume(vc, vols, nvol, b);
    S.svol[s] = v;
    S.stma[s] = vols[v].tma;
    const BrickPos bp = brick_pos(b - vc.base, vols[v].nbx, vols[v].nby);
    S.spos[s] = make_int4(bp.x0, bp.y0, bp.z0, 0);
    if (vols[v].tma) {
        mbar_arrive_expect_tx(&S.bars[s], CTILE * Vox<VT>::bytes);
        tma_load_3d(S.tiles[s], maps + v, &S.bars[s], bp.x0, bp.y0, bp.z0);
    }
}

// Count pass over all volumes of a batch, one brick per work item, bricks
// drawn from a counter (`ticket`, zero at launch) so that CTAs whose bricks
// were cheap take more, 2 tile stages: TMA volumes load by TMA, so the next
// tile loads while the current one is classified; the others are filled by
// 16-byte words (fill_tile) when their stage is refilled.  Thread 0 draws
// each refill's ticket one brick before it is used, so no CTA waits on the
// counter.
template <int VT>
__global__ void __launch_bounds__(CTHREADS)
    mc_classify_multi_kernel(const VolDesc *__restrict__ vols, const CUtensorMap *maps, int nvol, long long nbricks,
                             uint32_t *__restrict__ brick_tris, uint32_t *__restrict__ chunk,
                             unsigned long long *__restrict__ vol_sums, unsigned int *__restrict__ flags,
                             unsigned int *__restrict__ ticket) {
    using V = Vox<VT>;
    using T = typename V::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    ClsSmemMulti<VT> &S = *reinterpret_cast<ClsSmemMulti<VT> *>(smem_raw);
    const int tid = threadIdx.x;
    uint32_t phase[2] = {0, 0};
    VolCache vc;
    long long pend = -1;  // thread 0: the brick of the next refill
    for (int c = tid; c < 256; c += CTHREADS) S.ntri[c] = (c == 0 || c == 255) ? 0 : g_nverts[c] / 3;
    if (tid == 0) {
        S.abort = 0;
        for (int s = 0; s < 2; ++s) mbar_init(&S.bars[s], 1);
        fence_barrier_init();
        for (int s = 0; s < 2; ++s) {
            const long long b = (long long)atomicAdd(ticket, 1u);
            S.sb[s] = b < nbricks ? b : -1ll;
            if (b < nbricks) issue_cls_tile<VT>(S, s, vols, nvol, maps, b, vc);
        }
        pend = (long long)atomicAdd(ticket, 1u);
    }
    __syncthreads();
    // the plain-copy fills of the first two stages, one copy group each
    for (int s = 0; s < 2; ++s) {
        if (S.sb[s] >= 0 && !S.stma[s]) {
            const VolDesc &d = vols[S.svol[s]];
            fill_tile<VT, CTX, CTY, CTZ, false>(reinterpret_cast<T *>(S.tiles[s]), static_cast<const T *>(d.data),
                                                d.nx, d.ny, d.nz, S.spos[s].x, S.spos[s].y, S.spos[s].z);
        }
        cp_async_commit();
    }
    for (int i = 0;; ++i) {
        const int s = i & 1;
        // written by thread 0 two iterations back, barriers in between
        const long long b = S.sb[s];
        if (b < 0) break;  // uniform; tickets go to the stages in processing order
        T *tile = reinterpret_cast<T *>(S.tiles[s]);
        const int v = S.svol[s];
        const VolDesc &d = vols[v];
        const int4 sp = S.spos[s];
        BrickPos bp;
        bp.x0 = sp.x;
        bp.y0 = sp.y;
        bp.z0 = sp.z;
        if (S.stma[s]) {
            if (tid == 0) {
                if (!mbar_wait(&S.bars[s], phase[s])) S.abort = 1;
            }
            phase[s] ^= 1u;
        } else {
            cp_async_wait_group<1>();  // this stage's group (the newest is the other stage's)
        }
        __syncthreads();
        if (S.abort) break;
        // the brick that refills this stage: resolved by thread 0 now, read by
        // all after the barrier in tile_mixed; the ticket after it is drawn now
        // and used at the next refill
        if (tid == 0) {
            const long long nbt = pend < nbricks ? pend : -1ll;
            S.nxt_b = nbt;
            if (nbt >= 0) {
                const int nv = cached_volume(vc, vols, nvol, nbt);
                const BrickPos np = brick_pos(nbt - vc.base, vols[nv].nbx, vols[nv].nby);
                S.nxt = make_int4(nv, vols[nv].tma, np.x0, np.y0);
                S.nxt_z = np.z0;
                pend = (long long)atomicAdd(ticket, 1u);
            }
        }
        const bool mixed = tile_mixed<VT>(S, tile);
        const long long nb = S.nxt_b;
        if (mixed) {
            classify_brick<VT>(S, tile, d.nx, d.ny, d.nz, bp);
            __syncthreads();  // tile s consumed, red[] complete
        }
        // tile s is free: refill it
        if (nb >= 0) {
            const int4 nx4 = S.nxt;
            const int nz0 = S.nxt_z;
            if (nx4.y) {
                if (tid == 0) {
                    mbar_arrive_expect_tx(&S.bars[s], CTILE * Vox<VT>::bytes);
                    tma_load_3d(S.tiles[s], maps + nx4.x, &S.bars[s], nx4.z, nx4.w, nz0);
                }
            } else {
                const VolDesc &dn = vols[nx4.x];
                fill_tile<VT, CTX, CTY, CTZ, false>(tile, static_cast<const T *>(dn.data), dn.nx, dn.ny, dn.nz, nx4.z,
                                                    nx4.w, nz0);
            }
        }
        cp_async_commit();
        if (tid == 0) {
            unsigned int t = 0, o = 0;
            if (mixed) {
                t = S.red[0][0] + S.red[1][0];
                o = S.red[0][1] + S.red[1][1];
            }
            brick_tris[b] = t;
            if (t) {
                uint32_t *c = chunk + (b / CHUNK) * CHUNK_FIELDS;
                atomicAdd(c + 0, t);
                atomicAdd(c + 1, 1u);
                atomicAdd(c + 2, o);
                const int hc = heavy_class(t);
                if (hc >= 0) atomicAdd(c + 3 + hc, 1u);
                atomicAdd(&vol_sums[2 * v + 0], (unsigned long long)t);
                atomicAdd(&vol_sums[2 * v + 1], (unsigned long long)o);
            }
            S.sb[s] = nb;
            if (nb >= 0) {
                S.svol[s] = S.nxt.x;
                S.stma[s] = S.nxt.y;
                S.spos[s] = make_int4(S.nxt.z, S.nxt.w, S.nxt_z, 0);
            }
        }
    }
    cp_async_wait_all();
    pdl_trigger();  // the scan may be scheduled (it waits for this grid's completion)
    if (S.abort && tid == 0) {
        atomicOr(flags, 1u);
        for (int s = 0; s < 2; ++s) mbar_wait(&S.bars[s], phase[s], 100000000ull);
    }
}

template <int VT>
struct GenSmemMulti : GenSmem<VT, 2> {
    int svol[2];
    int stma[2];
    alignas(16) BatchBrick pipe;  // entry staged at the next refill (thread 0's pipeline)
};

template <int VT>
__device__ __forceinline__ void issue_gen_tile(GenSmemMulti<VT> &S, int s, const VolDesc *__restrict__ vols,
                                               const CUtensorMap *maps, const BatchBrick &r) {
    S.svol[s] = r.v;
    S.stma[s] = vols[r.v].tma;
    S.sbrick[s] = 0;
    S.svbase[s] = r.vbase;
    S.spos[s] = make_int4(r.x0, r.y0, r.z0, 0);
    if (vols[r.v].tma) {
        mbar_arrive_expect_tx(&S.bars[s], GTILE * Vox<VT>::bytes);
        tma_load_3d(S.tiles[s], maps + r.v, &S.bars[s], r.x0 - TXO, r.y0 - TYO, r.z0 - TZO);
    }
}

// Bricks of every volume of the batch from one active list, scheduled as in
// the single-volume launch: fixed serpentine first rounds, then entries from
// the counter, each entry's resolved record copied asynchronously one brick
// before it is staged.
template <int VT>
__global__ void __launch_bounds__(THREADS, 4)
    mc_generate_multi_kernel(const VolDesc *__restrict__ vols, const CUtensorMap *maps, int nvol,
                             const BatchBrick *__restrict__ list, MeshTotals *totals, MeshTotals *host) {
    using V = Vox<VT>;
    using T = typename V::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    GenSmemMulti<VT> &S = *reinterpret_cast<GenSmemMulti<VT> *>(smem_raw);
    const int tid = threadIdx.x;
    uint32_t phase[2] = {0, 0};
    load_tri_table(S.tri, tid, THREADS);
    S.nv[tid] = (tid == 0 || tid == 255) ? 0 : g_nverts[tid];
    pdl_wait();  // the batch's scan: active list, totals, cleared counter
    const unsigned int nactive = totals->active_bricks;
    unsigned int *ticket = &totals->gen_ticket;
    const unsigned int grid = gridDim.x, c = blockIdx.x;
    const unsigned int tbase = 3 * grid;  // list entry of ticket 0
    auto entry = [&](unsigned int r) { return r * grid + ((r & 1) ? grid - 1 - c : c); };
    unsigned int ptk = 0xffffffffu;  // list entry of the ticket drawn at the top of this brick
    bool have_pipe = false;          // S.pipe holds the entry of the next refill
    if (tid == 0) {
        S.abort = 0;
        for (int s = 0; s < 2; ++s) mbar_init(&S.bars[s], 1);
        fence_barrier_init();
        for (int s = 0; s < 2; ++s) {
            S.svol[s] = -1;
            const unsigned int w = entry(s);
            if (w < nactive) issue_gen_tile<VT>(S, s, vols, maps, list[w]);
        }
        const unsigned int w = entry(2);
        if (w < nactive) {
            cp_async_16(&S.pipe, list + w);
            cp_async_16(reinterpret_cast<unsigned char *>(&S.pipe) + 16, reinterpret_cast<const unsigned char *>(list + w) + 16);
            have_pipe = true;
        }
        if (tbase < nactive) ptk = 0;  // not ~0u: draw tickets at the tops of the bricks
    }
    __syncthreads();
    for (int it = 0;; ++it) {
        const int s = it & 1;
        T *tile = reinterpret_cast<T *>(S.tiles[s]);
        const int v = S.svol[s];
        if (v < 0) break;  // uniform
        if (tid == 0) {
            if (ptk != 0xffffffffu) ptk = tbase + atomicAdd(ticket, 1u);
            if (S.stma[s] && !mbar_wait(&S.bars[s], phase[s])) S.abort = 1;
        }
        if (S.stma[s]) phase[s] ^= 1u;
        const unsigned long long vbase = S.svbase[s];
        const int4 sp = S.spos[s];
        const VolDesc &d = vols[v];
        if (!S.stma[s])
            fill_tile<VT, TX, TY, TZ>(tile, static_cast<const T *>(d.data), d.nx, d.ny, d.nz, sp.x - TXO, sp.y - TYO,
                                      sp.z - TZO);
        __syncthreads();
        if (S.abort) break;
        GenOut o;
        o.soup = d.soup;
        o.normals = d.normals;
        o.vi2vox = d.vi2vox;
        o.ver_voxel = d.ver_voxel;
        o.tri_cube = d.tri_cube;
        o.cap = d.cap;
        o.zlim = d.nz - 1;
        generate_brick<VT>(S, tile, static_cast<const T *>(d.data), d.nx, d.ny, d.nz, d.cell, sp.x, sp.y, sp.z,
                           vbase, o);
        __syncthreads();  // tile s, the list and the stage are free again
        if (tid == 0) {
            S.svol[s] = -1;
            if (have_pipe) {
                cp_async_wait_all();
                issue_gen_tile<VT>(S, s, vols, maps, S.pipe);
            }
            have_pipe = ptk < nactive;
            if (have_pipe) {
                cp_async_16(&S.pipe, list + ptk);
                cp_async_16(reinterpret_cast<unsigned char *>(&S.pipe) + 16,
                            reinterpret_cast<const unsigned char *>(list + ptk) + 16);
            } else {
                ptk = 0xffffffffu;  // the list is exhausted: draw no more tickets
            }
        }
        // S.svol[s] is next read at the top of iteration it + 2, after the
        // barriers of iteration it + 1
    }
    if (S.abort && tid == 0) {
        atomicOr(&totals->flags, 1u);
        for (int s = 0; s < 2; ++s) mbar_wait(&S.bars[s], phase[s], 100000000ull);
    }
    // the last CTA out folds the flags into the mapped host copy, where the
    // batch's scan put the count launch's
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&totals->gen_exit, 1u) == gridDim.x - 1) {
            totals->gen_exit = 0;
            if (host) {
                host->flags |= *(volatile unsigned int *)&totals->flags;
                totals->flags = 0;
                __threadfence_system();
            }
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

// ---- host side ----------------------------------------------------------------
struct Scratch {
    uint32_t *tris;
    uint32_t *chunk;  // CHUNK_FIELDS per chunk of CHUNK bricks
    unsigned long long *vofs;
    uint32_t *active;
    unsigned long long *list_vofs;  // soup offset per active-list entry
    MeshTotals *totals;
    MeshTotals *host;  // mapped host copy of the totals, or null
};

// default launch configuration (the measured best on GB300; a context can
// choose another through mcg_mc_set_config, e.g. from the autotuner)
constexpr mcg_mc_config kDefaultMcConfig = {0, 4, 3, 0};

// Launch with programmatic stream serialisation: the kernel may start while
// the kernel before it on the stream drains (it waits with pdl_wait).
template <class... P, class... A>
cudaError_t launch_pdl(void (*kernel)(P...), unsigned int grid, unsigned int block, size_t smem, cudaStream_t s,
                       A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

template <int VT, bool TMA, int G, int XH, int CSTAGES, int NT>
void launch_classify_s(const CUtensorMap &map, const CUtensorMap &hmap, const mcg_volume *vol, const Geometry &g,
                       const Scratch &sc, int sms, cudaStream_t s) {
    const size_t smem = sizeof(ClsSmemG<VT, G, XH, CSTAGES, NT>);
    static int occ = 0;  // per instantiation; all devices of a run are the same part
    if (!occ) occ = occupancy(mc_classify_kernel<VT, TMA, G, XH, CSTAGES, NT>, NT, smem);
    const int ngx = (g.nbx + G - 1) / G;
    const long long nitems = (long long)ngx * g.nby * g.nbz;
    long long grid = (long long)sms * occ;
    if (grid > nitems) grid = nitems;
    launch_pdl(mc_classify_kernel<VT, TMA, G, XH, CSTAGES, NT>, (unsigned int)grid, NT, smem, s, map, hmap,
               static_cast<const typename Vox<VT>::T *>(vol->data), vol->nx, vol->ny, vol->nz, g.nbx, g.nby,
               (int)nitems, ngx, g.zbase, g.zlim, sc.tris, sc.chunk, &sc.totals->flags, &sc.totals->cls_ticket);
}

// classify configurations (mcg_mc_config.classify_shape):
//   0: 2 bricks, in-box halo (68-voxel box), 2 stages x 256 threads
//   1: 4 bricks, halo box, 2 stages x 256 threads
//   2: 4 bricks, halo box, 4 stages x 512 threads
//   3: 4 bricks, in-box halo (132-voxel box), 2 stages x 256 threads
//   4: 4 bricks, in-box halo (132-voxel box), 1 stage x 256 threads
//   5: 2 bricks, in-box halo (68-voxel box), 1 stage x 256 threads
// bricks per work item and in-box halo of the configuration, narrowed to
// what the volume's width allows
void classify_shape(int nx, int eb, int c, int &G, int &XH) {
    XH = (c == 1 || c == 2) ? 0 : 4;
    const int pref = (c == 0 || c == 5) ? 2 : 512 / (BX * eb);
    G = 1;
    if (pref >= 4 && nx >= BX * 4 + XH) G = 4;
    else if (pref >= 2 && nx >= BX * 2 + XH) G = 2;
}

template <int VT, bool TMA, int G, int XH>
void launch_classify_g(const CUtensorMap &map, const CUtensorMap &hmap, const mcg_volume *vol, const Geometry &g,
                       const Scratch &sc, int sms, cudaStream_t s, int c) {
    // without TMA only one stage is ever used
    if constexpr (!TMA) {
        launch_classify_s<VT, TMA, G, XH, 1, 256>(map, hmap, vol, g, sc, sms, s);
    } else {
        if (c == 2) launch_classify_s<VT, TMA, G, XH, 4, 512>(map, hmap, vol, g, sc, sms, s);
        else if (c >= 4) launch_classify_s<VT, TMA, G, XH, 1, 256>(map, hmap, vol, g, sc, sms, s);
        else launch_classify_s<VT, TMA, G, XH, 2, 256>(map, hmap, vol, g, sc, sms, s);
    }
}

template <int VT, int XH>
void launch_classify_x(bool tma, int G, const CUtensorMap &map, const CUtensorMap &hmap, const mcg_volume *vol,
                       const Geometry &g, const Scratch &sc, int sms, cudaStream_t s, int c) {
    if (G == 4) {
        if (tma) launch_classify_g<VT, true, 4, XH>(map, hmap, vol, g, sc, sms, s, c);
        else launch_classify_g<VT, false, 4, XH>(map, hmap, vol, g, sc, sms, s, c);
    } else if (G == 2) {
        if (tma) launch_classify_g<VT, true, 2, XH>(map, hmap, vol, g, sc, sms, s, c);
        else launch_classify_g<VT, false, 2, XH>(map, hmap, vol, g, sc, sms, s, c);
    } else {
        if (tma) launch_classify_g<VT, true, 1, XH>(map, hmap, vol, g, sc, sms, s, c);
        else launch_classify_g<VT, false, 1, XH>(map, hmap, vol, g, sc, sms, s, c);
    }
}

template <int VT, bool TMA, int MODE = 0>
void launch_generate_t(const CUtensorMap &map, const GenParams &p, const Geometry &g, int sms, cudaStream_t s) {
    const size_t smem = sizeof(GenSmem<VT, GEN_STAGES>);
    static int occ = 0;
    if (!occ) occ = occupancy(mc_generate_kernel<VT, TMA, MODE>, THREADS, smem);
    long long grid = (long long)sms * occ;
    if (grid > g.nbricks) grid = g.nbricks;
    // MODE 0 follows the scan directly; other launches follow a memset
    if (MODE == 0) launch_pdl(mc_generate_kernel<VT, TMA, MODE>, (unsigned int)grid, THREADS, smem, s, map, p);
    else mc_generate_kernel<VT, TMA, MODE><<<(int)grid, THREADS, smem, s>>>(map, p);
}

// classify + scan into sc; clears the timeout flag first
long long num_chunks(long long nbricks) { return (nbricks + CHUNK - 1) / CHUNK; }

cudaError_t launch_count_phase(const mcg_volume *vol, const Geometry &g, const Scratch &sc, int sms, cudaStream_t s,
                               const mcg_mc_config &cfg, bool clear = true, cudaEvent_t t0 = nullptr,
                               cudaEvent_t t1 = nullptr) {
    // flags and both work counters unless known to be zero; the chunk sums
    // are zero already (the previous scan cleared them)
    cudaError_t e = clear ? cudaMemsetAsync(&sc.totals->flags, 0, 3 * sizeof(unsigned int), s) : cudaSuccess;
    if (e != cudaSuccess) return e;
    CUtensorMap map, hmap;
    const int eb = vol->voxel_type == MCG_VOXEL_SHORT2 ? 4 : 8;
    int G, XH;
    classify_shape(vol->nx, eb, cfg.classify_shape, G, XH);
    if ((long long)((g.nbx + G - 1) / G) * g.nby * g.nbz > 0x7fffffffll) return cudaErrorInvalidValue;
    bool tma = encode_volume_map(&map, vol->data, vol->nx, vol->ny, vol->nz, eb, G * BX + XH, CTY, CTZ);
    if (tma && XH == 0) tma = encode_volume_map(&hmap, vol->data, vol->nx, vol->ny, vol->nz, eb, 16 / eb, CTY, CTZ);
    else memset(&hmap, 0, sizeof(hmap));
    if (!tma) {
        memset(&map, 0, sizeof(map));
        memset(&hmap, 0, sizeof(hmap));
    }
    const bool s2 = vol->voxel_type == MCG_VOXEL_SHORT2;
    if (t0) {
        const cudaError_t et = cudaEventRecord(t0, s);
        if (et != cudaSuccess) return et;
    }
    const int c = cfg.classify_shape;
    if (XH) {
        if (s2) launch_classify_x<MCG_VOXEL_SHORT2, 4>(tma, G, map, hmap, vol, g, sc, sms, s, c);
        else launch_classify_x<MCG_VOXEL_FLOAT2, 4>(tma, G, map, hmap, vol, g, sc, sms, s, c);
    } else {
        if (s2) launch_classify_x<MCG_VOXEL_SHORT2, 0>(tma, G, map, hmap, vol, g, sc, sms, s, c);
        else launch_classify_x<MCG_VOXEL_FLOAT2, 0>(tma, G, map, hmap, vol, g, sc, sms, s, c);
    }
    if (t1) {
        const cudaError_t et = cudaEventRecord(t1, s);
        if (et != cudaSuccess) return et;
    }
    launch_pdl(mc_scan_kernel<false>, (unsigned int)num_chunks(g.nbricks), CHUNK, 0, s, (const uint32_t *)sc.tris,
               sc.chunk, (long long)g.nbricks, sc.vofs, sc.active, sc.list_vofs, sc.totals, sc.host, ScanBatch{});
    return cudaGetLastError();
}

cudaError_t launch_generate_phase(const mcg_volume *vol, const Geometry &g, const Scratch &sc,
                                  const mcg_mesh_out *out, int sms, cudaStream_t s, const mcg_mc_config &cfg) {
    if (out->ver_voxel) {
        cudaError_t e = cudaMemsetAsync(out->ver_voxel, 0, sizeof(int16_t) * (size_t)vol->nx * vol->ny * vol->nz, s);
        if (e != cudaSuccess) return e;
    }
    // gen_ticket is zero: cleared by the count phase and by every generate launch at its end
    GenParams p;
    p.vol = vol->data;
    p.nx = vol->nx;
    p.ny = vol->ny;
    p.nz = vol->nz;
    p.cell = vol->cell;
    p.nbx = g.nbx;
    p.nby = g.nby;
    p.zbase = g.zbase;
    p.zlim = g.zlim;
    p.active = sc.active;
    p.brick_vofs = sc.vofs;
    p.list_vofs = sc.list_vofs;
    p.host = sc.host;
    p.fixed_rounds = (unsigned int)cfg.gen_fixed_rounds;
    p.totals = sc.totals;
    p.soup = out->soup;
    p.normals = out->soup_normals;
    p.vi2vox = out->vi2vox;
    p.ver_voxel = out->ver_voxel;
    p.tri_cube = out->tri_cube;
    p.cap = out->capacity_vertices;
    p.grad_pos = nullptr;
    p.grad_f = nullptr;
    p.n_grad = 0;
    CUtensorMap map;
    const int eb = vol->voxel_type == MCG_VOXEL_SHORT2 ? 4 : 8;
    const bool tma = encode_volume_map(&map, vol->data, vol->nx, vol->ny, vol->nz, eb, TX, TY, TZ);
    if (!tma) memset(&map, 0, sizeof(map));
    if (vol->voxel_type == MCG_VOXEL_SHORT2) {
        if (tma) launch_generate_t<MCG_VOXEL_SHORT2, true>(map, p, g, sms, s);
        else launch_generate_t<MCG_VOXEL_SHORT2, false>(map, p, g, sms, s);
    } else {
        if (tma) launch_generate_t<MCG_VOXEL_FLOAT2, true>(map, p, g, sms, s);
        else launch_generate_t<MCG_VOXEL_FLOAT2, false>(map, p, g, sms, s);
    }
    return cudaGetLastError();
}

Scratch ctx_scratch(mcg_context *ctx) {
    return Scratch{ctx->brick_tris, ctx->brick_occ, ctx->brick_vofs, ctx->active, ctx->list_vofs, ctx->d_totals,
                   ctx->h_totals_dev};
}

// The fused extraction with FG bricks per item applies to short2 volumes of
// at least one item box (FGeo<FG>::TX x 10 x 10) that TMA can describe; `map`
// receives the tensor map.
template <int FG>
bool fused_applies(const mcg_volume *vol, CUtensorMap *map) {
    constexpr int FTX = FGeo<FG>::TX;
    if (vol->voxel_type != MCG_VOXEL_SHORT2) return false;
    if (vol->nx < FTX || vol->ny < FTY || vol->nz < FTZ) return false;
    return encode_volume_map(map, vol->data, vol->nx, vol->ny, vol->nz, 4, FTX, FTY, FTZ);
}

// minimum resident CTAs per SM of the fused launch (shared memory bound)
template <int FG>
struct FMinB {
    static constexpr int v = FG == 4 ? 3 : 5;
};

// One fused launch over the whole volume.
template <int FG>
cudaError_t launch_fused(mcg_context *ctx, const CUtensorMap &map, const mcg_volume *vol, const mcg_mesh_out *out,
                         cudaStream_t s) {
    const Geometry g = geometry(vol->nx, vol->ny, vol->nz);
    const int ngx = (g.nbx + FG - 1) / FG;
    const long long nitems = (long long)ngx * g.nby * g.nbz;
    if (nitems > 0x7fffffffll) return cudaErrorInvalidValue;
    const long long ngroups = (nitems + FGROUP - 1) / FGROUP;
    const size_t icap = ctx->fx_item_cap, gcap = ctx->fx_group_cap;
    if (!ensure(&ctx->fx_item, &ctx->fx_item_cap, (size_t)nitems) ||
        !ensure(&ctx->fx_group, &ctx->fx_group_cap, (size_t)ngroups))
        return cudaErrorMemoryAllocation;
    cudaError_t e = cudaSuccess;
    // fresh allocations, and the wrap of the 22-bit epoch, start from entries
    // of epoch 0: every entry then belongs to an older launch of this cycle
    if (ctx->fx_item_cap != icap || ctx->fx_group_cap != gcap || ctx->fx_epoch + 1 >= (1u << FX_EPOCH_BITS)) {
        e = cudaMemsetAsync(ctx->fx_item, 0, sizeof(unsigned long long) * ctx->fx_item_cap, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->fx_group, 0, sizeof(unsigned long long) * ctx->fx_group_cap, s);
        if (e != cudaSuccess) return e;
        ctx->fx_epoch = 0;
    }
    // The launch accumulates the totals, so they must start at zero: the
    // previous fused launch on ctx leaves them so when the totals reached the
    // host through the mapped copy; every other count phase leaves its own
    // totals behind.
    if (!ctx->h_totals_dev || !ctx->counters_clean || !ctx->cls_fused) {
        e = cudaMemsetAsync(ctx->d_totals, 0, sizeof(MeshTotals), s);
        if (e != cudaSuccess) return e;
    }
    if (out->ver_voxel) {
        e = cudaMemsetAsync(out->ver_voxel, 0, sizeof(int16_t) * (size_t)vol->nx * vol->ny * vol->nz, s);
        if (e != cudaSuccess) return e;
    }
    FusedParams p;
    p.vol = vol->data;
    p.nx = vol->nx;
    p.ny = vol->ny;
    p.nz = vol->nz;
    p.cell = vol->cell;
    p.nbx = g.nbx;
    p.nby = g.nby;
    p.nitems = (int)nitems;
    p.ngx = ngx;
    p.zlim = g.zlim;
    p.item = ctx->fx_item;
    p.group = ctx->fx_group;
    p.epoch = ++ctx->fx_epoch;
    p.totals = ctx->d_totals;
    p.host = ctx->h_totals_dev;
    p.out.soup = out->soup;
    p.out.normals = out->soup_normals;
    p.out.vi2vox = out->vi2vox;
    p.out.ver_voxel = out->ver_voxel;
    p.out.tri_cube = out->tri_cube;
    p.out.cap = out->capacity_vertices;
    p.out.zlim = g.zlim;
    constexpr int NT = FGeo<FG>::NT;
    auto kernel = mc_fused_kernel<MCG_VOXEL_SHORT2, FG, FMinB<FG>::v>;
    const size_t smem = sizeof(FusedSmem<MCG_VOXEL_SHORT2, FG>);
    static int occ = 0;
    if (!occ) occ = occupancy(kernel, NT, smem);
    long long grid = (long long)ctx->num_sms * occ;
    if (grid > nitems) grid = nitems;
    if (ctx->time_kernels) {
        e = cudaEventRecord(ctx->tk0, s);
        if (e != cudaSuccess) return e;
    }
    e = launch_pdl(kernel, (unsigned int)grid, NT, smem, s, map, p);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess && ctx->time_kernels) {
        e = cudaEventRecord(ctx->tk1, s);
        if (e == cudaSuccess) ctx->timed = true;
    }
    return e;
}

}  // namespace
}  // namespace mcg

using namespace mcg;

// count phase over the cubes with z0 <= z < z1
static mcg_status classify_impl(mcg_context *ctx, const mcg_volume *vol, int32_t z0, int32_t z1,
                                mcg_stream_t stream) {
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const Geometry g = geometry_slab(vol->nx, vol->ny, z0, z1);
    if (!ensure(&ctx->brick_tris, &ctx->brick_tris_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->brick_occ, &ctx->brick_occ_cap, (size_t)(CHUNK_FIELDS * num_chunks(g.nbricks))) ||
        !ensure(&ctx->brick_vofs, &ctx->brick_vofs_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->active, &ctx->active_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->list_vofs, &ctx->list_vofs_cap, (size_t)g.nbricks))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    // chunk sums: zeroed once per allocation, then by each scan after use
    if (ctx->chunk_clean_cap != ctx->brick_occ_cap) {
        e = cudaMemsetAsync(ctx->brick_occ, 0, sizeof(uint32_t) * ctx->brick_occ_cap, s);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        ctx->chunk_clean_cap = ctx->brick_occ_cap;
    }
    if (ctx->time_kernels && !ctx->tk0) {
        e = cudaEventCreate(&ctx->tk0);
        if (e == cudaSuccess) e = cudaEventCreate(&ctx->tk1);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    }
    e = launch_count_phase(vol, g, ctx_scratch(ctx), ctx->num_sms, s, ctx->mc_cfg,
                           !ctx->h_totals_dev || !ctx->counters_clean,
                           ctx->time_kernels ? ctx->tk0 : nullptr, ctx->time_kernels ? ctx->tk1 : nullptr);
    if (e == cudaSuccess && ctx->time_kernels) ctx->timed = true;
    ctx->counters_clean = e == cudaSuccess && ctx->h_totals_dev != nullptr;
    if (e == cudaSuccess && !ctx->h_totals_dev)
        e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = mcg_counts_event(ctx, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    ctx->classified = true;
    ctx->cls_indexed = false;
    ctx->cls_fused = false;
    ctx->batch_classified = false;
    ctx->cls_data = vol->data;
    ctx->cls_nx = vol->nx;
    ctx->cls_ny = vol->ny;
    ctx->cls_nz = vol->nz;
    ctx->cls_vtype = vol->voxel_type;
    ctx->cls_z0 = z0;
    ctx->cls_z1 = z1;
    ctx->last_capacity = -1;
    return MCG_OK;
}

namespace mcg {
cudaError_t soup_count_phase(mcg_context *ctx, const mcg_volume *vol, cudaStream_t s) {
    const Geometry g = geometry(vol->nx, vol->ny, vol->nz);
    if (!ensure(&ctx->brick_tris, &ctx->brick_tris_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->brick_occ, &ctx->brick_occ_cap, (size_t)(CHUNK_FIELDS * num_chunks(g.nbricks))) ||
        !ensure(&ctx->brick_vofs, &ctx->brick_vofs_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->active, &ctx->active_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->list_vofs, &ctx->list_vofs_cap, (size_t)g.nbricks))
        return cudaErrorMemoryAllocation;
    if (ctx->chunk_clean_cap != ctx->brick_occ_cap) {
        const cudaError_t e = cudaMemsetAsync(ctx->brick_occ, 0, sizeof(uint32_t) * ctx->brick_occ_cap, s);
        if (e != cudaSuccess) return e;
        ctx->chunk_clean_cap = ctx->brick_occ_cap;
    }
    Scratch sc = ctx_scratch(ctx);
    sc.host = nullptr;  // the scan then leaves the flags and counters in d_totals
    ctx->counters_clean = false;
    return launch_count_phase(vol, g, sc, ctx->num_sms, s, ctx->mc_cfg, true);
}
}  // namespace mcg

mcg_status mcg_set_kernel_timing(mcg_context *ctx, int32_t enable) {
    if (!ctx) return MCG_ERR_INVALID_ARG;
    ctx->time_kernels = enable != 0;
    return MCG_OK;
}

mcg_status mcg_mc_count_kernel_ms(mcg_context *ctx, float *ms) {
    if (!ctx || !ms) return MCG_ERR_INVALID_ARG;
    if (!ctx->timed) return MCG_ERR_STATE;
    cudaError_t e = cudaEventSynchronize(ctx->tk1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, ctx->tk0, ctx->tk1);
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

mcg_status mcg_mc_classify(mcg_context *ctx, const mcg_volume *vol, mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol)) return MCG_ERR_INVALID_ARG;
    return classify_impl(ctx, vol, 0, vol->nz - 1, stream);
}

mcg_status mcg_mc_classify_slab(mcg_context *ctx, const mcg_volume *vol, int32_t z0, int32_t z1,
                                mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol)) return MCG_ERR_INVALID_ARG;
    if (z0 < 0 || z1 <= z0 || z1 > vol->nz - 1 || z0 % BZ != 0) return MCG_ERR_INVALID_ARG;
    return classify_impl(ctx, vol, z0, z1, stream);
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
    out->status = MCG_OK;
    if (ctx->h_totals->flags & 1u) out->status = MCG_ERR_TIMEOUT;
    else if (ctx->last_capacity >= 0 && out->vertices > ctx->last_capacity) out->status = MCG_ERR_CAPACITY;
    else if (ctx->cls_indexed && ctx->last_capacity_tris >= 0 && out->triangles > ctx->last_capacity_tris)
        out->status = MCG_ERR_CAPACITY;
    out->reserved = 0;
    return (mcg_status)out->status;
}

mcg_status mcg_mc_generate(mcg_context *ctx, const mcg_volume *vol, const mcg_mesh_out *out,
                           mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol) || !out || out->capacity_vertices < 0) return MCG_ERR_INVALID_ARG;
    if (!ctx->classified || ctx->cls_indexed || ctx->cls_fused || ctx->cls_data != vol->data ||
        ctx->cls_nx != vol->nx || ctx->cls_ny != vol->ny || ctx->cls_nz != vol->nz || ctx->cls_vtype != vol->voxel_type)
        return MCG_ERR_STATE;
    if (out->capacity_vertices > 0 && !out->soup && !out->soup_normals && !out->vi2vox &&
        !out->ver_voxel && !out->tri_cube)
        return MCG_ERR_INVALID_ARG;
    // ver_voxel is cleared whole before it is scattered: a slab would clear the
    // other slabs' entries
    const bool slab = ctx->cls_z0 != 0 || ctx->cls_z1 != vol->nz - 1;
    if (slab && out->ver_voxel) return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const Geometry g = geometry_slab(vol->nx, vol->ny, ctx->cls_z0, ctx->cls_z1);
    e = launch_generate_phase(vol, g, ctx_scratch(ctx), out, ctx->num_sms, s, ctx->mc_cfg);
    // the totals are re-read so a timeout flagged by generate is reported (the
    // launch writes the flags to the mapped host copy itself)
    if (e == cudaSuccess && !ctx->h_totals_dev)
        e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = mcg_counts_event(ctx, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    ctx->last_capacity = out->capacity_vertices;
    return MCG_OK;
}

mcg_status mcg_mc_extract(mcg_context *ctx, const mcg_volume *vol, const mcg_mesh_out *out,
                          mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol) || !out || out->capacity_vertices < 0) return MCG_ERR_INVALID_ARG;
    if (out->capacity_vertices > 0 && !out->soup && !out->soup_normals && !out->vi2vox && !out->ver_voxel &&
        !out->tri_cube)
        return MCG_ERR_INVALID_ARG;
    CUtensorMap map;
    const int fused = ctx->mc_cfg.fused;
    if ((fused == 1 && fused_applies<4>(vol, &map)) || (fused == 2 && fused_applies<2>(vol, &map))) {
        cudaStream_t s = (cudaStream_t)stream;
        cudaError_t e = cudaSetDevice(ctx->device);
            if (e == cudaSuccess && ctx->time_kernels && !ctx->tk0) {
            e = cudaEventCreate(&ctx->tk0);
            if (e == cudaSuccess) e = cudaEventCreate(&ctx->tk1);
        }
        if (e == cudaSuccess) e = fused == 1 ? launch_fused<4>(ctx, map, vol, out, s) : launch_fused<2>(ctx, map, vol, out, s);
        ctx->counters_clean = e == cudaSuccess && ctx->h_totals_dev != nullptr;
        if (e == cudaSuccess && !ctx->h_totals_dev)
            e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = mcg_counts_event(ctx, s);
        if (e != cudaSuccess) {
            ctx->classified = false;
            ctx->cls_fused = false;
            return mcg_cuda_fail(ctx, e);
        }
        ctx->classified = true;
        ctx->cls_indexed = false;
        ctx->cls_fused = true;
        ctx->batch_classified = false;
        ctx->cls_data = vol->data;
        ctx->cls_nx = vol->nx;
        ctx->cls_ny = vol->ny;
        ctx->cls_nz = vol->nz;
        ctx->cls_vtype = vol->voxel_type;
        ctx->cls_z0 = 0;
        ctx->cls_z1 = vol->nz - 1;
        ctx->last_capacity = out->capacity_vertices;
        return MCG_OK;
    }
    mcg_status st = mcg_mc_classify(ctx, vol, stream);
    if (st != MCG_OK) return st;
    return mcg_mc_generate(ctx, vol, out, stream);
}

mcg_status mcg_mc_get_config(const mcg_context *ctx, mcg_mc_config *cfg) {
    if (!ctx || !cfg) return MCG_ERR_INVALID_ARG;
    *cfg = ctx->mc_cfg;
    return MCG_OK;
}

mcg_status mcg_mc_set_config(mcg_context *ctx, const mcg_mc_config *cfg) {
    if (!ctx || !cfg) return MCG_ERR_INVALID_ARG;
    if (cfg->fused < 0 || cfg->fused > 2 || cfg->classify_shape < 0 || cfg->classify_shape > 5 ||
        cfg->gen_fixed_rounds < 0 || cfg->gen_fixed_rounds > 16 || cfg->reserved != 0)
        return MCG_ERR_INVALID_ARG;
    ctx->mc_cfg = *cfg;
    return MCG_OK;
}

mcg_status mcg_mc_extract_slab(mcg_context *ctx, const mcg_volume *vol, int32_t z0, int32_t z1,
                               const mcg_mesh_out *out, mcg_stream_t stream) {
    mcg_status st = mcg_mc_classify_slab(ctx, vol, z0, z1, stream);
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



mcg_status mcg_mc_backward(mcg_context *ctx, const mcg_volume *vol, const float *grad_pos, int64_t n_vertices,
                           float *grad_f, mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol) || n_vertices < 0 || !grad_f || (n_vertices > 0 && !grad_pos))
        return MCG_ERR_INVALID_ARG;
    if (!ctx->classified || ctx->cls_indexed || ctx->cls_fused || ctx->cls_data != vol->data ||
        ctx->cls_nx != vol->nx || ctx->cls_ny != vol->ny || ctx->cls_nz != vol->nz || ctx->cls_vtype != vol->voxel_type)
        return MCG_ERR_STATE;
    if (n_vertices == 0) return MCG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const Geometry g = geometry_slab(vol->nx, vol->ny, ctx->cls_z0, ctx->cls_z1);
    e = cudaMemsetAsync(&ctx->d_totals->gen_ticket, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    ctx->counters_clean = false;  // a timeout here leaves the flags set
    GenParams p;
    memset(&p, 0, sizeof(p));
    p.vol = vol->data;
    p.nx = vol->nx;
    p.ny = vol->ny;
    p.nz = vol->nz;
    p.cell = vol->cell;
    p.nbx = g.nbx;
    p.nby = g.nby;
    p.zbase = g.zbase;
    p.zlim = g.zlim;
    p.active = ctx->active;
    p.brick_vofs = ctx->brick_vofs;
    p.list_vofs = ctx->list_vofs;
    p.totals = ctx->d_totals;
    p.fixed_rounds = (unsigned int)ctx->mc_cfg.gen_fixed_rounds;
    p.grad_pos = grad_pos;
    p.grad_f = grad_f;
    p.n_grad = n_vertices;
    CUtensorMap map;
    const int eb = vol->voxel_type == MCG_VOXEL_SHORT2 ? 4 : 8;
    const bool tma = encode_volume_map(&map, vol->data, vol->nx, vol->ny, vol->nz, eb, TX, TY, TZ);
    if (!tma) memset(&map, 0, sizeof(map));
    if (vol->voxel_type == MCG_VOXEL_SHORT2) {
        if (tma) launch_generate_t<MCG_VOXEL_SHORT2, true, 1>(map, p, g, ctx->num_sms, s);
        else launch_generate_t<MCG_VOXEL_SHORT2, false, 1>(map, p, g, ctx->num_sms, s);
    } else {
        if (tma) launch_generate_t<MCG_VOXEL_FLOAT2, true, 1>(map, p, g, ctx->num_sms, s);
        else launch_generate_t<MCG_VOXEL_FLOAT2, false, 1>(map, p, g, ctx->num_sms, s);
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

// Zeroes what a batch's count launch accumulates into: the flags, the count
// and generate counters, the per-volume sums and the chunk sums.
__global__ void mc_batch_reset_kernel(MeshTotals *totals, unsigned long long *__restrict__ vol_sums, int nvol,
                                      uint32_t *__restrict__ chunk, long long nchunk_words) {
    const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    if (i0 == 0) {
        totals->flags = 0;
        totals->cls_ticket = 0;
        totals->gen_ticket = 0;
    }
    for (long long i = i0; i < 2LL * nvol; i += st) vol_sums[i] = 0;
    for (long long i = i0; i < nchunk_words; i += st) chunk[i] = 0;
}

// ---- batched extraction host side -------------------------------------------------
namespace mcg {
namespace {

// Device table layout: [VolDesc x nvol][pad to 64][classify maps x nvol][generate maps x nvol]
size_t btab_desc_bytes(int nvol) { return ((sizeof(VolDesc) * (size_t)nvol + 63) / 64) * 64; }
size_t btab_bytes(int nvol) { return btab_desc_bytes(nvol) + 2 * sizeof(CUtensorMap) * (size_t)nvol; }

// staging slot k of at least n bytes; its last copy has completed
mcg_status grow_pinned(mcg_context *ctx, int k, size_t n) {
    if (ctx->btab_pending[k]) {
        const cudaError_t e = cudaEventSynchronize(ctx->btab_copied[k]);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        ctx->btab_pending[k] = false;
    }
    if (ctx->h_btab_cap[k] >= n && ctx->h_btab[k]) return MCG_OK;
    if (ctx->h_btab[k]) cudaFreeHost(ctx->h_btab[k]);
    ctx->h_btab[k] = nullptr;
    ctx->h_btab_cap[k] = 0;
    if (cudaMallocHost((void **)&ctx->h_btab[k], n) != cudaSuccess) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    ctx->h_btab_cap[k] = n;
    return MCG_OK;
}

// Two spare stagings of at least n bytes for a later capture of this batch
// (its count and generate phases take one each); called outside captures.
mcg_status top_up_spares(mcg_context *ctx, size_t n) {
    if (ctx->btab_spare_cap < n) {
        for (unsigned char *b : ctx->btab_spare) cudaFreeHost(b);
        ctx->btab_spare.clear();
        ctx->btab_spare_cap = n;
    }
    while (ctx->btab_spare.size() < 2) {
        unsigned char *b = nullptr;
        if (cudaMallocHost((void **)&b, ctx->btab_spare_cap) != cudaSuccess)
            return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        ctx->btab_spare.push_back(b);
    }
    return MCG_OK;
}

bool batch_ok(const mcg_volume *vols, int32_t nvol) {
    if (!vols || nvol < 1) return false;
    for (int v = 0; v < nvol; ++v) {
        if (!vol_ok(&vols[v])) return false;
        if (vols[v].voxel_type != vols[0].voxel_type) return false;
    }
    return true;
}

// host copy of the table into pinned staging, then to the device on stream s
mcg_status upload_btab(mcg_context *ctx, const mcg_volume *vols, const mcg_mesh_out *outs, int32_t nvol,
                       bool with_maps, cudaStream_t s, long long *total_bricks) {
    const size_t bytes = btab_bytes(nvol);
    // Outside a capture the table goes through the two pinned slots used in
    // turn.  Inside one, the copy becomes a graph node that reads its source
    // at every replay, so the table is staged in a spare that no other call
    // writes again (kept until mcg_destroy); nothing may be allocated or
    // waited for then, so an earlier call of the batch outside the capture
    // has made the spares and sized the device table.
    const bool cap = mcg_capturing(s);
    unsigned char *hb = nullptr;
    int k = -1;
    if (cap) {
        if (ctx->d_btab_cap < bytes || ctx->btab_spare.empty() || ctx->btab_spare_cap < bytes) return MCG_ERR_STATE;
        hb = ctx->btab_spare.back();
        ctx->btab_spare.pop_back();
        ctx->btab_kept.push_back(hb);
    } else {
        if (!ensure(&ctx->d_btab, &ctx->d_btab_cap, bytes)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        k = ctx->btab_slot;
        mcg_status st = grow_pinned(ctx, k, bytes);
        if (st == MCG_OK) st = top_up_spares(ctx, bytes);
        if (st != MCG_OK) return st;
        ctx->btab_slot ^= 1;
        hb = ctx->h_btab[k];
    }
    if (with_maps) {
        if (ctx->batch_tma_cap < (size_t)nvol) {
            unsigned char *t = static_cast<unsigned char *>(realloc(ctx->batch_tma, (size_t)nvol));
            if (!t) return MCG_ERR_INVALID_ARG;
            ctx->batch_tma = t;
            ctx->batch_tma_cap = (size_t)nvol;
        }
    } else if (ctx->batch_tma_cap < (size_t)nvol) {
        return MCG_ERR_STATE;
    }
    VolDesc *desc = reinterpret_cast<VolDesc *>(hb);
    CUtensorMap *cmaps = reinterpret_cast<CUtensorMap *>(hb + btab_desc_bytes(nvol));
    CUtensorMap *gmaps = cmaps + nvol;
    long long base = 0;
    const int eb = vols[0].voxel_type == MCG_VOXEL_SHORT2 ? 4 : 8;
    for (int v = 0; v < nvol; ++v) {
        const Geometry g = geometry(vols[v].nx, vols[v].ny, vols[v].nz);
        VolDesc &d = desc[v];
        memset(&d, 0, sizeof(d));
        d.data = vols[v].data;
        d.nx = vols[v].nx;
        d.ny = vols[v].ny;
        d.nz = vols[v].nz;
        d.cell = vols[v].cell;
        d.nbx = g.nbx;
        d.nby = g.nby;
        d.brick_base = base;
        d.nbricks = g.nbricks;
        base += g.nbricks;
        if (outs) {
            d.soup = outs[v].soup;
            d.normals = outs[v].soup_normals;
            d.vi2vox = outs[v].vi2vox;
            d.ver_voxel = outs[v].ver_voxel;
            d.tri_cube = outs[v].tri_cube;
            d.cap = outs[v].capacity_vertices;
        }
        // TMA only when both boxes can be described (the flag serves both
        // passes); the maps are encoded and copied with the count phase's
        // table, the generate phase's table carries the flags it recorded
        if (with_maps) {
            const bool tc =
                encode_volume_map(&cmaps[v], vols[v].data, vols[v].nx, vols[v].ny, vols[v].nz, eb, CTX, CTY, CTZ);
            const bool tg = encode_volume_map(&gmaps[v], vols[v].data, vols[v].nx, vols[v].ny, vols[v].nz, eb, TX, TY, TZ);
            ctx->batch_tma[v] = tc && tg ? 1 : 0;
            if (!ctx->batch_tma[v]) {
                memset(&cmaps[v], 0, sizeof(CUtensorMap));
                memset(&gmaps[v], 0, sizeof(CUtensorMap));
            }
        }
        d.tma = ctx->batch_tma[v];
    }
    *total_bricks = base;
    const size_t n = with_maps ? bytes : btab_desc_bytes(nvol);
    cudaError_t e = cudaMemcpyAsync(ctx->d_btab, hb, n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !cap) e = cudaEventRecord(ctx->btab_copied[k], s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    if (!cap) ctx->btab_pending[k] = true;
    return MCG_OK;
}

// The mapped host copy of the totals when the batch's counts can reach the
// host without copies (the per-volume sums mapped too), else null.
MeshTotals *batch_host(mcg_context *ctx) {
    return ctx->h_totals_dev && ctx->h_vol_sums_dev ? ctx->h_totals_dev : nullptr;
}

template <int VT>
void launch_classify_multi(mcg_context *ctx, int nvol, long long nbricks, cudaStream_t s) {
    const size_t smem = sizeof(ClsSmemMulti<VT>);
    static int occ = 0;
    if (!occ) occ = occupancy(mc_classify_multi_kernel<VT>, CTHREADS, smem);
    long long grid = (long long)ctx->num_sms * occ;
    if (grid > nbricks) grid = nbricks;
    const VolDesc *desc = reinterpret_cast<const VolDesc *>(ctx->d_btab);
    const CUtensorMap *cmaps = reinterpret_cast<const CUtensorMap *>(ctx->d_btab + btab_desc_bytes(nvol));
    mc_classify_multi_kernel<VT><<<(int)grid, CTHREADS, smem, s>>>(desc, cmaps, nvol, nbricks, ctx->brick_tris,
                                                                    ctx->brick_occ, ctx->d_vol_sums,
                                                                    &ctx->d_totals->flags, &ctx->d_totals->cls_ticket);
}

// generate launch of a batch, chained to the batch's scan (programmatic
// dependent launch: its prologue overlaps the scan's tail)
template <int VT>
cudaError_t launch_generate_multi(mcg_context *ctx, int nvol, long long nbricks, cudaStream_t s) {
    const VolDesc *desc = reinterpret_cast<const VolDesc *>(ctx->d_btab);
    const BatchBrick *list = reinterpret_cast<const BatchBrick *>(ctx->batch_list);  // written by the batch's scan
    const size_t smem = sizeof(GenSmemMulti<VT>);
    static int occ = 0;
    if (!occ) occ = occupancy(mc_generate_multi_kernel<VT>, THREADS, smem);
    long long grid = (long long)ctx->num_sms * occ;
    if (grid > nbricks) grid = nbricks;
    const CUtensorMap *gmaps = reinterpret_cast<const CUtensorMap *>(ctx->d_btab + btab_desc_bytes(nvol)) + nvol;
    return launch_pdl(mc_generate_multi_kernel<VT>, (unsigned int)grid, THREADS, smem, s, desc, gmaps, nvol, list,
                      ctx->d_totals, batch_host(ctx));
}

// Bricks of a batch, or -1 when a volume or the sum is out of range.
long long batch_bricks(const mcg_volume *vols, int32_t nvol) {
    long long nbricks = 0;
    for (int v = 0; v < nvol; ++v) nbricks += geometry(vols[v].nx, vols[v].ny, vols[v].nz).nbricks;
    return nbricks >= (1ll << 32) ? -1 : nbricks;
}

// Sizes the context's scratch for a batch.  Inside a stream capture nothing
// may be allocated: an earlier call of the same batch outside the capture
// has sized every buffer (MCG_ERR_STATE otherwise).
mcg_status batch_scratch(mcg_context *ctx, int32_t nvol, long long nbricks, cudaStream_t s) {
    if (mcg_capturing(s) &&
        (ctx->brick_tris_cap < (size_t)nbricks || ctx->brick_occ_cap < (size_t)(CHUNK_FIELDS * num_chunks(nbricks)) ||
         ctx->brick_vofs_cap < (size_t)nbricks || ctx->active_cap < (size_t)nbricks ||
         ctx->d_vol_sums_cap < (size_t)(2 * nvol) || ctx->h_vol_sums_cap < (size_t)(2 * nvol) ||
         ctx->batch_list_cap < (size_t)nbricks * sizeof(BatchBrick)))
        return MCG_ERR_STATE;
    if (!ensure(&ctx->batch_list, &ctx->batch_list_cap, (size_t)nbricks * sizeof(BatchBrick)) ||
        !ensure(&ctx->brick_tris, &ctx->brick_tris_cap, (size_t)nbricks) ||
        !ensure(&ctx->brick_occ, &ctx->brick_occ_cap, (size_t)(CHUNK_FIELDS * num_chunks(nbricks))) ||
        !ensure(&ctx->brick_vofs, &ctx->brick_vofs_cap, (size_t)nbricks) ||
        !ensure(&ctx->active, &ctx->active_cap, (size_t)nbricks) ||
        !ensure(&ctx->d_vol_sums, &ctx->d_vol_sums_cap, (size_t)(2 * nvol)))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    if (ctx->h_vol_sums_cap < (size_t)(2 * nvol)) {
        if (ctx->counts_pending) cudaEventSynchronize(ctx->counts_ready);
        if (ctx->h_vol_sums) cudaFreeHost(ctx->h_vol_sums);
        ctx->h_vol_sums = nullptr;
        ctx->h_vol_sums_cap = 0;
        ctx->h_vol_sums_dev = nullptr;
        if (cudaHostAlloc((void **)&ctx->h_vol_sums, sizeof(unsigned long long) * 2 * nvol,
                          cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess)
            return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        ctx->h_vol_sums_cap = 2 * nvol;
        // the batch's scan writes the sums straight into host memory through
        // this address; without one the host copies them
        if (cudaHostGetDevicePointer((void **)&ctx->h_vol_sums_dev, ctx->h_vol_sums, 0) != cudaSuccess) {
            cudaGetLastError();
            ctx->h_vol_sums_dev = nullptr;
        }
    }
    return MCG_OK;
}

// The count launches of a batch whose table is on the device: one reset
// launch for the counters, the count pass, the scan (which also resolves
// the active list for the generate launch).
cudaError_t launch_batch_count(mcg_context *ctx, int32_t vtype, int32_t nvol, long long nbricks, cudaStream_t s) {
    const long long cw = (long long)CHUNK_FIELDS * num_chunks(nbricks);
    long long rg = (cw + 255) / 256;
    if (rg < 1) rg = 1;
    if (rg > 4LL * ctx->num_sms) rg = 4LL * ctx->num_sms;
    mc_batch_reset_kernel<<<(unsigned int)rg, 256, 0, s>>>(ctx->d_totals, ctx->d_vol_sums, nvol, ctx->brick_occ, cw);
    if (vtype == MCG_VOXEL_SHORT2) launch_classify_multi<MCG_VOXEL_SHORT2>(ctx, nvol, nbricks, s);
    else launch_classify_multi<MCG_VOXEL_FLOAT2>(ctx, nvol, nbricks, s);
    MeshTotals *host = batch_host(ctx);
    const ScanBatch bt{reinterpret_cast<const VolDesc *>(ctx->d_btab), nvol, ctx->d_vol_sums,
                       reinterpret_cast<BatchBrick *>(ctx->batch_list), host ? ctx->h_vol_sums_dev : nullptr};
    launch_pdl(mc_scan_kernel<true>, (unsigned int)num_chunks(nbricks), CHUNK, 0, s, (const uint32_t *)ctx->brick_tris,
               ctx->brick_occ, nbricks, ctx->brick_vofs, ctx->active, (unsigned long long *)nullptr, ctx->d_totals,
               host, bt);
    return cudaGetLastError();
}

// the totals and per-volume sums in the host copies, marked pending: written
// there by the kernels when mapped, copied otherwise
cudaError_t batch_counts_out(mcg_context *ctx, int32_t nvol, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    if (!batch_host(ctx)) {
        e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->h_vol_sums, ctx->d_vol_sums, sizeof(unsigned long long) * 2 * nvol,
                                cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = mcg_counts_event(ctx, s);
    return e;
}

// host state after a batch's count launches
void batch_state(mcg_context *ctx, const mcg_volume *vols, int32_t nvol, long long nbricks) {
    ctx->counters_clean = false;  // the batched launches leave the counters in use
    ctx->batch_classified = true;
    ctx->cls_fused = false;       // the batch's scan wrote the totals
    ctx->batch_nvol = nvol;
    ctx->batch_nbricks = nbricks;
    ctx->batch_vtype = vols[0].voxel_type;
    ctx->batch_first_data = vols[0].data;
    if (ctx->batch_caps_cap < (size_t)nvol) {
        delete[] ctx->batch_caps;
        ctx->batch_caps = new int64_t[nvol];
        ctx->batch_caps_cap = nvol;
    }
    for (int v = 0; v < nvol; ++v) ctx->batch_caps[v] = -1;
    ctx->classified = false;  // the single-volume state no longer matches the scratch
}

}  // namespace
}  // namespace mcg

mcg_status mcg_mc_classify_batched(mcg_context *ctx, const mcg_volume *vols, int32_t nvol, mcg_stream_t stream) {
    if (!ctx || !batch_ok(vols, nvol)) return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const long long nbricks = batch_bricks(vols, nvol);
    if (nbricks < 0) return MCG_ERR_INVALID_ARG;
    mcg_status st = batch_scratch(ctx, nvol, nbricks, s);
    if (st != MCG_OK) return st;
    long long total = 0;
    st = upload_btab(ctx, vols, nullptr, nvol, true, s, &total);
    if (st != MCG_OK) return st;
    e = launch_batch_count(ctx, vols[0].voxel_type, nvol, nbricks, s);
    if (e == cudaSuccess) e = batch_counts_out(ctx, nvol, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    batch_state(ctx, vols, nvol, nbricks);
    return MCG_OK;
}

mcg_status mcg_mc_counts_batched(mcg_context *ctx, mcg_mesh_counts *out, int32_t nvol) {
    if (!ctx || !out) return MCG_ERR_INVALID_ARG;
    if (!ctx->batch_classified) return MCG_ERR_STATE;
    if (nvol != ctx->batch_nvol) return MCG_ERR_INVALID_ARG;
    if (ctx->counts_pending) {
        cudaError_t e = cudaEventSynchronize(ctx->counts_ready);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        ctx->counts_pending = false;
    }
    mcg_status worst = MCG_OK;
    for (int v = 0; v < nvol; ++v) {
        mcg_mesh_counts &c = out[v];
        c.triangles = (int64_t)ctx->h_vol_sums[2 * v];
        c.vertices = 3 * c.triangles;
        c.occupied = (int64_t)ctx->h_vol_sums[2 * v + 1];
        c.active_bricks = 0;
        c.status = MCG_OK;
        if (ctx->h_totals->flags & 1u) c.status = MCG_ERR_TIMEOUT;
        else if (ctx->batch_caps[v] >= 0 && c.vertices > ctx->batch_caps[v]) c.status = MCG_ERR_CAPACITY;
        c.reserved = 0;
        if (c.status != MCG_OK && worst != MCG_ERR_TIMEOUT) worst = (mcg_status)c.status;
    }
    return worst;
}

mcg_status mcg_mc_generate_batched(mcg_context *ctx, const mcg_volume *vols, const mcg_mesh_out *outs, int32_t nvol,
                                   mcg_stream_t stream) {
    if (!ctx || !batch_ok(vols, nvol) || !outs) return MCG_ERR_INVALID_ARG;
    if (!ctx->batch_classified || nvol != ctx->batch_nvol || vols[0].voxel_type != ctx->batch_vtype ||
        vols[0].data != ctx->batch_first_data)
        return MCG_ERR_STATE;
    for (int v = 0; v < nvol; ++v)
        if (outs[v].capacity_vertices < 0) return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    for (int v = 0; v < nvol; ++v)
        if (outs[v].ver_voxel) {
            e = cudaMemsetAsync(outs[v].ver_voxel, 0, sizeof(int16_t) * (size_t)vols[v].nx * vols[v].ny * vols[v].nz, s);
            if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        }
    long long total = 0;
    mcg_status st = upload_btab(ctx, vols, outs, nvol, false, s, &total);
    if (st != MCG_OK) return st;
    if (total != ctx->batch_nbricks) return MCG_ERR_STATE;
    // the scan cleared the counter; calls on the context since may have used it
    e = cudaMemsetAsync(&ctx->d_totals->gen_ticket, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    if (vols[0].voxel_type == MCG_VOXEL_SHORT2) e = launch_generate_multi<MCG_VOXEL_SHORT2>(ctx, nvol, total, s);
    else e = launch_generate_multi<MCG_VOXEL_FLOAT2>(ctx, nvol, total, s);
    if (e == cudaSuccess && !batch_host(ctx))
        e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = mcg_counts_event(ctx, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    for (int v = 0; v < nvol; ++v) ctx->batch_caps[v] = outs[v].capacity_vertices;
    return MCG_OK;
}

mcg_status mcg_mc_extract_batched(mcg_context *ctx, const mcg_volume *vols, const mcg_mesh_out *outs, int32_t nvol,
                                  mcg_stream_t stream) {
    // count and generate without a host round trip in between: one table
    // upload (volumes, tensor maps and outputs), the reset, count, scan and
    // generate launches chained on the device, one copy of the counts at the end
    if (!ctx || !batch_ok(vols, nvol) || !outs) return MCG_ERR_INVALID_ARG;
    for (int v = 0; v < nvol; ++v)
        if (outs[v].capacity_vertices < 0) return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const long long nbricks = batch_bricks(vols, nvol);
    if (nbricks < 0) return MCG_ERR_INVALID_ARG;
    mcg_status st = batch_scratch(ctx, nvol, nbricks, s);
    if (st != MCG_OK) return st;
    for (int v = 0; v < nvol; ++v)
        if (outs[v].ver_voxel) {
            e = cudaMemsetAsync(outs[v].ver_voxel, 0, sizeof(int16_t) * (size_t)vols[v].nx * vols[v].ny * vols[v].nz, s);
            if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        }
    long long total = 0;
    st = upload_btab(ctx, vols, outs, nvol, true, s, &total);
    if (st != MCG_OK) return st;
    e = launch_batch_count(ctx, vols[0].voxel_type, nvol, nbricks, s);
    if (e == cudaSuccess) {
        if (vols[0].voxel_type == MCG_VOXEL_SHORT2) e = launch_generate_multi<MCG_VOXEL_SHORT2>(ctx, nvol, nbricks, s);
        else e = launch_generate_multi<MCG_VOXEL_FLOAT2>(ctx, nvol, nbricks, s);
    }
    if (e == cudaSuccess) e = batch_counts_out(ctx, nvol, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    batch_state(ctx, vols, nvol, nbricks);
    for (int v = 0; v < nvol; ++v) ctx->batch_caps[v] = outs[v].capacity_vertices;
    return MCG_OK;
}

// ---- extraction without any allocation ------------------------------------------
// For callers that cannot allocate device memory: the scratch of the three
// passes lives in one file-scope device array of fixed size.  The array is
// part of this library's device code: CUDA reserves it when it loads that
// code onto a device -- at the first use of any kernel of this file on the
// device under lazy module loading (CUDA_MODULE_LOADING=LAZY, the default),
// at context creation with CUDA_MODULE_LOADING=EAGER -- and holds it until
// the process exits.
namespace mcg {
namespace {

constexpr long long kNoAllocBricks = MCG_NOALLOC_MAX_BRICKS;
constexpr size_t kNoAllocTrisOff = 0;
constexpr size_t kNoAllocOccOff = kNoAllocTrisOff + sizeof(uint32_t) * kNoAllocBricks;
static_assert(CHUNK_FIELDS * ((kNoAllocBricks + CHUNK - 1) / CHUNK) <= kNoAllocBricks, "chunk sums fit their region");
constexpr size_t kNoAllocVofsOff = kNoAllocOccOff + sizeof(uint32_t) * kNoAllocBricks;
constexpr size_t kNoAllocActiveOff = kNoAllocVofsOff + sizeof(unsigned long long) * kNoAllocBricks;
constexpr size_t kNoAllocListVofsOff = kNoAllocActiveOff + sizeof(uint32_t) * kNoAllocBricks;
constexpr size_t kNoAllocTotalsOff = kNoAllocListVofsOff + sizeof(unsigned long long) * kNoAllocBricks;
constexpr size_t kNoAllocBytes = kNoAllocTotalsOff + 256;
static_assert(kNoAllocVofsOff % 8 == 0 && kNoAllocListVofsOff % 8 == 0 && kNoAllocTotalsOff % 8 == 0,
              "scratch alignment");
static_assert(kNoAllocBytes == MCG_NOALLOC_SCRATCH_BYTES, "scratch size stated in mcg.h");

// brick counts, soup offsets, active-brick list and totals of one call
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

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
    // the host-side symbol is only a stand-in: the kernels need the array's
    // device address on the current device.  It is looked up on every call
    // (no allocation once the module is loaded), so a module reloaded after
    // cudaDeviceReset is never addressed through a stale pointer.
    void *addr = nullptr;
    e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess || !addr) { cudaGetLastError(); return MCG_ERR_CUDA; }
    unsigned char *base = static_cast<unsigned char *>(addr);
    Scratch sc;
    sc.tris = reinterpret_cast<uint32_t *>(base + kNoAllocTrisOff);
    sc.chunk = reinterpret_cast<uint32_t *>(base + kNoAllocOccOff);  // CHUNK_FIELDS * 256 chunk sums at most
    sc.vofs = reinterpret_cast<unsigned long long *>(base + kNoAllocVofsOff);
    sc.active = reinterpret_cast<uint32_t *>(base + kNoAllocActiveOff);
    sc.list_vofs = reinterpret_cast<unsigned long long *>(base + kNoAllocListVofsOff);
    sc.host = nullptr;
    sc.totals = reinterpret_cast<MeshTotals *>(base + kNoAllocTotalsOff);
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    cudaStream_t s = (cudaStream_t)stream;
    // The count phase accumulates into the chunk sums and draws from the work
    // counters in the totals, and a completed scan leaves both clear; a call
    // that stopped between its launches (an error, or a call that overlapped
    // another) would leave them dirty for every later call.  So each call
    // clears them itself (memsets, no allocation); every other scratch entry
    // read later is written first by the launches below.
    e = cudaMemsetAsync(sc.chunk, 0, sizeof(uint32_t) * CHUNK_FIELDS * num_chunks(g.nbricks), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sc.totals, 0, sizeof(MeshTotals), s);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    e = launch_count_phase(vol, g, sc, sms, s, kDefaultMcConfig, false);
    if (e == cudaSuccess) e = launch_generate_phase(vol, g, sc, out, sms, s, kDefaultMcConfig);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    // counts: copy the totals out of the array into a host variable and wait
    MeshTotals t;
    e = cudaMemcpyAsync(&t, sc.totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    counts->occupied = (int64_t)t.occupied;
    counts->triangles = (int64_t)t.triangles;
    counts->vertices = (int64_t)t.vertices;
    counts->active_bricks = (int64_t)t.active_bricks;
    counts->status = MCG_OK;
    if (t.flags & 1u) counts->status = MCG_ERR_TIMEOUT;
    else if (counts->vertices > out->capacity_vertices) counts->status = MCG_ERR_CAPACITY;
    counts->reserved = 0;
    return (mcg_status)counts->status;
}
