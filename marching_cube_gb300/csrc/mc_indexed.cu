// Indexed marching-cubes extraction on sm_103a: one vertex per grid edge the
// surface crosses, shared by every triangle that uses it.
//
// The reference emits a triangle soup only (cu_marching_cubes_v1.cu:228-396)
// and merges vertices afterwards in its OBJ writer by comparing printed
// coordinates (cu_kinect_fusion_v1.cu:3625-3726).  Here the merge is exact
// and happens on the device: a vertex is identified by its grid edge.
//
// Ownership.  An edge is named by its lower voxel (x, y, z) and its axis.
// It carries a vertex iff its two voxels differ in sign (tsdf < 0) and at
// least one of the (up to four) cubes around it is valid -- inside the cube
// range and with no weight-0 corner.  Such a cube always emits triangles
// using the edge (its case is neither 0 nor 255 and the triangle table uses
// exactly the crossed edges), so every triangle edge has a vertex.  The
// brick whose voxel range [x0, x0+32) x [y0, y0+8) x [z0, z0+8) holds the
// lower voxel owns the edge; the last brick along an axis also owns voxel
// n-1 when the brick grid stops one short of it.
//
// Passes (bricks of 32x8x8 cubes, as the soup path):
//   1. mc_idx_count_kernel: per brick, triangles T and owned vertices U;
//   2. mc_idx_scan_kernel:  exclusive scans of T and U, active bricks;
//   3. mc_idx_vertex_kernel: every owned edge -> position, normal, and
//      edge_map[edge] = vertex id;
//   4. mc_idx_triangle_kernel: every triangle -> three edge_map lookups.
// All four read a 40x10x10 voxel tile per brick ([x0-4, x0+36) x
// [y0-1, y0+9) x [z0-1, z0+9); x rounded down to a 16-byte boundary) through
// a 2-stage TMA ring, and turn its 100 rows into 40-bit sign / weight-0
// masks: bit i of a row is voxel x0-4+i.  Cube validity of the 9x9 cube rows
// around the brick and the crossing of every edge come from shifts and
// ANDs of those masks.
//
// Vertex position: the reference's edge interpolation evaluated from the
// lower voxel to the upper one, t = (0 - f_lo) / (f_hi - f_lo + 1e-15f)
// (the soup evaluates each cube's edge in its own corner order, so a shared
// edge's soup copies can differ from each other in the last bit).  Normal:
// the reference's surface normal at that position.
#include "mc_common.cuh"

namespace mcg {
namespace {

constexpr int IX = 40, IY = 10, IZ = 10;  // tile extent
constexpr int ITILE = IX * IY * IZ;       // 4000 voxels
constexpr int IROWS = IY * IZ;            // 100 voxel rows
constexpr int ICR = 9;                    // cube rows per axis: y0-1 .. y0+7
constexpr int ITHREADS = 256;
constexpr int IWARPS = ITHREADS / 32;
constexpr int ISTAGES = 2;
constexpr int IOWN_ROWS = 81;             // owned voxel rows per brick, at most 9 x 9

// Row mask over the 40 voxels of a tile row: bit i = voxel x0-4+i negative /
// weight 0.  `row` is 16-byte aligned (40 voxels = 160 or 320 bytes).
template <int VT>
struct RowMask40;

template <>
struct RowMask40<MCG_VOXEL_SHORT2> {
    static __device__ __forceinline__ void build(const short2 *row, unsigned long long &neg,
                                                 unsigned long long &dead) {
        const uint4 *q = reinterpret_cast<const uint4 *>(row);
        unsigned long long n = 0, d = 0;
#pragma unroll
        for (int k = 0; k < 10; ++k) {
            const uint4 v = q[k];
            const unsigned int w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                n |= (unsigned long long)((w[j] >> 15) & 1u) << (4 * k + j);  // tsdf (low half) < 0
                d |= (unsigned long long)(w[j] < 0x10000u) << (4 * k + j);    // w (high half) == 0
            }
        }
        neg = n;
        dead = d;
    }
};

template <>
struct RowMask40<MCG_VOXEL_FLOAT2> {
    static __device__ __forceinline__ void build(const float2 *row, unsigned long long &neg,
                                                 unsigned long long &dead) {
        const float4 *q = reinterpret_cast<const float4 *>(row);
        unsigned long long n = 0, d = 0;
#pragma unroll
        for (int k = 0; k < 20; ++k) {
            const float4 v = q[k];
            n |= (unsigned long long)(v.x < 0.f) << (2 * k);
            n |= (unsigned long long)(v.z < 0.f) << (2 * k + 1);
            d |= (unsigned long long)(v.y == 0.f) << (2 * k);
            d |= (unsigned long long)(v.w == 0.f) << (2 * k + 1);
        }
        neg = n;
        dead = d;
    }
};

template <int VT>
struct IdxSmem {
    static constexpr int STAGE_BYTES = pad128(ITILE * Vox<VT>::bytes);
    unsigned char tiles[ISTAGES][STAGE_BYTES];
    unsigned long long neg[IROWS], dead[IROWS];
    unsigned long long valid[ICR * ICR];  // bit i: cube x0-4+i of cube row (cy, cz) is valid
    uint64_t bars[ISTAGES];
    long long sbrick[ISTAGES];
    unsigned int scan[ITHREADS];
    unsigned long long vmask[ITHREADS];  // vertex pass: owned crossed edges of each (row, axis) slot
    // triangle pass: per cube row (64, (z, y) order) the occupied cubes (bit
    // x), their triangle counts (4 bits per cube) and the row's first
    // triangle in the brick; the cube index of every cube of the brick
    unsigned int rowocc[BY * BZ];
    unsigned int rownib[BY * BZ][4];
    unsigned int rowoff[BY * BZ];
    unsigned char cci[BRICK_CUBES];
    unsigned int wsum[IWARPS][4];
    alignas(16) signed char tri[256][16];
    unsigned char ntri[256];
    int abort;
};

__device__ __forceinline__ int trow(int ty, int tz) { return tz * IY + ty; }

// voxel ranges a brick owns (lower voxels of its edges)
struct Own {
    int nx_own, ny_own, nz_own;  // 32/33, 8/9, 8/9
};

__device__ __forceinline__ Own ownership(BrickPos bp, int nbx, int nby, int nbz, int nx, int ny, int nz) {
    Own o;
    o.nx_own = (bp.x0 / BX == nbx - 1) ? nx - bp.x0 : BX;
    o.ny_own = (bp.y0 / BY == nby - 1) ? ny - bp.y0 : BY;
    o.nz_own = (bp.z0 / BZ == nbz - 1) ? nz - bp.z0 : BZ;
    return o;
}

// bits [lo, hi] of a 64-bit word (empty when hi < lo)
__device__ __forceinline__ unsigned long long bit_range(int lo, int hi) {
    if (hi < lo) return 0ull;
    const unsigned long long upto = hi >= 63 ? ~0ull : ((1ull << (hi + 1)) - 1ull);
    return upto & ~((1ull << lo) - 1ull);
}

// Row masks of the tile and validity of the 9x9 cube rows around the brick.
// Called by every thread; ends with a barrier.
template <int VT>
__device__ __forceinline__ void idx_prepare(IdxSmem<VT> &S, const typename Vox<VT>::T *tile, BrickPos bp, int nx,
                                            int ny, int nz) {
    const int tid = threadIdx.x;
    if (tid < IROWS) RowMask40<VT>::build(tile + tid * IX, S.neg[tid], S.dead[tid]);
    __syncthreads();
    if (tid < ICR * ICR) {
        const int cty = tid % ICR, ctz = tid / ICR;
        const int cy = bp.y0 - 1 + cty, cz = bp.z0 - 1 + ctz;
        unsigned long long v = 0;
        if (cy >= 0 && cy <= ny - 2 && cz >= 0 && cz <= nz - 2) {
            const int r00 = trow(cty, ctz), r01 = r00 + 1, r10 = r00 + IY, r11 = r10 + 1;
            const unsigned long long d = S.dead[r00] | S.dead[r01] | S.dead[r10] | S.dead[r11];
            // cube cx = x0-4+i exists for 0 <= cx <= nx-2 and needs voxel bit i+1 <= 39
            const int lo = bp.x0 >= 4 ? 0 : 4 - bp.x0;
            const int hi = min(38, nx - 2 - (bp.x0 - 4));
            v = ~(d | (d >> 1)) & bit_range(lo, hi);
        }
        S.valid[tid] = v;
    }
    __syncthreads();
}

template <int VT>
__device__ __forceinline__ unsigned long long valid_at(const IdxSmem<VT> &S, int cty, int ctz) {
    return (cty < ICR && ctz < ICR) ? S.valid[ctz * ICR + cty] : 0ull;
}

// Owned edges of axis `axis` whose lower voxel lies in tile row (ty, tz),
// 1 <= ty, tz <= 9: bit i = edge at x = x0-4+i.
template <int VT>
__device__ __forceinline__ unsigned long long owned_edges(const IdxSmem<VT> &S, int ty, int tz, int axis,
                                                          unsigned long long own_bits) {
    const unsigned long long n = S.neg[trow(ty, tz)];
    unsigned long long cross, share;
    if (axis == 0) {
        cross = n ^ (n >> 1);
        share = valid_at(S, ty, tz) | valid_at(S, ty - 1, tz) | valid_at(S, ty, tz - 1) | valid_at(S, ty - 1, tz - 1);
    } else if (axis == 1) {
        if (ty + 1 >= IY) return 0ull;
        cross = n ^ S.neg[trow(ty + 1, tz)];
        const unsigned long long v = valid_at(S, ty, tz) | valid_at(S, ty, tz - 1);
        share = v | (v << 1);
    } else {
        if (tz + 1 >= IZ) return 0ull;
        cross = n ^ S.neg[trow(ty, tz + 1)];
        const unsigned long long v = valid_at(S, ty, tz) | valid_at(S, ty - 1, tz);
        share = v | (v << 1);
    }
    return cross & share & own_bits;
}

// occupied cubes of brick cube row (cy, cz) = tile cube row (1+cy, 1+cz):
// bit i = cube x0-4+i, i in [4, 36)
template <int VT>
__device__ __forceinline__ CubeRow idx_cube_row(const IdxSmem<VT> &S, int cy, int cz) {
    CubeRow r;
    const int cty = cy + 1, ctz = cz + 1;
    const int r00 = trow(cty, ctz), r01 = r00 + 1, r10 = r00 + IY, r11 = r10 + 1;
    r.a = S.neg[r00];
    r.b = S.neg[r01];
    r.c = S.neg[r10];
    r.d = S.neg[r11];
    const unsigned long long all = r.a & (r.a >> 1) & r.b & (r.b >> 1) & r.c & (r.c >> 1) & r.d & (r.d >> 1);
    const unsigned long long any = r.a | (r.a >> 1) | r.b | (r.b >> 1) | r.c | (r.c >> 1) | r.d | (r.d >> 1);
    const unsigned long long occ = any & ~all & S.valid[ctz * ICR + cty] & (0xffffffffull << 4);
    r.occ = (unsigned int)(occ >> 4);  // bit x = brick cube x
    return r;
}

// cube index of brick cube x of a row built by idx_cube_row
__device__ __forceinline__ unsigned int idx_cube_index(const CubeRow &r, int x) {
    const int i = x + 4;
    return (unsigned int)(((r.a >> i) & 1) | (((r.a >> (i + 1)) & 1) << 1) | (((r.b >> (i + 1)) & 1) << 2) |
                          (((r.b >> i) & 1) << 3) | (((r.c >> i) & 1) << 4) | (((r.c >> (i + 1)) & 1) << 5) |
                          (((r.d >> (i + 1)) & 1) << 6) | (((r.d >> i) & 1) << 7));
}

// block-wide exclusive scan of one value per thread (ITHREADS); returns the
// thread's offset, *total the sum.  Ends with a barrier.
template <int VT>
__device__ __forceinline__ unsigned int block_scan(IdxSmem<VT> &S, unsigned int v, unsigned int *total) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) S.wsum[warp][0] = x;
    __syncthreads();
    unsigned int base = 0, all = 0;
#pragma unroll
    for (int w = 0; w < IWARPS; ++w) {
        const unsigned int s = S.wsum[w][0];
        if (w < warp) base += s;
        all += s;
    }
    __syncthreads();
    *total = all;
    return base + x - v;
}

// Streams bricks through the CTA's TMA ring (or plain loads) and calls
// body(tile, b, bp) for each.  Work items come from the device counter
// `ticket` (thread 0 draws the next refill one item ahead, so the counter's
// round trip overlaps the current brick); `list` (may be null) maps an item
// to a brick id.  Returns false when a bounded wait expired.
template <int VT, bool TMA, class Body>
__device__ __forceinline__ bool for_each_brick(IdxSmem<VT> &S, const CUtensorMap *map,
                                               const typename Vox<VT>::T *__restrict__ vol, int nx, int ny, int nz,
                                               int nbx, int nby, long long nitems, const uint32_t *list,
                                               unsigned int *ticket, Body body) {
    using V = Vox<VT>;
    using T = typename V::T;
    const int tid = threadIdx.x;
    auto draw = [&]() -> long long {
        const unsigned int t = atomicAdd(ticket, 1u);
        if ((long long)t >= nitems) return -1ll;
        return list ? (long long)list[t] : (long long)t;
    };
    long long pend = -1;
    if (tid == 0) {
        S.abort = 0;
        if (TMA) {
            for (int s = 0; s < ISTAGES; ++s) mbar_init(&S.bars[s], 1);
            fence_barrier_init();
            bool more = true;
            for (int s = 0; s < ISTAGES; ++s) {
                const long long b = more ? draw() : -1ll;
                more = b >= 0;
                S.sbrick[s] = b;
                if (!more) continue;
                const BrickPos bp = brick_pos(b, nbx, nby);
                mbar_arrive_expect_tx(&S.bars[s], ITILE * V::bytes);
                tma_load_3d(S.tiles[s], map, &S.bars[s], bp.x0 - 4, bp.y0 - 1, bp.z0 - 1);
            }
            if (more) pend = draw();
        }
    }
    __syncthreads();
    for (int it = 0;; ++it) {
        const int s = TMA ? it % ISTAGES : 0;
        T *tile = reinterpret_cast<T *>(S.tiles[s]);
        if (!TMA) {
            if (tid == 0) S.sbrick[0] = draw();
            __syncthreads();
        }
        const long long b = S.sbrick[s];
        if (b < 0) break;  // uniform
        if (TMA) {
            if (tid == 0 && !mbar_wait(&S.bars[s], (uint32_t)((it / ISTAGES) & 1))) S.abort = 1;
            __syncthreads();
            if (S.abort) break;
        } else {
            const BrickPos fp = brick_pos(b, nbx, nby);
            fill_tile<VT, IX, IY, IZ>(tile, vol, nx, ny, nz, fp.x0 - 4, fp.y0 - 1, fp.z0 - 1);
            __syncthreads();
        }
        body(tile, b, brick_pos(b, nbx, nby));
        __syncthreads();  // tile s and the shared scratch are free again
        if (TMA && tid == 0) {
            const long long nb2 = pend;
            S.sbrick[s] = nb2;
            if (nb2 >= 0) {
                const BrickPos np = brick_pos(nb2, nbx, nby);
                mbar_arrive_expect_tx(&S.bars[s], ITILE * V::bytes);
                tma_load_3d(S.tiles[s], map, &S.bars[s], np.x0 - 4, np.y0 - 1, np.z0 - 1);
                pend = draw();
            }
        }
        // S.sbrick[s] is next read at the top of iteration it + ISTAGES, after
        // the barriers of iteration it + 1; the plain path rewrites sbrick[0]
        // only after the barrier above
    }
    if (TMA && S.abort) {
        if (tid == 0)
            for (int s = 0; s < ISTAGES; ++s) mbar_wait(&S.bars[s], 0, 100000000ull);
        return false;
    }
    return true;
}

// True when the tile holds both negative and non-negative voxels; a tile of
// one sign has no crossed edge and no emitting cube.  Every thread; one barrier.
template <int VT>
__device__ __forceinline__ bool idx_tile_mixed(IdxSmem<VT> &S, const typename Vox<VT>::T *tile) {
    constexpr int NQ = ITILE * Vox<VT>::bytes / 16;
    const uint4 *q = reinterpret_cast<const uint4 *>(tile);
    unsigned int neg_any = 0, pos_any = 0;
    for (int i = threadIdx.x; i < NQ; i += ITHREADS) {
        const uint4 v = q[i];
        if (VT == MCG_VOXEL_SHORT2) {
            neg_any |= v.x | v.y | v.z | v.w;  // bit 15 of each word: tsdf sign
            pos_any |= ~(v.x & v.y & v.z & v.w);
        } else {
            const bool n0 = __uint_as_float(v.x) < 0.f, n1 = __uint_as_float(v.z) < 0.f;
            neg_any |= (unsigned int)(n0 | n1) << 15;
            pos_any |= (unsigned int)(!n0 | !n1) << 15;
        }
    }
    neg_any = __reduce_or_sync(0xffffffffu, neg_any & 0x8000u);
    pos_any = __reduce_or_sync(0xffffffffu, pos_any & 0x8000u);
    if ((threadIdx.x & 31) == 0) S.wsum[threadIdx.x >> 5][3] = (neg_any ? 1u : 0u) | (pos_any ? 2u : 0u);
    __syncthreads();
    unsigned int m = 0;
#pragma unroll
    for (int w = 0; w < IWARPS; ++w) m |= S.wsum[w][3];
    return m == 3u;
}

struct IdxParams {
    const void *vol;
    int nx, ny, nz;
    float cell;
    int nbx, nby, nbz;
    long long nbricks;
    uint32_t *brick_tris;
    uint32_t *brick_uniq;
    uint32_t *chunk;  // 4 per chunk: triangles, active bricks, occupied cubes, vertices
    const uint32_t *active;
    const unsigned long long *brick_tofs;  // triangle offsets
    const unsigned long long *brick_uofs;  // vertex offsets
    MeshTotals *totals;
    uint32_t *edge_map;
    uint32_t *cand;  // count pass: the bricks whose owned edges are counted (totals->idx_cand of them)
    mcg_indexed_out out;
};

template <int VT>
__device__ __forceinline__ void load_tables(IdxSmem<VT> &S) {
    load_tri_table(S.tri, threadIdx.x, ITHREADS);
    for (int c = threadIdx.x; c < 256; c += ITHREADS) S.ntri[c] = (c == 0 || c == 255) ? 0 : g_nverts[c] / 3;
}

// ---- pass 1: counts --------------------------------------------------------------
// The bricks whose owned edges can be vertices: a vertex needs a valid
// occupied cube around its edge, and the cubes around the edges a brick owns
// lie in the brick or in its neighbours at -x, -y, -z, -x-y, -x-z, -y-z; an
// occupied valid cube emits triangles, so a brick is listed when one of
// those seven bricks has triangles (counts of the soup's count pass).  The
// others own no vertex.  One thread per brick, one atomic per warp.
__global__ void __launch_bounds__(256) mc_idx_cand_kernel(IdxParams p) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool cand = false;
    if (b < p.nbricks) {
        const long long r = b / p.nbx;
        const int bx = (int)(b - r * p.nbx), by = (int)(r % p.nby), bz = (int)(r / p.nby);
        const long long sy = p.nbx, sz = (long long)p.nbx * p.nby;
#pragma unroll
        for (int k = 0; k < 7; ++k) {  // (dx, dy, dz) in {0,1}^3 but (1,1,1)
            const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
            if (bx >= dx && by >= dy && bz >= dz && p.brick_tris[b - dx - dy * sy - dz * sz] != 0u) cand = true;
        }
        if (!cand) p.brick_uniq[b] = 0u;
    }
    const unsigned int m = __ballot_sync(0xffffffffu, cand);
    if (m) {
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        unsigned int base = 0;
        if (lane == leader) base = atomicAdd(&p.totals->idx_cand, (unsigned int)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (cand) p.cand[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)b;
    }
}

// Per brick: triangles, active flag, occupied cubes, owned vertices, into the
// brick arrays and the chunk sums.  OWNED: the listed bricks only, owned
// vertices only -- the triangles come from the soup's count pass (occupied
// cubes then come from its totals).
template <int VT, bool TMA, bool OWNED>
__global__ void __launch_bounds__(ITHREADS) mc_idx_count_kernel(const __grid_constant__ CUtensorMap map, IdxParams p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    IdxSmem<VT> &S = *reinterpret_cast<IdxSmem<VT> *>(smem_raw);
    load_tables(S);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long nitems = OWNED ? (long long)p.totals->idx_cand : p.nbricks;
    const bool ok = for_each_brick<VT, TMA>(
        S, &map, static_cast<const typename Vox<VT>::T *>(p.vol), p.nx, p.ny, p.nz, p.nbx, p.nby, nitems,
        OWNED ? p.cand : nullptr, &p.totals->cls_ticket, [&](const typename Vox<VT>::T *tile, long long b, BrickPos bp) {
            if (!idx_tile_mixed<VT>(S, tile)) {
                if (tid == 0) {
                    if (!OWNED) p.brick_tris[b] = 0;
                    p.brick_uniq[b] = 0;
                }
                return;  // uniform across the CTA
            }
            idx_prepare<VT>(S, tile, bp, p.nx, p.ny, p.nz);
            unsigned int t = 0, o = 0, u = 0;
            if (!OWNED && tid < BY * BZ) {
                const CubeRow r = idx_cube_row<VT>(S, tid % BY, tid / BY);
                o = __popc(r.occ);
                unsigned int m = r.occ;
                while (m) {
                    const int x = __ffs(m) - 1;
                    m &= m - 1;
                    t += S.ntri[idx_cube_index(r, x)];
                }
            }
            if (tid < IOWN_ROWS) {
                const Own ow = ownership(bp, p.nbx, p.nby, p.nbz, p.nx, p.ny, p.nz);
                const int oy = tid % 9, oz = tid / 9;
                if (oy < ow.ny_own && oz < ow.nz_own) {
                    const unsigned long long own = bit_range(4, 3 + ow.nx_own);
                    for (int a = 0; a < 3; ++a) u += __popcll(owned_edges<VT>(S, oy + 1, oz + 1, a, own));
                }
            }
            t = __reduce_add_sync(0xffffffffu, t);
            o = __reduce_add_sync(0xffffffffu, o);
            u = __reduce_add_sync(0xffffffffu, u);
            if (lane == 0) {
                S.wsum[warp][0] = t;
                S.wsum[warp][1] = o;
                S.wsum[warp][2] = u;
            }
            __syncthreads();
            if (tid == 0) {
                unsigned int T = 0, O = 0, U = 0;
                for (int w = 0; w < IWARPS; ++w) {
                    T += S.wsum[w][0];
                    O += S.wsum[w][1];
                    U += S.wsum[w][2];
                }
                if (OWNED) T = p.brick_tris[b];
                else p.brick_tris[b] = T;
                p.brick_uniq[b] = U;
                if (T || U) {
                    uint32_t *c = p.chunk + (b / CHUNK) * 4;
                    atomicAdd(c + 0, T);
                    atomicAdd(c + 1, 1u);
                    atomicAdd(c + 2, O);
                    atomicAdd(c + 3, U);
                }
            }
        });
    if (!ok && tid == 0) atomicOr(&p.totals->flags, 1u);
}

// ---- pass 2: scan ----------------------------------------------------------------
// One CTA per chunk of CHUNK bricks: chunk bases from the chunk sums, then a
// scan of the chunk's bricks; CTA 0 writes the totals.
__global__ void __launch_bounds__(CHUNK)
    mc_idx_scan_kernel(const uint32_t *__restrict__ brick_tris, const uint32_t *__restrict__ brick_uniq,
                       const uint32_t *__restrict__ chunk, long long nb, unsigned long long *__restrict__ brick_tofs,
                       unsigned long long *__restrict__ brick_uofs, uint32_t *__restrict__ active,
                       MeshTotals *__restrict__ totals, int keep_occupied) {
    __shared__ unsigned long long s_part[7][CHUNK / 32];
    __shared__ unsigned long long s_base[3];
    __shared__ unsigned int s_w[3][CHUNK / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long j = blockIdx.x;
    const long long nchunks = (nb + CHUNK - 1) / CHUNK;
    const long long upto = j == 0 ? nchunks : j;
    // bases (tris, active, verts) and, for CTA 0, totals (tris, active, occupied, verts)
    unsigned long long acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (long long i = tid; i < upto; i += CHUNK) {
        const unsigned long long ct = chunk[i * 4 + 0], ca = chunk[i * 4 + 1], co = chunk[i * 4 + 2],
                                 cu = chunk[i * 4 + 3];
        if (i < j) {
            acc[0] += ct;
            acc[1] += ca;
            acc[2] += cu;
        }
        acc[3] += ct;
        acc[4] += ca;
        acc[5] += co;
        acc[6] += cu;
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) {
#pragma unroll
        for (int o = 16; o; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if (lane == 0) s_part[k][warp] = acc[k];
    }
    __syncthreads();
    if (tid == 0) {
        unsigned long long r[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 7; ++k)
            for (int w = 0; w < CHUNK / 32; ++w) r[k] += s_part[k][w];
        s_base[0] = r[0];
        s_base[1] = r[1];
        s_base[2] = r[2];
        if (j == 0) {
            totals->triangles = r[3];
            totals->active_bricks = (unsigned int)r[4];
            if (!keep_occupied) totals->occupied = r[5];
            totals->vertices = r[6];
        }
    }
    __syncthreads();
    const long long b = j * CHUNK + tid;
    const unsigned int t = b < nb ? brick_tris[b] : 0u;
    const unsigned int u = b < nb ? brick_uniq[b] : 0u;
    const unsigned int f = (t | u) != 0;
    unsigned int it = t, iu = u, ia = f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int x = __shfl_up_sync(0xffffffffu, it, o);
        const unsigned int y = __shfl_up_sync(0xffffffffu, iu, o);
        const unsigned int z = __shfl_up_sync(0xffffffffu, ia, o);
        if (lane >= o) {
            it += x;
            iu += y;
            ia += z;
        }
    }
    if (lane == 31) {
        s_w[0][warp] = it;
        s_w[1][warp] = iu;
        s_w[2][warp] = ia;
    }
    __syncthreads();
    unsigned int wt = 0, wu = 0, wa = 0;
    for (int w = 0; w < warp; ++w) {
        wt += s_w[0][w];
        wu += s_w[1][w];
        wa += s_w[2][w];
    }
    if (b < nb) {
        brick_tofs[b] = s_base[0] + wt + it - t;
        brick_uofs[b] = s_base[2] + wu + iu - u;
        if (f) active[s_base[1] + wa + ia - f] = (uint32_t)b;
    }
}

// ---- pass 3: vertices ---------------------------------------------------------------
// Thread k < 243 takes owned row k/3 (rows in (z, y) order) and axis k%3;
// vertex ids follow (row, axis, x).
template <int VT, bool TMA>
__global__ void __launch_bounds__(ITHREADS) mc_idx_vertex_kernel(const __grid_constant__ CUtensorMap map, IdxParams p) {
    using V = Vox<VT>;
    using T = typename V::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    IdxSmem<VT> &S = *reinterpret_cast<IdxSmem<VT> *>(smem_raw);
    const T *__restrict__ vol = static_cast<const T *>(p.vol);
    const int tid = threadIdx.x;
    const float cell = p.cell;
    const long long capv = p.out.capacity_vertices;
    const bool ok = for_each_brick<VT, TMA>(
        S, &map, vol, p.nx, p.ny, p.nz, p.nbx, p.nby, (long long)p.totals->active_bricks, p.active,
        &p.totals->gen_ticket, [&](const T *tile, long long b, BrickPos bp) {
            idx_prepare<VT>(S, tile, bp, p.nx, p.ny, p.nz);
            unsigned long long m = 0;
            int oy = 0, oz = 0, axis = 0;
            if (tid < 3 * IOWN_ROWS) {
                const Own ow = ownership(bp, p.nbx, p.nby, p.nbz, p.nx, p.ny, p.nz);
                const int row = tid / 3;
                axis = tid % 3;
                oy = row % 9;
                oz = row / 9;
                if (oy < ow.ny_own && oz < ow.nz_own)
                    m = owned_edges<VT>(S, oy + 1, oz + 1, axis, bit_range(4, 3 + ow.nx_own));
            }
            unsigned int total;
            const unsigned int off = block_scan(S, (unsigned int)__popcll(m), &total);
            // the brick's vertices spread evenly over the threads: vertex v
            // belongs to the last (row, axis) slot whose offset is <= v (slots
            // without vertices share their offset with the next slot)
            S.vmask[tid] = m;
            S.scan[tid] = off;
            __syncthreads();
            const unsigned long long vbase = p.brick_uofs[b];
            for (unsigned int v = tid; v < total; v += ITHREADS) {
                int k = 0;
                {
                    int hi = 3 * IOWN_ROWS - 1;
                    while (k < hi) {
                        const int mid = (k + hi + 1) >> 1;
                        if (S.scan[mid] <= v) k = mid; else hi = mid - 1;
                    }
                }
                const unsigned long long mk = S.vmask[k];
                const unsigned int j = v - S.scan[k];  // the j-th owned edge of the slot
                const unsigned int mlo = (unsigned int)mk, mhi = (unsigned int)(mk >> 32);
                const unsigned int plo = (unsigned int)__popc(mlo);
                const int i = j < plo ? (int)__fns(mlo, 0, (int)j + 1) : 32 + (int)__fns(mhi, 0, (int)(j - plo) + 1);
                const int axis = k % 3, oy = (k / 3) % 9, oz = (k / 3) / 9;
                const int ty = oy + 1, tz = oz + 1;
                const int dy = axis == 1, dz = axis == 2, dx = axis == 0;
                const unsigned long long vid = vbase + v;
                const int x = bp.x0 - 4 + i, y = bp.y0 + oy, z = bp.z0 + oz;
                const T lo = tile[(tz * IY + ty) * IX + i];
                const T hi = tile[((tz + dz) * IY + ty + dy) * IX + i + dx];
                const float f0 = V::f(lo), f1 = V::f(hi);
                // node coordinates (x + 0.5) * cell (cu_marching_cubes_v1.cu:243-254)
                const float p0x = ((float)x + 0.5f) * cell, p0y = ((float)y + 0.5f) * cell,
                            p0z = ((float)z + 0.5f) * cell;
                const float p1x = ((float)(x + dx) + 0.5f) * cell, p1y = ((float)(y + dy) + 0.5f) * cell,
                            p1z = ((float)(z + dz) + 0.5f) * cell;
                // vertex_interp (:256-264), lower voxel first
                const float t = (0.0f - f0) / (f1 - f0 + 1e-15f);
                const float px = p0x + t * (p1x - p0x);
                const float py = p0y + t * (p1y - p0y);
                const float pz = p0z + t * (p1z - p0z);
                const long long key = 3 * lin3(p.nx, p.ny, x, y, z) + axis;
                p.edge_map[key] = (uint32_t)vid;
                if ((long long)vid < capv) {
                    if (p.out.positions) {
                        p.out.positions[3 * vid] = px;
                        p.out.positions[3 * vid + 1] = py;
                        p.out.positions[3 * vid + 2] = pz;
                    }
                    if (p.out.normals) {
                        const float3 n = normal_global<VT>(vol, p.nx, p.ny, p.nz, cell, px, py, pz);
                        p.out.normals[3 * vid] = n.x;
                        p.out.normals[3 * vid + 1] = n.y;
                        p.out.normals[3 * vid + 2] = n.z;
                    }
                    if (p.out.vi2vox) {
                        // store_point (:336-343): floor(P / cell - 0.5)
                        p.out.vi2vox[3 * vid] = (int32_t)floorf(px / cell - 0.5f);
                        p.out.vi2vox[3 * vid + 1] = (int32_t)floorf(py / cell - 0.5f);
                        p.out.vi2vox[3 * vid + 2] = (int32_t)floorf(pz / cell - 0.5f);
                    }
                    if (p.out.vertex_edge) p.out.vertex_edge[vid] = key;
                }
            }
        });
    if (!ok && tid == 0) atomicOr(&p.totals->flags, 1u);
}

// ---- pass 4: triangles -------------------------------------------------------------
// edge e of cube (cx, cy, cz) -> 3 * linear index of its lower voxel + axis
__device__ __forceinline__ long long edge_key(int nx, int ny, int cx, int cy, int cz, int e) {
    const int a = c_ea(e), b = c_eb(e);
    const int ax = c_cx(a), bx = c_cx(b), ay = c_cy(a), by = c_cy(b), az = c_cz(a), bz = c_cz(b);
    const int axis = ax != bx ? 0 : (ay != by ? 1 : 2);
    return 3 * lin3(nx, ny, cx + min(ax, bx), cy + min(ay, by), cz + min(az, bz)) + axis;
}

template <int VT, bool TMA>
__global__ void __launch_bounds__(ITHREADS)
    mc_idx_triangle_kernel(const __grid_constant__ CUtensorMap map, IdxParams p) {
    using T = typename Vox<VT>::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    IdxSmem<VT> &S = *reinterpret_cast<IdxSmem<VT> *>(smem_raw);
    load_tables(S);
    const int tid = threadIdx.x;
    const long long capt = p.out.capacity_triangles;
    const bool ok = for_each_brick<VT, TMA>(
        S, &map, static_cast<const T *>(p.vol), p.nx, p.ny, p.nz, p.nbx, p.nby, (long long)p.totals->active_bricks,
        p.active, &p.totals->idx_ticket, [&](const T *tile, long long b, BrickPos bp) {
            if (p.brick_tris[b] == 0) return;  // uniform across the CTA
            idx_prepare<VT>(S, tile, bp, p.nx, p.ny, p.nz);
            // one thread per cube row: occupancy, triangles per cube, row total
            unsigned int rt = 0;
            if (tid < BY * BZ) {
                const int row = tid;
                const CubeRow r = idx_cube_row<VT>(S, row % BY, row / BY);
                unsigned int nib[4] = {0u, 0u, 0u, 0u};
                unsigned int m = r.occ;
                while (m) {
                    const int x = __ffs(m) - 1;
                    m &= m - 1;
                    const unsigned int ci = idx_cube_index(r, x);
                    const unsigned int nt = S.ntri[ci];
                    S.cci[row * BX + x] = (unsigned char)ci;
                    nib[x >> 3] |= nt << ((x & 7) * 4);
                    rt += nt;
                }
                S.rowocc[row] = r.occ;
#pragma unroll
                for (int k = 0; k < 4; ++k) S.rownib[row][k] = nib[k];
            }
            unsigned int total;
            const unsigned int rbase = block_scan(S, rt, &total);
            if (tid < BY * BZ) S.rowoff[tid] = rbase;
            __syncthreads();
            // the brick's triangles spread evenly over the threads, in the
            // soup's order: rows in (z, y) order, cubes in x order, table order
            const unsigned long long tbase = p.brick_tofs[b];
            for (unsigned int t = tid; t < total; t += ITHREADS) {
                int row = 0;
                {
                    int hi = BY * BZ - 1;
                    while (row < hi) {
                        const int mid = (row + hi + 1) >> 1;
                        if (S.rowoff[mid] <= t) row = mid; else hi = mid - 1;
                    }
                }
                unsigned int j = t - S.rowoff[row];
                unsigned int m = S.rowocc[row];
                int x = 0;
                for (;;) {
                    x = __ffs(m) - 1;
                    const unsigned int n = (S.rownib[row][x >> 3] >> ((x & 7) * 4)) & 15u;
                    if (j < n) break;
                    j -= n;
                    m &= m - 1;
                }
                const unsigned long long tt = tbase + t;
                if ((long long)tt >= capt) continue;
                const unsigned int ci = S.cci[row * BX + x];
                const int gx = bp.x0 + x, gy = bp.y0 + row % BY, gz = bp.z0 + row / BY;
                // the soup's slot k holds edge tri[3j + 2 - k] (:322-333)
                if (p.out.triangles) {
                    const int e2 = S.tri[ci][3 * j + 2], e1 = S.tri[ci][3 * j + 1], e0 = S.tri[ci][3 * j];
                    p.out.triangles[3 * tt] = p.edge_map[edge_key(p.nx, p.ny, gx, gy, gz, e2)];
                    p.out.triangles[3 * tt + 1] = p.edge_map[edge_key(p.nx, p.ny, gx, gy, gz, e1)];
                    p.out.triangles[3 * tt + 2] = p.edge_map[edge_key(p.nx, p.ny, gx, gy, gz, e0)];
                }
                if (p.out.tri_cube) p.out.tri_cube[tt] = lin3(p.nx, p.ny, gx, gy, gz);
            }
        });
    if (!ok && tid == 0) atomicOr(&p.totals->flags, 1u);
}

// ---- host side -----------------------------------------------------------------------
template <int VT, bool TMA>
void launch_idx(int pass, const CUtensorMap &map, const IdxParams &p, int sms, long long items, cudaStream_t s) {
    const size_t smem = sizeof(IdxSmem<VT>);
    static int occ[3] = {0, 0, 0};
    long long grid;
    if (pass == 0) {
        if (!occ[0]) occ[0] = occupancy(mc_idx_count_kernel<VT, TMA, true>, ITHREADS, smem);
        grid = (long long)sms * occ[0];
    } else if (pass == 1) {
        if (!occ[1]) occ[1] = occupancy(mc_idx_vertex_kernel<VT, TMA>, ITHREADS, smem);
        grid = (long long)sms * occ[1];
    } else {
        if (!occ[2]) occ[2] = occupancy(mc_idx_triangle_kernel<VT, TMA>, ITHREADS, smem);
        grid = (long long)sms * occ[2];
    }
    if (grid > items) grid = items;
    if (grid < 1) grid = 1;
    if (pass == 0) mc_idx_count_kernel<VT, TMA, true><<<(int)grid, ITHREADS, smem, s>>>(map, p);
    else if (pass == 1) mc_idx_vertex_kernel<VT, TMA><<<(int)grid, ITHREADS, smem, s>>>(map, p);
    else mc_idx_triangle_kernel<VT, TMA><<<(int)grid, ITHREADS, smem, s>>>(map, p);
}

void launch_idx_pass(int pass, const mcg_volume *vol, const IdxParams &p, int sms, long long items, cudaStream_t s) {
    CUtensorMap map;
    const int eb = vol->voxel_type == MCG_VOXEL_SHORT2 ? 4 : 8;
    const bool tma = encode_volume_map(&map, vol->data, vol->nx, vol->ny, vol->nz, eb, IX, IY, IZ);
    if (!tma) memset(&map, 0, sizeof(map));
    if (vol->voxel_type == MCG_VOXEL_SHORT2) {
        if (tma) launch_idx<MCG_VOXEL_SHORT2, true>(pass, map, p, sms, items, s);
        else launch_idx<MCG_VOXEL_SHORT2, false>(pass, map, p, sms, items, s);
    } else {
        if (tma) launch_idx<MCG_VOXEL_FLOAT2, true>(pass, map, p, sms, items, s);
        else launch_idx<MCG_VOXEL_FLOAT2, false>(pass, map, p, sms, items, s);
    }
}

IdxParams idx_params(mcg_context *ctx, const mcg_volume *vol, const Geometry &g) {
    IdxParams p;
    memset(&p, 0, sizeof(p));
    p.vol = vol->data;
    p.nx = vol->nx;
    p.ny = vol->ny;
    p.nz = vol->nz;
    p.cell = vol->cell;
    p.nbx = g.nbx;
    p.nby = g.nby;
    p.nbz = g.nbz;
    p.nbricks = g.nbricks;
    p.brick_tris = ctx->brick_tris;
    p.brick_uniq = ctx->brick_uniq;
    p.chunk = ctx->brick_occ;
    p.active = ctx->active;
    p.brick_tofs = ctx->brick_vofs;
    p.brick_uofs = ctx->brick_uofs;
    p.totals = ctx->d_totals;
    p.edge_map = ctx->edge_map;
    return p;
}

long long idx_chunks(long long nbricks) { return (nbricks + CHUNK - 1) / CHUNK; }

}  // namespace
}  // namespace mcg

using namespace mcg;

mcg_status mcg_mc_classify_indexed(mcg_context *ctx, const mcg_volume *vol, mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol)) return MCG_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const Geometry g = geometry(vol->nx, vol->ny, vol->nz);
    const long long nch = idx_chunks(g.nbricks);
    if (!ensure(&ctx->brick_uniq, &ctx->brick_uniq_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->brick_uofs, &ctx->brick_uofs_cap, (size_t)g.nbricks) ||
        !ensure(&ctx->idx_cand, &ctx->idx_cand_cap, (size_t)g.nbricks))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    // the soup's count phase: brick triangle counts, occupied cubes; its scan
    // leaves the chunk sums zero for the sums below
    e = soup_count_phase(ctx, vol, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    // the counters the count phase used, and the candidate count
    e = cudaMemsetAsync(&ctx->d_totals->cls_ticket, 0, 3 * sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(&ctx->d_totals->idx_cand, 0, sizeof(unsigned int), s);
    ctx->chunk_clean_cap = 0;  // these sums stay behind: the next count phase clears the array first
    ctx->counters_clean = false;
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    IdxParams p = idx_params(ctx, vol, g);
    p.cand = ctx->idx_cand;
    mc_idx_cand_kernel<<<(unsigned int)((g.nbricks + 255) / 256), 256, 0, s>>>(p);
    launch_idx_pass(0, vol, p, ctx->num_sms, g.nbricks, s);
    mc_idx_scan_kernel<<<(unsigned int)nch, CHUNK, 0, s>>>(ctx->brick_tris, ctx->brick_uniq, ctx->brick_occ,
                                                          g.nbricks, ctx->brick_vofs, ctx->brick_uofs, ctx->active,
                                                          ctx->d_totals, 1);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = mcg_counts_event(ctx, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    ctx->classified = true;
    ctx->cls_indexed = true;
    ctx->cls_fused = false;  // the indexed scan wrote the totals
    ctx->batch_classified = false;
    ctx->cls_data = vol->data;
    ctx->cls_nx = vol->nx;
    ctx->cls_ny = vol->ny;
    ctx->cls_nz = vol->nz;
    ctx->cls_vtype = vol->voxel_type;
    ctx->cls_z0 = 0;
    ctx->cls_z1 = vol->nz - 1;
    ctx->last_capacity = -1;
    ctx->last_capacity_tris = -1;
    return MCG_OK;
}

mcg_status mcg_mc_generate_indexed(mcg_context *ctx, const mcg_volume *vol, const mcg_indexed_out *out,
                                   mcg_stream_t stream) {
    if (!ctx || !vol_ok(vol) || !out || out->capacity_vertices < 0 || out->capacity_triangles < 0)
        return MCG_ERR_INVALID_ARG;
    if (!ctx->classified || !ctx->cls_indexed || ctx->cls_data != vol->data || ctx->cls_nx != vol->nx ||
        ctx->cls_ny != vol->ny || ctx->cls_nz != vol->nz || ctx->cls_vtype != vol->voxel_type)
        return MCG_ERR_STATE;
    if (out->capacity_vertices > (int64_t)0xffffffffll) return MCG_ERR_INVALID_ARG;  // 32-bit vertex ids
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const Geometry g = geometry(vol->nx, vol->ny, vol->nz);
    const size_t nedges = 3 * (size_t)vol->nx * vol->ny * vol->nz;
    if (!ensure(&ctx->edge_map, &ctx->edge_map_cap, nedges)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    IdxParams p = idx_params(ctx, vol, g);
    p.out = *out;
    e = cudaMemsetAsync(&ctx->d_totals->gen_ticket, 0, 2 * sizeof(unsigned int), s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    launch_idx_pass(1, vol, p, ctx->num_sms, g.nbricks, s);
    launch_idx_pass(2, vol, p, ctx->num_sms, g.nbricks, s);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->h_totals, ctx->d_totals, sizeof(MeshTotals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = mcg_counts_event(ctx, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    ctx->last_capacity = out->capacity_vertices;
    ctx->last_capacity_tris = out->capacity_triangles;
    return MCG_OK;
}

mcg_status mcg_mc_extract_indexed(mcg_context *ctx, const mcg_volume *vol, const mcg_indexed_out *out,
                                  mcg_stream_t stream) {
    const mcg_status st = mcg_mc_classify_indexed(ctx, vol, stream);
    if (st != MCG_OK) return st;
    return mcg_mc_generate_indexed(ctx, vol, out, stream);
}
