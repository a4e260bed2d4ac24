// Mesh writers on sm_103a: the binary PLY soup and the de-duplicated OBJ of
// cu_voxel_rlc_to_mesh / cu_voxel_to_mesh (cu_kinect_fusion_v1.cu:3394-3424,
// 3625-3726), byte for byte.
//
// PLY: the header is printed on the host; the body (per vertex position and
// normal, per triangle uint8 3 + int32 3i, 3i+1, 3i+2) is assembled on the
// device and copied out once.
//
// OBJ: the reference keys a vertex by the text "%.4f_%.4f_%.4f" of its
// position in a std::map and writes a vertex the first time its key is
// seen.  Here the key is the same number in integer form: x * 10^4 is exact
// in binary64 for a binary32 x (24 + 10 significant bits), and rounding it
// to the nearest integer, ties to even, is the rounding printf applies, so
// two positions print the same key exactly when their three rounded
// integers agree (a negative value that rounds to zero keeps its own key,
// as "-0.0000" does; positions are packed 21 bits each: |x| < 104.8575, the
// reference's 25-byte key buffer overflows from 100 m on anyway).  Keys go
// into an open-addressing hash table (atomicCAS on the key, atomicMin of the
// first soup index); a scan of "first occurrence" flags numbers the vertices
// in the reference's order.  Triangles with two equal ids are dropped as
// the reference drops them.  Text: "%f" is x * 10^6 (exact in binary64)
// rounded ties-to-even, then integer digits; every record's length is
// computed, scanned, and the record written at its offset.  The qi_volume
// listing ("%d %hd %hd %d %d %d") comes out of the same pass.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "mcg_internal.h"

namespace mcg {
namespace {

constexpr int MW_THREADS = 256;
constexpr unsigned long long MW_EMPTY = ~0ull;
constexpr long long MW_KEY_LIM = 1 << 20;     // 21-bit key fields
constexpr long long MW_NEG0 = -(MW_KEY_LIM - 1);  // a negative value that prints as "-0.0000"

struct Vtx {
    float x, y, z;
    int32_t vx, vy, vz;
    int16_t tsdf, w;
};
static_assert(sizeof(Vtx) == 28, "vertex_voxel layout");

// ---- decimal text ------------------------------------------------------------
__device__ __forceinline__ int mw_udigits(unsigned long long v) {
    int d = 1;
    while (v >= 10ull) {
        v /= 10ull;
        ++d;
    }
    return d;
}

// "%d" of a 32-bit int
__device__ __forceinline__ int mw_int_len(long long v) { return (v < 0 ? 1 : 0) + mw_udigits((unsigned long long)(v < 0 ? -v : v)); }
__device__ __forceinline__ char *mw_put_uint(char *p, unsigned long long v, int digits) {
    for (int i = digits - 1; i >= 0; --i) {
        p[i] = (char)('0' + (int)(v % 10ull));
        v /= 10ull;
    }
    return p + digits;
}
__device__ __forceinline__ char *mw_put_int(char *p, long long v) {
    if (v < 0) *p++ = '-';
    const unsigned long long a = (unsigned long long)(v < 0 ? -v : v);
    return mw_put_uint(p, a, mw_udigits(a));
}

// "%f" of a float (6 decimals); non-finite values print as glibc does
struct Fixed {
    bool neg, nan, inf;
    unsigned long long ip, fp;  // integer part, 6 fraction digits
};
__device__ __forceinline__ Fixed mw_fixed(float x) {
    Fixed f;
    const double d = (double)x;
    f.neg = signbit(d);
    f.nan = isnan(d);
    f.inf = isinf(d);
    f.ip = f.fp = 0;
    if (!f.nan && !f.inf) {
        const unsigned long long N = (unsigned long long)rint(fabs(d) * 1e6);  // exact product, ties to even
        f.ip = N / 1000000ull;
        f.fp = N % 1000000ull;
    }
    return f;
}
__device__ __forceinline__ int mw_fixed_len(const Fixed &f) {
    if (f.nan || f.inf) return 3 + (f.neg ? 1 : 0);
    return (f.neg ? 1 : 0) + mw_udigits(f.ip) + 7;
}
__device__ __forceinline__ char *mw_put_fixed(char *p, const Fixed &f) {
    if (f.neg) *p++ = '-';
    if (f.nan || f.inf) {
        const char *s = f.nan ? "nan" : "inf";
        p[0] = s[0];
        p[1] = s[1];
        p[2] = s[2];
        return p + 3;
    }
    p = mw_put_uint(p, f.ip, mw_udigits(f.ip));
    *p++ = '.';
    return mw_put_uint(p, f.fp, 6);
}

// ---- keys ------------------------------------------------------------------------
// the "%.4f" text of x as an integer: x * 10^4 rounded ties-to-even, and
// MW_NEG0 for a negative x that rounds to zero (printed "-0.0000")
__device__ __forceinline__ long long mw_key4(float x) {
    const long long k = (long long)rint((double)x * 1e4);
    return (k == 0 && signbit(x)) ? MW_NEG0 : k;
}
__device__ __forceinline__ bool mw_key_ok(long long k) { return k > MW_NEG0 - 1 && k < MW_KEY_LIM; }

__device__ __forceinline__ unsigned long long mw_hash(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// insert every soup vertex's key; slot[i] = its table slot, first[slot] = min i
__global__ void __launch_bounds__(MW_THREADS) mw_insert(const Vtx *__restrict__ v, const float *__restrict__ nrm,
                                                        long long n,
                                                        unsigned long long *__restrict__ keys, int *__restrict__ first,
                                                        long long tmask, int *__restrict__ slot,
                                                        int *__restrict__ flags) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float *n3 = nrm + 3 * i;
        if (!(fabsf(v[i].x) < 105.0f && fabsf(v[i].y) < 105.0f && fabsf(v[i].z) < 105.0f) ||
            !(fabsf(n3[0]) < 1e9f && fabsf(n3[1]) < 1e9f && fabsf(n3[2]) < 1e9f)) {
            atomicOr(flags, 1);  // outside the key range, or not finite
            slot[i] = -1;
            continue;
        }
        const long long kx = mw_key4(v[i].x), ky = mw_key4(v[i].y), kz = mw_key4(v[i].z);
        if (!mw_key_ok(kx) || !mw_key_ok(ky) || !mw_key_ok(kz)) {
            atomicOr(flags, 1);
            slot[i] = -1;
            continue;
        }
        const unsigned long long key = ((unsigned long long)(kx + MW_KEY_LIM) << 42) |
                                       ((unsigned long long)(ky + MW_KEY_LIM) << 21) |
                                       (unsigned long long)(kz + MW_KEY_LIM);
        unsigned long long h = mw_hash(key) & (unsigned long long)tmask;
        // the table has at least twice the vertices: a free or equal slot is always found
        for (long long probe = 0; probe <= tmask; ++probe) {
            const unsigned long long prev = atomicCAS(&keys[h], MW_EMPTY, key);
            if (prev == MW_EMPTY || prev == key) break;
            h = (h + 1) & (unsigned long long)tmask;
        }
        atomicMin(&first[h], (int)i);
        slot[i] = (int)h;
    }
}

// exclusive block scan of one int per thread; *total the block's sum
__device__ __forceinline__ int mw_block_excl(int v, int *s_w, int *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    int pre = 0, all = 0;
#pragma unroll
    for (int i = 0; i < MW_THREADS / 32; ++i) {
        pre += i < wid ? s_w[i] : 0;
        all += s_w[i];
    }
    __syncthreads();
    *total = all;
    return pre + inc - v;
}

constexpr int MW_PER = 8;                       // items per thread in the scans
constexpr int MW_TILE = MW_THREADS * MW_PER;    // items per CTA

// flag of item i: first occurrence of its key (mode 0), a kept triangle (mode 1)
__device__ __forceinline__ int mw_flag(int mode, long long i, const int *slot, const int *first, const int *id) {
    if (mode == 0) {
        const int s = slot[i];
        return s >= 0 && first[s] == (int)i ? 1 : 0;
    }
    const int a = id[3 * i], b = id[3 * i + 1], c = id[3 * i + 2];
    return (a != b && a != c && b != c) ? 1 : 0;
}

__global__ void __launch_bounds__(MW_THREADS) mw_count(int mode, long long n, const int *__restrict__ slot,
                                                       const int *__restrict__ first, const int *__restrict__ id,
                                                       long long *__restrict__ tile_sum) {
    __shared__ int s_w[MW_THREADS / 32];
    const long long b = (long long)blockIdx.x * MW_TILE + (long long)threadIdx.x * MW_PER;
    int c = 0;
    for (int k = 0; k < MW_PER; ++k)
        if (b + k < n) c += mw_flag(mode, b + k, slot, first, id);
    int total;
    mw_block_excl(c, s_w, &total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// one CTA: exclusive scan of the tile sums, total in *total
__global__ void __launch_bounds__(1024) mw_tiles(long long *__restrict__ tile_sum, long long ntiles,
                                                 long long *__restrict__ total) {
    if (threadIdx.x != 0) return;
    long long run = 0;
    for (long long t = 0; t < ntiles; ++t) {
        const long long v = tile_sum[t];
        tile_sum[t] = run;
        run += v;
    }
    *total = run;
}

// rank of every flagged item: mode 0 -> uid of first occurrences and the
// inverse map order[uid] = i; mode 1 -> kept triangle index, tri_of[k] = t
__global__ void __launch_bounds__(MW_THREADS) mw_rank(int mode, long long n, const int *__restrict__ slot,
                                                      const int *__restrict__ first, const int *__restrict__ id,
                                                      const long long *__restrict__ tile_ofs, int *__restrict__ rank,
                                                      int *__restrict__ order) {
    __shared__ int s_w[MW_THREADS / 32];
    const long long b = (long long)blockIdx.x * MW_TILE + (long long)threadIdx.x * MW_PER;
    int f[MW_PER], c = 0;
    for (int k = 0; k < MW_PER; ++k) {
        f[k] = b + k < n ? mw_flag(mode, b + k, slot, first, id) : 0;
        c += f[k];
    }
    int total;
    long long r = tile_ofs[blockIdx.x] + mw_block_excl(c, s_w, &total);
    for (int k = 0; k < MW_PER; ++k) {
        if (b + k >= n) break;
        if (f[k]) {
            if (rank) rank[b + k] = (int)r;
            order[r] = (int)(b + k);
            ++r;
        }
    }
}

// 1-based OBJ id of every soup vertex: the uid of its key's first occurrence + 1
__global__ void mw_ids(long long n, const int *__restrict__ slot, const int *__restrict__ first,
                       const int *__restrict__ uid, int *__restrict__ id) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        id[i] = uid[first[slot[i]]] + 1;
}

// record lengths: kind 0 vertex ("v ..\nvn ..\n"), 1 face, 2 qi line
__device__ int mw_vertex_len(const Vtx &v, const float *nrm) {
    return 2 + mw_fixed_len(mw_fixed(v.x)) + 1 + mw_fixed_len(mw_fixed(v.y)) + 1 + mw_fixed_len(mw_fixed(v.z)) + 1 +
           3 + mw_fixed_len(mw_fixed(nrm[0])) + 1 + mw_fixed_len(mw_fixed(nrm[1])) + 1 +
           mw_fixed_len(mw_fixed(nrm[2])) + 1;
}
__device__ int mw_face_len(int a, int b, int c) { return 2 + mw_int_len(a) + 1 + mw_int_len(b) + 1 + mw_int_len(c) + 1; }
__device__ int mw_qi_len(int count, const Vtx &v) {
    return mw_int_len(count) + 1 + mw_int_len(v.tsdf) + 1 + mw_int_len(v.w) + 1 + mw_int_len(v.vx) + 1 +
           mw_int_len(v.vy) + 1 + mw_int_len(v.vz) + 1;
}

__global__ void __launch_bounds__(MW_THREADS) mw_lengths(int kind, long long m, const Vtx *__restrict__ v,
                                                         const float *__restrict__ nrm, const int *__restrict__ order,
                                                         const int *__restrict__ id, long long *__restrict__ len) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (long long)gridDim.x * blockDim.x) {
        const int i = order[r];
        if (kind == 0)
            len[r] = mw_vertex_len(v[i], nrm + 3ll * i);
        else if (kind == 1)
            len[r] = mw_face_len(id[3ll * i], id[3ll * i + 1], id[3ll * i + 2]);
        else
            len[r] = mw_qi_len((int)r + 1, v[i]);
    }
}

__global__ void __launch_bounds__(MW_THREADS) mw_write(int kind, long long m, const Vtx *__restrict__ v,
                                                       const float *__restrict__ nrm, const int *__restrict__ order,
                                                       const int *__restrict__ id, const long long *__restrict__ ofs,
                                                       long long base, char *__restrict__ out) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (long long)gridDim.x * blockDim.x) {
        const int i = order[r];
        char *p = out + base + ofs[r];
        if (kind == 0) {
            const float *n3 = nrm + 3ll * i;
            *p++ = 'v';
            *p++ = ' ';
            p = mw_put_fixed(p, mw_fixed(v[i].x));
            *p++ = ' ';
            p = mw_put_fixed(p, mw_fixed(v[i].y));
            *p++ = ' ';
            p = mw_put_fixed(p, mw_fixed(v[i].z));
            *p++ = '\n';
            *p++ = 'v';
            *p++ = 'n';
            *p++ = ' ';
            p = mw_put_fixed(p, mw_fixed(n3[0]));
            *p++ = ' ';
            p = mw_put_fixed(p, mw_fixed(n3[1]));
            *p++ = ' ';
            p = mw_put_fixed(p, mw_fixed(n3[2]));
            *p++ = '\n';
        } else if (kind == 1) {
            *p++ = 'f';
            *p++ = ' ';
            p = mw_put_int(p, id[3ll * i]);
            *p++ = ' ';
            p = mw_put_int(p, id[3ll * i + 1]);
            *p++ = ' ';
            p = mw_put_int(p, id[3ll * i + 2]);
            *p++ = '\n';
        } else {
            p = mw_put_int(p, (long long)r + 1);
            *p++ = ' ';
            p = mw_put_int(p, v[i].tsdf);
            *p++ = ' ';
            p = mw_put_int(p, v[i].w);
            *p++ = ' ';
            p = mw_put_int(p, v[i].vx);
            *p++ = ' ';
            p = mw_put_int(p, v[i].vy);
            *p++ = ' ';
            p = mw_put_int(p, v[i].vz);
            *p++ = '\n';
        }
    }
}

// PLY body: n x (position, normal), then n/3 x (uint8 3, int32 3t, 3t+1, 3t+2)
__global__ void __launch_bounds__(MW_THREADS) mw_ply_body(const Vtx *__restrict__ v, const float *__restrict__ nrm,
                                                          long long n, unsigned char *__restrict__ out) {
    const long long nf = n / 3;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n + nf;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n) {
            float *q = reinterpret_cast<float *>(out + 24ll * i);
            q[0] = v[i].x;
            q[1] = v[i].y;
            q[2] = v[i].z;
            q[3] = nrm[3 * i];
            q[4] = nrm[3 * i + 1];
            q[5] = nrm[3 * i + 2];
        } else {
            const long long t = i - n;
            unsigned char *q = out + 24ll * n + 13ll * t;
            q[0] = 3;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const unsigned idx = (unsigned)(3 * t + k);
#pragma unroll
                for (int b = 0; b < 4; ++b) q[1 + 4 * k + b] = (unsigned char)(idx >> (8 * b));
            }
        }
    }
}

// exclusive scan of m lengths (one CTA of 1024, serial per thread slice)
__global__ void __launch_bounds__(1024) mw_scan_len(long long *__restrict__ len, long long m,
                                                    long long *__restrict__ total) {
    __shared__ long long s_w[32];
    const long long per = (m + 1023) / 1024;
    const long long b = per * threadIdx.x, e = min(m, b + per);
    long long sum = 0;
    for (long long i = b; i < e; ++i) sum += len[i];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    long long pre = 0, all = 0;
    for (int i = 0; i < 32; ++i) {
        pre += i < wid ? s_w[i] : 0;
        all += s_w[i];
    }
    long long run = pre + inc - sum;
    for (long long i = b; i < e; ++i) {
        const long long l = len[i];
        len[i] = run;
        run += l;
    }
    if (threadIdx.x == 0) *total = all;
}

std::string ply_header(long long n) {
    char buf[512];
    snprintf(buf, sizeof(buf),
             "ply\nformat binary_little_endian 1.0\nelement vertex %d\nproperty float32 x\nproperty float32 y\n"
             "property float32 z\nproperty float32 nx\nproperty float32 ny\nproperty float32 nz\n"
             "element face %d\nproperty list uint8 int32 vertex_indices\nend_header\n",
             (int)n, (int)(n / 3));
    return buf;
}

const char kQiHeader[] = "qi tsdf w vx vy vz\n";

int grid_for(mcg_context *ctx, long long n) {
    const long long g = (n + MW_THREADS - 1) / MW_THREADS;
    return (int)std::max<long long>(1, std::min<long long>(g, (long long)ctx->num_sms * 16));
}

// Device OBJ and qi text in ctx->mw_text (obj at 0, qi after it); sizes out.
mcg_status obj_build(mcg_context *ctx, const Vtx *v, const float *nrm, long long n, long long *obj_size,
                     long long *qi_size, cudaStream_t s) {
    long long tsize = 1;
    while (tsize < 2 * n + 2) tsize <<= 1;
    const long long nt = n / 3;
    const long long ntiles = std::max<long long>((n + MW_TILE - 1) / MW_TILE, 1);
    // scratch: keys (8 B) + first (4) per table slot; slot, uid, id, order (4 each) per vertex;
    // tri ranks (4) per triangle; lengths (8) per record; tile sums; flags + totals
    if (!ensure(&ctx->mw_keys, &ctx->mw_keys_cap, (size_t)tsize) ||
        !ensure(&ctx->mw_int, &ctx->mw_int_cap, (size_t)(tsize + 4 * n + nt + 16)) ||
        !ensure(&ctx->mw_len, &ctx->mw_len_cap, (size_t)(2 * n + nt + ntiles + 16)))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    int *first = ctx->mw_int, *slot = first + tsize, *uid = slot + n, *id = uid + n, *order = id + n,
        *tord = order + n, *flags = tord + nt;
    long long *tile = ctx->mw_len, *tot = tile + ntiles, *len = tot + 8;  // tot[0..7]
    cudaError_t e;
    if ((e = cudaMemsetAsync(ctx->mw_keys, 0xff, (size_t)tsize * 8, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(first, 0x7f, (size_t)tsize * 4, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(flags, 0, 4, s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    const int g = grid_for(ctx, n);
    if (n > 0) mw_insert<<<g, MW_THREADS, 0, s>>>(v, nrm, n, ctx->mw_keys, first, tsize - 1, slot, flags);
    int h_flags = 0;
    if ((e = cudaMemcpyAsync(&h_flags, flags, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    if (h_flags) return MCG_ERR_TOO_LARGE;
    // vertex order: first occurrences
    mw_count<<<(unsigned)ntiles, MW_THREADS, 0, s>>>(0, n, slot, first, id, tile);
    mw_tiles<<<1, 1024, 0, s>>>(tile, ntiles, tot + 0);
    mw_rank<<<(unsigned)ntiles, MW_THREADS, 0, s>>>(0, n, slot, first, id, tile, uid, order);
    if (n > 0) mw_ids<<<g, MW_THREADS, 0, s>>>(n, slot, first, uid, id);
    // kept triangles
    const long long ttiles = std::max<long long>((nt + MW_TILE - 1) / MW_TILE, 1);
    mw_count<<<(unsigned)ttiles, MW_THREADS, 0, s>>>(1, nt, slot, first, id, tile);
    mw_tiles<<<1, 1024, 0, s>>>(tile, ttiles, tot + 1);
    mw_rank<<<(unsigned)ttiles, MW_THREADS, 0, s>>>(1, nt, slot, first, id, tile, nullptr, tord);
    long long counts[2];
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(counts, tot, 16, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    const long long nu = counts[0], nk = counts[1];
    // record lengths: vertices, faces, qi lines
    long long *lv = len, *lf = lv + nu, *lq = lf + nk;
    const int gu = grid_for(ctx, nu), gk = grid_for(ctx, nk);
    if (nu > 0) mw_lengths<<<gu, MW_THREADS, 0, s>>>(0, nu, v, nrm, order, id, lv);
    if (nk > 0) mw_lengths<<<gk, MW_THREADS, 0, s>>>(1, nk, v, nrm, tord, id, lf);
    if (nu > 0) mw_lengths<<<gu, MW_THREADS, 0, s>>>(2, nu, v, nrm, order, id, lq);
    mw_scan_len<<<1, 1024, 0, s>>>(lv, nu, tot + 2);
    mw_scan_len<<<1, 1024, 0, s>>>(lf, nk, tot + 3);
    mw_scan_len<<<1, 1024, 0, s>>>(lq, nu, tot + 4);
    long long sz[3];
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(sz, tot + 2, 24, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    const long long hq = (long long)sizeof(kQiHeader) - 1;
    *obj_size = sz[0] + sz[1];
    *qi_size = hq + sz[2];
    if (!ensure(&ctx->mw_text, &ctx->mw_text_cap, (size_t)(*obj_size + *qi_size + 16)))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    char *text = reinterpret_cast<char *>(ctx->mw_text);
    if (nu > 0) mw_write<<<gu, MW_THREADS, 0, s>>>(0, nu, v, nrm, order, id, lv, 0, text);
    if (nk > 0) mw_write<<<gk, MW_THREADS, 0, s>>>(1, nk, v, nrm, tord, id, lf, sz[0], text);
    if ((e = cudaMemcpyAsync(text + *obj_size, kQiHeader, (size_t)hq, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    if (nu > 0) mw_write<<<gu, MW_THREADS, 0, s>>>(2, nu, v, nrm, order, id, lq, *obj_size + hq, text);
    if ((e = cudaGetLastError()) != cudaSuccess) return mcg_cuda_fail(ctx, e);
    return MCG_OK;
}

mcg_status ply_build(mcg_context *ctx, const Vtx *v, const float *nrm, long long n, cudaStream_t s) {
    const long long body = 24 * n + 13 * (n / 3);
    if (!ensure(&ctx->mw_text, &ctx->mw_text_cap, (size_t)body + 16)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    if (n > 0) mw_ply_body<<<grid_for(ctx, n + n / 3), MW_THREADS, 0, s>>>(v, nrm, n, ctx->mw_text);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
}

bool write_all(FILE *f, const void *p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" mcg_status mcg_mesh_ply(mcg_context *ctx, const mcg_vertex_voxel *soup, const float *normals,
                                   int64_t n_vertices, uint8_t *image, int64_t capacity, int64_t *size,
                                   mcg_stream_t stream) {
    if (!ctx || !size || n_vertices < 0 || n_vertices > INT32_MAX || (n_vertices > 0 && (!soup || !normals)))
        return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const std::string head = ply_header(n_vertices);
    const long long body = 24 * n_vertices + 13 * (n_vertices / 3);
    *size = (int64_t)head.size() + body;
    if (!image && capacity == 0) return MCG_OK;
    if (!image || capacity < *size) return MCG_ERR_CAPACITY;
    const cudaStream_t s = (cudaStream_t)stream;
    mcg_status st = ply_build(ctx, reinterpret_cast<const Vtx *>(soup), normals, n_vertices, s);
    if (st != MCG_OK) return st;
    memcpy(image, head.data(), head.size());
    if ((e = cudaMemcpyAsync(image + head.size(), ctx->mw_text, (size_t)body, cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    return MCG_OK;
}

extern "C" mcg_status mcg_mesh_obj(mcg_context *ctx, const mcg_vertex_voxel *soup, const float *normals,
                                   int64_t n_vertices, uint8_t *obj, int64_t obj_capacity, int64_t *obj_size,
                                   uint8_t *qi, int64_t qi_capacity, int64_t *qi_size, mcg_stream_t stream) {
    if (!ctx || !obj_size || !qi_size || n_vertices < 0 || n_vertices > INT32_MAX / 2 ||
        (n_vertices > 0 && (!soup || !normals)))
        return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const cudaStream_t s = (cudaStream_t)stream;
    long long os = 0, qs = 0;
    mcg_status st = obj_build(ctx, reinterpret_cast<const Vtx *>(soup), normals, n_vertices, &os, &qs, s);
    if (st != MCG_OK) return st;
    *obj_size = os;
    *qi_size = qs;
    if (!obj && obj_capacity == 0 && !qi && qi_capacity == 0) return MCG_OK;  // size query
    if (obj_capacity < os || qi_capacity < (qi ? qs : 0) || (!obj && os > 0)) return MCG_ERR_CAPACITY;
    if ((os > 0 && (e = cudaMemcpyAsync(obj, ctx->mw_text, (size_t)os, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (qi && (e = cudaMemcpyAsync(qi, ctx->mw_text + os, (size_t)qs, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    return MCG_OK;
}

extern "C" mcg_status mcg_mesh_write(mcg_context *ctx, const mcg_vertex_voxel *soup, const float *normals,
                                     int64_t n_vertices, const char *path, const char *qi_path, mcg_stream_t stream) {
    if (!ctx || !path) return MCG_ERR_INVALID_ARG;
    const char *ext = strrchr(path, '.');
    const bool ply = ext && strcmp(ext, ".ply") == 0, obj = ext && strcmp(ext, ".obj") == 0;
    if (!ply && !obj) return MCG_ERR_INVALID_ARG;  // the reference prints "Invalid file extension"
    std::vector<uint8_t> a, b;
    int64_t sa = 0, sb = 0;
    mcg_status st;
    if (ply) {
        if ((st = mcg_mesh_ply(ctx, soup, normals, n_vertices, nullptr, 0, &sa, stream)) != MCG_OK) return st;
        a.resize((size_t)sa);
        if ((st = mcg_mesh_ply(ctx, soup, normals, n_vertices, a.data(), sa, &sa, stream)) != MCG_OK) return st;
    } else {
        // the text is built once on the device; the sizes come back with it
        if (n_vertices < 0 || n_vertices > INT32_MAX / 2 || (n_vertices > 0 && (!soup || !normals)))
            return MCG_ERR_INVALID_ARG;
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
        const cudaStream_t s = (cudaStream_t)stream;
        long long os = 0, qs = 0;
        if ((st = obj_build(ctx, reinterpret_cast<const Vtx *>(soup), normals, n_vertices, &os, &qs, s)) != MCG_OK)
            return st;
        a.resize((size_t)os);
        b.resize((size_t)qs);
        if ((os > 0 && (e = cudaMemcpyAsync(a.data(), ctx->mw_text, (size_t)os, cudaMemcpyDeviceToHost, s)) !=
                           cudaSuccess) ||
            (e = cudaMemcpyAsync(b.data(), ctx->mw_text + os, (size_t)qs, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return mcg_cuda_fail(ctx, e);
        sa = os;
        sb = qs;
    }
    FILE *f = fopen(path, ply ? "wb" : "w");
    if (!f) return MCG_ERR_IO;
    bool ok = write_all(f, a.data(), (size_t)sa);
    ok = (fclose(f) == 0) && ok;
    if (ok && obj && qi_path) {
        FILE *q = fopen(qi_path, "wt");
        if (!q) return MCG_ERR_IO;
        ok = write_all(q, b.data(), (size_t)sb);
        ok = (fclose(q) == 0) && ok;
    }
    return ok ? MCG_OK : MCG_ERR_IO;
}
