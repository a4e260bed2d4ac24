// Run-length volume decoder on sm_103a (cu_kinect_fusion_v1.cu:1419-1447 per
// slice, :1533-1600 per file).
//
// Only the compressed image crosses the host link: it is copied to the
// device in slabs of whole slices on a copy stream while earlier slabs
// expand (from a file: pieces read by host threads into pinned buffers while
// the GPU copies and expands the pieces before).  One CTA expands one
// z-slice, 4096 16-bit words at a time:
//  * every word is a record header, or the first or second word of a
//    literal; which one follows from the words before it through a
//    three-state machine (header -> header, or -> literal 1 for kinds 0 and
//    3; literal 1 -> literal 2 -> header).  Each thread composes the state
//    maps of its 16 words and a block scan of the compositions (carrying the
//    state from the chunk before) gives every word its state;
//  * a block scan of the run lengths of the headers places each run in the
//    slice; runs go to shared memory as (start, voxel);
//  * the chunk's voxels are written by all threads, coalesced, each voxel
//    finding its run by binary search over the run starts.
// The slice is full once its voxels are placed; records after that are
// ignored.  A record that is needed and has length 0, runs past the slice
// or lacks its literal, or a stream that ends early, is an error
// (MCG_ERR_FORMAT), exactly the checks of the host decoder.
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <stdint.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "mcg_internal.h"

namespace mcg {
namespace {

constexpr int RD_THREADS = 256;
constexpr int RD_WPT = 16;                     // words per thread
constexpr int RD_CHUNK = RD_THREADS * RD_WPT;  // words per chunk
constexpr unsigned RD_ID = 0u | (1u << 2) | (2u << 4);  // identity state map

// state maps: 2 bits per entry state (0 header, 1 literal word 1, 2 literal word 2)
__device__ __forceinline__ unsigned rd_apply(unsigned f, unsigned s) { return (f >> (2 * s)) & 3u; }
__device__ __forceinline__ unsigned rd_then(unsigned a, unsigned b) {  // a, then b
    return rd_apply(b, rd_apply(a, 0)) | (rd_apply(b, rd_apply(a, 1)) << 2) | (rd_apply(b, rd_apply(a, 2)) << 4);
}
__device__ __forceinline__ unsigned rd_word_map(unsigned w) {
    const unsigned kind = w >> 14;
    return ((kind == 0u || kind == 3u) ? 1u : 0u) | (2u << 2);  // header -> literal 1 / header; 1 -> 2; 2 -> 0
}

// exclusive block scan of a value under an associative op; returns the
// exclusive prefix, *total the block total
template <class T, class Op>
__device__ __forceinline__ T rd_block_scan(T v, T id, Op op, T *s_w, T *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc = op(u, inc);
    }
    T ex = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) ex = id;
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    T pre = id, all = id;
#pragma unroll
    for (int i = 0; i < RD_THREADS / 32; ++i) {
        if (i < wid) pre = op(pre, s_w[i]);
        all = op(all, s_w[i]);
    }
    __syncthreads();
    *total = all;
    return op(pre, ex);
}

__device__ __forceinline__ uint32_t rd_pack(unsigned tsdf16, unsigned w16) { return (tsdf16 & 0xffffu) | (w16 << 16); }

// ---- chunk-parallel expansion ---------------------------------------------
// A chunk is RD_CHUNK words of one slice.  Its summary holds, for each state
// the chunk may be entered in, the state it leaves in (the map f) and the
// voxels its headers emit; summaries compose associatively, so a scan along
// the slice gives every chunk its entry state and first voxel.

struct Sum {
    unsigned f;
    long long v[3];
};

__device__ __forceinline__ long long sum_pick(const Sum &x, unsigned e) {  // x.v[e] without local memory
    return e == 0u ? x.v[0] : (e == 1u ? x.v[1] : x.v[2]);
}

__device__ __forceinline__ Sum sum_then(const Sum &a, const Sum &b) {
    Sum r;
    r.f = rd_then(a.f, b.f);
#pragma unroll
    for (int e = 0; e < 3; ++e) r.v[e] = a.v[e] + sum_pick(b, rd_apply(a.f, (unsigned)e));
    return r;
}

__device__ __forceinline__ Sum sum_shfl_up(const Sum &x, int o) {
    Sum r;
    r.f = __shfl_up_sync(0xffffffffu, x.f, o);
#pragma unroll
    for (int e = 0; e < 3; ++e) r.v[e] = __shfl_up_sync(0xffffffffu, x.v[e], o);
    return r;
}

// exclusive block scan of summaries; *total the block's composition
__device__ __forceinline__ Sum sum_block_scan(const Sum &x, Sum *s_w, Sum *total) {
    const Sum id{RD_ID, {0, 0, 0}};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Sum inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Sum u = sum_shfl_up(inc, o);
        if (lane >= o) inc = sum_then(u, inc);
    }
    Sum ex = sum_shfl_up(inc, 1);
    if (lane == 0) ex = id;
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    Sum pre = id, all = id;
#pragma unroll
    for (int i = 0; i < RD_THREADS / 32; ++i) {
        if (i < wid) pre = sum_then(pre, s_w[i]);
        all = sum_then(all, s_w[i]);
    }
    __syncthreads();
    *total = all;
    return sum_then(pre, ex);
}

struct Dir {
    const long long *off, *len;  // byte range of each slice's records in the image
    const long long *cbase;      // first chunk of each slice (nz + 1 entries)
    int nz;
};

// slice of chunk c, and its words [c0, c0 + cw) of nw
__device__ __forceinline__ void rd_chunk(const Dir &d, long long c, int *z, long long *c0, int *cw, long long *nw) {
    int lo = 0, hi = d.nz - 1;  // last slice with cbase <= c
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d.cbase[mid] <= c)
            lo = mid;
        else
            hi = mid - 1;
    }
    *z = lo;
    *nw = d.len[lo] / 2;
    *c0 = (c - d.cbase[lo]) * RD_CHUNK;
    *cw = (int)min((long long)RD_CHUNK, *nw - *c0);
}

// the chunk's words (+2 past its end for a literal that straddles it) into W,
// zeros after them.  The chunk starts at any byte: 16-byte pieces are read
// from the aligned address below it and shifted into place; only pieces
// holding kept words are read, which stay within 32 bytes past the slice's
// bytes (the image buffer has 64 bytes of slack after the image).
__device__ __forceinline__ void rd_load(const uint8_t *__restrict__ img, const Dir &d, int z, long long c0, int cw,
                                        long long nw, uint16_t *W) {
    const uint8_t *first = img + d.off[z] + 2 * c0;
    const uint4 *p = reinterpret_cast<const uint4 *>((uintptr_t)first & ~(uintptr_t)15);
    const unsigned sh = (unsigned)((uintptr_t)first & 15);
    const unsigned q = sh >> 2, r = 8u * (sh & 3u);
    const long long lim = min((long long)cw + 2, nw - c0);  // words to keep
    constexpr int PIECES = (RD_CHUNK + 8) / 8;                // 8 words per piece
    const long long loaded = (lim + 7) / 8;                   // pieces holding kept words
    for (int j = threadIdx.x; j < PIECES; j += RD_THREADS) {
        if (j >= loaded) {  // nothing to keep: no read past the slice's bytes
            reinterpret_cast<uint4 *>(W)[j] = make_uint4(0, 0, 0, 0);
            continue;
        }
        const uint4 lo = __ldg(p + j), hi = __ldg(p + j + 1);
        const unsigned x[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        unsigned o[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // words k+q and k+q+1 of x without a dynamic register index
            const unsigned a = q == 0 ? x[k] : q == 1 ? x[k + 1] : q == 2 ? x[k + 2] : x[k + 3];
            const unsigned b = q == 0 ? x[k + 1] : q == 1 ? x[k + 2] : q == 2 ? x[k + 3] : x[k + 4];
            o[k] = __funnelshift_r(a, b, r);
        }
        const long long w0 = 8ll * j;  // first word of the piece
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (w0 + 2 * k >= lim) o[k] = 0;
            else if (w0 + 2 * k + 1 >= lim) o[k] &= 0xffffu;
        }
        reinterpret_cast<uint4 *>(W)[j] = make_uint4(o[0], o[1], o[2], o[3]);
    }
    __syncthreads();
}

// this thread's 16 words and the 2 after them, from shared memory into
// registers with two 16-byte loads (conflict-free) and one 4-byte load
__device__ __forceinline__ void rd_words(const uint16_t *W, int b, unsigned w[RD_WPT + 2]) {
    const uint4 *p = reinterpret_cast<const uint4 *>(W + b);
    const uint4 a = p[0], c = p[1];
    const unsigned x[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        w[2 * k] = x[k] & 0xffffu;
        w[2 * k + 1] = x[k] >> 16;
    }
    const unsigned t = *reinterpret_cast<const unsigned *>(W + b + RD_WPT);
    w[RD_WPT] = t & 0xffffu;
    w[RD_WPT + 1] = t >> 16;
}

// pass 1: summaries of chunks c0 + blockIdx.x
__global__ void __launch_bounds__(RD_THREADS) rle_summarize(const uint8_t *__restrict__ img, Dir d, long long cfirst,
                                                            Sum *__restrict__ sums) {
    __shared__ __align__(16) uint16_t W[RD_CHUNK + 8];
    __shared__ Sum s_w[RD_THREADS / 32];
    const long long c = cfirst + blockIdx.x;
    int z, cw;
    long long c0, nw;
    rd_chunk(d, c, &z, &c0, &cw, &nw);
    rd_load(img, d, z, c0, cw, nw, W);
    const int b = threadIdx.x * RD_WPT, nk = max(0, min(cw, b + RD_WPT) - b);
    unsigned w[RD_WPT + 2];
    rd_words(W, b, w);
    Sum t;
    t.f = 0;
#pragma unroll
    for (unsigned en = 0; en < 3; ++en) {
        unsigned s = en;
        long long v = 0;
#pragma unroll
        for (int k = 0; k < RD_WPT; ++k) {
            if (k < nk) {
                if (s == 0u) v += w[k] & 0x3fff;
                s = rd_apply(rd_word_map(w[k]), s);
            }
        }
        t.v[en] = v;
        t.f |= s << (2 * en);
    }
    Sum total;
    sum_block_scan(t, s_w, &total);
    if (threadIdx.x == 0) sums[c] = total;
}

// pass 2: one CTA per slice z0 + blockIdx.x: entry state and first voxel of
// each of its chunks; a slice whose records end before it is full is an error
__global__ void __launch_bounds__(RD_THREADS) rle_slice_scan(Dir d, int z0, long long xy,
                                                             const Sum *__restrict__ sums,
                                                             unsigned char *__restrict__ entry,
                                                             long long *__restrict__ first, int *__restrict__ err) {
    __shared__ Sum s_w[RD_THREADS / 32];
    const int z = z0 + blockIdx.x;
    const long long cb = d.cbase[z], ce = d.cbase[z + 1];
    unsigned state = 0;
    long long out = 0;
    for (long long k = cb; k < ce; k += RD_THREADS) {
        const long long c = k + threadIdx.x;
        const Sum x = c < ce ? sums[c] : Sum{RD_ID, {0, 0, 0}};
        Sum total;
        const Sum pre = sum_block_scan(x, s_w, &total);
        if (c < ce) {
            entry[c] = (unsigned char)rd_apply(pre.f, state);
            first[c] = out + sum_pick(pre, state);
        }
        out += sum_pick(total, state);
        state = rd_apply(total.f, state);
    }
    if (threadIdx.x == 0 && out < xy) atomicOr(err, 1);
}

// pass 3: expand chunks cfirst + blockIdx.x
__global__ void __launch_bounds__(RD_THREADS) rle_expand(const uint8_t *__restrict__ img, Dir d, long long cfirst,
                                                         long long xy, const unsigned char *__restrict__ entry_of,
                                                         const long long *__restrict__ first_of,
                                                         uint32_t *__restrict__ vol, int *__restrict__ err) {
    __shared__ __align__(16) uint16_t W[RD_CHUNK + 8];
    __shared__ int rs[RD_CHUNK];
    __shared__ uint32_t rv[RD_CHUNK];
    __shared__ unsigned s_f[RD_THREADS / 32];
    __shared__ int s_i[RD_THREADS / 32];
    const long long c = cfirst + blockIdx.x;
    const long long out = first_of[c], n = xy;
    if (out >= n) return;  // records after a full slice are ignored
    int z, cw;
    long long c0, nw;
    rd_chunk(d, c, &z, &c0, &cw, &nw);
    rd_load(img, d, z, c0, cw, nw, W);
    const unsigned state = entry_of[c];
    uint32_t *out_slice = vol + (long long)z * xy;
    bool bad = false;
    const int b = threadIdx.x * RD_WPT, nk = max(0, min(cw, b + RD_WPT) - b);
    unsigned w[RD_WPT + 2];
    rd_words(W, b, w);
    unsigned f = RD_ID;
#pragma unroll
    for (int k = 0; k < RD_WPT; ++k)
        if (k < nk) f = rd_then(f, rd_word_map(w[k]));
    unsigned fall;
    const unsigned fpre = rd_block_scan<unsigned>(f, RD_ID, [](unsigned a, unsigned c2) { return rd_then(a, c2); },
                                                  s_f, &fall);
    const unsigned entry = rd_apply(fpre, state);
    int nrec = 0;
    long long nvox = 0;
    unsigned s = entry;
#pragma unroll
    for (int k = 0; k < RD_WPT; ++k) {
        if (k < nk) {
            if (s == 0u) {
                ++nrec;
                nvox += w[k] & 0x3fff;
            }
            s = rd_apply(rd_word_map(w[k]), s);
        }
    }
    int rtot;
    long long vtot;
    const int r0 = rd_block_scan<int>(nrec, 0, [](int a, int c2) { return a + c2; }, s_i, &rtot);
    __shared__ long long s_l[RD_THREADS / 32];
    const long long v0 = rd_block_scan<long long>(nvox, 0, [](long long a, long long c2) { return a + c2; }, s_l, &vtot);
    s = entry;
    int r = r0;
    long long o = v0;
#pragma unroll
    for (int k = 0; k < RD_WPT; ++k) {
        if (k < nk) {
            const unsigned wk = w[k];
            if (s == 0u) {
                const unsigned cnt = wk & 0x3fff, kind = wk >> 14;
                uint32_t val;
                bool lit_ok = true;
                if (kind == 1u) {
                    val = rd_pack((unsigned)kMaxTsdf, 0u);
                } else if (kind == 2u) {
                    val = rd_pack((unsigned)(-kMaxTsdf), 0u);
                } else {
                    lit_ok = c0 + b + k + 2 < nw;
                    val = rd_pack(w[k + 1], w[k + 2]);
                }
                const long long start = out + o;
                if (start < n && (cnt == 0u || start + (long long)cnt > n || !lit_ok)) bad = true;
                rs[r] = (int)min(o, (long long)INT32_MAX);
                rv[r] = val;
                ++r;
                o += cnt;
            }
            s = rd_apply(rd_word_map(wk), s);
        }
    }
    __syncthreads();
    const long long end = min(n, out + vtot);
    for (long long q = out + threadIdx.x; q < end; q += RD_THREADS) {
        const int rel = (int)(q - out);
        int lo = 0, hi = rtot - 1;  // last run with start <= rel
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (rs[mid] <= rel)
                lo = mid;
            else
                hi = mid - 1;
        }
        out_slice[q] = rv[lo];
    }
    if (bad) atomicOr(err, 1);
}

struct Slab {
    int z0, z1;      // slices
    int64_t b0, b1;  // image bytes that hold them (b0 = end of the previous slab)
};

// The three passes over slices [z0, z1), once the stream s has their bytes
// and their directory entries (offsets, lengths, chunk bases).
cudaError_t launch_expand(mcg_context *ctx, const Slab &sl, const long long *cbase_host, int64_t xy, void *vol,
                          cudaStream_t s) {
    if (sl.z1 <= sl.z0) return cudaSuccess;
    const int nz = ctx->rd_dir_n;
    const Dir d{ctx->rd_dir, ctx->rd_dir + nz, ctx->rd_dir + 2 * nz, nz};
    const long long cf = cbase_host[sl.z0], nc = cbase_host[sl.z1] - cf;
    Sum *sums = reinterpret_cast<Sum *>(ctx->rd_sum);
    unsigned char *entry = ctx->rd_entry;
    if (nc > 0) rle_summarize<<<(unsigned)nc, RD_THREADS, 0, s>>>(ctx->rle_image, d, cf, sums);
    rle_slice_scan<<<sl.z1 - sl.z0, RD_THREADS, 0, s>>>(d, sl.z0, xy, sums, entry, ctx->rd_first, ctx->rd_err);
    if (nc > 0)
        rle_expand<<<(unsigned)nc, RD_THREADS, 0, s>>>(ctx->rle_image, d, cf, xy, entry, ctx->rd_first,
                                                      static_cast<uint32_t *>(vol), ctx->rd_err);
    return cudaGetLastError();
}

constexpr int64_t RD_SLAB = (int64_t)64 << 20;  // image bytes per copy

// device buffers for an image of `size` bytes and nz slices: the image, the
// directory (offsets, lengths, chunk bases) and the per-chunk arrays
mcg_status prepare(mcg_context *ctx, int nz, int64_t size) {
    const size_t chunks = (size_t)(size / (2 * RD_CHUNK)) + (size_t)nz + 1;  // bounds the chunks of any image
    if (!ensure(&ctx->rle_image, &ctx->rle_image_cap, (size_t)size + 64) ||
        !ensure(&ctx->rd_dir, &ctx->rd_dir_cap, 3 * (size_t)nz + 1) || !ensure(&ctx->rd_err, &ctx->rd_err_cap, 1) ||
        !ensure(&ctx->rd_sum, &ctx->rd_sum_cap, chunks * sizeof(Sum)) ||
        !ensure(&ctx->rd_first, &ctx->rd_first_cap, chunks) || !ensure(&ctx->rd_entry, &ctx->rd_entry_cap, chunks))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    ctx->rd_dir_n = nz;
    return MCG_OK;
}

// chunks of a slice of len record bytes
inline long long slice_chunks(long long len) { return (len / 2 + RD_CHUNK - 1) / RD_CHUNK; }

mcg_status finish(mcg_context *ctx, cudaStream_t s) {
    int h_err = 0;
    cudaError_t e = cudaMemcpyAsync(&h_err, ctx->rd_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    return h_err ? MCG_ERR_FORMAT : MCG_OK;
}

bool pread_full(int fd, uint8_t *dst, int64_t n, int64_t off) {
    while (n > 0) {
        const ssize_t r = pread(fd, dst, (size_t)std::min<int64_t>(n, (int64_t)1 << 30), (off_t)off);
        if (r <= 0) {
            if (r < 0 && errno == EINTR) continue;
            return false;
        }
        dst += r;
        off += r;
        n -= r;
    }
    return true;
}

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" mcg_status mcg_rle_decode(mcg_context *ctx, const uint8_t *image, int64_t size, void *vol,
                                     int64_t capacity_voxels, mcg_stream_t stream) {
    if (!ctx || !image || !vol) return MCG_ERR_INVALID_ARG;
    int32_t dims[3];
    float params[3];
    mcg_status st = mcg_rle_header(image, size, dims, params);
    if (st != MCG_OK) return st;
    const int64_t xy = (int64_t)dims[0] * dims[1];
    if (xy * dims[2] > capacity_voxels) return MCG_ERR_CAPACITY;
    if (xy > INT32_MAX / 2) return MCG_ERR_TOO_LARGE;
    const int nz = dims[2];
    std::vector<long long> dir(3 * (size_t)nz + 1);  // offsets, lengths, chunk bases
    long long *cbase = dir.data() + 2 * (size_t)nz;
    int64_t p = 40;
    cbase[0] = 0;
    for (int z = 0; z < nz; ++z) {
        if (p + 4 > size) return MCG_ERR_FORMAT;
        uint32_t s32;
        memcpy(&s32, image + p, 4);
        p += 4;
        if (p + (int64_t)s32 > size) return MCG_ERR_FORMAT;
        dir[z] = p;
        dir[nz + z] = s32;
        cbase[z + 1] = cbase[z] + slice_chunks(s32);
        p += s32;
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    if ((st = prepare(ctx, nz, p)) != MCG_OK) return st;
    const cudaStream_t s = (cudaStream_t)stream;
    if ((e = cudaMemsetAsync(ctx->rd_err, 0, sizeof(int), s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(ctx->rd_dir, dir.data(), dir.size() * sizeof(long long), cudaMemcpyHostToDevice, s)) !=
            cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    // slabs of whole slices: each copied on a copy stream, then expanded on
    // s while the next slab copies
    cudaStream_t cs = nullptr;
    std::vector<cudaEvent_t> evs;
    auto done = [&](mcg_status r) {
        if (cs) cudaStreamSynchronize(cs);
        cudaStreamSynchronize(s);  // the directory copy reads dir
        for (auto ev : evs) cudaEventDestroy(ev);
        if (cs) cudaStreamDestroy(cs);
        return r;
    };
    cudaEvent_t ev = nullptr;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) {
        cs = nullptr;
        return done(mcg_cuda_fail(ctx, e));
    }
    auto new_event = [&]() -> cudaError_t {
        const cudaError_t r = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (r == cudaSuccess) evs.push_back(ev);
        return r;
    };
    // the copies wait for earlier work on s (an earlier decode reads the image buffer)
    if ((e = new_event()) != cudaSuccess || (e = cudaEventRecord(ev, s)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(cs, ev, 0)) != cudaSuccess)
        return done(mcg_cuda_fail(ctx, e));
    Slab sl{0, 0, 0, 0};
    while (sl.z1 < nz) {
        sl.z0 = sl.z1;
        sl.b0 = sl.b1;
        while (sl.z1 < nz && (sl.z1 == sl.z0 || dir[sl.z1] + dir[nz + sl.z1] - sl.b0 <= RD_SLAB)) ++sl.z1;
        sl.b1 = dir[sl.z1 - 1] + dir[nz + sl.z1 - 1];
        if ((e = cudaMemcpyAsync(ctx->rle_image + sl.b0, image + sl.b0, (size_t)(sl.b1 - sl.b0),
                                 cudaMemcpyHostToDevice, cs)) != cudaSuccess ||
            (e = new_event()) != cudaSuccess || (e = cudaEventRecord(ev, cs)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(s, ev, 0)) != cudaSuccess ||
            (e = launch_expand(ctx, sl, cbase, xy, vol, s)) != cudaSuccess)
            return done(mcg_cuda_fail(ctx, e));
    }
    return done(finish(ctx, s));
}

extern "C" mcg_status mcg_rle_decode_file(mcg_context *ctx, const char *path, void *vol, int64_t capacity_voxels,
                                          int32_t dims[3], float params[3], mcg_stream_t stream) {
    if (!ctx || !path || !vol || !dims || !params) return MCG_ERR_INVALID_ARG;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return MCG_ERR_IO;
    struct stat sb;
    uint8_t head[40];
    if (fstat(fd, &sb) != 0 || !pread_full(fd, head, std::min<int64_t>(40, (int64_t)sb.st_size), 0)) {
        close(fd);
        return MCG_ERR_IO;
    }
    const int64_t size = (int64_t)sb.st_size;
    mcg_status st = mcg_rle_header(head, size, dims, params);
    const int64_t xy = (int64_t)dims[0] * dims[1];
    if (st == MCG_OK && xy * dims[2] > capacity_voxels) st = MCG_ERR_CAPACITY;
    if (st == MCG_OK && xy > INT32_MAX / 2) st = MCG_ERR_TOO_LARGE;
    cudaError_t e = cudaSuccess;
    if (st == MCG_OK && (e = cudaSetDevice(ctx->device)) != cudaSuccess) st = mcg_cuda_fail(ctx, e);
    const int nz = dims[2];
    if (st == MCG_OK) st = prepare(ctx, nz, size);
    if (st == MCG_OK && !ctx->h_rd_stage) {
        if (cudaMallocHost((void **)&ctx->h_rd_stage, 2 * (size_t)RD_SLAB) != cudaSuccess) {
            ctx->h_rd_stage = nullptr;
            st = mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        }
    }
    if (st != MCG_OK) {
        close(fd);
        return st;
    }
    const cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t copied[2] = {nullptr, nullptr};
    std::vector<long long> dir(3 * (size_t)nz + 1, 0);  // offsets, lengths, chunk bases
    long long *cbase = dir.data() + 2 * (size_t)nz;
    for (int b = 0; b < 2 && st == MCG_OK; ++b)
        if ((e = cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming)) != cudaSuccess) st = mcg_cuda_fail(ctx, e);
    if (st == MCG_OK && (e = cudaMemsetAsync(ctx->rd_err, 0, sizeof(int), s)) != cudaSuccess) st = mcg_cuda_fail(ctx, e);
    // Pieces of RD_SLAB bytes are read by host threads into two pinned
    // buffers and copied on s; the directory is walked in the host copy as
    // pieces arrive, and the slices that end inside the resident bytes are
    // expanded after each piece.
    int z_walk = 0, z_done = 0;
    int64_t p = 40;          // next slice byte count
    uint8_t cnt_buf[4];      // a count split across two pieces
    int cnt_have = 0;
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    for (int64_t b0 = 0, piece = 0; st == MCG_OK && b0 < size; b0 += RD_SLAB, ++piece) {
        const int64_t n = std::min<int64_t>(RD_SLAB, size - b0);
        uint8_t *buf = ctx->h_rd_stage + (size_t)(piece & 1) * RD_SLAB;
        if (piece >= 2 && (e = cudaEventSynchronize(copied[piece & 1])) != cudaSuccess) {
            st = mcg_cuda_fail(ctx, e);
            break;
        }
        const int nt = (int)std::min<int64_t>(std::min(16, hw), (n + (1 << 20) - 1) >> 20);
        std::atomic<int> ok{1};
        std::vector<std::thread> pool;
        const int64_t part = (n + nt - 1) / nt;
        for (int t = 0; t < nt; ++t) {
            const int64_t a = t * part, c = std::min(n, a + part);
            if (a >= c) break;
            pool.emplace_back([&, a, c]() {
                if (!pread_full(fd, buf + a, c - a, b0 + a)) ok.store(0);
            });
        }
        for (auto &th : pool) th.join();
        if (!ok.load()) {
            st = MCG_ERR_IO;
            break;
        }
        if ((e = cudaMemcpyAsync(ctx->rle_image + b0, buf, (size_t)n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaEventRecord(copied[piece & 1], s)) != cudaSuccess) {
            st = mcg_cuda_fail(ctx, e);
            break;
        }
        // walk the directory through this piece
        const int64_t b1 = b0 + n;
        while (z_walk < nz && p < b1) {
            while (cnt_have < 4 && p + cnt_have < b1) {
                cnt_buf[cnt_have] = buf[p + cnt_have - b0];
                ++cnt_have;
            }
            if (cnt_have < 4) break;  // the count continues in the next piece
            uint32_t s32;
            memcpy(&s32, cnt_buf, 4);
            cnt_have = 0;
            p += 4;
            if (p + (int64_t)s32 > size) {
                st = MCG_ERR_FORMAT;
                break;
            }
            dir[z_walk] = p;
            dir[nz + z_walk] = s32;
            cbase[z_walk + 1] = cbase[z_walk] + slice_chunks(s32);
            p += s32;
            ++z_walk;
        }
        if (st != MCG_OK) break;
        // slices complete in [0, b1): those walked whose bytes end by b1
        int z_ready = z_done;
        while (z_ready < z_walk && dir[z_ready] + dir[nz + z_ready] <= b1) ++z_ready;
        if (z_ready > z_done) {
            if ((e = cudaMemcpyAsync(ctx->rd_dir + z_done, dir.data() + z_done, (size_t)(z_ready - z_done) * 8,
                                     cudaMemcpyHostToDevice, s)) != cudaSuccess ||
                (e = cudaMemcpyAsync(ctx->rd_dir + nz + z_done, dir.data() + nz + z_done,
                                     (size_t)(z_ready - z_done) * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
                (e = cudaMemcpyAsync(ctx->rd_dir + 2 * nz + z_done, cbase + z_done, (size_t)(z_ready - z_done + 1) * 8,
                                     cudaMemcpyHostToDevice, s)) != cudaSuccess) {
                st = mcg_cuda_fail(ctx, e);
                break;
            }
            const Slab sl{z_done, z_ready, 0, 0};
            if ((e = launch_expand(ctx, sl, cbase, xy, vol, s)) != cudaSuccess) {
                st = mcg_cuda_fail(ctx, e);
                break;
            }
            z_done = z_ready;
        }
    }
    if (st == MCG_OK && z_walk < nz) st = MCG_ERR_FORMAT;  // the file ends inside the directory
    mcg_status fin = finish(ctx, s);
    if (st == MCG_OK) st = fin;
    for (int b = 0; b < 2; ++b)
        if (copied[b]) cudaEventDestroy(copied[b]);
    close(fd);
    return st;
}
