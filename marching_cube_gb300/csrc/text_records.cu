// Text-record volume loader on sm_103a.
//
// Replaces the host loop of cu_voxel_rlc_to_mesh (cu_kinect_fusion_v1.cu:
// 3289-3361).  The input is a stream of integers read five at a time as
// "x y z sdf weight" records by `ifs >> int`; the records inside the window
// [xs, xs+dim) x [ys, ys+dim) x [zs, zs+dim) fill a dim^3 short2 volume in
// arrival order (z fastest, then y, then x, :3327-3352) until dim^3 are
// stored.
//
// Extraction rules (C++ formatted input of int, classic locale): white space
// (space, \t \n \v \f \r) is skipped; a field is an optional sign and decimal
// digits and must lie in int's range.  An extraction therefore starts at
// every non-white-space byte that follows white space, the start of the
// text, or the last digit of a field (a sign or any other byte right after
// digits begins the next extraction).  A start whose field has no digits or
// leaves int's range is a failure; the stream ends at the first one.
//
// Device passes (64-byte slice per thread, 16 KiB segment per CTA):
//   tr_count   extraction starts per segment, lowest failing start (atomicMin)
//   tr_scan    exclusive segment offsets (one CTA)
//   tr_fields  the value of every field before the first failure, in order
//   tr_window  in-window complete records per CTA range
//   tr_wscan   exclusive CTA offsets, the fields around the end (one CTA)
//   tr_place   slot s of the s-th in-window record -> voxel (z = s % dim,
//              y = s / dim % dim, x = s / dim^2)
// How the reference loop ends (a repeated last record, a partial record, a
// failed field that repeats into every remaining slot) is decided on the
// host from the fields around the end (text_finish).
//
// Host text reaches the device through pinned staging buffers filled by
// reader threads (memcpy from memory, pread from a file), each with its own
// stream, so reading and the host-to-device copies overlap.
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <limits.h>
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

constexpr int TR_THREADS = 256;
constexpr int TR_SLICE = 64;                       // bytes per thread
constexpr int64_t TR_SEG = TR_THREADS * TR_SLICE;  // bytes per CTA
constexpr int TR_SCAN_THREADS = 1024;
constexpr unsigned long long TR_NONE = ~0ull;

// device results of one parse, read back by the host
struct TextScan {
    unsigned long long first_fail;  // offset of the first failed extraction, TR_NONE if none
    long long total;                // extraction starts in the text
    long long n_tok;                // fields before the first failure
    long long n_win;                // complete in-window records
    int fail_value;                 // value the failed extraction leaves (0, INT_MAX or INT_MIN)
    int fail_eof;                   // the failed extraction reached end of file
    int last_byte;                  // T[L-1], -1 for an empty text
    int tail_n;                     // fields in tail[]
    int tail[12];                   // the last complete record and the fields after it
};

__device__ __forceinline__ bool tr_space(unsigned c) { return c == 32u || (c - 9u) < 5u; }
__device__ __forceinline__ bool tr_digit(unsigned c) { return (c - 48u) < 10u; }
__device__ __forceinline__ bool tr_sign(unsigned c) { return c == 43u || c == 45u; }
__device__ __forceinline__ bool tr_start(unsigned prev, unsigned c) {
    return !tr_space(c) && (tr_space(prev) || (tr_digit(prev) && !tr_digit(c)));
}

struct Field {
    int64_t pos;
    int value;
    int ok;
    int eof;
};

// magnitudes above 2^31 saturate at 2^31 + 1: enough to tell INT_MIN apart
__device__ __forceinline__ unsigned long long tr_acc(unsigned long long m, unsigned c) {
    m = m * 10ull + (c - 48u);
    return m > 2147483648ull ? 2147483649ull : m;
}

__device__ __forceinline__ Field tr_finish(int64_t pos, bool neg, int nd, unsigned long long m, bool eof) {
    Field f{pos, 0, 0, eof ? 1 : 0};
    if (nd == 0) return f;  // no digits: 0
    if (neg ? m > 2147483648ull : m > 2147483647ull) {
        f.value = neg ? INT_MIN : INT_MAX;
        return f;
    }
    f.value = neg ? (int)(0ll - (long long)m) : (int)m;
    f.ok = 1;
    return f;
}

// the 64 bytes [base, base + 64) as 16 little-endian words; bytes at or past
// L read as 0 and are never examined
template <bool ALIGNED>
__device__ __forceinline__ void tr_load(const uint8_t *__restrict__ T, int64_t L, int64_t base, uint32_t w[16]) {
    if (ALIGNED && base + TR_SLICE <= L) {
        const uint4 *p = reinterpret_cast<const uint4 *>(T + base);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 v = __ldg(p + q);
            w[4 * q] = v.x;
            w[4 * q + 1] = v.y;
            w[4 * q + 2] = v.z;
            w[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < 16; ++q) w[q] = 0;
#pragma unroll
        for (int k = 0; k < TR_SLICE; ++k)
            if (base + k < L) w[k >> 2] |= (uint32_t)__ldg(T + base + k) << (8 * (k & 3));
    }
}

__device__ __forceinline__ unsigned tr_byte(const uint32_t w[16], int k) { return (w[k >> 2] >> (8 * (k & 3))) & 0xffu; }

__device__ __forceinline__ int tr_starts(const uint32_t w[16], int n, unsigned prev) {
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < TR_SLICE; ++k) {
        const unsigned c = tr_byte(w, k);
        if (k < n && tr_start(prev, c)) ++cnt;
        prev = c;
    }
    return cnt;
}

// Calls f(Field) for every extraction that starts in [base, base + n), in
// order.  A field still open at the end of the slice continues in T.
template <class F>
__device__ __forceinline__ void tr_walk(const uint8_t *__restrict__ T, int64_t L, int64_t base, const uint32_t w[16],
                                        int n, unsigned prev, F &&f) {
    bool open = false, neg = false;
    int64_t pos = 0;
    int nd = 0;
    unsigned long long m = 0;
#pragma unroll
    for (int k = 0; k < TR_SLICE; ++k) {
        if (k < n) {
            const unsigned c = tr_byte(w, k);
            if (tr_start(prev, c)) {
                if (open) f(tr_finish(pos, neg, nd, m, false));
                open = true;
                pos = base + k;
                neg = c == 45u;
                nd = 0;
                m = 0;
                if (tr_digit(c)) {
                    nd = 1;
                    m = c - 48u;
                } else if (!tr_sign(c)) {
                    f(Field{pos, 0, 0, 0});  // not a number
                    open = false;
                }
            } else if (open) {
                if (tr_digit(c)) {
                    m = tr_acc(m, c);
                    ++nd;
                } else {  // white space after the field, or no digit after a sign
                    f(tr_finish(pos, neg, nd, m, false));
                    open = false;
                }
            }
            prev = c;
        }
    }
    if (open) {
        int64_t j = base + n;
        while (j < L) {
            const unsigned c = __ldg(T + j);
            if (!tr_digit(c)) break;
            m = tr_acc(m, c);
            ++nd;
            ++j;
        }
        f(tr_finish(pos, neg, nd, m, j >= L));
    }
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <bool ALIGNED>
__global__ void __launch_bounds__(TR_THREADS) tr_count(const uint8_t *__restrict__ T, int64_t L,
                                                       long long *__restrict__ seg_count,
                                                       unsigned long long *__restrict__ first_fail) {
    __shared__ int s_cnt[TR_THREADS / 32];
    __shared__ unsigned long long s_fail[TR_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * TR_SEG + (int64_t)threadIdx.x * TR_SLICE;
    int cnt = 0;
    unsigned long long fail = TR_NONE;
    if (base < L) {
        uint32_t w[16];
        tr_load<ALIGNED>(T, L, base, w);
        const int n = (int)min((int64_t)TR_SLICE, L - base);
        const unsigned prev = base == 0 ? 32u : __ldg(T + base - 1);
        tr_walk(T, L, base, w, n, prev, [&](const Field &f) {
            ++cnt;
            if (!f.ok && fail == TR_NONE) fail = (unsigned long long)f.pos;
        });
    }
    cnt = warp_sum(cnt);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, fail, o);
        fail = v < fail ? v : fail;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        s_cnt[wid] = cnt;
        s_fail[wid] = fail;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long tot = 0;
        unsigned long long mf = TR_NONE;
        for (int i = 0; i < TR_THREADS / 32; ++i) {
            tot += s_cnt[i];
            mf = s_fail[i] < mf ? s_fail[i] : mf;
        }
        seg_count[blockIdx.x] = tot;
        if (mf != TR_NONE) atomicMin(first_fail, mf);
    }
}

// exclusive scan of n counts by one CTA of TR_SCAN_THREADS threads; returns the total
__device__ long long block_scan_exclusive(const long long *__restrict__ in, long long *__restrict__ out, long long n) {
    __shared__ long long s_w[TR_SCAN_THREADS / 32];
    __shared__ long long s_total;
    const long long per = (n + TR_SCAN_THREADS - 1) / TR_SCAN_THREADS;
    const long long b = per * threadIdx.x, e = min(n, b + per);
    long long sum = 0;
    for (long long i = b; i < e; ++i) sum += in[i];
    // warp inclusive scan
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long run = 0;
        for (int i = 0; i < TR_SCAN_THREADS / 32; ++i) {
            const long long v = s_w[i];
            s_w[i] = run;
            run += v;
        }
        s_total = run;
    }
    __syncthreads();
    long long run = s_w[wid] + inc - sum;
    for (long long i = b; i < e; ++i) {
        const long long v = in[i];
        out[i] = run;
        run += v;
    }
    const long long total = s_total;
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(TR_SCAN_THREADS) tr_scan(const long long *__restrict__ seg_count,
                                                           long long *__restrict__ seg_ofs, long long nseg,
                                                           TextScan *__restrict__ res) {
    const long long total = block_scan_exclusive(seg_count, seg_ofs, nseg);
    if (threadIdx.x == 0) {
        res->total = total;
        res->n_tok = total;  // replaced by tr_fields when a field fails
    }
}

template <bool ALIGNED>
__global__ void __launch_bounds__(TR_THREADS) tr_fields(const uint8_t *__restrict__ T, int64_t L,
                                                        const long long *__restrict__ seg_ofs,
                                                        TextScan *__restrict__ res, int *__restrict__ tok) {
    __shared__ int s_w[TR_THREADS / 32];
    const unsigned long long ff = res->first_fail;
    const int64_t base = (int64_t)blockIdx.x * TR_SEG + (int64_t)threadIdx.x * TR_SLICE;
    uint32_t w[16];
    int n = 0, cnt = 0;
    unsigned prev = 32u;
    if (base < L) {
        tr_load<ALIGNED>(T, L, base, w);
        n = (int)min((int64_t)TR_SLICE, L - base);
        prev = base == 0 ? 32u : __ldg(T + base - 1);
        cnt = tr_starts(w, n, prev);
    }
    // block exclusive scan of cnt
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    int wofs = 0;
    for (int i = 0; i < wid; ++i) wofs += s_w[i];
    if (base >= L || (ff != TR_NONE && (unsigned long long)base > ff)) return;
    long long j = seg_ofs[blockIdx.x] + wofs + inc - cnt;
    tr_walk(T, L, base, w, n, prev, [&](const Field &f) {
        const unsigned long long p = (unsigned long long)f.pos;
        if (p < ff) {
            tok[j] = f.value;
        } else if (p == ff) {
            res->n_tok = j;
            res->fail_value = f.value;
            res->fail_eof = f.eof;
        }
        ++j;
    });
}

__device__ __forceinline__ bool tr_inside(const int *__restrict__ r, long long xs, long long ys, long long zs,
                                          long long dim) {
    const long long x = r[0], y = r[1], z = r[2];
    return xs <= x && x < xs + dim && ys <= y && y < ys + dim && zs <= z && z < zs + dim;
}

struct Window {
    long long xs, ys, zs, dim;
};

__global__ void __launch_bounds__(TR_THREADS) tr_window(const int *__restrict__ tok, const TextScan *__restrict__ res,
                                                        Window win, long long *__restrict__ cta_count) {
    __shared__ int s_w[TR_THREADS / 32];
    const long long R = res->n_tok / 5;
    const long long r0 = R * blockIdx.x / gridDim.x, r1 = R * (blockIdx.x + 1) / gridDim.x;
    int cnt = 0;
    for (long long r = r0 + threadIdx.x; r < r1; r += TR_THREADS)
        cnt += tr_inside(tok + 5 * r, win.xs, win.ys, win.zs, win.dim) ? 1 : 0;
    cnt = warp_sum(cnt);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int i = 0; i < TR_THREADS / 32; ++i) t += s_w[i];
        cta_count[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(TR_SCAN_THREADS) tr_wscan(const long long *__restrict__ cta_count,
                                                            long long *__restrict__ cta_ofs, int nctas,
                                                            const int *__restrict__ tok, const uint8_t *__restrict__ T,
                                                            int64_t L, TextScan *__restrict__ res) {
    const long long total = block_scan_exclusive(cta_count, cta_ofs, nctas);
    if (threadIdx.x == 0) {
        res->n_win = total;
        const long long nt = res->n_tok, R = nt / 5;
        const long long from = R >= 1 ? 5 * R - 5 : 0;
        const int cnt = (int)(nt - from);
        for (int i = 0; i < cnt; ++i) res->tail[i] = tok[from + i];
        res->tail_n = cnt;
        res->last_byte = L > 0 ? (int)T[L - 1] : -1;
    }
}

__device__ __forceinline__ uint32_t tr_pack(int sdf, int w) {
    return (uint32_t)(uint16_t)(uint32_t)sdf | ((uint32_t)(uint16_t)(uint32_t)w << 16);
}

__device__ __forceinline__ unsigned long long tr_slot_index(unsigned long long s, unsigned long long dim) {
    const unsigned long long dd = dim * dim;
    const unsigned long long xi = s / dd, rem = s - xi * dd;
    const unsigned long long yi = rem / dim, zi = rem - yi * dim;
    return (zi * dim + yi) * dim + xi;
}

__global__ void __launch_bounds__(TR_THREADS) tr_place(const int *__restrict__ tok, const TextScan *__restrict__ res,
                                                       Window win, const long long *__restrict__ cta_ofs,
                                                       uint32_t *__restrict__ vol) {
    __shared__ int s_w[TR_THREADS / 32];
    const long long R = res->n_tok / 5;
    const long long r0 = R * blockIdx.x / gridDim.x, r1 = R * (blockIdx.x + 1) / gridDim.x;
    const long long cap = win.dim * win.dim * win.dim;
    long long slot0 = cta_ofs[blockIdx.x];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (long long rb = r0; rb < r1 && slot0 < cap; rb += TR_THREADS) {
        const long long r = rb + threadIdx.x;
        const bool in = r < r1 && tr_inside(tok + 5 * r, win.xs, win.ys, win.zs, win.dim);
        const unsigned bal = __ballot_sync(0xffffffffu, in);
        if (lane == 0) s_w[wid] = __popc(bal);
        __syncthreads();
        int wofs = 0, tot = 0;
#pragma unroll
        for (int i = 0; i < TR_THREADS / 32; ++i) {
            wofs += i < wid ? s_w[i] : 0;
            tot += s_w[i];
        }
        if (in) {
            const long long s = slot0 + wofs + __popc(bal & ((1u << lane) - 1u));
            if (s < cap)
                vol[tr_slot_index((unsigned long long)s, (unsigned long long)win.dim)] =
                    tr_pack(tok[5 * r + 3], tok[5 * r + 4]);
        }
        slot0 += tot;
        __syncthreads();
    }
}

// slots [s0, s1) <- one record
__global__ void tr_fill(uint32_t *__restrict__ vol, long long dim, long long s0, long long s1, uint32_t v) {
    for (long long s = s0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; s < s1;
         s += (long long)gridDim.x * blockDim.x)
        vol[tr_slot_index((unsigned long long)s, (unsigned long long)dim)] = v;
}

uint32_t host_pack(int sdf, int w) { return (uint32_t)(uint16_t)(uint32_t)sdf | ((uint32_t)(uint16_t)(uint32_t)w << 16); }

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// The last iteration of the reference loop, from the fields around the end:
//  * clean end of file, k = n_tok % 5 fields of a partial record: one more
//    record, its first k fields new and the rest kept from the record before;
//  * clean end of file, no partial record: the record before is evaluated
//    again unless its last field ran into end of file (no trailing white
//    space), or the text has no field at all (one record of zeros);
//  * a failed field at k: the first k fields new, the failed field's value
//    (0, INT_MAX or INT_MIN), the rest kept.  If the failure reached end of
//    file the record is evaluated once; otherwise the loop repeats it
//    forever: it fills every remaining slot when it lies inside the window,
//    and the reference never ends when it does not (MCG_ERR_FORMAT).
mcg_status text_finish(mcg_context *ctx, const TextScan &r, bool loop_runs, const Window &win, uint32_t *vol,
                       long long *stored, int *filled_rest, cudaStream_t s) {
    const long long cap = win.dim * win.dim * win.dim;
    long long S = std::min(r.n_win, cap);
    *filled_rest = 0;
    mcg_status st = MCG_OK;
    if (S < cap && loop_runs) {
        const long long R = r.n_tok / 5;
        const int k = (int)(r.n_tok % 5);
        int prev[5] = {0, 0, 0, 0, 0};
        const int *lo = r.tail;
        if (R >= 1) {
            for (int i = 0; i < 5; ++i) prev[i] = r.tail[i];
            lo = r.tail + 5;
        }
        int v[5];
        for (int i = 0; i < 5; ++i) v[i] = i < k ? lo[i] : prev[i];
        bool evaluate = false, stuck = false;
        if (r.first_fail == TR_NONE) {
            const bool digit_end = r.last_byte >= '0' && r.last_byte <= '9';
            evaluate = k > 0 || r.n_tok == 0 || !digit_end;
        } else {
            v[k] = r.fail_value;
            evaluate = true;
            stuck = !r.fail_eof;
        }
        if (evaluate) {
            const bool inside = win.xs <= v[0] && v[0] < win.xs + win.dim && win.ys <= v[1] &&
                                v[1] < win.ys + win.dim && win.zs <= v[2] && v[2] < win.zs + win.dim;
            if (inside) {
                const long long s1 = stuck ? cap : S + 1;
                const long long n = s1 - S;
                const int blocks = (int)std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * 8);
                tr_fill<<<blocks, 256, 0, s>>>(vol, win.dim, S, s1, host_pack(v[3], v[4]));
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
                if (stuck) *filled_rest = 1;
                S = s1;
            } else if (stuck) {
                st = MCG_ERR_FORMAT;
            }
        }
    }
    *stored = S;
    return st;
}

bool grow_bytes(uint8_t **p, size_t *cap, size_t n) { return ensure(p, cap, n); }

// Parses L bytes of device text into vol.  loop_runs = false when the line
// skip after the seek reached end of file (the loop body never runs).
mcg_status text_parse(mcg_context *ctx, const uint8_t *T, int64_t L, bool loop_runs, int dim,
                      const int32_t origin[3], uint32_t *vol, mcg_text_info *info, cudaStream_t s) {
    const Window win{origin[0], origin[1], origin[2], dim};
    const long long cap = win.dim * win.dim * win.dim;
    cudaError_t e = cudaMemsetAsync(vol, 0, (size_t)cap * 4, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const bool aligned = ((uintptr_t)T & 15) == 0;
    const long long nseg = (L + TR_SEG - 1) / TR_SEG;
    const int nctas = ctx->num_sms * 4;
    if (nseg > INT_MAX) return MCG_ERR_TOO_LARGE;
    if (!ensure(&ctx->tr_scan, &ctx->tr_scan_cap, sizeof(TextScan)) || !ensure(&ctx->tr_seg, &ctx->tr_seg_cap, 2 * (size_t)nseg + 2) ||
        !ensure(&ctx->tr_cta, &ctx->tr_cta_cap, 2 * (size_t)nctas))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    if (!ctx->h_tr_scan && cudaMallocHost((void **)&ctx->h_tr_scan, sizeof(TextScan)) != cudaSuccess) {
        ctx->h_tr_scan = nullptr;
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    }
    TextScan *d_res = reinterpret_cast<TextScan *>(ctx->tr_scan);
    TextScan *h_res = reinterpret_cast<TextScan *>(ctx->h_tr_scan);
    long long *seg_count = ctx->tr_seg, *seg_ofs = ctx->tr_seg + nseg + 1;
    if ((e = cudaMemsetAsync(d_res, 0, sizeof(TextScan), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(&d_res->first_fail, 0xff, sizeof(unsigned long long), s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    if (L > 0) {
        if (aligned)
            tr_count<true><<<(unsigned)nseg, TR_THREADS, 0, s>>>(T, L, seg_count, &d_res->first_fail);
        else
            tr_count<false><<<(unsigned)nseg, TR_THREADS, 0, s>>>(T, L, seg_count, &d_res->first_fail);
        tr_scan<<<1, TR_SCAN_THREADS, 0, s>>>(seg_count, seg_ofs, nseg, d_res);
        if ((e = cudaGetLastError()) != cudaSuccess) return mcg_cuda_fail(ctx, e);
        if ((e = cudaMemcpyAsync(h_res, d_res, sizeof(TextScan), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return mcg_cuda_fail(ctx, e);
        if (!ensure(&ctx->tr_tok, &ctx->tr_tok_cap, (size_t)h_res->total + 1))
            return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        if (aligned)
            tr_fields<true><<<(unsigned)nseg, TR_THREADS, 0, s>>>(T, L, seg_ofs, d_res, ctx->tr_tok);
        else
            tr_fields<false><<<(unsigned)nseg, TR_THREADS, 0, s>>>(T, L, seg_ofs, d_res, ctx->tr_tok);
        tr_window<<<nctas, TR_THREADS, 0, s>>>(ctx->tr_tok, d_res, win, ctx->tr_cta);
        tr_wscan<<<1, TR_SCAN_THREADS, 0, s>>>(ctx->tr_cta, ctx->tr_cta + nctas, nctas, ctx->tr_tok, T, L, d_res);
        tr_place<<<nctas, TR_THREADS, 0, s>>>(ctx->tr_tok, d_res, win, ctx->tr_cta + nctas, vol);
        if ((e = cudaGetLastError()) != cudaSuccess) return mcg_cuda_fail(ctx, e);
    } else {
        // no text: no field, no failure, no window record
        if ((e = cudaMemsetAsync(&d_res->last_byte, 0xff, sizeof(int), s)) != cudaSuccess) return mcg_cuda_fail(ctx, e);
    }
    if ((e = cudaMemcpyAsync(h_res, d_res, sizeof(TextScan), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    const TextScan r = *h_res;
    long long stored = 0;
    int filled = 0;
    const mcg_status st = text_finish(ctx, r, loop_runs, win, vol, &stored, &filled, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return mcg_cuda_fail(ctx, e);
    if (info) {
        info->bytes = L;
        info->numbers = r.n_tok;
        info->records = r.n_tok / 5;
        info->stored = stored;
        info->fail_offset = r.first_fail == TR_NONE ? -1 : (int64_t)r.first_fail;
        info->filled_rest = filled;
        info->reserved = 0;
    }
    return st;
}

bool text_args_ok(int dim, const int32_t origin[3], const void *vol) {
    return vol && origin && dim > 0 && dim <= 4096;
}

// ---- staged upload ---------------------------------------------------------
constexpr int TR_READERS = 8;
constexpr size_t TR_PIECE = (size_t)16 << 20;

// read(off, n, dst) copies bytes [off, off + n) of the source; false on error
template <class Read>
mcg_status stage_upload(mcg_context *ctx, int64_t L, const Read &read, uint8_t *dst, cudaStream_t s) {
    if (L <= 0) return MCG_OK;
    if (!ctx->h_tr_stage) {
        if (cudaMallocHost((void **)&ctx->h_tr_stage, 2 * TR_READERS * TR_PIECE) != cudaSuccess) {
            ctx->h_tr_stage = nullptr;
            return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        }
    }
    cudaEvent_t ready;
    cudaError_t e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    cudaEventRecord(ready, s);  // earlier work on s that reads dst comes first
    const int64_t npieces = (L + (int64_t)TR_PIECE - 1) / (int64_t)TR_PIECE;
    const int nthreads = (int)std::min<int64_t>(TR_READERS, npieces);
    std::atomic<int> status{MCG_OK};
    std::atomic<int> cuda_err{0};
    std::vector<std::thread> pool;
    const int device = ctx->device;
    uint8_t *stage = ctx->h_tr_stage;
    for (int t = 0; t < nthreads; ++t) {
        pool.emplace_back([&, t]() {
            cudaSetDevice(device);
            cudaStream_t ws = nullptr;
            cudaEvent_t ev[2] = {nullptr, nullptr};
            cudaError_t err = cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking);
            for (int b = 0; b < 2 && err == cudaSuccess; ++b) err = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(ws, ready, 0);
            int64_t round = 0;
            for (int64_t p = t; p < npieces && err == cudaSuccess && status.load() == MCG_OK; p += nthreads, ++round) {
                const int b = (int)(round & 1);
                uint8_t *buf = stage + ((size_t)t * 2 + b) * TR_PIECE;
                if (round >= 2 && (err = cudaEventSynchronize(ev[b])) != cudaSuccess) break;
                const int64_t off = p * (int64_t)TR_PIECE;
                const int64_t n = std::min<int64_t>((int64_t)TR_PIECE, L - off);
                if (!read(off, n, buf)) {
                    int expect = MCG_OK;
                    status.compare_exchange_strong(expect, MCG_ERR_IO);
                    break;
                }
                if ((err = cudaMemcpyAsync(dst + off, buf, (size_t)n, cudaMemcpyHostToDevice, ws)) != cudaSuccess) break;
                err = cudaEventRecord(ev[b], ws);
            }
            // the parse runs on s once every copy has landed, and the staging
            // buffers are reused by the next call: wait for the copies
            if (ws) {
                const cudaError_t e2 = cudaStreamSynchronize(ws);
                if (err == cudaSuccess) err = e2;
            }
            for (int b = 0; b < 2; ++b)
                if (ev[b]) cudaEventDestroy(ev[b]);
            if (ws) cudaStreamDestroy(ws);
            if (err != cudaSuccess) {
                int expect = 0;
                cuda_err.compare_exchange_strong(expect, (int)err);
            }
        });
    }
    for (auto &th : pool) th.join();
    cudaEventDestroy(ready);
    if (cuda_err.load() != 0) return mcg_cuda_fail(ctx, (cudaError_t)cuda_err.load());
    return (mcg_status)status.load();
}

bool pread_all(int fd, uint8_t *dst, int64_t n, int64_t off) {
    while (n > 0) {
        const ssize_t r = pread(fd, dst, (size_t)std::min<int64_t>(n, (int64_t)1 << 30), (off_t)off);
        if (r < 0) {
            if (errno == EINTR) continue;
            return false;
        }
        if (r == 0) return false;
        dst += r;
        off += r;
        n -= r;
    }
    return true;
}

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" mcg_status mcg_text_records_parse(mcg_context *ctx, const void *text, int64_t len, int32_t dim,
                                             const int32_t origin[3], void *vol, mcg_text_info *info,
                                             mcg_stream_t stream) {
    if (!ctx || len < 0 || (len > 0 && !text) || !text_args_ok(dim, origin, vol)) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    return text_parse(ctx, static_cast<const uint8_t *>(text), len, true, dim, origin, static_cast<uint32_t *>(vol),
                      info, (cudaStream_t)stream);
}

extern "C" mcg_status mcg_text_records_load(mcg_context *ctx, const void *text, int64_t len, int32_t dim,
                                            const int32_t origin[3], void *vol, mcg_text_info *info,
                                            mcg_stream_t stream) {
    if (!ctx || len < 0 || (len > 0 && !text) || !text_args_ok(dim, origin, vol)) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const cudaStream_t s = (cudaStream_t)stream;
    if (!grow_bytes(&ctx->tr_text, &ctx->tr_text_cap, (size_t)len + 16)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    cudaPointerAttributes attr;
    const bool pinned = cudaPointerGetAttributes(&attr, text) == cudaSuccess && attr.type == cudaMemoryTypeHost;
    cudaGetLastError();
    mcg_status st;
    if (pinned) {
        e = cudaMemcpyAsync(ctx->tr_text, text, (size_t)len, cudaMemcpyHostToDevice, s);
        st = e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
    } else {
        const uint8_t *src = static_cast<const uint8_t *>(text);
        st = stage_upload(ctx, len, [src](int64_t off, int64_t n, uint8_t *dst) {
            memcpy(dst, src + off, (size_t)n);
            return true;
        }, ctx->tr_text, s);
    }
    if (st != MCG_OK) return st;
    return text_parse(ctx, ctx->tr_text, len, true, dim, origin, static_cast<uint32_t *>(vol), info, s);
}

extern "C" mcg_status mcg_text_records_load_file(mcg_context *ctx, const char *path, int64_t tail_bytes, int32_t dim,
                                                 const int32_t origin[3], void *vol, mcg_text_info *info,
                                                 mcg_stream_t stream) {
    if (!ctx || !path || !text_args_ok(dim, origin, vol)) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    const cudaStream_t s = (cudaStream_t)stream;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return MCG_ERR_IO;
    struct stat sb;
    if (fstat(fd, &sb) != 0) {
        close(fd);
        return MCG_ERR_IO;
    }
    const int64_t flen = (int64_t)sb.st_size;
    int64_t start = 0;
    bool loop_runs = true;
    if (tail_bytes > 0 && flen > tail_bytes) {
        // the line cut by the seek is skipped, up to and including its '\n'
        start = flen - tail_bytes;
        uint8_t buf[4096];
        bool found = false;
        while (!found && start < flen) {
            const int64_t n = std::min<int64_t>((int64_t)sizeof(buf), flen - start);
            if (!pread_all(fd, buf, n, start)) {
                close(fd);
                return MCG_ERR_IO;
            }
            const void *nl = memchr(buf, '\n', (size_t)n);
            if (nl) {
                start += (const uint8_t *)nl - buf + 1;
                found = true;
            } else {
                start += n;
            }
        }
        loop_runs = found;
    }
    const int64_t L = flen - start;
    if (!grow_bytes(&ctx->tr_text, &ctx->tr_text_cap, (size_t)L + 16)) {
        close(fd);
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    }
    const mcg_status st = stage_upload(ctx, L, [fd, start](int64_t off, int64_t n, uint8_t *dst) {
        return pread_all(fd, dst, n, start + off);
    }, ctx->tr_text, s);
    close(fd);
    if (st != MCG_OK) return st;
    return text_parse(ctx, ctx->tr_text, L, loop_runs, dim, origin, static_cast<uint32_t *>(vol), info, s);
}
