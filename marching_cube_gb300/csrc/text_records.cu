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
// Device passes (32-byte slice per thread, 8 KiB segment per CTA), run per
// 64 MiB chunk of text as the chunks land:
//   tr_count   extraction starts per segment, lowest failing start (atomicMin);
//              byte classes as bit masks (SWAR), an exact byte walk only for
//              slices with ten-digit runs or the first failure
//   tr_scan    exclusive segment offsets, continuing the running total (one CTA)
//   tr_fields  the value of every field before the first failure, in order
//   tr_window  in-window records among those the chunk completes, per CTA
//   tr_wscan   exclusive CTA offsets, continuing the running count (one CTA)
//   tr_place   the s-th in-window record -> slot s of an arrival-order array
// and once at the end:
//   tr_transpose  slot s -> voxel (z = s % dim, y = s / dim % dim,
//              x = s / dim^2) through shared-memory tiles; unfilled -> 0
// How the reference loop ends (a repeated last record, a partial record, a
// failed field that repeats into every remaining slot) is decided on the
// host from the fields around the end (text_finish).
//
// Host text in memory is copied chunk by chunk on a copy stream (the driver
// moves pageable memory at about the pinned rate on this platform); a file
// is read chunk by chunk by host threads (pread) into two pinned staging
// buffers, so file reads, copies and the passes overlap.
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
constexpr int TR_SLICE = 32;                       // bytes per thread
constexpr int TR_WORDS = TR_SLICE / 4;
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
    int incomplete;                 // a field ran past the bytes resident at its pass
    long long rec_done;             // records windowed by the chunks so far
    long long cur_rb, cur_re;       // the record range of the current chunk
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

// nw little-endian words of T from byte base; bytes at or past L read as 0
template <bool ALIGNED, int NW>
__device__ __forceinline__ void tr_load(const uint8_t *__restrict__ T, int64_t L, int64_t base, uint32_t *w) {
    if (ALIGNED && base + 4 * NW <= L) {
        const uint4 *p = reinterpret_cast<const uint4 *>(T + base);
#pragma unroll
        for (int q = 0; q < NW / 4; ++q) {
            const uint4 v = __ldg(p + q);
            w[4 * q] = v.x;
            w[4 * q + 1] = v.y;
            w[4 * q + 2] = v.z;
            w[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < NW; ++q) w[q] = 0;
#pragma unroll
        for (int k = 0; k < 4 * NW; ++k)
            if (base + k < L) w[k >> 2] |= (uint32_t)__ldg(T + base + k) << (8 * (k & 3));
    }
}

__device__ __forceinline__ unsigned tr_byte(const uint32_t *w, int k) { return (w[k >> 2] >> (8 * (k & 3))) & 0xffu; }

// Exact walk (any field length, failures): calls f(Field) for every
// extraction that starts in [base, base + n), in order.  A field still open
// at the end of the slice continues in T, up to the resident bytes [0, La).
template <class F>
__device__ __forceinline__ void tr_walk(const uint8_t *__restrict__ T, int64_t L, int64_t La, int64_t base,
                                        const uint32_t *w, int n, unsigned prev, int *incomplete, F &&f) {
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
        while (j < La) {
            const unsigned c = __ldg(T + j);
            if (!tr_digit(c)) break;
            m = tr_acc(m, c);
            ++nd;
            ++j;
        }
        if (j >= La && La < L) atomicOr(incomplete, 1);  // the rest of the field is not resident yet
        f(tr_finish(pos, neg, nd, m, j >= L));
    }
}

// ---- byte classes as bit masks (bit k = byte k) -----------------------------
// SWAR over 32-bit words: with t = x & 0x7f7f7f7f, the high bit of byte i of
// t + (0x80 - c) * 0x01010101 is set iff (byte i & 0x7f) >= c (no carries
// cross bytes); bytes >= 0x80 belong to no class.
__device__ __forceinline__ uint32_t tr_ge(uint32_t t, uint32_t c) { return t + (0x80u - c) * 0x01010101u; }
// bits 7, 15, 23, 31 -> bits 0..3 (the partial products never overlap)
__device__ __forceinline__ uint32_t tr_movemask(uint32_t m) { return ((m & 0x80808080u) * 0x00204081u) >> 28; }
__device__ __forceinline__ uint32_t tr_digits4(uint32_t x) {
    const uint32_t t = x & 0x7f7f7f7fu;
    return tr_movemask(tr_ge(t, 0x30) & ~tr_ge(t, 0x3a) & ~x);
}

struct Masks {
    uint32_t D, S, G, Mn;  // digit, white space, sign, '-'
    uint32_t start;        // an extraction starts here
    uint32_t invalid;      // ... and fails at once (no digit follows)
    uint32_t Dnext;        // digits among the 16 bytes after the slice
};

// look: the 16 bytes after the slice (0 past L)
__device__ __forceinline__ Masks tr_masks(const uint32_t *w, const uint32_t *look, int n, unsigned prev) {
    Masks m{0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int q = 0; q < TR_WORDS; ++q) {
        const uint32_t x = w[q], t = x & 0x7f7f7f7fu, lo7 = ~x;
        const uint32_t dig = tr_ge(t, 0x30) & ~tr_ge(t, 0x3a) & lo7;
        const uint32_t ws = ((tr_ge(t, 0x09) & ~tr_ge(t, 0x0e)) | (tr_ge(t, 0x20) & ~tr_ge(t, 0x21))) & lo7;
        const uint32_t minus = tr_ge(t, 0x2d) & ~tr_ge(t, 0x2e) & lo7;
        const uint32_t sg = (tr_ge(t, 0x2b) & ~tr_ge(t, 0x2c) & lo7) | minus;
        m.D |= tr_movemask(dig) << (4 * q);
        m.S |= tr_movemask(ws) << (4 * q);
        m.G |= tr_movemask(sg) << (4 * q);
        m.Mn |= tr_movemask(minus) << (4 * q);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) m.Dnext |= tr_digits4(look[q]) << (4 * q);
    const uint32_t valid = n >= 32 ? ~0u : ((1u << n) - 1u);
    m.D &= valid;
    m.S &= valid;
    m.G &= valid;
    m.Mn &= valid;
    if (n < 32) m.Dnext = 0;
    const uint32_t N = ~m.S & valid;
    const uint32_t Dp = (m.D << 1) | (uint32_t)((prev - 48u) < 10u);
    const uint32_t Sp = (m.S << 1) | (uint32_t)tr_space(prev);
    m.start = N & (Sp | (Dp & ~m.D));
    const uint32_t Dn = (m.D >> 1) | ((m.Dnext & 1u) << 31);
    m.invalid = m.start & ~(m.D | (m.G & Dn));
    return m;
}

// true when a digit run of ten or more may lie in the slice, or the run at
// its end continues into the next bytes to ten or more: such fields may
// leave int's range and take the exact walk
__device__ __forceinline__ bool tr_long_run(const Masks &m) {
    uint32_t r = m.D;
#pragma unroll
    for (int i = 1; i < 10; ++i) r &= m.D >> i;
    if (r) return true;
    const int top = __clz(~m.D);          // digits ending the slice
    const int more = __ffs(~m.Dnext) - 1;  // digits starting the next bytes (-1: all 16)
    return top + (more < 0 ? 16 : more) >= 10;
}

// Value of the nd (1..9) decimal digits at T[pos]: eight bytes gathered
// little-endian (first digit lowest) as two words, '0' subtracted, shifted
// so the digits fill the top bytes, then pairs and quads combined by
// multiply-add (10, 100) inside each word and the words by 10000; a ninth
// digit last.
template <bool ALIGNED>
__device__ __forceinline__ unsigned tr_value(const uint8_t *__restrict__ T, int64_t L, int64_t pos, int nd) {
    uint32_t lo = 0, hi = 0;
    const int64_t a = pos & ~3ll;
    if (ALIGNED && a + 12 <= L) {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(T + a);
        const uint32_t w0 = __ldg(p), w1 = __ldg(p + 1), w2 = __ldg(p + 2);
        const unsigned sh = (unsigned)(pos - a) * 8u;
        lo = __funnelshift_r(w0, w1, sh);
        hi = __funnelshift_r(w1, w2, sh);
    } else {
        for (int i = 0; i < 8 && i < nd; ++i) {
            const uint32_t b = __ldg(T + pos + i);
            if (i < 4)
                lo |= b << (8 * i);
            else
                hi |= b << (8 * (i - 4));
        }
    }
    const int n8 = nd < 8 ? nd : 8;
    lo -= 0x30303030u;  // a borrow out of lo only leaves bytes that are shifted out
    hi -= 0x30303030u;
    const unsigned s = 8u * (unsigned)(8 - n8);
    if (s >= 32) {
        hi = lo << (s - 32);
        lo = 0;
    } else {
        hi = __funnelshift_l(lo, hi, s);
        lo <<= s;
    }
    lo = (lo * 10u + (lo >> 8)) & 0x00FF00FFu;
    hi = (hi * 10u + (hi >> 8)) & 0x00FF00FFu;
    lo = (lo * 100u + (lo >> 16)) & 0xFFFFu;
    hi = (hi * 100u + (hi >> 16)) & 0xFFFFu;
    unsigned v = lo * 10000u + hi;
    if (nd > 8) v = v * 10u + (__ldg(T + pos + 8) - 48u);
    return v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// the slice of this thread: words, its masks, prev byte and length
template <bool ALIGNED>
__device__ __forceinline__ int tr_slice(const uint8_t *__restrict__ T, int64_t L, int64_t base, uint32_t *w,
                                        unsigned *prev, Masks *m) {
    uint32_t look[4];
    tr_load<ALIGNED, TR_WORDS>(T, L, base, w);
    tr_load<ALIGNED, 4>(T, L, base + TR_SLICE, look);
    const int n = (int)min((int64_t)TR_SLICE, L - base);
    *prev = base == 0 ? 32u : __ldg(T + base - 1);
    *m = tr_masks(w, look, n, *prev);
    return n;
}

// segments seg0 + blockIdx.x; the bytes [0, La) are resident
template <bool ALIGNED>
__global__ void __launch_bounds__(TR_THREADS) tr_count(const uint8_t *__restrict__ T, int64_t L, int64_t La,
                                                       long long seg0, long long *__restrict__ seg_count,
                                                       TextScan *__restrict__ res) {
    __shared__ int s_cnt[TR_THREADS / 32];
    __shared__ unsigned long long s_fail[TR_THREADS / 32];
    const long long seg = seg0 + blockIdx.x;
    const int64_t base = seg * TR_SEG + (int64_t)threadIdx.x * TR_SLICE;
    int cnt = 0;
    unsigned long long fail = TR_NONE;
    if (base < L) {
        uint32_t w[TR_WORDS];
        unsigned prev;
        Masks m;
        const int n = tr_slice<ALIGNED>(T, L, base, w, &prev, &m);
        if (tr_long_run(m)) {
            tr_walk(T, L, La, base, w, n, prev, &res->incomplete, [&](const Field &f) {
                ++cnt;
                if (!f.ok && fail == TR_NONE) fail = (unsigned long long)f.pos;
            });
        } else {
            cnt = __popc(m.start);
            if (m.invalid) fail = (unsigned long long)(base + __ffs(m.invalid) - 1);
        }
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
        seg_count[seg] = tot;
        if (mf != TR_NONE) atomicMin(&res->first_fail, mf);
    }
}

// exclusive scan of n counts by one CTA of TR_SCAN_THREADS threads; returns the total
__device__ long long block_scan_exclusive(const long long *__restrict__ in, long long *__restrict__ out, long long n,
                                          long long carry = 0) {
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
    long long run = carry + s_w[wid] + inc - sum;
    for (long long i = b; i < e; ++i) {
        const long long v = in[i];
        out[i] = run;
        run += v;
    }
    const long long total = s_total;
    __syncthreads();
    return total;
}

// segment offsets of one chunk, continuing the running total in res->total;
// after the last chunk n_tok = total unless a field failed (tr_fields sets it)
__global__ void __launch_bounds__(TR_SCAN_THREADS) tr_scan(const long long *__restrict__ seg_count,
                                                           long long *__restrict__ seg_ofs, long long nseg,
                                                           TextScan *__restrict__ res, int last) {
    const long long carry = res->total;
    const long long total = block_scan_exclusive(seg_count, seg_ofs, nseg, carry);
    if (threadIdx.x == 0) {
        res->total = carry + total;
        if (last && res->first_fail == TR_NONE) res->n_tok = carry + total;
    }
}

template <bool ALIGNED>
__global__ void __launch_bounds__(TR_THREADS) tr_fields(const uint8_t *__restrict__ T, int64_t L, int64_t La,
                                                        long long seg0, const long long *__restrict__ seg_ofs,
                                                        TextScan *__restrict__ res, int *__restrict__ tok,
                                                        long long tok_cap) {
    __shared__ int s_w[TR_THREADS / 32];
    const unsigned long long ff = res->first_fail;
    const long long seg = seg0 + blockIdx.x;
    const int64_t base = seg * TR_SEG + (int64_t)threadIdx.x * TR_SLICE;
    uint32_t w[TR_WORDS];
    int n = 0, cnt = 0;
    unsigned prev = 32u;
    Masks m{0, 0, 0, 0, 0, 0, 0};
    if (base < L) {
        n = tr_slice<ALIGNED>(T, L, base, w, &prev, &m);
        cnt = __popc(m.start);
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
    long long j = seg_ofs[seg] + wofs + inc - cnt;
    if (j + cnt > tok_cap) {  // cannot happen: tok_cap bounds the extractions of any text
        atomicOr(&res->incomplete, 2);
        return;
    }
    const bool has_fail = ff != TR_NONE && (unsigned long long)(base + TR_SLICE) > ff;
    if (has_fail || tr_long_run(m)) {
        tr_walk(T, L, La, base, w, n, prev, &res->incomplete, [&](const Field &f) {
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
        return;
    }
    // every field of the slice is valid and shorter than ten digits: one
    // field per set bit of the start mask, its digits converted eight at a
    // time (tr_value)
    const int more = __ffs(~m.Dnext) - 1;  // digits opening the next bytes (< 10 here)
    uint32_t st = m.start;
    while (st) {
        const int p = __ffs(st) - 1;
        st &= st - 1;
        const int q = p + (int)((m.G >> p) & 1u);  // first digit
        int nd = q < 32 ? __ffs(~(m.D >> q)) - 1 : 0;
        if (nd < 0 || q + nd == 32) nd = (32 - q) + more;
        const unsigned v = tr_value<ALIGNED>(T, L, base + q, nd);
        tok[j++] = ((m.Mn >> p) & 1u) ? -(int)v : (int)v;
    }
}

__device__ __forceinline__ bool tr_inside(const int *__restrict__ r, long long xs, long long ys, long long zs,
                                          long long dim) {
    const long long x = r[0], y = r[1], z = r[2];
    return xs <= x && x < xs + dim && ys <= y && y < ys + dim && zs <= z && z < zs + dim;
}

struct Window {
    long long xs, ys, zs, dim;
};

// Records complete after the current chunk: [rec_done, Re), Re = fields so
// far / 5, or n_tok / 5 once a field has failed (a failure is always known
// by the chunk that holds it, and n_tok is final then).
__device__ __forceinline__ void tr_records(const TextScan *res, long long *rb, long long *re) {
    *rb = res->rec_done;
    *re = (res->first_fail == TR_NONE ? res->total : res->n_tok) / 5;
}

__global__ void __launch_bounds__(TR_THREADS) tr_window(const int *__restrict__ tok, const TextScan *__restrict__ res,
                                                        Window win, long long *__restrict__ cta_count) {
    __shared__ int s_w[TR_THREADS / 32];
    long long Rb, Re;
    tr_records(res, &Rb, &Re);
    const long long R = Re - Rb;
    const long long r0 = Rb + R * blockIdx.x / gridDim.x, r1 = Rb + R * (blockIdx.x + 1) / gridDim.x;
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

// CTA slot offsets of the current chunk's records, continuing the running
// in-window count n_win; fixes the chunk's record range for tr_place.  After
// the last chunk: the fields around the end and the last byte for the host.
__global__ void __launch_bounds__(TR_SCAN_THREADS) tr_wscan(const long long *__restrict__ cta_count,
                                                            long long *__restrict__ cta_ofs, int nctas,
                                                            const int *__restrict__ tok, const uint8_t *__restrict__ T,
                                                            int64_t L, TextScan *__restrict__ res, int last) {
    long long Rb, Re;
    tr_records(res, &Rb, &Re);
    const long long carry = res->n_win;
    const long long total = block_scan_exclusive(cta_count, cta_ofs, nctas, carry);
    if (threadIdx.x == 0) {
        res->n_win = carry + total;
        res->cur_rb = Rb;
        res->cur_re = Re;
        res->rec_done = Re;
        if (last) {
            const long long nt = res->n_tok, R = nt / 5;
            const long long from = R >= 1 ? 5 * R - 5 : 0;
            const int cnt = (int)(nt - from);
            for (int i = 0; i < cnt; ++i) res->tail[i] = tok[from + i];
            res->tail_n = cnt;
            res->last_byte = L > 0 ? (int)T[L - 1] : -1;
        }
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
                                                       uint32_t *__restrict__ arr) {
    __shared__ int s_w[TR_THREADS / 32];
    const long long Rb = res->cur_rb, R = res->cur_re - Rb;
    const long long r0 = Rb + R * blockIdx.x / gridDim.x, r1 = Rb + R * (blockIdx.x + 1) / gridDim.x;
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
            if (s < cap) arr[s] = tr_pack(tok[5 * r + 3], tok[5 * r + 4]);
        }
        slot0 += tot;
        __syncthreads();
    }
}

// arrival order -> volume: arr[(xi*dim + yi)*dim + zi] -> vol[(zi*dim + yi)*dim + xi]
// through a 32 x 32 (x, z) tile per CTA at one y; slots past the stored ones
// read as zero
__global__ void __launch_bounds__(256) tr_transpose(const uint32_t *__restrict__ arr,
                                                    const TextScan *__restrict__ res, long long dim,
                                                    uint32_t *__restrict__ vol) {
    __shared__ uint32_t tile[32][33];
    const long long cap = dim * dim * dim;
    const long long S = min(res->n_win, cap);
    const long long zi0 = (long long)blockIdx.x * 32, xi0 = (long long)blockIdx.y * 32, yi = blockIdx.z;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const long long xi = xi0 + threadIdx.y + 8 * r, zi = zi0 + threadIdx.x;
        const long long sl = (xi * dim + yi) * dim + zi;
        tile[threadIdx.y + 8 * r][threadIdx.x] = (xi < dim && zi < dim && sl < S) ? arr[sl] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const long long zi = zi0 + threadIdx.y + 8 * r, xi = xi0 + threadIdx.x;
        if (zi < dim && xi < dim) vol[(zi * dim + yi) * dim + xi] = tile[threadIdx.x][threadIdx.y + 8 * r];
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

bool text_args_ok(int dim, const int32_t origin[3], const void *vol) {
    return vol && origin && dim > 0 && dim <= 4096;
}

constexpr int64_t TR_CHUNK = (int64_t)64 << 20;  // bytes per pipelined chunk, a multiple of TR_SEG
static_assert(TR_CHUNK % TR_SEG == 0, "chunks hold whole segments");

// Parses the L bytes of text at T (device) into vol.  The text arrives in
// chunks of TR_CHUNK bytes: feed(i, off, n, cs) enqueues chunk i's bytes
// [off, off + n) into T on stream cs (a null feed: the text is resident).
// Chunk i is counted, scanned (carrying the running total), its fields
// converted and the records it completes placed once chunk i + 1 has
// landed, so the passes overlap the copies; the transpose runs at the end.  A field longer than a chunk
// that runs past the resident bytes sets `incomplete`, and the whole text is
// parsed again once resident.  loop_runs = false when the line skip after
// the seek reached end of file (the reference loop body never runs).
template <class Feed>
mcg_status text_run(mcg_context *ctx, const uint8_t *T, int64_t L, const Feed *feed, bool loop_runs, int dim,
                    const int32_t origin[3], uint32_t *vol, mcg_text_info *info, cudaStream_t s) {
    const Window win{origin[0], origin[1], origin[2], dim};
    const long long cap = win.dim * win.dim * win.dim;
    const bool aligned = ((uintptr_t)T & 15) == 0;
    const long long nseg = (L + TR_SEG - 1) / TR_SEG;
    const int nctas = ctx->num_sms * 4;
    const long long tok_cap = L / 2 + 64;  // no three extraction starts are adjacent
    cudaError_t e;
    if (!ensure(&ctx->tr_scan, &ctx->tr_scan_cap, sizeof(TextScan)) ||
        !ensure(&ctx->tr_seg, &ctx->tr_seg_cap, 2 * (size_t)nseg + 2) ||
        !ensure(&ctx->tr_cta, &ctx->tr_cta_cap, 2 * (size_t)nctas) ||
        !ensure(&ctx->tr_arr, &ctx->tr_arr_cap, (size_t)cap) || !ensure(&ctx->tr_tok, &ctx->tr_tok_cap, (size_t)tok_cap))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    if (!ctx->h_tr_scan && cudaMallocHost((void **)&ctx->h_tr_scan, sizeof(TextScan)) != cudaSuccess) {
        ctx->h_tr_scan = nullptr;
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    }
    TextScan *d_res = reinterpret_cast<TextScan *>(ctx->tr_scan);
    TextScan *h_res = reinterpret_cast<TextScan *>(ctx->h_tr_scan);
    long long *seg_count = ctx->tr_seg, *seg_ofs = ctx->tr_seg + nseg + 1;
    if ((e = cudaMemsetAsync(d_res, 0, sizeof(TextScan), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(&d_res->first_fail, 0xff, sizeof(unsigned long long), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(&d_res->last_byte, 0xff, sizeof(int), s)) != cudaSuccess)
        return mcg_cuda_fail(ctx, e);
    const long long nchunks = (L + TR_CHUNK - 1) / TR_CHUNK;
    cudaStream_t cs = nullptr;
    std::vector<cudaEvent_t> landed;
    auto cleanup = [&]() {
        for (auto ev : landed)
            if (ev) cudaEventDestroy(ev);
        if (cs) cudaStreamDestroy(cs);
    };
    mcg_status st = MCG_OK;
    auto fail = [&](cudaError_t err) {
        if (cs) cudaStreamSynchronize(cs);
        cleanup();
        return mcg_cuda_fail(ctx, err);
    };
    if (feed && nchunks > 0) {
        landed.assign((size_t)nchunks, nullptr);
        if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
        for (auto &ev : landed)
            if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
        // the copies wait for earlier work on s (a previous parse reads T)
        if ((e = cudaEventRecord(landed[0], s)) != cudaSuccess || (e = cudaStreamWaitEvent(cs, landed[0], 0)) != cudaSuccess)
            return fail(e);
    }
    auto chunk_bytes = [&](long long i) { return std::min<int64_t>(TR_CHUNK, L - i * TR_CHUNK); };
    auto parse_chunk = [&](long long i) -> cudaError_t {
        const long long s0 = i * (TR_CHUNK / TR_SEG), s1 = std::min(nseg, (i + 1) * (TR_CHUNK / TR_SEG));
        const int64_t La = feed ? std::min<int64_t>(L, (i + 2) * TR_CHUNK) : L;
        cudaError_t err;
        if (feed && (err = cudaStreamWaitEvent(s, landed[(size_t)std::min(i + 1, nchunks - 1)], 0)) != cudaSuccess)
            return err;
        const unsigned g = (unsigned)(s1 - s0);
        if (aligned)
            tr_count<true><<<g, TR_THREADS, 0, s>>>(T, L, La, s0, seg_count, d_res);
        else
            tr_count<false><<<g, TR_THREADS, 0, s>>>(T, L, La, s0, seg_count, d_res);
        tr_scan<<<1, TR_SCAN_THREADS, 0, s>>>(seg_count + s0, seg_ofs + s0, s1 - s0, d_res, i == nchunks - 1);
        if (aligned)
            tr_fields<true><<<g, TR_THREADS, 0, s>>>(T, L, La, s0, seg_ofs, d_res, ctx->tr_tok, tok_cap);
        else
            tr_fields<false><<<g, TR_THREADS, 0, s>>>(T, L, La, s0, seg_ofs, d_res, ctx->tr_tok, tok_cap);
        // the records completed by this chunk
        tr_window<<<nctas, TR_THREADS, 0, s>>>(ctx->tr_tok, d_res, win, ctx->tr_cta);
        tr_wscan<<<1, TR_SCAN_THREADS, 0, s>>>(ctx->tr_cta, ctx->tr_cta + nctas, nctas, ctx->tr_tok, T, L, d_res,
                                              i == nchunks - 1);
        tr_place<<<nctas, TR_THREADS, 0, s>>>(ctx->tr_tok, d_res, win, ctx->tr_cta + nctas, ctx->tr_arr);
        return cudaGetLastError();
    };
    for (long long i = 0; i < nchunks; ++i) {
        if (feed) {
            if ((st = (*feed)(i, i * TR_CHUNK, chunk_bytes(i), cs)) != MCG_OK) {
                cudaStreamSynchronize(cs);
                cleanup();
                return st;
            }
            if ((e = cudaEventRecord(landed[(size_t)i], cs)) != cudaSuccess) return fail(e);
        }
        if (i >= 1 && (e = parse_chunk(i - 1)) != cudaSuccess) return fail(e);
    }
    if (nchunks > 0 && (e = parse_chunk(nchunks - 1)) != cudaSuccess) return fail(e);
    {
        const unsigned t = (unsigned)((dim + 31) / 32);
        tr_transpose<<<dim3(t, t, (unsigned)dim), dim3(32, 8), 0, s>>>(ctx->tr_arr, d_res, win.dim, vol);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpyAsync(h_res, d_res, sizeof(TextScan), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(e);
    if (cs && (e = cudaStreamSynchronize(cs)) != cudaSuccess) return fail(e);
    cleanup();
    const TextScan r = *h_res;
    if (r.incomplete & 2) return MCG_ERR_STATE;  // the field bound was violated: a defect, not an input error
    if (r.incomplete) {
        // a field longer than a chunk: everything is resident now
        return text_run<Feed>(ctx, T, L, nullptr, loop_runs, dim, origin, vol, info, s);
    }
    long long stored = 0;
    int filled = 0;
    st = text_finish(ctx, r, loop_runs, win, vol, &stored, &filled, s);
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

struct NoFeed {
    mcg_status operator()(long long, int64_t, int64_t, cudaStream_t) const { return MCG_OK; }
};

constexpr int TR_READERS = 16;

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

// File chunks: host threads pread a chunk into one of two pinned staging
// buffers, then one copy moves it to the device; the buffer is reused two
// chunks later, once that copy has finished.
struct FileFeed {
    mcg_context *ctx;
    int fd;
    int64_t start;  // file offset of text byte 0
    uint8_t *dst;   // device text
    cudaEvent_t copied[2];
    mcg_status operator()(long long i, int64_t off, int64_t n, cudaStream_t cs) const {
        uint8_t *buf = ctx->h_tr_stage + (size_t)(i & 1) * TR_CHUNK;
        if (i >= 2 && cudaEventSynchronize(copied[i & 1]) != cudaSuccess) return mcg_cuda_fail(ctx, cudaGetLastError());
        const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
        const int nt = (int)std::min<int64_t>(std::min(TR_READERS, hw), (n + (1 << 20) - 1) >> 20);
        std::atomic<int> ok{1};
        std::vector<std::thread> pool;
        const int64_t part = (n + nt - 1) / nt;
        for (int t = 0; t < nt; ++t) {
            const int64_t a = t * part, b = std::min(n, a + part);
            if (a >= b) break;
            pool.emplace_back([&, a, b]() {
                if (!pread_all(fd, buf + a, b - a, start + off + a)) ok.store(0);
            });
        }
        for (auto &th : pool) th.join();
        if (!ok.load()) return MCG_ERR_IO;
        cudaError_t e = cudaMemcpyAsync(dst + off, buf, (size_t)n, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaEventRecord(copied[i & 1], cs);
        return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
    }
};

struct HostFeed {
    mcg_context *ctx;
    const uint8_t *src;
    uint8_t *dst;
    mcg_status operator()(long long, int64_t off, int64_t n, cudaStream_t cs) const {
        // the driver moves pageable host memory at about the pinned rate on
        // this platform: no staging copy
        const cudaError_t e = cudaMemcpyAsync(dst + off, src + off, (size_t)n, cudaMemcpyHostToDevice, cs);
        return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(ctx, e);
    }
};

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" mcg_status mcg_text_records_parse(mcg_context *ctx, const void *text, int64_t len, int32_t dim,
                                             const int32_t origin[3], void *vol, mcg_text_info *info,
                                             mcg_stream_t stream) {
    if (!ctx || len < 0 || (len > 0 && !text) || !text_args_ok(dim, origin, vol)) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    return text_run<NoFeed>(ctx, static_cast<const uint8_t *>(text), len, nullptr, true, dim, origin,
                            static_cast<uint32_t *>(vol), info, (cudaStream_t)stream);
}

extern "C" mcg_status mcg_text_records_load(mcg_context *ctx, const void *text, int64_t len, int32_t dim,
                                            const int32_t origin[3], void *vol, mcg_text_info *info,
                                            mcg_stream_t stream) {
    if (!ctx || len < 0 || (len > 0 && !text) || !text_args_ok(dim, origin, vol)) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    if (!ensure(&ctx->tr_text, &ctx->tr_text_cap, (size_t)len + 16)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    const HostFeed feed{ctx, static_cast<const uint8_t *>(text), ctx->tr_text};
    return text_run(ctx, ctx->tr_text, len, &feed, true, dim, origin, static_cast<uint32_t *>(vol), info,
                    (cudaStream_t)stream);
}

extern "C" mcg_status mcg_text_records_load_file(mcg_context *ctx, const char *path, int64_t tail_bytes, int32_t dim,
                                                 const int32_t origin[3], void *vol, mcg_text_info *info,
                                                 mcg_stream_t stream) {
    if (!ctx || !path || !text_args_ok(dim, origin, vol)) return MCG_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
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
    FileFeed feed{ctx, fd, start, nullptr, {nullptr, nullptr}};
    mcg_status st = MCG_OK;
    if (!ensure(&ctx->tr_text, &ctx->tr_text_cap, (size_t)L + 16)) st = mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    if (st == MCG_OK && !ctx->h_tr_stage) {
        if (cudaMallocHost((void **)&ctx->h_tr_stage, 2 * (size_t)TR_CHUNK) != cudaSuccess) {
            ctx->h_tr_stage = nullptr;
            st = mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
        }
    }
    for (int b = 0; b < 2 && st == MCG_OK; ++b)
        if ((e = cudaEventCreateWithFlags(&feed.copied[b], cudaEventDisableTiming)) != cudaSuccess)
            st = mcg_cuda_fail(ctx, e);
    if (st == MCG_OK) {
        feed.dst = ctx->tr_text;
        st = text_run(ctx, ctx->tr_text, L, &feed, loop_runs, dim, origin, static_cast<uint32_t *>(vol), info,
                      (cudaStream_t)stream);
    }
    for (int b = 0; b < 2; ++b)
        if (feed.copied[b]) cudaEventDestroy(feed.copied[b]);
    close(fd);
    return st;
}
