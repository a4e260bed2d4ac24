// Run-length encoding of a device volume on the GPU (the file format of
// cu_kinect_fusion_v1.cu:1303-1600, described in rle.cpp).
//
// The reference encodes slice after slice on one host thread
// (cu_voxel_run_length_encode_slice, :1367-1417).  Here one CTA encodes one
// z-slice, sweeping it in chunks of 4096 voxels (16 per thread) and carrying
// the run state from chunk to chunk:
//   - voxel i starts a run when i = 0 or it differs from voxel i-1 (tsdf
//     only in the reference format, the whole voxel in the lossless one);
//   - a record starts at every run start and every 16383 voxels into a run
//     (the 14-bit count), as the sequential encoder splits long runs;
//   - a record is 2 bytes (kinds 1/2: +-32766 with, in the lossless format,
//     w = 0) or 6 bytes (kind 3: header + the record's first voxel).
// Pass 1 (count) sums each slice's record bytes; the host turns them into
// slice offsets; pass 2 (write) emits the records into a device image, each
// record's count being the distance to the next record start (the last one
// of a chunk waits for the next chunk).  The image then crosses to the host
// in one copy.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>
#include <vector>

#include "mcg_internal.h"
#include "tma.cuh"

namespace mcg {
namespace {

constexpr int RT = 256;            // threads per CTA
constexpr int RV = 16;             // voxels per thread per chunk
constexpr int RCHUNK = RT * RV;    // 4096
constexpr unsigned kMaxRun = 0x3fffu;

__device__ __forceinline__ bool same_voxel(uint32_t a, uint32_t b, bool lossless) {
    return lossless ? a == b : ((a ^ b) & 0xffffu) == 0u;
}

// record kind of a record whose first voxel is v (put_run in rle.cpp)
__device__ __forceinline__ unsigned record_kind(uint32_t v, bool lossless) {
    const int16_t t = (int16_t)(v & 0xffffu);
    const bool w0 = (v >> 16) == 0u;
    if (t == (int16_t)kMaxTsdf && (!lossless || w0)) return 1u;
    if (t == (int16_t)-kMaxTsdf && (!lossless || w0)) return 2u;
    return 3u;
}

// write pass: the chunk's record starts
struct RleSmem {
    uint32_t pos[RCHUNK];   // record starts of the chunk (slice index)
    uint32_t vox[RCHUNK];   // their first voxels
    uint32_t boff[RCHUNK];  // their byte offsets from the chunk's first record
    uint32_t wn[RT / 32], wb[RT / 32];
    int wr[RT / 32];
};

// count pass: two chunk buffers, the next chunk's asynchronous copies in
// flight while the current one is scanned
struct RleCountSmem {
    alignas(16) uint32_t stage[2][RCHUNK];
    uint32_t wn[RT / 32], wb[RT / 32];
    int wr[RT / 32];
};

template <bool WRITE>
using RleS = typename std::conditional<WRITE, RleSmem, RleCountSmem>::type;

// block-wide exclusive sums of two values; totals returned through refs
template <class SM>
__device__ __forceinline__ void scan2(SM &S, uint32_t a, uint32_t b, uint32_t &ea, uint32_t &eb, uint32_t &ta,
                                      uint32_t &tb) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = a, y = b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t p = __shfl_up_sync(0xffffffffu, x, o), q = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) {
            x += p;
            y += q;
        }
    }
    if (lane == 31) {
        S.wn[warp] = x;
        S.wb[warp] = y;
    }
    __syncthreads();
    uint32_t ba = 0, bb = 0, sa = 0, sb = 0;
#pragma unroll
    for (int w = 0; w < RT / 32; ++w) {
        if (w < warp) {
            ba += S.wn[w];
            bb += S.wb[w];
        }
        sa += S.wn[w];
        sb += S.wb[w];
    }
    __syncthreads();
    ea = ba + x - a;
    eb = bb + y - b;
    ta = sa;
    tb = sb;
}

// block-wide inclusive max-scan of a signed value (run starts, -1 = none)
template <class SM>
__device__ __forceinline__ int scan_max(SM &S, int v, int carry) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int p = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o && p > x) x = p;
    }
    if (lane == 31) S.wr[warp] = x;
    __syncthreads();
    int m = carry;
#pragma unroll
    for (int w = 0; w < RT / 32; ++w)
        if (w < warp && S.wr[w] > m) m = S.wr[w];
    __syncthreads();
    return x > m ? x : m;
}

__device__ __forceinline__ void put16(uint8_t *img, unsigned long long off, unsigned v) {
    *reinterpret_cast<uint16_t *>(img + off) = (uint16_t)v;
}

// emit one record at byte offset off
__device__ __forceinline__ void emit(uint8_t *img, unsigned long long off, uint32_t v, unsigned count,
                                     bool lossless) {
    const unsigned kind = record_kind(v, lossless);
    put16(img, off, count | (kind << 14));
    if (kind == 3u) {
        put16(img, off + 2, v & 0xffffu);
        put16(img, off + 4, v >> 16);
    }
}

// count pass: chunk starting at c0 into buffer buf by asynchronous copies
// (16 bytes at a time when vec: the slice is 16-byte aligned), zero past
// the slice; one commit group per call
__device__ __forceinline__ void rle_issue_chunk(RleCountSmem &S, const uint32_t *__restrict__ sl, int xy, int c0,
                                                int buf, bool vec) {
    const int i0 = c0 + threadIdx.x * RV;
    uint32_t *dst = S.stage[buf] + threadIdx.x * RV;
    if (vec && i0 + RV <= xy) {
#pragma unroll
        for (int q = 0; q < RV / 4; ++q) cp_async_16(dst + 4 * q, sl + i0 + 4 * q);
    } else {
#pragma unroll
        for (int j = 0; j < RV; ++j) {
            const bool in = i0 + j < xy;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst + j)),
                         "l"(in ? sl + i0 + j : sl), "r"(in ? 4u : 0u)
                         : "memory");
        }
    }
    cp_async_commit();
}

// WRITE = false: slice_bytes[z] = record bytes of slice z.  WRITE = true:
// slice z goes to img + slice_off[z]: its byte count (uint32) then records.
// vec: the slices are 16-byte aligned (count pass only).
template <bool WRITE>
__global__ void __launch_bounds__(RT) rle_encode_kernel(const uint32_t *__restrict__ vol, int xy, int lossless_i,
                                                        unsigned long long *__restrict__ slice_bytes,
                                                        const unsigned long long *__restrict__ slice_off,
                                                        uint8_t *__restrict__ img, int vec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RleS<WRITE> &S = *reinterpret_cast<RleS<WRITE> *>(smem_raw);
    const bool lossless = lossless_i != 0;
    const int z = blockIdx.x;
    const uint32_t *sl = vol + (long long)z * xy;
    const int tid = threadIdx.x;
    uint8_t *out = WRITE ? img + slice_off[z] + 4 : nullptr;
    uint32_t prev = 0;            // voxel before the chunk
    int rs_carry = -1;            // run start in force at the chunk's start
    unsigned long long bytes = 0; // bytes of the records started before the chunk
    int pend = -1;                // record open at the chunk's start (WRITE)
    uint32_t pend_v = 0;
    unsigned long long pend_off = 0;
    // slice indices fit 32 bits: the host rejects slices whose image could
    // pass the format's 32-bit byte count
    if constexpr (!WRITE) rle_issue_chunk(S, sl, xy, 0, 0, vec != 0);
    int buf = 0;
    for (int c0 = 0; c0 < xy; c0 += RCHUNK, buf ^= 1) {
        const int i0 = c0 + tid * RV;
        uint32_t v[RV];
        uint32_t left;
        if constexpr (WRITE) {
#pragma unroll
            for (int j = 0; j < RV; ++j) v[j] = i0 + j < xy ? __ldg(sl + i0 + j) : 0u;
            // previous voxel of each thread's first voxel
            left = __shfl_up_sync(0xffffffffu, v[RV - 1], 1);
            if ((tid & 31) == 0) {
                if (tid == 0) left = prev;
                else left = i0 - 1 < xy ? __ldg(sl + i0 - 1) : 0u;
            }
        } else {
            // the next chunk's copies go out first (its buffer was last read
            // before the barriers of the previous chunk), then this chunk's land
            if (c0 + RCHUNK < xy) rle_issue_chunk(S, sl, xy, c0 + RCHUNK, buf ^ 1, vec != 0);
            else cp_async_commit();
            cp_async_wait_group<1>();
            __syncthreads();
            const uint4 *src = reinterpret_cast<const uint4 *>(S.stage[buf] + tid * RV);
#pragma unroll
            for (int q = 0; q < RV / 4; ++q) {
                const uint4 w = src[q];
                v[4 * q] = w.x;
                v[4 * q + 1] = w.y;
                v[4 * q + 2] = w.z;
                v[4 * q + 3] = w.w;
            }
            left = tid == 0 ? prev : S.stage[buf][tid * RV - 1];
        }
        // run starts (local inclusive max), then the block max-scan
        int rs_loc = -1;
        uint32_t chg = 0;
#pragma unroll
        for (int j = 0; j < RV; ++j) {
            const int i = i0 + j;
            const uint32_t pv = j == 0 ? left : v[j - 1];
            const bool c = i < xy && (i == 0 || !same_voxel(v[j], pv, lossless));
            if (c) {
                chg |= 1u << j;
                rs_loc = i;
            }
        }
        const int rs_incl = scan_max(S, rs_loc, rs_carry);
        // run start in force before this thread's first voxel: the exclusive value
        int rs = __shfl_up_sync(0xffffffffu, rs_incl, 1);
        if ((tid & 31) == 0) {
            // exclusive across warps: the block max of everything before this warp
            rs = rs_carry;
            for (int w = 0; w < (tid >> 5); ++w)
                if (S.wr[w] > rs) rs = S.wr[w];
        }
        // record starts and their bytes; d = voxels since the run start, mod 16383
        uint32_t rec = 0, nrec = 0, nb = 0;
        unsigned d = (unsigned)(i0 - rs) % kMaxRun;
#pragma unroll
        for (int j = 0; j < RV; ++j) {
            const int i = i0 + j;
            if (i >= xy) break;
            if (chg & (1u << j)) d = 0;
            if (d == 0) {
                rec |= 1u << j;
                ++nrec;
                nb += record_kind(v[j], lossless) == 3u ? 6u : 2u;
            }
            d = d + 1 == kMaxRun ? 0u : d + 1;
        }
        uint32_t er, eb, tr, tb;
        scan2(S, nrec, nb, er, eb, tr, tb);
        if constexpr (WRITE) {
            uint32_t k = er, b = eb;
#pragma unroll
            for (int j = 0; j < RV; ++j) {
                if (!(rec & (1u << j))) continue;
                S.pos[k] = (uint32_t)(i0 + j);
                S.vox[k] = v[j];
                S.boff[k] = b;
                b += record_kind(v[j], lossless) == 3u ? 6u : 2u;
                ++k;
            }
            __syncthreads();
            if (tr > 0) {
                if (tid == 0 && pend >= 0) emit(out, pend_off, pend_v, (unsigned)((int)S.pos[0] - pend), lossless);
                for (uint32_t q = tid; q + 1 < tr; q += RT)
                    emit(out, bytes + S.boff[q], S.vox[q], S.pos[q + 1] - S.pos[q], lossless);
                pend = (int)S.pos[tr - 1];
                pend_v = S.vox[tr - 1];
                pend_off = bytes + S.boff[tr - 1];
            }
            __syncthreads();  // pos / vox / boff are rewritten by the next chunk
        }
        (void)buf;
        bytes += tb;
        // carries: the run start in force and the voxel at the chunk's end
        if (tid == RT - 1) {
            S.wr[0] = rs_incl;
            S.wn[0] = v[RV - 1];
        }
        __syncthreads();
        rs_carry = S.wr[0];
        prev = S.wn[0];
        __syncthreads();
    }
    if (WRITE) {
        if (tid == 0) {
            if (pend >= 0) emit(out, pend_off, pend_v, (unsigned)(xy - pend), lossless);
            const uint32_t n32 = (uint32_t)bytes;
            uint8_t *cnt = img + slice_off[z];
            put16(cnt, 0, n32 & 0xffffu);
            put16(cnt, 2, n32 >> 16);
        }
    } else if (tid == 0) {
        slice_bytes[z] = bytes;
    }
}

const char kTagRef[16] = "VOLUME_TSDF_RGB";
const char kTagLossless[16] = "VOLUME_TSDF_W32";

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" mcg_status mcg_rle_encode(mcg_context *ctx, const void *vol, int32_t nx, int32_t ny, int32_t nz,
                                         float min_t, float max_t, float grid_s, int32_t lossless, uint8_t *image,
                                         int64_t capacity, int64_t *size, mcg_stream_t stream) {
    // image == NULL with capacity == 0 asks for the image size only
    const bool query = !image && capacity == 0;
    if (!ctx || !vol || (!image && !query) || !size || nx <= 0 || ny <= 0 || nz <= 0) return MCG_ERR_INVALID_ARG;
    *size = 0;
    const long long xy = (long long)nx * ny;
    // record counts are 14-bit and slice byte counts 32-bit (the file format)
    if (6 * xy > 0xffffffffll) return MCG_ERR_TOO_LARGE;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    if (!ensure(&ctx->rle_slices, &ctx->rle_slices_cap, (size_t)2 * nz))
        return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    unsigned long long *d_bytes = ctx->rle_slices, *d_off = ctx->rle_slices + nz;
    const size_t smem = sizeof(RleSmem), csmem = sizeof(RleCountSmem);
    cudaFuncSetAttribute(rle_encode_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem);
    cudaFuncSetAttribute(rle_encode_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int vec = ((reinterpret_cast<uintptr_t>(vol) & 15u) == 0 && xy % 4 == 0) ? 1 : 0;
    rle_encode_kernel<false><<<nz, RT, csmem, s>>>(static_cast<const uint32_t *>(vol), (int)xy, lossless ? 1 : 0,
                                                   d_bytes, nullptr, nullptr, vec);
    e = cudaGetLastError();
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    std::vector<unsigned long long> bytes(nz), off(nz);
    e = cudaMemcpyAsync(bytes.data(), d_bytes, sizeof(unsigned long long) * nz, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    unsigned long long o = 40;
    for (int z = 0; z < nz; ++z) {
        off[z] = o;
        o += 4 + bytes[z];
    }
    if (query || (long long)o > capacity) {
        *size = (int64_t)o;
        return query ? MCG_OK : MCG_ERR_CAPACITY;
    }
    if (!ensure(&ctx->rle_image, &ctx->rle_image_cap, (size_t)o)) return mcg_cuda_fail(ctx, cudaErrorMemoryAllocation);
    e = cudaMemcpyAsync(d_off, off.data(), sizeof(unsigned long long) * nz, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    rle_encode_kernel<true><<<nz, RT, smem, s>>>(static_cast<const uint32_t *>(vol), (int)xy, lossless ? 1 : 0, nullptr,
                                                 d_off, ctx->rle_image, 0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    // header (:1303-1310), then the slices
    memcpy(image, lossless ? kTagLossless : kTagRef, 16);
    const int32_t dims[3] = {nx, ny, nz};
    memcpy(image + 16, dims, 12);
    memcpy(image + 28, &min_t, 4);
    memcpy(image + 32, &max_t, 4);
    memcpy(image + 36, &grid_s, 4);
    e = cudaMemcpyAsync(image + 40, ctx->rle_image + 40, o - 40, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return mcg_cuda_fail(ctx, e);
    *size = (int64_t)o;
    return MCG_OK;
}
