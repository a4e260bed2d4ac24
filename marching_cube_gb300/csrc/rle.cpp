// Run-length volume codec (cu_kinect_fusion_v1.cu:1303-1600).
//
// File layout (kept byte-identical to the reference):
//   16-byte format tag "VOLUME_TSDF_RGB\0" (cu_kinect_fusion_v1.h:40)
//   int32 size.x, size.y, size.z; float min_t, max_t, grid_s     (:1303-1310)
//   per z-slice: uint32 byte count, then that many record bytes     (:1345-1351)
// Records (:1362-1365) are little-endian 16-bit words, run length n in bits
// 0-13 (1..16383) and kind v in bits 14-15: v=1 run of {+32766, w=0},
// v=2 run of {-32766, w=0}, v=3 run of the literal voxel that follows
// (int16 tsdf, uint16 w).  The reference encoder compares tsdf only, so the
// weights inside a run are those of its first voxel; the lossless variant
// (tag "VOLUME_TSDF_W32\0") compares whole voxels and uses kinds 1/2 only
// for w == 0.
//
// The reference codes slices one after another on one host thread and copies
// every slice separately.  Here a device volume is encoded by the GPU
// (rle_gpu.cu) and images are decoded by the GPU (rle_decode.cu); host
// volumes are encoded, and images decoded to host memory, slice-parallel on
// all host threads.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "mcg_internal.h"

namespace mcg {
namespace {

const char kTagRef[16] = "VOLUME_TSDF_RGB";
const char kTagLossless[16] = "VOLUME_TSDF_W32";

struct HVox {
    int16_t tsdf;
    uint16_t w;
};

inline void put16(uint8_t *b, unsigned v) {
    b[0] = (uint8_t)(v & 0xff);
    b[1] = (uint8_t)(v >> 8);
}

inline int64_t put_run(uint8_t *b, HVox first, unsigned n, bool lossless) {
    bool empty = first.tsdf == kMaxTsdf, null = first.tsdf == -kMaxTsdf;
    if (lossless && first.w != 0) empty = null = false;
    if (empty) { put16(b, n | (1u << 14)); return 2; }
    if (null) { put16(b, n | (2u << 14)); return 2; }
    put16(b, n | (3u << 14));
    put16(b + 2, (uint16_t)first.tsdf);
    put16(b + 4, first.w);
    return 6;
}

// cu_voxel_run_length_encode_slice (:1367-1417)
int64_t encode_slice(const HVox *s, int64_t n, bool lossless, uint8_t *buf) {
    if (n <= 0) return 0;
    int64_t o = 0;
    HVox old = s[0];
    unsigned count = 0;
    for (int64_t i = 0; i < n; ++i) {
        const HVox cur = s[i];
        const bool same = cur.tsdf == old.tsdf && (!lossless || cur.w == old.w);
        if (same) {
            if (++count > 0x3fff) --count;
            else continue;
        }
        o += put_run(buf + o, old, count, lossless);
        count = 1;
        old = cur;
    }
    o += put_run(buf + o, old, count, lossless);
    return o;
}

// cu_voxel_run_length_decode_slice (:1419-1447) with bounds checks: zero
// length records, runs past the slice and truncated streams are errors.
bool decode_slice(const uint8_t *buf, int64_t nbytes, HVox *out, int64_t n) {
    int64_t p = 0, o = 0;
    while (o < n) {
        if (p + 2 > nbytes) return false;
        const unsigned r = (unsigned)buf[p] | ((unsigned)buf[p + 1] << 8);
        p += 2;
        const unsigned cnt = r & 0x3fffu, v = r >> 14;
        HVox val;
        if (v == 1) val = HVox{(int16_t)kMaxTsdf, 0};
        else if (v == 2) val = HVox{(int16_t)-kMaxTsdf, 0};
        else {
            if (p + 4 > nbytes) return false;
            val.tsdf = (int16_t)((unsigned)buf[p] | ((unsigned)buf[p + 1] << 8));
            val.w = (uint16_t)((unsigned)buf[p + 2] | ((unsigned)buf[p + 3] << 8));
            p += 4;
        }
        if (cnt == 0 || o + (int64_t)cnt > n) return false;
        std::fill(out + o, out + o + cnt, val);
        o += cnt;
    }
    return true;
}

int host_threads() {
    unsigned n = std::thread::hardware_concurrency();
    return n ? (int)std::min(n, 64u) : 1;
}

template <class F>
void parallel_for(int n, F f) {
    const int nt = std::min(host_threads(), n);
    if (nt <= 1) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&]() {
            for (int i = next++; i < n; i = next++) f(i);
        });
    for (auto &x : th) x.join();
}

}  // namespace
}  // namespace mcg

using namespace mcg;

extern "C" {

int64_t mcg_rle_bound(int32_t nx, int32_t ny, int32_t nz) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
    // header + per slice (count + worst case one 6-byte literal per voxel)
    return 40 + (int64_t)nz * (4 + 6 * (int64_t)nx * ny);
}

mcg_status mcg_rle_header(const uint8_t *image, int64_t size, int32_t dims[3], float params[3]) {
    if (!image || !dims || !params) return MCG_ERR_INVALID_ARG;
    if (size < 40) return MCG_ERR_FORMAT;
    if (memcmp(image, kTagRef, 16) != 0 && memcmp(image, kTagLossless, 16) != 0) return MCG_ERR_FORMAT;
    memcpy(dims, image + 16, 12);
    memcpy(params, image + 28, 12);
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return MCG_ERR_FORMAT;
    return MCG_OK;
}

mcg_status mcg_rle_encode_host(const void *vol, int32_t nx, int32_t ny, int32_t nz, float min_t, float max_t,
                               float grid_s, int32_t lossless, uint8_t *image, int64_t capacity, int64_t *size) {
    if (!vol || !image || !size || nx <= 0 || ny <= 0 || nz <= 0) return MCG_ERR_INVALID_ARG;
    *size = 0;
    if (capacity < 40) return MCG_ERR_CAPACITY;
    memcpy(image, lossless ? kTagLossless : kTagRef, 16);
    const int32_t dims[3] = {nx, ny, nz};
    memcpy(image + 16, dims, 12);
    memcpy(image + 28, &min_t, 4);
    memcpy(image + 32, &max_t, 4);
    memcpy(image + 36, &grid_s, 4);
    const int64_t xy = (int64_t)nx * ny;
    const HVox *v = static_cast<const HVox *>(vol);
    // encode slices in parallel into private buffers, then concatenate in order
    const int batch = std::max(1, std::min(nz, 4 * host_threads()));
    std::vector<std::vector<uint8_t>> enc(batch);
    std::vector<int64_t> sz(batch);
    int64_t o = 40;
    for (int z0 = 0; z0 < nz; z0 += batch) {
        const int ns = std::min(batch, nz - z0);
        parallel_for(ns, [&](int i) {
            enc[i].resize((size_t)(6 * xy + 16));
            sz[i] = encode_slice(v + (int64_t)(z0 + i) * xy, xy, lossless != 0, enc[i].data());
        });
        for (int i = 0; i < ns; ++i) {
            if (o + 4 + sz[i] > capacity) return MCG_ERR_CAPACITY;
            const uint32_t s32 = (uint32_t)sz[i];
            memcpy(image + o, &s32, 4);
            memcpy(image + o + 4, enc[i].data(), (size_t)sz[i]);
            o += 4 + sz[i];
        }
    }
    *size = o;
    return MCG_OK;
}

mcg_status mcg_rle_decode_host(const uint8_t *image, int64_t size, void *vol, int64_t capacity_voxels) {
    if (!image || !vol) return MCG_ERR_INVALID_ARG;
    int32_t dims[3];
    float params[3];
    mcg_status st = mcg_rle_header(image, size, dims, params);
    if (st != MCG_OK) return st;
    const int64_t xy = (int64_t)dims[0] * dims[1];
    if (xy * dims[2] > capacity_voxels) return MCG_ERR_CAPACITY;
    std::vector<int64_t> off(dims[2]), len(dims[2]);
    int64_t p = 40;
    for (int z = 0; z < dims[2]; ++z) {
        if (p + 4 > size) return MCG_ERR_FORMAT;
        uint32_t s32;
        memcpy(&s32, image + p, 4);
        p += 4;
        if (p + (int64_t)s32 > size) return MCG_ERR_FORMAT;
        off[z] = p;
        len[z] = s32;
        p += s32;
    }
    HVox *v = static_cast<HVox *>(vol);
    std::atomic<bool> bad(false);
    parallel_for(dims[2], [&](int z) {
        if (!decode_slice(image + off[z], len[z], v + (int64_t)z * xy, xy)) bad = true;
    });
    return bad ? MCG_ERR_FORMAT : MCG_OK;
}

}  // extern "C"
