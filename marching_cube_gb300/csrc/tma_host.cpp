// Tensor-map encoding for the TMA tile loads.  cuTensorMapEncodeTiled is a
// driver function; it is fetched once through the runtime's driver entry
// point so the library does not link libcuda directly.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "tma.cuh"

namespace mcg {
namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

EncodeTiledFn g_encode = nullptr;
std::once_flag g_once;

void load_encode() {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_encode = reinterpret_cast<EncodeTiledFn>(fn);
    cudaGetLastError();
}

}  // namespace

bool encode_volume_map(CUtensorMap *map, const void *data, int nx, int ny, int nz, int elem_bytes, int box_x,
                       int box_y, int box_z) {
    std::call_once(g_once, load_encode);
    if (!g_encode || !data) return false;
    if (elem_bytes != 4 && elem_bytes != 8) return false;
    if ((reinterpret_cast<uintptr_t>(data) & 15) != 0) return false;
    const uint64_t row = (uint64_t)nx * elem_bytes;
    if (row % 16 != 0) return false;  // strides must be multiples of 16 bytes
    if ((uint64_t)box_x * elem_bytes % 16 != 0) return false;
    if (box_x > 256 || box_y > 256 || box_z > 256) return false;
    // smaller volumes use the plain-load path: keep every box inside the tensor extent
    if (nx < box_x || ny < box_y || nz < box_z) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {row, row * (uint64_t)ny};
    const cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, (cuuint32_t)box_z};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType dt = elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_UINT64;
    // out-of-bounds elements are filled with zeros: {tsdf 0, w 0} is a
    // weight-zero voxel, which no emitting cube ever contains
    const CUresult r = g_encode(map, dt, 3, const_cast<void *>(data), dims, strides, box, estr,
                                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace mcg
