// Harness around the reference's live marching-cubes and surface-normal code,
// compiled for the host by oracle/ref/build_ref.py.  TEST INFRASTRUCTURE
// ONLY: a second checker of the oracle, built from the reference's own source.
//
// Included from the reference (by line range, see build_ref.py):
//   cu_marching_cubes_v1.cu:31-33    texture references triTex / numVertsTex
//   cu_marching_cubes_v1.cu:49-95    CubeIndexEstimator (readTsdf, computeCubeIndex)
//   cu_marching_cubes_v1.cu:228-370  TrianglesGenerator (getNodeCoo, vertex_interp,
//                                    operator(), store_point) and its kernel
//   cu_marching_cubes_v1.cu:469-1028 edgeTable, triTable, numVertsTable
//   cu_kinect_fusion_v1.cu:3146-3242 _d_voxel_extract_surface_normal,
//                                    d_voxel_extract_surface_normal(s)
// and, whole, the reference headers cu_vector_functions.h, structure.h,
// cu_memory.hpp (ptr_step) and cu_kinect_fusion_v1.h (d_unpack_tsdf,
// CU_VOXEL_MAX_TSDF).
//
// What the harness itself does, in place of code that cannot run here:
//  * the occupied-voxel pass (cu_marching_cubes_v1.cu:97-206) is warp-vote
//    code; the harness visits the cubes x < nx-1, y < ny-1, z < nz-1 in
//    linear order (:126-129), asks the reference's computeCubeIndex for each
//    and keeps those with (cubeindex == 0 || cubeindex == 255) ? 0 :
//    numVertsTable[cubeindex] > 0 vertices (:136-140).  The list is therefore
//    in linear order -- the oracle's canonical order -- where the GPU
//    reference's depends on the order in which warps win an atomicAdd;
//  * thrust::exclusive_scan of the counts (:208-225) is a plain loop;
//  * the kernels run one thread at a time (oracle/ref/shim/ref_device.h).
//
// Out-of-range reads.  The reference reads outside the volume where a vertex
// voxel or a normal sample leaves it (UB there).  The harness runs the code
// on a copy of the volume with two slices of padding on each side: zeros
// for the generator (so a voxel read outside [0, N) gives tsdf = w = 0 and a
// ver_voxel write lands in the padding) and the +32766 sentinel for the
// normals (so a sample outside [0, N) gives the zero normal) -- the
// behaviour the oracle and the CUDA library define for those cases.
#include "cu_vector_functions.h"
#include "cu_geometry_functions.h"
#include "structure.h"
#include "cu_memory.hpp"
#include "cu_kinect_fusion_v1.h"

#include <vector>

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;

#include "mc_textures.inc"
#include "mc_cube_index.inc"
#include "mc_generator.inc"
#include "mc_tables.inc"
#include "kf_normals.inc"

namespace {

void bind_tables() {
    triTex.table = &triTable[0][0];
    numVertsTex.table = numVertsTable;
}

struct Padded {
    std::vector<cu_voxel_t> buf;
    long long pad;
    cu_voxel_t *data() { return buf.data() + pad; }
};

Padded padded(const cu_voxel_t *vol, int nx, int ny, int nz, short fill_tsdf) {
    Padded p;
    const long long n = (long long)nx * ny * nz;
    p.pad = 2ll * nx * ny + 2ll * nx + 64;
    cu_voxel_t f;
    f.tsdf = fill_tsdf;
    f.w = 0;
    p.buf.assign((size_t)(n + 2 * p.pad), f);
    std::memcpy(p.buf.data() + p.pad, vol, sizeof(cu_voxel_t) * (size_t)n);
    return p;
}

void set_thread(long long i, int block) {
    blockDim = dim3(block, 1, 1);
    blockIdx = make_uint3((unsigned)(i / block), 0, 0);
    threadIdx = make_uint3((unsigned)(i % block), 0, 0);
}

// occupied cubes in linear order and their vertex counts
void occupied(const cu_voxel_t *data, int nx, int ny, int nz, std::vector<int> &ids, std::vector<int> &counts) {
    bind_tables();
    CubeIndexEstimator ce;
    ce.volume = ptr_step<cu_voxel_t>(const_cast<cu_voxel_t *>(data), sizeof(cu_voxel_t) * (size_t)nx);
    for (int z = 0; z < nz - 1; ++z)
        for (int y = 0; y < ny - 1; ++y)
            for (int x = 0; x < nx - 1; ++x) {
                float field[8];
                const int ci = ce.computeCubeIndex(ny, x, y, z, field);
                const int nv = (ci == 0 || ci == 255) ? 0 : tex1Dfetch(numVertsTex, ci);
                if (nv > 0) {
                    ids.push_back(ny * nx * z + nx * y + x);
                    counts.push_back(nv);
                }
            }
}

}  // namespace

extern "C" {

// cube index of every cube (x < nx-1, y < ny-1, z < nz-1), [z][y][x]
void ref_mc_cube_index(const cu_voxel_t *vol, int nx, int ny, int nz, unsigned char *ci) {
    CubeIndexEstimator ce;
    ce.volume = ptr_step<cu_voxel_t>(const_cast<cu_voxel_t *>(vol), sizeof(cu_voxel_t) * (size_t)nx);
    long long k = 0;
    for (int z = 0; z < nz - 1; ++z)
        for (int y = 0; y < ny - 1; ++y)
            for (int x = 0; x < nx - 1; ++x) {
                float field[8];
                ci[k++] = (unsigned char)ce.computeCubeIndex(ny, x, y, z, field);
            }
}

// occupied cubes and soup vertices
long long ref_mc_count(const cu_voxel_t *vol, int nx, int ny, int nz, long long *n_occupied) {
    std::vector<int> ids, counts;
    occupied(vol, nx, ny, nz, ids, counts);
    long long total = 0;
    for (int c : counts) total += c;
    *n_occupied = (long long)ids.size();
    return total;
}

// The whole MarchingCubes::run (cu_marching_cubes_v1.cu:416-467) plus the
// normals pass of its driver (cu_kinect_fusion_v1.cu:3236-3242): soup,
// vertexindex_to_voxel, ver_voxel (zeroed first, as :438) and normals, in
// the order of the occupied list (linear cube order, table slot order).
// Returns the vertex count, or -count when cap is too small (nothing written).
long long ref_mc_extract(const cu_voxel_t *vol, int nx, int ny, int nz, float cell, vertex_voxel *out,
                         int3 *vi2vox, short *ver_voxel, float3 *normals, long long cap) {
    const long long n = (long long)nx * ny * nz;
    Padded zp = padded(vol, nx, ny, nz, 0);
    std::vector<int> ids, counts;
    occupied(zp.data(), nx, ny, nz, ids, counts);
    std::vector<int> offs(ids.size());
    long long total = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
        offs[i] = (int)total;
        total += counts[i];
    }
    if (total > cap) return -total;
    std::vector<short> vv((size_t)(n + 2 * zp.pad), 0);
    std::vector<int3> v2v((size_t)(total > 0 ? total : 1));
    TrianglesGenerator tg;
    tg.volume = ptr_step<cu_voxel_t>(zp.data(), sizeof(cu_voxel_t) * (size_t)nx);
    tg.occupied_voxels = ids.data();
    tg.vertex_ofssets = offs.data();
    tg.voxels_count = (int)ids.size();
    tg.cell_size = make_float3(cell, cell, cell);
    tg.output = out;
    tg.vetexindex_to_voxel = v2v.data();
    tg.ver_voxel = vv.data() + zp.pad;
    const int3 size = make_int3(nx, ny, nz);
    for (long long i = 0; i < (long long)ids.size(); ++i) {
        set_thread(i, TrianglesGenerator::CTA_SIZE);
        trianglesGeneratorKernel(tg, size);
    }
    if (vi2vox) std::memcpy(vi2vox, v2v.data(), sizeof(int3) * (size_t)total);
    if (ver_voxel) std::memcpy(ver_voxel, vv.data() + zp.pad, sizeof(short) * (size_t)n);
    if (normals && total > 0) {
        Padded sp = padded(vol, nx, ny, nz, CU_VOXEL_MAX_TSDF);
        cu_voxel v;
        v.size = size;
        v.size_xy = nx * ny;
        v.min_t = v.max_t = 0.0f;
        v.grid_s = cell;
        v.data = sp.data();
        for (long long i = 0; i < total; ++i) {
            set_thread(i, 256);
            d_voxel_extract_surface_normals(v, (int)total, out, normals);
        }
    }
    return total;
}

// d_voxel_extract_surface_normals over n arbitrary vertex records
void ref_surface_normals(const cu_voxel_t *vol, int nx, int ny, int nz, float cell, vertex_voxel *verts,
                         long long n, float3 *normals) {
    Padded sp = padded(vol, nx, ny, nz, CU_VOXEL_MAX_TSDF);
    cu_voxel v;
    v.size = make_int3(nx, ny, nz);
    v.size_xy = nx * ny;
    v.min_t = v.max_t = 0.0f;
    v.grid_s = cell;
    v.data = sp.data();
    for (long long i = 0; i < n; ++i) {
        set_thread(i, 256);
        d_voxel_extract_surface_normals(v, (int)n, verts, normals);
    }
}

}  // extern "C"
