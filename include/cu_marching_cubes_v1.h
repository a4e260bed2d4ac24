/*
 * cu_marching_cubes_v1.h -- the reference's MarchingCubes class
 * (cu_marching_cubes_v1.h:28-65) over the C ABI in mcg.h.
 */
#ifndef MCG_CU_MARCHING_CUBES_V1_H
#define MCG_CU_MARCHING_CUBES_V1_H

#include <vector_types.h>

#include "cu_memory.hpp"
#include "mcg.h"
#include "structure.h"

class MarchingCubes {
public:
    enum {
        POINTS_PER_TRIANGLE = 3,
        DEFAULT_TRIANGLES_BUFFER_SIZE = 9 * 1000 * 1000 * POINTS_PER_TRIANGLE
    };

    /* ctor: the tables live in the library; this creates the per-instance
     * context (scratch, counters) on the current device */
    MarchingCubes();
    ~MarchingCubes();
    MarchingCubes(const MarchingCubes &) = delete;
    MarchingCubes &operator=(const MarchingCubes &) = delete;

    /* cu_marching_cubes_v1.cu:416-467.  Returns a non-owning view of the
     * first (3 * triangles) records of triangles_buffer, or an empty array
     * when no cube is occupied.  Empty buffers are allocated; a buffer that
     * is too small is grown to the needed size (the reference truncates or
     * overruns it).  vertexindex_to_voxel gets vox_pos per record and
     * ver_voxel (one short per voxel) the tsdf at each vertex voxel. */
    cu_array<vertex_voxel> run(cu_voxel &tsdf, cu_array<vertex_voxel> &triangles_buffer,
                               cu_array<int3> &vertexindex_to_voxel, cu_array<short> &ver_voxel);

    /* same, with the fused surface normal of every record
     * (d_voxel_extract_surface_normals, cu_kinect_fusion_v1.cu:3236-3242) */
    cu_array<vertex_voxel> run(cu_voxel &tsdf, cu_array<vertex_voxel> &triangles_buffer,
                               cu_array<int3> &vertexindex_to_voxel, cu_array<short> &ver_voxel,
                               cu_array<float3> &normals);

    /* counts of the last run */
    const mcg_mesh_counts &counts() const { return counts_; }

    /* adjoint of the last run's soup positions (no counterpart in the
     * reference): grad_pos holds dL/dP per soup vertex of that run, in its
     * order; dL/df (f = tsdf / 32766) is accumulated into grad_tsdf (one
     * float per voxel, allocated and zeroed here when empty).  The volume
     * must be unchanged since run(). */
    void backward(cu_voxel &tsdf, const cu_array<float3> &grad_pos, cu_array<float> &grad_tsdf);

private:
    cu_array<vertex_voxel> run_impl(cu_voxel &tsdf, cu_array<vertex_voxel> &triangles_buffer,
                                    cu_array<int3> &vertexindex_to_voxel, cu_array<short> &ver_voxel,
                                    cu_array<float3> *normals);
    mcg_context *ctx_;
    mcg_mesh_counts counts_;
};

#endif
