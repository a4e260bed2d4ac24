/*
 * structure.h -- voxel, volume and vertex types of the TSDF -> mesh path,
 * layout-compatible with the reference's structure.h:14-35 (cu_voxel_t is a
 * short2, vertex_voxel is 28 bytes), so existing buffers pass through.
 */
#ifndef MCG_STRUCTURE_H
#define MCG_STRUCTURE_H

#include <vector_types.h> /* CUDA int3, float3, short2, uchar3 */

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;

typedef struct _CU_COLOR_T {
    uchar p[3];
} cu_color_t;

/* structure.h:14-18 */
typedef struct _CU_VOXEL_T {
    short tsdf; /* normalised tsdf, +-32766 sentinels */
    ushort w;   /* weight */
} cu_voxel_t;

/* structure.h:20-27: data is a device pointer, [z][y][x] */
typedef struct _CU_VOXEL {
    int3 size;
    int size_xy; /* size.x * size.y */
    float min_t;
    float max_t;
    float grid_s;
    cu_voxel_t *data;
} cu_voxel;

/* structure.h:29-35 */
typedef struct _VERTEX_VOXEL {
    float3 ver_pos;
    int3 vox_pos;
    short tsdf;
    short w;
} vertex_voxel;

#define cu_voxel_access_z(v, _z) ((v)->data + (size_t)(_z) * (v)->size_xy)
#define cu_voxel_access_yz(v, _y, _z) (cu_voxel_access_z(v, _z) + (size_t)(_y) * (v)->size.x)
#define cu_voxel_access_xyz(v, _x, _y, _z) (cu_voxel_access_yz(v, _y, _z) + (_x))

#ifdef __cplusplus
static_assert(sizeof(cu_voxel_t) == 4, "cu_voxel_t is a short2");
static_assert(sizeof(vertex_voxel) == 28, "vertex_voxel is 28 bytes");
#endif

#endif
