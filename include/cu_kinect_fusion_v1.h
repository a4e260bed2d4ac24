/*
 * cu_kinect_fusion_v1.h -- the reference's host interface for the TSDF ->
 * mesh path (cu_kinect_fusion_v1.h:30-46, :176-245) over the C ABI in
 * mcg.h.  Camera types follow cu_geometry_functions.h:96-108; colour is not
 * part of the voxel (structure.h:14-18), so colour arguments are ignored.
 */
#ifndef MCG_CU_KINECT_FUSION_V1_H
#define MCG_CU_KINECT_FUSION_V1_H

#include <vector_types.h>

#include "cu_memory.hpp"
#include "mcg.h"
#include "structure.h"

#define KINECT_DEPTH_MIN 0.0f /* metre */
#define KINECT_DEPTH_MAX 2.0f /* metre */
#define CU_VOXEL_MAX_W 0xffff
#define CU_VOXEL_MAX_TSDF 0x7ffe /* 32766 */
#define CU_VOXEL_UB_W 50.0f

static const char VOLUME_FORMAT[16] = "VOLUME_TSDF_RGB";

/* cu_vector_functions.h:383-386: 3x3 matrix as three float3 columns */
typedef struct _float33 {
    float3 p[3];
} float33;

/* cu_geometry_functions.h:96-101 */
typedef struct _float_camera_intrinsic {
    float2 fc;    /* focal lengths */
    float2 cc;    /* principal point */
    float dc[5];  /* distortion, unused by this path */
} float_camera_intrinsic;

/* cu_geometry_functions.h:104-108: camera -> global, R column-major */
typedef struct _float_camera_extrinsic {
    float33 R;
    float3 t;
} float_camera_extrinsic;

/* ---- volumes (cu_kinect_fusion_v1.cu:381-414) ---- */
/* allocates v->data if NULL, then every voxel -> {-32766, 0} */
void cu_voxel_new(cu_voxel *v, int3 size, float min_t, float max_t, float grid_s);
void cu_voxel_delete(cu_voxel *v);

/* ---- integrate (cu_kinect_fusion_v1.cu:534-549) ---- */
/* d_depth_ptr: device metres [size.y][size.x]; d_normal_ptr: NULL or device
 * camera-frame normal map; d_color_ptr: ignored */
void _cu_voxel_volumetric_integration(cu_voxel v, float_camera_intrinsic ci, float_camera_extrinsic ce,
                                      int2 size, float *d_depth_ptr, float3 *d_normal_ptr, uchar3 *d_color_ptr,
                                      bool is_dynamic);

/* ---- ray casting (cu_kinect_fusion_v1.cu:965-986) ---- */
/* depth (metres) and camera-frame normal maps of size.x x size.y pixels
 * (device pointers; n_ptr may be NULL); c_ptr (may be NULL) is filled with
 * white, the reference's default, since the voxel carries no colour */
void _cu_voxel_extract_depth_and_normal_map(cu_voxel v, float_camera_intrinsic ci, float_camera_extrinsic ce,
                                            int2 size, float *d_ptr, float3 *n_ptr, uchar3 *c_ptr);

/* ---- depth maps (cu_kinect_fusion_v1.cu:99-151, :275-295) ---- */
/* host buffers in and out, as the reference's host wrappers */
void cu_meter_to_vertex(float_camera_intrinsic k, int2 size, float *h_meter, float3 *h_vertex);
void cu_kinect_depth_to_vertex(float_camera_intrinsic k, int2 size, short *h_depth, float3 *h_vertex);
void cu_kinect_depth_to_normal(float_camera_intrinsic k, int2 size, short *h_depth, float3 *h_normal);
/* device buffers: depth (mm) -> metre / vertex / normal maps in one pass;
 * any output may be NULL */
void cu_kinect_depth_to_maps(float_camera_intrinsic k, int2 size, const unsigned short *d_depth_mm,
                             float *d_meter, float3 *d_vertex, float3 *d_normal);

/* ---- surface normals (cu_kinect_fusion_v1.cu:3236-3242) ---- */
void cu_voxel_extract_surface_normals(cu_voxel v, int size, const vertex_voxel *d_vertex, float3 *d_normal);

/* ---- RLE volume I/O (cu_kinect_fusion_v1.cu:1451-1600) ---- */
/* encode: if file_name does not exist the whole local volume is written;
 * otherwise the window [begin_local, begin_local+size) of v_local replaces
 * [begin_global, ...) of the stored volume.  decode: if v_local->data is
 * NULL the whole stored volume is loaded; otherwise the window is read into
 * v_local.  Errors are printed and leave the file / volume unchanged. */
void cu_voxel_run_length_encode(cu_voxel *v_local, const char *file_name, int3 begin_local, int3 begin_global,
                                int3 size);
void cu_voxel_run_length_decode(cu_voxel *v_local, const char *file_name, int3 begin_local, int3 begin_global,
                                int3 size);

/* ---- mesh drivers (cu_kinect_fusion_v1.cu:3261-3737) ---- */
/* text "x y z sdf weight" records -> volume_dim^3 volume -> mesh file
 * (.ply: binary soup with normals; .obj: vertices merged by their %.4f
 * coordinates, degenerate faces dropped) */
void cu_voxel_rlc_to_mesh(const char *file_input, const char *file_output, int volume_dim);
/* short2 volume (device or host memory) -> mesh file */
void cu_voxel_to_mesh(short2 *_local_volume_data, unsigned int _size_x, unsigned int _size_y, unsigned int _size_z,
                      float _grid_s, const char *file_output);

#endif
