/*
 * CPU oracle for the TSDF -> mesh path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithms, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * Nothing in the product (marching_cube_gb300/, include/) links or calls it.
 *
 * PARITY STATUS: parity unpinned by the reference's own tests -- the
 * reference ships no tests, fixtures or golden vectors, and its GPU code
 * cannot be built here (texture references and non-_sync warp votes that
 * nvcc 13 rejects, missing CUDA-samples headers, integrate / vmap / nmap /
 * RLE inside `#if 0`).  The oracle is pinned instead by analytic
 * known-answer tests (tests/test_oracle_kat.py) and by golden fixtures it
 * must reproduce (tests/golden/).
 *
 * Arithmetic convention ("FP32 mirror"): every float expression of the
 * reference is evaluated in IEEE binary32, in source order, with no FMA
 * contraction (compiled with -ffp-contract=off); `/` and sqrtf are
 * correctly rounded.  The CUDA kernels are built with --fmad=false and the
 * same operation order, so the two agree bit for bit.  The *_f64 entry
 * points evaluate positions and normals in binary64 for tolerance checks.
 */
#ifndef ORC_ORACLE_H
#define ORC_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* structure.h:14-18 cu_voxel_t, bit-compatible with short2 */
typedef struct { int16_t tsdf; uint16_t w; } orc_voxel;
/* FP32 volume voxel (tsdf, weight) used by the differentiable path */
typedef struct { float tsdf; float w; } orc_voxel_f32;
/* structure.h:29-35 vertex_voxel, 28 bytes */
typedef struct { float x, y, z; int32_t vx, vy, vz; int16_t tsdf; int16_t w; } orc_vertex_voxel;
/* cu_geometry_functions.h:96-101 float_camera_intrinsic */
typedef struct { float fx, fy, cx, cy; float dc[5]; } orc_intrinsic;
/* cu_geometry_functions.h:104-108 float_camera_extrinsic, camera->global,
 * R stored column-major as three float3 columns */
typedef struct { float r[9]; float t[3]; } orc_extrinsic;

enum { ORC_VOXEL_SHORT2 = 0, ORC_VOXEL_FLOAT2 = 1 };

/* ---- marching cubes (cu_marching_cubes_v1.cu) --------------------------- */
/* cube index and emitted-vertex count of every cube (x,y,z) with
 * x<nx-1, y<ny-1, z<nz-1, stored [z][y][x] over (nx-1)(ny-1)(nz-1) */
void orc_mc_classify(const void *vol, int vtype, int nx, int ny, int nz,
                     uint8_t *cube_index, uint8_t *num_verts);
/* occupied cubes and triangles in the volume */
void orc_mc_count(const void *vol, int vtype, int nx, int ny, int nz,
                  int64_t *n_occupied, int64_t *n_triangles, int nthreads);
/* Full extraction in canonical order (cube linear id, then table slot).
 * Any output pointer may be NULL.  ver_voxel (nx*ny*nz shorts) is zeroed
 * first.  Writes at most cap_verts soup vertices; returns the total. */
int64_t orc_mc_extract(const void *vol, int vtype, int nx, int ny, int nz, float cell,
                       orc_vertex_voxel *soup, float *normals, int32_t *vi2vox,
                       int16_t *ver_voxel, int64_t *tri_cube, int64_t cap_verts,
                       int nthreads);
/* binary64 positions / normals in the same canonical order */
int64_t orc_mc_extract_f64(const void *vol, int vtype, int nx, int ny, int nz, double cell,
                           double *pos, double *normals, int64_t cap_verts);
/* surface normal at one point (kf.cu:3146-3233), FP32 mirror */
void orc_surface_normal(const void *vol, int vtype, int nx, int ny, int nz, float cell,
                        const float p[3], float n[3]);

/* ---- voxel init (kf.cu:364-398) ---------------------------------------- */
void orc_voxel_init(orc_voxel *vol, int64_t n);

/* ---- depth maps (kf.cu:99-151) ----------------------------------------- */
void orc_depth_to_meter(const uint16_t *depth_mm, int64_t n, float dmin, float dmax, float *meter);
void orc_meter_to_vertex(const orc_intrinsic *k, int w, int h, const float *meter, float *vertex);
void orc_vertex_to_normal(int w, int h, const float *vertex, float *normal);
/* kf.cu:416-425 depth (z) -> ray length */
void orc_depth_scale(const orc_intrinsic *k, int w, int h, const float *depth, float *scaled);

/* ---- integrate (kf.cu:427-549), in place ------------------------------- */
void orc_integrate(void *vol, int vtype, int nx, int ny, int nz, float min_t, float max_t,
                   float grid_s, const orc_intrinsic *k, const orc_extrinsic *e, int w, int h,
                   const float *depth_m, const float *normals, int is_dynamic, int nthreads);

/* ---- RLE codec (kf.cu:1303-1600) --------------------------------------- */
/* encode one slice; lossless=0 is the reference format (runs compare tsdf
 * only), lossless=1 compares whole voxels.  buf needs 6*n bytes.  Returns
 * bytes written. */
int64_t orc_rle_encode_slice(const orc_voxel *s, int64_t n, int lossless, uint8_t *buf);
/* decode one slice of n voxels; returns bytes consumed, or -1 if the record
 * stream is malformed or does not cover exactly n voxels */
int64_t orc_rle_decode_slice(const uint8_t *buf, int64_t nbytes, orc_voxel *out, int64_t n);
/* whole file image (header + per-slice dumps); returns size or -1 */
int64_t orc_rle_encode_volume(const orc_voxel *vol, int nx, int ny, int nz, float min_t,
                              float max_t, float grid_s, int lossless, uint8_t *out, int64_t cap);
/* returns 0 on success; dims/params out; vol may be NULL to query dims */
int orc_rle_decode_volume(const uint8_t *img, int64_t nbytes, orc_voxel *vol, int64_t cap_voxels,
                          int dims[3], float params[3]);

/* ---- adjoints (binary64; no counterpart in the reference) -------------- */
/* linear voxel indices of the two corners of each soup vertex's edge,
 * canonical order; returns the vertex total */
int64_t orc_mc_edges(const void *vol, int vtype, int nx, int ny, int nz, int64_t *va, int64_t *vb,
                     int64_t cap_verts);
/* dL/df (f = tsdf, or tsdf/32766 for short2) += adjoint of the soup
 * positions for dL/dP (canonical order, n vertices); cube cases fixed */
int64_t orc_mc_backward_f64(const void *vol, int vtype, int nx, int ny, int nz, double cell,
                            const double *grad_pos, int64_t n, double *grad_f);
/* n_frames integrate steps on a float2 volume in binary64 (vol0: float2 or
 * NULL = (-1, 0)); decisions from the FP32 mirror at (float)depth.
 * signature: hash of every decision, to tell when a perturbation changes one */
void orc_integrate_seq_f64(const float *vol0, int nx, int ny, int nz, float min_t, float max_t, float grid_s,
                           const orc_intrinsic *k, int n_frames, const orc_extrinsic *poses, int w, int h,
                           const double *depth, const float *normals, int is_dynamic, double *F, double *W,
                           uint64_t *signature, int nthreads);
/* its adjoint: dL/ddepth += ..., dL/d(F0, W0) written (may be NULL) */
void orc_integrate_seq_backward_f64(const float *vol0, int nx, int ny, int nz, float min_t, float max_t,
                                    float grid_s, const orc_intrinsic *k, int n_frames,
                                    const orc_extrinsic *poses, int w, int h, const double *depth,
                                    const float *normals, int is_dynamic, const double *gF_end,
                                    const double *gW_end, double *g_depth, double *gF0, double *gW0,
                                    int nthreads);

/* ---- indexed mesh (no counterpart in the reference) -------------------- */
/* position / normal / voxel of the vertex on grid edge keys[i] =
 * 3 * linear index of the lower voxel + axis, interpolated lower -> upper */
void orc_mc_edge_vertices(const void *vol, int vtype, int nx, int ny, int nz, float cell, const int64_t *keys,
                          int64_t n, float *pos, float *normals, int32_t *vi2vox);

/* ---- ray casting (kf.cu:551-659, 786-986), short2 volumes --------------- */
/* camera set-up (:965-986): IM = (K R^T)^-1 as columns IM[j][i], cc = t /
 * grid_s; 0 if singular */
int orc_raycast_setup(const orc_intrinsic *k, const orc_extrinsic *e, float grid_s, float IM[3][3], float cc[3]);
/* depth (metres, 0 = no hit) and normal (may be NULL) maps of w x h pixels;
 * 0 (nothing written) if the camera matrix is singular */
int orc_raycast(const orc_voxel *vol, int nx, int ny, int nz, float grid_s, const orc_intrinsic *k,
                const orc_extrinsic *e, int w, int h, float *depth, float *normal, int nthreads);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
