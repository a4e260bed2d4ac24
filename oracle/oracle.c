/*
 * CPU oracle for the TSDF -> mesh path.  TEST INFRASTRUCTURE ONLY -- see
 * oracle.h for the parity status ("parity unpinned" by reference tests) and
 * the FP32-mirror convention.  Build: oracle/Makefile (-ffp-contract=off).
 *
 * Each function cites the reference lines it restates.  Paths are relative
 * to the reference project root.
 */
#include "oracle.h"
#include "mc_tables.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_TSDF 32766   /* cu_kinect_fusion_v1.h:44 CU_VOXEL_MAX_TSDF */
#define ORC_MAX_W 65535      /* cu_kinect_fusion_v1.h:42 CU_VOXEL_MAX_W */
#define ORC_UB_W 50.0f       /* cu_kinect_fusion_v1.h:46 CU_VOXEL_UB_W */

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int nthreads_or_default(int n) { return n > 0 ? n : orc_max_threads(); }

/* ------------------------------------------------------------------------ */
/* voxel access                                                              */
/* ------------------------------------------------------------------------ */

/* cu_kinect_fusion_v1.h:253-256 d_unpack_tsdf: (float)tsdf / 32766 */
static inline float unpack_tsdf(int16_t t) { return (float)t / (float)ORC_MAX_TSDF; }

/* value, weight-is-zero flag and raw tsdf of voxel at linear index i */
static inline float vox_f(const void *vol, int vtype, int64_t i) {
    if (vtype == ORC_VOXEL_SHORT2) return unpack_tsdf(((const orc_voxel *)vol)[i].tsdf);
    return ((const orc_voxel_f32 *)vol)[i].tsdf;
}
static inline int vox_w0(const void *vol, int vtype, int64_t i) {
    if (vtype == ORC_VOXEL_SHORT2) return ((const orc_voxel *)vol)[i].w == 0;
    return ((const orc_voxel_f32 *)vol)[i].w == 0.0f;
}
static inline int vox_neg(const void *vol, int vtype, int64_t i) {
    /* f < 0 (cu_marching_cubes_v1.cu:84-91); for short2 this is tsdf < 0 */
    if (vtype == ORC_VOXEL_SHORT2) return ((const orc_voxel *)vol)[i].tsdf < 0;
    return ((const orc_voxel_f32 *)vol)[i].tsdf < 0.0f;
}

/* ------------------------------------------------------------------------ */
/* marching cubes: classification (cu_marching_cubes_v1.cu:53-95, 126-137)   */
/* ------------------------------------------------------------------------ */

/* corner c of cube (x,y,z): order (x,y,z),(x+1,y,z),(x+1,y+1,z),(x,y+1,z),
 * then the same at z+1 (cu_marching_cubes_v1.cu:74-81) */
static const int CX[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int CY[8] = {0, 0, 1, 1, 0, 0, 1, 1};
static const int CZ[8] = {0, 0, 0, 0, 1, 1, 1, 1};
/* edge -> (first, second) corner in vertex_interp argument order
 * (cu_marching_cubes_v1.cu:304-315) */
static const int EA[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
static const int EB[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};

static inline int64_t lin(int nx, int ny, int x, int y, int z) {
    return ((int64_t)z * ny + y) * nx + x;
}

/* cube index; 0 when any corner weight is zero (computeCubeIndex) */
static inline int cube_index(const void *vol, int vtype, int nx, int ny, int x, int y, int z) {
    int ci = 0;
    for (int c = 0; c < 8; ++c) {
        int64_t i = lin(nx, ny, x + CX[c], y + CY[c], z + CZ[c]);
        if (vox_w0(vol, vtype, i)) return 0;
        ci |= vox_neg(vol, vtype, i) << c;
    }
    return ci;
}

/* emitted vertices (OccupiedVoxels::operator(), cu_marching_cubes_v1.cu:136) */
static inline int cube_nverts(int ci) {
    return (ci == 0 || ci == 255) ? 0 : orc_num_verts[ci];
}

void orc_mc_classify(const void *vol, int vtype, int nx, int ny, int nz,
                     uint8_t *cube_index_out, uint8_t *num_verts_out) {
    int cx = nx - 1, cy = ny - 1, cz = nz - 1;
    if (cx <= 0 || cy <= 0 || cz <= 0) return;
    for (int z = 0; z < cz; ++z)
        for (int y = 0; y < cy; ++y)
            for (int x = 0; x < cx; ++x) {
                int ci = cube_index(vol, vtype, nx, ny, x, y, z);
                int64_t o = ((int64_t)z * cy + y) * cx + x;
                if (cube_index_out) cube_index_out[o] = (uint8_t)ci;
                if (num_verts_out) num_verts_out[o] = (uint8_t)cube_nverts(ci);
            }
}

/* per z-slice triangle/occupied counts, cubes z in [0, nz-2] */
static void slice_counts(const void *vol, int vtype, int nx, int ny, int nz,
                         int64_t *tri, int64_t *occ, int nthreads) {
    int cz = nz - 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int z = 0; z < cz; ++z) {
        int64_t t = 0, o = 0;
        for (int y = 0; y + 1 < ny; ++y)
            for (int x = 0; x + 1 < nx; ++x) {
                int nv = cube_nverts(cube_index(vol, vtype, nx, ny, x, y, z));
                t += nv / 3;
                o += nv > 0;
            }
        tri[z] = t;
        occ[z] = o;
    }
}

void orc_mc_count(const void *vol, int vtype, int nx, int ny, int nz,
                  int64_t *n_occupied, int64_t *n_triangles, int nthreads) {
    int64_t o = 0, t = 0;
    if (nx >= 2 && ny >= 2 && nz >= 2) {
        int cz = nz - 1;
        int64_t *tri = (int64_t *)calloc(cz, sizeof(int64_t));
        int64_t *occ = (int64_t *)calloc(cz, sizeof(int64_t));
        slice_counts(vol, vtype, nx, ny, nz, tri, occ, nthreads_or_default(nthreads));
        for (int z = 0; z < cz; ++z) { t += tri[z]; o += occ[z]; }
        free(tri);
        free(occ);
    }
    if (n_occupied) *n_occupied = o;
    if (n_triangles) *n_triangles = t;
}

/* ------------------------------------------------------------------------ */
/* surface normal (cu_kinect_fusion_v1.cu:3146-3233), FP32 mirror           */
/* ------------------------------------------------------------------------ */

/* cu_math_functions.h:99-103 float_interpolation_bilinear */
static inline float bilinear(float v0, float v1, float v2, float v3, float x, float y) {
    float a = 1.0f - x, b = 1.0f - y;
    return v0 * a * b + v1 * x * b + v2 * a * y + v3 * x * y;
}

/* cu_vector_functions.h:258-264 float3_unit (divides only if |n| > eps) */
static inline void unit3(float n[3]) {
    float norm = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (norm > FLT_EPSILON || norm < -FLT_EPSILON) {
        n[0] = n[0] / norm;
        n[1] = n[1] / norm;
        n[2] = n[2] / norm;
    }
}

/* The reference addresses the 8 samples linearly from the start of slice
 * p_i.z (index = p_i.y*X + p_i.x, then +1, +X, +XY); at the max faces this
 * reads the neighbouring row/slice, and past the end of the volume it reads
 * outside the allocation.  The mirror keeps the linear addressing and
 * returns the zero normal when any of the 8 addresses is outside [0, N). */
void orc_surface_normal(const void *vol, int vtype, int nx, int ny, int nz, float cell,
                        const float p[3], float n[3]) {
    float pf[3] = {p[0] / cell, p[1] / cell, p[2] / cell};   /* kf.cu:3241 */
    int pi[3] = {(int)pf[0], (int)pf[1], (int)pf[2]};        /* kf.cu:3230 */
    float tf[3] = {pf[0] - (float)pi[0], pf[1] - (float)pi[1], pf[2] - (float)pi[2]};
    int64_t xy = (int64_t)nx * ny, N = xy * nz;
    int64_t base = (int64_t)pi[2] * xy + (int64_t)pi[1] * nx + pi[0];
    /* V000, V100, V110, V010 in slice z; same in slice z+1 */
    const int64_t off[8] = {0, 1, 1 + nx, nx, xy, xy + 1, xy + 1 + nx, xy + nx};
    /* sdfs[] slot of each sample (kf.cu:3156-3194) */
    const int slot[8] = {0, 1, 6, 2, 3, 4, 7, 5};
    float s[8];
    n[0] = n[1] = n[2] = 0.0f;
    for (int k = 0; k < 8; ++k) {
        int64_t a = base + off[k];
        if (a < 0 || a >= N) return;
        if (vtype == ORC_VOXEL_SHORT2) {
            int16_t t = ((const orc_voxel *)vol)[a].tsdf;
            if (t == ORC_MAX_TSDF || t == -ORC_MAX_TSDF) return;
            s[slot[k]] = unpack_tsdf(t);
        } else {
            s[slot[k]] = ((const orc_voxel_f32 *)vol)[a].tsdf;
        }
    }
    float s1, s2;
    s1 = bilinear(s[0], s[2], s[3], s[5], tf[1], tf[2]);
    s2 = bilinear(s[1], s[6], s[4], s[7], tf[1], tf[2]);
    n[0] = s2 - s1;
    s1 = bilinear(s[0], s[1], s[3], s[4], tf[0], tf[2]);
    s2 = bilinear(s[2], s[6], s[5], s[7], tf[0], tf[2]);
    n[1] = s2 - s1;
    s1 = bilinear(s[0], s[1], s[2], s[6], tf[0], tf[1]);
    s2 = bilinear(s[3], s[4], s[5], s[7], tf[0], tf[1]);
    n[2] = s2 - s1;
    unit3(n);
}

static void surface_normal_f64(const void *vol, int vtype, int nx, int ny, int nz, double cell,
                               const double p[3], double n[3]) {
    double pf[3] = {p[0] / cell, p[1] / cell, p[2] / cell};
    int pi[3] = {(int)pf[0], (int)pf[1], (int)pf[2]};
    double tf[3] = {pf[0] - pi[0], pf[1] - pi[1], pf[2] - pi[2]};
    int64_t xy = (int64_t)nx * ny, N = xy * nz;
    int64_t base = (int64_t)pi[2] * xy + (int64_t)pi[1] * nx + pi[0];
    const int64_t off[8] = {0, 1, 1 + nx, nx, xy, xy + 1, xy + 1 + nx, xy + nx};
    const int slot[8] = {0, 1, 6, 2, 3, 4, 7, 5};
    double s[8];
    n[0] = n[1] = n[2] = 0.0;
    for (int k = 0; k < 8; ++k) {
        int64_t a = base + off[k];
        if (a < 0 || a >= N) return;
        if (vtype == ORC_VOXEL_SHORT2) {
            int16_t t = ((const orc_voxel *)vol)[a].tsdf;
            if (t == ORC_MAX_TSDF || t == -ORC_MAX_TSDF) return;
            s[slot[k]] = (double)t / ORC_MAX_TSDF;
        } else {
            s[slot[k]] = ((const orc_voxel_f32 *)vol)[a].tsdf;
        }
    }
#define BIL(v0, v1, v2, v3, x, y) \
    ((v0) * (1 - (x)) * (1 - (y)) + (v1) * (x) * (1 - (y)) + (v2) * (1 - (x)) * (y) + (v3) * (x) * (y))
    n[0] = BIL(s[1], s[6], s[4], s[7], tf[1], tf[2]) - BIL(s[0], s[2], s[3], s[5], tf[1], tf[2]);
    n[1] = BIL(s[2], s[6], s[5], s[7], tf[0], tf[2]) - BIL(s[0], s[1], s[3], s[4], tf[0], tf[2]);
    n[2] = BIL(s[3], s[4], s[5], s[7], tf[0], tf[1]) - BIL(s[0], s[1], s[2], s[6], tf[0], tf[1]);
#undef BIL
    double norm = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (norm > FLT_EPSILON) { n[0] /= norm; n[1] /= norm; n[2] /= norm; }
}

/* ------------------------------------------------------------------------ */
/* marching cubes: generation (cu_marching_cubes_v1.cu:228-366)             */
/* ------------------------------------------------------------------------ */

/* getNodeCoo (:243-254): ((float)i + 0.5f) * cell */
static inline float node(int i, float cell) { return ((float)i + 0.5f) * cell; }

/* vertex_interp (:256-264) on one axis */
static inline float interp1(float p0, float p1, float t) { return p0 + t * (p1 - p0); }

static void emit_cube(const void *vol, int vtype, int nx, int ny, int nz, float cell,
                      int x, int y, int z, int ci, int64_t o, int64_t cap,
                      orc_vertex_voxel *soup, float *normals, int32_t *vi2vox,
                      int16_t *ver_voxel, int64_t *tri_cube) {
    int64_t xy = (int64_t)nx * ny, N = xy * nz;
    float f[8], vp[8][3];
    for (int c = 0; c < 8; ++c) {
        f[c] = vox_f(vol, vtype, lin(nx, ny, x + CX[c], y + CY[c], z + CZ[c]));
        vp[c][0] = node(x + CX[c], cell);
        vp[c][1] = node(y + CY[c], cell);
        vp[c][2] = node(z + CZ[c], cell);
    }
    int nv = orc_num_verts[ci];
    for (int i = 0; i < nv; ++i) {
        /* out[o+i+2]=e[tri[i]], out[o+i+1]=e[tri[i+1]], out[o+i]=e[tri[i+2]]
         * (:322-333): output slot k of triangle j takes edge tri[3j+2-k] */
        int j = i / 3, k = i % 3;
        int e = orc_tri_table[ci][3 * j + 2 - k];
        int a = EA[e], b = EB[e];
        float t = (0.0f - f[a]) / (f[b] - f[a] + 1e-15f);
        float P[3] = {interp1(vp[a][0], vp[b][0], t), interp1(vp[a][1], vp[b][1], t),
                      interp1(vp[a][2], vp[b][2], t)};
        int64_t idx = o + i;
        if (idx >= cap) continue;
        /* store_point (:336-367): voxel of the vertex and its tsdf / w */
        int v[3];
        for (int d = 0; d < 3; ++d) v[d] = (int)floorf(P[d] / cell - 0.5f);
        int64_t li = ((int64_t)v[2] * ny + v[1]) * nx + v[0];
        int16_t vt = 0, vw = 0;
        if (li >= 0 && li < N) {
            if (vtype == ORC_VOXEL_SHORT2) {
                vt = ((const orc_voxel *)vol)[li].tsdf;
                vw = (int16_t)((const orc_voxel *)vol)[li].w;
            }
            if (ver_voxel) ver_voxel[li] = vt;
        }
        if (soup) {
            orc_vertex_voxel *r = soup + idx;
            r->x = P[0]; r->y = P[1]; r->z = P[2];
            r->vx = v[0]; r->vy = v[1]; r->vz = v[2];
            r->tsdf = vt; r->w = vw;
        }
        if (vi2vox) { vi2vox[3 * idx] = v[0]; vi2vox[3 * idx + 1] = v[1]; vi2vox[3 * idx + 2] = v[2]; }
        if (normals) orc_surface_normal(vol, vtype, nx, ny, nz, cell, P, normals + 3 * idx);
        if (tri_cube && k == 0) tri_cube[idx / 3] = lin(nx, ny, x, y, z);
    }
}

int64_t orc_mc_extract(const void *vol, int vtype, int nx, int ny, int nz, float cell,
                       orc_vertex_voxel *soup, float *normals, int32_t *vi2vox,
                       int16_t *ver_voxel, int64_t *tri_cube, int64_t cap_verts,
                       int nthreads) {
    if (ver_voxel) memset(ver_voxel, 0, sizeof(int16_t) * (size_t)nx * ny * nz);
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    nthreads = nthreads_or_default(nthreads);
    int cz = nz - 1;
    int64_t *tri = (int64_t *)calloc(cz + 1, sizeof(int64_t));
    int64_t *occ = (int64_t *)calloc(cz, sizeof(int64_t));
    slice_counts(vol, vtype, nx, ny, nz, tri, occ, nthreads);
    /* exclusive scan of per-slice vertex counts (cu_marching_cubes_v1.cu:208-225) */
    int64_t run = 0;
    for (int z = 0; z < cz; ++z) { int64_t t = tri[z]; tri[z] = run; run += 3 * t; }
    int64_t total = run;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int z = 0; z < cz; ++z) {
        int64_t o = tri[z];
        for (int y = 0; y + 1 < ny; ++y)
            for (int x = 0; x + 1 < nx; ++x) {
                int ci = cube_index(vol, vtype, nx, ny, x, y, z);
                int nv = cube_nverts(ci);
                if (!nv) continue;
                emit_cube(vol, vtype, nx, ny, nz, cell, x, y, z, ci, o, cap_verts, soup, normals,
                          vi2vox, ver_voxel, tri_cube);
                o += nv;
            }
    }
    free(tri);
    free(occ);
    return total;
}

int64_t orc_mc_extract_f64(const void *vol, int vtype, int nx, int ny, int nz, double cell,
                           double *pos, double *normals, int64_t cap_verts) {
    int64_t o = 0;
    for (int z = 0; z + 1 < nz; ++z)
        for (int y = 0; y + 1 < ny; ++y)
            for (int x = 0; x + 1 < nx; ++x) {
                int ci = cube_index(vol, vtype, nx, ny, x, y, z);
                int nv = cube_nverts(ci);
                if (!nv) continue;
                double f[8], vp[8][3];
                for (int c = 0; c < 8; ++c) {
                    int64_t li = lin(nx, ny, x + CX[c], y + CY[c], z + CZ[c]);
                    f[c] = vtype == ORC_VOXEL_SHORT2
                               ? (double)((const orc_voxel *)vol)[li].tsdf / ORC_MAX_TSDF
                               : (double)((const orc_voxel_f32 *)vol)[li].tsdf;
                    vp[c][0] = (x + CX[c] + 0.5) * cell;
                    vp[c][1] = (y + CY[c] + 0.5) * cell;
                    vp[c][2] = (z + CZ[c] + 0.5) * cell;
                }
                for (int i = 0; i < nv; ++i, ++o) {
                    if (o >= cap_verts) continue;
                    int j = i / 3, k = i % 3;
                    int e = orc_tri_table[ci][3 * j + 2 - k];
                    int a = EA[e], b = EB[e];
                    double t = -f[a] / (f[b] - f[a] + 1e-15);
                    double P[3];
                    for (int d = 0; d < 3; ++d) P[d] = vp[a][d] + t * (vp[b][d] - vp[a][d]);
                    if (pos) { pos[3 * o] = P[0]; pos[3 * o + 1] = P[1]; pos[3 * o + 2] = P[2]; }
                    if (normals) surface_normal_f64(vol, vtype, nx, ny, nz, cell, P, normals + 3 * o);
                }
            }
    return o;
}

/* ------------------------------------------------------------------------ */
/* voxel init (cu_kinect_fusion_v1.cu:364-379)                               */
/* ------------------------------------------------------------------------ */
void orc_voxel_init(orc_voxel *vol, int64_t n) {
    for (int64_t i = 0; i < n; ++i) { vol[i].tsdf = -ORC_MAX_TSDF; vol[i].w = 0; }
}

/* ------------------------------------------------------------------------ */
/* depth maps (cu_kinect_fusion_v1.cu:99-151)                                */
/* ------------------------------------------------------------------------ */

/* d_kinect_depth_to_meter (:99-113), OpenNI branch; invalid metre = 0 */
void orc_depth_to_meter(const uint16_t *depth_mm, int64_t n, float dmin, float dmax, float *meter) {
    for (int64_t i = 0; i < n; ++i) {
        float m = (float)depth_mm[i] / 1000.0f;
        if (m < dmin || m > dmax) m = 0.0f;
        meter[i] = m;
    }
}

/* d_img_meter_to_vertex (:116-127) with float_camera_intrinsic_unproject_3
 * (cu_geometry_functions.h:237-246); invalid vertex = (0,0,0) */
void orc_meter_to_vertex(const orc_intrinsic *k, int w, int h, const float *meter, float *vertex) {
    for (int i = 0; i < h; ++i)
        for (int j = 0; j < w; ++j) {
            int64_t x = (int64_t)i * w + j;
            float m = meter[x];
            float *v = vertex + 3 * x;
            v[0] = v[1] = v[2] = 0.0f;
            if (m != 0.0f) {
                float px = ((float)j - k->cx) / k->fx;
                float py = ((float)i - k->cy) / k->fy;
                v[0] = px * m;
                v[1] = py * m;
                v[2] = m;
            }
        }
}

static inline int vertex_valid(const float *v) { return !(v[0] == 0.0f && v[1] == 0.0f && v[2] == 0.0f); }

/* d_img_vertex_to_normal (:130-151); invalid normal = (0,0,0) */
void orc_vertex_to_normal(int w, int h, const float *vertex, float *normal) {
    for (int i = 0; i < h; ++i)
        for (int j = 0; j < w; ++j) {
            int64_t idx = (int64_t)i * w + j;
            float n[3] = {0.0f, 0.0f, 0.0f};
            if (i < h - 1 && j < w - 1) {
                const float *vc = vertex + 3 * idx, *vx = vertex + 3 * (idx + 1),
                            *vy = vertex + 3 * (idx + w);
                if (vertex_valid(vc) && vertex_valid(vx) && vertex_valid(vy)) {
                    float tx[3] = {vx[0] - vc[0], vx[1] - vc[1], vx[2] - vc[2]};
                    float ty[3] = {vc[0] - vy[0], vc[1] - vy[1], vc[2] - vy[2]};
                    n[0] = tx[1] * ty[2] - tx[2] * ty[1];
                    n[1] = tx[2] * ty[0] - tx[0] * ty[2];
                    n[2] = tx[0] * ty[1] - tx[1] * ty[0];
                    unit3(n);
                }
            }
            normal[3 * idx] = n[0];
            normal[3 * idx + 1] = n[1];
            normal[3 * idx + 2] = n[2];
        }
}

/* d_voxel_volumetric_depth_scaling (:416-425) */
void orc_depth_scale(const orc_intrinsic *k, int w, int h, const float *depth, float *scaled) {
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            float px = ((float)x - k->cx) / k->fx;
            float py = ((float)y - k->cy) / k->fy;
            int64_t i = (int64_t)y * w + x;
            scaled[i] = depth[i] * sqrtf(px * px + py * py + 1.0f);
        }
}

/* ------------------------------------------------------------------------ */
/* integrate (cu_kinect_fusion_v1.cu:427-532)                                */
/* ------------------------------------------------------------------------ */

/* __float2int_rn: round half to even, saturating, NaN -> 0 */
static inline int f2i_rn(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v < -2147483648.0f) return (-2147483647 - 1);
    return (int)nearbyintf(v);
}

/* d_pack_tsdf / d_pack_weight / d_unpack_weight (cu_kinect_fusion_v1.h:152-171);
 * the weight codec is this self-consistent pair, not the live w/16 variant
 * at cu_kinect_fusion_v1.h:247-250 (only w==0 matters to extraction) */
static inline int16_t pack_tsdf(float f) { return (int16_t)(int)(f * (float)ORC_MAX_TSDF); }
static inline uint16_t pack_weight(float w) {
    w = (w < ORC_UB_W) ? w / ORC_UB_W : 1.0f;
    return (uint16_t)(w * (float)ORC_MAX_W + 0.5f);
}
static inline float unpack_weight(uint16_t w) { return (float)w / (float)ORC_MAX_W * ORC_UB_W; }

void orc_integrate(void *vol, int vtype, int nx, int ny, int nz, float min_t, float max_t,
                   float grid_s, const orc_intrinsic *k, const orc_extrinsic *e, int w, int h,
                   const float *depth_m, const float *normals, int is_dynamic, int nthreads) {
    nthreads = nthreads_or_default(nthreads);
    float *ds = (float *)malloc(sizeof(float) * (size_t)w * h);
    orc_depth_scale(k, w, h, depth_m, ds);
    const float *R = e->r; /* columns R[0..2], R[3..5], R[6..8] */
#pragma omp parallel for collapse(2) schedule(static) num_threads(nthreads)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            float p[3] = {-grid_s, (float)y * grid_s, (float)z * grid_s};
            for (int x = 0; x < nx; ++x) {
                p[0] += grid_s; /* accumulated, as in the reference (:444) */
                /* float_camera_extrinsic_backward (geo:125-129), matrix33_tv */
                float v0 = p[0] - e->t[0], v1 = p[1] - e->t[1], v2 = p[2] - e->t[2];
                float q0 = R[0] * v0 + R[1] * v1 + R[2] * v2;
                float q1 = R[3] * v0 + R[4] * v1 + R[5] * v2;
                float q2 = R[6] * v0 + R[7] * v1 + R[8] * v2;
                if (q2 < FLT_MIN) continue;
                /* float_camera_intrinsic_project_3 (geo:232-235) */
                float u_f = k->fx * (q0 / q2) + k->cx;
                float v_f = k->fy * (q1 / q2) + k->cy;
                int u = f2i_rn(u_f), v = f2i_rn(v_f);
                if (u < 0 || v < 0 || u >= (w - 2) || v >= (h - 2)) continue;
                float z_val = ds[(int64_t)v * w + u];
                if (!(z_val > FLT_MIN)) continue;
                float qn = sqrtf(q0 * q0 + q1 * q1 + q2 * q2);
                float sdf = z_val - qn;
                if (!(sdf >= -min_t)) continue;
                if (sdf > 0.0f) {
                    sdf = sdf / max_t;
                    if (sdf > 1.0f) sdf = 1.0f;
                } else {
                    sdf = sdf / min_t;
                }
                float weight = 1.0f;
                if (normals) {
                    const float *n = normals + 3 * ((int64_t)v * w + u);
                    if (!vertex_valid(n)) continue; /* invalid normal = (0,0,0) */
                    weight = -(n[0] * (q0 / qn) + n[1] * (q1 / qn) + n[2] * (q2 / qn));
                    if (weight < FLT_MIN) continue;
                }
                weight = weight / z_val;
                int64_t li = lin(nx, ny, x, y, z);
                float sdf1, w1;
                if (vtype == ORC_VOXEL_SHORT2) {
                    orc_voxel *vx = (orc_voxel *)vol + li;
                    sdf1 = unpack_tsdf(vx->tsdf);
                    w1 = unpack_weight(vx->w);
                } else {
                    orc_voxel_f32 *vx = (orc_voxel_f32 *)vol + li;
                    sdf1 = vx->tsdf;
                    w1 = vx->w;
                }
                if (is_dynamic) {
                    float d = fabsf(sdf - sdf1);
                    weight = weight * (1.0f + d * d * 10.0f);
                }
                float w2 = w1 + weight;
                float sdf2 = (w1 * sdf1 + weight * sdf) / w2;
                if (vtype == ORC_VOXEL_SHORT2) {
                    orc_voxel *vx = (orc_voxel *)vol + li;
                    vx->tsdf = pack_tsdf(sdf2);
                    vx->w = pack_weight(w2);
                } else {
                    orc_voxel_f32 *vx = (orc_voxel_f32 *)vol + li;
                    vx->tsdf = sdf2;
                    vx->w = w2;
                }
            }
        }
    free(ds);
}

/* ------------------------------------------------------------------------ */
/* RLE codec (cu_kinect_fusion_v1.cu:1303-1447)                              */
/* ------------------------------------------------------------------------ */

/* cu_voxel_rle (:1362-1365): 16-bit record, n in bits 0-13, v in bits 14-15 */
static inline void put_rec(uint8_t *b, unsigned n, unsigned v) {
    unsigned r = (n & 0x3fffu) | (v << 14);
    b[0] = (uint8_t)(r & 0xff);
    b[1] = (uint8_t)(r >> 8);
}

static int64_t put_run(uint8_t *b, orc_voxel first, unsigned n, int lossless) {
    int empty = first.tsdf == ORC_MAX_TSDF, null = first.tsdf == -ORC_MAX_TSDF;
    if (lossless && first.w != 0) empty = null = 0;
    if (empty) { put_rec(b, n, 1); return 2; }
    if (null) { put_rec(b, n, 2); return 2; }
    put_rec(b, n, 3);
    b[2] = (uint8_t)((uint16_t)first.tsdf & 0xff);
    b[3] = (uint8_t)((uint16_t)first.tsdf >> 8);
    b[4] = (uint8_t)(first.w & 0xff);
    b[5] = (uint8_t)(first.w >> 8);
    return 6;
}

/* cu_voxel_run_length_encode_slice (:1367-1417) */
int64_t orc_rle_encode_slice(const orc_voxel *s, int64_t n, int lossless, uint8_t *buf) {
    if (n <= 0) return 0;
    int64_t o = 0;
    orc_voxel old = s[0];
    unsigned count = 0;
    for (int64_t i = 0; i < n; ++i) {
        orc_voxel cur = s[i];
        int same = cur.tsdf == old.tsdf && (!lossless || cur.w == old.w);
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

/* cu_voxel_run_length_decode_slice (:1419-1447), with bounds checks: a
 * zero-length record, a run past the slice end or a truncated stream is an
 * error here (the reference loops or overruns on those). */
int64_t orc_rle_decode_slice(const uint8_t *buf, int64_t nbytes, orc_voxel *out, int64_t n) {
    int64_t p = 0, o = 0;
    while (o < n) {
        if (p + 2 > nbytes) return -1;
        unsigned r = (unsigned)buf[p] | ((unsigned)buf[p + 1] << 8);
        p += 2;
        unsigned cnt = r & 0x3fffu, v = r >> 14;
        orc_voxel val;
        if (v == 1) { val.tsdf = ORC_MAX_TSDF; val.w = 0; }
        else if (v == 2) { val.tsdf = -ORC_MAX_TSDF; val.w = 0; }
        else {
            /* v == 3 literal; v == 0 is never written and decodes as a literal */
            if (p + 4 > nbytes) return -1;
            val.tsdf = (int16_t)((unsigned)buf[p] | ((unsigned)buf[p + 1] << 8));
            val.w = (uint16_t)((unsigned)buf[p + 2] | ((unsigned)buf[p + 3] << 8));
            p += 4;
        }
        if (cnt == 0 || o + cnt > n) return -1;
        for (unsigned i = 0; i < cnt; ++i) out[o + i] = val;
        o += cnt;
    }
    return p;
}

static const char FMT_REF[16] = "VOLUME_TSDF_RGB";   /* cu_kinect_fusion_v1.h:40 */
static const char FMT_LOSSLESS[16] = "VOLUME_TSDF_W32";

/* header (:1303-1310): 16-byte tag, int3 size, min_t, max_t, grid_s; then
 * per slice a uint32 byte count and the slice records (:1345-1351) */
int64_t orc_rle_encode_volume(const orc_voxel *vol, int nx, int ny, int nz, float min_t,
                              float max_t, float grid_s, int lossless, uint8_t *out, int64_t cap) {
    int64_t xy = (int64_t)nx * ny;
    if (cap < 40) return -1;
    memcpy(out, lossless ? FMT_LOSSLESS : FMT_REF, 16);
    int32_t dims[3] = {nx, ny, nz};
    memcpy(out + 16, dims, 12);
    memcpy(out + 28, &min_t, 4);
    memcpy(out + 32, &max_t, 4);
    memcpy(out + 36, &grid_s, 4);
    int64_t o = 40;
    uint8_t *tmp = (uint8_t *)malloc((size_t)(6 * xy + 16));
    for (int z = 0; z < nz; ++z) {
        int64_t sz = orc_rle_encode_slice(vol + z * xy, xy, lossless, tmp);
        if (o + 4 + sz > cap) { free(tmp); return -1; }
        uint32_t s32 = (uint32_t)sz;
        memcpy(out + o, &s32, 4);
        memcpy(out + o + 4, tmp, (size_t)sz);
        o += 4 + sz;
    }
    free(tmp);
    return o;
}

int orc_rle_decode_volume(const uint8_t *img, int64_t nbytes, orc_voxel *vol, int64_t cap_voxels,
                          int dims[3], float params[3]) {
    if (nbytes < 40) return -1;
    if (memcmp(img, FMT_REF, 16) != 0 && memcmp(img, FMT_LOSSLESS, 16) != 0) return -2;
    int32_t d[3];
    memcpy(d, img + 16, 12);
    memcpy(params, img + 28, 12);
    dims[0] = d[0]; dims[1] = d[1]; dims[2] = d[2];
    if (d[0] <= 0 || d[1] <= 0 || d[2] <= 0) return -1;
    if (!vol) return 0;
    int64_t xy = (int64_t)d[0] * d[1];
    if (xy * d[2] > cap_voxels) return -3;
    int64_t p = 40;
    for (int z = 0; z < d[2]; ++z) {
        if (p + 4 > nbytes) return -1;
        uint32_t sz;
        memcpy(&sz, img + p, 4);
        p += 4;
        if (p + (int64_t)sz > nbytes) return -1;
        if (orc_rle_decode_slice(img + p, sz, vol + z * xy, xy) < 0) return -1;
        p += sz;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* adjoints (binary64).  No counterpart in the reference: these are the      */
/* derivatives of the forward restatements above, with every discrete        */
/* choice (cube case, pixel, truncation, clamp) taken from the FP32 mirror   */
/* and held fixed, and every continuous value computed in binary64.          */
/* ------------------------------------------------------------------------ */

static inline double vox_f64(const void *vol, int vtype, int64_t i) {
    return vtype == ORC_VOXEL_SHORT2 ? (double)((const orc_voxel *)vol)[i].tsdf / ORC_MAX_TSDF
                                     : (double)((const orc_voxel_f32 *)vol)[i].tsdf;
}

int64_t orc_mc_edges(const void *vol, int vtype, int nx, int ny, int nz, int64_t *va, int64_t *vb,
                     int64_t cap_verts) {
    int64_t o = 0;
    for (int z = 0; z + 1 < nz; ++z)
        for (int y = 0; y + 1 < ny; ++y)
            for (int x = 0; x + 1 < nx; ++x) {
                int ci = cube_index(vol, vtype, nx, ny, x, y, z);
                int nv = cube_nverts(ci);
                for (int i = 0; i < nv; ++i, ++o) {
                    if (o >= cap_verts) continue;
                    int j = i / 3, kk = i % 3;
                    int e = orc_tri_table[ci][3 * j + 2 - kk];
                    int a = EA[e], b = EB[e];
                    va[o] = lin(nx, ny, x + CX[a], y + CY[a], z + CZ[a]);
                    vb[o] = lin(nx, ny, x + CX[b], y + CY[b], z + CZ[b]);
                }
            }
    return o;
}

/* P = p_a + t (p_b - p_a), t = -f_a / (f_b - f_a + 1e-15)
 * (cu_marching_cubes_v1.cu:256-264) */
int64_t orc_mc_backward_f64(const void *vol, int vtype, int nx, int ny, int nz, double cell,
                            const double *grad_pos, int64_t n, double *grad_f) {
    int64_t o = 0;
    for (int z = 0; z + 1 < nz; ++z)
        for (int y = 0; y + 1 < ny; ++y)
            for (int x = 0; x + 1 < nx; ++x) {
                int ci = cube_index(vol, vtype, nx, ny, x, y, z);
                int nv = cube_nverts(ci);
                for (int i = 0; i < nv; ++i, ++o) {
                    if (o >= n) continue;
                    int j = i / 3, kk = i % 3;
                    int e = orc_tri_table[ci][3 * j + 2 - kk];
                    int a = EA[e], b = EB[e];
                    int64_t la = lin(nx, ny, x + CX[a], y + CY[a], z + CZ[a]);
                    int64_t lb = lin(nx, ny, x + CX[b], y + CY[b], z + CZ[b]);
                    double fa = vox_f64(vol, vtype, la), fb = vox_f64(vol, vtype, lb);
                    double g = 0.0;
                    g += grad_pos[3 * o + 0] * (double)(CX[b] - CX[a]) * cell;
                    g += grad_pos[3 * o + 1] * (double)(CY[b] - CY[a]) * cell;
                    g += grad_pos[3 * o + 2] * (double)(CZ[b] - CZ[a]) * cell;
                    double D = fb - fa + 1e-15;
                    grad_f[la] += g * (-(fb + 1e-15)) / (D * D);
                    grad_f[lb] += g * fa / (D * D);
                }
            }
    return o;
}

/* FP32 decisions of one integrate observation, exactly as orc_integrate
 * takes them.  branch: 0 sdf <= 0, 1 0 < sdf <= max_t, 2 clamped at 1. */
static int decide32(const orc_extrinsic *e, const orc_intrinsic *k, int w, int h, float min_t, float max_t,
                    const float *ds, const float *normals, float px, float py, float pz, int64_t *pix,
                    int *u_out, int *v_out, int *branch) {
    const float *R = e->r;
    float v0 = px - e->t[0], v1 = py - e->t[1], v2 = pz - e->t[2];
    float q0 = R[0] * v0 + R[1] * v1 + R[2] * v2;
    float q1 = R[3] * v0 + R[4] * v1 + R[5] * v2;
    float q2 = R[6] * v0 + R[7] * v1 + R[8] * v2;
    if (q2 < FLT_MIN) return 0;
    float u_f = k->fx * (q0 / q2) + k->cx;
    float v_f = k->fy * (q1 / q2) + k->cy;
    int u = f2i_rn(u_f), v = f2i_rn(v_f);
    if (u < 0 || v < 0 || u >= (w - 2) || v >= (h - 2)) return 0;
    int64_t p = (int64_t)v * w + u;
    float z_val = ds[p];
    if (!(z_val > FLT_MIN)) return 0;
    float qn = sqrtf(q0 * q0 + q1 * q1 + q2 * q2);
    float sdf = z_val - qn;
    if (!(sdf >= -min_t)) return 0;
    int br = 0;
    if (sdf > 0.0f) {
        br = (sdf / max_t > 1.0f) ? 2 : 1;
    }
    if (normals) {
        const float *n = normals + 3 * p;
        if (!vertex_valid(n)) return 0;
        float wgt = -(n[0] * (q0 / qn) + n[1] * (q1 / qn) + n[2] * (q2 / qn));
        if (wgt < FLT_MIN) return 0;
    }
    *pix = p;
    *u_out = u;
    *v_out = v;
    *branch = br;
    return 1;
}

/* binary64 values of one observation given its decisions */
typedef struct {
    double s, w0, z, dsdz, c;
} orc_obs64;

static orc_obs64 observe64(const orc_extrinsic *e, const orc_intrinsic *k, double min_t, double max_t,
                           const float *nrm, int u, int v, int branch, double depth, double px, double py,
                           double pz) {
    const float *R = e->r;
    double v0 = px - e->t[0], v1 = py - e->t[1], v2 = pz - e->t[2];
    double q0 = R[0] * v0 + R[1] * v1 + R[2] * v2;
    double q1 = R[3] * v0 + R[4] * v1 + R[5] * v2;
    double q2 = R[6] * v0 + R[7] * v1 + R[8] * v2;
    double cx = ((double)u - k->cx) / k->fx, cy = ((double)v - k->cy) / k->fy;
    orc_obs64 o;
    o.c = sqrt(cx * cx + cy * cy + 1.0);
    o.z = depth * o.c;
    double qn = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
    double s = o.z - qn;
    if (branch == 0) { o.s = s / min_t; o.dsdz = 1.0 / min_t; }
    else if (branch == 1) { o.s = s / max_t; o.dsdz = 1.0 / max_t; }
    else { o.s = 1.0; o.dsdz = 0.0; }
    double wgt = 1.0;
    if (nrm) wgt = -(nrm[0] * (q0 / qn) + nrm[1] * (q1 / qn) + nrm[2] * (q2 / qn));
    o.w0 = wgt / o.z;
    return o;
}

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

/* scaled FP32 depth of every frame, from (float)depth */
static float *scaled_frames(const orc_intrinsic *k, int n_frames, int w, int h, const double *depth) {
    size_t plane = (size_t)w * h;
    float *d32 = (float *)malloc(sizeof(float) * plane);
    float *ds = (float *)malloc(sizeof(float) * plane * n_frames);
    for (int f = 0; f < n_frames; ++f) {
        for (size_t i = 0; i < plane; ++i) d32[i] = (float)depth[f * plane + i];
        orc_depth_scale(k, w, h, d32, ds + f * plane);
    }
    free(d32);
    return ds;
}

void orc_integrate_seq_f64(const float *vol0, int nx, int ny, int nz, float min_t, float max_t, float grid_s,
                           const orc_intrinsic *k, int n_frames, const orc_extrinsic *poses, int w, int h,
                           const double *depth, const float *normals, int is_dynamic, double *F, double *W,
                           uint64_t *signature, int nthreads) {
    nthreads = nthreads_or_default(nthreads);
    size_t plane = (size_t)w * h;
    float *ds = scaled_frames(k, n_frames, w, h, depth);
    uint64_t sig = 0;
#pragma omp parallel for collapse(2) schedule(static) num_threads(nthreads) reduction(+ : sig)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            float px = -grid_s;
            for (int x = 0; x < nx; ++x) {
                px += grid_s;
                int64_t li = lin(nx, ny, x, y, z);
                double Fc = vol0 ? vol0[2 * li] : -1.0, Wc = vol0 ? vol0[2 * li + 1] : 0.0;
                for (int f = 0; f < n_frames; ++f) {
                    int64_t pix; int u, v, br;
                    const float *nf = normals ? normals + 3 * plane * f : NULL;
                    int ok = decide32(poses + f, k, w, h, min_t, max_t, ds + plane * f, nf, px,
                                      (float)y * grid_s, (float)z * grid_s, &pix, &u, &v, &br);
                    sig += mix64(((uint64_t)li * (uint64_t)n_frames + (uint64_t)f) * 0x9e3779b97f4a7c15ULL +
                                 (ok ? (uint64_t)pix * 4u + (uint64_t)br + 1u : 0u));
                    if (!ok) continue;
                    orc_obs64 o = observe64(poses + f, k, min_t, max_t, nf ? nf + 3 * pix : NULL, u, v, br,
                                            depth[plane * f + pix], px, (double)((float)y * grid_s),
                                            (double)((float)z * grid_s));
                    double wv = o.w0;
                    if (is_dynamic) { double d = o.s - Fc; wv = wv * (1.0 + d * d * 10.0); }
                    double Wn = Wc + wv;
                    Fc = (Wc * Fc + wv * o.s) / Wn;
                    Wc = Wn;
                }
                F[li] = Fc;
                W[li] = Wc;
            }
        }
    free(ds);
    if (signature) *signature = sig;
}

void orc_integrate_seq_backward_f64(const float *vol0, int nx, int ny, int nz, float min_t, float max_t,
                                    float grid_s, const orc_intrinsic *k, int n_frames,
                                    const orc_extrinsic *poses, int w, int h, const double *depth,
                                    const float *normals, int is_dynamic, const double *gF_end,
                                    const double *gW_end, double *g_depth, double *gF0, double *gW0,
                                    int nthreads) {
    nthreads = nthreads_or_default(nthreads);
    size_t plane = (size_t)w * h;
    float *ds = scaled_frames(k, n_frames, w, h, depth);
#pragma omp parallel num_threads(nthreads)
    {
        double *Fp = (double *)malloc(sizeof(double) * n_frames);
        double *Wp = (double *)malloc(sizeof(double) * n_frames);
        orc_obs64 *ob = (orc_obs64 *)malloc(sizeof(orc_obs64) * n_frames);
        int64_t *px_of = (int64_t *)malloc(sizeof(int64_t) * n_frames);
        int *okf = (int *)malloc(sizeof(int) * n_frames);
#pragma omp for collapse(2) schedule(dynamic, 4)
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y) {
                float px = -grid_s;
                for (int x = 0; x < nx; ++x) {
                    px += grid_s;
                    int64_t li = lin(nx, ny, x, y, z);
                    double gF = gF_end[li], gW = gW_end ? gW_end[li] : 0.0;
                    if (gF != 0.0 || gW != 0.0) {
                        double Fc = vol0 ? vol0[2 * li] : -1.0, Wc = vol0 ? vol0[2 * li + 1] : 0.0;
                        for (int f = 0; f < n_frames; ++f) {
                            int64_t pix; int u, v, br;
                            const float *nf = normals ? normals + 3 * plane * f : NULL;
                            Fp[f] = Fc;
                            Wp[f] = Wc;
                            okf[f] = decide32(poses + f, k, w, h, min_t, max_t, ds + plane * f, nf, px,
                                              (float)y * grid_s, (float)z * grid_s, &pix, &u, &v, &br);
                            if (!okf[f]) continue;
                            px_of[f] = pix;
                            ob[f] = observe64(poses + f, k, min_t, max_t, nf ? nf + 3 * pix : NULL, u, v, br,
                                              depth[plane * f + pix], px, (double)((float)y * grid_s),
                                              (double)((float)z * grid_s));
                            double wv = ob[f].w0;
                            if (is_dynamic) { double d = ob[f].s - Fc; wv = wv * (1.0 + d * d * 10.0); }
                            double Wn = Wc + wv;
                            Fc = (Wc * Fc + wv * ob[f].s) / Wn;
                            Wc = Wn;
                        }
                        for (int f = n_frames - 1; f >= 0; --f) {
                            if (!okf[f]) continue;
                            const orc_obs64 o = ob[f];
                            double mult = 1.0, d = 0.0, wv = o.w0;
                            if (is_dynamic) { d = o.s - Fp[f]; mult = 1.0 + d * d * 10.0; wv = wv * mult; }
                            double Wn = Wp[f] + wv;
                            double Fn = (Wp[f] * Fp[f] + wv * o.s) / Wn;
                            double gs = gF * wv / Wn;
                            double gw = gF * (o.s - Fn) / Wn + gW;
                            double gFp = gF * Wp[f] / Wn;
                            double gWp = gF * (Fp[f] - Fn) / Wn + gW;
                            double gw0 = gw;
                            if (is_dynamic) {
                                double t = gw * o.w0 * 20.0 * d;
                                gs += t;
                                gFp -= t;
                                gw0 = gw * mult;
                            }
                            double gz = gs * o.dsdz - gw0 * o.w0 / o.z;
                            double add = gz * o.c;
#pragma omp atomic
                            g_depth[plane * f + px_of[f]] += add;
                            gF = gFp;
                            gW = gWp;
                        }
                    }
                    if (gF0) gF0[li] = gF;
                    if (gW0) gW0[li] = gW;
                }
            }
        free(Fp); free(Wp); free(ob); free(px_of); free(okf);
    }
    free(ds);
}

/* ------------------------------------------------------------------------ */
/* indexed mesh vertices (no counterpart in the reference): the vertex of    */
/* grid edge `key` = 3 * lin(x, y, z) + axis, interpolated from the lower    */
/* voxel to the upper one with vertex_interp (:256-264), FP32 mirror.        */
/* ------------------------------------------------------------------------ */
void orc_mc_edge_vertices(const void *vol, int vtype, int nx, int ny, int nz, float cell, const int64_t *keys,
                          int64_t n, float *pos, float *normals, int32_t *vi2vox) {
    for (int64_t i = 0; i < n; ++i) {
        int64_t k = keys[i];
        int axis = (int)(k % 3);
        int64_t li = k / 3;
        int x = (int)(li % nx), y = (int)((li / nx) % ny), z = (int)(li / ((int64_t)nx * ny));
        int dx = axis == 0, dy = axis == 1, dz = axis == 2;
        float f0 = vox_f(vol, vtype, li);
        float f1 = vox_f(vol, vtype, lin(nx, ny, x + dx, y + dy, z + dz));
        float t = (0.0f - f0) / (f1 - f0 + 1e-15f);
        float P[3] = {interp1(node(x, cell), node(x + dx, cell), t), interp1(node(y, cell), node(y + dy, cell), t),
                      interp1(node(z, cell), node(z + dz, cell), t)};
        if (pos) { pos[3 * i] = P[0]; pos[3 * i + 1] = P[1]; pos[3 * i + 2] = P[2]; }
        if (vi2vox)
            for (int d = 0; d < 3; ++d) vi2vox[3 * i + d] = (int)floorf(P[d] / cell - 0.5f);
        if (normals) orc_surface_normal(vol, vtype, nx, ny, nz, cell, P, normals + 3 * i);
    }
}

/* ------------------------------------------------------------------------ */
/* ray casting (cu_kinect_fusion_v1.cu:551-659, 786-986), short2 volumes,    */
/* FP32 mirror.  Colour is not part of the voxel, so it is not produced.     */
/* ------------------------------------------------------------------------ */

/* d_voxel_extract_trilinear_interpolated_sdf (:551-657): the samples in the
 * order V000, V100, V010, V001, V101, V011, V110, V111; the first +-32766 met
 * returns +-1; float_interpolation_trilinear (cu_math_functions.h:107-111) */
static float trilinear_sdf(const orc_voxel *vol, int nx, int ny, const float p[3]) {
    int pi[3] = {(int)p[0], (int)p[1], (int)p[2]};
    float t[3] = {p[0] - (float)pi[0], p[1] - (float)pi[1], p[2] - (float)pi[2]};
    static const int O[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 0}, {1, 1, 1}};
    float s[8];
    for (int k = 0; k < 8; ++k) {
        int16_t v = vol[lin(nx, ny, pi[0] + O[k][0], pi[1] + O[k][1], pi[2] + O[k][2])].tsdf;
        if (v == ORC_MAX_TSDF) return 1.0f;
        if (v == -ORC_MAX_TSDF) return -1.0f;
        s[k] = unpack_tsdf(v);
    }
    float a = 1.0f - t[0], b = 1.0f - t[1], c = 1.0f - t[2];
    float x = t[0], y = t[1], z = t[2];
    return s[0] * a * b * c + s[1] * x * b * c + s[2] * a * y * c + s[3] * a * b * z + s[4] * x * b * z +
           s[5] * a * y * z + s[6] * x * y * c + s[7] * x * y * z;
}

/* camera set-up of _cu_voxel_extract_depth_and_normal_map (:965-986):
 * K (cu_geometry_functions.h:248-255), M = K R^T (matrix33_mt), IM = M^-1
 * (float33_inv, cu_vector_functions.h:555-575), camera centre t / grid_s.
 * Matrices are three column vectors m[j][i] (column j, component i).
 * Returns 0 when M is singular (the reference then launches nothing). */
int orc_raycast_setup(const orc_intrinsic *k, const orc_extrinsic *e, float grid_s, float IM[3][3], float cc[3]) {
    float K[3][3] = {{k->fx, 0.0f, 0.0f}, {0.0f, k->fy, 0.0f}, {k->cx, k->cy, 1.0f}};
    float R[3][3];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) R[j][i] = e->r[3 * j + i];
    float M[3][3];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) M[j][i] = K[0][i] * R[0][j] + K[1][i] * R[1][j] + K[2][i] * R[2][j];
    float A = M[2][2] * M[1][1] - M[2][1] * M[1][2];
    float B = M[0][2] * M[2][1] - M[0][1] * M[2][2];
    float C = M[0][1] * M[1][2] - M[0][2] * M[1][1];
    float det = M[0][0] * A + M[1][0] * B + M[2][0] * C;
    if (det > -FLT_EPSILON && det < FLT_EPSILON) return 0;
    IM[0][0] = A;
    IM[0][1] = B;
    IM[0][2] = C;
    IM[1][0] = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    IM[1][1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
    IM[1][2] = M[0][2] * M[1][0] - M[0][0] * M[1][2];
    IM[2][0] = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    IM[2][1] = M[0][1] * M[2][0] - M[0][0] * M[2][1];
    IM[2][2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) IM[j][i] = IM[j][i] / det;
    for (int i = 0; i < 3; ++i) cc[i] = e->t[i] / grid_s;
    return 1;
}

/* d_voxel_extract_depth_and_normal_map (:786-963) for every pixel.  depth:
 * w*h metres (0 where nothing is hit); normal: w*h*3 (may be NULL),
 * (0,0,0) where nothing is hit.  Returns 0 (and writes nothing) when the
 * camera matrix is singular. */
int orc_raycast(const orc_voxel *vol, int nx, int ny, int nz, float grid_s, const orc_intrinsic *k,
                const orc_extrinsic *e, int w, int h, float *depth, float *normal, int nthreads) {
    float IM[3][3], cc[3];
    if (!orc_raycast_setup(k, e, grid_s, IM, cc)) return 0;
    nthreads = nthreads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int64_t idx = (int64_t)y * w + x;
            depth[idx] = 0.0f;
            if (normal) normal[3 * idx] = normal[3 * idx + 1] = normal[3 * idx + 2] = 0.0f;
            const float margin = 1.0f;
            float x_max = (float)nx - margin, y_max = (float)ny - margin, z_max = (float)nz - margin;
            const float dt_max = 1.0f, dt_min = 0.25f;
            float dt = dt_max;
            int dt_status = 0;
            float fx = (float)x, fy = (float)y;
            /* float33_mv_2 (cu_vector_functions.h:623-626, matrix33_mv_2) */
            float rd[3] = {IM[0][0] * fx + IM[1][0] * fy + IM[2][0], IM[0][1] * fx + IM[1][1] * fy + IM[2][1],
                           IM[0][2] * fx + IM[1][2] * fy + IM[2][2]};
            unit3(rd);
            for (int i = 0; i < 3; ++i)
                if (rd[i] == 0.0f) rd[i] = (float)1e-15;
            float t_min = FLT_MAX, t_max = 0.0f, t, t1 = 0.0f, t2, sdf, sdf1 = 1.0f;
            const float lo[3] = {margin, margin, margin}, hi[3] = {x_max, y_max, z_max};
            /* entry / exit over the six faces x = margin, x_max, y = ..., z = ... */
            for (int ax = 0; ax < 3; ++ax) {
                int a1 = ax == 0 ? 1 : 0, a2 = ax == 2 ? 1 : 2;
                for (int side = 0; side < 2; ++side) {
                    float plane = side == 0 ? margin : hi[ax];
                    t = (plane - cc[ax]) / rd[ax];
                    if (t > 0) {
                        float u1 = rd[a1] * t + cc[a1];
                        float u2 = rd[a2] * t + cc[a2];
                        if (u1 > lo[a1] && u1 < hi[a1] && u2 > lo[a2] && u2 < hi[a2]) {
                            if (t < t_min) t_min = t;
                            if (t > t_max) t_max = t;
                        }
                    }
                }
            }
            if (t_min == FLT_MAX && t_max == 0.0f) continue;
            if (t_min == t_max) t_min = dt * margin;
            for (t = t_min; t < t_max; t += dt) {
                float p[3] = {rd[0] * t + cc[0], rd[1] * t + cc[1], rd[2] * t + cc[2]};
                if (p[0] < 0.0f || p[1] < 0.0f || p[2] < 0.0f || p[0] >= x_max || p[1] >= y_max || p[2] >= z_max)
                    continue;
                sdf = trilinear_sdf(vol, nx, ny, p);
                if (sdf < 0.0f && sdf > -1.0f && sdf1 >= 0.0f && sdf1 < 1.0f) {
                    t2 = t1 - dt * sdf1 / (sdf - sdf1); /* eq. (15) */
                    float np[3] = {rd[0] * t2, rd[1] * t2, rd[2] * t2};
                    float tp[3] = {np[0] + cc[0], np[1] + cc[1], np[2] + cc[2]};
                    float p2x = (fx - k->cx) / k->fx, p2y = (fy - k->cy) / k->fy;
                    float nn = sqrtf(np[0] * np[0] + np[1] * np[1] + np[2] * np[2]);
                    depth[idx] = nn / sqrtf(p2x * p2x + p2y * p2y + 1.0f) * grid_s;
                    if (normal) {
                        float sn[3];
                        orc_surface_normal(vol, ORC_VOXEL_SHORT2, nx, ny, nz, 1.0f, tp, sn);
                        /* float33_tv (matrix33_tv): R^T n */
                        for (int i = 0; i < 3; ++i)
                            normal[3 * idx + i] = e->r[3 * i] * sn[0] + e->r[3 * i + 1] * sn[1] + e->r[3 * i + 2] * sn[2];
                    }
                    break;
                } else if (sdf1 <= 0.0f && sdf1 > -1.0f && sdf >= 0.0f && sdf < 1.0f) {
                    break; /* back face */
                }
                if (sdf > -1.0f && sdf < 1.0f) {
                    if (!dt_status) {
                        t -= dt;
                        dt_status = 1;
                        dt = dt_min;
                        continue;
                    }
                } else if (dt_status) {
                    dt_status = 0;
                    dt = dt_max;
                }
                t1 = t;
                sdf1 = sdf;
            }
        }
    return 1;
}
