/*
 * mcg.h -- C ABI of the GB300 TSDF -> mesh library (libmcg.so).
 *
 * Plain C: pointers, sizes and status codes only.  Every entry point takes
 * an explicit CUDA stream (mcg_stream_t == cudaStream_t, NULL = legacy
 * default stream) and keeps all state in an mcg_context, so calls on
 * different contexts are independent.  Device pointers are CUDA device (or
 * managed) allocations; "host" pointers are ordinary host memory.
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the reference project root; mc.cu = cu_marching_cubes_v1.cu,
 * kf.cu / kf.h = cu_kinect_fusion_v1.cu / .h).  The reference aborts the
 * process on CUDA errors (cu_device.h checkCudaErrors); this ABI returns a
 * status instead.
 */
#ifndef MCG_H
#define MCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCG_VERSION 100

typedef struct CUstream_st *mcg_stream_t; /* identical to cudaStream_t */
typedef struct mcg_context mcg_context;   /* opaque per-instance state */

typedef enum mcg_status {
    MCG_OK = 0,
    MCG_ERR_INVALID_ARG = 1, /* bad pointer, size or combination of arguments */
    MCG_ERR_CAPACITY = 2,    /* output larger than the buffers given; counts hold the need */
    MCG_ERR_CUDA = 3,        /* a CUDA call failed; mcg_last_cuda_error() has the code */
    MCG_ERR_TIMEOUT = 4,     /* a bounded device-side wait expired */
    MCG_ERR_IO = 5,          /* file could not be opened / read / written */
    MCG_ERR_FORMAT = 6,      /* malformed RLE stream or file header */
    MCG_ERR_STATE = 7,       /* call order violated (e.g. generate without classify) */
    MCG_ERR_TOO_LARGE = 8    /* input above a fixed limit (mcg_mc_extract_noalloc's scratch, mcg_integrate_backward's frame count) */
} mcg_status;

/* voxel storage types */
enum {
    MCG_VOXEL_SHORT2 = 0, /* structure.h:14-18 cu_voxel_t {short tsdf; ushort w}, == short2 */
    MCG_VOXEL_FLOAT2 = 1  /* {float tsdf; float w}: FP32 volume of the differentiable path */
};

/* structure.h:29-35 vertex_voxel, 28 bytes, byte-compatible */
typedef struct mcg_vertex_voxel {
    float x, y, z;        /* ver_pos */
    int32_t vx, vy, vz;   /* vox_pos = floor(ver_pos / cell - 0.5) */
    int16_t tsdf, w;      /* voxel vox_pos as stored */
} mcg_vertex_voxel;

/* cu_geometry_functions.h:96-101 float_camera_intrinsic (fc, cc, dc[5]) */
typedef struct mcg_intrinsic { float fx, fy, cx, cy; float dc[5]; } mcg_intrinsic;
/* cu_geometry_functions.h:104-108 float_camera_extrinsic, camera -> global:
 * r = rotation, column-major (three float3 columns), t = translation */
typedef struct mcg_extrinsic { float r[9]; float t[3]; } mcg_extrinsic;

/* structure.h:20-27 cu_voxel, minus the truncation fields.  data is a dense
 * [z][y][x] device array (x fastest, no pitch), aligned to the voxel size
 * (4 bytes for short2, 8 for float2; MCG_ERR_INVALID_ARG otherwise). */
typedef struct mcg_volume {
    const void *data;
    int32_t nx, ny, nz;
    int32_t voxel_type; /* MCG_VOXEL_* */
    float cell;         /* grid_s, voxel edge length */
} mcg_volume;

/* Outputs of one extraction; every pointer is a device array or NULL.
 * Soup arrays hold up to capacity_vertices entries (3 per triangle). */
typedef struct mcg_mesh_out {
    mcg_vertex_voxel *soup; /* MarchingCubes::run triangles_buffer            */
    float *soup_normals;    /* float3 per soup vertex (d_voxel_extract_surface_normals) */
    int32_t *vi2vox;        /* int3 per soup vertex (vertexindex_to_voxel)    */
    int16_t *ver_voxel;     /* nx*ny*nz shorts: zeroed, then tsdf at each vertex voxel */
    int64_t *tri_cube;      /* linear id z*nx*ny + y*nx + x of each triangle's cube */
    int64_t capacity_vertices;
} mcg_mesh_out;

typedef struct mcg_mesh_counts {
    int64_t occupied;  /* cubes that emit triangles (getOccupiedVoxels' count) */
    int64_t triangles;
    int64_t vertices;  /* soup vertices, 3 * triangles */
    int64_t active_bricks; /* 32x8x8-cube bricks that emit triangles */
    int32_t status;    /* MCG_OK, or MCG_ERR_CAPACITY if the last generate was truncated */
    int32_t reserved;
} mcg_mesh_counts;

/* ---- context ----------------------------------------------------------- */
const char *mcg_status_string(int status);
int mcg_version(void);
/* replaces the globals of mc.cu:29-51 (volume_size, textures, counters) */
mcg_status mcg_create(mcg_context **out, int device);
mcg_status mcg_destroy(mcg_context *ctx);
int mcg_last_cuda_error(const mcg_context *ctx);

/* ---- voxel init: kf.cu:364-398 (d_voxel_initialize in cu_voxel_new) ----- */
/* every voxel -> {tsdf = -32766, w = 0} (FLOAT2: {-1, 0}) */
mcg_status mcg_voxel_init(mcg_context *ctx, void *vol, int32_t voxel_type, int64_t n_voxels,
                          mcg_stream_t stream);

/* ---- marching cubes: mc.cu:416-467 MarchingCubes::run ------------------- */
/* Count phase (getOccupiedVoxels mc.cu:185-206 + computeOffsetsAndTotalVertexes
 * mc.cu:208-225).  Asynchronous; the counts become readable through
 * mcg_mc_counts once the stream reaches this point. */
mcg_status mcg_mc_classify(mcg_context *ctx, const mcg_volume *vol, mcg_stream_t stream);
/* Waits for the last classify/generate on ctx and reports counts. */
mcg_status mcg_mc_counts(mcg_context *ctx, mcg_mesh_counts *out);
/* Generation phase (generateTriangles mc.cu:372-396 + normals kf.cu:3236-3242)
 * over the volume passed to the preceding mcg_mc_classify on this ctx.
 * Writes at most capacity_vertices soup vertices; the rest is dropped and
 * mcg_mc_counts reports MCG_ERR_CAPACITY with the full size. */
mcg_status mcg_mc_generate(mcg_context *ctx, const mcg_volume *vol, const mcg_mesh_out *out,
                           mcg_stream_t stream);
/* MarchingCubes::run (mc.cu:416-467) in one call, no host synchronisation:
 * the same soup, side outputs, order and counts as mcg_mc_classify +
 * mcg_mc_generate.  With mcg_mc_config.fused set, short2 volumes of at
 * least 132 x 10 x 10 voxels (68 x 10 x 10 with 2-brick items) that TMA can
 * describe run as one fused launch (count, offsets and generation
 * together); the counts are then readable
 * through mcg_mc_counts, but the count phase's brick list is not kept, so
 * mcg_mc_generate / mcg_mc_backward on this ctx need a mcg_mc_classify first
 * (MCG_ERR_STATE otherwise).  Other volumes take the two launches. */
mcg_status mcg_mc_extract(mcg_context *ctx, const mcg_volume *vol, const mcg_mesh_out *out,
                          mcg_stream_t stream);
/* Launch configuration of the marching-cubes kernels on a context (no
 * counterpart in the reference; the reference's launch shapes are fixed).
 * Defaults are the measured best on GB300 for the 512^3 fusion volume
 * (fused 0, classify_shape 4, gen_fixed_rounds 3); the autotuner
 * (marching_cube_gb300.tune) times the choices on a volume and sets them.
 *   fused            mcg_mc_extract: 0 always the count + generate launches;
 *                    1 the fused launch where it applies, work items of 4
 *                    bricks (132-voxel tiles, 256 threads); 2 the same with
 *                    items of 2 bricks (68-voxel tiles, 128 threads)
 *   classify_shape   count-pass work item, 0..5: 2 bricks in a 68-voxel box,
 *                    2 stages (0); 4 bricks with a separate halo box, 2
 *                    stages (1) or 4 stages of 512 threads (2); 4 bricks in a
 *                    132-voxel box, 2 stages (3) or 1 stage (4); 2 bricks in a
 *                    68-voxel box, 1 stage (5) -- all 256 threads unless said
 *   gen_fixed_rounds generate: bricks each CTA takes in fixed serpentine
 *                    rounds before drawing from the counter, 0..16 */
typedef struct mcg_mc_config {
    int32_t fused;
    int32_t classify_shape;
    int32_t gen_fixed_rounds;
    int32_t reserved;
} mcg_mc_config;
mcg_status mcg_mc_get_config(const mcg_context *ctx, mcg_mc_config *cfg);
mcg_status mcg_mc_set_config(mcg_context *ctx, const mcg_mc_config *cfg);
/* Measurement (no counterpart in the reference).  With enable != 0, every
 * later count phase on ctx records CUDA events on its stream around the
 * classify kernel alone (not the scan), and every fused mcg_mc_extract around
 * its one kernel; mcg_mc_count_kernel_ms waits for the last such pair and
 * gives its duration in milliseconds (MCG_ERR_STATE when none was recorded).
 * The events keep the next launch from starting while the kernel drains, so
 * leave this off outside measurement. */
mcg_status mcg_set_kernel_timing(mcg_context *ctx, int32_t enable);
mcg_status mcg_mc_count_kernel_ms(mcg_context *ctx, float *ms);
/* Indexed extraction (no counterpart in the reference, whose OBJ writer
 * merges soup vertices by their printed coordinates, kf.cu:3625-3726): one
 * vertex per grid edge the surface crosses, shared by every triangle using
 * it.  A vertex is on the edge from voxel (x, y, z) to its +1 neighbour
 * along `axis`; vertex_edge names it 3 * (linear index of (x, y, z)) + axis
 * (0 x, 1 y, 2 z).  Its position is mc.cu:256-264's interpolation taken from
 * the lower voxel to the upper one; its normal is kf.cu:3146-3242's at that
 * position.  Triangles are the soup's, in the soup's order and winding,
 * as 3 vertex indices.  Every output pointer may be NULL. */
typedef struct mcg_indexed_out {
    float *positions;      /* 3 floats per vertex */
    float *normals;        /* 3 floats per vertex */
    int32_t *vi2vox;       /* 3 ints per vertex: floor(P / cell - 0.5) (mc.cu:336-343) */
    int64_t *vertex_edge;  /* 1 per vertex */
    uint32_t *triangles;   /* 3 vertex indices per triangle */
    int64_t *tri_cube;     /* 1 per triangle: linear index of its cube */
    int64_t capacity_vertices;   /* <= 2^32 - 1 */
    int64_t capacity_triangles;
} mcg_indexed_out;
/* Count phase of the indexed mesh; mcg_mc_counts then reports triangles
 * and vertices = unique vertices.  Asynchronous. */
mcg_status mcg_mc_classify_indexed(mcg_context *ctx, const mcg_volume *vol, mcg_stream_t stream);
/* Writes at most capacity_vertices vertices and capacity_triangles
 * triangles; mcg_mc_counts reports MCG_ERR_CAPACITY with the full sizes.
 * Keeps 12 bytes per voxel of edge -> vertex map in ctx (touched only at
 * crossed edges). */
mcg_status mcg_mc_generate_indexed(mcg_context *ctx, const mcg_volume *vol, const mcg_indexed_out *out,
                                   mcg_stream_t stream);
mcg_status mcg_mc_extract_indexed(mcg_context *ctx, const mcg_volume *vol, const mcg_indexed_out *out,
                                  mcg_stream_t stream);
/* Slabs (no counterpart in the reference): the count phase, and with it the
 * next mcg_mc_generate, over the cubes with z0 <= z < z1 only, z0 a multiple
 * of 8 (the brick depth), 0 <= z0 < z1 <= nz - 1.  Soup offsets start at 0
 * in each slab; positions, voxels, tri_cube and normals are those of the
 * whole volume, and the slabs' soups of consecutive ranges concatenate to
 * the whole volume's soup.  This is the unit a multi-GPU split hands to
 * each device; the per-slab vertex totals are the only exchange.  ver_voxel
 * is not available for a slab short of the whole volume (MCG_ERR_INVALID_ARG:
 * it is cleared whole before the scatter). */
mcg_status mcg_mc_classify_slab(mcg_context *ctx, const mcg_volume *vol, int32_t z0, int32_t z1,
                                mcg_stream_t stream);
mcg_status mcg_mc_extract_slab(mcg_context *ctx, const mcg_volume *vol, int32_t z0, int32_t z1,
                               const mcg_mesh_out *out, mcg_stream_t stream);
/* Batched extraction: nvol volumes of any sizes (same voxel type) in one
 * launch per pass (replaces a loop of MarchingCubes::run calls).  Outputs
 * of volume v go to outs[v], in the same order and bit-identical to a
 * single-volume extraction of that volume.  counts: nvol entries.
 * mcg_mc_extract_batched chains the count, scan and generate launches on
 * the device (preallocated outputs, no host round trip); classify, counts,
 * generate size the outputs from the counts first.  Inside a stream capture
 * the calls allocate and wait for nothing: make the same call once outside
 * the capture first (MCG_ERR_STATE otherwise); the graph keeps its own copy
 * of the volume table, so later calls on the context may use other
 * batches no larger than the captured one. */
mcg_status mcg_mc_classify_batched(mcg_context *ctx, const mcg_volume *vols, int32_t nvol, mcg_stream_t stream);
mcg_status mcg_mc_counts_batched(mcg_context *ctx, mcg_mesh_counts *counts, int32_t nvol);
mcg_status mcg_mc_generate_batched(mcg_context *ctx, const mcg_volume *vols, const mcg_mesh_out *outs,
                                   int32_t nvol, mcg_stream_t stream);
mcg_status mcg_mc_extract_batched(mcg_context *ctx, const mcg_volume *vols, const mcg_mesh_out *outs,
                                  int32_t nvol, mcg_stream_t stream);
/* No counterpart in the reference.  The same extraction as mcg_mc_extract
 * for callers that cannot allocate device memory -- a process whose device
 * memory is owned by another allocator (a caching allocator or an arena
 * reserved at start-up, where a stray cudaMalloc can fail or fragment the
 * budget), or a real-time loop that forbids allocation once running
 * (cudaMalloc/cudaFree may synchronise the device and take unbounded time).
 * It takes no context and allocates nothing itself: its scratch is one
 * static device array of MCG_NOALLOC_SCRATCH_BYTES (about 1.75 MiB), held on
 * every device that loads the library's extraction code until the process
 * exits.  CUDA reserves that array (with the code) when it loads the code
 * onto a device: under lazy module loading (CUDA_MODULE_LOADING=LAZY, the
 * default) at the first call on that device that uses the extraction
 * kernels -- often this function's first call -- and at context creation
 * with CUDA_MODULE_LOADING=EAGER.  So make one call on each device before
 * device memory is committed to the other allocator or the real-time loop
 * starts, and before any stream capture.  Volumes with more than
 * MCG_NOALLOC_MAX_BRICKS bricks of 32x8x8 cubes (e.g. larger than 513^3
 * voxels) are rejected with MCG_ERR_TOO_LARGE before anything is launched.
 * Each call looks up the array's device address on the current device
 * (cudaGetSymbolAddress) and clears the parts of it that must start at zero,
 * so a call that failed half-way leaves nothing behind for the next one.
 * Every call shares the one array, so calls whose work overlaps on the GPU
 * (other streams, other host threads) race and corrupt each other's
 * results: serialise them.  The call waits for its stream to finish and
 * fills *counts (status MCG_ERR_CAPACITY if the soup was truncated: the
 * records that fit are written, in the order of mcg_mc_extract). */
#define MCG_NOALLOC_MAX_BRICKS 65536
#define MCG_NOALLOC_SCRATCH_BYTES (65536 * 28 + 256)
mcg_status mcg_mc_extract_noalloc(const mcg_volume *vol, const mcg_mesh_out *out,
                                  mcg_mesh_counts *counts, mcg_stream_t stream);
/* kf.cu:3227-3242 d_voxel_extract_surface_normal(s) for n arbitrary vertex
 * records (the normal of ver_pos); normals is float3[n] */
mcg_status mcg_mc_normals(mcg_context *ctx, const mcg_volume *vol, const mcg_vertex_voxel *verts,
                          int64_t n, float *normals, mcg_stream_t stream);

/* Adjoint of the soup positions (no counterpart in the reference; the
 * positions follow mc.cu:243-264).  grad_pos: dL/dP, float3 per soup vertex
 * in the order of the last mcg_mc_generate on ctx for this volume, the first
 * n_vertices of them.  Accumulates dL/df into grad_f (one float per voxel,
 * f = tsdf for FLOAT2 volumes, tsdf/32766 for SHORT2); the caller
 * initialises grad_f.  Topology is held fixed (the derivative of the cube
 * cases is zero almost everywhere).  FP32 accumulation with atomics. */
mcg_status mcg_mc_backward(mcg_context *ctx, const mcg_volume *vol, const float *grad_pos, int64_t n_vertices,
                           float *grad_f, mcg_stream_t stream);

/* ---- depth maps: kf.cu:99-151 (d_kinect_depth_to_meter, d_img_meter_to_vertex,
 * d_img_vertex_to_normal), fused --------------------------------------------- */
/* depth_mm: uint16 millimetres [h][w] (device).  meter/vertex/normal may be
 * NULL individually.  Invalid metre = 0, invalid vertex/normal = (0,0,0). */
mcg_status mcg_depth_to_maps(mcg_context *ctx, const mcg_intrinsic *k, int32_t w, int32_t h,
                             const uint16_t *depth_mm, float depth_min, float depth_max,
                             float *meter, float *vertex, float *normal, mcg_stream_t stream);
/* kf.cu:116-127 on a metre image */
mcg_status mcg_meter_to_vertex(mcg_context *ctx, const mcg_intrinsic *k, int32_t w, int32_t h,
                               const float *meter, float *vertex, mcg_stream_t stream);
/* kf.cu:130-151 */
mcg_status mcg_vertex_to_normal(mcg_context *ctx, int32_t w, int32_t h, const float *vertex,
                                float *normal, mcg_stream_t stream);

/* ---- integrate: kf.cu:534-549 _cu_voxel_volumetric_integration ---------- */
/* Projective TSDF update of vol (device, in place) with one depth frame in
 * metres (device float [h][w]).  normals: NULL or float3 [h][w] camera-frame
 * normal map (normal-weighted update).  Colour is not part of the volume. */
mcg_status mcg_integrate(mcg_context *ctx, void *vol, int32_t voxel_type, int32_t nx, int32_t ny,
                         int32_t nz, float min_t, float max_t, float grid_s,
                         const mcg_intrinsic *k, const mcg_extrinsic *e, int32_t w, int32_t h,
                         const float *depth_m, const float *normals, int32_t is_dynamic,
                         mcg_stream_t stream);

/* Same update with the camera pose read from device memory: pose_dev holds
 * 12 floats, the rotation column-major (r[9]) then t[3], as mcg_extrinsic.
 * A CUDA graph captured around this call stays valid when the pose buffer
 * is rewritten between replays. */
mcg_status mcg_integrate_device_pose(mcg_context *ctx, void *vol, int32_t voxel_type, int32_t nx, int32_t ny,
                                     int32_t nz, float min_t, float max_t, float grid_s, const mcg_intrinsic *k,
                                     const float *pose_dev, int32_t w, int32_t h, const float *depth_m,
                                     const float *normals, int32_t is_dynamic, mcg_stream_t stream);

/* Adjoint of n_frames integrate steps on a FLOAT2 volume (no counterpart in
 * the reference; the forward is kf.cu:427-532 as mcg_integrate computes it).
 * vol0: the volume before the first frame (nx*ny*nz float2), or NULL for the
 * initial state (tsdf -1, weight 0).  poses_dev: n_frames x 12 floats on the
 * device (rotation column-major, then t, as mcg_integrate_device_pose).
 * depth_m: n_frames x h x w z-depth in metres; normals: NULL or
 * n_frames x h x w float3 (held constant).  grad_f / grad_w: dL/dtsdf and
 * dL/dweight after the last frame (grad_w may be NULL = 0).  Accumulates
 * dL/ddepth into grad_depth (n_frames x h x w; the caller initialises it);
 * grad_f0 / grad_w0 (may be NULL) receive dL/dtsdf and dL/dweight of vol0.
 * The pixel choices, truncation and clamping of the forward are held fixed.
 * MCG_ERR_TOO_LARGE above 512 frames per call: split the sequence and chain
 * the calls through vol0 / grad_f0 / grad_w0. */
mcg_status mcg_integrate_backward(mcg_context *ctx, const void *vol0, int32_t nx, int32_t ny, int32_t nz,
                                  float min_t, float max_t, float grid_s, const mcg_intrinsic *k, int32_t n_frames,
                                  const float *poses_dev, int32_t w, int32_t h, const float *depth_m,
                                  const float *normals, int32_t is_dynamic, const float *grad_f,
                                  const float *grad_w, float *grad_depth, float *grad_f0, float *grad_w0,
                                  mcg_stream_t stream);

/* ---- ray casting: kf.cu:786-986 (_cu_voxel_extract_depth_and_normal_map) */
/* Depth (metres, z-depth; 0 where the ray finds no zero crossing) and, if
 * normal is not NULL, camera-frame normals (float3, (0,0,0) where none) of a
 * w x h image seen by (k, e) (camera -> global) in a short2 volume of cell
 * size grid_s.  The march, the trilinear sampler (kf.cu:551-657) and the
 * surface normal (kf.cu:3146-3233) are the reference's; colour is not part
 * of the voxel and is not produced.  When K R^T is singular nothing is
 * written, as the reference then launches nothing. */
mcg_status mcg_raycast(mcg_context *ctx, const void *vol, int32_t nx, int32_t ny, int32_t nz, float grid_s,
                       const mcg_intrinsic *k, const mcg_extrinsic *e, int32_t w, int32_t h, float *depth,
                       float *normal, mcg_stream_t stream);

/* ---- depth pyramid and ICP: kf.cu:66-80, 226-261, 988-1301 ---------------- */
/* d_pyramid_down: dst (dw x dh) from src (sw x sh): the mean of the valid
 * src values within sigma of the centre pixel (2x, 2y) over the clipped
 * 5 x 5 window from (2x - 2, 2y - 2); masks are 0 / 0xff per pixel. */
mcg_status mcg_pyramid_down(mcg_context *ctx, int32_t sw, int32_t sh, int32_t dw, int32_t dh, const float *src,
                            const uint8_t *src_mask, float *dst, uint8_t *dst_mask, float sigma, mcg_stream_t stream);
/* to_mask = 1: d_float_data_to_mask (mask = data != 0 ? 0xff : 0);
 * to_mask = 0: d_float_mask_to_data (data = 0 where mask == 0). */
mcg_status mcg_depth_mask(mcg_context *ctx, int64_t n, float *data, uint8_t *mask, int32_t to_mask,
                          mcg_stream_t stream);
/* nwf_icp_projective_3d_params */
typedef struct mcg_icp_params {
    float nt;          /* a match needs dot(n1, R n2) > nt */
    float dt;          /* ... and |v1 - (R v2 + t)| < dt */
    float rt, tt;      /* bounds of one step's rotation (rad) / translation components */
    int32_t it_max;    /* iterations (the reference's icp_it_max of the level) */
    int32_t bilinear;  /* 0: nearest pixel (step 1), 1: bilinear sub-pixel (step 4) */
} mcg_icp_params;
/* One correspondence pass at pose_rel (steps 1/4, 2, 3): v21 (3 floats per
 * pixel of map 1; x = FLT_MAX where there is no match), A (6 columns of
 * w1*h1 floats), b, inlier flags; each output may be NULL (A and b
 * together).  Maps are float3 device arrays (vertex and unit normal; a zero
 * normal marks an invalid pixel).  Synchronous. */
mcg_status mcg_icp_correspond(mcg_context *ctx, const mcg_icp_params *params, const mcg_intrinsic *k2,
                              const mcg_extrinsic *pose_rel, int32_t w1, int32_t h1, int32_t w2, int32_t h2,
                              const float *v1, const float *n1, const float *v2, const float *n2, float *v21,
                              float *A, float *b, uint8_t *inlier, mcg_stream_t stream);
/* _cu_icp_projective_3d: point-to-plane ICP aligning map 2 to map 1 (pose
 * maps map-2 points into map 1's frame), starting from and updating
 * *pose_rel.  Per iteration one fused correspondence + normal-equation
 * kernel (binary64 sums of the reference's binary32 products) and one
 * device solve (Cholesky, |det| > 1e-15, 1-norm rcond > 5e-5, increment
 * bounds, Rodrigues exp, compose, stop when the distance grows or drops
 * below 1e-5); no host round trip inside the loop.  *ok = the reference's
 * return value; the pose and the inlier map (may be NULL) are written only
 * when *ok.  Synchronous at the end. */
mcg_status mcg_icp(mcg_context *ctx, const mcg_icp_params *params, const mcg_intrinsic *k2, mcg_extrinsic *pose_rel,
                   int32_t w1, int32_t h1, int32_t w2, int32_t h2, const float *v1, const float *n1, const float *v2,
                   const float *n2, uint8_t *inlier, int32_t *ok, int32_t *iterations, mcg_stream_t stream);

/* ---- RLE volume codec: kf.cu:1303-1600 ----------------------------------- */
/* upper bound of the encoded file image size */
int64_t mcg_rle_bound(int32_t nx, int32_t ny, int32_t nz);
/* Encode a device short2 volume into a host file image (header + per-slice
 * dumps, the reference's file layout), on the GPU (kf.cu:1367-1417 encodes
 * one slice at a time on the host).  lossless = 0 writes the reference
 * format (runs compare tsdf only; weights inside a run are not kept);
 * lossless = 1 writes the same layout with tag "VOLUME_TSDF_W32" and runs
 * that compare whole voxels.  The image is assembled in device memory kept
 * by ctx and copied out once.  image = NULL with capacity = 0 returns the
 * exact image size in *size; a smaller capacity gives MCG_ERR_CAPACITY with
 * the size in *size.  MCG_ERR_TOO_LARGE when a slice could exceed the
 * format's 32-bit slice byte count (more than 715 827 882 voxels per
 * slice).  Synchronous. */
mcg_status mcg_rle_encode(mcg_context *ctx, const void *vol, int32_t nx, int32_t ny, int32_t nz,
                          float min_t, float max_t, float grid_s, int32_t lossless,
                          uint8_t *image, int64_t capacity, int64_t *size, mcg_stream_t stream);
/* Parse the header of a host file image: dims[3] and params {min_t,max_t,grid_s}. */
mcg_status mcg_rle_header(const uint8_t *image, int64_t size, int32_t dims[3], float params[3]);
/* Same codec on host memory (vol: host short2 [z][y][x]); no CUDA needed. */
mcg_status mcg_rle_encode_host(const void *vol, int32_t nx, int32_t ny, int32_t nz, float min_t, float max_t,
                               float grid_s, int32_t lossless, uint8_t *image, int64_t capacity, int64_t *size);
mcg_status mcg_rle_decode_host(const uint8_t *image, int64_t size, void *vol, int64_t capacity_voxels);
/* Decode a host file image into a device short2 volume of capacity voxels
 * (kf.cu:1533-1563 reads and decodes slice by slice on the host): the
 * compressed image moves to the device in slabs of whole slices and the
 * runs are expanded on the GPU, one CTA per slice; the validity checks are
 * the host decoder's (MCG_ERR_FORMAT).  Synchronous. */
mcg_status mcg_rle_decode(mcg_context *ctx, const uint8_t *image, int64_t size, void *vol,
                          int64_t capacity_voxels, mcg_stream_t stream);
/* The same from a file, streamed: pieces are read by host threads into
 * pinned buffers and copied while the slices already resident expand.
 * dims / params receive the header (size.xyz; min_t, max_t, grid_s).
 * MCG_ERR_IO when the file cannot be read.  Synchronous. */
mcg_status mcg_rle_decode_file(mcg_context *ctx, const char *path, void *vol, int64_t capacity_voxels,
                               int32_t dims[3], float params[3], mcg_stream_t stream);

/* ---- mesh writers: kf.cu:3394-3424 (PLY), 3625-3726 (OBJ) ------------------- */
/* Binary little-endian PLY of a soup, the reference's bytes: header, per
 * vertex position + normal (float3 each), per triangle uint8 3 + int32
 * 3t, 3t+1, 3t+2.  soup / normals: device arrays of n_vertices entries
 * (normals 3 floats each).  image = NULL with capacity 0 returns the size in
 * *size; a smaller capacity gives MCG_ERR_CAPACITY.  Built on the device,
 * copied out once.  Synchronous. */
mcg_status mcg_mesh_ply(mcg_context *ctx, const mcg_vertex_voxel *soup, const float *normals, int64_t n_vertices,
                        uint8_t *image, int64_t capacity, int64_t *size, mcg_stream_t stream);
/* OBJ text with the reference's vertex merge (a vertex is new when the text
 * "%.4f_%.4f_%.4f" of its position is new; "v %f %f %f" + "vn %f %f %f" per
 * new vertex, "f a b c" per triangle of three distinct ids) and the
 * qi_volume listing ("qi tsdf w vx vy vz", then "%d %hd %hd %d %d %d" per
 * vertex), byte for byte, built on the device (hash merge of the exact
 * integer keys, GPU number formatting).  NULL buffers with capacities 0
 * return the sizes; a smaller capacity gives MCG_ERR_CAPACITY; qi may be
 * NULL.  MCG_ERR_TOO_LARGE for positions at 104.8575 or more from the
 * origin (where the reference's key buffer overflows) or non-finite /
 * huge values.  Synchronous. */
mcg_status mcg_mesh_obj(mcg_context *ctx, const mcg_vertex_voxel *soup, const float *normals, int64_t n_vertices,
                        uint8_t *obj, int64_t obj_capacity, int64_t *obj_size, uint8_t *qi, int64_t qi_capacity,
                        int64_t *qi_size, mcg_stream_t stream);
/* Writes path by its extension (".ply" or ".obj"; anything else:
 * MCG_ERR_INVALID_ARG, the reference prints "Invalid file extension"); for
 * OBJ also qi_path when not NULL (the reference writes "qi_volume.txt").
 * MCG_ERR_IO when a file cannot be written. */
mcg_status mcg_mesh_write(mcg_context *ctx, const mcg_vertex_voxel *soup, const float *normals, int64_t n_vertices,
                          const char *path, const char *qi_path, mcg_stream_t stream);

/* ---- text-record volume loader: kf.cu:3289-3361 ---------------------------- */
/* The loop of cu_voxel_rlc_to_mesh: integers read five at a time as
 * "x y z sdf weight" records with `ifs >> int` (C++ formatted input:
 * white space skipped, optional sign, decimal digits, int range); records
 * inside [origin, origin + dim)^3 fill the dim^3 short2 device volume vol in
 * arrival order, z fastest, then y, then x (v[zi*dim*dim + yi*dim + xi] =
 * {(short)sdf, (ushort)weight}), until dim^3 are stored.  The reference
 * passes origin {512, 512, 0}.  The volume is zeroed first (the reference's
 * host array is uninitialised).  The end of the stream follows the
 * reference's `while (!ifs.eof())` loop: text ending in white space repeats
 * the last record; a partial record takes its missing fields from the record
 * before; a failed field (no digits, or outside int) reads 0 / INT_MAX /
 * INT_MIN, and unless it ran into end of file that record repeats into every
 * remaining voxel -- or, when it lies outside the window, the reference
 * never returns: MCG_ERR_FORMAT here, with the voxels stored before it.
 * Parsed on the device; synchronous. */
typedef struct mcg_text_info {
    int64_t bytes;        /* text bytes parsed */
    int64_t numbers;      /* integers extracted before the stream ended */
    int64_t records;      /* complete records, numbers / 5 */
    int64_t stored;       /* voxels written in arrival order (<= dim^3) */
    int64_t fail_offset;  /* byte offset of the first failed extraction, -1 if none */
    int32_t filled_rest;  /* 1: a failed record inside the window filled the remaining voxels */
    int32_t reserved;
} mcg_text_info;
/* text: device bytes (e.g. read by GPUDirect or produced on the device) */
mcg_status mcg_text_records_parse(mcg_context *ctx, const void *text, int64_t len, int32_t dim,
                                  const int32_t origin[3], void *vol, mcg_text_info *info, mcg_stream_t stream);
/* text: host bytes (pageable or pinned), copied to the device in one copy */
mcg_status mcg_text_records_load(mcg_context *ctx, const void *text, int64_t len, int32_t dim,
                                 const int32_t origin[3], void *vol, mcg_text_info *info, mcg_stream_t stream);
/* The last tail_bytes of a file, as kf.cu:3316-3317 seeks (tail 11e9), read
 * by host threads through pinned staging while earlier pieces copy: the
 * line cut by the seek is skipped.  A file no longer than tail_bytes (or
 * tail_bytes <= 0) is read whole, from offset 0, without skipping a line;
 * the reference's seek fails there and its loop never ends.  MCG_ERR_IO when
 * the file cannot be opened or read. */
mcg_status mcg_text_records_load_file(mcg_context *ctx, const char *path, int64_t tail_bytes, int32_t dim,
                                      const int32_t origin[3], void *vol, mcg_text_info *info,
                                      mcg_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* MCG_H */
