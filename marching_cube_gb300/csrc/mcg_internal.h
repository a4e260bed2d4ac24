// Internal declarations shared by the libmcg translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "mcg.h"

namespace mcg {

constexpr int kMaxTsdf = 32766;  // cu_kinect_fusion_v1.h:44 CU_VOXEL_MAX_TSDF
constexpr int kMaxW = 65535;     // cu_kinect_fusion_v1.h:42 CU_VOXEL_MAX_W
constexpr float kUbW = 50.0f;    // cu_kinect_fusion_v1.h:46 CU_VOXEL_UB_W

// Totals written by the scan kernel (device) and copied to pinned memory.
struct MeshTotals {
    unsigned long long occupied;
    unsigned long long triangles;
    unsigned long long vertices;
    unsigned int active_bricks;
    unsigned int flags;       // bit 0: a bounded device wait expired (set by the kernels, cleared by the host)
    unsigned int cls_ticket;  // work counters of the count, generate and (indexed) triangle launches,
    unsigned int gen_ticket;  // zeroed before each (the generate launch also zeroes its own at exit)
    unsigned int idx_ticket;
    unsigned int scan_done;   // finished CTAs of the scan / generate launch (the last one resets it)
    unsigned int gen_exit;
    unsigned int idx_cand;    // indexed count phase: bricks listed for the owned-edge count
};
static_assert(sizeof(MeshTotals) <= 256, "MeshTotals fits the totals region of the fixed scratch");

// Grows a device allocation; returns false on cudaMalloc failure.
template <class T>
bool ensure(T **ptr, size_t *cap, size_t n) {
    if (*cap >= n && *ptr) return true;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    size_t want = n ? n : 1;
    if (cudaMalloc((void **)ptr, want * sizeof(T)) != cudaSuccess) return false;
    *cap = want;
    return true;
}

}  // namespace mcg

struct mcg_context {
    int device = 0;
    int num_sms = 0;
    int last_cuda_error = 0;

    // marching-cubes scratch (one entry per brick)
    uint32_t *brick_tris = nullptr;
    size_t brick_tris_cap = 0;
    uint32_t *brick_occ = nullptr;  // per-chunk sums of the count pass (CHUNK_FIELDS per chunk)
    size_t brick_occ_cap = 0;
    unsigned long long *brick_vofs = nullptr;
    size_t brick_vofs_cap = 0;
    uint32_t *active = nullptr;
    size_t active_cap = 0;
    unsigned long long *list_vofs = nullptr;  // soup offset per active-list entry
    size_t list_vofs_cap = 0;
    unsigned char *batch_list = nullptr;  // resolved active-list entries of a batch (32 B each)
    size_t batch_list_cap = 0;
    // indexed extraction: owned vertices and their offsets per brick, and
    // the vertex id of every grid edge (3 per voxel, written sparsely)
    uint32_t *brick_uniq = nullptr;
    size_t brick_uniq_cap = 0;
    unsigned long long *brick_uofs = nullptr;
    size_t brick_uofs_cap = 0;
    uint32_t *edge_map = nullptr;
    size_t edge_map_cap = 0;
    // fused extraction: per work item its triangle count and per group of
    // items its aggregate / inclusive prefix, each tagged with the launch's
    // epoch (entries of older launches read as unpublished), zeroed at
    // allocation and when the epoch wraps
    unsigned long long *fx_item = nullptr;
    size_t fx_item_cap = 0;
    unsigned long long *fx_group = nullptr;
    size_t fx_group_cap = 0;
    unsigned int fx_epoch = 0;
    mcg::MeshTotals *d_totals = nullptr;
    mcg::MeshTotals *h_totals = nullptr;  // pinned, mapped
    mcg::MeshTotals *h_totals_dev = nullptr;  // device address of h_totals; null if it has none
    size_t chunk_clean_cap = 0;  // brick_occ entries known to be zero (the scan re-zeroes what it used)
    // flags and work counters of d_totals known to be zero: the last scan and
    // generate CTAs reset them when the totals reach the host through
    // h_totals_dev; any other launch over them, or an error, clears this
    bool counters_clean = false;
    cudaEvent_t counts_ready = nullptr;
    bool time_kernels = false;  // events around the classify kernel (mcg_set_kernel_timing)
    bool timed = false;         // a pair has been recorded
    cudaEvent_t tk0 = nullptr, tk1 = nullptr;
    bool counts_pending = false;

    // geometry of the last classify (generate must match it)
    bool classified = false;
    const void *cls_data = nullptr;
    int cls_nx = 0, cls_ny = 0, cls_nz = 0, cls_vtype = 0;
    int cls_z0 = 0, cls_z1 = 0;  // cube layers z0 <= z < z1 of the last count phase
    int64_t last_capacity = -1;
    bool cls_indexed = false;        // the last classify was mcg_mc_classify_indexed
    bool cls_fused = false;          // the last count phase was a fused extraction (counts only, no brick list)
    mcg_mc_config mc_cfg = {0, 4, 3, 0};  // launch configuration (mcg_mc_set_config)
    int64_t last_capacity_tris = -1;  // indexed: triangle capacity of the last generate
    uint32_t *idx_cand = nullptr;     // indexed: bricks whose owned edges are counted
    size_t idx_cand_cap = 0;

    // batched extraction: device tables (volume descriptors, classify and
    // generate tensor maps), pinned staging for them, per-volume sums
    unsigned char *d_btab = nullptr;
    size_t d_btab_cap = 0;
    // pinned staging of the table, two slots used in turn: a call waits only
    // for the copy out of the slot two calls back
    unsigned char *h_btab[2] = {nullptr, nullptr};
    size_t h_btab_cap[2] = {0, 0};
    cudaEvent_t btab_copied[2] = {nullptr, nullptr};
    bool btab_pending[2] = {false, false};
    int btab_slot = 0;
    // pinned stagings for batched calls inside a stream capture (the graph's
    // copy node reads its source at every replay): two spares made by the
    // last call outside a capture, and those a graph took, kept until
    // mcg_destroy
    std::vector<unsigned char *> btab_spare;
    size_t btab_spare_cap = 0;
    std::vector<unsigned char *> btab_kept;
    unsigned char *batch_tma = nullptr;  // per volume of the classified batch: both boxes encodable
    size_t batch_tma_cap = 0;
    unsigned long long *d_vol_sums = nullptr;
    size_t d_vol_sums_cap = 0;
    unsigned long long *h_vol_sums = nullptr;  // pinned, mapped
    unsigned long long *h_vol_sums_dev = nullptr;  // its device address; null if it has none
    size_t h_vol_sums_cap = 0;
    int batch_nvol = 0;
    long long batch_nbricks = 0;
    bool batch_classified = false;
    int batch_vtype = 0;
    const void *batch_first_data = nullptr;
    int64_t *batch_caps = nullptr;  // host, last generate's capacities
    size_t batch_caps_cap = 0;

    // GPU run-length encoder: per-slice byte counts / offsets and the image
    unsigned long long *rle_slices = nullptr;
    size_t rle_slices_cap = 0;
    uint8_t *rle_image = nullptr;
    size_t rle_image_cap = 0;
    // GPU run-length decoder: slice offsets then lengths, error flag, pinned
    // staging of file pieces
    long long *rd_dir = nullptr;  // slice offsets, lengths, first chunks
    size_t rd_dir_cap = 0;
    int rd_dir_n = 0;
    int *rd_err = nullptr;
    size_t rd_err_cap = 0;
    unsigned char *rd_sum = nullptr;  // per-chunk summaries, entry states, first voxels
    size_t rd_sum_cap = 0;
    unsigned char *rd_entry = nullptr;
    size_t rd_entry_cap = 0;
    long long *rd_first = nullptr;
    size_t rd_first_cap = 0;
    uint8_t *h_rd_stage = nullptr;

    // mesh writers: key table, int scratch (first index per slot; slot,
    // uid, id, order per vertex; kept triangles; flags), lengths/offsets and
    // the assembled file body
    unsigned long long *mw_keys = nullptr;
    size_t mw_keys_cap = 0;
    int *mw_int = nullptr;
    size_t mw_int_cap = 0;
    long long *mw_len = nullptr;
    size_t mw_len_cap = 0;
    unsigned char *mw_text = nullptr;
    size_t mw_text_cap = 0;

    // ICP: loop state (device + pinned copy), per-CTA sums, a pose for the
    // single correspondence pass, inlier flags of the passes
    unsigned char *icp_state = nullptr;
    size_t icp_state_cap = 0;
    unsigned char *h_icp_state = nullptr;  // pinned
    double *icp_partial = nullptr;
    size_t icp_partial_cap = 0;
    float *icp_pose = nullptr;
    size_t icp_pose_cap = 0;
    uint8_t *icp_inlier = nullptr;
    size_t icp_inlier_cap = 0;

    // integrate scratch
    float *depth_scaled = nullptr;
    size_t depth_scaled_cap = 0;
    int2 *integ_rows = nullptr;  // per voxel row: the candidate x interval of the frame
    size_t integ_rows_cap = 0;
    unsigned int *integ_zmax = nullptr;  // the frame's largest ray-length depth (float bits)
    size_t integ_zmax_cap = 0;
    // x coordinates of the voxel centres as the reference accumulates them
    // (p.x += grid_s per voxel), one device table per (nx, grid_s) seen on
    // this context, built once and never rewritten, so the calls on several
    // volumes of a frame (and a graph captured around them) share them
    struct RayX {
        int nx;
        float g;
        float *d;
    };
    std::vector<RayX> ray_x;

    // text-record loader: the text on the device, its fields, per-segment
    // and per-CTA counts, the result block and pinned staging
    uint8_t *tr_text = nullptr;
    size_t tr_text_cap = 0;
    int *tr_tok = nullptr;
    size_t tr_tok_cap = 0;
    long long *tr_seg = nullptr;
    size_t tr_seg_cap = 0;
    long long *tr_cta = nullptr;
    size_t tr_cta_cap = 0;
    uint32_t *tr_arr = nullptr;  // voxels in arrival order
    size_t tr_arr_cap = 0;
    unsigned char *tr_scan = nullptr;
    size_t tr_scan_cap = 0;
    unsigned char *h_tr_scan = nullptr;   // pinned
    uint8_t *h_tr_stage = nullptr;        // pinned, reader-thread staging
};

// records a CUDA failure on ctx and returns the matching status
mcg_status mcg_cuda_fail(mcg_context *ctx, cudaError_t e);

namespace mcg {
// The soup extraction's count phase (count launch + scan) over the whole
// volume, its totals left in ctx->d_totals (no mapped host copy), for the
// indexed extraction, which takes the brick triangle counts from it.
cudaError_t soup_count_phase(mcg_context *ctx, const mcg_volume *vol, cudaStream_t s);
}  // namespace mcg

// true while `s` is being captured into a CUDA graph
inline bool mcg_capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return st == cudaStreamCaptureStatusActive;
}

// Marks the counts copied to pinned memory on stream s as pending.  During
// capture no event is recorded: the copy is a node of the graph, and the
// caller reads the counts after synchronising the graph's stream.
inline cudaError_t mcg_counts_event(mcg_context *ctx, cudaStream_t s) {
    if (mcg_capturing(s)) {
        ctx->counts_pending = false;
        return cudaSuccess;
    }
    cudaError_t e = cudaEventRecord(ctx->counts_ready, s);
    if (e == cudaSuccess) ctx->counts_pending = true;
    return e;
}
