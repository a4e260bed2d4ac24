// Context lifetime, status strings and error plumbing of the C ABI.
#include <cuda_runtime.h>

#include <new>

#include "mcg_internal.h"

mcg_status mcg_cuda_fail(mcg_context *ctx, cudaError_t e) {
    if (ctx) {
        ctx->last_cuda_error = (int)e;
        ctx->counters_clean = false;
    }
    cudaGetLastError();  // clear a sticky-free error so later calls can proceed
    return MCG_ERR_CUDA;
}

extern "C" {

const char *mcg_status_string(int status) {
    switch (status) {
        case MCG_OK: return "ok";
        case MCG_ERR_INVALID_ARG: return "invalid argument";
        case MCG_ERR_CAPACITY: return "output capacity exceeded";
        case MCG_ERR_CUDA: return "CUDA error";
        case MCG_ERR_TIMEOUT: return "device wait timed out";
        case MCG_ERR_IO: return "I/O error";
        case MCG_ERR_FORMAT: return "malformed stream or header";
        case MCG_ERR_STATE: return "call order violated";
        case MCG_ERR_TOO_LARGE: return "volume exceeds the fixed scratch of the no-allocation entry point, or more than 512 frames per adjoint call";
        default: return "unknown status";
    }
}

int mcg_version(void) { return MCG_VERSION; }

mcg_status mcg_create(mcg_context **out, int device) {
    if (!out) return MCG_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) { cudaGetLastError(); return MCG_ERR_CUDA; }
    if (device < 0 || device >= count) return MCG_ERR_INVALID_ARG;
    mcg_context *ctx = new (std::nothrow) mcg_context();
    if (!ctx) return MCG_ERR_INVALID_ARG;
    ctx->device = device;
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_totals, sizeof(mcg::MeshTotals));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_totals, 0, sizeof(mcg::MeshTotals));
    if (e == cudaSuccess)
        e = cudaHostAlloc((void **)&ctx->h_totals, sizeof(mcg::MeshTotals), cudaHostAllocMapped | cudaHostAllocPortable);
    // the count and generate launches write the totals straight into host memory
    // through this address; without one the host copies them
    if (e == cudaSuccess && cudaHostGetDevicePointer((void **)&ctx->h_totals_dev, ctx->h_totals, 0) != cudaSuccess) {
        cudaGetLastError();
        ctx->h_totals_dev = nullptr;
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->counts_ready, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k)
        e = cudaEventCreateWithFlags(&ctx->btab_copied[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        mcg_destroy(ctx);
        return MCG_ERR_CUDA;
    }
    *ctx->h_totals = mcg::MeshTotals{};
    *out = ctx;
    return MCG_OK;
}

mcg_status mcg_destroy(mcg_context *ctx) {
    if (!ctx) return MCG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->counts_ready) cudaEventSynchronize(ctx->counts_ready);
    cudaFree(ctx->brick_tris);
    cudaFree(ctx->brick_occ);
    cudaFree(ctx->brick_vofs);
    cudaFree(ctx->active);
    cudaFree(ctx->list_vofs);
    cudaFree(ctx->batch_list);
    cudaFree(ctx->brick_uniq);
    cudaFree(ctx->brick_uofs);
    cudaFree(ctx->edge_map);
    cudaFree(ctx->fx_item);
    cudaFree(ctx->idx_cand);
    cudaFree(ctx->fx_group);
    cudaFree(ctx->d_totals);
    if (ctx->h_totals) cudaFreeHost(ctx->h_totals);
    if (ctx->counts_ready) cudaEventDestroy(ctx->counts_ready);
    if (ctx->tk0) cudaEventDestroy(ctx->tk0);
    if (ctx->tk1) cudaEventDestroy(ctx->tk1);
    for (int k = 0; k < 2; ++k)
        if (ctx->btab_copied[k]) cudaEventSynchronize(ctx->btab_copied[k]);
    cudaFree(ctx->d_btab);
    for (int k = 0; k < 2; ++k) {
        if (ctx->h_btab[k]) cudaFreeHost(ctx->h_btab[k]);
        if (ctx->btab_copied[k]) cudaEventDestroy(ctx->btab_copied[k]);
    }
    for (unsigned char *b : ctx->btab_kept) cudaFreeHost(b);
    for (unsigned char *b : ctx->btab_spare) cudaFreeHost(b);
    free(ctx->batch_tma);
    cudaFree(ctx->d_vol_sums);
    if (ctx->h_vol_sums) cudaFreeHost(ctx->h_vol_sums);
    delete[] ctx->batch_caps;
    cudaFree(ctx->rle_slices);
    cudaFree(ctx->rle_image);
    cudaFree(ctx->rd_dir);
    cudaFree(ctx->rd_err);
    cudaFree(ctx->rd_sum);
    cudaFree(ctx->rd_entry);
    cudaFree(ctx->rd_first);
    if (ctx->h_rd_stage) cudaFreeHost(ctx->h_rd_stage);
    cudaFree(ctx->mw_keys);
    cudaFree(ctx->mw_int);
    cudaFree(ctx->mw_len);
    cudaFree(ctx->mw_text);
    cudaFree(ctx->icp_state);
    if (ctx->h_icp_state) cudaFreeHost(ctx->h_icp_state);
    cudaFree(ctx->icp_partial);
    cudaFree(ctx->icp_pose);
    cudaFree(ctx->icp_inlier);
    cudaFree(ctx->depth_scaled);
    cudaFree(ctx->integ_rows);
    cudaFree(ctx->integ_zmax);
    for (const auto &r : ctx->ray_x) cudaFree(r.d);
    cudaFree(ctx->tr_text);
    cudaFree(ctx->tr_tok);
    cudaFree(ctx->tr_seg);
    cudaFree(ctx->tr_cta);
    cudaFree(ctx->tr_arr);
    cudaFree(ctx->tr_scan);
    if (ctx->h_tr_scan) cudaFreeHost(ctx->h_tr_scan);
    if (ctx->h_tr_stage) cudaFreeHost(ctx->h_tr_stage);
    delete ctx;
    return MCG_OK;
}

int mcg_last_cuda_error(const mcg_context *ctx) { return ctx ? ctx->last_cuda_error : 0; }

}  // extern "C"
