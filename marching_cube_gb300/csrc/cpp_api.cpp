// The reference's C++ host interface (cu_memory.hpp, cu_marching_cubes_v1.h,
// cu_kinect_fusion_v1.h) implemented over the C ABI.  Everything here is
// host code: containers, the MarchingCubes class, camera/RLE/mesh-file
// drivers.  The kernels are reached only through mcg_* calls.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <string>
#include <vector>

#include "cu_kinect_fusion_v1.h"
#include "cu_marching_cubes_v1.h"
#include "cu_memory.hpp"
#include "mcg.h"
#include "structure.h"

namespace {

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw mcg_cuda_error(std::string(what) + ": " + cudaGetErrorString(e), (int)e);
    }
}

void check_status(mcg_status st, mcg_context *ctx, const char *what) {
    if (st != MCG_OK)
        throw mcg_cuda_error(std::string(what) + ": " + mcg_status_string(st),
                             st == MCG_ERR_CUDA ? mcg_last_cuda_error(ctx) : (int)st);
}

int *new_ref() { return reinterpret_cast<int *>(new std::atomic<int>(1)); }
int add_ref(int *r, int d) { return reinterpret_cast<std::atomic<int> *>(r)->fetch_add(d) + d; }
void del_ref(int *r) { delete reinterpret_cast<std::atomic<int> *>(r); }

// one context per thread for the free functions (the reference's globals
// were single-threaded; per-thread contexts keep the calls re-entrant)
struct ThreadCtx {
    mcg_context *ctx = nullptr;
    int device = -1;
    ~ThreadCtx() {
        if (ctx) mcg_destroy(ctx);
    }
};

mcg_context *thread_ctx() {
    static thread_local ThreadCtx t;
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    if (!t.ctx || t.device != dev) {
        if (t.ctx) mcg_destroy(t.ctx);
        t.ctx = nullptr;
        check_status(mcg_create(&t.ctx, dev), nullptr, "mcg_create");
        t.device = dev;
    }
    return t.ctx;
}

mcg_intrinsic to_intrinsic(const float_camera_intrinsic &k) {
    mcg_intrinsic m;
    m.fx = k.fc.x;
    m.fy = k.fc.y;
    m.cx = k.cc.x;
    m.cy = k.cc.y;
    for (int i = 0; i < 5; ++i) m.dc[i] = k.dc[i];
    return m;
}

mcg_extrinsic to_extrinsic(const float_camera_extrinsic &e) {
    mcg_extrinsic m;
    for (int c = 0; c < 3; ++c) {
        m.r[3 * c + 0] = e.R.p[c].x;
        m.r[3 * c + 1] = e.R.p[c].y;
        m.r[3 * c + 2] = e.R.p[c].z;
    }
    m.t[0] = e.t.x;
    m.t[1] = e.t.y;
    m.t[2] = e.t.z;
    return m;
}

mcg_volume to_volume(const cu_voxel &v) {
    mcg_volume m;
    m.data = v.data;
    m.nx = v.size.x;
    m.ny = v.size.y;
    m.nz = v.size.z;
    m.voxel_type = MCG_VOXEL_SHORT2;
    m.cell = v.grid_s;
    return m;
}

}  // namespace

// ---------------------------------------------------------------------------
// containers (cu_memory.cpp:45-345 semantics)
// ---------------------------------------------------------------------------
cu_memory::cu_memory() : data_(0), size_bytes_(0), refcount_(0) {}
cu_memory::cu_memory(void *ptr_arg, size_t size_bytes_arg) : data_(ptr_arg), size_bytes_(size_bytes_arg), refcount_(0) {}
cu_memory::cu_memory(size_t size_bytes_arg) : data_(0), size_bytes_(0), refcount_(0) { create(size_bytes_arg); }
cu_memory::~cu_memory() { release(); }
cu_memory::cu_memory(const cu_memory &o) : data_(o.data_), size_bytes_(o.size_bytes_), refcount_(o.refcount_) {
    if (refcount_) add_ref(refcount_, 1);
}
cu_memory &cu_memory::operator=(const cu_memory &o) {
    if (this != &o) {
        if (o.refcount_) add_ref(o.refcount_, 1);
        release();
        data_ = o.data_;
        size_bytes_ = o.size_bytes_;
        refcount_ = o.refcount_;
    }
    return *this;
}
void cu_memory::create(size_t n) {
    if (n == size_bytes_) return;
    if (n > 0) {
        if (data_) release();
        check(cudaMalloc(&data_, n), "cu_memory::create");
        size_bytes_ = n;
        refcount_ = new_ref();
    }
}
void cu_memory::copy_to(cu_memory &other) const {
    if (empty()) {
        other.release();
        return;
    }
    other.create(size_bytes_);
    check(cudaMemcpy(other.data_, data_, size_bytes_, cudaMemcpyDeviceToDevice), "cu_memory::copy_to");
}
void cu_memory::release() {
    if (refcount_ && add_ref(refcount_, -1) == 0) {
        del_ref(refcount_);
        cudaFree(data_);
    }
    data_ = 0;
    size_bytes_ = 0;
    refcount_ = 0;
}
void cu_memory::upload(const void *h, size_t n) {
    create(n);
    check(cudaMemcpy(data_, h, size_bytes_, cudaMemcpyHostToDevice), "cu_memory::upload");
}
void cu_memory::download(void *h) const {
    check(cudaMemcpy(h, data_, size_bytes_, cudaMemcpyDeviceToHost), "cu_memory::download");
}
void cu_memory::swap(cu_memory &o) {
    std::swap(data_, o.data_);
    std::swap(size_bytes_, o.size_bytes_);
    std::swap(refcount_, o.refcount_);
}

cu_memory_host::cu_memory_host() : data_(0), size_bytes_(0), refcount_(0) {}
cu_memory_host::cu_memory_host(void *p, size_t n) : data_(p), size_bytes_(n), refcount_(0) {}
cu_memory_host::cu_memory_host(size_t n) : data_(0), size_bytes_(0), refcount_(0) { create(n); }
cu_memory_host::~cu_memory_host() { release(); }
cu_memory_host::cu_memory_host(const cu_memory_host &o) : data_(o.data_), size_bytes_(o.size_bytes_), refcount_(o.refcount_) {
    if (refcount_) add_ref(refcount_, 1);
}
cu_memory_host &cu_memory_host::operator=(const cu_memory_host &o) {
    if (this != &o) {
        if (o.refcount_) add_ref(o.refcount_, 1);
        release();
        data_ = o.data_;
        size_bytes_ = o.size_bytes_;
        refcount_ = o.refcount_;
    }
    return *this;
}
void cu_memory_host::create(size_t n) {
    if (n == size_bytes_) return;
    if (n > 0) {
        if (data_) release();
        check(cudaMallocHost(&data_, n), "cu_memory_host::create");
        size_bytes_ = n;
        refcount_ = new_ref();
    }
}
void cu_memory_host::copy_to(cu_memory_host &other) const {
    if (empty()) {
        other.release();
        return;
    }
    other.create(size_bytes_);
    memcpy(other.data_, data_, size_bytes_);
}
void cu_memory_host::release() {
    if (refcount_ && add_ref(refcount_, -1) == 0) {
        del_ref(refcount_);
        cudaFreeHost(data_);
    }
    data_ = 0;
    size_bytes_ = 0;
    refcount_ = 0;
}
void cu_memory_host::upload(const void *p, size_t n) {
    create(n);
    memcpy(data_, p, n);
}
void cu_memory_host::download(void *p) const { memcpy(p, data_, size_bytes_); }
void cu_memory_host::swap(cu_memory_host &o) {
    std::swap(data_, o.data_);
    std::swap(size_bytes_, o.size_bytes_);
    std::swap(refcount_, o.refcount_);
}

cu_memory_2d::cu_memory_2d() : data_(0), step_(0), colsBytes_(0), rows_(0), refcount_(0) {}
cu_memory_2d::cu_memory_2d(int r, int cb) : data_(0), step_(0), colsBytes_(0), rows_(0), refcount_(0) { create(r, cb); }
cu_memory_2d::cu_memory_2d(int r, int cb, void *d, size_t s) : data_(d), step_(s), colsBytes_(cb), rows_(r), refcount_(0) {}
cu_memory_2d::~cu_memory_2d() { release(); }
cu_memory_2d::cu_memory_2d(const cu_memory_2d &o)
    : data_(o.data_), step_(o.step_), colsBytes_(o.colsBytes_), rows_(o.rows_), refcount_(o.refcount_) {
    if (refcount_) add_ref(refcount_, 1);
}
cu_memory_2d &cu_memory_2d::operator=(const cu_memory_2d &o) {
    if (this != &o) {
        if (o.refcount_) add_ref(o.refcount_, 1);
        release();
        data_ = o.data_;
        step_ = o.step_;
        colsBytes_ = o.colsBytes_;
        rows_ = o.rows_;
        refcount_ = o.refcount_;
    }
    return *this;
}
void cu_memory_2d::create(int r, int cb) {
    if (colsBytes_ == cb && rows_ == r) return;
    if (r > 0 && cb > 0) {
        if (data_) release();
        check(cudaMallocPitch(&data_, &step_, (size_t)cb, (size_t)r), "cu_memory_2d::create");
        colsBytes_ = cb;
        rows_ = r;
        refcount_ = new_ref();
    }
}
void cu_memory_2d::release() {
    if (refcount_ && add_ref(refcount_, -1) == 0) {
        del_ref(refcount_);
        cudaFree(data_);
    }
    data_ = 0;
    step_ = 0;
    colsBytes_ = 0;
    rows_ = 0;
    refcount_ = 0;
}
void cu_memory_2d::copy_to(cu_memory_2d &other) const {
    if (empty()) {
        other.release();
        return;
    }
    other.create(rows_, colsBytes_);
    check(cudaMemcpy2D(other.data_, other.step_, data_, step_, colsBytes_, rows_, cudaMemcpyDeviceToDevice),
          "cu_memory_2d::copy_to");
}
void cu_memory_2d::upload(const void *h, size_t hs, int r, int cb) {
    create(r, cb);
    check(cudaMemcpy2D(data_, step_, h, hs, cb, r, cudaMemcpyHostToDevice), "cu_memory_2d::upload");
}
void cu_memory_2d::download(void *h, size_t hs) const {
    check(cudaMemcpy2D(h, hs, data_, step_, colsBytes_, rows_, cudaMemcpyDeviceToHost), "cu_memory_2d::download");
}
void cu_memory_2d::swap(cu_memory_2d &o) {
    std::swap(data_, o.data_);
    std::swap(step_, o.step_);
    std::swap(colsBytes_, o.colsBytes_);
    std::swap(rows_, o.rows_);
    std::swap(refcount_, o.refcount_);
}

// ---------------------------------------------------------------------------
// MarchingCubes (cu_marching_cubes_v1.cu:406-467)
// ---------------------------------------------------------------------------
MarchingCubes::MarchingCubes() : ctx_(nullptr) {
    memset(&counts_, 0, sizeof(counts_));
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    check_status(mcg_create(&ctx_, dev), nullptr, "mcg_create");
}

MarchingCubes::~MarchingCubes() {
    if (ctx_) mcg_destroy(ctx_);
}

cu_array<vertex_voxel> MarchingCubes::run(cu_voxel &tsdf, cu_array<vertex_voxel> &triangles_buffer,
                                          cu_array<int3> &vertexindex_to_voxel, cu_array<short> &ver_voxel) {
    return run_impl(tsdf, triangles_buffer, vertexindex_to_voxel, ver_voxel, nullptr);
}

cu_array<vertex_voxel> MarchingCubes::run(cu_voxel &tsdf, cu_array<vertex_voxel> &triangles_buffer,
                                          cu_array<int3> &vertexindex_to_voxel, cu_array<short> &ver_voxel,
                                          cu_array<float3> &normals) {
    return run_impl(tsdf, triangles_buffer, vertexindex_to_voxel, ver_voxel, &normals);
}

cu_array<vertex_voxel> MarchingCubes::run_impl(cu_voxel &tsdf, cu_array<vertex_voxel> &triangles_buffer,
                                               cu_array<int3> &vertexindex_to_voxel, cu_array<short> &ver_voxel,
                                               cu_array<float3> *normals) {
    const mcg_volume vol = to_volume(tsdf);
    check_status(mcg_mc_classify(ctx_, &vol, nullptr), ctx_, "mcg_mc_classify");
    check_status(mcg_mc_counts(ctx_, &counts_), ctx_, "mcg_mc_counts");
    const size_t n = (size_t)counts_.vertices;
    const size_t nvox = (size_t)tsdf.size.x * tsdf.size.y * tsdf.size.z;
    // empty or too small buffers are sized from the count phase
    if (triangles_buffer.size() < (n ? n : 1)) triangles_buffer.create(n ? n : 1);
    if (vertexindex_to_voxel.size() < (n ? n : 1)) vertexindex_to_voxel.create(n ? n : 1);
    if (ver_voxel.size() < nvox) ver_voxel.create(nvox);
    if (normals && normals->size() < (n ? n : 1)) normals->create(n ? n : 1);
    mcg_mesh_out out;
    out.soup = reinterpret_cast<mcg_vertex_voxel *>(triangles_buffer.ptr());
    out.soup_normals = normals ? reinterpret_cast<float *>(normals->ptr()) : nullptr;
    out.vi2vox = reinterpret_cast<int32_t *>(vertexindex_to_voxel.ptr());
    out.ver_voxel = reinterpret_cast<int16_t *>(ver_voxel.ptr());
    out.tri_cube = nullptr;
    out.capacity_vertices = (int64_t)n;
    check_status(mcg_mc_generate(ctx_, &vol, &out, nullptr), ctx_, "mcg_mc_generate");
    check_status(mcg_mc_counts(ctx_, &counts_), ctx_, "mcg_mc_counts");
    if (n == 0) return cu_array<vertex_voxel>();
    return cu_array<vertex_voxel>(triangles_buffer.ptr(), n);
}

void MarchingCubes::backward(cu_voxel &tsdf, const cu_array<float3> &grad_pos, cu_array<float> &grad_tsdf) {
    const mcg_volume vol = to_volume(tsdf);
    const size_t nvox = (size_t)tsdf.size.x * tsdf.size.y * tsdf.size.z;
    if (grad_tsdf.empty()) {
        grad_tsdf.create(nvox);
        check(cudaMemset(grad_tsdf.ptr(), 0, nvox * sizeof(float)), "cudaMemset");
    } else if (grad_tsdf.size() < nvox) {
        throw std::invalid_argument("MarchingCubes::backward: grad_tsdf smaller than the volume");
    }
    const int64_t n = (int64_t)std::min<size_t>(grad_pos.size(), (size_t)counts_.vertices);
    check_status(mcg_mc_backward(ctx_, &vol, reinterpret_cast<const float *>(grad_pos.ptr()), n, grad_tsdf.ptr(),
                                 nullptr),
                 ctx_, "mcg_mc_backward");
    check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

// ---------------------------------------------------------------------------
// volumes, integrate, depth maps
// ---------------------------------------------------------------------------
void cu_voxel_new(cu_voxel *v, int3 size, float min_t, float max_t, float grid_s) {
    v->size = size;
    v->min_t = min_t;
    v->max_t = max_t;
    v->grid_s = grid_s;
    v->size_xy = size.x * size.y;
    const size_t n = (size_t)v->size_xy * size.z;
    if (v->data == NULL) check(cudaMalloc((void **)&v->data, n * sizeof(cu_voxel_t)), "cu_voxel_new");
    mcg_context *ctx = thread_ctx();
    check_status(mcg_voxel_init(ctx, v->data, MCG_VOXEL_SHORT2, (int64_t)n, nullptr), ctx, "mcg_voxel_init");
    check(cudaDeviceSynchronize(), "cu_voxel_new");
}

void cu_voxel_delete(cu_voxel *v) {
    if (v->data) {
        cudaFree(v->data);
        v->data = NULL;
        v->size.x = v->size.y = v->size.z = 0;
        v->min_t = v->max_t = v->grid_s = 0.0f;
        v->size_xy = 0;
    }
}

void _cu_voxel_volumetric_integration(cu_voxel v, float_camera_intrinsic ci, float_camera_extrinsic ce, int2 size,
                                      float *d_depth_ptr, float3 *d_normal_ptr, uchar3 *d_color_ptr,
                                      bool is_dynamic) {
    (void)d_color_ptr;
    mcg_context *ctx = thread_ctx();
    const mcg_intrinsic k = to_intrinsic(ci);
    const mcg_extrinsic e = to_extrinsic(ce);
    check_status(mcg_integrate(ctx, v.data, MCG_VOXEL_SHORT2, v.size.x, v.size.y, v.size.z, v.min_t, v.max_t,
                               v.grid_s, &k, &e, size.x, size.y, d_depth_ptr, (const float *)d_normal_ptr,
                               is_dynamic ? 1 : 0, nullptr),
                 ctx, "mcg_integrate");
    check(cudaDeviceSynchronize(), "_cu_voxel_volumetric_integration");
}

void _cu_voxel_extract_depth_and_normal_map(cu_voxel v, float_camera_intrinsic ci, float_camera_extrinsic ce,
                                            int2 size, float *d_ptr, float3 *n_ptr, uchar3 *c_ptr) {
    mcg_context *ctx = thread_ctx();
    const mcg_intrinsic k = to_intrinsic(ci);
    const mcg_extrinsic e = to_extrinsic(ce);
    // the voxel carries no colour: the colour map keeps the reference's default, white
    if (c_ptr) check(cudaMemset(c_ptr, 0xff, sizeof(uchar3) * (size_t)size.x * size.y), "cudaMemset");
    check_status(mcg_raycast(ctx, v.data, v.size.x, v.size.y, v.size.z, v.grid_s, &k, &e, size.x, size.y, d_ptr,
                             (float *)n_ptr, nullptr),
                 ctx, "mcg_raycast");
    check(cudaDeviceSynchronize(), "_cu_voxel_extract_depth_and_normal_map");
}

void cu_kinect_depth_to_maps(float_camera_intrinsic k, int2 size, const unsigned short *d_depth_mm, float *d_meter,
                             float3 *d_vertex, float3 *d_normal) {
    mcg_context *ctx = thread_ctx();
    const mcg_intrinsic m = to_intrinsic(k);
    check_status(mcg_depth_to_maps(ctx, &m, size.x, size.y, d_depth_mm, KINECT_DEPTH_MIN, KINECT_DEPTH_MAX, d_meter,
                                   (float *)d_vertex, (float *)d_normal, nullptr),
                 ctx, "mcg_depth_to_maps");
}

void cu_meter_to_vertex(float_camera_intrinsic k, int2 size, float *h_meter, float3 *h_vertex) {
    mcg_context *ctx = thread_ctx();
    const size_t n = (size_t)size.x * size.y;
    cu_array<float> m;
    m.upload(h_meter, n);
    cu_array<float3> v(n);
    const mcg_intrinsic kk = to_intrinsic(k);
    check_status(mcg_meter_to_vertex(ctx, &kk, size.x, size.y, m.ptr(), (float *)v.ptr(), nullptr), ctx,
                 "mcg_meter_to_vertex");
    v.download(h_vertex);
}

static void depth_maps_host(float_camera_intrinsic k, int2 size, short *h_depth, float3 *h_vertex,
                            float3 *h_normal) {
    const size_t n = (size_t)size.x * size.y;
    cu_array<unsigned short> d;
    d.upload(reinterpret_cast<unsigned short *>(h_depth), n);
    cu_array<float3> v, nn;
    if (h_vertex) v.create(n);
    if (h_normal) nn.create(n);
    cu_kinect_depth_to_maps(k, size, d.ptr(), nullptr, h_vertex ? v.ptr() : nullptr, h_normal ? nn.ptr() : nullptr);
    if (h_vertex) v.download(h_vertex);
    if (h_normal) nn.download(h_normal);
}

void cu_kinect_depth_to_vertex(float_camera_intrinsic k, int2 size, short *h_depth, float3 *h_vertex) {
    depth_maps_host(k, size, h_depth, h_vertex, nullptr);
}

void cu_kinect_depth_to_normal(float_camera_intrinsic k, int2 size, short *h_depth, float3 *h_normal) {
    depth_maps_host(k, size, h_depth, nullptr, h_normal);
}

void cu_voxel_extract_surface_normals(cu_voxel v, int size, const vertex_voxel *d_vertex, float3 *d_normal) {
    mcg_context *ctx = thread_ctx();
    const mcg_volume vol = to_volume(v);
    check_status(mcg_mc_normals(ctx, &vol, reinterpret_cast<const mcg_vertex_voxel *>(d_vertex), size,
                                (float *)d_normal, nullptr),
                 ctx, "mcg_mc_normals");
}

// ---------------------------------------------------------------------------
// RLE volume I/O with windows (cu_kinect_fusion_v1.cu:1451-1600)
// ---------------------------------------------------------------------------
namespace {

bool read_file(const char *name, std::vector<uint8_t> &buf) {
    FILE *fp = fopen(name, "rb");
    if (!fp) return false;
    fseek(fp, 0, SEEK_END);
    const long n = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    buf.resize(n > 0 ? (size_t)n : 0);
    const size_t got = n > 0 ? fread(buf.data(), 1, (size_t)n, fp) : 0;
    fclose(fp);
    return got == buf.size();
}

bool write_file(const char *name, const uint8_t *p, size_t n) {
    FILE *fp = fopen(name, "wb");
    if (!fp) return false;
    const size_t put = fwrite(p, 1, n, fp);
    fclose(fp);
    return put == n;
}

void download_volume(const cu_voxel *v, std::vector<cu_voxel_t> &h) {
    h.resize((size_t)v->size_xy * v->size.z);
    check(cudaMemcpy(h.data(), v->data, h.size() * sizeof(cu_voxel_t), cudaMemcpyDeviceToHost), "download volume");
}

}  // namespace

void cu_voxel_run_length_encode(cu_voxel *v_local, const char *file_name, int3 begin_local, int3 begin_global,
                                int3 size) {
    std::vector<uint8_t> img;
    if (!read_file(file_name, img)) {
        // no file yet: the whole local volume (:1455-1478)
        mcg_context *ctx = thread_ctx();
        img.resize((size_t)mcg_rle_bound(v_local->size.x, v_local->size.y, v_local->size.z));
        int64_t n = 0;
        check_status(mcg_rle_encode(ctx, v_local->data, v_local->size.x, v_local->size.y, v_local->size.z,
                                    v_local->min_t, v_local->max_t, v_local->grid_s, 0, img.data(),
                                    (int64_t)img.size(), &n, nullptr),
                     ctx, "mcg_rle_encode");
        if (!write_file(file_name, img.data(), (size_t)n)) fprintf(stderr, "cu_voxel_run_length_encode - cannot write %s\n", file_name);
        return;
    }
    // window update of an existing file (:1479-1528)
    const int3 end_local = make_int3(begin_local.x + size.x, begin_local.y + size.y, begin_local.z + size.z);
    if (end_local.x > v_local->size.x || end_local.y > v_local->size.y || end_local.z > v_local->size.z) {
        fprintf(stderr, "cu_voxel_run_length_encode - out of bound.\n");
        return;
    }
    int32_t dims[3];
    float params[3];
    if (mcg_rle_header(img.data(), (int64_t)img.size(), dims, params) != MCG_OK) {
        fprintf(stderr, "cu_voxel_run_length_encode - invalid format.\n");
        return;
    }
    if (begin_global.x + size.x > dims[0] || begin_global.y + size.y > dims[1] || begin_global.z + size.z > dims[2] ||
        v_local->grid_s != params[2]) {
        fprintf(stderr, "cu_voxel_run_length_encode - out of bound.\n");
        return;
    }
    std::vector<cu_voxel_t> global((size_t)dims[0] * dims[1] * dims[2]);
    if (mcg_rle_decode_host(img.data(), (int64_t)img.size(), global.data(), (int64_t)global.size()) != MCG_OK) {
        fprintf(stderr, "cu_voxel_run_length_encode - malformed file.\n");
        return;
    }
    std::vector<cu_voxel_t> local;
    download_volume(v_local, local);
    for (int z = 0; z < size.z; ++z)
        for (int y = 0; y < size.y; ++y)
            memcpy(&global[((size_t)(z + begin_global.z) * dims[1] + y + begin_global.y) * dims[0] + begin_global.x],
                   &local[((size_t)(z + begin_local.z) * v_local->size.y + y + begin_local.y) * v_local->size.x +
                          begin_local.x],
                   sizeof(cu_voxel_t) * size.x);
    std::vector<uint8_t> out((size_t)mcg_rle_bound(dims[0], dims[1], dims[2]));
    int64_t n = 0;
    if (mcg_rle_encode_host(global.data(), dims[0], dims[1], dims[2], params[0], params[1], params[2], 0, out.data(),
                            (int64_t)out.size(), &n) != MCG_OK ||
        !write_file(file_name, out.data(), (size_t)n))
        fprintf(stderr, "cu_voxel_run_length_encode - cannot write %s\n", file_name);
}

void cu_voxel_run_length_decode(cu_voxel *v_local, const char *file_name, int3 begin_local, int3 begin_global,
                                int3 size) {
    uint8_t head[40];
    FILE *fp = fopen(file_name, "rb");
    const size_t got = fp ? fread(head, 1, sizeof(head), fp) : 0;
    if (fp) fclose(fp);
    if (!fp) {
        fprintf(stderr, "cu_voxel_run_length_decode - fail to open %s file.\n", file_name);
        return;
    }
    int32_t dims[3];
    float params[3];
    if (mcg_rle_header(head, (int64_t)got, dims, params) != MCG_OK) {
        fprintf(stderr, "cu_voxel_run_length_decode - invalid format.\n");
        return;
    }
    mcg_context *ctx = thread_ctx();
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    if (v_local->data == NULL) {
        // whole volume (:1542-1563), streamed from the file and expanded on the GPU
        v_local->size = make_int3(dims[0], dims[1], dims[2]);
        v_local->size_xy = dims[0] * dims[1];
        v_local->min_t = params[0];
        v_local->max_t = params[1];
        v_local->grid_s = params[2];
        check(cudaMalloc((void **)&v_local->data, n * sizeof(cu_voxel_t)), "cu_voxel_run_length_decode");
        check_status(mcg_rle_decode_file(ctx, file_name, v_local->data, (int64_t)n, dims, params, nullptr), ctx,
                     "mcg_rle_decode_file");
        return;
    }
    // window read into an allocated volume (:1564-1600): the whole file is
    // expanded on the GPU, then the window copied device to device
    if (begin_local.x + size.x > v_local->size.x || begin_local.y + size.y > v_local->size.y ||
        begin_local.z + size.z > v_local->size.z || begin_global.x + size.x > dims[0] ||
        begin_global.y + size.y > dims[1] || begin_global.z + size.z > dims[2] || v_local->grid_s != params[2]) {
        fprintf(stderr, "cu_voxel_run_length_decode - out of bound.\n");
        return;
    }
    cu_voxel_t *global = nullptr;
    check(cudaMalloc((void **)&global, n * sizeof(cu_voxel_t)), "cu_voxel_run_length_decode");
    const mcg_status st = mcg_rle_decode_file(ctx, file_name, global, (int64_t)n, dims, params, nullptr);
    if (st != MCG_OK) {
        cudaFree(global);
        fprintf(stderr, "cu_voxel_run_length_decode - malformed file.\n");
        return;
    }
    cudaError_t e = cudaSuccess;
    for (int z = 0; z < size.z && e == cudaSuccess; ++z)
        e = cudaMemcpy2D(cu_voxel_access_yz(v_local, begin_local.y, z + begin_local.z) + begin_local.x,
                         sizeof(cu_voxel_t) * v_local->size.x,
                         global + ((size_t)(z + begin_global.z) * dims[1] + begin_global.y) * dims[0] + begin_global.x,
                         sizeof(cu_voxel_t) * dims[0], sizeof(cu_voxel_t) * size.x, size.y, cudaMemcpyDeviceToDevice);
    cudaFree(global);
    check(e, "cu_voxel_run_length_decode");
}

// ---------------------------------------------------------------------------
// mesh drivers and writers (cu_kinect_fusion_v1.cu:3261-3737)
// ---------------------------------------------------------------------------
namespace {

void mesh_to_file(cu_voxel &volume, const char *file_output, const char *who) {
    MarchingCubes mc;
    cu_array<vertex_voxel> tri;
    cu_array<int3> vi2vox;
    cu_array<short> ver_voxel;
    cu_array<float3> normals;
    cu_array<vertex_voxel> mesh = mc.run(volume, tri, vi2vox, ver_voxel, normals);
    printf("%s - # of triangles = %lld\n", who, (long long)mc.counts().triangles);
    // the writers run on the GPU (mesh_writers.cu): the reference's PLY bytes,
    // and its OBJ with the "%.4f" vertex merge plus qi_volume.txt
    const char *ext = strrchr(file_output, '.');
    const bool obj = ext && strcmp(ext, ".obj") == 0;
    mcg_context *ctx = thread_ctx();
    const mcg_status st =
        mcg_mesh_write(ctx, reinterpret_cast<const mcg_vertex_voxel *>(mesh.ptr()),
                       reinterpret_cast<const float *>(normals.ptr()), (int64_t)mesh.size(), file_output,
                       obj ? "qi_volume.txt" : nullptr, nullptr);
    if (st == MCG_ERR_INVALID_ARG)
        fprintf(stderr, "%s - Invalid file extension (%s)\n", who, ext ? ext : "");
    else if (st == MCG_ERR_IO)
        fprintf(stderr, "%s - cannot write %s\n", who, file_output);
    else
        check_status(st, ctx, who);
}

}  // namespace

void cu_voxel_to_mesh(short2 *_local_volume_data, unsigned int _size_x, unsigned int _size_y, unsigned int _size_z,
                      float _grid_s, const char *file_output) {
    cu_voxel volume;
    memset(&volume, 0, sizeof(volume));
    volume.grid_s = _grid_s;
    volume.size = make_int3((int)_size_x, (int)_size_y, (int)_size_z);
    volume.size_xy = (int)(_size_x * _size_y);
    const size_t n = (size_t)_size_x * _size_y * _size_z;
    // the reference copies the buffer into a fresh volume (:3534-3551); the
    // buffer may be device or host memory here
    check(cudaMalloc((void **)&volume.data, n * sizeof(cu_voxel_t)), "cu_voxel_to_mesh");
    check(cudaMemcpy(volume.data, _local_volume_data, n * sizeof(cu_voxel_t), cudaMemcpyDefault), "cu_voxel_to_mesh");
    try {
        mesh_to_file(volume, file_output, "cu_voxel_to_mesh");
    } catch (...) {
        cu_voxel_delete(&volume);
        throw;
    }
    cu_voxel_delete(&volume);
}

void cu_voxel_rlc_to_mesh(const char *file_input, const char *file_output, int volume_dim) {
    // text records "x y z sdf weight" of the last 11e9 bytes; the records
    // inside [512, 512+dim) x [512, 512+dim) x [0, dim) fill the volume in
    // arrival order, z fastest, then y, then x (:3289-3358), parsed on the
    // GPU by mcg_text_records_load_file; grid 3 mm (:3270).  A file shorter
    // than the tail is read whole (the reference's seek fails there).
    cu_voxel volume;
    memset(&volume, 0, sizeof(volume));
    volume.grid_s = 0.003f;
    volume.size = make_int3(volume_dim, volume_dim, volume_dim);
    volume.size_xy = volume_dim * volume_dim;
    const size_t n = (size_t)volume_dim * volume_dim * volume_dim;
    check(cudaMalloc((void **)&volume.data, n * sizeof(cu_voxel_t)), "cu_voxel_rlc_to_mesh");
    try {
        mcg_context *ctx = thread_ctx();
        const int32_t origin[3] = {512, 512, 0};
        mcg_text_info info;
        const mcg_status st = mcg_text_records_load_file(ctx, file_input, 11000000000LL, volume_dim, origin,
                                                         volume.data, &info, nullptr);
        if (st == MCG_ERR_IO) {
            printf("fail to open %s", file_input);
            cu_voxel_delete(&volume);
            return;
        }
        check_status(st, ctx, "cu_voxel_rlc_to_mesh");
        mesh_to_file(volume, file_output, "cu_voxel_rlc_to_mesh");
    } catch (...) {
        cu_voxel_delete(&volume);
        throw;
    }
    cu_voxel_delete(&volume);
}
