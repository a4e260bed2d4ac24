// Exercises the reference-compatible C++ interface (include/structure.h,
// cu_memory.hpp, cu_marching_cubes_v1.h, cu_kinect_fusion_v1.h) the way a
// caller of the reference does: volume in, mesh file out; integrate; RLE;
// a text-record dump to a mesh (cu_voxel_rlc_to_mesh).
// Usage: dropin_main <workdir>   (prints one JSON line of results)
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "cu_kinect_fusion_v1.h"
#include "cu_marching_cubes_v1.h"
#include "cu_memory.hpp"
#include "structure.h"

static std::vector<short2> sphere(int n, float r) {
    std::vector<short2> v((size_t)n * n * n);
    const float c = n / 2.0f;
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                const float dx = x + 0.5f - c, dy = y + 0.5f - c, dz = z + 0.5f - c;
                float sd = (sqrtf(dx * dx + dy * dy + dz * dz) - r) / 5.0f;
                sd = sd < -1 ? -1 : sd > 1 ? 1 : sd;
                short2 s;
                s.x = (short)(sd * 32767.0f);
                s.y = (short)(1 + (x + y + z) % 100);
                v[((size_t)z * n + y) * n + x] = s;
            }
    return v;
}

int main(int argc, char **argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    const int n = 48;
    std::vector<short2> h = sphere(n, 15.0f);
    // 1. cu_voxel_to_mesh with a host buffer -> PLY and OBJ
    cu_voxel_to_mesh(h.data(), n, n, n, 0.01f, (dir + "/sphere.ply").c_str());
    cu_voxel_to_mesh(h.data(), n, n, n, 0.01f, (dir + "/sphere.obj").c_str());
    // 2. MarchingCubes::run on a device volume
    cu_voxel vol;
    memset(&vol, 0, sizeof(vol));
    cu_voxel_new(&vol, make_int3(n, n, n), 0.03f, 0.03f, 0.01f);
    cudaMemcpy(vol.data, h.data(), h.size() * sizeof(short2), cudaMemcpyHostToDevice);
    MarchingCubes mc;
    cu_array<vertex_voxel> tri;
    cu_array<int3> vi2vox;
    cu_array<short> ver_voxel;
    cu_array<vertex_voxel> mesh = mc.run(vol, tri, vi2vox, ver_voxel);
    // copies share the buffer; the returned view does not own it
    cu_array<vertex_voxel> copy = tri;
    const bool shared = copy.ptr() == tri.ptr() && mesh.ptr() == tri.ptr();
    // 2b. adjoint of the run's positions for a constant dL/dP (order-free)
    {
        std::vector<float3> gp(mesh.size(), make_float3(1.0f, 0.5f, -0.25f));
        cu_array<float3> grad_pos;
        grad_pos.upload(gp);
        cu_array<float> grad_tsdf;
        mc.backward(vol, grad_pos, grad_tsdf);
        std::vector<float> g;
        grad_tsdf.download(g);
        FILE *f = fopen((dir + "/grad_tsdf.bin").c_str(), "wb");
        if (f) {
            fwrite(g.data(), sizeof(float), g.size(), f);
            fclose(f);
        }
    }
    // 3. RLE: write the whole volume, then rewrite a window, read back
    const std::string rle = dir + "/vol.rle";
    remove(rle.c_str());
    cu_voxel_run_length_encode(&vol, rle.c_str(), make_int3(0, 0, 0), make_int3(0, 0, 0), make_int3(0, 0, 0));
    cu_voxel back;
    memset(&back, 0, sizeof(back));
    cu_voxel_run_length_decode(&back, rle.c_str(), make_int3(0, 0, 0), make_int3(0, 0, 0), make_int3(0, 0, 0));
    std::vector<short2> hb((size_t)n * n * n);
    cudaMemcpy(hb.data(), back.data, hb.size() * sizeof(short2), cudaMemcpyDeviceToHost);
    size_t tsdf_equal = 0;
    for (size_t i = 0; i < hb.size(); ++i) tsdf_equal += hb[i].x == h[i].x;
    // window: local 8^3 sub-volume of -32766/w=0 written at global (4, 5, 6)
    cu_voxel win;
    memset(&win, 0, sizeof(win));
    cu_voxel_new(&win, make_int3(8, 8, 8), 0.03f, 0.03f, 0.01f);
    cu_voxel_run_length_encode(&win, rle.c_str(), make_int3(0, 0, 0), make_int3(4, 5, 6), make_int3(8, 8, 8));
    cu_voxel part;
    memset(&part, 0, sizeof(part));
    cu_voxel_new(&part, make_int3(10, 10, 10), 0.03f, 0.03f, 0.01f);
    cu_voxel_run_length_decode(&part, rle.c_str(), make_int3(0, 0, 0), make_int3(3, 4, 5), make_int3(10, 10, 10));
    std::vector<short2> hp(1000);
    cudaMemcpy(hp.data(), part.data, hp.size() * sizeof(short2), cudaMemcpyDeviceToHost);
    // global (4..11, 5..12, 6..13) is -32766 now; part starts at global (3,4,5)
    const short2 inner = hp[(2 * 10 + 2) * 10 + 2];   // global (5, 6, 7)
    const short2 outer = hp[0];                       // global (3, 4, 5): original
    const short2 orig = h[((size_t)5 * n + 4) * n + 3];
    // 4. integrate one frame into a fresh volume through the reference signature
    cu_voxel fv;
    memset(&fv, 0, sizeof(fv));
    cu_voxel_new(&fv, make_int3(32, 32, 32), 0.15f, 0.15f, 0.05f);
    float_camera_intrinsic k;
    memset(&k, 0, sizeof(k));
    k.fc = make_float2(60.0f, 60.0f);
    k.cc = make_float2(31.5f, 31.5f);
    float_camera_extrinsic e;
    memset(&e, 0, sizeof(e));
    e.R.p[0] = make_float3(1, 0, 0);
    e.R.p[1] = make_float3(0, 1, 0);
    e.R.p[2] = make_float3(0, 0, 1);
    e.t = make_float3(0.6f, 0.6f, 0.0f);
    std::vector<float> depth(64 * 64, 1.0f);
    float *d_depth = nullptr;
    cudaMalloc((void **)&d_depth, depth.size() * sizeof(float));
    cudaMemcpy(d_depth, depth.data(), depth.size() * sizeof(float), cudaMemcpyHostToDevice);
    _cu_voxel_volumetric_integration(fv, k, e, make_int2(64, 64), d_depth, nullptr, nullptr, false);
    short2 probe;
    cudaMemcpy(&probe, fv.data + ((size_t)18 * 32 + 12) * 32 + 12, sizeof(short2), cudaMemcpyDeviceToHost);
    // 5. vmap on host buffers
    std::vector<float> meter(16 * 12, 1.5f);
    std::vector<float3> vtx(16 * 12);
    cu_meter_to_vertex(k, make_int2(16, 12), meter.data(), vtx.data());
    // 6. cu_voxel_rlc_to_mesh: the sphere as text records of the window at
    //    (512, 512, 0), x outermost, z innermost, trailing newline
    {
        FILE *f = fopen((dir + "/sphere_dump.vol").c_str(), "w");
        if (f) {
            for (int x = 0; x < n; ++x)
                for (int y = 0; y < n; ++y)
                    for (int z = 0; z < n; ++z) {
                        const short2 s = h[((size_t)z * n + y) * n + x];
                        fprintf(f, "%d %d %d %d %d\n", 512 + x, 512 + y, z, (int)s.x, (int)(unsigned short)s.y);
                    }
            fclose(f);
        }
        cu_voxel_rlc_to_mesh((dir + "/sphere_dump.vol").c_str(), (dir + "/text.ply").c_str(), n);
    }
    printf("{\"triangles\": %lld, \"mesh_size\": %zu, \"shared\": %d, \"tsdf_equal\": %zu, \"voxels\": %zu, "
           "\"inner\": [%d, %d], \"outer\": [%d, %d], \"orig\": [%d, %d], \"probe\": [%d, %d], "
           "\"vtx0\": [%g, %g, %g]}\n",
           (long long)mc.counts().triangles, mesh.size(), shared ? 1 : 0, tsdf_equal, hb.size(), inner.x,
           (unsigned short)inner.y, outer.x, (unsigned short)outer.y, orig.x, (unsigned short)orig.y, probe.x,
           (unsigned short)probe.y, vtx[0].x, vtx[0].y, vtx[0].z);
    cudaFree(d_depth);
    cu_voxel_delete(&vol);
    cu_voxel_delete(&back);
    cu_voxel_delete(&win);
    cu_voxel_delete(&part);
    cu_voxel_delete(&fv);
    return 0;
}
