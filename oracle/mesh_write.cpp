// CPU oracle of the mesh writers.  TEST INFRASTRUCTURE ONLY: used by tests/
// and bench.py's CPU-baseline leg as the checker, never by the product.
//
// Restates the writers of cu_voxel_rlc_to_mesh / cu_voxel_to_mesh with the
// same stdio calls, so glibc does every number conversion:
//   binary PLY soup (cu_kinect_fusion_v1.cu:3394-3424): header, per vertex
//     position then normal (float3 each), per triangle uint8 3 + int32
//     (3i, 3i+1, 3i+2);
//   OBJ (:3625-3726): a vertex is new when the key "%.4f_%.4f_%.4f" of its
//     position was not seen before (std::map); a new vertex writes
//     "v %f %f %f" and "vn %f %f %f" and a "qi tsdf w vx vy vz" line
//     ("%d %hd %hd %d %d %d"); a triangle writes "f a b c" with the ids of
//     its three keys unless two of them are equal.
// Output goes to memory (open_memstream) instead of files.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <string>
#include <vector>

namespace {

struct Vtx {  // structure.h vertex_voxel, 28 bytes
    float x, y, z;
    int32_t vx, vy, vz;
    int16_t tsdf, w;
};
static_assert(sizeof(Vtx) == 28, "vertex_voxel layout");

// closes the stream (which sets *buf and *len) and copies the bytes out
int64_t take(FILE *f, char **buf, size_t *len, uint8_t *out, int64_t cap) {
    fclose(f);
    const int64_t n = (int64_t)*len;
    if (out && cap >= n) memcpy(out, *buf, *len);
    free(*buf);
    return n;
}

}  // namespace

extern "C" {

// Returns the image size; the image is copied when cap is large enough.
int64_t orc_mesh_ply(const void *soup, const float *normals, int64_t n, uint8_t *out, int64_t cap) {
    const Vtx *v = static_cast<const Vtx *>(soup);
    char *buf = nullptr;
    size_t len = 0;
    FILE *fp = open_memstream(&buf, &len);
    fprintf(fp, "ply\n");
    fprintf(fp, "format binary_little_endian 1.0\n");
    fprintf(fp, "element vertex %d\n", (int)n);
    fprintf(fp, "property float32 x\n");
    fprintf(fp, "property float32 y\n");
    fprintf(fp, "property float32 z\n");
    fprintf(fp, "property float32 nx\n");
    fprintf(fp, "property float32 ny\n");
    fprintf(fp, "property float32 nz\n");
    fprintf(fp, "element face %d\n", (int)(n / 3));
    fprintf(fp, "property list uint8 int32 vertex_indices\n");
    fprintf(fp, "end_header\n");
    for (int64_t i = 0; i < n; ++i) {
        fwrite(&v[i].x, sizeof(float), 3, fp);
        fwrite(normals + 3 * i, sizeof(float), 3, fp);
    }
    const unsigned char prop = 3;
    for (int64_t i = 0; i < n / 3; ++i) {
        const int face[3] = {(int)(3 * i), (int)(3 * i + 1), (int)(3 * i + 2)};
        fwrite(&prop, 1, 1, fp);
        fwrite(face, sizeof(int), 3, fp);
    }
    return take(fp, &buf, &len, out, cap);
}

// OBJ and qi images; sizes in sizes[0], sizes[1].
void orc_mesh_obj(const void *soup, const float *normals, int64_t n, uint8_t *obj, int64_t obj_cap, uint8_t *qi,
                  int64_t qi_cap, int64_t *sizes) {
    const Vtx *v = static_cast<const Vtx *>(soup);
    char *ob = nullptr, *qb = nullptr;
    size_t ol = 0, ql = 0;
    FILE *fp = open_memstream(&ob, &ol);
    FILE *fq = open_memstream(&qb, &ql);
    fprintf(fq, "qi tsdf w vx vy vz\n");
    std::map<std::string, int> id;
    std::vector<std::string> keys((size_t)n);
    int count = 0;
    for (int64_t i = 0; i < n; ++i) {
        char str[64];
        snprintf(str, sizeof(str), "%.4f_%.4f_%.4f", v[i].x, v[i].y, v[i].z);
        std::string s(str);
        if (id.find(s) == id.end()) {
            fprintf(fp, "v %f %f %f\n", v[i].x, v[i].y, v[i].z);
            fprintf(fp, "vn %f %f %f\n", normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
            id[s] = ++count;
            fprintf(fq, "%d %hd %hd %d %d %d\n", count, v[i].tsdf, v[i].w, v[i].vx, v[i].vy, v[i].vz);
        }
        keys[(size_t)i] = s;
    }
    for (int64_t t = 0; t < n / 3; ++t) {
        const int a = id[keys[3 * t]], b = id[keys[3 * t + 1]], c = id[keys[3 * t + 2]];
        if (a == b || a == c || b == c) continue;
        fprintf(fp, "f %d %d %d\n", a, b, c);
    }
    sizes[0] = take(fp, &ob, &ol, obj, obj_cap);
    sizes[1] = take(fq, &qb, &ql, qi, qi_cap);
}

}  // extern "C"
