// CPU oracle of the text-record volume loader.  TEST INFRASTRUCTURE ONLY:
// used by tests/ and bench.py's CPU-baseline leg as the checker, never by
// the product.
//
// Restates the loop of cu_voxel_rlc_to_mesh (cu_kinect_fusion_v1.cu:3289-3361)
// over std::istream, so that every extraction `is >> int` (white-space
// skipping, signs, range failures, end-of-file bits) is libstdc++'s own:
//
//   seekg(-11e9, end); getline(...)                     (:3316-3317)
//   while (!is.eof()) {
//       is >> x >> y >> z >> sdf >> weight;               (:3320)
//       if (x, y, z inside [xs, xs+dim) x [ys, ys+dim) x [zs, zs+dim)) {
//           v[zi*dim*dim + yi*dim + xi] = {sdf, weight};  (:3327-3328)
//           zi++, carrying into yi, then xi; break once xi == dim
//       }
//   }
//
// Three changes, each where the reference has no defined result:
//  * the volume starts zeroed (the reference's `new cu_voxel_t[]` is left
//    uninitialised);
//  * a file no longer than the tail starts at offset 0 without skipping a
//    line (the reference's negative seek fails there and its loop never
//    ends), and the line cut by the seek is skipped whatever its length
//    (getline(temp, 256) fails on 256 characters or more);
//  * a failed extraction that leaves the record outside the window stops the
//    loop with status 1: the stream stays failed without reaching end of
//    file, so the reference would repeat the same record forever.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <istream>
#include <streambuf>
#include <string>

namespace {

struct MemBuf : std::streambuf {
    MemBuf(const char *b, int64_t n) {
        char *p = const_cast<char *>(b);
        setg(p, p, p + n);
    }
};

// stats[0] voxels stored, stats[1] loop iterations, stats[2] status
void run(std::istream &is, int dim, int xs, int ys, int zs, int16_t *vol, int64_t *stats) {
    int x = 0, y = 0, z = 0, sdf = 0, weight = 0;
    const int64_t d = dim;
    int64_t xi = 0, yi = 0, zi = 0;
    while (!is.eof()) {
        is >> x >> y >> z >> sdf >> weight;
        ++stats[1];
        if (xs <= x && x < xs + dim && ys <= y && y < ys + dim && zs <= z && z < zs + dim) {
            int16_t *v = vol + 2 * (zi * d * d + yi * d + xi);
            v[0] = (int16_t)(uint16_t)(uint32_t)sdf;     // short tsdf
            v[1] = (int16_t)(uint16_t)(uint32_t)weight;  // ushort w
            ++stats[0];
            if (++zi >= d) {
                zi = 0;
                ++yi;
            }
            if (yi >= d) {
                yi = 0;
                ++xi;
            }
            if (xi >= d) break;
        } else if (is.fail() && !is.eof()) {
            stats[2] = 1;
            break;
        }
    }
}

}  // namespace

extern "C" {

// Parse a text held in memory (no seek).  Returns 0.
int orc_text_load(const char *text, int64_t len, int dim, int xs, int ys, int zs, int16_t *vol, int64_t *stats) {
    std::memset(vol, 0, sizeof(int16_t) * 2 * (size_t)dim * dim * dim);
    stats[0] = stats[1] = stats[2] = 0;
    MemBuf buf(text, len);
    std::istream is(&buf);
    run(is, dim, xs, ys, zs, vol, stats);
    return 0;
}

// Parse the last tail_bytes of a file (the reference's seek and line skip).
// Returns 0, or -1 when the file cannot be opened.
int orc_text_load_file(const char *path, int64_t tail_bytes, int dim, int xs, int ys, int zs, int16_t *vol,
                       int64_t *stats) {
    std::memset(vol, 0, sizeof(int16_t) * 2 * (size_t)dim * dim * dim);
    stats[0] = stats[1] = stats[2] = 0;
    std::ifstream is(path, std::ios_base::in);
    if (!is.is_open()) return -1;
    is.seekg(0, std::ios::end);
    const int64_t len = (int64_t)is.tellg();
    if (tail_bytes > 0 && len > tail_bytes) {
        is.seekg(len - tail_bytes, std::ios::beg);
        std::string skip;
        std::getline(is, skip);
    } else {
        is.seekg(0, std::ios::beg);
    }
    run(is, dim, xs, ys, zs, vol, stats);
    return 0;
}

}  // extern "C"
