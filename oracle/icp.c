/* CPU oracle of the depth pyramid and projective point-to-plane ICP.
 * TEST INFRASTRUCTURE ONLY: used by tests/ and bench.py's CPU-baseline leg as
 * the checker, never by the product.
 *
 * Per-pixel work is the FP32 mirror of the reference (binary32, source
 * order, no contraction):
 *   orc_float_data_to_mask / orc_float_mask_to_data   kf.cu:66-80
 *   orc_pyramid_down                                  kf.cu:226-261
 *   orc_icp_correspond: step 1 (nearest pixel, kf.cu:988-1029) or step 4
 *     (bilinear, kf.cu:1031-1074), then step 2's row of A and b
 *     (kf.cu:1076-1106) and step 3's inlier flag (kf.cu:1108-1114).
 * The normal equations and the solve follow _cu_icp_projective_3d
 * (kf.cu:1126-1301) in binary64: AtA and Atb are sums of the binary32
 * products A_i * A_j and A_i * b (the reference multiplies with nppsMul_32f
 * and sums with thrust in binary32); Cholesky, the determinant test
 * (|det| > 1e-15), the 1-norm reciprocal condition number (> 5e-5; computed
 * exactly from the inverse, where LAPACK spocon estimates it), the
 * back-substitution, the increment bounds, the rotation exp([w]x) by
 * Rodrigues' formula, compose(pose, inc) and the stopping rule
 * (md' > md or md' < 1e-5 ends the loop).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct { float x, y, z; } f3;

/* kf.cu:66-72 */
void orc_float_data_to_mask(int64_t n, const float *data, uint8_t *mask) {
    for (int64_t i = 0; i < n; ++i) mask[i] = data[i] != 0.0f ? 0xff : 0;
}

/* kf.cu:74-80 */
void orc_float_mask_to_data(int64_t n, const uint8_t *mask, float *data) {
    for (int64_t i = 0; i < n; ++i)
        if (mask[i] == 0) data[i] = 0.0f;
}

/* kf.cu:226-261: 5x5 window from (2x-2, 2y-2), clipped; values within sigma
 * of the centre averaged */
void orc_pyramid_down(int sw, int sh, int dw, int dh, const float *s, const uint8_t *sm, float *d, uint8_t *dm,
                      float sigma) {
    const int D = 5, H = D >> 1;
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            int si = (y << 1) * sw + (x << 1);
            const int di = y * dw + x;
            dm[di] = 0;
            if (!sm[si]) continue;
            const float center = s[si];
            const int tx = (x << 1) - H + D < sw - 1 ? (x << 1) - H + D : sw - 1;
            const int ty = (y << 1) - H + D < sh - 1 ? (y << 1) - H + D : sh - 1;
            float sum = 0.0f;
            int count = 0;
            for (int cy = (y << 1) - H > 0 ? (y << 1) - H : 0; cy < ty; ++cy)
                for (int cx = (x << 1) - H > 0 ? (x << 1) - H : 0; cx < tx; ++cx) {
                    si = cy * sw + cx;
                    if (sm[si]) {
                        const float val = s[si];
                        if (fabsf(val - center) < sigma) {
                            sum += val;
                            ++count;
                        }
                    }
                }
            if (count) {
                d[di] = sum / count;
                dm[di] = 0xff;
            }
        }
}

/* pose: r column-major (columns r[0..2], r[3..5], r[6..8]), t */
static f3 fwd(const float *r, const float *t, f3 p) { /* float_camera_extrinsic_forward */
    f3 q;
    q.x = r[0] * p.x + r[3] * p.y + r[6] * p.z;
    q.y = r[1] * p.x + r[4] * p.y + r[7] * p.z;
    q.z = r[2] * p.x + r[5] * p.y + r[8] * p.z;
    q.x = q.x + t[0];
    q.y = q.y + t[1];
    q.z = q.z + t[2];
    return q;
}
static f3 bwd(const float *r, const float *t, f3 p) { /* float_camera_extrinsic_backward */
    f3 d, q;
    d.x = p.x - t[0];
    d.y = p.y - t[1];
    d.z = p.z - t[2];
    q.x = r[0] * d.x + r[1] * d.y + r[2] * d.z;
    q.y = r[3] * d.x + r[4] * d.y + r[5] * d.z;
    q.z = r[6] * d.x + r[7] * d.y + r[8] * d.z;
    return q;
}
static f3 rot(const float *r, f3 p) { /* float33_mv */
    f3 q;
    q.x = r[0] * p.x + r[3] * p.y + r[6] * p.z;
    q.y = r[1] * p.x + r[4] * p.y + r[7] * p.z;
    q.z = r[2] * p.x + r[5] * p.y + r[8] * p.z;
    return q;
}
static int nz(f3 n) { return n.x != 0.0f || n.y != 0.0f || n.z != 0.0f; }
/* CUDA's float -> int conversions (cvt.rni / cvt.rzi): NaN -> 0, saturating */
static int f2i(float x, int nearest) {
    if (isnan(x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return nearest ? (int)nearbyintf(x) : (int)x;
}
static float dist(f3 a, f3 b) { /* float3_distance */
    float d = a.x - b.x, s = d * d;
    d = a.y - b.y;
    s += d * d;
    d = a.z - b.z;
    s += d * d;
    return sqrtf(s);
}
static f3 bilerp(const f3 *v, float x, float y) { /* vector3_interpolation_bilinear */
    const float a = 1.0f - x, b = 1.0f - y;
    const float ab = a * b, xb = x * b, ay = a * y, xy = x * y;
    f3 u;
    u.x = v[0].x * ab + v[1].x * xb + v[2].x * ay + v[3].x * xy;
    u.y = v[0].y * ab + v[1].y * xb + v[2].y * ay + v[3].y * xy;
    u.z = v[0].z * ab + v[1].z * xb + v[2].z * ay + v[3].z * xy;
    return u;
}

/* One correspondence pass: v21 (FLT_MAX in x when none), the 6 columns of
 * A (column-major, n rows each), b and the inlier flags.  k = {fx, fy, cx, cy}. */
void orc_icp_correspond(int bilinear, float nt, float dt, const float *k, const float *r, const float *t, int w1,
                        int h1, int w2, int h2, const float *v1p, const float *n1p, const float *v2p, const float *n2p,
                        float *v21p, float *A, float *b, uint8_t *inlier) {
    const f3 *v1 = (const f3 *)v1p, *n1 = (const f3 *)n1p, *v2 = (const f3 *)v2p, *n2 = (const f3 *)n2p;
    f3 *v21 = (f3 *)v21p;
    const int64_t rows = (int64_t)w1 * h1;
    for (int64_t idx = 0; idx < rows; ++idx) {
        const f3 a1 = v1[idx], m1 = n1[idx];
        f3 out;
        out.x = FLT_MAX;
        out.y = out.z = 0.0f;
        int found = 0;
        if (nz(m1)) {
            const f3 p3 = bwd(r, t, a1);
            /* float_camera_intrinsic_project_3: fc * (x / z, y / z) + cc */
            const float px = k[0] * (p3.x / p3.z) + k[2], py = k[1] * (p3.y / p3.z) + k[3];
            if (!bilinear) {
                const int ix = f2i(px, 1), iy = f2i(py, 1); /* __float2int_rn */
                if (ix >= 0 && iy >= 0 && ix < w2 && iy < h2) {
                    const int64_t j = (int64_t)iy * w2 + ix;
                    f3 m2 = n2[j];
                    if (nz(m2)) {
                        m2 = rot(r, m2);
                        if (m1.x * m2.x + m1.y * m2.y + m1.z * m2.z > nt) {
                            const f3 a2 = fwd(r, t, v2[j]);
                            if (dist(a1, a2) < dt) {
                                out = a2;
                                found = 1;
                            }
                        }
                    }
                }
            } else {
                const int ix = f2i(px, 0), iy = f2i(py, 0); /* (int) truncation */
                if (ix >= 0 && iy >= 0 && ix < w2 - 1 && iy < h2 - 1) {
                    const int64_t j = (int64_t)iy * w2 + ix;
                    f3 nn[4] = {n2[j], n2[j + 1], n2[j + w2], n2[j + w2 + 1]};
                    if (nz(nn[0]) && nz(nn[1]) && nz(nn[2]) && nz(nn[3])) {
                        const float du = px - ix, dv = py - iy;
                        f3 m2 = rot(r, bilerp(nn, du, dv));
                        if (m1.x * m2.x + m1.y * m2.y + m1.z * m2.z > nt) {
                            nn[0] = v2[j];
                            nn[1] = v2[j + 1];
                            nn[2] = v2[j + w2];
                            nn[3] = v2[j + w2 + 1];
                            const f3 a2 = fwd(r, t, bilerp(nn, du, dv));
                            if (dist(a1, a2) < dt) {
                                out = a2;
                                found = 1;
                            }
                        }
                    }
                }
            }
        }
        if (v21) v21[idx] = out;
        if (inlier) inlier[idx] = found ? 0xff : 0;
        if (A) {
            if (!found) {
                for (int c = 0; c < 6; ++c) A[c * rows + idx] = 0.0f;
                b[idx] = 0.0f;
            } else {
                A[0 * rows + idx] = m1.z * out.y - m1.y * out.z;
                A[1 * rows + idx] = m1.x * out.z - m1.z * out.x;
                A[2 * rows + idx] = m1.y * out.x - m1.x * out.y;
                A[3 * rows + idx] = m1.x;
                A[4 * rows + idx] = m1.y;
                A[5 * rows + idx] = m1.z;
                b[idx] = m1.x * a1.x + m1.y * a1.y + m1.z * a1.z - m1.x * out.x - m1.y * out.y - m1.z * out.z;
            }
        }
    }
}

/* AtA (upper triangle, row-major 21 entries: (0,0),(0,1)..(0,5),(1,1)..) and
 * Atb as binary64 sums of the binary32 products */
void orc_icp_normal_equations(int64_t rows, const float *A, const float *b, double *ata, double *atb) {
    int k = 0;
    for (int i = 0; i < 6; ++i) {
        for (int j = i; j < 6; ++j) {
            double s = 0.0;
            for (int64_t r = 0; r < rows; ++r) s += (double)(A[i * rows + r] * A[j * rows + r]);
            ata[k++] = s;
        }
        double s = 0.0;
        for (int64_t r = 0; r < rows; ++r) s += (double)(A[i * rows + r] * b[r]);
        atb[i] = s;
    }
}

/* The solve of one iteration (kf.cu:1177-1262) on binary64 sums.  Returns
 * 1 and x (w, t) when the step is taken, 0 when the loop must stop with
 * failure; md is the mahalanobis distance Atb . x. */
int orc_icp_solve(const double *ata21, const double *atb, double *x, double *md) {
    double M[6][6], L[6][6];
    int k = 0, count = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) M[i][j] = M[j][i] = ata21[k++];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < i; ++j)
            if (M[i][j] != 0.0) ++count;
    if (count == 0) return 0; /* empty */
    memset(L, 0, sizeof(L));
    for (int j = 0; j < 6; ++j) { /* Cholesky, lower */
        double d = M[j][j];
        for (int p = 0; p < j; ++p) d -= L[j][p] * L[j][p];
        if (!(d > 0.0)) return 0;
        L[j][j] = sqrt(d);
        for (int i = j + 1; i < 6; ++i) {
            double s = M[i][j];
            for (int p = 0; p < j; ++p) s -= L[i][p] * L[j][p];
            L[i][j] = s / L[j][j];
        }
    }
    double det = 1.0;
    for (int i = 0; i < 6; ++i) det *= L[i][i] * L[i][i];
    if (!(fabs(det) > 1e-15)) return 0;
    /* 1-norm of M and of its inverse (columns of the inverse by solves) */
    double anorm = 0.0, inorm = 0.0;
    for (int j = 0; j < 6; ++j) {
        double c = 0.0;
        for (int i = 0; i < 6; ++i) c += fabs(M[i][j]);
        if (c > anorm) anorm = c;
    }
    for (int j = 0; j < 6; ++j) {
        double y[6], z[6];
        for (int i = 0; i < 6; ++i) {
            double s = i == j ? 1.0 : 0.0;
            for (int p = 0; p < i; ++p) s -= L[i][p] * y[p];
            y[i] = s / L[i][i];
        }
        for (int i = 5; i >= 0; --i) {
            double s = y[i];
            for (int p = i + 1; p < 6; ++p) s -= L[p][i] * z[p];
            z[i] = s / L[i][i];
        }
        double c = 0.0;
        for (int i = 0; i < 6; ++i) c += fabs(z[i]);
        if (c > inorm) inorm = c;
    }
    const double rcond = 1.0 / (anorm * inorm);
    if (!(rcond > 5e-5)) return 0;
    double y[6];
    for (int i = 0; i < 6; ++i) {
        double s = atb[i];
        for (int p = 0; p < i; ++p) s -= L[i][p] * y[p];
        y[i] = s / L[i][i];
    }
    for (int i = 5; i >= 0; --i) {
        double s = y[i];
        for (int p = i + 1; p < 6; ++p) s -= L[p][i] * x[p];
        x[i] = s / L[i][i];
    }
    double m = 0.0;
    for (int i = 0; i < 6; ++i) m += atb[i] * x[i];
    *md = m;
    return 1;
}

/* exp([w]x), column-major: R v = v + sin(th)/th w x v + (1-cos(th))/th^2 w x (w x v) */
void orc_so3_exp(const double *w, double *R) {
    const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2], th = sqrt(th2);
    double a, b;
    if (th < 1e-12) {
        a = 1.0;
        b = 0.5;
    } else {
        a = sin(th) / th;
        b = (1.0 - cos(th)) / th2;
    }
    const double K[3][3] = {{0, -w[2], w[1]}, {w[2], 0, -w[0]}, {-w[1], w[0], 0}};  /* K[row][col] */
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            double kk = 0.0;
            for (int p = 0; p < 3; ++p) kk += K[r][p] * K[p][c];
            R[3 * c + r] = (r == c ? 1.0 : 0.0) + a * K[r][c] + b * kk;
        }
}

/* _cu_icp_projective_3d: iterates correspond / equations / solve / update
 * on a binary32 pose (r column-major, t) updated in place; rt result.
 * Scratch: v21 (3 n), A (6 n), b (n) floats. */
int orc_icp(int bilinear, float nt, float dt, float rtb, float ttb, int it_max, const float *k, float *r, float *t,
            int w1, int h1, int w2, int h2, const float *v1, const float *n1, const float *v2, const float *n2,
            uint8_t *inlier, float *v21, float *A, float *b, int *iterations) {
    int it = it_max, rt = 1, iters = 0;
    double md = FLT_MAX;
    const int64_t rows = (int64_t)w1 * h1;
    do {
        ++iters;
        orc_icp_correspond(bilinear, nt, dt, k, r, t, w1, h1, w2, h2, v1, n1, v2, n2, v21, A, b, inlier);
        double ata[21], atb[6], x[6], mdn;
        orc_icp_normal_equations(rows, A, b, ata, atb);
        rt = orc_icp_solve(ata, atb, x, &mdn);
        if (rt) {
            if (fabs(x[0]) > rtb || fabs(x[1]) > rtb || fabs(x[2]) > rtb || fabs(x[3]) > ttb || fabs(x[4]) > ttb ||
                fabs(x[5]) > ttb) {
                rt = 0; /* out of bound */
            } else {
                double Ri[9];
                orc_so3_exp(x, Ri);
                float ri[9], ti[3] = {(float)x[3], (float)x[4], (float)x[5]};
                for (int i = 0; i < 9; ++i) ri[i] = (float)Ri[i];
                /* float_camera_extrinsic_compose(pose, inc): R = Ri R, t = Ri t + ti */
                float nr[9], nt3[3];
                for (int c = 0; c < 3; ++c)
                    for (int rr = 0; rr < 3; ++rr)
                        nr[3 * c + rr] = ri[rr] * r[3 * c] + ri[3 + rr] * r[3 * c + 1] + ri[6 + rr] * r[3 * c + 2];
                for (int rr = 0; rr < 3; ++rr) nt3[rr] = ri[rr] * t[0] + ri[3 + rr] * t[1] + ri[6 + rr] * t[2];
                for (int rr = 0; rr < 3; ++rr) nt3[rr] = nt3[rr] + ti[rr];
                memcpy(r, nr, sizeof(nr));
                memcpy(t, nt3, sizeof(nt3));
                if (mdn > md || mdn < 1e-5) it = 1;
                md = mdn;
            }
        }
    } while (--it && rt);
    if (iterations) *iterations = iters;
    return rt;
}
