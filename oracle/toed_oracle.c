/*
 * toed_oracle.c -- CPU restatement of the Third-Order Edge Detector hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/, the
 * smoke() entry and bench.py's CPU-baseline leg call it as the checker.  The
 * product (the CUDA library) never links or calls it.
 *
 * Two pipelines are restated, each with the same loop order and the same
 * floating-point association as the reference so that, given identical taps,
 * results are bit-identical in double precision:
 *
 *  1. TOED detection (reference cpu_toed.cpp):
 *     - taps            cpu_toed.cpp:141-167 (formula in the comments :141-162)
 *     - convolve_img    cpu_toed.cpp:128-369 (4 sub-grids, direct 2-D sums,
 *                       zero padding, TO orientation :227-232)
 *     - NMS + fit       cpu_toed.cpp:379-506
 *     - compaction      cpu_toed.cpp:508-538 (row-major over the 2x grid,
 *                       x_out = (pos_x-1)/2, y_out = (pos_y-1)/2)
 *     - MATLAB QaD orientation (third_order_edge_detector.m:91-141):
 *                       toed_oracle_detect_qad, derivatives cubic-interpolated
 *                       at the subpixel point
 *     - extension: NMS and peak fit along the corrected normal (the
 *                       third-order vector) instead of the gradient,
 *                       toed_oracle_detect_ex(nms_dir = 1)
 *     Extensions over the reference (which hard-codes sigma = 2 through literal
 *     taps, kernel 17 and threshold 2): any sigma with taps from the
 *     reference's own commented formula, any half-width r, any threshold,
 *     double input.  With the reference's literal taps passed in, the output
 *     equals the reference's bit for bit (pinned by tests/test_oracle_pin.py).
 *
 *  2. Subpixel TO correction (reference subpix_TO_correction/
 *     subpix_to_correction.cpp, interp_n = 0):
 *     - build_gaussian_kernels  :195-214
 *     - estimate_orientation    :307-375 (triangle r=4, symmetric padding,
 *                                         gradient2 with one-sided borders)
 *     - compute_dir_from_theta  :296-305
 *     - nms_token               :413-519 (margin 3)
 *     - conv_separable_circular :377-411 (circular padding)
 *     - interp2_cubic           :521-556 (Keys a=-0.5, clamp to edge)
 *     - remove_isolated_edgels  :563-621 (cell grid of size radius, 3x3 cells)
 *     - run                     :623-736
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off), so that x86
 * and aarch64 hosts evaluate the same operation sequence.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <omp.h>

#define ORACLE_PI 3.14159265358979323846

/* ------------------------------------------------------------------------ */
/* Taps                                                                      */
/* ------------------------------------------------------------------------ */
/*
 * Layout of the tap block (8 arrays of n = 2r+3 doubles), index k <-> offset
 * x = k - (r+1) (+0.5 for the shifted set):
 *   0: G      1: Gx      2: Gxx      3: Gxxx          (unshifted)
 *   4: G_sh   5: Gx_sh   6: Gxx_sh   7: Gxxx_sh       (shifted by +0.5)
 * Formulas: the reference's commented generator, cpu_toed.cpp:141-162 /
 * gpu_toed.hpp:350-366:
 *   G    = exp(-x^2/2s^2) / (sqrt(2 pi) s)
 *   Gx   = -x exp(..) / (sqrt(2 pi) s^3)
 *   Gxx  = (x^2 - s^2) exp(..) / (sqrt(2 pi) s^5)
 *   Gxxx = x (3 s^2 - x^2) exp(..) / (sqrt(2 pi) s^7)
 */
void toed_oracle_taps(double sigma, int r, double *taps)
{
    const int n = 2 * r + 3;
    const double s = sigma;
    const double nrm = sqrt(2.0 * ORACLE_PI);
    for (int sh = 0; sh < 2; sh++) {
        const double d = sh ? 0.5 : 0.0;
        for (int k = 0; k < n; k++) {
            const double x = (double)(k - (r + 1)) + d;
            const double e = exp(-(x * x) / (2.0 * s * s));
            taps[(4 * sh + 0) * n + k] = e / (nrm * s);
            taps[(4 * sh + 1) * n + k] = (-x * e) / (nrm * s * s * s);
            taps[(4 * sh + 2) * n + k] = ((x * x - s * s) * e) / (nrm * s * s * s * s * s);
            taps[(4 * sh + 3) * n + k] = ((x * (3.0 * s * s - x * x)) * e) /
                                         (nrm * s * s * s * s * s * s * s);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* TOED: derivative planes on the 2x grid (cpu_toed.cpp:128-369)              */
/* ------------------------------------------------------------------------ */
/*
 * img: H*W doubles row-major.  Outputs are (2H)*(2W) row-major planes; any of
 * them may be NULL except where noted.  taps: block from toed_oracle_taps
 * (or the reference's literal table) for half-width r.
 */
static inline void to_orientation(double fx, double fy, double fxx, double fxy,
                                  double fyy, double fxxy, double fxyy,
                                  double fxxx, double fyyy, double *ori)
{
    /* cpu_toed.cpp:227-232 */
    double tix = fx * (2 * fxx * fxx + 2 * fxy * fxy) + fy * (2 * fxx * fxy + 2 * fyy * fxy) +
                 2 * fx * fy * fxxy + fy * fy * fxyy + fx * fx * fxxx;
    double tiy = fx * (2 * fxx * fxy + 2 * fyy * fxy) + fy * (2 * fyy * fyy + 2 * fxy * fxy) +
                 2 * fx * fy * fxyy + fx * fx * fxxy + fy * fy * fyyy;
    double m = sqrt(tix * tix + tiy * tiy);
    tix /= m;
    tiy /= m;
    *ori = atan2(tix, -tiy);
}

/* The third-order vector itself (cpu_toed.cpp:227-230), before normalisation. */
static inline void to_vector(double fx, double fy, double fxx, double fxy, double fyy, double fxxy,
                             double fxyy, double fxxx, double fyyy, double *tix, double *tiy)
{
    *tix = fx * (2 * fxx * fxx + 2 * fxy * fxy) + fy * (2 * fxx * fxy + 2 * fyy * fxy) +
           2 * fx * fy * fxxy + fy * fy * fxyy + fx * fx * fxxx;
    *tiy = fx * (2 * fxx * fxy + 2 * fyy * fxy) + fy * (2 * fyy * fyy + 2 * fxy * fxy) +
           2 * fx * fy * fxyy + fx * fx * fxxy + fy * fy * fyyy;
}

static void oracle_planes(const double *img, int H, int W, int r, const double *taps, int nthreads,
                          double *Ix, double *Iy, double *mag, double *ori, double *derivs9,
                          double *tvec);

void toed_oracle_planes(const double *img, int H, int W, int r, const double *taps,
                        int nthreads, double *Ix, double *Iy, double *mag, double *ori,
                        double *derivs9 /* optional: 9 planes of (2H)(2W) */)
{
    oracle_planes(img, H, W, r, taps, nthreads, Ix, Iy, mag, ori, derivs9, NULL);
}

/* tvec (optional): 2 planes, the third-order vector (TO_Ix, TO_Iy) per point. */
static void oracle_planes(const double *img, int H, int W, int r, const double *taps, int nthreads,
                          double *Ix, double *Iy, double *mag, double *ori, double *derivs9,
                          double *tvec)
{
    const int n = 2 * r + 3;
    const double *G = taps + 0 * n, *Gx = taps + 1 * n, *Gxx = taps + 2 * n, *Gxxx = taps + 3 * n;
    const double *G_sh = taps + 4 * n, *Gx_sh = taps + 5 * n, *Gxx_sh = taps + 6 * n,
                 *Gxxx_sh = taps + 7 * n;
    const int cent = r, ci = r + 1;
    const int W2 = 2 * W;
    const size_t P2 = (size_t)(2 * H) * (size_t)W2;
    if (nthreads > 0) omp_set_num_threads(nthreads);

#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            /* four sub-grids: (a,b) in {(0,0),(0,1),(1,0),(1,1)} = rows si+a, cols sj+b */
            for (int sg = 0; sg < 4; sg++) {
                const int a = sg >> 1, b = sg & 1;
                double fx = 0, fy = 0, fxx = 0, fyy = 0, fxy = 0, fxxy = 0, fxyy = 0, fxxx = 0,
                       fyyy = 0;
                if (sg == 0) {
                    /* cpu_toed.cpp:205-221: 17x17 at sigma 2, taps index q+cent+1 */
                    for (int p = -cent; p <= cent; p++) {
                        for (int q = -cent; q <= cent; q++) {
                            if ((i - p) < 0 || (j - q) < 0 || (i - p) >= H || (j - q) >= W) continue;
                            const double v = img[(size_t)(i - p) * W + (j - q)];
                            const int kq = q + cent + 1, kp = p + cent + 1;
                            fx += v * (Gx[kq] * G[kp]);
                            fy += v * (G[kq] * Gx[kp]);
                            fxx += v * Gxx[kq] * G[kp];
                            fxy += v * Gx[kq] * Gx[kp];
                            fyy += v * G[kq] * Gxx[kp];
                            fxxy += v * Gxx[kq] * Gx[kp];
                            fxyy += v * Gx[kq] * Gxx[kp];
                            fxxx += v * Gxxx[kq] * G[kp];
                            fyyy += v * G[kq] * Gxxx[kp];
                        }
                    }
                } else {
                    /* cpu_toed.cpp:246-262 (b=1), :287-303 (a=1), :328-344 (a=b=1) */
                    const double *XG = b ? G_sh : G, *XGx = b ? Gx_sh : Gx, *XGxx = b ? Gxx_sh : Gxx,
                                 *XGxxx = b ? Gxxx_sh : Gxxx;
                    const double *YG = a ? G_sh : G, *YGx = a ? Gx_sh : Gx, *YGxx = a ? Gxx_sh : Gxx,
                                 *YGxxx = a ? Gxxx_sh : Gxxx;
                    for (int p = -ci; p <= ci; p++) {
                        for (int q = -ci; q <= ci; q++) {
                            if ((i - p) < 0 || (j - q) < 0 || (i - p) >= H || (j - q) >= W) continue;
                            const double v = img[(size_t)(i - p) * W + (j - q)];
                            const int kq = q + ci, kp = p + ci;
                            fx += v * XGx[kq] * YG[kp];
                            fy += v * XG[kq] * YGx[kp];
                            fxx += v * XGxx[kq] * YG[kp];
                            fxy += v * XGx[kq] * YGx[kp];
                            fyy += v * XG[kq] * YGxx[kp];
                            fxxy += v * XGxx[kq] * YGx[kp];
                            fxyy += v * XGx[kq] * YGxx[kp];
                            fxxx += v * XGxxx[kq] * YG[kp];
                            fyyy += v * XG[kq] * YGxxx[kp];
                        }
                    }
                }
                const size_t o = (size_t)(2 * i + a) * W2 + (size_t)(2 * j + b);
                if (Ix) Ix[o] = fx;
                if (Iy) Iy[o] = fy;
                if (mag) mag[o] = sqrt(fx * fx + fy * fy);
                if (ori) to_orientation(fx, fy, fxx, fxy, fyy, fxxy, fxyy, fxxx, fyyy, &ori[o]);
                if (tvec) to_vector(fx, fy, fxx, fxy, fyy, fxxy, fxyy, fxxx, fyyy, &tvec[o], &tvec[P2 + o]);
                if (derivs9) {
                    const double d9[9] = {fx, fy, fxx, fxy, fyy, fxxy, fxyy, fxxx, fyyy};
                    for (int k = 0; k < 9; k++) derivs9[(size_t)k * P2 + o] = d9[k];
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* TOED: NMS with parabola fit (cpu_toed.cpp:379-506)                        */
/* ------------------------------------------------------------------------ */
/*
 * Sector selection and neighbour interpolation shared by the TOED NMS
 * (cpu_toed.cpp:414-462) and nms_token (subpix_to_correction.cpp:453-493).
 * M(i,j) accessor = plane[(i)*w + (j)].  Returns slope, fp, fm.
 */
static inline void nms_sector(const double *M, int w, int i, int j, double gx, double gy,
                              double nx, double ny, double *slope_o, double *fp_o, double *fm_o)
{
#define MM(ii, jj) M[(size_t)(ii) * w + (jj)]
    double slope = 0, fp = 0, fm = 0;
    if ((gx >= 0) && (gy >= 0)) {
        if (gx >= gy) {
            slope = ny / nx;
            fp = MM(i, j + 1) * (1 - slope) + MM(i + 1, j + 1) * slope;
            fm = MM(i, j - 1) * (1 - slope) + MM(i - 1, j - 1) * slope;
        } else {
            slope = nx / ny;
            fp = MM(i + 1, j) * (1 - slope) + MM(i + 1, j + 1) * slope;
            fm = MM(i - 1, j) * (1 - slope) + MM(i - 1, j - 1) * slope;
        }
    } else if ((gx < 0) && (gy >= 0)) {
        if (fabs(gx) < gy) {
            slope = -nx / ny;
            fp = MM(i + 1, j) * (1 - slope) + MM(i + 1, j - 1) * slope;
            fm = MM(i - 1, j) * (1 - slope) + MM(i - 1, j + 1) * slope;
        } else {
            slope = -ny / nx;
            fp = MM(i, j - 1) * (1 - slope) + MM(i + 1, j - 1) * slope;
            fm = MM(i, j + 1) * (1 - slope) + MM(i - 1, j + 1) * slope;
        }
    } else if ((gx < 0) && (gy < 0)) {
        if (fabs(gx) >= fabs(gy)) {
            slope = ny / nx;
            fp = MM(i, j - 1) * (1 - slope) + MM(i - 1, j - 1) * slope;
            fm = MM(i, j + 1) * (1 - slope) + MM(i + 1, j + 1) * slope;
        } else {
            slope = nx / ny;
            fp = MM(i - 1, j) * (1 - slope) + MM(i - 1, j - 1) * slope;
            fm = MM(i + 1, j) * (1 - slope) + MM(i + 1, j + 1) * slope;
        }
    } else if ((gx >= 0) && (gy < 0)) {
        if (gx < fabs(gy)) {
            slope = -nx / ny;
            fp = MM(i - 1, j) * (1 - slope) + MM(i - 1, j + 1) * slope;
            fm = MM(i + 1, j) * (1 - slope) + MM(i + 1, j - 1) * slope;
        } else {
            slope = -ny / nx;
            fp = MM(i, j + 1) * (1 - slope) + MM(i - 1, j + 1) * slope;
            fm = MM(i, j - 1) * (1 - slope) + MM(i + 1, j - 1) * slope;
        }
    }
#undef MM
    *slope_o = slope;
    *fp_o = fp;
    *fm_o = fm;
}

/*
 * NMS over the 2x grid interior [10, 2H-10) x [10, 2W-10) (cpu_toed.cpp:400-401).
 * pos_x/pos_y/smag: (2H)(2W) planes, zeroed here, written where accepted.
 */
static void oracle_nms(const double *Ix, const double *Iy, const double *mag, const double *tvec, int H2,
                       int W2, double threshold, int nthreads, double *pos_x, double *pos_y, double *smag);

void toed_oracle_nms(const double *Ix, const double *Iy, const double *mag, int H2, int W2,
                     double threshold, int nthreads, double *pos_x, double *pos_y, double *smag)
{
    oracle_nms(Ix, Iy, mag, NULL, H2, W2, threshold, nthreads, pos_x, pos_y, smag);
}

/*
 * tvec == NULL: the reference's NMS along the first-order gradient (Ix, Iy).
 * tvec != NULL (extension, no counterpart in the reference): the same
 * candidates (threshold and gradient checks, :403, :407), but the sector,
 * the interpolated neighbours, the parabola fit and the subpixel offset are
 * taken along the unit third-order vector (TO_Ix, TO_Iy) -- the corrected
 * normal of the edge, whose tangent is the emitted orientation
 * atan2(TO_Ix, -TO_Iy) -- instead of along the gradient; a point whose
 * vector vanishes has no direction and is skipped.
 */
static void oracle_nms(const double *Ix, const double *Iy, const double *mag, const double *tvec, int H2,
                       int W2, double threshold, int nthreads, double *pos_x, double *pos_y, double *smag)
{
    const size_t P2 = (size_t)H2 * W2;
    memset(pos_x, 0, P2 * sizeof(double));
    memset(pos_y, 0, P2 * sizeof(double));
    memset(smag, 0, P2 * sizeof(double));
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
    for (int j = 10; j < W2 - 10; j++) {
        for (int i = 10; i < H2 - 10; i++) {
            const size_t o = (size_t)i * W2 + j;
            const double m = mag[o];
            if (m <= threshold) continue;                                  /* :403 */
            if ((fabs(Ix[o]) < 10e-6) && (fabs(Iy[o]) < 10e-6)) continue; /* :407 */
            double dx = Ix[o], dy = Iy[o], dm = m;
            if (tvec) {
                dx = tvec[o];
                dy = tvec[P2 + o];
                dm = sqrt(dx * dx + dy * dy);
                if (!(dm > 0) || !isfinite(dm)) continue;
            }
            const double nx = dx / dm, ny = dy / dm; /* :411-412 */
            double slope, fp, fm;
            nms_sector(mag, W2, i, j, dx, dy, nx, ny, &slope, &fp, &fm);
            const double s = sqrt(1 + slope * slope); /* :465 */
            if ((m > fm && m > fp) || (m > fm && m >= fp) || (m >= fm && m > fp)) {
                const double A = (fm + fp - 2 * m) / (2 * s * s); /* :471-476 */
                const double B = (fp - fm) / (2 * s);
                const double C = m;
                const double s_star = -B / (2 * A);
                const double max_f = A * s_star * s_star + B * s_star + C;
                if (fabs(s_star) <= sqrt(2.0)) { /* :478 */
                    const double gxs = max_f * nx, gys = max_f * ny;
                    pos_x[o] = j + s_star * nx; /* :488-489 */
                    pos_y[o] = i + s_star * ny;
                    smag[o] = sqrt(gxs * gxs + gys * gys);
                }
            }
        }
    }
}

/* Row-major compaction over the 2x grid (cpu_toed.cpp:510-538).  Returns N. */
long toed_oracle_compact(const double *pos_x, const double *pos_y, const double *ori,
                         const double *smag, int H2, int W2, double *edges, long capacity,
                         int64_t *index_out)
{
    long n = 0;
    for (int i = 0; i < H2; i++) {
        for (int j = 0; j < W2; j++) {
            const size_t o = (size_t)i * W2 + j;
            if (pos_x[o] != 0) {
                if (n < capacity) {
                    edges[4 * n + 0] = (pos_x[o] - 1) / 2;
                    edges[4 * n + 1] = (pos_y[o] - 1) / 2;
                    edges[4 * n + 2] = ori[o];
                    edges[4 * n + 3] = smag[o];
                    if (index_out) index_out[n] = (int64_t)o;
                }
                n++;
            }
        }
    }
    return n;
}

/*
 * Whole TOED pipeline.  taps may be NULL (then generated from sigma for
 * half-width r).  edges: capacity*4 doubles.  Optional plane outputs (may be
 * NULL): planes4 = 4 planes (Ix, Iy, mag, ori), posmaps = 3 planes
 * (pos_x, pos_y, strength), each (2H)(2W); index_out = 2x-grid linear index
 * (row * 2W + col) of each edgel.  Returns N (may exceed capacity; only the
 * first `capacity` edgels are written).
 */
long toed_oracle_detect_ex(const double *img, int H, int W, double sigma, int r, const double *taps_in,
                           double threshold, int nthreads, double *edges, long capacity, double *planes4,
                           double *posmaps, int64_t *index_out, int nms_dir);

long toed_oracle_detect(const double *img, int H, int W, double sigma, int r,
                        const double *taps_in, double threshold, int nthreads, double *edges,
                        long capacity, double *planes4, double *posmaps, int64_t *index_out)
{
    return toed_oracle_detect_ex(img, H, W, sigma, r, taps_in, threshold, nthreads, edges, capacity, planes4,
                                 posmaps, index_out, 0);
}

/* nms_dir 0: NMS along the gradient (the reference); 1: along the corrected
 * normal, the third-order vector (see oracle_nms). */
long toed_oracle_detect_ex(const double *img, int H, int W, double sigma, int r, const double *taps_in,
                           double threshold, int nthreads, double *edges, long capacity, double *planes4,
                           double *posmaps, int64_t *index_out, int nms_dir)
{
    const int n = 2 * r + 3;
    double *taps = (double *)malloc(sizeof(double) * 8 * n);
    if (taps_in)
        memcpy(taps, taps_in, sizeof(double) * 8 * n);
    else
        toed_oracle_taps(sigma, r, taps);
    const int H2 = 2 * H, W2 = 2 * W;
    const size_t P2 = (size_t)H2 * W2;
    double *pl = planes4 ? planes4 : (double *)malloc(sizeof(double) * 4 * P2);
    double *pm = posmaps ? posmaps : (double *)malloc(sizeof(double) * 3 * P2);
    double *tv = nms_dir ? (double *)malloc(sizeof(double) * 2 * P2) : NULL;
    memset(pl, 0, sizeof(double) * 4 * P2);
    oracle_planes(img, H, W, r, taps, nthreads, pl, pl + P2, pl + 2 * P2, pl + 3 * P2, NULL, tv);
    oracle_nms(pl, pl + P2, pl + 2 * P2, tv, H2, W2, threshold, nthreads, pm, pm + P2, pm + 2 * P2);
    free(tv);
    long N = toed_oracle_compact(pm, pm + P2, pl + 3 * P2, pm + 2 * P2, H2, W2, edges, capacity,
                                 index_out);
    if (!planes4) free(pl);
    if (!posmaps) free(pm);
    free(taps);
    return N;
}

/* ------------------------------------------------------------------------ */
/* Subpixel TO correction (subpix_to_correction.cpp), interp_n = 0            */
/* ------------------------------------------------------------------------ */
static inline int wrap_idx(int i, int n)
{ /* :40-45 */
    int r = i % n;
    if (r < 0) r += n;
    return r;
}

static inline int wrap_symmetric(int i, int n)
{ /* :47-55 */
    if (n <= 1) return 0;
    while (i < 0 || i >= n) {
        if (i < 0)
            i = -i - 1;
        else
            i = 2 * n - i - 1;
    }
    return i;
}

static inline double cubic_kernel(double s)
{ /* :57-67, Keys a = -0.5 */
    const double a = -0.5;
    double x = fabs(s);
    if (x <= 1.0) return ((a + 2) * x - (a + 3)) * x * x + 1;
    if (x < 2.0) return ((a * x - 5 * a) * x + 8 * a) * x - 4 * a;
    return 0;
}

static inline double wrap_mod_pi(double a)
{ /* :216-222 */
    double r = fmod(a, M_PI);
    if (r < 0) r += M_PI;
    return r;
}

/* build_gaussian_kernels :195-214.  k3: 3 arrays of 2*rad+1 (G, dG, d2G). */
int subpix_oracle_kernels(double sigma, double *k3)
{
    const int rad = (int)ceil(sigma * 4);
    const int ksz = 2 * rad + 1;
    const double s2 = sigma * sigma, s3 = s2 * sigma, s5 = s2 * s3;
    const double nrm = sqrt(2.0 * M_PI);
    for (int k = -rad; k <= rad; k++) {
        double kk = (double)k;
        double e = exp(-(kk * kk) / (2.0 * s2));
        k3[0 * ksz + k + rad] = e / (nrm * sigma);
        k3[1 * ksz + k + rad] = -kk * e / (nrm * s3);
        k3[2 * ksz + k + rad] = (kk * kk - s2) * e / (nrm * s5);
    }
    return rad;
}

/* estimate_orientation :307-375.  theta out: h*w. */
void subpix_oracle_orientation(const double *E, int h, int w, double *theta)
{
    const int r = 4, ksz = 2 * r + 1;
    double tri[9], tri_sum = 0;
    for (int k = -r; k <= r; k++) {
        tri[k + r] = (double)(r + 1 - abs(k));
        tri_sum += tri[k + r];
    }
    for (int k = 0; k < ksz; k++) tri[k] /= tri_sum;
    const size_t n = (size_t)h * w;
    double *tmp = (double *)malloc(n * sizeof(double));
    double *sm = (double *)malloc(n * sizeof(double));
    double *Ox = (double *)malloc(n * sizeof(double));
    double *Oy = (double *)malloc(n * sizeof(double));
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            double acc = 0;
            for (int q = -r; q <= r; q++) acc += E[(size_t)i * w + wrap_symmetric(j - q, w)] * tri[q + r];
            tmp[(size_t)i * w + j] = acc;
        }
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            double acc = 0;
            for (int p = -r; p <= r; p++) acc += tmp[(size_t)wrap_symmetric(i - p, h) * w + j] * tri[p + r];
            sm[(size_t)i * w + j] = acc;
        }
#define DX(a, i, j)                                                                          \
    ((j) == 0 ? (a)[(size_t)(i) * w + 1] - (a)[(size_t)(i) * w + 0]                          \
              : ((j) == w - 1 ? (a)[(size_t)(i) * w + (w - 1)] - (a)[(size_t)(i) * w + (w - 2)] \
                              : 0.5 * ((a)[(size_t)(i) * w + ((j) + 1)] - (a)[(size_t)(i) * w + ((j) - 1)])))
#define DY(a, i, j)                                                                          \
    ((i) == 0 ? (a)[(size_t)1 * w + (j)] - (a)[(j)]                                          \
              : ((i) == h - 1 ? (a)[(size_t)(h - 1) * w + (j)] - (a)[(size_t)(h - 2) * w + (j)] \
                              : 0.5 * ((a)[(size_t)((i) + 1) * w + (j)] - (a)[(size_t)((i) - 1) * w + (j)])))
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            Ox[(size_t)i * w + j] = DX(sm, i, j);
            Oy[(size_t)i * w + j] = DY(sm, i, j);
        }
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            double Oxx = DX(Ox, i, j);
            double Oxy = DX(Oy, i, j);
            double Oyy = DY(Oy, i, j);
            double sgn = (Oxy < 0) ? 1.0 : ((Oxy > 0) ? -1.0 : 0.0);
            double ang = atan(Oyy * sgn / (Oxx + 1e-5));
            theta[(size_t)i * w + j] = wrap_mod_pi(ang);
        }
#undef DX
#undef DY
    free(tmp);
    free(sm);
    free(Ox);
    free(Oy);
}

/* conv_separable_circular :377-411 */
static void conv_sep_circ(const double *src, double *dst, double *tmp, int h, int w, int rad,
                          const double *kx, const double *ky)
{
#pragma omp parallel
    {
#pragma omp for schedule(static)
        for (int i = 0; i < h; i++)
            for (int j = 0; j < w; j++) {
                double acc = 0;
                for (int q = -rad; q <= rad; q++) acc += src[(size_t)i * w + wrap_idx(j - q, w)] * kx[q + rad];
                tmp[(size_t)i * w + j] = acc;
            }
#pragma omp for schedule(static)
        for (int i = 0; i < h; i++)
            for (int j = 0; j < w; j++) {
                double acc = 0;
                for (int p = -rad; p <= rad; p++) acc += tmp[(size_t)wrap_idx(i - p, h) * w + j] * ky[p + rad];
                dst[(size_t)i * w + j] = acc;
            }
    }
}

/* interp2_cubic :521-556 */
static double interp2_cubic(const double *src, int h, int w, double x, double y)
{
    int x0 = (int)floor(x), y0 = (int)floor(y);
    double fx = x - x0, fy = y - y0;
    double wx[4], wy[4];
    wx[0] = cubic_kernel(fx + 1);
    wx[1] = cubic_kernel(fx);
    wx[2] = cubic_kernel(fx - 1);
    wx[3] = cubic_kernel(fx - 2);
    wy[0] = cubic_kernel(fy + 1);
    wy[1] = cubic_kernel(fy);
    wy[2] = cubic_kernel(fy - 1);
    wy[3] = cubic_kernel(fy - 2);
    double acc = 0;
    for (int p = 0; p < 4; p++) {
        double row = 0;
        int ii = y0 - 1 + p;
        ii = (ii < 0) ? 0 : (ii >= h ? h - 1 : ii);
        for (int q = 0; q < 4; q++) {
            int jj = x0 - 1 + q;
            jj = (jj < 0) ? 0 : (jj >= w ? w - 1 : jj);
            row += src[(size_t)ii * w + jj] * wx[q];
        }
        acc += row * wy[p];
    }
    return acc;
}

/* bilinear_resize :69-90 -- corner-aligned resize to the 2^n work grid */
static void bilinear_resize(const double *src, int sh, int sw, double *dst, int dh, int dw)
{
    for (int i = 0; i < dh; i++) {
        const double y = (dh == 1) ? 0 : (double)i * (sh - 1) / (double)(dh - 1);
        const int y0 = (int)floor(y);
        const int y1 = (y0 + 1 < sh - 1) ? y0 + 1 : sh - 1;
        const double fy = y - y0;
        for (int j = 0; j < dw; j++) {
            const double x = (dw == 1) ? 0 : (double)j * (sw - 1) / (double)(dw - 1);
            const int x0 = (int)floor(x);
            const int x1 = (x0 + 1 < sw - 1) ? x0 + 1 : sw - 1;
            const double fx = x - x0;
            const double v00 = src[(size_t)y0 * sw + x0], v01 = src[(size_t)y0 * sw + x1];
            const double v10 = src[(size_t)y1 * sw + x0], v11 = src[(size_t)y1 * sw + x1];
            dst[(size_t)i * dw + j] = (1 - fy) * ((1 - fx) * v00 + fx * v01) + fy * ((1 - fx) * v10 + fx * v11);
        }
    }
}

/*
 * Whole TO-correction pipeline (run :623-736 after set_edgemap / optional
 * set_orientation or estimate_orientation).
 *   E: h*w edge map.  theta_in: optional h*w orientation (radians); NULL ->
 *   estimate_orientation.  edges: capacity*4 out (x, y, ori, strength).
 *   TO_E / TO_O: optional dense h*w outputs.  nms_out: optional 4 planes
 *   (nms_x, nms_y, nms_mag, valid) for plane-level tests; theta_out: optional.
 * Returns N after isolated-edgel removal.
 */
long subpix_oracle_run_n(const double *E_in, int h0, int w0, int interp_n, double thresh, double sigma,
                         double nbr_radius, const double *theta_in0, int nthreads, double *edges,
                         long capacity, double *TO_E, double *TO_O, double *nms_out,
                         double *theta_out, double *planes10)
{
    if (nthreads > 0) omp_set_num_threads(nthreads);
    /* interp_n > 0: the work grid is (h0-1) 2^n + 1 by (w0-1) 2^n + 1, the
     * map (and a given orientation) bilinearly resized onto it
     * (set_edgemap / set_orientation :224-244), the NMS margin 3 * 2^n
     * (:628-630), positions divided by 2^n (:657, :696-697) and the dense
     * maps kept at the original size (:707-715). */
    const int sc = 1 << (interp_n > 0 ? interp_n : 0);
    const int h = (h0 - 1) * sc + 1, w = (w0 - 1) * sc + 1;
    const size_t n = (size_t)h * w, n0 = (size_t)h0 * w0;
    double *E_work = NULL, *th_work = NULL;
    const double *E = E_in, *theta_in = theta_in0;
    if (sc > 1) {
        E_work = (double *)malloc(n * sizeof(double));
        bilinear_resize(E_in, h0, w0, E_work, h, w);
        E = E_work;
        if (theta_in0) {
            th_work = (double *)malloc(n * sizeof(double));
            bilinear_resize(theta_in0, h0, w0, th_work, h, w);
            theta_in = th_work;
        }
    }
    const int rad = (int)ceil(sigma * 4);
    const int ksz = 2 * rad + 1;
    double *k3 = (double *)malloc(sizeof(double) * 3 * ksz);
    subpix_oracle_kernels(sigma, k3);
    const double *G = k3, *dG = k3 + ksz, *d2G = k3 + 2 * ksz;

    double *theta = (double *)malloc(n * sizeof(double));
    if (theta_in)
        memcpy(theta, theta_in, n * sizeof(double));
    else
        subpix_oracle_orientation(E, h, w, theta);
    if (theta_out) memcpy(theta_out, theta, n * sizeof(double));

    double *dirx = (double *)malloc(n * sizeof(double));
    double *diry = (double *)malloc(n * sizeof(double));
    for (size_t k = 0; k < n; k++) { /* compute_dir_from_theta :296-305 */
        double a = wrap_mod_pi(theta[k]);
        dirx[k] = cos(a);
        diry[k] = sin(a);
    }

    /* nms_token(margin = 3 * 2^n) :413-519 */
    const int margin = 3 * sc;
    double *nx_ = (double *)calloc(n, sizeof(double));
    double *ny_ = (double *)calloc(n, sizeof(double));
    double *nm_ = (double *)calloc(n, sizeof(double));
    unsigned char *nv_ = (unsigned char *)calloc(n, 1);
    const int j0 = margin + 1, j1 = w - (margin + 2), i0 = margin + 1, i1 = h - (margin + 2);
#pragma omp parallel for schedule(dynamic)
    for (int j = j0; j < j1; j++) {
        for (int i = i0; i < i1; i++) {
            const size_t o = (size_t)i * w + j;
            if (E[o] <= thresh) continue;
            const double gx = dirx[o], gy = diry[o];
            if (fabs(gx) < 1e-5 && fabs(gy) < 1e-5) continue;
            const double mag_dir = sqrt(gx * gx + gy * gy);
            const double nx = gx / mag_dir, ny = gy / mag_dir;
            const double f = E[o];
            double slope, fp, fm;
            nms_sector(E, w, i, j, gx, gy, nx, ny, &slope, &fp, &fm);
            if (!((f > fm && f > fp) || (f > fm && f >= fp) || (f >= fm && f > fp))) continue;
            const double s = sqrt(1 + slope * slope);
            const double A = (fm + fp - 2 * f) / (2 * s * s);
            const double B = (fp - fm) / (2 * s);
            const double C = f;
            if (fabs(A) < 1e-16) continue;
            const double s_star = -B / (2 * A);
            const double max_f = A * s_star * s_star + B * s_star + C;
            if (fabs(s_star) <= sqrt(2.0)) {
                nx_[o] = (double)j + s_star * nx;
                ny_[o] = (double)i + s_star * ny;
                nm_[o] = fabs(max_f);
                nv_[o] = 1;
            }
        }
    }
    if (nms_out) {
        memcpy(nms_out, nx_, n * sizeof(double));
        memcpy(nms_out + n, ny_, n * sizeof(double));
        memcpy(nms_out + 2 * n, nm_, n * sizeof(double));
        for (size_t k = 0; k < n; k++) nms_out[3 * n + k] = nv_[k];
    }

    /* Hx, Hy and the 8 circular separable convolutions :634-648 */
    double *Hx = (double *)malloc(n * sizeof(double));
    double *Hy = (double *)malloc(n * sizeof(double));
    for (size_t k = 0; k < n; k++) {
        Hx[k] = E[k] * dirx[k];
        Hy[k] = E[k] * diry[k];
    }
    double *tmp = (double *)malloc(n * sizeof(double));
    double *P = (double *)malloc(8 * n * sizeof(double));
    double *Px = P, *Py = P + n, *Pxx = P + 2 * n, *Pxy = P + 3 * n, *Pyy = P + 4 * n,
           *Hxx = P + 5 * n, *Hyy = P + 6 * n, *Hxy = P + 7 * n;
    conv_sep_circ(E, Px, tmp, h, w, rad, dG, G);
    conv_sep_circ(E, Py, tmp, h, w, rad, G, dG);
    conv_sep_circ(E, Pxx, tmp, h, w, rad, d2G, G);
    conv_sep_circ(E, Pxy, tmp, h, w, rad, dG, dG);
    conv_sep_circ(E, Pyy, tmp, h, w, rad, G, d2G);
    conv_sep_circ(Hx, Hxx, tmp, h, w, rad, dG, G);
    conv_sep_circ(Hy, Hyy, tmp, h, w, rad, G, dG);
    conv_sep_circ(Hy, Hxy, tmp, h, w, rad, dG, G);
    if (planes10) {
        /* order: Px Py Pxx Pxy Pyy Hxx Hyy Hxy Hx Hy */
        memcpy(planes10, P, 8 * n * sizeof(double));
        memcpy(planes10 + 8 * n, Hx, n * sizeof(double));
        memcpy(planes10 + 9 * n, Hy, n * sizeof(double));
    }

    /* per-edgel correction :663-700 (serial, row-major) */
    long cnt = 0;
    for (size_t k = 0; k < n; k++) cnt += nv_[k];
    double *L = (double *)malloc(sizeof(double) * 4 * (cnt > 0 ? cnt : 1));
    long m = 0;
    for (int i = 0; i < h; i++) {
        for (int j = 0; j < w; j++) {
            const size_t o = (size_t)i * w + j;
            if (!nv_[o]) continue;
            const double sx = nx_[o], sy = ny_[o], mag_e = nm_[o];
            double Px_e = interp2_cubic(Px, h, w, sx, sy);
            double Py_e = interp2_cubic(Py, h, w, sx, sy);
            double Pxx_e = interp2_cubic(Pxx, h, w, sx, sy);
            double Pyy_e = interp2_cubic(Pyy, h, w, sx, sy);
            double Pxy_e = interp2_cubic(Pxy, h, w, sx, sy);
            double Hx_e = interp2_cubic(Hx, h, w, sx, sy);
            double Hxx_e = interp2_cubic(Hxx, h, w, sx, sy);
            double Hxy_e = interp2_cubic(Hxy, h, w, sx, sy);
            double Hyy_e = interp2_cubic(Hyy, h, w, sx, sy);
            double Hy_e = interp2_cubic(Hy, h, w, sx, sy);
            double Fx = Px_e * Hxx_e + Pxx_e * Hx_e + Py_e * Hxy_e + Pxy_e * Hy_e;
            double Fy = Px_e * Hxy_e + Pxy_e * Hx_e + Py_e * Hyy_e + Pyy_e * Hy_e;
            double Fm = sqrt(Fx * Fx + Fy * Fy);
            double ori;
            if (Fm < 1e-12) {
                ori = atan2(dirx[o], -diry[o]);
            } else {
                Fx /= Fm;
                Fy /= Fm;
                ori = atan2(Fx, -Fy);
            }
            L[4 * m + 0] = sx / (double)sc; /* coord_scale :696-697 */
            L[4 * m + 1] = sy / (double)sc;
            L[4 * m + 2] = ori;
            L[4 * m + 3] = mag_e;
            m++;
        }
    }

    /* remove_isolated_edgels :563-621 -- cell grid of size radius, 3x3 cells */
    long kept = m;
    if (nbr_radius > 0 && m >= 2) {
        const double r2 = nbr_radius * nbr_radius;
        const double inv = 1 / nbr_radius;
        int *cx = (int *)malloc(sizeof(int) * m), *cy = (int *)malloc(sizeof(int) * m);
        int minx = 0, miny = 0, maxx = 0, maxy = 0;
        for (long k = 0; k < m; k++) {
            cx[k] = (int)floor(L[4 * k + 0] * inv);
            cy[k] = (int)floor(L[4 * k + 1] * inv);
            if (k == 0 || cx[k] < minx) minx = cx[k];
            if (k == 0 || cy[k] < miny) miny = cy[k];
            if (k == 0 || cx[k] > maxx) maxx = cx[k];
            if (k == 0 || cy[k] > maxy) maxy = cy[k];
        }
        /* bucket the edgels by cell (counting sort, stable) */
        const long gw = (long)(maxx - minx + 1), gh = (long)(maxy - miny + 1);
        long *start = (long *)calloc((size_t)(gw * gh + 1), sizeof(long));
        long *items = (long *)malloc(sizeof(long) * m);
        for (long k = 0; k < m; k++) start[(cy[k] - miny) * gw + (cx[k] - minx) + 1]++;
        for (long c = 0; c < gw * gh; c++) start[c + 1] += start[c];
        long *fill = (long *)malloc(sizeof(long) * (size_t)(gw * gh));
        memcpy(fill, start, sizeof(long) * (size_t)(gw * gh));
        for (long k = 0; k < m; k++) items[fill[(cy[k] - miny) * gw + (cx[k] - minx)]++] = k;
        unsigned char *keep = (unsigned char *)calloc((size_t)m, 1);
        for (long k = 0; k < m; k++) {
            int found = 0;
            for (int dy = -1; dy <= 1 && !found; dy++) {
                for (int dx = -1; dx <= 1 && !found; dx++) {
                    long gx = cx[k] + dx - minx, gy = cy[k] + dy - miny;
                    if (gx < 0 || gy < 0 || gx >= gw || gy >= gh) continue;
                    long c = gy * gw + gx;
                    for (long t = start[c]; t < start[c + 1]; t++) {
                        long q = items[t];
                        if (q == k) continue;
                        double ddx = L[4 * k + 0] - L[4 * q + 0];
                        double ddy = L[4 * k + 1] - L[4 * q + 1];
                        if (ddx * ddx + ddy * ddy <= r2) {
                            found = 1;
                            break;
                        }
                    }
                }
            }
            keep[k] = (unsigned char)found;
        }
        long wpos = 0;
        for (long k = 0; k < m; k++) {
            if (keep[k]) {
                if (wpos != k) memcpy(&L[4 * wpos], &L[4 * k], 4 * sizeof(double));
                wpos++;
            }
        }
        kept = wpos;
        free(cx);
        free(cy);
        free(start);
        free(items);
        free(fill);
        free(keep);
    }

    /* dense TO maps :708-715 (later edgels overwrite earlier ones) */
    if (TO_E) memset(TO_E, 0, n0 * sizeof(double));
    if (TO_O) memset(TO_O, 0, n0 * sizeof(double));
    for (long k = 0; k < kept; k++) {
        int X = (int)round(L[4 * k + 0]);
        int Y = (int)round(L[4 * k + 1]);
        X = X < 0 ? 0 : (X > w0 - 1 ? w0 - 1 : X);
        Y = Y < 0 ? 0 : (Y > h0 - 1 ? h0 - 1 : Y);
        if (TO_E) TO_E[(size_t)Y * w0 + X] = L[4 * k + 3];
        if (TO_O) TO_O[(size_t)Y * w0 + X] = L[4 * k + 2];
    }
    for (long k = 0; k < kept && k < capacity; k++) memcpy(&edges[4 * k], &L[4 * k], 4 * sizeof(double));

    free(k3);
    free(theta);
    free(dirx);
    free(diry);
    free(nx_);
    free(ny_);
    free(nm_);
    free(nv_);
    free(Hx);
    free(Hy);
    free(tmp);
    free(P);
    free(L);
    free(E_work);
    free(th_work);
    return kept;
}

long subpix_oracle_run(const double *E, int h, int w, double thresh, double sigma,
                       double nbr_radius, const double *theta_in, int nthreads, double *edges,
                       long capacity, double *TO_E, double *TO_O, double *nms_out,
                       double *theta_out, double *planes10)
{
    return subpix_oracle_run_n(E, h, w, 0, thresh, sigma, nbr_radius, theta_in, nthreads, edges, capacity,
                               TO_E, TO_O, nms_out, theta_out, planes10);
}


/* ------------------------------------------------------------------------ */
/* TOED, MATLAB "quick and dirty" orientation mode                           */
/* ------------------------------------------------------------------------ */
/*
 * third_order_edge_detector.m:91-141 with QaD_flag set: the nine derivatives
 * are interpolated with MATLAB's interp2 'cubic' (cubic convolution, Keys
 * a = -1/2, the same kernel the reference restates as cubic_kernel /
 * interp2_cubic, subpix_to_correction.cpp:57-67, :521-556) at each edgel's
 * subpixel point, and the orientation is atan2(Fx, -Fy) of the third-order
 * vector built from them (:127-141) instead of the vector at the grid point
 * (cpu_toed.cpp:227-232).  Here the derivatives are the C++ detector's own
 * (the 2x grid of cpu_toed.cpp:204-344, zero padding) and the subpixel
 * point is its NMS position in 2x-grid units (cpu_toed.cpp:488-489);
 * positions and strengths are those of the grid mode.  Same arguments as
 * toed_oracle_detect without the plane outputs; index_out is required.
 */
long toed_oracle_detect_qad(const double *img, int H, int W, double sigma, int r,
                            const double *taps_in, double threshold, int nthreads, double *edges,
                            long capacity, int64_t *index_out)
{
    const int n = 2 * r + 3;
    double *taps = (double *)malloc(sizeof(double) * 8 * n);
    if (taps_in)
        memcpy(taps, taps_in, sizeof(double) * 8 * n);
    else
        toed_oracle_taps(sigma, r, taps);
    const int H2 = 2 * H, W2 = 2 * W;
    const size_t P2 = (size_t)H2 * W2;
    double *pm = (double *)malloc(sizeof(double) * 3 * P2);
    double *d9 = (double *)malloc(sizeof(double) * 9 * P2);
    const long N = toed_oracle_detect(img, H, W, sigma, r, taps, threshold, nthreads, edges, capacity,
                                      NULL, pm, index_out);
    toed_oracle_planes(img, H, W, r, taps, nthreads, NULL, NULL, NULL, NULL, d9);
    const long m = N < capacity ? N : capacity;
#pragma omp parallel for schedule(static)
    for (long e = 0; e < m; e++) {
        const size_t o = (size_t)index_out[e];
        const double px = pm[o], py = pm[P2 + o];
        double d[9];
        for (int k = 0; k < 9; k++) d[k] = interp2_cubic(d9 + (size_t)k * P2, H2, W2, px, py);
        to_orientation(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8], &edges[4 * e + 2]);
    }
    free(d9);
    free(pm);
    free(taps);
    return N;
}
