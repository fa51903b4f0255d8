/*
 * dc_oracle.c -- CPU oracle for the Fletcher TTI propagation path.
 *
 * TEST INFRASTRUCTURE ONLY (see dc_oracle.h).  A restatement of the
 * reference algorithm in our own C; nothing in the product library uses it.
 *
 * Build without FMA contraction (-ffp-contract=off) so that the float path
 * reproduces the reference's OpenMP results bit for bit on x86-64 and on
 * aarch64 alike.
 */
#include "dc_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- finite-difference coefficients ----------------------------------
 * 8th-order central differences, include/derivatives.h:15-38.  Written as
 * the exact rationals; rounded to float they equal the reference literals.
 *   first derivative   L1..L4 = 4/5, -1/5, 4/105, -1/280
 *   cross terms        L_ab   = L_a * L_b (rounded once from the exact value)
 *   second derivative  K0..K4 = -205/72, 8/5, -1/5, 8/315, -1/560          */
static const double kK_d[5] = {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0,
                               8.0 / 315.0, -1.0 / 560.0};
static const double kL_d[5] = {0.0, 4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0,
                               -1.0 / 280.0};
/* The ten (a,b) index pairs of the cross operator, in the order in which
 * include/derivatives.h:58-89 sums them: L11 L12 L13 L14 L22 L23 L24 L33 L34
 * L44. */
static const int kPairs[10][2] = {{1, 1}, {1, 2}, {1, 3}, {1, 4}, {2, 2},
                                  {2, 3}, {2, 4}, {3, 3}, {3, 4}, {4, 4}};

static float kK_f[5], kLab_f[10];
static double kLab_d[10];
static int coef_ready = 0;

static void init_coefs(void) {
  if (coef_ready) return;
  for (int k = 0; k < 5; ++k) kK_f[k] = (float)kK_d[k];
  for (int g = 0; g < 10; ++g) {
    /* exact rational product, rounded once */
    double v = kL_d[kPairs[g][0]] * kL_d[kPairs[g][1]];
    kLab_d[g] = v;
    kLab_f[g] = (float)v;
  }
  coef_ready = 1;
}

/* ---- type-generic stencil ------------------------------------------------
 * The body below is instantiated for float (T=float) and double (T=double).
 * Operation order follows include/derivatives.h:47-91 and
 * include/sample_compute.h:106-185 exactly: C evaluates + and - left to
 * right, so each accumulation below is the reference's expression tree.   */

#define O_DEFINE_STENCIL(T, SUF, KK, LAB)                                      \
  static inline T der2_##SUF(const T *p, long i, long s, T d2inv) {            \
    /* include/derivatives.h:47-54 */                                          \
    T acc = KK[0] * p[i];                                                      \
    acc = acc + KK[1] * (p[i + s] + p[i - s]);                                 \
    acc = acc + KK[2] * (p[i + 2 * s] + p[i - 2 * s]);                         \
    acc = acc + KK[3] * (p[i + 3 * s] + p[i - 3 * s]);                         \
    acc = acc + KK[4] * (p[i + 4 * s] + p[i - 4 * s]);                         \
    return acc * d2inv;                                                        \
  }                                                                            \
  static inline T cross_##SUF(const T *p, long i, long s1, long s2, T dinv) {  \
    /* include/derivatives.h:56-91: group (a,b) sums the quad with offsets   \
     * (a*s2, b*s1) and, for a != b, the mirrored quad (b*s2, a*s1), each   \
     * quad ordered (+,+) - (+,-) - (-,+) + (-,-). */                          \
    T total = 0;                                                               \
    for (int g = 0; g < 10; ++g) {                                             \
      const long a = kPairs[g][0], b = kPairs[g][1];                           \
      T acc = p[i + a * s2 + b * s1];                                          \
      acc = acc - p[i + a * s2 - b * s1];                                      \
      acc = acc - p[i - a * s2 + b * s1];                                      \
      acc = acc + p[i - a * s2 - b * s1];                                      \
      if (a != b) {                                                            \
        acc = acc + p[i + b * s2 + a * s1];                                    \
        acc = acc - p[i + b * s2 - a * s1];                                    \
        acc = acc - p[i - b * s2 + a * s1];                                    \
        acc = acc + p[i - b * s2 - a * s1];                                    \
      }                                                                        \
      const T term = LAB[g] * acc;                                             \
      total = (g == 0) ? term : total + term;                                  \
    }                                                                          \
    return total * dinv;                                                       \
  }

O_DEFINE_STENCIL(float, f, kK_f, kLab_f)
O_DEFINE_STENCIL(double, d, kK_d, kLab_d)

/* Per-point coefficients of the TTI operator. */
typedef struct {
  float cxx, cyy, czz, cxy, cyz, cxz, v2px, v2pz, v2sz, v2pn;
} o_pointcoef;

/* Constant-angle factors of include/sample_compute.h:9-18 (the reference
 * CUDA path): theta = pi/4, phi = 1 rad, eps = 0.24, delta = 0.10. */
static const float kRefCudaCh[6] = {0.1459632909f, 0.3540367091f, 0.5f,
                                    0.4546487134f, 0.8414709848f,
                                    0.5403023059f};
static const float kRefCudaV2px = 1.48f, kRefCudaV2pn = 1.2f;

/* The p/q update at one point, include/sample_compute.h:106-185
 * (sample_compute), float.  g is the sponge factor (1 in the interior, where
 * the update reduces exactly to the reference's). */
static inline void point_f32(long i, long sX, long sY, long sZ,
                             const float inv[6], float dt, const float *pc,
                             const float *qc, float *pp, float *qp,
                             const o_pointcoef *c, float g) {
  const float dxxinv = inv[0], dyyinv = inv[1], dzzinv = inv[2];
  const float dxyinv = inv[3], dxzinv = inv[4], dyzinv = inv[5];
  const float pxx = der2_f(pc, i, sX, dxxinv);
  const float pyy = der2_f(pc, i, sY, dyyinv);
  const float pzz = der2_f(pc, i, sZ, dzzinv);
  const float pxy = cross_f(pc, i, sX, sY, dxyinv);
  const float pyz = cross_f(pc, i, sY, sZ, dyzinv);
  const float pxz = cross_f(pc, i, sX, sZ, dxzinv);
  const float h1p = c->cxx * pxx + c->cyy * pyy + c->czz * pzz +
                    c->cxy * pxy + c->cxz * pxz + c->cyz * pyz;
  const float h2p = pxx + pyy + pzz - h1p;

  const float qxx = der2_f(qc, i, sX, dxxinv);
  const float qyy = der2_f(qc, i, sY, dyyinv);
  const float qzz = der2_f(qc, i, sZ, dzzinv);
  const float qxy = cross_f(qc, i, sX, sY, dxyinv);
  const float qyz = cross_f(qc, i, sY, sZ, dyzinv);
  const float qxz = cross_f(qc, i, sX, sZ, dxzinv);
  const float h1q = c->cxx * qxx + c->cyy * qyy + c->czz * qzz +
                    c->cxy * qxy + c->cxz * qxz + c->cyz * qyz;
  const float h2q = qxx + qyy + qzz - h1q;

  const float h1pmq = h1p - h1q;
  const float h2pmq = h2p - h2q;
  const float rhsp = c->v2px * h2p + c->v2pz * h1q + c->v2sz * h1pmq;
  const float rhsq = c->v2pn * h2p + c->v2pz * h1q - c->v2sz * h2pmq;
  if (g == 1.0f) {
    pp[i] = 2.0f * pc[i] - pp[i] + rhsp * dt * dt;
    qp[i] = 2.0f * qc[i] - qp[i] + rhsq * dt * dt;
  } else {
    /* damped leapfrog: both time levels scaled by g */
    pp[i] = (2.0f * pc[i] - g * pp[i] + rhsp * dt * dt) * g;
    qp[i] = (2.0f * qc[i] - g * qp[i] + rhsq * dt * dt) * g;
  }
}

/* Same update in double precision (FP64 oracle). */
static inline void point_f64(long i, long sX, long sY, long sZ,
                             const double inv[6], double dt,
                             const double *pc, const double *qc, double *pp,
                             double *qp, const o_pointcoef *c, double g) {
  const double pxx = der2_d(pc, i, sX, inv[0]);
  const double pyy = der2_d(pc, i, sY, inv[1]);
  const double pzz = der2_d(pc, i, sZ, inv[2]);
  const double pxy = cross_d(pc, i, sX, sY, inv[3]);
  const double pyz = cross_d(pc, i, sY, sZ, inv[5]);
  const double pxz = cross_d(pc, i, sX, sZ, inv[4]);
  const double h1p = (double)c->cxx * pxx + (double)c->cyy * pyy +
                     (double)c->czz * pzz + (double)c->cxy * pxy +
                     (double)c->cxz * pxz + (double)c->cyz * pyz;
  const double h2p = pxx + pyy + pzz - h1p;
  const double qxx = der2_d(qc, i, sX, inv[0]);
  const double qyy = der2_d(qc, i, sY, inv[1]);
  const double qzz = der2_d(qc, i, sZ, inv[2]);
  const double qxy = cross_d(qc, i, sX, sY, inv[3]);
  const double qyz = cross_d(qc, i, sY, sZ, inv[5]);
  const double qxz = cross_d(qc, i, sX, sZ, inv[4]);
  const double h1q = (double)c->cxx * qxx + (double)c->cyy * qyy +
                     (double)c->czz * qzz + (double)c->cxy * qxy +
                     (double)c->cxz * qxz + (double)c->cyz * qyz;
  const double h2q = qxx + qyy + qzz - h1q;
  const double h1pmq = h1p - h1q, h2pmq = h2p - h2q;
  const double rhsp =
      (double)c->v2px * h2p + (double)c->v2pz * h1q + (double)c->v2sz * h1pmq;
  const double rhsq =
      (double)c->v2pn * h2p + (double)c->v2pz * h1q - (double)c->v2sz * h2pmq;
  pp[i] = (2.0 * pc[i] - g * pp[i] + rhsp * dt * dt) * g;
  qp[i] = (2.0 * qc[i] - g * qp[i] + rhsq * dt * dt) * g;
}

static inline void load_coef(int kind, long i, const float *const coef[O_NCOEF],
                             const float *vpz, const float *vsv,
                             o_pointcoef *c) {
  if (kind == O_KIND_F32_REFCUDA) {
    /* include/sample_compute.h:51-54: v2* derived from vpz/vsv */
    const float v2pz = vpz[i] * vpz[i];
    c->cxx = kRefCudaCh[0];
    c->cyy = kRefCudaCh[1];
    c->czz = kRefCudaCh[2];
    c->cxy = kRefCudaCh[3];
    c->cyz = kRefCudaCh[4];
    c->cxz = kRefCudaCh[5];
    c->v2pz = v2pz;
    c->v2sz = vsv[i] * vsv[i];
    c->v2px = v2pz * kRefCudaV2px;
    c->v2pn = v2pz * kRefCudaV2pn;
  } else {
    c->cxx = coef[O_CH1DXX][i];
    c->cyy = coef[O_CH1DYY][i];
    c->czz = coef[O_CH1DZZ][i];
    c->cxy = coef[O_CH1DXY][i];
    c->cyz = coef[O_CH1DYZ][i];
    c->cxz = coef[O_CH1DXZ][i];
    c->v2px = coef[O_V2PX][i];
    c->v2pz = coef[O_V2PZ][i];
    c->v2sz = coef[O_V2SZ][i];
    c->v2pn = coef[O_V2PN][i];
  }
}

int o_step(int kind, long sx, long sy, long sz, const long b0[3],
           const long b1[3], float dx, float dy, float dz, float dt,
           const void *pc_, const void *qc_, void *pp_, void *qp_,
           const float *const coef[O_NCOEF], const float *vpz,
           const float *vsv, const float *const sponge[3], int nthreads) {
  init_coefs();
  const long lo[3] = {4, 4, 4}, hi[3] = {sx - 4, sy - 4, sz - 4};
  for (int d = 0; d < 3; ++d) {
    if (b1[d] <= b0[d]) return 0; /* empty box: nothing to do */
    if (b0[d] < lo[d] || b1[d] > hi[d]) return -1;
  }
  const long sX = 1, sY = sx, sZ = sx * sy;
  /* include/sample_compute.h:128-133 */
  const float finv[6] = {1.0f / (dx * dx), 1.0f / (dy * dy), 1.0f / (dz * dz),
                         1.0f / (dx * dy), 1.0f / (dx * dz), 1.0f / (dy * dz)};
  const double dinv[6] = {1.0 / ((double)dx * dx), 1.0 / ((double)dy * dy),
                          1.0 / ((double)dz * dz), 1.0 / ((double)dx * dy),
                          1.0 / ((double)dx * dz), 1.0 / ((double)dy * dz)};
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long z = b0[2]; z < b1[2]; ++z) {
    for (long y = b0[1]; y < b1[1]; ++y) {
      for (long x = b0[0]; x < b1[0]; ++x) {
        const long i = x + y * sY + z * sZ;
        o_pointcoef c;
        load_coef(kind, i, coef, vpz, vsv, &c);
        float g = 1.0f;
        if (sponge && sponge[0]) g = sponge[0][x] * sponge[1][y] * sponge[2][z];
        if (kind == O_KIND_F64) {
          point_f64(i, sX, sY, sZ, dinv, (double)dt, (const double *)pc_,
                    (const double *)qc_, (double *)pp_, (double *)qp_, &c,
                    (double)g);
        } else {
          point_f32(i, sX, sY, sZ, finv, dt, (const float *)pc_,
                    (const float *)qc_, (float *)pp_, (float *)qp_, &c, g);
        }
      }
    }
  }
  return 0;
}

/* ---- FP64 step, separable cross derivatives ------------------------------
 * The same update as point_f64 (sample_compute, include/sample_compute.h:
 * 106-185, in double), with each cross derivative evaluated as two first
 * derivatives: include/derivatives.h:56-91 sums L_a * L_b over the quads
 * (+-a s2, +-b s1), and L_ab = L_a * L_b (:22-31 are products of :16-19),
 * so derCross(p, s1, s2) = D_s2(D_s1 p) with D(f)(i) = sum_k L_k (f(i+k s) -
 * f(i-k s)).  In double precision the two forms agree to rounding (~1e-16);
 * this one costs ~5x fewer operations, which makes FP64 runs of a few
 * 10^7 points over 10^3 steps practical.  `work` holds 4 n doubles: the x-
 * and y-derivatives of pc and qc. */
static void first_derivs(long sx, long sy, long sz, const double *restrict f,
                         double *restrict fx, double *restrict fy, int nthreads) {
  const long sY = sx, sZ = sx * sy;
  const double L1 = kL_d[1], L2 = kL_d[2], L3 = kL_d[3], L4 = kL_d[4];
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long z = 0; z < sz; ++z)
    for (long y = 4; y < sy - 4; ++y) {
      const long r = y * sY + z * sZ;
      for (long x = 0; x < sx; ++x) {
        const long i = r + x;
        fy[i] = L1 * (f[i + sY] - f[i - sY]) + L2 * (f[i + 2 * sY] - f[i - 2 * sY]) +
                L3 * (f[i + 3 * sY] - f[i - 3 * sY]) + L4 * (f[i + 4 * sY] - f[i - 4 * sY]);
      }
      for (long x = 4; x < sx - 4; ++x) {
        const long i = r + x;
        fx[i] = L1 * (f[i + 1] - f[i - 1]) + L2 * (f[i + 2] - f[i - 2]) +
                L3 * (f[i + 3] - f[i - 3]) + L4 * (f[i + 4] - f[i - 4]);
      }
    }
}

static inline double d1_at(const double *f, long i, long s) {
  return kL_d[1] * (f[i + s] - f[i - s]) + kL_d[2] * (f[i + 2 * s] - f[i - 2 * s]) +
         kL_d[3] * (f[i + 3 * s] - f[i - 3 * s]) + kL_d[4] * (f[i + 4 * s] - f[i - 4 * s]);
}

static inline double d2_at(const double *f, long i, long s) {
  return kK_d[0] * f[i] + kK_d[1] * (f[i + s] + f[i - s]) +
         kK_d[2] * (f[i + 2 * s] + f[i - 2 * s]) + kK_d[3] * (f[i + 3 * s] + f[i - 3 * s]) +
         kK_d[4] * (f[i + 4 * s] + f[i - 4 * s]);
}

/* One row of o_step_f64_sep: points x in [4, sx-4) of the row starting at
 * `r` (every pointer is the array base; restrict lets the compiler
 * vectorise along x). */
typedef struct {
  const float *c[O_NCOEF];
  double inv[6], dt2;
  long sY, sZ;
} sep_row_args;

static void sep_row(const sep_row_args *a, long r, long x0, long x1,
                    const double *restrict pc, const double *restrict qc,
                    double *restrict pp, double *restrict qp,
                    const double *restrict px, const double *restrict py,
                    const double *restrict qx, const double *restrict qy,
                    const float *restrict gx, float gy, float gz) {
  const long sY = a->sY, sZ = a->sZ;
  const double ixx = a->inv[0], iyy = a->inv[1], izz = a->inv[2], ixy = a->inv[3],
               ixz = a->inv[4], iyz = a->inv[5], dt2 = a->dt2;
  const float *restrict c_xx = a->c[O_CH1DXX], *restrict c_yy = a->c[O_CH1DYY],
              *restrict c_zz = a->c[O_CH1DZZ], *restrict c_xy = a->c[O_CH1DXY],
              *restrict c_yz = a->c[O_CH1DYZ], *restrict c_xz = a->c[O_CH1DXZ],
              *restrict c_px = a->c[O_V2PX], *restrict c_pz = a->c[O_V2PZ],
              *restrict c_sz = a->c[O_V2SZ], *restrict c_pn = a->c[O_V2PN];
  for (long x = x0; x < x1; ++x) {
    const long i = r + x;
    const double pxx = d2_at(pc, i, 1) * ixx, pyy = d2_at(pc, i, sY) * iyy,
                 pzz = d2_at(pc, i, sZ) * izz;
    const double pxy = d1_at(py, i, 1) * ixy, pyz = d1_at(py, i, sZ) * iyz,
                 pxz = d1_at(px, i, sZ) * ixz;
    const double qxx = d2_at(qc, i, 1) * ixx, qyy = d2_at(qc, i, sY) * iyy,
                 qzz = d2_at(qc, i, sZ) * izz;
    const double qxy = d1_at(qy, i, 1) * ixy, qyz = d1_at(qy, i, sZ) * iyz,
                 qxz = d1_at(qx, i, sZ) * ixz;
    const double cxx = c_xx[i], cyy = c_yy[i], czz = c_zz[i], cxy = c_xy[i],
                 cyz = c_yz[i], cxz = c_xz[i];
    const double h1p = cxx * pxx + cyy * pyy + czz * pzz + cxy * pxy + cxz * pxz + cyz * pyz;
    const double h2p = pxx + pyy + pzz - h1p;
    const double h1q = cxx * qxx + cyy * qyy + czz * qzz + cxy * qxy + cxz * qxz + cyz * qyz;
    const double h2q = qxx + qyy + qzz - h1q;
    const double v2px = c_px[i], v2pz = c_pz[i], v2sz = c_sz[i], v2pn = c_pn[i];
    const double rhsp = v2px * h2p + v2pz * h1q + v2sz * (h1p - h1q);
    const double rhsq = v2pn * h2p + v2pz * h1q - v2sz * (h2p - h2q);
    const double g = (double)(gx[x] * gy * gz); /* (gx * gy) * gz in float, as o_step */
    pp[i] = (2.0 * pc[i] - g * pp[i] + rhsp * dt2) * g;
    qp[i] = (2.0 * qc[i] - g * qp[i] + rhsq * dt2) * g;
  }
}

int o_step_f64_sep(long sx, long sy, long sz, float dx, float dy, float dz, float dt,
                   const double *pc, const double *qc, double *pp, double *qp,
                   const float *const coef[O_NCOEF], const float *const sponge[3],
                   double *work, int nthreads) {
  init_coefs();
  if (sx < 9 || sy < 9 || sz < 9) return -1;
  if (nthreads < 1) nthreads = 1;
  const long n = sx * sy * sz;
  double *pxd = work, *pyd = work + n, *qxd = work + 2 * n, *qyd = work + 3 * n;
  first_derivs(sx, sy, sz, pc, pxd, pyd, nthreads);
  first_derivs(sx, sy, sz, qc, qxd, qyd, nthreads);
  /* without a sponge every profile is 1 (g = 1 exactly) */
  float *ones = NULL;
  const float *gxa = sponge ? sponge[0] : NULL, *gya = sponge ? sponge[1] : NULL,
              *gza = sponge ? sponge[2] : NULL;
  if (!sponge) {
    const long m = sx > sy ? (sx > sz ? sx : sz) : (sy > sz ? sy : sz);
    ones = (float *)malloc(sizeof(float) * (size_t)m);
    if (!ones) return -1;
    for (long k = 0; k < m; ++k) ones[k] = 1.0f;
    gxa = gya = gza = ones;
  }
  sep_row_args a;
  for (int k = 0; k < O_NCOEF; ++k) a.c[k] = coef[k];
  a.inv[0] = 1.0 / ((double)dx * dx);
  a.inv[1] = 1.0 / ((double)dy * dy);
  a.inv[2] = 1.0 / ((double)dz * dz);
  a.inv[3] = 1.0 / ((double)dx * dy);
  a.inv[4] = 1.0 / ((double)dx * dz);
  a.inv[5] = 1.0 / ((double)dy * dz);
  a.dt2 = (double)dt * (double)dt;
  a.sY = sx;
  a.sZ = sx * sy;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long z = 4; z < sz - 4; ++z)
    for (long y = 4; y < sy - 4; ++y)
      sep_row(&a, y * a.sY + z * a.sZ, 4, sx - 4, pc, qc, pp, qp, pxd, pyd, qxd, qyd, gxa,
              gya[y], gza[z]);
  free(ones);
  return 0;
}

/* ---- medium set-up --------------------------------------------------- */

void o_default_anisotropy(long n, float *vpz, float *vsv, float *epsilon,
                          float *delta, float *phi, float *theta) {
  /* src/precomp.c:156-169 with SIGMA = 0.75 <= MAX_SIGMA = 10
   * (include/precomp.h:3-4): vsv = vpz*sqrtf(|eps-delta|/SIGMA), the
   * division done in double as in the reference. */
  for (long i = 0; i < n; ++i) {
    vpz[i] = 3000.0;
    epsilon[i] = 0.24;
    delta[i] = 0.1;
    phi[i] = 1.0;
    theta[i] = atanf(1.0);
    vsv[i] = vpz[i] * sqrtf(fabsf(epsilon[i] - delta[i]) / 0.75);
  }
}

void o_precomp(long n, const float *theta, const float *phi, const float *vsv,
               const float *vpz, const float *epsilon, const float *delta,
               float *const out[O_NCOEF]) {
  /* src/precomp.c:85-105: double-precision libm trig rounded to float, float
   * products; v2px/v2pn scale in double then round. */
  for (long i = 0; i < n; ++i) {
    const float st = sin(theta[i]);
    const float ct = cos(theta[i]);
    const float s2t = sin(2.0 * theta[i]);
    const float sp = sin(phi[i]);
    const float cp = cos(phi[i]);
    const float s2p = sin(2.0 * phi[i]);
    out[O_CH1DXX][i] = st * st * cp * cp;
    out[O_CH1DYY][i] = st * st * sp * sp;
    out[O_CH1DZZ][i] = ct * ct;
    out[O_CH1DXY][i] = st * st * s2p;
    out[O_CH1DYZ][i] = s2t * sp;
    out[O_CH1DXZ][i] = s2t * cp;
  }
  for (long i = 0; i < n; ++i) {
    out[O_V2SZ][i] = vsv[i] * vsv[i];
    out[O_V2PZ][i] = vpz[i] * vpz[i];
    out[O_V2PX][i] = out[O_V2PZ][i] * (1.0 + 2.0 * epsilon[i]);
    out[O_V2PN][i] = out[O_V2PZ][i] * (1.0 + 2.0 * delta[i]);
  }
}

/* Distance and reference cell of one axis inside the absorbing shell,
 * src/boundary.c:57-89. */
static inline int shell_dist(int g, int first_in, int bord_len, int n) {
  if (g > bord_len + n) return g - bord_len - n;
  if (g < first_in) return first_in - g;
  return 0;
}

void o_random_velocity_boundary(int local_sx, int local_sy, int local_sz,
                                int global_sx, int global_sy, int global_sz,
                                int start_x, int start_y, int start_z, int nx,
                                int ny, int nz, int bord, int absorb,
                                float *vpz, float *vsv, unsigned int *seed) {
  /* src/boundary.c:7-104.  Every cell of the shell region draws one rand_r
   * value in global z,y,x order, whether or not it lies in this partition,
   * so that partitions agree on the sequence.  Cells outside the shell and
   * outside the interior (the stencil halo) are zeroed. */
  const int bord_len = bord + absorb - 1;
  const int first_in = bord_len + 1;
  const float frac = 1.0f / (float)absorb;
  const float max_p = 3000.0f;
  const float max_s = max_p * sqrtf(fabsf(0.24f - 0.1f) / 0.75f);
  const int end_x = start_x + local_sx, end_y = start_y + local_sy,
            end_z = start_z + local_sz;
  for (int gz = 0; gz < global_sz; ++gz) {
    for (int gy = 0; gy < global_sy; ++gy) {
      for (int gx = 0; gx < global_sx; ++gx) {
        const int inside = gz >= first_in && gz <= bord_len + nz &&
                           gy >= first_in && gy <= bord_len + ny &&
                           gx >= first_in && gx <= bord_len + nx;
        if (inside) continue;
        const int in_shell = gz >= bord && gz <= 2 * bord_len + nz &&
                             gy >= bord && gy <= 2 * bord_len + ny &&
                             gx >= bord && gx <= 2 * bord_len + nx;
        const int mine = gx >= start_x && gx < end_x && gy >= start_y &&
                         gy < end_y && gz >= start_z && gz < end_z;
        if (in_shell) {
          const float r = (float)rand_r(seed) / (float)RAND_MAX;
          if (!mine) continue;
          const long i = (long)(gx - start_x) +
                         (long)(gy - start_y) * local_sx +
                         (long)(gz - start_z) * local_sx * local_sy;
          int d = shell_dist(gy, first_in, bord_len, ny);
          const int dz_ = shell_dist(gz, first_in, bord_len, nz);
          const int dx_ = shell_dist(gx, first_in, bord_len, nx);
          d = d > dz_ ? d : dz_;
          d = d > dx_ ? d : dx_;
          const float w = (float)d * frac;
          vpz[i] = max_p * (1.0f - w) + max_p * r * w;
          vsv[i] = max_s * (1.0f - w) + max_s * r * w;
        } else if (mine) {
          const long i = (long)(gx - start_x) +
                         (long)(gy - start_y) * local_sx +
                         (long)(gz - start_z) * local_sx * local_sy;
          vpz[i] = 0.0f;
          vsv[i] = 0.0f;
        }
      }
    }
  }
}

float o_source(float dt, int it, double fcut) {
  /* src/calculate_source.c:10-17 (constants :6-8: pi^3, 2*sqrt(pi),
   * 3*sqrt(pi)); tf, fc and expo are stored in float as there. */
  const double pi_cube = 31.00627668029982017537;
  const double two_sqrt_pi = 3.54490770181103205458;
  const double three_sqrt_pi = 5.31736155271654808184;
  const float tf = two_sqrt_pi / fcut;
  const float fc = fcut / three_sqrt_pi;
  const float fct = fc * (((float)it) * dt - tf);
  const float expo = pi_cube * fct * fct;
  return (1.0f - 2.0f * expo) * expf(-expo);
}

void o_sponge_profile(long s, long a, double kappa, float *g) {
  for (long i = 0; i < s; ++i) {
    long d = 0;
    if (a > 0 && i >= 4 && i < s - 4) {
      const long lo = (4 + a) - i;           /* low side: 1..a */
      const long hi = i - (s - 5 - a);       /* high side: 1..a */
      d = lo > d ? lo : d;
      d = hi > d ? hi : d;
    }
    const double t = a > 0 ? kappa * (double)d / (double)a : 0.0;
    g[i] = (float)exp(-t * t);
  }
}

float o_round_f16(float x) {
  /* IEEE binary16, round to nearest even (GCC's _Float16 conversion) */
  return (float)(_Float16)x;
}

float o_round_bf16(float x) {
  /* bfloat16: keep the top 16 bits, round to nearest even; NaN stays NaN */
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

static void round_store(const o_run_cfg *cfg, float *f, int comp) {
  const long sx = cfg->sx, sy = cfg->sy, sz = cfg->sz;
  const float sc = ldexpf(1.0f, cfg->store_exp[comp]);
  const float inv = ldexpf(1.0f, -cfg->store_exp[comp]);
  for (long z = 4; z < sz - 4; ++z)
    for (long y = 4; y < sy - 4; ++y)
      for (long x = 4; x < sx - 4; ++x) {
        const long i = x + y * sx + z * sx * sy;
        const float v = f[i] * sc;
        f[i] = (cfg->store == O_STORE_F16 ? o_round_f16(v) : o_round_bf16(v)) * inv;
      }
}

/* ---- time loop ----------------------------------------------------------- */

static void swap_ptr(void **a, void **b) {
  void *t = *a;
  *a = *b;
  *b = t;
}

int o_run(const o_run_cfg *cfg, void *pp0, void *pc0, void *qp0, void *qc0) {
  const long sx = cfg->sx, sy = cfg->sy, sz = cfg->sz;
  const long n = sx * sy * sz;
  const int sep = cfg->kind == O_KIND_F64_SEP;
  const int f64 = cfg->kind == O_KIND_F64 || sep;
  const size_t esz = f64 ? sizeof(double) : sizeof(float);
  void *pp = pp0, *pc = pc0, *qp = qp0, *qc = qc0;
  const long b0[3] = {4, 4, 4}, b1[3] = {sx - 4, sy - 4, sz - 4};
  const float *const *sp = cfg->sponge[0] ? cfg->sponge : NULL;
  double *work = NULL;
  if (sep) {
    if (cfg->coef[0] == NULL) return -1;
    work = (double *)calloc((size_t)n * 4, sizeof(double));
    if (!work) return -1;
  }
  for (int it = 0; it < cfg->steps; ++it) {
    /* src/worker.c:467-470: the source goes into pc and qc before the
     * stencil reads them */
    if (cfg->src_index >= 0 && cfg->src) {
      const float s = cfg->src[it];
      if (f64) {
        ((double *)pc)[cfg->src_index] += (double)s;
        ((double *)qc)[cfg->src_index] += (double)s;
      } else {
        ((float *)pc)[cfg->src_index] += s;
        ((float *)qc)[cfg->src_index] += s;
      }
    }
    const int rc =
        sep ? o_step_f64_sep(sx, sy, sz, cfg->dx, cfg->dy, cfg->dz, cfg->dt,
                             (const double *)pc, (const double *)qc, (double *)pp,
                             (double *)qp, cfg->coef, sp, work, cfg->nthreads)
            : o_step(cfg->kind, sx, sy, sz, b0, b1, cfg->dx, cfg->dy, cfg->dz,
                     cfg->dt, pc, qc, pp, qp, cfg->coef, cfg->vpz, cfg->vsv, sp,
                     cfg->nthreads);
    if (rc != 0) {
      free(work);
      return -1;
    }
    if (!f64 && cfg->store != O_STORE_F32) {
      round_store(cfg, (float *)pp, 0);
      round_store(cfg, (float *)qp, 1);
    }
    /* src/worker.c:506 */
    swap_ptr(&pp, &pc);
    swap_ptr(&qp, &qc);
    if (cfg->traces && cfg->nrec > 0) {
      for (long r = 0; r < cfg->nrec; ++r) {
        const long i = cfg->rec[r];
        cfg->traces[(long)it * cfg->nrec + r] =
            f64 ? ((double *)pc)[i] : (double)((float *)pc)[i];
      }
    }
    if (cfg->energy) {
      double e = 0.0;
      for (long z = 4; z < sz - 4; ++z) {
        double ez = 0.0;
        for (long y = 4; y < sy - 4; ++y)
          for (long x = 4; x < sx - 4; ++x) {
            const long i = x + y * sx + z * sx * sy;
            const double p = f64 ? ((double *)pc)[i] : ((float *)pc)[i];
            const double q = f64 ? ((double *)qc)[i] : ((float *)qc)[i];
            ez += p * p + q * q;
          }
        e += ez;
      }
      cfg->energy[it] = e;
    }
  }
  free(work);
  if (cfg->steps % 2 == 1) {
    /* results live in the caller's pp/qp buffers: swap contents back */
    void *tmp = malloc((size_t)n * esz);
    if (!tmp) return -1;
    memcpy(tmp, pc0, (size_t)n * esz);
    memcpy(pc0, pp0, (size_t)n * esz);
    memcpy(pp0, tmp, (size_t)n * esz);
    memcpy(tmp, qc0, (size_t)n * esz);
    memcpy(qc0, qp0, (size_t)n * esz);
    memcpy(qp0, tmp, (size_t)n * esz);
    free(tmp);
  }
  return 0;
}

double o_rel_l2_f32(long n, const float *a, const float *b) {
  double num = 0.0, den = 0.0;
  for (long i = 0; i < n; ++i) {
    const double d = (double)a[i] - (double)b[i];
    num += d * d;
    den += (double)b[i] * (double)b[i];
  }
  return den > 0.0 ? sqrt(num / den) : sqrt(num);
}
