/*
 * dc_oracle.h -- CPU oracle for the Fletcher TTI propagation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (Dannful/distributed-cube-average) used as the checker for the
 * GB300 CUDA path and as the timed CPU baseline ("port").  Nothing in the
 * product library links, loads or calls it; only tests/, the smoke check in
 * __graft_entry__.py and the cpu_baseline leg of bench.py do.
 *
 * Each function cites the reference file:line it restates.  The float path
 * keeps the reference's operation order so that, compiled without FMA
 * contraction, it is bit-identical to the reference's OpenMP path
 * (src/openmp_propagate.c -> include/sample_compute.h:sample_compute).
 * That claim is pinned by the golden fixtures under tests/golden/, which
 * were produced by the reference's own sources (see oracle/build_oracle.py
 * and tests/golden/make_golden.py).
 *
 * Layout: x fastest, index = x + y*sx + z*sx*sy (include/indexing.h:15-21),
 * padded sizes sx,sy,sz with a 4-cell stencil halo (include/definitions.h:4).
 */
#ifndef DC_ORACLE_H
#define DC_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Coefficient array order = field order of dc_precomp_vars
 * (include/precomp.h:6-17). */
enum {
  O_CH1DXX = 0, O_CH1DYY, O_CH1DZZ, O_CH1DXY, O_CH1DYZ, O_CH1DXZ,
  O_V2PX, O_V2PZ, O_V2SZ, O_V2PN, O_NCOEF
};

/* Arithmetic variants of one time step. */
enum {
  O_KIND_F32 = 0,        /* sample_compute (10 coefficient arrays), float */
  O_KIND_F32_REFCUDA = 1,/* sample_compute_optimized (vpz/vsv, const angles) */
  O_KIND_F64 = 2,        /* sample_compute restated in double precision */
  O_KIND_F64_SEP = 3     /* the same in double, cross terms as D_a(D_b p)
                            (o_run only: whole compute region, 10 arrays) */
};

/* ---- medium set-up (host) ------------------------------------------- */

/* Default homogeneous medium, src/precomp.c:156-169. */
void o_default_anisotropy(long n, float *vpz, float *vsv, float *epsilon,
                          float *delta, float *phi, float *theta);

/* Trig + velocity precompute, src/precomp.c:85-105.  out[k] has n floats. */
void o_precomp(long n, const float *theta, const float *phi, const float *vsv,
               const float *vpz, const float *epsilon, const float *delta,
               float *const out[O_NCOEF]);

/* Random velocity boundary, src/boundary.c:7-104 (glibc rand_r sequence). */
void o_random_velocity_boundary(int local_sx, int local_sy, int local_sz,
                                int global_sx, int global_sy, int global_sz,
                                int start_x, int start_y, int start_z, int nx,
                                int ny, int nz, int bord, int absorb,
                                float *vpz, float *vsv, unsigned int *seed);

/* Ricker-type source, src/calculate_source.c:10-17, with FCUT as a
 * parameter (the reference fixes FCUT=40 at :5). */
float o_source(float dt, int it, double fcut);

/* Sponge profile along one axis of padded size s, absorbing width a:
 * g[i] = exp(-(kappa*d/a)^2), d = cells into the absorbing shell (0 inside
 * the physical interior and in the halo).  New component: the reference has
 * no sponge. */
void o_sponge_profile(long s, long a, double kappa, float *g);

/* ---- one time step over a box ----------------------------------------- */

/* Updates pp/qp in place over [b0,b1) (half-open per axis), like
 * dc_propagate (src/openmp_propagate.c:6-32).  kind selects the arithmetic.
 * coef: O_NCOEF arrays (kind F32/F64) -- ignored for REFCUDA.
 * vpz/vsv: used by REFCUDA only.  sponge: three profiles gx,gy,gz or NULL.
 * For kind F64 the field pointers are double*.  Returns 0 or -1 on a box
 * outside [4, s-4). */
int o_step(int kind, long sx, long sy, long sz, const long b0[3],
           const long b1[3], float dx, float dy, float dz, float dt,
           const void *pc, const void *qc, void *pp, void *qp,
           const float *const coef[O_NCOEF], const float *vpz,
           const float *vsv, const float *const sponge[3], int nthreads);

/* One FP64 step over the whole compute region [4, s-4)^3 with the cross
 * derivatives as D_a(D_b p) (see O_KIND_F64_SEP); work: 4 n doubles. */
int o_step_f64_sep(long sx, long sy, long sz, float dx, float dy, float dz, float dt,
                   const double *pc, const double *qc, double *pp, double *qp,
                   const float *const coef[O_NCOEF], const float *const sponge[3],
                   double *work, int nthreads);

/* ---- time loop -------------------------------------------------------- */

typedef struct {
  int kind;                      /* O_KIND_* */
  long sx, sy, sz;               /* padded sizes */
  float dx, dy, dz, dt;
  int steps;
  long src_index;                /* -1: no source */
  const float *src;              /* [steps] amplitudes, added to pc and qc */
  const float *coef[O_NCOEF];
  const float *vpz, *vsv;
  const float *sponge[3];        /* gx[sx], gy[sy], gz[sz] or NULLs */
  long nrec;                     /* receivers: trace[it*nrec+r] = p after it */
  const long *rec;
  double *traces;                /* [steps*nrec] or NULL */
  double *energy;                /* [steps]: sum(p^2+q^2) over [4,s-4)^3 */
  int nthreads;
  /* Mixed-precision storage emulation (this library's own form, not the
   * reference's): after each step every updated pp/qp value is rounded to
   * `store` (O_STORE_*) after scaling by 2^store_exp[0] (p) / [1] (q). */
  int store;
  int store_exp[2];
} o_run_cfg;

enum { O_STORE_F32 = 0, O_STORE_F16 = 1, O_STORE_BF16 = 2 };

/* Round-to-nearest-even of x to FP16 / BF16, returned as float. */
float o_round_f16(float x);
float o_round_bf16(float x);

/* One-rank replay of dc_worker_process (src/worker.c:466-511): per step
 * add source to pc and qc, update [4,s-4)^3, swap.  On return pc/qc hold the
 * final current fields and pp/qp the previous ones (the buffers are swapped
 * back when `steps` is odd).  Field pointers are float* or double* (F64). */
int o_run(const o_run_cfg *cfg, void *pp, void *pc, void *qp, void *qc);

/* Relative L2 distance ||a-b|| / ||b|| over n floats, in double. */
double o_rel_l2_f32(long n, const float *a, const float *b);

#ifdef __cplusplus
}
#endif

#endif
