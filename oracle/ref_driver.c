/*
 * ref_driver.c -- one-rank driver around the reference's own sources.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_oracle.py compiles this file
 * together with the reference's src/openmp_propagate.c, src/precomp.c,
 * src/boundary.c, src/calculate_source.c, src/device_data.c and src/log.c
 * (read where they lie; never copied) into oracle/_ref/libref.so.  It is
 * used to pin the oracle restatement (dc_oracle.c) and to generate the
 * golden fixtures in tests/golden/.
 *
 * The time loop replays dc_worker_process for one rank (src/worker.c:466-
 * 511) with the same region split as dc_compute_boundaries and
 * dc_compute_interior (src/worker.c:321-402): six 4-thick shells and the
 * interior, each handed to the reference's dc_propagate.
 *
 * ref_run(kind=1) replays the reference CUDA backend's arithmetic on the
 * host: src/cuda_propagate.cu:25-29 calls sample_compute_optimized
 * (include/sample_compute.h:21-102) for every point of the box; here the
 * same header-inline function is called from a host loop.
 *
 * Built with -DREF_DEVICE_BACKEND and linked with the reference's
 * src/cuda_propagate.cu and src/device_data.cu instead (librefcuda.so), the
 * same loop runs the reference's own GPU path: dc_device_data_init copies
 * the host arrays to the device, dc_propagate launches propagate_kernel for
 * each box and synchronises, dc_device_data_get_results copies pc and qc
 * back into the caller's arrays.  kind 1 is not available there (the
 * fields live on the device).
 */
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "boundary.h"
#include "calculate_source.h"
#include "dc_process.h"
#include "device_data.h"
#include "precomp.h"
#include "propagate.h"
#include "sample_compute.h"

typedef void (*box_fn)(const size_t s[3], const size_t e[3],
                       const size_t sizes[3], dc_device_data *data, float dx,
                       float dy, float dz, float dt);

/* The linked backend's dc_propagate (OpenMP, or CUDA in librefcuda.so). */
static void box_backend(const size_t s[3], const size_t e[3],
                        const size_t sizes[3], dc_device_data *data, float dx,
                        float dy, float dz, float dt) {
  const int coords[3] = {0, 0, 0}, topo[3] = {1, 1, 1};
  dc_propagate(s, e, sizes, coords, topo, data, dx, dy, dz, dt);
}

#ifndef REF_DEVICE_BACKEND
static void box_refcuda(const size_t s[3], const size_t e[3],
                        const size_t sizes[3], dc_device_data *data, float dx,
                        float dy, float dz, float dt) {
  if (e[0] <= s[0] || e[1] <= s[1] || e[2] <= s[2]) return;
  for (size_t z = s[2]; z < e[2]; z++)
    for (size_t y = s[1]; y < e[1]; y++)
      for (size_t x = s[0]; x < e[0]; x++)
        sample_compute_optimized(x, y, z, sizes[0], sizes[1], sizes[2], 0, 0,
                                 0, 1, 1, 1, dx, dy, dz, dt, data->pc,
                                 data->qc, data->pp, data->qp, data->vpz,
                                 data->vsv);
}
#endif

/* The region split of src/worker.c:321-402 for one rank. */
static void one_step(box_fn fn, const size_t sizes[3], dc_device_data *data,
                     float dx, float dy, float dz, float dt) {
  const size_t r = 4;
  size_t s[3], e[3];
  if (!(sizes[0] >= 4 * r && sizes[1] >= 4 * r && sizes[2] >= 4 * r)) {
    s[0] = s[1] = s[2] = r;
    e[0] = sizes[0] - r;
    e[1] = sizes[1] - r;
    e[2] = sizes[2] - r;
    fn(s, e, sizes, data, dx, dy, dz, dt);
    return;
  }
  for (int side = 0; side < 2; side++) {
    s[0] = side == 0 ? r : sizes[0] - 2 * r;
    e[0] = side == 0 ? 2 * r : sizes[0] - r;
    s[1] = r; e[1] = sizes[1] - r;
    s[2] = r; e[2] = sizes[2] - r;
    fn(s, e, sizes, data, dx, dy, dz, dt);
  }
  for (int side = 0; side < 2; side++) {
    s[0] = 2 * r; e[0] = sizes[0] - 2 * r;
    s[1] = side == 0 ? r : sizes[1] - 2 * r;
    e[1] = side == 0 ? 2 * r : sizes[1] - r;
    s[2] = r; e[2] = sizes[2] - r;
    fn(s, e, sizes, data, dx, dy, dz, dt);
  }
  for (int side = 0; side < 2; side++) {
    s[0] = 2 * r; e[0] = sizes[0] - 2 * r;
    s[1] = 2 * r; e[1] = sizes[1] - 2 * r;
    s[2] = side == 0 ? r : sizes[2] - 2 * r;
    e[2] = side == 0 ? 2 * r : sizes[2] - r;
    fn(s, e, sizes, data, dx, dy, dz, dt);
  }
  s[0] = s[1] = s[2] = 2 * r;
  e[0] = sizes[0] - 2 * r;
  e[1] = sizes[1] - 2 * r;
  e[2] = sizes[2] - 2 * r;
  fn(s, e, sizes, data, dx, dy, dz, dt);
}

/* Threads an OpenMP parallel region of the linked backend uses (1 in the
 * device build). */
int ref_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/*
 * Runs `steps` steps.  kind 0: the linked backend's dc_propagate (OpenMP
 * path with 10 precomputed coefficient arrays in `coef`, dc_precomp_vars
 * order; or the reference CUDA path with vpz/vsv); kind 1: the reference
 * CUDA arithmetic replayed on the host (vpz/vsv; not in the device build).
 * src[it] is added to pc and qc at src_index before step it (src_index < 0:
 * none).  Buffers rotate as in the reference; on return *out_pc/*out_qc
 * point at the final fields (one of the caller's buffers).  *seconds (if
 * not NULL) receives the wall time of the time loop alone, between
 * dc_device_data_init and dc_device_data_get_results (the CUDA backend
 * synchronises after every dc_propagate, src/cuda_propagate.cu:63).
 * Returns 0, or -1 for a kind the build does not have.
 */
int ref_run_timed(int kind, long sx, long sy, long sz, float dx, float dy,
                  float dz, float dt, int steps, long src_index,
                  const float *src, float *const coef[10], float *vpz,
                  float *vsv, float *pp, float *pc, float *qp, float *qc,
                  float **out_pc, float **out_qc, double *seconds) {
  static char hostname[256];
  dc_process_t proc;
  box_fn fn = box_backend;
#ifdef REF_DEVICE_BACKEND
  if (kind != 0) return -1;
#else
  if (kind == 1) fn = box_refcuda;
#endif
  memset(&proc, 0, sizeof(proc));
  /* src/device_data.cu:18-33 picks the device by host name among the
   * workers: one worker, rank 0 */
  proc.hostnames = hostname;
  proc.num_workers = 1;
  proc.sizes[0] = (size_t)sx;
  proc.sizes[1] = (size_t)sy;
  proc.sizes[2] = (size_t)sz;
  proc.pp = pp;
  proc.pc = pc;
  proc.qp = qp;
  proc.qc = qc;
  proc.anisotropy_vars.vpz = vpz;
  proc.anisotropy_vars.vsv = vsv;
  if (coef) {
    proc.precomp_vars.ch1dxx = coef[0];
    proc.precomp_vars.ch1dyy = coef[1];
    proc.precomp_vars.ch1dzz = coef[2];
    proc.precomp_vars.ch1dxy = coef[3];
    proc.precomp_vars.ch1dyz = coef[4];
    proc.precomp_vars.ch1dxz = coef[5];
    proc.precomp_vars.v2px = coef[6];
    proc.precomp_vars.v2pz = coef[7];
    proc.precomp_vars.v2sz = coef[8];
    proc.precomp_vars.v2pn = coef[9];
  }
  dc_device_data *data = dc_device_data_init(&proc);
  const double t0 = now_s();
  for (int it = 0; it < steps; it++) {
    if (src_index >= 0 && src) dc_device_add_source(data, (size_t)src_index, src[it]);
    one_step(fn, proc.sizes, data, dx, dy, dz, dt);
    dc_device_swap_arrays(data);
  }
  const double t1 = now_s();
  if (seconds) *seconds = t1 - t0;
  dc_device_data_get_results(&proc, data);
  *out_pc = proc.pc;
  *out_qc = proc.qc;
  dc_device_data_free(data);
  return 0;
}

int ref_run(int kind, long sx, long sy, long sz, float dx, float dy, float dz,
            float dt, int steps, long src_index, const float *src,
            float *const coef[10], float *vpz, float *vsv, float *pp,
            float *pc, float *qp, float *qc, float **out_pc, float **out_qc) {
  return ref_run_timed(kind, sx, sy, sz, dx, dy, dz, dt, steps, src_index, src,
                       coef, vpz, vsv, pp, pc, qp, qc, out_pc, out_qc, NULL);
}
