/*
 * dc_gb300 -- single-GPU command-line driver with the reference's options.
 *
 * Replaces the reference's MPI entry point (src/main.c), one-rank worker
 * loop (src/worker.c:451-525) and result writer (src/coordinator.c:116-219)
 * for one GB300:
 *   - the same required options as src/main.c:16-29 (--size-x/y/z, --dx/dy/dz,
 *     --dt, -t/--time-max, -a/--absorption, -o/--output-file);
 *   - the same padded sizes s = n + 2a + 8 (src/main.c:94-99), iteration count
 *     ceil(time_max / dt) in float (src/main.c:132), source at the global
 *     centre (src/coordinator.c:11-16), default medium with the random
 *     velocity boundary (src/main.c:158-172);
 *   - the same output file: the final pc block then the qc block, float32,
 *     the whole padded cube with zeros in the 4-cell halo -- written with two
 *     bulk writes instead of one seek + write per element;
 *   - the same CSV timing lines (src/main.c:200-215).
 * Extensions (optional): --steps, --fcut, --kernel, --loop, --boundary,
 * --sponge-kappa, --learned-weights, --checkpoint, --resume,
 * --print-iterations.  --boundary learned keeps the default medium in the
 * absorbing zone (no random velocity boundary) and corrects its outer cells
 * with the learned thin layer (weights: a .npy file of
 * DC_GB300_MLP_PARAMS float32 values, by default data/learned_layer8.npy
 * beside the executable).
 */
#include <argp.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "dc_gb300.h"

enum {
  K_SX = 128, K_SY, K_SZ, K_DX, K_DY, K_DZ, K_DT, /* src/main.c:17-23 */
  K_STEPS = 200, K_FCUT, K_KERNEL, K_LOOP, K_BOUNDARY, K_KAPPA, K_CKPT, K_RESUME,
  K_PRINT_IT, K_WEIGHTS
};

enum { B_RVB = 0, B_SPONGE = 1, B_LEARNED = 2 };

typedef struct {
  size_t size_x, size_y, size_z;
  float dx, dy, dz, dt, time_max;
  size_t absorption;
  char *output_file;
  long steps;
  double fcut;
  int kernel;         /* DC_GB300_KERNEL_* */
  int loop_abi;       /* 1: the reference ABI loop, 0: dc_gb300_run */
  int boundary;       /* B_RVB, B_SPONGE (random velocity boundary + sponge), B_LEARNED */
  double kappa;
  char *weights;
  char *checkpoint, *resume;
  int print_iterations;
} cli_args;

static struct argp_option options[] = {
    {"size-x", K_SX, "INTEGER", 0, "Grid size in X"},
    {"size-y", K_SY, "INTEGER", 0, "Grid size in Y"},
    {"size-z", K_SZ, "INTEGER", 0, "Grid size in Z"},
    {"dx", K_DX, "FLOAT", 0, "Step size in X"},
    {"dy", K_DY, "FLOAT", 0, "Step size in Y"},
    {"dz", K_DZ, "FLOAT", 0, "Step size in Z"},
    {"dt", K_DT, "FLOAT", 0, "Step size in time"},
    {"time-max", 't', "FLOAT", 0, "Max time"},
    {"absorption", 'a', "INTEGER", 0, "Absorption zone size"},
    {"output-file", 'o', "PATH", 0, "Path to the file to output the results to"},
    {"steps", K_STEPS, "INTEGER", 0, "Time steps (overrides ceil(time-max/dt))"},
    {"fcut", K_FCUT, "FLOAT", 0, "Source cut-off frequency (default 40; peak = fcut/3)"},
    {"kernel", K_KERNEL, "fast|exact", 0, "Stencil arithmetic (default fast)"},
    {"loop", K_LOOP, "graph|abi", 0, "Time loop: graph-captured runs (default) or the reference ABI calls"},
    {"boundary", K_BOUNDARY, "rvb|sponge|learned", 0, "Absorbing boundary (default rvb)"},
    {"sponge-kappa", K_KAPPA, "FLOAT", 0, "Sponge strength (default 0.35)"},
    {"learned-weights", K_WEIGHTS, "PATH", 0, "Network of --boundary learned (.npy)"},
    {"checkpoint", K_CKPT, "PATH", 0, "Write a checkpoint after the run"},
    {"resume", K_RESUME, "PATH", 0, "Resume from a checkpoint"},
    {"print-iterations", K_PRINT_IT, 0, 0, "Print the iteration count and exit"},
    {0}};

static error_t parse_opt(int key, char *arg, struct argp_state *state) {
  cli_args *a = state->input;
  switch (key) {
  case K_SX: a->size_x = atoi(arg); break;
  case K_SY: a->size_y = atoi(arg); break;
  case K_SZ: a->size_z = atoi(arg); break;
  case K_DX: a->dx = atof(arg); break;
  case K_DY: a->dy = atof(arg); break;
  case K_DZ: a->dz = atof(arg); break;
  case K_DT: a->dt = atof(arg); break;
  case 't': a->time_max = atof(arg); break;
  case 'a': a->absorption = atoi(arg); break;
  case 'o': a->output_file = strdup(arg); break;
  case K_STEPS: a->steps = atol(arg); break;
  case K_FCUT: a->fcut = atof(arg); break;
  case K_KERNEL:
    if (strcmp(arg, "exact") == 0) a->kernel = DC_GB300_KERNEL_EXACT;
    else if (strcmp(arg, "fast") == 0) a->kernel = DC_GB300_KERNEL_FAST;
    else argp_error(state, "--kernel must be fast or exact");
    break;
  case K_LOOP:
    if (strcmp(arg, "abi") == 0) a->loop_abi = 1;
    else if (strcmp(arg, "graph") == 0) a->loop_abi = 0;
    else argp_error(state, "--loop must be graph or abi");
    break;
  case K_BOUNDARY:
    if (strcmp(arg, "sponge") == 0) a->boundary = B_SPONGE;
    else if (strcmp(arg, "rvb") == 0) a->boundary = B_RVB;
    else if (strcmp(arg, "learned") == 0) a->boundary = B_LEARNED;
    else argp_error(state, "--boundary must be rvb, sponge or learned");
    break;
  case K_WEIGHTS: a->weights = strdup(arg); break;
  case K_KAPPA: a->kappa = atof(arg); break;
  case K_CKPT: a->checkpoint = strdup(arg); break;
  case K_RESUME: a->resume = strdup(arg); break;
  case K_PRINT_IT: a->print_iterations = 1; break;
  case ARGP_KEY_END:
    /* src/main.c:64-70: every reference option is required */
    if (a->size_x == 0 || a->size_y == 0 || a->size_z == 0 || a->dx == 0 || a->dy == 0 ||
        a->dz == 0 || a->time_max == 0 || a->dt == 0 || a->absorption == 0 ||
        (a->output_file == NULL && !a->print_iterations))
      argp_usage(state);
    break;
  default:
    return ARGP_ERR_UNKNOWN;
  }
  return 0;
}

static struct argp argp_def = {options, parse_opt, NULL,
                               "Fletcher TTI propagation on one GB300 (dc_gb300)"};

/* Reads a .npy file holding exactly `count` little-endian float32 values
 * (format versions 1 and 2, C order). */
static int read_npy_f32(const char *path, float *out, size_t count) {
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  unsigned char head[10];
  int ok = fread(head, 1, 8, f) == 8 && memcmp(head, "\x93NUMPY", 6) == 0;
  unsigned long hlen = 0;
  if (ok && head[6] == 1) {
    unsigned char b[2];
    ok = fread(b, 1, 2, f) == 2;
    hlen = b[0] | (unsigned long)b[1] << 8;
  } else if (ok && (head[6] == 2 || head[6] == 3)) {
    unsigned char b[4];
    ok = fread(b, 1, 4, f) == 4;
    hlen = b[0] | (unsigned long)b[1] << 8 | (unsigned long)b[2] << 16 | (unsigned long)b[3] << 24;
  } else {
    ok = 0;
  }
  char *hdr = ok && hlen < 65536 ? (char *)malloc(hlen + 1) : NULL;
  ok = ok && hdr && fread(hdr, 1, hlen, f) == hlen;
  if (ok) {
    hdr[hlen] = 0;
    char shape[64];
    snprintf(shape, sizeof(shape), "(%zu,)", count);
    ok = strstr(hdr, "'<f4'") && strstr(hdr, "'fortran_order': False") && strstr(hdr, shape);
  }
  free(hdr);
  ok = ok && fread(out, sizeof(float), count, f) == count;
  fclose(f);
  return ok ? 0 : -1;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void die(const char *what) {
  fprintf(stderr, "[dc_gb300] %s: %s\n", what, dc_gb300_last_error());
  exit(1);
}

/* Writes pc then qc over the whole padded cube with zeros in the halo
 * (src/coordinator.c:129-205). */
static int write_results(const char *path, const float *pc, const float *qc, size_t sx,
                         size_t sy, size_t sz) {
  const size_t n = sx * sy * sz;
  float *buf = (float *)malloc(sizeof(float) * n);
  if (!buf) return -1;
  FILE *f = fopen(path, "wb");
  if (!f) {
    free(buf);
    return -1;
  }
  int ok = 1;
  for (int k = 0; k < 2 && ok; ++k) {
    const float *src = k == 0 ? pc : qc;
    memset(buf, 0, sizeof(float) * n);
    for (size_t z = 4; z + 4 < sz; ++z)
      for (size_t y = 4; y + 4 < sy; ++y)
        memcpy(buf + 4 + y * sx + z * sx * sy, src + 4 + y * sx + z * sx * sy,
               sizeof(float) * (sx - 8));
    ok = fwrite(buf, sizeof(float), n, f) == n;
  }
  ok = (fclose(f) == 0) && ok;
  free(buf);
  return ok ? 0 : -1;
}

int main(int argc, char **argv) {
  cli_args a;
  memset(&a, 0, sizeof(a));
  a.steps = -1;
  a.fcut = 40.0;
  a.kappa = 0.35;
  argp_parse(&argp_def, argc, argv, 0, 0, &a);

  const size_t sx = a.size_x + 2 * a.absorption + 8; /* src/main.c:94-99 */
  const size_t sy = a.size_y + 2 * a.absorption + 8;
  const size_t sz = a.size_z + 2 * a.absorption + 8;
  /* src/main.c:132: float division, then ceil */
  const unsigned int iterations =
      a.steps >= 0 ? (unsigned int)a.steps : (unsigned int)ceil(a.time_max / a.dt);
  if (a.print_iterations) {
    printf("%u\n", iterations);
    return 0;
  }
  const size_t n = sx * sy * sz;
  const size_t src = sx / 2 + (sy / 2) * sx + (sz / 2) * sx * sy; /* src/coordinator.c:11-16 */

  const double t0 = now_s();
  /* medium: src/main.c:158-172 for the one rank at the origin */
  dc_anisotropy_t aniso = dc_compute_anisotropy_vars((int)sx, (int)sy, (int)sz);
  unsigned int seed = 0;
  if (a.boundary != B_LEARNED) /* the learned layer absorbs in the default medium */
    randomVelocityBoundaryPartition((int)sx, (int)sy, (int)sz, (int)sx, (int)sy, (int)sz, 0, 0,
                                    0, (int)a.size_x, (int)a.size_y, (int)a.size_z, 4,
                                    (int)a.absorption, aniso.vpz, aniso.vsv, &seed);
  dc_precomp_vars pre = dc_compute_precomp_vars((int)sx, (int)sy, (int)sz, aniso);
  float *pc = (float *)calloc(n, sizeof(float));
  float *qc = (float *)calloc(n, sizeof(float));
  if (!pc || !qc) {
    fprintf(stderr, "[dc_gb300] OOM: could not allocate field arrays\n");
    return 1;
  }
  float *amp = (float *)malloc(sizeof(float) * ((size_t)iterations + 1));
  for (unsigned int it = 0; it <= iterations; ++it)
    amp[it] = dc_gb300_source(a.dt, (int)it, a.fcut);

  double loop_t0 = 0, loop_t1 = 0;
  if (a.loop_abi) {
    /* src/worker.c:451-525 through the reference ABI, one box per step */
    if (a.boundary != B_RVB || a.checkpoint || a.resume) {
      fprintf(stderr,
              "[dc_gb300] --loop abi supports neither the sponge, the learned layer nor "
              "checkpoints\n");
      return 1;
    }
    if (a.kernel == DC_GB300_KERNEL_EXACT) setenv("DC_GB300_KERNEL", "exact", 1);
    dc_process_t proc;
    memset(&proc, 0, sizeof(proc));
    proc.topology[0] = proc.topology[1] = proc.topology[2] = 1;
    proc.iterations = iterations;
    proc.source_index = (int)src;
    proc.dx = a.dx;
    proc.dy = a.dy;
    proc.dz = a.dz;
    proc.dt = a.dt;
    proc.sizes[0] = sx;
    proc.sizes[1] = sy;
    proc.sizes[2] = sz;
    proc.anisotropy_vars = aniso;
    proc.precomp_vars = pre;
    proc.pc = pc;
    proc.qc = qc;
    proc.num_workers = 1;
    dc_device_data *data = dc_device_data_init(&proc);
    const size_t b0[3] = {4, 4, 4}, b1[3] = {sx - 4, sy - 4, sz - 4};
    const int coords[3] = {0, 0, 0}, topo[3] = {1, 1, 1};
    loop_t0 = now_s();
    for (unsigned int it = 0; it < iterations; ++it) {
      dc_device_add_source(data, src, amp[it]);
      dc_propagate(b0, b1, proc.sizes, coords, topo, data, a.dx, a.dy, a.dz, a.dt);
      dc_device_swap_arrays(data);
    }
    dc_device_data_get_results(&proc, data);
    loop_t1 = now_s();
    dc_device_data_free(data);
  } else {
    dc_gb300_config cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.sx = (long)sx;
    cfg.sy = (long)sy;
    cfg.sz = (long)sz;
    cfg.dx = a.dx;
    cfg.dy = a.dy;
    cfg.dz = a.dz;
    cfg.dt = a.dt;
    cfg.kernel = a.kernel;
    cfg.medium = DC_GB300_MEDIUM_PRECOMP;
    cfg.device = getenv("DC_GB300_DEVICE") ? atoi(getenv("DC_GB300_DEVICE")) : 0;
    dc_gb300_sim *sim = NULL;
    if (dc_gb300_create(&cfg, &sim) != DC_GB300_OK) die("create");
    if (dc_gb300_set_precomp(sim, &pre) != DC_GB300_OK) die("set_precomp");
    if (dc_gb300_set_fields(sim, NULL, NULL, NULL, NULL) != DC_GB300_OK) die("set_fields");
    if (dc_gb300_set_source(sim, (long)src, amp, (int)iterations + 1) != DC_GB300_OK)
      die("set_source");
    /* after set_source: the checkpoint records whether pc holds the next
       step's source already */
    if (a.resume && dc_gb300_load_checkpoint(sim, a.resume) != DC_GB300_OK) die("resume");
    dc_gb300_mlp *mlp = NULL;
    if (a.boundary == B_LEARNED) {
      char def[PATH_MAX];
      const char *wpath = a.weights;
      if (!wpath) { /* data/learned_layer8.npy beside the executable */
        const ssize_t len = readlink("/proc/self/exe", def, sizeof(def) - 40);
        if (len <= 0) die("locate the executable");
        def[len] = 0;
        char *slash = strrchr(def, '/');
        strcpy(slash ? slash + 1 : def, "data/learned_layer8.npy");
        wpath = def;
      }
      float *w = (float *)malloc(sizeof(float) * DC_GB300_MLP_PARAMS);
      if (!w || read_npy_f32(wpath, w, DC_GB300_MLP_PARAMS) != 0) {
        fprintf(stderr, "[dc_gb300] cannot read network weights from %s\n", wpath);
        return 1;
      }
      if (dc_gb300_mlp_create(cfg.device, &mlp) != DC_GB300_OK) die("mlp_create");
      if (dc_gb300_mlp_set_params(mlp, w) != DC_GB300_OK) die("mlp_set_params");
      free(w);
      if (dc_gb300_set_learned_layer(sim, mlp, (int)a.absorption) != DC_GB300_OK)
        die("set_learned_layer");
    }
    if (a.boundary == B_SPONGE) {
      float *g[3];
      const size_t s3[3] = {sx, sy, sz};
      for (int d = 0; d < 3; ++d) {
        g[d] = (float *)malloc(sizeof(float) * s3[d]);
        dc_gb300_sponge_profile((long)s3[d], (long)a.absorption, a.kappa, g[d]);
      }
      if (dc_gb300_set_sponge(sim, g[0], g[1], g[2]) != DC_GB300_OK) die("set_sponge");
      for (int d = 0; d < 3; ++d) free(g[d]);
    }
    const long done = dc_gb300_steps_done(sim);
    const long todo = (long)iterations > done ? (long)iterations - done : 0;
    loop_t0 = now_s();
    if (dc_gb300_run(sim, (int)todo) != DC_GB300_OK) die("run");
    if (dc_gb300_synchronize(sim) != DC_GB300_OK) die("synchronize");
    if (dc_gb300_get_fields(sim, NULL, pc, NULL, qc) != DC_GB300_OK) die("get_fields");
    loop_t1 = now_s();
    if (a.checkpoint && dc_gb300_save_checkpoint(sim, a.checkpoint) != DC_GB300_OK)
      die("checkpoint");
    dc_gb300_destroy(sim);
    dc_gb300_mlp_destroy(mlp);
  }
  const double total = now_s() - t0;
  if (a.output_file && write_results(a.output_file, pc, qc, sx, sy, sz) != 0) {
    fprintf(stderr, "[dc_gb300] Failed to write output file: %s\n", a.output_file);
    return 1;
  }
  /* src/main.c:200-215: compute region (s-8)^3 x iterations */
  const double msamples =
      (double)(sx - 8) * (double)(sy - 8) * (double)(sz - 8) * (double)iterations / 1e6;
  printf("rank,total_time,msamples_per_s\n");
  printf("%d,%lf,%lf\n", 0, total, msamples / (loop_t1 - loop_t0 > 0 ? loop_t1 - loop_t0 : 1));
  printf("*,%lf,%lf\n", total, msamples / total);

  dc_free_anisotropy_vars(&aniso);
  dc_free_precomp_vars(&pre);
  free(pc);
  free(qc);
  free(amp);
  free(a.output_file);
  free(a.weights);
  return 0;
}
