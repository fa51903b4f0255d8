/*
 * dc_gb300.h -- C ABI of libdc_gb300.so, a GB300-native (sm_103a) Fletcher
 * TTI pseudo-acoustic propagator that drops in for the time-step path of
 * Dannful/distributed-cube-average.
 *
 * Part 1 re-declares the reference's own entry points and ABI structs with
 * identical signatures and layouts, so the reference's host code (src/
 * worker.c, src/main.c) links against this library in place of its CUDA or
 * OpenMP backend (reference Makefile:30-60 picks one backend at link time).
 * Each declaration cites the reference declaration it replaces.
 *
 * Part 2 is this library's own API (dc_gb300_*): status-returning, one
 * stream per simulation, multi-step runs captured in CUDA graphs, fused
 * source injection, sponge, receivers and energy.
 *
 * Conventions shared by both parts:
 *   - arrays are x fastest: index = x + y*sx + z*sx*sy
 *     (reference include/indexing.h:15-21); sizes include the 4-cell stencil
 *     halo (include/definitions.h:4);
 *   - only points in [4, s-4) per axis are ever updated.
 */
#ifndef DC_GB300_H
#define DC_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ====================================================================== */
/* Part 1 -- the reference ABI                                            */
/* ====================================================================== */

#ifndef DC_GB300_NO_REFERENCE_TYPES
/* include/precomp.h:6-17 */
typedef struct {
  float *ch1dxx;
  float *ch1dyy;
  float *ch1dzz;
  float *ch1dxy;
  float *ch1dyz;
  float *ch1dxz;
  float *v2px;
  float *v2pz;
  float *v2sz;
  float *v2pn;
} dc_precomp_vars;

/* include/precomp.h:19-26 */
typedef struct {
  float *theta;
  float *phi;
  float *vsv;
  float *vpz;
  float *epsilon;
  float *delta;
} dc_anisotropy_t;

/* include/dc_process.h:7-21 (DIMENSIONS = 3, NEIGHBOURHOOD = 27) */
typedef struct {
  int rank;
  int coordinates[3];
  int neighbours[27];
  int topology[3];
  unsigned int iterations;
  int source_index;
  float dx, dy, dz, dt;
  size_t sizes[3];
  dc_anisotropy_t anisotropy_vars;
  dc_precomp_vars precomp_vars;
  float *pp, *pc, *qp, *qc;
  char *hostnames;
  size_t num_workers;
} dc_process_t;

/* include/device_data.h:11-15.  The field and medium pointers are device
 * pointers into this library's arrays, in this library's device layout:
 *   - p and q are stored interleaved as (p, q) pairs, so qp == pp + 1 and
 *     qc == pc + 1 and consecutive points of one field are 2 floats apart;
 *   - rows are `pitch` points apart, pitch = sx rounded up to a multiple of
 *     4 (dc_gb300_device_pitch());
 *   - vpz/vsv are interleaved pairs (vsv == vpz + 1); the ten coefficients
 *     are grouped per point -- (ch1dxx, ch1dyy, ch1dxy, ch1dzz),
 *     (ch1dxz, ch1dyz, v2px, v2pz), (v2sz, v2pn) -- and each precomp_vars
 *     pointer addresses its lane of the group.
 * The reference's host code only hands these pointers back to the entry
 * points below (src/worker.c:482-485, :500-501), which understand the
 * layout; dc_device_data_get_results returns dense host arrays. */
typedef struct {
  float *pp, *pc, *qp, *qc;
  float *vpz, *vsv;
  dc_precomp_vars precomp_vars;
} dc_device_data;
#endif /* DC_GB300_NO_REFERENCE_TYPES */

/* include/propagate.h:13-18 -- src/cuda_propagate.cu:32-69.
 * Updates pp/qp in place for every point of the half-open box
 * [start_coords, end_coords) of an array of extent `sizes`.
 * process_coordinates/topology are accepted and ignored, as in the
 * reference (include/sample_compute.h:23-25).  Launches asynchronously on
 * the simulation's stream (the reference synchronises after every call);
 * dc_device_data_get_results synchronises.  A box outside [4, size-4) or
 * sizes that differ from the ones given to dc_device_data_init print an
 * error and exit(1), like the reference's error path. */
void dc_propagate(const size_t start_coords[3], const size_t end_coords[3],
                  const size_t sizes[3], const int process_coordinates[3],
                  const int topology[3], dc_device_data *data, const float dx,
                  const float dy, const float dz, const float dt);

/* include/device_data.h:17 -- src/device_data.cu:35-94.
 * Allocates the device arrays and copies pp, pc, qp, qc and the medium from
 * the process.  The medium comes from process->precomp_vars (all ten arrays)
 * when ch1dxx is non-NULL, else from process->anisotropy_vars (the trig
 * precompute then runs on the GPU in FP64).  vpz/vsv are copied when
 * present.  Selects CUDA device 0 unless DC_GB300_DEVICE is set (the
 * reference picks by hostname rank, src/device_data.cu:18-33).
 * Environment: DC_GB300_KERNEL=fast|exact selects the stencil arithmetic;
 * DC_GB300_MEDIUM=precomp|vpz_vsv selects the medium form (vpz_vsv = the
 * reference CUDA backend's constant-angle arithmetic,
 * include/sample_compute.h:9-18).
 * Host arrays the GPU can address (pinned or registered memory, and plain
 * malloc'd memory where the GPU reads pageable memory through the host's
 * page tables, as on NVLink-C2C systems) are read in place by the packing
 * kernels, one pass at the link's bandwidth; other memory is staged through
 * copies.  DC_GB300_STAGED_COPIES=1 stages every host array. */
dc_device_data *dc_device_data_init(dc_process_t *process);

/* include/device_data.h:19 -- src/device_data.cu:96-105 */
void dc_device_data_free(dc_device_data *data);

/* include/device_data.h:21 -- src/device_data.cu:107-117.
 * Waits for all queued work, then copies pc and qc to process->pc/qc. */
void dc_device_data_get_results(dc_process_t *process, dc_device_data *data);

/* include/device_data.h:23 -- src/device_data.cu:119-129: pointer swap
 * pp<->pc, qp<->qc (host side; no device work). */
void dc_device_swap_arrays(dc_device_data *data);

/* include/device_data.h:25 -- src/device_data.cu:131-139:
 * pc[index] += source; qc[index] += source (queued on the stream). */
void dc_device_add_source(dc_device_data *data, size_t index, float source);

/* include/device_data.h:27-31 -- src/device_data.cu:141-161.  Copies the
 * box [start,end) of the device array `from_array` into the dense host
 * buffer (x fastest).  Synchronous. */
void dc_device_extract_halo_face(dc_device_data *data, float *buffer,
                                 const size_t start_coords[3],
                                 const size_t end_coords[3],
                                 const size_t sizes[3],
                                 const float *from_array);

/* include/device_data.h:33-37 -- src/device_data.cu:163-183.  Copies the
 * dense host buffer into the box [start,end) of `to_array`.  Synchronous. */
void dc_device_insert_halo_face(dc_device_data *data, const float *buffer,
                                const size_t start_coords[3],
                                const size_t end_coords[3],
                                const size_t sizes[3], float *to_array);

/* include/precomp.h:28-29 -- src/precomp.c:9-108.  Host arrays (malloc'd,
 * freed with dc_free_precomp_vars).  The trigonometry runs on the GPU in
 * FP64 and is rounded to float as the reference rounds its host libm
 * results. */
dc_precomp_vars dc_compute_precomp_vars(int sx, int sy, int sz,
                                        dc_anisotropy_t anisotropy);

/* include/precomp.h:30 -- src/precomp.c:110-171: default homogeneous
 * medium (vpz 3000, eps 0.24, delta 0.10, phi 1 rad, theta pi/4, SIGMA
 * rule for vsv), malloc'd host arrays. */
dc_anisotropy_t dc_compute_anisotropy_vars(int sx, int sy, int sz);

/* include/precomp.h:31 -- src/precomp.c:189-211 */
void dc_free_precomp_vars(dc_precomp_vars *vars);

/* include/precomp.h:32 -- src/precomp.c:173-187 */
void dc_free_anisotropy_vars(dc_anisotropy_t *anisotropy);

/* include/boundary.h:5-12 -- src/boundary.c:7-104: random velocity
 * boundary on host arrays, same glibc rand_r sequence. */
void randomVelocityBoundaryPartition(int local_sx, int local_sy, int local_sz,
                                     int global_sx, int global_sy,
                                     int global_sz, int start_x, int start_y,
                                     int start_z, int nx, int ny, int nz,
                                     int bord, int absorb, float *vpz,
                                     float *vsv, unsigned int *seed);

/* include/calculate_source.h:3 -- src/calculate_source.c:10-17 (FCUT=40). */
float dc_calculate_source(float dt, int it);

/* ====================================================================== */
/* Part 2 -- this library's own API                                       */
/* ====================================================================== */

/* Status codes. */
enum {
  DC_GB300_OK = 0,
  DC_GB300_ERR_ARG = 1,     /* invalid argument (size, box, pointer) */
  DC_GB300_ERR_CUDA = 2,    /* a CUDA runtime/driver call failed */
  DC_GB300_ERR_NOMEM = 3,   /* allocation failed */
  DC_GB300_ERR_DEVICE = 4,  /* no usable sm_103 device */
  DC_GB300_ERR_TIMEOUT = 5, /* a bounded device wait gave up */
  DC_GB300_ERR_STATE = 6    /* call not valid in the current state */
};

/* Stencil arithmetic. */
enum {
  DC_GB300_KERNEL_FAST = 0,  /* separable cross derivatives, FMA */
  DC_GB300_KERNEL_EXACT = 1  /* the reference's operation order, no FMA:
                                bit-identical to the reference OpenMP path */
};

/* Medium form read by the stencil. */
enum {
  DC_GB300_MEDIUM_PRECOMP = 0,     /* ten FP32 coefficients (64 B/update) */
  DC_GB300_MEDIUM_VPZ_VSV = 1,     /* vpz/vsv + the reference CUDA backend's
                                      constant angles (32 B/update) */
  DC_GB300_MEDIUM_PRECOMP_F16 = 2, /* mixed precision: the fast kernel reads an
                                      FP16 copy of the ten coefficients, the
                                      velocity terms scaled by a power of two;
                                      arithmetic and wavefields stay FP32
                                      (44 B/update) */
  DC_GB300_MEDIUM_PRECOMP_BF16 = 3 /* the same with a BF16 copy */
};

typedef struct dc_gb300_sim dc_gb300_sim;

typedef struct {
  long sx, sy, sz;          /* padded sizes incl. 4-cell halo, each >= 9 */
  float dx, dy, dz, dt;
  int kernel;               /* DC_GB300_KERNEL_* */
  int medium;               /* DC_GB300_MEDIUM_* */
  int device;               /* CUDA ordinal; < 0 = current device */
} dc_gb300_config;

/* Last error message of the calling thread ("" if none). */
const char *dc_gb300_last_error(void);

/* Library version string. */
const char *dc_gb300_version(void);

int dc_gb300_create(const dc_gb300_config *cfg, dc_gb300_sim **out);
void dc_gb300_destroy(dc_gb300_sim *sim);

/* The reference-ABI view of a simulation (shares its arrays). */
dc_device_data *dc_gb300_device_data(dc_gb300_sim *sim);
/* The simulation behind a dc_device_data from dc_device_data_init. */
dc_gb300_sim *dc_gb300_from_device_data(dc_device_data *data);
long dc_gb300_device_pitch(const dc_gb300_sim *sim);

/* Medium from dense host arrays (sx*sy*sz floats each; read in place when
 * the GPU can address them, see dc_device_data_init). */
int dc_gb300_set_precomp(dc_gb300_sim *sim, const dc_precomp_vars *host);
int dc_gb300_set_vpz_vsv(dc_gb300_sim *sim, const float *vpz,
                         const float *vsv);
/* Uploads theta, phi, vsv, vpz, epsilon, delta and runs the FP64 trig
 * precompute of src/precomp.c:85-105 on the GPU. */
int dc_gb300_set_anisotropy(dc_gb300_sim *sim, const dc_anisotropy_t *host);

/* Copies the device medium back to dense host arrays (sx*sy*sz floats
 * each; NULL members are skipped).  Synchronous. */
int dc_gb300_get_precomp(dc_gb300_sim *sim, const dc_precomp_vars *host);
int dc_gb300_get_vpz_vsv(dc_gb300_sim *sim, float *vpz, float *vsv);

/* The reference's one-rank medium generated on the GPU: the default
 * anisotropy (src/precomp.c:156-169), the random velocity boundary of
 * src/boundary.c:7-104 with the same glibc rand_r sequence (replayed by
 * skip-ahead, not a serial sweep) and the FP64 trig precompute.  The
 * simulation's sizes must be n + 2*absorb + 8 per axis (src/main.c:94-99). */
int dc_gb300_generate_reference(dc_gb300_sim *sim, long nx, long ny, long nz,
                                long absorb, unsigned int seed);

/* Seeded layered medium generated on the GPU (see dc_gb300_layered_spec). */
#define DC_GB300_MAX_LAYERS 32
#define DC_GB300_MAX_FEATURES 128
typedef struct {
  int nlayers;
  float layer_top[DC_GB300_MAX_LAYERS]; /* first global z of each layer */
  float vp[DC_GB300_MAX_LAYERS];
  float epsilon[DC_GB300_MAX_LAYERS];
  float delta[DC_GB300_MAX_LAYERS];
  float vp_noise;                   /* relative amplitude (0.02 = 2 %) */
  float theta_lo, theta_hi;         /* marginal range of theta */
  float phi_lo, phi_hi;             /* marginal range of phi */
  float sigma_ratio;                /* vsv = vp*sqrt(|eps-delta|/ratio) */
  /* random Fourier features: field = sqrt(2/n) sum cos(k.r + ph) with
   * k = (kx,ky,kz) in radians per cell and r the global cell index */
  int n_noise, n_theta, n_phi;
  float k_noise[DC_GB300_MAX_FEATURES][4];  /* kx, ky, kz, phase */
  float k_theta[DC_GB300_MAX_FEATURES][4];
  float k_phi[DC_GB300_MAX_FEATURES][4];
  /* global origin of this array inside a larger model (crops) */
  long ox, oy, oz;
} dc_gb300_layered_spec;
int dc_gb300_generate_layered(dc_gb300_sim *sim,
                              const dc_gb300_layered_spec *spec);

/* Fields from dense host arrays; NULL means zeros.  Resets the step
 * counter to 0. */
int dc_gb300_set_fields(dc_gb300_sim *sim, const float *pp, const float *pc,
                        const float *qp, const float *qc);
/* Copies the fields to dense host arrays (NULL skips one; written in place
 * when the GPU can address them).  Synchronous. */
int dc_gb300_get_fields(dc_gb300_sim *sim, float *pp, float *pc, float *qp,
                        float *qc);

/* Point source at linear index `index`: before step it, amplitudes[it] is
 * added to pc and qc (src/worker.c:467-470); steps beyond `count` add 0.
 * index < 0 removes the source.  The addition for step it+1 is fused into
 * the store of step it; the fields returned by dc_gb300_get_fields and saved
 * by checkpoints are nevertheless exactly the reference's state after the
 * steps run (without the next step's amplitude). */
int dc_gb300_set_source(dc_gb300_sim *sim, long index,
                        const float *amplitudes, int count);

/* Sponge: after each update the new value is multiplied by
 * g = gx[x]*gy[y]*gz[z] and the previous field is damped by g before use.
 * NULL pointers remove it. */
int dc_gb300_set_sponge(dc_gb300_sim *sim, const float *gx, const float *gy,
                        const float *gz);

/* Receivers: after step it, trace[it*count + r] = p at index[r] (the new
 * field, before the next step's source).  Capacity max_steps rows. */
int dc_gb300_set_receivers(dc_gb300_sim *sim, const long *index, int count,
                           int max_steps);
int dc_gb300_get_traces(dc_gb300_sim *sim, float *out, int steps);

/* Energy: after step it, energy[it] = sum(p^2 + q^2) over [4,s-4)^3 of the
 * new fields, accumulated in FP64 across blocks. */
int dc_gb300_enable_energy(dc_gb300_sim *sim, int max_steps);
int dc_gb300_get_energy(dc_gb300_sim *sim, double *out, int steps);

/* Advances `steps` time steps (source -> stencil over [4,s-4)^3 -> swap),
 * queued on the simulation's stream; runs of >= 2 steps are replayed from
 * a captured CUDA graph. */
int dc_gb300_run(dc_gb300_sim *sim, int steps);
int dc_gb300_synchronize(dc_gb300_sim *sim);
long dc_gb300_steps_done(const dc_gb300_sim *sim);

/* One stencil pass over a box without source or swap (the dc_propagate
 * semantics, status-returning). */
int dc_gb300_propagate_box(dc_gb300_sim *sim, const size_t start[3],
                           const size_t end[3]);

/* Checkpoint / resume.  The file holds a 64-byte header (magic "DCGB300C",
 * version 1, sx, sy, sz, steps done, whether pc/qc already contain the next
 * step's source) followed by the dense float32 arrays pp, qp, pc, qc.
 * Loading requires a simulation of the same sizes and restores the step
 * counter, so a resumed run continues bit-identically.  Synchronous. */
int dc_gb300_save_checkpoint(dc_gb300_sim *sim, const char *path);
int dc_gb300_load_checkpoint(dc_gb300_sim *sim, const char *path);

/* Kernel launches issued by this simulation so far (stencil + helpers). */
long dc_gb300_kernel_launches(const dc_gb300_sim *sim);

/* Stream of the simulation (a cudaStream_t) for event timing. */
void *dc_gb300_stream(dc_gb300_sim *sim);

/* The wavelet of dc_calculate_source with the cut-off frequency as a
 * parameter (the reference fixes FCUT = 40, src/calculate_source.c:5); the
 * Ricker peak frequency is fcut / 3. */
float dc_gb300_source(float dt, int it, double fcut);

/* Sponge profile along one axis of padded size s with absorbing width a:
 * g[i] = exp(-(kappa*d/a)^2), d = cells into the shell (1 next to the
 * physical interior .. a next to the halo), 1 elsewhere. */
void dc_gb300_sponge_profile(long s, long a, double kappa, float *g);

/* ---- Part 3: batched shots over one shared medium (no counterpart in the
 * reference, whose time loop src/worker.c:466-511 advances one shot) ----
 *
 * A batch holds one medium box and any number of shots.  A shot is a box
 * cropped out of the medium, with its own (p, q) wavefields, wavelet, sponge
 * and receivers, stepped exactly as a dc_gb300_sim with the fast kernel
 * steps its cube (bit-identical fields for the same cropped medium).  One
 * step of all shots is one launch of a persistent kernel per 64 shots;
 * runs are captured into CUDA graphs. */
typedef struct dc_gb300_batch dc_gb300_batch;

typedef struct {
  long mx, my, mz;          /* medium box sizes (x fastest) */
  float dx, dy, dz, dt;
  int medium;               /* DC_GB300_MEDIUM_PRECOMP, _PRECOMP_F16 or _PRECOMP_BF16 */
  int device;               /* CUDA ordinal; -1 = current */
  int max_steps;            /* capacity of wavelet tables and traces */
} dc_gb300_batch_config;

typedef struct {
  long sx, sy, sz;          /* padded sizes of the shot box (>= 9) */
  long ox, oy, oz;          /* medium position of the box's point (0, 0, 0); ox % 4 == 0 */
  long src_x, src_y, src_z; /* source in box coordinates, inside [4, s-4)^3 */
  double fcut;              /* wavelet cut-off frequency (Ricker peak fcut / 3) */
  long absorb;              /* sponge width in cells (0: none) */
  double kappa;             /* sponge strength (dc_gb300_sponge_profile) */
} dc_gb300_shot;

int dc_gb300_batch_create(const dc_gb300_batch_config *cfg, dc_gb300_batch **out);
int dc_gb300_batch_destroy(dc_gb300_batch *batch);
/* Medium of the whole box: the layered generator, or dense host arrays of
 * mx*my*mz coefficients in the reference's precomp layout. */
int dc_gb300_batch_generate_layered(dc_gb300_batch *batch, const dc_gb300_layered_spec *spec);
int dc_gb300_batch_set_precomp(dc_gb300_batch *batch, const dc_precomp_vars *vars);
/* Adds a shot with zero wavefields; *index receives its number. */
int dc_gb300_batch_add_shot(dc_gb300_batch *batch, const dc_gb300_shot *shot, int *index);
/* Receivers of one shot as (x, y, z) triples in box coordinates; traces
 * (p before the next step's source, [step][receiver]) restart from zero. */
int dc_gb300_batch_set_receivers(dc_gb300_batch *batch, int shot, int count, const long *xyz);
/* Applies a learned thin absorbing layer `layer` cells wide (see Part 4)
 * to every shot after each step (0 turns it off).  Set it after adding
 * every shot: dc_gb300_batch_add_shot fails while a layer is set. */
struct dc_gb300_mlp;
int dc_gb300_batch_set_learned_layer(dc_gb300_batch *batch, const struct dc_gb300_mlp *mlp,
                                     int layer);
/* Tile rows (8 or 16) and z-chunks per column (1..64). */
int dc_gb300_batch_set_tiles(dc_gb300_batch *batch, int ty, int zsplit);
int dc_gb300_batch_tiles(const dc_gb300_batch *batch, int *ty, int *zsplit);
/* Grid of the batch kernel: persistent CTAs striding over the work items
 * (1, the default) or one CTA per work item (0).  dc_gb300_batch_grid
 * returns the current choice. */
int dc_gb300_batch_set_grid(dc_gb300_batch *batch, int persistent);
int dc_gb300_batch_grid(const dc_gb300_batch *batch);
/* Times every candidate -- tile rows x z-split x grid (persistent or one
 * CTA per work item) -- for `steps` steps on this batch, keeps the fastest
 * (ms per step in *ms; the grid choice via dc_gb300_batch_grid) and returns
 * the batch to step 0 with zero wavefields and traces: call it before the
 * first run. */
int dc_gb300_batch_autotune(dc_gb300_batch *batch, int steps, int *ty, int *zsplit, float *ms);
/* Queues `steps` steps of every shot (asynchronous on the batch's stream). */
int dc_gb300_batch_run(dc_gb300_batch *batch, int steps);
int dc_gb300_batch_synchronize(dc_gb300_batch *batch);
/* Dense sx*sy*sz fields of one shot (any pointer may be NULL); the same
 * observable state as a dc_gb300_sim after the same steps.  Synchronous. */
int dc_gb300_batch_get_fields(dc_gb300_batch *batch, int shot, float *pp, float *pc, float *qp,
                              float *qc);
int dc_gb300_batch_get_traces(dc_gb300_batch *batch, int shot, int steps, float *out);
int dc_gb300_batch_steps_done(const dc_gb300_batch *batch);
long dc_gb300_batch_kernel_launches(const dc_gb300_batch *batch);
void *dc_gb300_batch_stream(dc_gb300_batch *batch);
/* Updated points per step summed over the shots ((s-8) per axis). */
long long dc_gb300_batch_points(const dc_gb300_batch *batch);

/* ---- Part 4: the learned thin absorbing layer (no counterpart in the
 * reference, which absorbs with its random velocity boundary,
 * src/boundary.c:7-104) ----
 *
 * A layer of L cells between the interior and the 4-cell halo, corrected
 * after every stencil pass by an MLP: for each layer cell, the cell and the
 * 7 cells inward along its boundary normal, p and q at t+1 (the stencil's
 * output) and t, are 32 features; r = their rms; the network maps x / r
 * through 32 -> 32 -> 32 -> 2 (GELU; BF16 weights and activations, FP32
 * accumulation; first-layer bias per depth in the layer) and r * output is
 * added to the cell's (p, q).  Parameters (FP32, DC_GB300_MLP_PARAMS):
 * W1[32][32] | b1[DEPTHS][32] | W2[32][32] | b2[32] | W3[2][32] | b3[2].
 * Samples are rows of 33 floats (32 features, then the depth); targets rows
 * of 2 floats. */
#define DC_GB300_MLP_IN 32
#define DC_GB300_MLP_HIDDEN 32
#define DC_GB300_MLP_OUT 2
#define DC_GB300_MLP_DEPTHS 16
#define DC_GB300_MLP_PARAMS (32 * 32 + 16 * 32 + 32 * 32 + 32 + 2 * 32 + 2)

typedef struct dc_gb300_mlp dc_gb300_mlp;

int dc_gb300_mlp_create(int device, dc_gb300_mlp **out);
int dc_gb300_mlp_destroy(dc_gb300_mlp *mlp);
/* Seeded initialisation (normal, std 1/sqrt(fan-in); output layer x 0.01). */
int dc_gb300_mlp_init(dc_gb300_mlp *mlp, unsigned int seed);
int dc_gb300_mlp_set_params(dc_gb300_mlp *mlp, const float *params);
int dc_gb300_mlp_get_params(dc_gb300_mlp *mlp, float *params);
/* Device address of the parameters the kernels read (weights rounded to
 * BF16); stable for the MLP's lifetime. */
const float *dc_gb300_mlp_device_params(const dc_gb300_mlp *mlp);
/* Corrections r * y for n device samples into device out[n][2]. */
int dc_gb300_mlp_forward(dc_gb300_mlp *mlp, const float *samples, long long n, float *out);
/* Gradient (host grad[DC_GB300_MLP_PARAMS]) of sum |r*y - target|^2 over
 * the n device samples; loss[0] = that sum, loss[1] = sum r^2. */
int dc_gb300_mlp_gradient(dc_gb300_mlp *mlp, const float *samples, const float *targets,
                          long long n, float *grad, double *loss);
/* `steps` Adam steps (lr, betas 0.9 / 0.999) on minibatches of `batch`
 * samples drawn with replacement from the n device samples; loss_hist
 * (host, may be NULL) receives each step's sum|r*y - t|^2 / sum r^2. */
int dc_gb300_mlp_train(dc_gb300_mlp *mlp, const float *samples, const float *targets,
                       long long n, int steps, int batch, float lr, unsigned long long seed,
                       float *loss_hist);
/* The layer cells of a padded box (sx, sy, sz) with a layer `layer` cells
 * wide, in the order the kernels use: cells[4*i..4*i+3] = x, y, z and
 * axis | side << 2 | depth << 3 (axis of the normal, side 1 = high end,
 * depth 0 = next to the interior).  Writes at most `cap` entries (cells may
 * be NULL) and returns the count, or -1 on invalid geometry.  Host only. */
long long dc_gb300_layer_cells(long sx, long sy, long sz, int layer, int *cells, long long cap);
/* How a step applies the layer: the corrected cells split into face lines,
 * corrected in place by one fused pass, and edge cells, whose corrections
 * are computed into a buffer and then added.  lines[4*i..4*i+3] = x, y, z of
 * a line's outermost cell and axis | side << 2 (the line is the 4 cells
 * from there inward); edge[] holds dc_gb300_layer_cells entries.  Writes at
 * most lines_cap / edge_cap entries (either array may be NULL) and the
 * counts to *n_lines / *n_edge; returns DC_GB300_OK or an error.  Host only. */
int dc_gb300_layer_plan(long sx, long sy, long sz, int layer, int *lines, long long lines_cap,
                        int *edge, long long edge_cap, long long *n_lines, long long *n_edge);
/* Applies the MLP after every stencil pass of dc_gb300_run to the layer
 * cells of a layer `layer` cells wide (1..DC_GB300_MLP_DEPTHS; 0 turns it
 * off).  The simulation reads the MLP's parameters at every step: keep the
 * MLP alive while it is set, and do not train it or set its parameters
 * while a run that uses it may still be executing (the MLP and the
 * simulation have separate streams; synchronise the simulation first). */
int dc_gb300_set_learned_layer(dc_gb300_sim *sim, const dc_gb300_mlp *mlp, int layer);
/* Teacher-forced training samples: the fields of `wide` (t and t-1) are
 * cropped at offset[] to the box of `thin` (zero halo), `thin` steps once
 * (its own sponge, no source, no learned layer) and `wide` steps once; each
 * layer cell of `thin` appends a sample (features of the thin step, depth)
 * to the device array samples[cap][33] and a target (wide field at t+1
 * minus the thin step) to targets[cap][2].  *count = samples written. */
int dc_gb300_lb_sample(dc_gb300_sim *wide, dc_gb300_sim *thin, const long offset[3], int layer,
                       float *samples, float *targets, long long cap, long long *count);
/* Rollout samples (training on the states the layer itself produces): the
 * fields of `wide` are cropped into `thin` once, then `steps` times `thin`
 * steps with its learned layer (recording each layer cell's features before
 * its correction) and `wide` steps; targets are the wide field minus the
 * thin stencil's output.  `thin` must have a learned layer and no source.
 * Writes steps x (layer cells) samples; *count = that number. */
int dc_gb300_lb_rollout(dc_gb300_sim *wide, dc_gb300_sim *thin, const long offset[3], int steps,
                        float *samples, float *targets, long long cap, long long *count);

/* Runs `steps` time steps of the exact kernel (reference arithmetic, no
 * source, no sponge) over caller-owned device buffers and allocates no
 * device memory.  No counterpart in the reference: it serves callers that
 * cannot call cudaMalloc -- applications that own all device memory
 * themselves (a pre-sized pool, buffers registered with a communication
 * library) and time loops that must not allocate between steps.
 *
 *   cfg     sizes, spacings, dt, device; kernel must be
 *           DC_GB300_KERNEL_EXACT, medium DC_GB300_MEDIUM_PRECOMP or
 *           DC_GB300_MEDIUM_VPZ_VSV
 *   pairs   {previous, current}: two device buffers of interleaved (p, q)
 *           pairs, pitch = round_up(sx, 4) points per row, sy*sz rows --
 *           the layout of dc_device_data; on return pairs[1] holds the
 *           newest field and pairs[0] the one before it
 *   medium  device buffer in the grouped coefficient layout (PRECOMP) or
 *           of (vpz, vsv) pairs (VPZ_VSV), same pitch
 *   steps   0 .. 4096 (the scratch maximum); larger counts fail with
 *           DC_GB300_ERR_ARG and an explanatory message
 *   energy  host array of `steps` doubles receiving the per-step energy
 *           sum(p^2 + q^2) of each new field, or NULL
 *   stream  cudaStream_t to run on (NULL = legacy default stream);
 *           synchronised before return
 *
 * The only device memory used besides the caller's buffers is a fixed
 * 33 KB file-scope scratch array per device (per-step energy accumulators
 * and a step counter).  Every call synchronises `stream` and reads the
 * energy back, so no call may run while a stream capture is active: a call
 * on a capturing stream fails with DC_GB300_ERR_ARG and leaves the capture
 * untouched.  The first call on a device looks up the scratch address
 * (cudaGetSymbolAddress); it is kept for the life of the process: a
 * cudaDeviceReset between calls is not supported.  Each call clears the
 * part of the scratch it uses; all calls on a device share it, so calls
 * that overlap on the GPU race. */
int dc_gb300_exact_steps_noalloc(const dc_gb300_config *cfg, float *pairs[2],
                                 const float *medium, int steps, double *energy,
                                 void *stream);

#ifdef __cplusplus
}
#endif

#endif /* DC_GB300_H */
