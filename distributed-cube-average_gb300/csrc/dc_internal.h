// dc_internal.h -- internal declarations shared by the CUDA translation
// units of libdc_gb300.so.  Not part of the public ABI (include/dc_gb300.h).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "dc_gb300.h"

namespace dcg {

// ---------------------------------------------------------------------------
// Finite-difference coefficients: 8th-order central differences of the
// reference (include/derivatives.h:15-38), as exact rationals rounded once
// (they round to the same floats as the reference's decimal literals).
// ---------------------------------------------------------------------------
#define DCG_K0 (-205.0f / 72.0f)
#define DCG_K1 (8.0f / 5.0f)
#define DCG_K2 (-1.0f / 5.0f)
#define DCG_K3 (8.0f / 315.0f)
#define DCG_K4 (-1.0f / 560.0f)
#define DCG_L1 (4.0f / 5.0f)
#define DCG_L2 (-1.0f / 5.0f)
#define DCG_L3 (4.0f / 105.0f)
#define DCG_L4 (-1.0f / 280.0f)

// The ten medium coefficients of a point are stored grouped, so one thread
// reads all of them with three vector loads:
//   G0 float4 (cxx, cyy, cxy, czz)   at coef[4*i .. 4*i+3]
//   G1 float4 (cxz, cyz, v2px, v2pz) at coef[4*count + 4*i ..]
//   G2 float2 (v2sz, v2pn)           at coef[8*count + 2*i ..]
// (count = padded points).  DevCoef numbers the coefficients in that order.
enum DevCoef {
  DC_CXX = 0, DC_CYY, DC_CXY, DC_CZZ, DC_CXZ, DC_CYZ,
  DC_V2PX, DC_V2PZ, DC_V2SZ, DC_V2PN, DC_NCOEF
};

__host__ __device__ __forceinline__ long long coef_index(int k, long long i, long long count) {
  return k < 4 ? 4 * i + k : (k < 8 ? 4 * count + 4 * i + (k - 4) : 8 * count + 2 * i + (k - 8));
}

// Reduced-precision copy of the medium for the fast kernel (the mixed
// form) in three arrays: 8 bytes (cxx, cyy, cxy, czz), 8 bytes (cxz, cyz,
// v2px, v2pz) and 4 bytes (v2sz, v2pn) per point, 16 bits per value.
//  * CF_F16: the six angle terms as 16-bit fixed point (value x 2^15,
//    round to nearest, clamped to [-32768, 32767], stored + 32768); the four
//    velocity terms
//    as FP16 ratios d = v / b - 1 to an FP32 base b per medium row (the
//    midrange of the row's non-zero values), decoded as v = b + b * d.
//  * CF_BF16: all ten values rounded to BF16, the velocity terms scaled by
//    2^-vexp; the kernel folds 2^vexp into dt^2.
enum CoefForm { CF_F32 = 0, CF_VV = 1, CF_F16 = 2, CF_BF16 = 3 };
// Device slot of each dc_precomp_vars field (reference order ch1dxx, ch1dyy,
// ch1dzz, ch1dxy, ch1dyz, ch1dxz, v2px, v2pz, v2sz, v2pn).
constexpr int kRefToDev[10] = {DC_CXX, DC_CYY, DC_CZZ, DC_CXY, DC_CYZ,
                               DC_CXZ, DC_V2PX, DC_V2PZ, DC_V2SZ, DC_V2PN};

constexpr int kHalo = 4;  // stencil radius (include/definitions.h:4)

// Error word bits written by kernels.
enum : int { kErrTimeout = 1, kErrAlign = 2 };

struct StepParams {
  int x0, x1, y0, y1, z0, z1;   // half-open box of updated points
  int tile_x0, tile_y0;         // origin of the block grid (tile_x0 % 4 == 0)
  int zchunk;                   // output planes per block
  long long pitch, plane;       // floats between rows / planes
  float dxxinv, dyyinv, dzzinv, dxyinv, dxzinv, dyzinv;
  // fast kernel: FD weights pre-scaled by the grid spacing
  float w2x[5], w2y[5], w2z[5];  // K_i / da^2 (second derivative)
  float w1x[4], w1y[4], w1z[4];  // L_i / da   (first derivative, i = 1..4)
  float dt, dt2;
  float dt2_iso;  // dt2 / d^2 when dx = dy = dz (unscaled weights in the stencil)
  // Wavefields are stored as interleaved (p, q) pairs: `prev` holds
  // (pp, qp) and is updated in place, `cur` holds (pc, qc).
  float2 *prev;
  const float2 *cur;
  const float *coef;            // grouped FP32 coefficients (see coef_index)
  const float *vv;              // (vpz, vsv) pairs (VPZ_VSV medium)
  long long count;              // floats per array (incl. pitch padding)
  const float *sponge;          // gx[sx] | gy[sy] | gz[sz], or null
  int sponge_oy, sponge_oz;     // offsets of gy / gz in `sponge`
  // fused source: the value added when storing step `step` is
  // src_table[step + 1] (it becomes pc of the next step)
  int src_x, src_y, src_z;      // src_x < 0: none
  const float *src_table;
  int src_count;
  const int *d_step;            // device step counter (graph replays)
  float *src_pre;               // (p, q) at the source point before injection
  int step_offset;              // step = *d_step + step_offset
  // fused energy: sum(p^2+q^2) of the new fields, one double per step
  double *energy;
  int energy_cap;
  // fused receivers: per (x, y) column a run [start, start + count) of
  // receivers sorted by z (rec_z) with their trace slots (rec_r); traces
  // are [step][nrec] p values before the next step's source
  const int2 *rec_col;          // [sy][sx] or null
  const int *rec_z, *rec_r;
  float *traces;
  int nrec, trace_cap, col_stride;
  int *err;
  // position of the box's point (0, 0, 0) in the medium's arrays (the
  // batched form crops shots out of one shared medium; 0 otherwise)
  int mox, moy, moz;
};

// One launch of the batched fast kernel: up to kMaxBatchShots shots, each a
// box with its own wavefields, source, sponge and receivers, cropped out of
// one shared medium.  Work items are column tiles (x, y) x z-chunks of every
// shot, numbered shot by shot; persistent CTAs stride over them.
constexpr int kMaxBatchShots = 64;
struct BatchLaunch {
  CUtensorMap tm_l, tm_o1, tm_o2;  // shared medium (coefficient groups)
  CUtensorMap tm_vb;                // FP16 medium: velocity bases per row
  const CUtensorMap *maps;          // [shot][4]: halo of buffer 0, 1; own tile of buffer 0, 1
  const int *order;                 // launch order of the work items (null: shot by shot)
  int nshots;
  int cur_buf;                      // buffer holding (pc, qc) in every shot
  int n_items;
  int *err;
  int item_prefix[kMaxBatchShots + 1];
  int tiles_x[kMaxBatchShots], tiles_y[kMaxBatchShots];
  StepParams shot[kMaxBatchShots];
};

struct Sim {
  dc_gb300_sim *handle = nullptr;
  int device = 0;
  cudaStream_t stream = nullptr;
  long long sx = 0, sy = 0, sz = 0, pitch = 0, plane = 0, count = 0;
  float dx = 0, dy = 0, dz = 0, dt = 0;
  int kernel = DC_GB300_KERNEL_FAST;
  int medium = DC_GB300_MEDIUM_PRECOMP;
  // two pair buffers of `count` (p, q) elements; which one is "previous"
  // and which "current" is read from the reference-ABI view (abi.pp/abi.pc)
  float2 *pq[2] = {nullptr, nullptr};
  float *coef = nullptr;       // grouped FP32 coefficients (see coef_index)
  float *vv = nullptr;         // (vpz, vsv) pairs
  // reduced-precision copy used by the fast kernel (DC_GB300_MEDIUM_*_F16/BF16)
  void *coef16 = nullptr;      // [count] x 8 B, [count] x 8 B, [count] x 4 B
  float4 *vbase = nullptr;     // CF_F16: velocity bases per row, [sz][sy]
  int coef_form = CF_F32;      // CoefForm the fast kernel reads
  int vexp = 0;                // velocity terms stored scaled by 2^-vexp
  bool coef16_stale = true;
  float *sponge = nullptr;     // [sx + sy + sz]
  bool has_sponge = false;
  // source
  long long src_gi = -1;
  int src_x = -1, src_y = -1, src_z = -1;
  float *d_src = nullptr;
  int src_count = 0;
  long long src_applied_step = -1;  // pc already holds src(step) for it
  float *d_src_pre = nullptr;       // values the stencil stored before that
  // receivers (see StepParams::rec_col)
  int2 *d_rec_col = nullptr;
  int *d_rec_z = nullptr, *d_rec_r = nullptr;
  int nrec = 0;
  float *d_traces = nullptr;
  int trace_cap = 0;
  // energy
  double *d_energy = nullptr;
  int energy_cap = 0;
  // counters and status
  int *d_step = nullptr;
  long long steps_done = 0;
  int *d_err = nullptr;
  long long launches = 0;
  int config_version = 0;
  // tensor maps for the fast kernel (encoded for one tile shape)
  CUtensorMap tm_halo[2], tm_own[2], tm_c[4];  // tm_c: L, O1, O2, row bases
  bool deep_ring = false;  // fast FP32 sweep with the 4-stage TMA ring
  int fast_slots = 0;      // fast-sweep CTAs resident on the device at once
  int maps_tx = 0, maps_ty = 0;
  // learned absorbing layer, applied after every stencil pass of a run
  const float *lb_params = nullptr;  // MLP compute parameters (device, owned by the MLP)
  int4 *d_lb_cells = nullptr;        // layer-cell table (recorded rollout steps)
  float2 *d_lb_corr = nullptr;       // corrections of one step
  long long lb_cells = 0;
  int4 *d_lb_lines = nullptr;        // face lines and edge cells (every other step)
  int4 *d_lb_edge = nullptr;
  long long lb_lines = 0, lb_edge = 0;
  int lb_layer = 0;
  float *lb_rec = nullptr;           // rollout training: record the step's samples here
  // captured multi-step graphs, keyed by start parity of the pc buffer
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int graph_steps[2] = {0, 0};
  int graph_version[2] = {-1, -1};
  int graph_pc[2] = {-1, -1};
};

// Fast-kernel tile geometry (chosen at compile time; see tti_fast.cu).
struct FastShape {
  int tx, ty, zchunk;
};
// Tile shape and z-chunk of a fast pass over an nx x ny x nz box.
FastShape fast_shape(const Sim *sim, long long nx, long long ny, long long nz);
bool fast_encode_maps(Sim *sim, std::string *err);
// Tile rows (TY) of the fast kernel for coefficient form `form`: 8 unless
// DC_GB300_FAST_TY selects 16.
int fast_default_ty(int form);
// Whether tile rows `ty` are compiled for coefficient form `form` (8 and 16).
bool fast_tile_rows_valid(int ty, int form);
// Tensor maps of one (p, q) pair buffer for tiles of 32 x ty: the halo box
// (read as the current field) and the own tile (previous field).
bool fast_encode_pair_maps(const float2 *buf, long long sx, long long sy, long long sz,
                           long long pitch, int ty, CUtensorMap *halo, CUtensorMap *own,
                           std::string *err);
// Tensor maps of the three coefficient groups of a medium in form `form`.
// out[0..2] = the groups L, O1, O2; out[3] = the FP16 form's row bases
// (vbase, [sz][sy] float4; a copy of out[2] for the other forms).
bool fast_encode_medium_maps(int form, const float *coef, const void *coef16, const float *vv,
                             const float4 *vbase, long long sx, long long sy, long long sz,
                             long long pitch, long long count, int ty, CUtensorMap out[4],
                             std::string *err);
// Batched fast kernel (always with the sponge).  `blocks` = persistent CTAs.
cudaError_t batch_prepare(int ty, int form);  // shared-memory attributes
// `sponge` false: every shot's sponge profile is 1 (the no-sponge sweep)
int batch_blocks_per_sm(int ty, int form, bool iso, bool sponge);
cudaError_t launch_batch(cudaStream_t st, const BatchLaunch &bl, int ty, int form, bool iso,
                         bool sponge, int blocks);

// Launchers.  Return the cudaError_t of the launch.
cudaError_t launch_fast(Sim *sim, const StepParams &prm, int cur_buf,
                        int prev_buf);
cudaError_t launch_exact(Sim *sim, const StepParams &prm);
cudaError_t launch_add_source(cudaStream_t st, float2 *cur, long long gi,
                              const float *table, int count,
                              const int *d_step, int step_offset);
cudaError_t launch_add_value(cudaStream_t st, float2 *cur, long long gi,
                             float value);
// Dense (x fastest, no pitch) p and q arrays <-> pitched pair buffer; a null
// dense pointer reads as zeros / is skipped.
cudaError_t launch_pack(cudaStream_t st, float2 *dst, const float *p,
                        const float *q, long long sx, long long sy,
                        long long sz, long long pitch);
cudaError_t launch_unpack(cudaStream_t st, const float2 *src, float *p,
                          float *q, long long sx, long long sy, long long sz,
                          long long pitch);
// One component (0 = p, 1 = q) of a box of a pair buffer <-> dense buffer.
cudaError_t launch_box_copy(cudaStream_t st, float2 *pairs, int comp,
                            float *dense, const long long b0[3],
                            const long long b1[3], long long pitch,
                            long long plane, bool to_dense);
cudaError_t launch_advance_step(cudaStream_t st, int *d_step, int by);
// Precompute from dense anisotropy arrays (n points) into grouped
// coefficients at dense indices (count = n); callers repack to the pitch.
cudaError_t launch_precomp(cudaStream_t st, const float *theta,
                           const float *phi, const float *vsv,
                           const float *vpz, const float *eps,
                           const float *delta, float *coef, long long count,
                           long long n);
// One coefficient (DevCoef k): dense device array <-> grouped pitched
// coefficients (count = padded points; pitch = sx and count = n address a
// dense grouped block).
cudaError_t launch_coef_component(cudaStream_t st, float *coef, float *dense, int k,
                                  long long sx, long long sy, long long sz, long long pitch,
                                  long long count, bool to_grouped);
// The ten dense coefficient arrays (dc_precomp_vars order, x fastest, no
// pitch) -> grouped pitched coefficients in one pass; the sources may be any
// memory the device can read (device, pinned host, or pageable host on
// systems whose GPU uses the host page tables).
struct CoefSources {
  const float *p[10];
};
cudaError_t launch_coef_gather(cudaStream_t st, float *coef, const CoefSources &src,
                               long long sx, long long sy, long long sz, long long pitch,
                               long long count);
// max |v2px|, |v2pz|, |v2sz|, |v2pn| as float bits, atomically into *out.
cudaError_t launch_coef_vmax(cudaStream_t st, const float *coef, long long count,
                             unsigned int *out);
// Grouped dense (count_d = n) -> grouped pitched.
cudaError_t launch_coef_repitch(cudaStream_t st, float *coef, const float *grouped_dense,
                                long long sx, long long sy, long long sz, long long pitch,
                                long long count);
// FP32 grouped -> BF16 copy (form CF_BF16) with velocity terms scaled by
// 2^-vexp.
cudaError_t launch_coef_narrow(cudaStream_t st, const float *coef, void *coef16, int form,
                               int vexp, long long count);
// FP32 grouped -> the CF_F16 copy (fixed-point angle terms, FP16 velocity
// ratios) and its per-row velocity bases vbase[sz * sy] (rows of sx points
// at the given pitch).
cudaError_t launch_coef_rowref(cudaStream_t st, const float *coef, void *coef16, float4 *vbase,
                               long long sx, long long sy, long long sz, long long pitch,
                               long long count);
cudaError_t launch_layered(cudaStream_t st, const dc_gb300_layered_spec &spec,
                           float *coef, float *vv, long long sx, long long sy,
                           long long sz, long long pitch, long long count);

// The reference's one-rank medium (default anisotropy, random velocity
// boundary with the glibc rand_r sequence, trig precompute) generated on the
// GPU.  consts: frac, max_p, max_s, default vsv, theta, phi -- computed on the
// host exactly as the reference's C computes them.
cudaError_t launch_reference_medium(cudaStream_t st, const int n[3], int absorb,
                                    unsigned int seed, const float consts[6], float *coef,
                                    float *vv, long long pitch, long long count);

// Tensor-map encoding through the driver entry point (no -lcuda needed).
bool encode_tiled(CUtensorMap *map, const void *base, int rank,
                  const uint64_t *dims, const uint64_t *strides_bytes,
                  const uint32_t *box, std::string *err,
                  CUtensorMapDataType type = CU_TENSOR_MAP_DATA_TYPE_FLOAT32);

// Learned absorbing layer (dc_learned.cu).  Layer cells of a box with a
// layer of `layer` cells: {x, y, z, axis | side << 2 | depth << 3}.
std::vector<int4> layer_cells(long long sx, long long sy, long long sz, int layer);
// The corrected cells split into face lines (corrected in one fused pass,
// in place) and edge cells (network into a correction buffer, then added).
struct LayerPlan {
  std::vector<int4> lines;  // outermost cell of each face line, meta = axis | side << 2
  std::vector<int4> edge;   // layer_cells entries
};
LayerPlan layer_plan(long long sx, long long sy, long long sz, int layer);
// Corrections of every layer cell from the new (t+1) and current (t)
// fields, then added to the new field.
// `rec` (may be null) also receives every cell's features (sample rows).
cudaError_t launch_lb_step(cudaStream_t st, const float *params, const int4 *cells, long long n,
                           float2 *nw, const float2 *cur, long long pitch, long long plane,
                           float2 *corr, float *rec);
// Rollout targets from recorded rows: wide (at `off`) minus features 0 / 8.
cudaError_t launch_lb_target(cudaStream_t st, const int4 *cells, long long n, const float *rows,
                             const float2 *wide, long long wpitch, long long wplane,
                             const int off[3], float *ts);
// Training samples ([n][33] features + depth, [n][2] targets) of a thin box
// stepped from a crop of a wide box at `off`.
cudaError_t launch_lb_sample(cudaStream_t st, const int4 *cells, long long n, const float2 *nw,
                             const float2 *cur, long long pitch, long long plane,
                             const float2 *wide, long long wpitch, long long wplane,
                             const int off[3], float *xs, float *ts);
// Learned layer over a batch: cells carry their shot in meta bits 8..31.
struct LbShot {
  float2 *pq[2];              // the shot's pair buffers
  long long pitch, plane;
};
cudaError_t launch_lb_batch_step(cudaStream_t st, const float *params, const int4 *cells,
                                 long long n, const LbShot *shots, int cur_buf, float2 *corr);
// The in-step correction through the face lines and the edge cells.
// Bit-identical to launch_lb_step over all corrected cells.
cudaError_t launch_lb_fused(cudaStream_t st, const float *params, int layer, const int4 *lines,
                            long long nl, const int4 *edge, long long ne, float2 *nw,
                            const float2 *cur, long long pitch, long long plane, float2 *corr);
cudaError_t launch_lb_batch_fused(cudaStream_t st, const float *params, int layer,
                                  const int4 *lines, long long nl, const int4 *edge, long long ne,
                                  const LbShot *shots, int cur_buf, float2 *corr);
// Thin pair buffer <- box of a wide pair buffer at `off`, zero halo.
cudaError_t launch_crop(cudaStream_t st, float2 *dst, long long sx, long long sy, long long sz,
                        long long pitch, const float2 *src, long long wpitch, long long wplane,
                        const int off[3]);

// FD weights, inverse spacings, dt and dt^2 of a pass (the vexp scaling of
// the narrow medium forms is applied by the caller).
void fill_weights(StepParams *p, float dx, float dy, float dz, float dt);

// Thread-local error text for dc_gb300_last_error().
void set_error(const std::string &msg);

}  // namespace dcg

// The simulation handle.  `abi` must stay the first member: the reference
// ABI hands out &handle->abi and dc_gb300_from_device_data() casts back.
struct dc_gb300_sim {
  dc_device_data abi;
  dcg::Sim *impl;
};
