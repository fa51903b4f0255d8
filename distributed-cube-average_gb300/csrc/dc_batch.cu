// dc_batch.cu -- many shots over one shared medium, advanced together.
//
// A batch holds one medium box (the model plus room for every shot's
// absorbing layer and halo) and any number of shots.  Each shot is a box
// cropped out of the medium at (ox, oy, oz) with its own (p, q) wavefields,
// source wavelet, sponge and receivers.  One step of all shots is one launch
// of the persistent batch kernel per group of up to kMaxBatchShots shots;
// steps are captured into CUDA graphs of kGraphSteps steps.  Tile rows (TY)
// and the z-split of each column are chosen by dc_gb300_batch_autotune,
// which times every candidate on the batch itself.
//
// The reference has no batched form: its one time loop (src/worker.c:466-511)
// advances one shot.  Each shot here follows that loop exactly as a
// dc_gb300_sim with the fast kernel does (the same sweep code and
// arithmetic), so a shot's fields are bit-identical to those of a
// single-shot simulation over the same cropped medium.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "dc_internal.h"

namespace dcg {
namespace {

constexpr int kGraphSteps = 32;  // steps per captured graph (even)

struct BShot {
  dc_gb300_shot cfg;
  long long pitch = 0, plane = 0, count = 0;
  float2 *pq[2] = {nullptr, nullptr};
  long long src_gi = 0;              // pitched index of the source
  std::vector<float> sponge;         // gx | gy | gz
  std::vector<float> src;            // wavelet, max_steps + 1 samples
  std::vector<int2> rec_col;         // [sy][sx] (empty: no receivers)
  std::vector<int> rec_z, rec_r;
  int nrec = 0;
};

struct Batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  long long mx = 0, my = 0, mz = 0, mpitch = 0, mplane = 0, mcount = 0;
  float dx = 0, dy = 0, dz = 0, dt = 0;
  int medium = DC_GB300_MEDIUM_PRECOMP;
  int coef_form = CF_F32;
  int vexp = 0;
  bool medium_set = false, narrow_stale = true;
  float *coef = nullptr;   // grouped FP32 coefficients of the medium box
  void *coef16 = nullptr;  // FP16/BF16 copy (narrow forms)
  float4 *vbase = nullptr; // FP16 form: velocity bases per medium row
  int max_steps = 0;
  std::vector<BShot> shots;
  // device tables (rebuilt by prepare)
  CUtensorMap *d_maps = nullptr;
  int *d_order = nullptr;          // work items in medium order, all groups
  float *d_sponge = nullptr, *d_src = nullptr, *d_src_pre = nullptr, *d_traces = nullptr;
  int2 *d_rec_col = nullptr;
  int *d_rec_z = nullptr, *d_rec_r = nullptr;
  std::vector<long long> trace_off;  // per shot, in floats
  int *d_step = nullptr, *d_err = nullptr;
  std::vector<BatchLaunch> groups;   // one launch per group of shots
  int blocks = 0;
  bool prepared = false;
  int ty = 8, zsplit = 1;
  bool persistent = true;  // persistent CTAs, or one CTA per work item
  bool sponge = true;      // some shot's sponge profile differs from 1
  int steps_done = 0;
  int src_applied_step = -1;
  long launches = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  // learned thin layer on every shot (after each step's stencil launches)
  const float *lb_params = nullptr;
  int lb_layer = 0;
  // With the layer, the shots split into two halves, each its own chain of
  // launches in the step graph (stencil, then its layer), so one half's
  // network overlaps the other half's stencil.
  struct LbBranch {
    int4 *d_lines = nullptr;   // face lines (meta bits 8..31: the shot)
    int4 *d_edge = nullptr;    // edge cells
    float2 *d_corr = nullptr;  // edge-cell corrections
    long long nl = 0, ne = 0;
  } lb[2];
  LbShot *d_lb_shots = nullptr;
  long long lb_cells = 0;      // corrected cells in all (0: no layer)
  int nbranch = 1;             // launch chains per step (2 with the layer and >= 2 shots)
  std::vector<int> group_first, group_branch;  // per launch group: first shot, chain
  cudaStream_t side = nullptr;                 // the second chain's stream
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

// Learned-layer launches of one step: the face-line pass, then the edge
// cells' network and add.
long lb_launches(const Batch *b) {
  if (b->lb_cells <= 0) return 0;
  long n = 0;
  for (int br = 0; br < b->nbranch; ++br)
    n += (b->lb[br].nl > 0 ? 1 : 0) + (b->lb[br].ne > 0 ? 2 : 0);
  return n;
}

// The launch chain of shot k.
int branch_of(const Batch *b, size_t k) {
  return b->nbranch == 2 && k >= (b->shots.size() + 1) / 2 ? 1 : 0;
}

void free_layer(Batch *b) {
  for (auto &l : b->lb) {
    cudaFree(l.d_lines);
    cudaFree(l.d_edge);
    cudaFree(l.d_corr);
    l = Batch::LbBranch{};
  }
  cudaFree(b->d_lb_shots);
  b->d_lb_shots = nullptr;
  b->lb_cells = 0;
  b->nbranch = 1;
}

int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

#define BATCH_TRY(call)                                                              \
  do {                                                                               \
    const cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                           \
      return fail(DC_GB300_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

Batch *impl(dc_gb300_batch *b);

void drop_graphs(Batch *b) {
  for (auto &g : b->graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

void free_tables(Batch *b) {
  cudaFree(b->d_maps);
  cudaFree(b->d_order);
  b->d_order = nullptr;
  cudaFree(b->d_sponge);
  cudaFree(b->d_src);
  cudaFree(b->d_src_pre);
  cudaFree(b->d_traces);
  cudaFree(b->d_rec_col);
  cudaFree(b->d_rec_z);
  cudaFree(b->d_rec_r);
  b->d_maps = nullptr;
  b->d_sponge = b->d_src = b->d_src_pre = b->d_traces = nullptr;
  b->d_rec_col = nullptr;
  b->d_rec_z = b->d_rec_r = nullptr;
  b->prepared = false;
  drop_graphs(b);
}

void release(Batch *b) {
  drop_graphs(b);
  free_tables(b);
  for (auto &s : b->shots) {
    cudaFree(s.pq[0]);
    cudaFree(s.pq[1]);
  }
  free_layer(b);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->side) cudaStreamDestroy(b->side);
  cudaFree(b->coef);
  cudaFree(b->coef16);
  cudaFree(b->vbase);
  cudaFree(b->d_step);
  cudaFree(b->d_err);
  if (b->stream) cudaStreamDestroy(b->stream);
}

// The 16-bit copy of the medium (the same encodings as a single-shot
// simulation): FP16 with per-row velocity bases, or BF16 with the velocity
// terms scaled by 2^-vexp.
int refresh_narrow(Batch *b) {
  if (!(b->coef_form == CF_F16 || b->coef_form == CF_BF16) || !b->narrow_stale)
    return DC_GB300_OK;
  if (b->coef_form == CF_F16) {
    BATCH_TRY(launch_coef_rowref(b->stream, b->coef, b->coef16, b->vbase, b->mx, b->my, b->mz,
                                 b->mpitch, b->mcount));
    BATCH_TRY(cudaStreamSynchronize(b->stream));
    b->vexp = 0;
    b->narrow_stale = false;
    b->prepared = false;
    drop_graphs(b);
    return DC_GB300_OK;
  }
  unsigned int *d_max = nullptr;
  unsigned int bits = 0;
  BATCH_TRY(cudaMalloc(&d_max, sizeof(unsigned int)));
  BATCH_TRY(cudaMemsetAsync(d_max, 0, sizeof(unsigned int), b->stream));
  BATCH_TRY(launch_coef_vmax(b->stream, b->coef, b->mcount, d_max));
  BATCH_TRY(cudaMemcpyAsync(&bits, d_max, sizeof(bits), cudaMemcpyDeviceToHost, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  cudaFree(d_max);
  float vmax;
  std::memcpy(&vmax, &bits, sizeof(vmax));
  int e = 0;
  if (vmax > 0.0f && std::isfinite(vmax)) {
    std::frexp(vmax, &e);
    e -= 14;
  }
  b->vexp = e;
  BATCH_TRY(launch_coef_narrow(b->stream, b->coef, b->coef16, b->coef_form, b->vexp, b->mcount));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  b->narrow_stale = false;
  b->prepared = false;
  drop_graphs(b);
  return DC_GB300_OK;
}

// Builds the device tables and the launch parameters for tile rows `ty`
// and `zsplit` z-chunks per column.
int prepare(Batch *b, int ty, int zsplit, bool persistent) {
  if (!b->medium_set) return fail(DC_GB300_ERR_STATE, "batch medium not set");
  if (b->shots.empty()) return fail(DC_GB300_ERR_STATE, "batch has no shots");
  int rc = refresh_narrow(b);
  if (rc != DC_GB300_OK) return rc;
  free_tables(b);
  b->ty = ty;
  b->zsplit = zsplit;
  b->persistent = persistent;
  const int n = static_cast<int>(b->shots.size());
  std::string err;
  CUtensorMap tm_c[4];
  if (!fast_encode_medium_maps(b->coef_form, b->coef, b->coef16, nullptr, b->vbase, b->mx,
                               b->my, b->mz, b->mpitch, b->mcount, ty, tm_c, &err))
    return fail(DC_GB300_ERR_CUDA, err);
  std::vector<CUtensorMap> maps(static_cast<size_t>(n) * 4);
  for (int i = 0; i < n; ++i) {
    const BShot &s = b->shots[i];
    for (int buf = 0; buf < 2; ++buf)
      if (!fast_encode_pair_maps(s.pq[buf], s.cfg.sx, s.cfg.sy, s.cfg.sz, s.pitch, ty,
                                 &maps[4 * i + buf], &maps[4 * i + 2 + buf], &err))
        return fail(DC_GB300_ERR_CUDA, err);
  }
  // concatenated host tables
  std::vector<float> sponge, src;
  std::vector<long long> sponge_off(n), src_off(n), col_off(n), rec_off(n);
  std::vector<int2> cols;
  std::vector<int> rz, rr;
  b->trace_off.assign(n, 0);
  long long traces = 0;
  for (int i = 0; i < n; ++i) {
    const BShot &s = b->shots[i];
    sponge_off[i] = static_cast<long long>(sponge.size());
    sponge.insert(sponge.end(), s.sponge.begin(), s.sponge.end());
    src_off[i] = static_cast<long long>(src.size());
    src.insert(src.end(), s.src.begin(), s.src.end());
    col_off[i] = static_cast<long long>(cols.size());
    rec_off[i] = static_cast<long long>(rz.size());
    if (s.nrec > 0) {
      cols.insert(cols.end(), s.rec_col.begin(), s.rec_col.end());
      rz.insert(rz.end(), s.rec_z.begin(), s.rec_z.end());
      rr.insert(rr.end(), s.rec_r.begin(), s.rec_r.end());
    }
    b->trace_off[i] = traces;
    traces += static_cast<long long>(s.nrec) * b->max_steps;
  }
  BATCH_TRY(cudaMalloc(&b->d_maps, sizeof(CUtensorMap) * maps.size()));
  BATCH_TRY(cudaMemcpyAsync(b->d_maps, maps.data(), sizeof(CUtensorMap) * maps.size(),
                            cudaMemcpyHostToDevice, b->stream));
  BATCH_TRY(cudaMalloc(&b->d_sponge, sizeof(float) * sponge.size()));
  BATCH_TRY(cudaMemcpyAsync(b->d_sponge, sponge.data(), sizeof(float) * sponge.size(),
                            cudaMemcpyHostToDevice, b->stream));
  BATCH_TRY(cudaMalloc(&b->d_src, sizeof(float) * src.size()));
  BATCH_TRY(cudaMemcpyAsync(b->d_src, src.data(), sizeof(float) * src.size(),
                            cudaMemcpyHostToDevice, b->stream));
  BATCH_TRY(cudaMalloc(&b->d_src_pre, sizeof(float) * 2 * n));
  BATCH_TRY(cudaMemsetAsync(b->d_src_pre, 0, sizeof(float) * 2 * n, b->stream));
  if (!cols.empty()) {
    BATCH_TRY(cudaMalloc(&b->d_rec_col, sizeof(int2) * cols.size()));
    BATCH_TRY(cudaMemcpyAsync(b->d_rec_col, cols.data(), sizeof(int2) * cols.size(),
                              cudaMemcpyHostToDevice, b->stream));
    BATCH_TRY(cudaMalloc(&b->d_rec_z, sizeof(int) * rz.size()));
    BATCH_TRY(cudaMemcpyAsync(b->d_rec_z, rz.data(), sizeof(int) * rz.size(),
                              cudaMemcpyHostToDevice, b->stream));
    BATCH_TRY(cudaMalloc(&b->d_rec_r, sizeof(int) * rr.size()));
    BATCH_TRY(cudaMemcpyAsync(b->d_rec_r, rr.data(), sizeof(int) * rr.size(),
                              cudaMemcpyHostToDevice, b->stream));
  }
  if (traces > 0) {
    BATCH_TRY(cudaMalloc(&b->d_traces, sizeof(float) * traces));
    BATCH_TRY(cudaMemsetAsync(b->d_traces, 0, sizeof(float) * traces, b->stream));
  }
  // launch parameters, one group per kMaxBatchShots shots
  StepParams common{};
  fill_weights(&common, b->dx, b->dy, b->dz, b->dt);
  if (b->coef_form == CF_BF16) {
    common.dt2 = ldexpf(common.dt2, b->vexp);
    common.dt2_iso = ldexpf(common.dt2_iso, b->vexp);
  }
  b->groups.clear();
  b->group_first.clear();
  b->group_branch.clear();
  long long max_items = 0;
  // launch groups of up to kMaxBatchShots shots, never spanning two chains
  std::vector<std::pair<int, int>> spans;  // [first, last) shots
  for (int br = 0; br < b->nbranch; ++br) {
    int lo = 0, hi = n;
    if (b->nbranch == 2) {
      lo = br == 0 ? 0 : (n + 1) / 2;
      hi = br == 0 ? (n + 1) / 2 : n;
    }
    for (int g0 = lo; g0 < hi; g0 += kMaxBatchShots) {
      spans.emplace_back(g0, std::min(hi, g0 + kMaxBatchShots));
      b->group_branch.push_back(br);
    }
  }
  for (const auto &span : spans) {
    const int g0 = span.first;
    BatchLaunch bl;
    std::memset(&bl, 0, sizeof(bl));
    bl.tm_l = tm_c[0];
    bl.tm_o1 = tm_c[1];
    bl.tm_o2 = tm_c[2];
    bl.tm_vb = tm_c[3];
    bl.maps = b->d_maps + 4 * g0;
    bl.nshots = span.second - g0;
    b->group_first.push_back(g0);
    bl.err = b->d_err;
    long long items = 0;
    for (int k = 0; k < bl.nshots; ++k) {
      const int i = g0 + k;
      const BShot &s = b->shots[i];
      StepParams p = common;
      p.x0 = p.y0 = p.z0 = 4;
      p.x1 = static_cast<int>(s.cfg.sx - 4);
      p.y1 = static_cast<int>(s.cfg.sy - 4);
      p.z1 = static_cast<int>(s.cfg.sz - 4);
      p.tile_x0 = 4;
      p.tile_y0 = 4;
      const int nzc = p.z1 - p.z0;
      p.zchunk = (nzc + zsplit - 1) / zsplit;
      p.pitch = s.pitch;
      p.plane = s.plane;
      p.count = s.count;
      p.sponge = b->d_sponge + sponge_off[i];
      p.sponge_oy = static_cast<int>(s.cfg.sx);
      p.sponge_oz = static_cast<int>(s.cfg.sx + s.cfg.sy);
      p.src_x = static_cast<int>(s.cfg.src_x);
      p.src_y = static_cast<int>(s.cfg.src_y);
      p.src_z = static_cast<int>(s.cfg.src_z);
      p.src_table = b->d_src + src_off[i];
      p.src_count = b->max_steps + 1;
      p.d_step = b->d_step;
      p.src_pre = b->d_src_pre + 2 * i;
      if (s.nrec > 0) {
        p.rec_col = b->d_rec_col + col_off[i];
        p.rec_z = b->d_rec_z + rec_off[i];
        p.rec_r = b->d_rec_r + rec_off[i];
        p.traces = b->d_traces + b->trace_off[i];
        p.nrec = s.nrec;
        p.trace_cap = b->max_steps;
        p.col_stride = static_cast<int>(s.cfg.sx);
      }
      p.err = b->d_err;
      p.mox = static_cast<int>(s.cfg.ox);
      p.moy = static_cast<int>(s.cfg.oy);
      p.moz = static_cast<int>(s.cfg.oz);
      bl.shot[k] = p;
      bl.tiles_x[k] = (p.x1 - p.tile_x0 + 31) / 32;
      bl.tiles_y[k] = (p.y1 - p.tile_y0 + ty - 1) / ty;
      bl.item_prefix[k] = static_cast<int>(items);
      items += static_cast<long long>(bl.tiles_x[k]) * bl.tiles_y[k] *
               ((nzc + p.zchunk - 1) / p.zchunk);
    }
    if (items > (1ll << 30)) return fail(DC_GB300_ERR_ARG, "too many work items in a launch");
    bl.item_prefix[bl.nshots] = static_cast<int>(items);
    bl.n_items = static_cast<int>(items);
    max_items = std::max(max_items, items);
    b->groups.push_back(bl);
  }
  // Launch order: the crops overlap in the shared medium, so the items are
  // sorted by their medium position (z-chunk, tile row, tile column, then
  // shot).  CTAs that run together then read the same medium columns and
  // all but the first find them in L2.  Every item writes its own outputs,
  // so the order changes no result.
  std::vector<int> order;
  std::vector<size_t> group_off;
  for (const BatchLaunch &bl : b->groups) {
    group_off.push_back(order.size());
    struct Key {
      long long z, y, x;
      int s, item;
    };
    std::vector<Key> keys;
    keys.reserve(static_cast<size_t>(bl.n_items));
    for (int s = 0; s < bl.nshots; ++s) {
      const StepParams &p = bl.shot[s];
      for (int local = 0; local < bl.item_prefix[s + 1] - bl.item_prefix[s]; ++local) {
        const int ix = local % bl.tiles_x[s];
        const int iy = (local / bl.tiles_x[s]) % bl.tiles_y[s];
        const int iz = local / (bl.tiles_x[s] * bl.tiles_y[s]);
        const long long mx = p.mox + p.tile_x0 + 32ll * ix, my = p.moy + p.tile_y0 + ty * iy;
        const long long mz = p.moz + p.z0 + static_cast<long long>(iz) * p.zchunk;
        keys.push_back(Key{mz / std::max(1, p.zchunk), my / ty, mx / 32, s,
                           bl.item_prefix[s] + local});
      }
    }
    std::stable_sort(keys.begin(), keys.end(), [](const Key &a, const Key &c) {
      if (a.z != c.z) return a.z < c.z;
      if (a.y != c.y) return a.y < c.y;
      if (a.x != c.x) return a.x < c.x;
      return a.s < c.s;
    });
    for (const Key &k : keys) order.push_back(k.item);
  }
  BATCH_TRY(cudaMalloc(&b->d_order, sizeof(int) * std::max<size_t>(order.size(), 1)));
  BATCH_TRY(cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * order.size(),
                            cudaMemcpyHostToDevice, b->stream));
  for (size_t g = 0; g < b->groups.size(); ++g) b->groups[g].order = b->d_order + group_off[g];
  b->sponge = std::any_of(sponge.begin(), sponge.end(), [](float g) { return g != 1.0f; });
  BATCH_TRY(batch_prepare(ty, b->coef_form));
  const bool iso = b->dx == b->dy && b->dy == b->dz;
  const int per_sm = batch_blocks_per_sm(ty, b->coef_form, iso, b->sponge);
  if (per_sm < 1) return fail(DC_GB300_ERR_CUDA, "batch kernel does not fit an SM");
  int sms = 0;
  BATCH_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
  b->blocks = static_cast<int>(std::min<long long>(max_items, static_cast<long long>(sms) * per_sm));
  if (!b->persistent) b->blocks = static_cast<int>(max_items);  // one CTA per work item
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  b->prepared = true;
  return DC_GB300_OK;
}

// Queues one step of every shot with (pc, qc) in buffer `cur`, the j-th
// step of a sequence (step = *d_step + j).
// Queues one step of the shots of chain `br` on stream `st`.
cudaError_t queue_chain(Batch *b, int cur, int j, int br, cudaStream_t st) {
  const bool iso = b->dx == b->dy && b->dy == b->dz;
  for (size_t g = 0; g < b->groups.size(); ++g) {
    if (b->group_branch[g] != br) continue;
    BatchLaunch &bl = b->groups[g];
    bl.cur_buf = cur;
    for (int k = 0; k < bl.nshots; ++k) {
      bl.shot[k].step_offset = j;
      bl.shot[k].prev = b->shots[b->group_first[g] + k].pq[1 - cur];  // written in place
    }
    ++b->launches;
    const cudaError_t e = launch_batch(st, bl, b->ty, b->coef_form, iso, b->sponge, b->blocks);
    if (e != cudaSuccess) return e;
  }
  if (b->lb_cells > 0) {  // the chain's learned layers, after its stencil launches
    const Batch::LbBranch &l = b->lb[br];
    b->launches += (l.nl > 0 ? 1 : 0) + (l.ne > 0 ? 2 : 0);
    return launch_lb_batch_fused(st, b->lb_params, b->lb_layer, l.d_lines, l.nl, l.d_edge, l.ne,
                                 b->d_lb_shots, cur, l.d_corr);
  }
  return cudaSuccess;
}

// Queues `steps` steps, the first with (pc, qc) in buffer `cur0`: with two
// chains the side stream forks from the batch stream and joins it again at
// the end.
cudaError_t queue_steps(Batch *b, int cur0, int steps) {
  if (b->nbranch == 1) {
    for (int j = 0; j < steps; ++j) {
      const cudaError_t e = queue_chain(b, (cur0 + j) & 1, j, 0, b->stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  cudaError_t e = cudaEventRecord(b->ev_fork, b->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(b->side, b->ev_fork, 0);
  for (int j = 0; j < steps && e == cudaSuccess; ++j) {
    e = queue_chain(b, (cur0 + j) & 1, j, 0, b->stream);
    if (e == cudaSuccess) e = queue_chain(b, (cur0 + j) & 1, j, 1, b->side);
  }
  if (e == cudaSuccess) e = cudaEventRecord(b->ev_join, b->side);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->ev_join, 0);
  return e;
}

bool source_pending(const Batch *b) {
  return b->steps_done > 0 && b->src_applied_step == b->steps_done;
}

int check_err(Batch *b) {
  int h = 0;
  BATCH_TRY(cudaMemcpyAsync(&h, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  if (h) cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream);
  if (h & kErrTimeout) return fail(DC_GB300_ERR_TIMEOUT, "a TMA wait in the batch kernel timed out");
  if (h & kErrAlign) return fail(DC_GB300_ERR_CUDA, "shared-memory window not 128-byte aligned");
  return DC_GB300_OK;
}

// Runs `steps` steps: the first source injection, graphs of kGraphSteps
// steps, then single launches.
int run_steps(Batch *b, int steps) {
  if (!b->prepared) {
    const int rc = prepare(b, b->ty, b->zsplit, b->persistent);
    if (rc != DC_GB300_OK) return rc;
  }
  if (b->steps_done + steps > b->max_steps)
    return fail(DC_GB300_ERR_ARG, "run exceeds the batch's max_steps");
  if (b->src_applied_step != b->steps_done) {
    const int cur = b->steps_done & 1;
    for (size_t i = 0; i < b->shots.size(); ++i) {
      ++b->launches;
      BATCH_TRY(launch_add_source(b->stream, b->shots[i].pq[cur], b->shots[i].src_gi,
                                  b->d_src + i * (b->max_steps + 1), b->max_steps + 1,
                                  b->d_step, 0));
    }
  }
  int left = steps;
  while (left >= kGraphSteps) {
    const int cur = b->steps_done & 1;
    if (!b->graph[cur]) {
      cudaGraph_t g = nullptr;
      BATCH_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      const long before = b->launches;
      cudaError_t e = cudaSuccess;
      e = queue_steps(b, cur, kGraphSteps);
      if (e == cudaSuccess) e = launch_advance_step(b->stream, b->d_step, kGraphSteps);
      const cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
      b->launches = before;
      if (e != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(DC_GB300_ERR_CUDA, std::string("batch graph capture: ") +
                                           cudaGetErrorString(e != cudaSuccess ? e : ee));
      }
      e = cudaGraphInstantiate(&b->graph[cur], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess)
        return fail(DC_GB300_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    BATCH_TRY(cudaGraphLaunch(b->graph[cur], b->stream));
    b->launches += static_cast<long>(kGraphSteps) *
                       (static_cast<long>(b->groups.size()) + lb_launches(b)) + 1;
    left -= kGraphSteps;
    b->steps_done += kGraphSteps;
  }
  if (left > 0) BATCH_TRY(queue_steps(b, b->steps_done & 1, left));
  if (left > 0) {
    ++b->launches;
    BATCH_TRY(launch_advance_step(b->stream, b->d_step, left));
    b->steps_done += left;
  }
  b->src_applied_step = b->steps_done;
  return DC_GB300_OK;
}

// Back to the state after dc_gb300_batch_add_shot: zero fields, step 0.
int reset_state(Batch *b) {
  for (auto &s : b->shots)
    for (auto *p : s.pq) BATCH_TRY(cudaMemsetAsync(p, 0, sizeof(float2) * s.count, b->stream));
  BATCH_TRY(cudaMemsetAsync(b->d_step, 0, sizeof(int), b->stream));
  long long traces = 0;
  for (auto &s : b->shots) traces += static_cast<long long>(s.nrec) * b->max_steps;
  if (b->d_traces && traces > 0)
    BATCH_TRY(cudaMemsetAsync(b->d_traces, 0, sizeof(float) * traces, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  b->steps_done = 0;
  b->src_applied_step = -1;
  return DC_GB300_OK;
}

}  // namespace
}  // namespace dcg

struct dc_gb300_batch {
  dcg::Batch impl;
};

namespace dcg {
namespace {
Batch *impl(dc_gb300_batch *b) { return b ? &b->impl : nullptr; }
}  // namespace
}  // namespace dcg

using dcg::Batch;
using dcg::fail;

extern "C" int dc_gb300_batch_create(const dc_gb300_batch_config *cfg, dc_gb300_batch **out) {
  if (!cfg || !out) return fail(DC_GB300_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->mx < 9 || cfg->my < 9 || cfg->mz < 9 || cfg->mx > (1 << 30) || cfg->my > (1 << 30) ||
      cfg->mz > (1 << 30))
    return fail(DC_GB300_ERR_ARG, "medium sizes must lie in [9, 2^30]");
  if (!(cfg->dx > 0 && cfg->dy > 0 && cfg->dz > 0 && cfg->dt > 0))
    return fail(DC_GB300_ERR_ARG, "dx, dy, dz and dt must be positive");
  if (cfg->medium != DC_GB300_MEDIUM_PRECOMP && cfg->medium != DC_GB300_MEDIUM_PRECOMP_F16 &&
      cfg->medium != DC_GB300_MEDIUM_PRECOMP_BF16)
    return fail(DC_GB300_ERR_ARG, "batch medium must be PRECOMP, PRECOMP_F16 or PRECOMP_BF16");
  if (cfg->max_steps < 1) return fail(DC_GB300_ERR_ARG, "max_steps must be positive");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(DC_GB300_ERR_DEVICE, "no CUDA device");
  int dev = cfg->device;
  if (dev < 0) BATCH_TRY(cudaGetDevice(&dev));
  if (dev >= ndev) return fail(DC_GB300_ERR_DEVICE, "device ordinal out of range");
  cudaDeviceProp prop;
  BATCH_TRY(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3)
    return fail(DC_GB300_ERR_DEVICE, std::string("this build targets sm_103a; device is ") + prop.name);
  BATCH_TRY(cudaSetDevice(dev));
  auto *h = new dc_gb300_batch();
  Batch *b = &h->impl;
  b->device = dev;
  b->mx = cfg->mx;
  b->my = cfg->my;
  b->mz = cfg->mz;
  b->mpitch = (cfg->mx + 3) / 4 * 4;
  b->mplane = b->mpitch * cfg->my;
  b->mcount = b->mplane * cfg->mz;
  b->dx = cfg->dx;
  b->dy = cfg->dy;
  b->dz = cfg->dz;
  b->dt = cfg->dt;
  b->medium = cfg->medium;
  b->coef_form = cfg->medium == DC_GB300_MEDIUM_PRECOMP_F16    ? dcg::CF_F16
                 : cfg->medium == DC_GB300_MEDIUM_PRECOMP_BF16 ? dcg::CF_BF16
                                                               : dcg::CF_F32;
  b->max_steps = cfg->max_steps;
  b->ty = dcg::fast_default_ty(b->coef_form);
  auto bail = [&](int code, const std::string &msg) {
    dcg::release(b);
    delete h;
    return fail(code, msg);
  };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(DC_GB300_ERR_CUDA, "cudaStreamCreate");
  if (cudaMalloc(&b->coef, sizeof(float) * 10 * b->mcount) != cudaSuccess)
    return bail(DC_GB300_ERR_NOMEM, "medium coefficients");
  if (b->coef_form != dcg::CF_F32 && cudaMalloc(&b->coef16, 20 * b->mcount) != cudaSuccess)
    return bail(DC_GB300_ERR_NOMEM, "narrow medium copy");
  if (b->coef_form == dcg::CF_F16 &&
      cudaMalloc(&b->vbase, sizeof(float4) * b->my * b->mz) != cudaSuccess)
    return bail(DC_GB300_ERR_NOMEM, "velocity bases");
  if (cudaMalloc(&b->d_step, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&b->d_err, sizeof(int)) != cudaSuccess)
    return bail(DC_GB300_ERR_NOMEM, "counters");
  cudaMemsetAsync(b->coef, 0, sizeof(float) * 10 * b->mcount, b->stream);
  cudaMemsetAsync(b->d_step, 0, sizeof(int), b->stream);
  cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream);
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bail(DC_GB300_ERR_CUDA, "set-up");
  *out = h;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_destroy(dc_gb300_batch *h) {
  if (!h) return DC_GB300_OK;
  cudaSetDevice(h->impl.device);
  dcg::release(&h->impl);
  delete h;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_generate_layered(dc_gb300_batch *h,
                                               const dc_gb300_layered_spec *spec) {
  Batch *b = dcg::impl(h);
  if (!b || !spec) return fail(DC_GB300_ERR_ARG, "null argument");
  if (spec->nlayers < 1 || spec->nlayers > DC_GB300_MAX_LAYERS || spec->n_noise < 0 ||
      spec->n_noise > DC_GB300_MAX_FEATURES || spec->n_theta < 0 ||
      spec->n_theta > DC_GB300_MAX_FEATURES || spec->n_phi < 0 ||
      spec->n_phi > DC_GB300_MAX_FEATURES || !(spec->sigma_ratio > 0))
    return fail(DC_GB300_ERR_ARG, "invalid layered-medium spec");
  BATCH_TRY(cudaSetDevice(b->device));
  ++b->launches;
  BATCH_TRY(dcg::launch_layered(b->stream, *spec, b->coef, nullptr, b->mx, b->my, b->mz,
                                b->mpitch, b->mcount));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  b->medium_set = true;
  b->narrow_stale = true;
  b->prepared = false;
  dcg::drop_graphs(b);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_set_precomp(dc_gb300_batch *h, const dc_precomp_vars *v) {
  Batch *b = dcg::impl(h);
  if (!b || !v) return fail(DC_GB300_ERR_ARG, "null argument");
  const float *f[10] = {v->ch1dxx, v->ch1dyy, v->ch1dzz, v->ch1dxy, v->ch1dyz,
                        v->ch1dxz, v->v2px,   v->v2pz,   v->v2sz,   v->v2pn};
  for (const float *p : f)
    if (!p) return fail(DC_GB300_ERR_ARG, "null coefficient array");
  BATCH_TRY(cudaSetDevice(b->device));
  const long long n = b->mx * b->my * b->mz;
  float *dense = nullptr;
  BATCH_TRY(cudaMalloc(&dense, sizeof(float) * n));
  for (int k = 0; k < 10; ++k) {
    cudaError_t e = cudaMemcpyAsync(dense, f[k], sizeof(float) * n, cudaMemcpyHostToDevice,
                                    b->stream);
    if (e == cudaSuccess)
      e = dcg::launch_coef_component(b->stream, b->coef, dense, dcg::kRefToDev[k], b->mx, b->my,
                                     b->mz, b->mpitch, b->mcount, true);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
      cudaFree(dense);
      return fail(DC_GB300_ERR_CUDA, std::string("batch medium upload: ") + cudaGetErrorString(e));
    }
  }
  cudaFree(dense);
  b->launches += 10;
  b->medium_set = true;
  b->narrow_stale = true;
  b->prepared = false;
  dcg::drop_graphs(b);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_add_shot(dc_gb300_batch *h, const dc_gb300_shot *shot, int *index) {
  Batch *b = dcg::impl(h);
  if (!b || !shot) return fail(DC_GB300_ERR_ARG, "null argument");
  if (b->lb_cells > 0)
    return fail(DC_GB300_ERR_STATE, "add every shot before setting the learned layer");
  const dc_gb300_shot &c = *shot;
  if (c.sx < 9 || c.sy < 9 || c.sz < 9)
    return fail(DC_GB300_ERR_ARG, "every padded shot size must be at least 9");
  if (c.ox < 0 || c.oy < 0 || c.oz < 0 || c.ox + c.sx > b->mx || c.oy + c.sy > b->my ||
      c.oz + c.sz > b->mz)
    return fail(DC_GB300_ERR_ARG, "the shot box must lie inside the medium box");
  if (c.ox % 4 != 0)
    return fail(DC_GB300_ERR_ARG, "shot ox must be a multiple of 4 (16-byte TMA coordinates)");
  if (c.src_x < 4 || c.src_x >= c.sx - 4 || c.src_y < 4 || c.src_y >= c.sy - 4 || c.src_z < 4 ||
      c.src_z >= c.sz - 4)
    return fail(DC_GB300_ERR_ARG, "the source must lie in the updated region [4, s-4)^3");
  if (!(c.fcut > 0)) return fail(DC_GB300_ERR_ARG, "fcut must be positive");
  if (c.absorb < 0 || 2 * c.absorb + 8 > std::min(c.sx, std::min(c.sy, c.sz)))
    return fail(DC_GB300_ERR_ARG, "absorbing width does not fit the shot box");
  BATCH_TRY(cudaSetDevice(b->device));
  dcg::BShot s;
  s.cfg = c;
  s.pitch = (c.sx + 3) / 4 * 4;
  s.plane = s.pitch * c.sy;
  s.count = s.plane * c.sz;
  s.src_gi = c.src_z * s.plane + c.src_y * s.pitch + c.src_x;
  for (auto &p : s.pq) {
    if (cudaMalloc(&p, sizeof(float2) * s.count) != cudaSuccess) {
      cudaFree(s.pq[0]);
      cudaFree(s.pq[1]);
      return fail(DC_GB300_ERR_NOMEM, "shot wavefields");
    }
    BATCH_TRY(cudaMemsetAsync(p, 0, sizeof(float2) * s.count, b->stream));
  }
  s.sponge.resize(c.sx + c.sy + c.sz);
  dc_gb300_sponge_profile(c.sx, c.absorb, c.kappa, s.sponge.data());
  dc_gb300_sponge_profile(c.sy, c.absorb, c.kappa, s.sponge.data() + c.sx);
  dc_gb300_sponge_profile(c.sz, c.absorb, c.kappa, s.sponge.data() + c.sx + c.sy);
  s.src.resize(b->max_steps + 1);
  for (int it = 0; it <= b->max_steps; ++it) s.src[it] = dc_gb300_source(b->dt, it, c.fcut);
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  b->shots.push_back(std::move(s));
  if (index) *index = static_cast<int>(b->shots.size()) - 1;

  b->prepared = false;
  dcg::drop_graphs(b);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_set_receivers(dc_gb300_batch *h, int shot, int count,
                                            const long *xyz) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  if (shot < 0 || shot >= static_cast<int>(b->shots.size()))
    return fail(DC_GB300_ERR_ARG, "shot index out of range");
  if (count < 0 || (count > 0 && !xyz)) return fail(DC_GB300_ERR_ARG, "receivers invalid");
  dcg::BShot &s = b->shots[shot];
  const long long sx = s.cfg.sx, sy = s.cfg.sy, sz = s.cfg.sz;
  struct Rec {
    long long col;
    int z, r;
  };
  std::vector<Rec> recs(count);
  for (int r = 0; r < count; ++r) {
    const long long x = xyz[3 * r], y = xyz[3 * r + 1], z = xyz[3 * r + 2];
    if (x < 4 || x >= sx - 4 || y < 4 || y >= sy - 4 || z < 4 || z >= sz - 4)
      return fail(DC_GB300_ERR_ARG, "receivers must lie in the updated region [4, s-4)^3");
    recs[r] = Rec{y * sx + x, static_cast<int>(z), r};
  }
  std::sort(recs.begin(), recs.end(), [](const Rec &a, const Rec &c) {
    return a.col != c.col ? a.col < c.col : (a.z != c.z ? a.z < c.z : a.r < c.r);
  });
  s.rec_col.assign(count > 0 ? static_cast<size_t>(sx * sy) : 0, make_int2(0, 0));
  s.rec_z.resize(count);
  s.rec_r.resize(count);
  for (int k = 0; k < count; ++k) {
    int2 &c = s.rec_col[recs[k].col];
    if (c.y == 0) c.x = k;
    ++c.y;
    s.rec_z[k] = recs[k].z;
    s.rec_r[k] = recs[k].r;
  }
  s.nrec = count;
  cudaSetDevice(b->device);
  dcg::free_tables(b);  // traces restart from zero
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_set_learned_layer(dc_gb300_batch *h, const dc_gb300_mlp *mlp,
                                                int layer) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  if (layer < 0 || layer > DC_GB300_MLP_DEPTHS)
    return fail(DC_GB300_ERR_ARG, "layer width must lie in [0, DC_GB300_MLP_DEPTHS]");
  if (layer > 0 && !mlp) return fail(DC_GB300_ERR_ARG, "null MLP");
  BATCH_TRY(cudaSetDevice(b->device));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  dcg::drop_graphs(b);
  dcg::free_layer(b);
  b->prepared = false;  // the launch groups follow the chains
  b->lb_layer = 0;
  b->lb_params = nullptr;
  if (layer == 0) return DC_GB300_OK;
  if (b->shots.size() > (1u << 23)) return fail(DC_GB300_ERR_ARG, "too many shots");
  if (b->shots.size() >= 2) {
    if (!b->side) BATCH_TRY(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
    if (!b->ev_fork) BATCH_TRY(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    if (!b->ev_join) BATCH_TRY(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming));
    b->nbranch = 2;
  }
  std::vector<int4> lines[2], edge[2];
  std::vector<dcg::LbShot> tab;
  long long total = 0;
  for (size_t k = 0; k < b->shots.size(); ++k) {
    const int br = dcg::branch_of(b, k);
    const dcg::BShot &s = b->shots[k];
    if (s.cfg.sx < 2 * layer + 16 || s.cfg.sy < 2 * layer + 16 || s.cfg.sz < 2 * layer + 16)
      return fail(DC_GB300_ERR_ARG, "every shot's interior must keep at least 8 cells per axis");
    const dcg::LayerPlan plan = dcg::layer_plan(s.cfg.sx, s.cfg.sy, s.cfg.sz, layer);
    for (int4 v : plan.lines) {
      v.w |= static_cast<int>(k) << 8;
      lines[br].push_back(v);
    }
    for (int4 v : plan.edge) {
      v.w |= static_cast<int>(k) << 8;
      edge[br].push_back(v);
    }
    total += static_cast<long long>(dcg::layer_cells(s.cfg.sx, s.cfg.sy, s.cfg.sz, layer).size());
    tab.push_back(dcg::LbShot{{s.pq[0], s.pq[1]}, s.pitch, s.plane});
  }
  for (int br = 0; br < b->nbranch; ++br) {
    Batch::LbBranch &l = b->lb[br];
    l.nl = static_cast<long long>(lines[br].size());
    l.ne = static_cast<long long>(edge[br].size());
    BATCH_TRY(cudaMalloc(&l.d_lines, sizeof(int4) * std::max(l.nl, 1LL)));
    BATCH_TRY(cudaMalloc(&l.d_edge, sizeof(int4) * std::max(l.ne, 1LL)));
    BATCH_TRY(cudaMalloc(&l.d_corr, sizeof(float2) * std::max(l.ne, 1LL)));
    if (l.nl > 0)
      BATCH_TRY(cudaMemcpyAsync(l.d_lines, lines[br].data(), sizeof(int4) * l.nl,
                                cudaMemcpyHostToDevice, b->stream));
    if (l.ne > 0)
      BATCH_TRY(cudaMemcpyAsync(l.d_edge, edge[br].data(), sizeof(int4) * l.ne,
                                cudaMemcpyHostToDevice, b->stream));
  }
  BATCH_TRY(cudaMalloc(&b->d_lb_shots, sizeof(dcg::LbShot) * tab.size()));
  BATCH_TRY(cudaMemcpyAsync(b->d_lb_shots, tab.data(), sizeof(dcg::LbShot) * tab.size(),
                            cudaMemcpyHostToDevice, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  b->lb_cells = total;
  b->lb_layer = layer;
  b->lb_params = dc_gb300_mlp_device_params(mlp);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_set_tiles(dc_gb300_batch *h, int ty, int zsplit) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  if (!dcg::fast_tile_rows_valid(ty, b->coef_form) || zsplit < 1 || zsplit > 64)
    return fail(DC_GB300_ERR_ARG,
                "tile rows must be 8 or 16 and zsplit in [1, 64]");
  BATCH_TRY(cudaSetDevice(b->device));
  b->ty = ty;
  b->zsplit = zsplit;
  b->prepared = false;
  dcg::drop_graphs(b);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_autotune(dc_gb300_batch *h, int steps, int *ty_out,
                                       int *zsplit_out, float *ms_out) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  if (steps < 1) return fail(DC_GB300_ERR_ARG, "autotune needs at least one step");
  BATCH_TRY(cudaSetDevice(b->device));
  const int tys[2] = {8, 16};
  const int splits[4] = {1, 2, 4, 8};
  int best_ty = b->ty, best_split = b->zsplit;
  bool best_persistent = b->persistent;
  float best = -1.0f;
  cudaEvent_t e0, e1;
  BATCH_TRY(cudaEventCreate(&e0));
  BATCH_TRY(cudaEventCreate(&e1));
  int rc = DC_GB300_OK;
  for (int t : tys) {
    for (int zs : splits) {
     for (int pers = 1; pers >= 0; --pers) {
      rc = dcg::prepare(b, t, zs, pers != 0);
      if (rc != DC_GB300_OK) break;
      rc = dcg::reset_state(b);
      if (rc != DC_GB300_OK) break;
      // one untimed step (first use of this configuration), then timed ones
      cudaError_t e = dcg::queue_steps(b, 0, 1);
      if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
      if (e == cudaSuccess) e = dcg::queue_steps(b, 1, steps);
      if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        rc = fail(DC_GB300_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
        break;
      }
      rc = dcg::check_err(b);
      if (rc != DC_GB300_OK) break;
      ms /= steps;
      if (best < 0 || ms < best) {
        best = ms;
        best_ty = t;
        best_split = zs;
        best_persistent = pers != 0;
      }
     }
     if (rc != DC_GB300_OK) break;
    }
    if (rc != DC_GB300_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != DC_GB300_OK) return rc;
  rc = dcg::prepare(b, best_ty, best_split, best_persistent);
  if (rc != DC_GB300_OK) return rc;
  rc = dcg::reset_state(b);
  if (rc != DC_GB300_OK) return rc;
  if (ty_out) *ty_out = best_ty;
  if (zsplit_out) *zsplit_out = best_split;
  if (ms_out) *ms_out = best;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_run(dc_gb300_batch *h, int steps) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  if (steps < 0) return fail(DC_GB300_ERR_ARG, "negative step count");
  if (steps == 0) return DC_GB300_OK;
  BATCH_TRY(cudaSetDevice(b->device));
  return dcg::run_steps(b, steps);
}

extern "C" int dc_gb300_batch_synchronize(dc_gb300_batch *h) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  BATCH_TRY(cudaSetDevice(b->device));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  return dcg::check_err(b);
}

extern "C" int dc_gb300_batch_get_fields(dc_gb300_batch *h, int shot, float *pp, float *pc,
                                         float *qp, float *qc) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  if (shot < 0 || shot >= static_cast<int>(b->shots.size()))
    return fail(DC_GB300_ERR_ARG, "shot index out of range");
  BATCH_TRY(cudaSetDevice(b->device));
  const dcg::BShot &s = b->shots[shot];
  const long long n = s.cfg.sx * s.cfg.sy * s.cfg.sz;
  const int cur = b->steps_done & 1;
  float *d = nullptr;
  BATCH_TRY(cudaMalloc(&d, sizeof(float) * 4 * n));
  cudaError_t e = dcg::launch_unpack(b->stream, s.pq[1 - cur], d, d + n, s.cfg.sx, s.cfg.sy,
                                     s.cfg.sz, s.pitch);
  if (e == cudaSuccess)
    e = dcg::launch_unpack(b->stream, s.pq[cur], d + 2 * n, d + 3 * n, s.cfg.sx, s.cfg.sy,
                           s.cfg.sz, s.pitch);
  float *outs[4] = {pp, qp, pc, qc};
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    if (outs[k])
      e = cudaMemcpyAsync(outs[k], d + k * n, sizeof(float) * n, cudaMemcpyDeviceToHost,
                          b->stream);
  float pre[2] = {0.0f, 0.0f};
  const bool pending = dcg::source_pending(b);
  if (e == cudaSuccess && pending)
    e = cudaMemcpyAsync(pre, b->d_src_pre + 2 * shot, sizeof(pre), cudaMemcpyDeviceToHost,
                        b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(d);
  if (e != cudaSuccess)
    return fail(DC_GB300_ERR_CUDA, std::string("batch get_fields: ") + cudaGetErrorString(e));
  if (pending) {  // the stored pc/qc hold the next step's amplitude already
    const long long di = s.cfg.src_x + s.cfg.src_y * s.cfg.sx + s.cfg.src_z * s.cfg.sx * s.cfg.sy;
    if (pc) pc[di] = pre[0];
    if (qc) qc[di] = pre[1];
  }
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_get_traces(dc_gb300_batch *h, int shot, int steps, float *out) {
  Batch *b = dcg::impl(h);
  if (!b || !out) return fail(DC_GB300_ERR_ARG, "null argument");
  if (shot < 0 || shot >= static_cast<int>(b->shots.size()))
    return fail(DC_GB300_ERR_ARG, "shot index out of range");
  const dcg::BShot &s = b->shots[shot];
  if (s.nrec == 0) return fail(DC_GB300_ERR_STATE, "shot has no receivers");
  if (steps < 0 || steps > b->max_steps) return fail(DC_GB300_ERR_ARG, "steps out of range");
  if (!b->prepared || !b->d_traces) {
    std::memset(out, 0, sizeof(float) * static_cast<size_t>(steps) * s.nrec);
    return DC_GB300_OK;
  }
  BATCH_TRY(cudaSetDevice(b->device));
  BATCH_TRY(cudaMemcpyAsync(out, b->d_traces + b->trace_off[shot],
                            sizeof(float) * static_cast<size_t>(steps) * s.nrec,
                            cudaMemcpyDeviceToHost, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_steps_done(const dc_gb300_batch *h) {
  return h ? h->impl.steps_done : -1;
}

extern "C" long dc_gb300_batch_kernel_launches(const dc_gb300_batch *h) {
  return h ? h->impl.launches : -1;
}

extern "C" void *dc_gb300_batch_stream(dc_gb300_batch *h) {
  return h ? static_cast<void *>(h->impl.stream) : nullptr;
}

extern "C" long long dc_gb300_batch_points(const dc_gb300_batch *h) {
  if (!h) return -1;
  long long n = 0;
  for (const auto &s : h->impl.shots) n += (s.cfg.sx - 8) * (s.cfg.sy - 8) * (s.cfg.sz - 8);
  return n;
}

extern "C" int dc_gb300_batch_set_grid(dc_gb300_batch *h, int persistent) {
  Batch *b = dcg::impl(h);
  if (!b) return fail(DC_GB300_ERR_ARG, "null batch");
  BATCH_TRY(cudaSetDevice(b->device));
  b->persistent = persistent != 0;
  b->prepared = false;
  dcg::drop_graphs(b);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_batch_grid(const dc_gb300_batch *h) {
  return h ? (h->impl.persistent ? 1 : 0) : -1;
}

extern "C" int dc_gb300_batch_tiles(const dc_gb300_batch *h, int *ty, int *zsplit) {
  if (!h) return fail(DC_GB300_ERR_ARG, "null batch");
  if (ty) *ty = h->impl.ty;
  if (zsplit) *zsplit = h->impl.zsplit;
  return DC_GB300_OK;
}
