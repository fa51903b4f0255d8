// dc_runtime.cu -- simulation object, device memory, graph-captured time
// loop, and the reference's device-data / propagate entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "dc_internal.h"

namespace dcg {

namespace {
thread_local std::string g_err;
constexpr int kGraphChunk = 64;  // steps per captured graph (even)
constexpr int kExactZChunk = 16;
}  // namespace

void set_error(const std::string &msg) { g_err = msg; }

namespace {

#define DCG_TRY(call)                                                       \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      set_error(std::string(#call) + ": " + cudaGetErrorString(e_));       \
      return DC_GB300_ERR_CUDA;                                             \
    }                                                                       \
  } while (0)

int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

long long round_up4(long long v) { return (v + 3) / 4 * 4; }

// The address at which kernels on `dev` may read or write the caller's array
// `p` in place, or nullptr when it has to be staged through a copy.  Direct
// access covers device memory of `dev`, managed memory, pinned or registered
// host memory and -- where the GPU reaches pageable memory through the host's
// page tables (NVLink-C2C systems such as GB300) -- plain malloc'd memory.
// Reading in place moves the data once, at the link's bandwidth, with no
// staging buffer.  DC_GB300_STAGED_COPIES=1 stages every host array.
template <typename T>
T *direct_view(T *p, int dev) {
  if (!p) return nullptr;
  static const bool staged = [] {
    const char *e = std::getenv("DC_GB300_STAGED_COPIES");
    return e && std::strcmp(e, "1") == 0;
  }();
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  switch (a.type) {
    case cudaMemoryTypeDevice:
      return a.device == dev ? p : nullptr;
    case cudaMemoryTypeManaged:
      return p;
    case cudaMemoryTypeHost:
      return staged ? nullptr : static_cast<T *>(a.devicePointer);
    default: {
      if (staged) return nullptr;
      int ats = 0;
      if (cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
          cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      return ats ? p : nullptr;
    }
  }
}

Sim *impl(dc_gb300_sim *h) { return h ? h->impl : nullptr; }

// Pair buffer that holds the field whose p component is `p` and q component
// `q` (q == p + 1), or -1.
int pair_of(const Sim *s, const float *p, const float *q) {
  for (int b = 0; b < 2; ++b) {
    const float *base = reinterpret_cast<const float *>(s->pq[b]);
    if (p == base && q == base + 1) return b;
  }
  return -1;
}

// Pair buffer and component (0 = p, 1 = q) of a field pointer, or -1.
int component_of(const Sim *s, const float *f, int *comp) {
  for (int b = 0; b < 2; ++b) {
    const float *base = reinterpret_cast<const float *>(s->pq[b]);
    if (f == base || f == base + 1) {
      *comp = static_cast<int>(f - base);
      return b;
    }
  }
  return -1;
}

// Buffers of the current and previous fields, or false when the ABI view
// has been rearranged into something the kernels cannot address.
bool roles(const Sim *s, int *cur, int *prev) {
  const dc_device_data &a = s->handle->abi;
  *cur = pair_of(s, a.pc, a.qc);
  *prev = pair_of(s, a.pp, a.qp);
  return *cur >= 0 && *prev >= 0 && *cur != *prev;
}

// Keeps the reference-ABI view in step with the device arrays.
void refresh_abi(Sim *s) {
  dc_device_data &a = s->handle->abi;
  // (vpz, vsv) pairs; each coefficient points at its lane of the grouped
  // layout (see coef_index)
  a.vpz = s->vv;
  a.vsv = s->vv ? s->vv + 1 : nullptr;
  dc_precomp_vars &p = a.precomp_vars;
  float *c = s->coef;
  const long long n = s->count;
  p.ch1dxx = c ? c + coef_index(DC_CXX, 0, n) : nullptr;
  p.ch1dyy = c ? c + coef_index(DC_CYY, 0, n) : nullptr;
  p.ch1dzz = c ? c + coef_index(DC_CZZ, 0, n) : nullptr;
  p.ch1dxy = c ? c + coef_index(DC_CXY, 0, n) : nullptr;
  p.ch1dyz = c ? c + coef_index(DC_CYZ, 0, n) : nullptr;
  p.ch1dxz = c ? c + coef_index(DC_CXZ, 0, n) : nullptr;
  p.v2px = c ? c + coef_index(DC_V2PX, 0, n) : nullptr;
  p.v2pz = c ? c + coef_index(DC_V2PZ, 0, n) : nullptr;
  p.v2sz = c ? c + coef_index(DC_V2SZ, 0, n) : nullptr;
  p.v2pn = c ? c + coef_index(DC_V2PN, 0, n) : nullptr;
}

void drop_graphs(Sim *s) {
  for (int i = 0; i < 2; ++i) {
    if (s->graph[i]) cudaGraphExecDestroy(s->graph[i]);
    s->graph[i] = nullptr;
    s->graph_version[i] = -1;
  }
}

void free_layer(Sim *s) {
  cudaFree(s->d_lb_cells);
  cudaFree(s->d_lb_corr);
  cudaFree(s->d_lb_lines);
  cudaFree(s->d_lb_edge);
  s->d_lb_cells = s->d_lb_lines = s->d_lb_edge = nullptr;
  s->d_lb_corr = nullptr;
  s->lb_cells = s->lb_lines = s->lb_edge = 0;
  s->lb_layer = 0;
  s->lb_params = nullptr;
}

void release(Sim *s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  drop_graphs(s);
  for (float2 *&f : s->pq) {
    cudaFree(f);
    f = nullptr;
  }
  cudaFree(s->coef);
  cudaFree(s->coef16);
  cudaFree(s->vbase);
  cudaFree(s->vv);
  cudaFree(s->sponge);
  cudaFree(s->d_src);
  cudaFree(s->d_src_pre);
  cudaFree(s->d_rec_col);
  cudaFree(s->d_rec_z);
  cudaFree(s->d_rec_r);
  cudaFree(s->d_traces);
  cudaFree(s->d_energy);
  cudaFree(s->d_step);
  cudaFree(s->d_err);
  free_layer(s);
  if (s->stream) cudaStreamDestroy(s->stream);
}

}  // namespace

// FD weights, inverse spacings, dt and dt^2 of a pass.
void fill_weights(StepParams *p, float dx, float dy, float dz, float dt) {
  // include/sample_compute.h:40-45 (float, IEEE division)
  p->dxxinv = 1.0f / (dx * dx);
  p->dyyinv = 1.0f / (dy * dy);
  p->dzzinv = 1.0f / (dz * dz);
  p->dxyinv = 1.0f / (dx * dy);
  p->dxzinv = 1.0f / (dx * dz);
  p->dyzinv = 1.0f / (dy * dz);
  {
    const double K[5] = {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0};
    const double L[4] = {4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0};
    const double hx = dx, hy = dy, hz = dz;
    for (int k = 0; k < 5; ++k) {
      p->w2x[k] = static_cast<float>(K[k] / (hx * hx));
      p->w2y[k] = static_cast<float>(K[k] / (hy * hy));
      p->w2z[k] = static_cast<float>(K[k] / (hz * hz));
    }
    for (int k = 0; k < 4; ++k) {
      p->w1x[k] = static_cast<float>(L[k] / hx);
      p->w1y[k] = static_cast<float>(L[k] / hy);
      p->w1z[k] = static_cast<float>(L[k] / hz);
    }
  }
  p->dt = dt;
  p->dt2 = dt * dt;
  p->dt2_iso = static_cast<float>(static_cast<double>(p->dt2) / (static_cast<double>(dx) * dx));
}

namespace {

// Fills the parameters of one stencil pass over a box.
StepParams make_params(Sim *s, const long long b0[3], const long long b1[3],
                       float dx, float dy, float dz, float dt) {
  StepParams p{};
  p.x0 = static_cast<int>(b0[0]);
  p.x1 = static_cast<int>(b1[0]);
  p.y0 = static_cast<int>(b0[1]);
  p.y1 = static_cast<int>(b1[1]);
  p.z0 = static_cast<int>(b0[2]);
  p.z1 = static_cast<int>(b1[2]);
  p.tile_x0 = p.x0 & ~3;
  p.tile_y0 = p.y0;
  p.zchunk = s->kernel == DC_GB300_KERNEL_FAST
                 ? fast_shape(s, p.x1 - p.tile_x0, p.y1 - p.tile_y0, p.z1 - p.z0).zchunk
                 : kExactZChunk;
  p.pitch = s->pitch;
  p.plane = s->plane;
  fill_weights(&p, dx, dy, dz, dt);
  // the BF16 medium stores the velocity terms scaled by 2^-vexp
  if (s->coef_form == CF_BF16) {
    p.dt2 = ldexpf(p.dt2, s->vexp);
    p.dt2_iso = ldexpf(p.dt2_iso, s->vexp);
  }
  const dc_device_data &a = s->handle->abi;
  p.prev = reinterpret_cast<float2 *>(a.pp);
  p.cur = reinterpret_cast<const float2 *>(a.pc);
  p.coef = s->coef;
  p.vv = s->vv;
  p.count = s->count;
  p.sponge = nullptr;
  p.src_x = -1;
  p.src_y = -1;
  p.src_z = -1;
  p.d_step = s->d_step;
  p.src_pre = s->d_src_pre;
  p.err = s->d_err;
  return p;
}

cudaError_t launch_pass(Sim *s, const StepParams &p) {
  ++s->launches;
  if (s->kernel == DC_GB300_KERNEL_EXACT) return launch_exact(s, p);
  int cur = -1, prev = -1;
  roles(s, &cur, &prev);  // checked by the callers
  return launch_fast(s, p, cur, prev);
}

void swap_roles(dc_device_data *a) {
  std::swap(a->pp, a->pc);
  std::swap(a->qp, a->qc);
}

// Kernel launches of one step: the stencil pass, then with a learned layer
// the face-line pass and the edge cells' network and add.
long long launches_per_step(const Sim *s) {
  if (s->lb_cells <= 0) return 1;
  return 1 + (s->lb_lines > 0 ? 1 : 0) + (s->lb_edge > 0 ? 2 : 0);
}

// Queues one full time step (j-th of a run): fused source for the next
// step, stencil over [4, s-4)^3, receiver gather; then swaps the roles.
cudaError_t queue_step(Sim *s, int j) {
  const long long b0[3] = {4, 4, 4};
  const long long b1[3] = {s->sx - 4, s->sy - 4, s->sz - 4};
  StepParams p = make_params(s, b0, b1, s->dx, s->dy, s->dz, s->dt);
  p.step_offset = j;
  if (s->has_sponge) {
    p.sponge = s->sponge;
    p.sponge_oy = static_cast<int>(s->sx);
    p.sponge_oz = static_cast<int>(s->sx + s->sy);
  }
  if (s->src_gi >= 0) {
    p.src_x = s->src_x;
    p.src_y = s->src_y;
    p.src_z = s->src_z;
    p.src_table = s->d_src;
    p.src_count = s->src_count;
  }
  p.energy = s->d_energy;
  p.energy_cap = s->energy_cap;
  if (s->nrec > 0) {
    p.rec_col = s->d_rec_col;
    p.rec_z = s->d_rec_z;
    p.rec_r = s->d_rec_r;
    p.traces = s->d_traces;
    p.nrec = s->nrec;
    p.trace_cap = s->trace_cap;
    p.col_stride = static_cast<int>(s->sx);
  }
  cudaError_t e = launch_pass(s, p);
  if (e != cudaSuccess) return e;
  if (s->lb_cells > 0) {  // learned layer: correct the new field's layer cells
    int cur = -1, prev = -1;
    roles(s, &cur, &prev);
    if (s->lb_rec) {  // recorded rollout step: every cell's features in table order
      s->launches += 2;
      e = launch_lb_step(s->stream, s->lb_params, s->d_lb_cells, s->lb_cells, s->pq[prev],
                         s->pq[cur], s->pitch, s->plane, s->d_lb_corr, s->lb_rec);
    } else {
      s->launches += launches_per_step(s) - 1;
      e = launch_lb_fused(s->stream, s->lb_params, s->lb_layer, s->d_lb_lines, s->lb_lines,
                          s->d_lb_edge, s->lb_edge, s->pq[prev], s->pq[cur], s->pitch,
                          s->plane, s->d_lb_corr);
    }
    if (e != cudaSuccess) return e;
  }
  swap_roles(&s->handle->abi);
  return cudaSuccess;
}

// After a run the source point of pc/qc already holds the next step's
// amplitude (fused into the last store); the reference adds it only at the
// start of the next step.  The values before that addition are kept in
// d_src_pre so every observable state is the reference's.
bool source_pending(const Sim *s) {
  return s->src_gi >= 0 && s->steps_done > 0 && s->src_applied_step == s->steps_done;
}

// Puts the pre-injection values back into the device field and marks the
// source of the current step as not applied (the next run re-adds it).
cudaError_t settle_source(Sim *s) {
  if (!source_pending(s)) return cudaSuccess;
  int cur = -1, prev = -1;
  roles(s, &cur, &prev);
  cudaError_t e = cudaMemcpyAsync(s->pq[cur] + s->src_gi, s->d_src_pre, sizeof(float2),
                                  cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) s->src_applied_step = -1;
  return e;
}

// Dense index of the source point (for patching host copies).
long long source_dense(const Sim *s) {
  const long long z = s->src_gi / s->plane, r = s->src_gi % s->plane;
  const long long y = r / s->pitch, x = r % s->pitch;
  return x + y * s->sx + z * s->sx * s->sy;
}

int check_err_word(Sim *s) {
  int h = 0;
  DCG_TRY(cudaMemcpyAsync(&h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  if (h) cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream);
  if (h & kErrTimeout)
    return fail(DC_GB300_ERR_TIMEOUT, "a TMA wait in the stencil kernel timed out");
  if (h & kErrAlign)
    return fail(DC_GB300_ERR_CUDA, "shared-memory window not 128-byte aligned");
  return DC_GB300_OK;
}

bool env_is(const char *name, const char *value) {
  const char *v = std::getenv(name);
  return v && std::strcmp(v, value) == 0;
}

[[noreturn]] void abi_die(const char *where) {
  std::fprintf(stderr, "[dc_gb300] %s: %s\n", where, g_err.c_str());
  std::exit(1);
}

}  // namespace
}  // namespace dcg

using namespace dcg;

// ===========================================================================
// dc_gb300_* API
// ===========================================================================

extern "C" const char *dc_gb300_last_error(void) { return g_err.c_str(); }

extern "C" const char *dc_gb300_version(void) { return "dc_gb300 1.0 (sm_103a)"; }

extern "C" int dc_gb300_create(const dc_gb300_config *cfg, dc_gb300_sim **out) {
  if (!cfg || !out) return fail(DC_GB300_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->sx < 9 || cfg->sy < 9 || cfg->sz < 9)
    return fail(DC_GB300_ERR_ARG, "every size must be >= 9 (4-cell halo on both sides)");
  if (cfg->sx > (1 << 30) || cfg->sy > (1 << 30) || cfg->sz > (1 << 30))
    return fail(DC_GB300_ERR_ARG, "size too large");
  if (cfg->kernel != DC_GB300_KERNEL_FAST && cfg->kernel != DC_GB300_KERNEL_EXACT)
    return fail(DC_GB300_ERR_ARG, "unknown kernel");
  if (cfg->medium < DC_GB300_MEDIUM_PRECOMP || cfg->medium > DC_GB300_MEDIUM_PRECOMP_BF16)
    return fail(DC_GB300_ERR_ARG, "unknown medium form");
  if (!(cfg->dx > 0 && cfg->dy > 0 && cfg->dz > 0 && cfg->dt > 0))
    return fail(DC_GB300_ERR_ARG, "dx, dy, dz and dt must be positive");
  int dev = cfg->device;
  if (dev < 0) DCG_TRY(cudaGetDevice(&dev));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(DC_GB300_ERR_DEVICE, "no CUDA device");
  if (dev >= ndev) return fail(DC_GB300_ERR_DEVICE, "device ordinal out of range");
  cudaDeviceProp prop;
  DCG_TRY(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3)
    return fail(DC_GB300_ERR_DEVICE,
                std::string("this build targets sm_103a; device is ") + prop.name);
  DCG_TRY(cudaSetDevice(dev));

  auto *h = new dc_gb300_sim();
  auto *s = new Sim();
  h->impl = s;
  s->handle = h;
  s->device = dev;
  s->sx = cfg->sx;
  s->sy = cfg->sy;
  s->sz = cfg->sz;
  s->pitch = round_up4(cfg->sx);
  s->plane = s->pitch * s->sy;
  s->count = s->plane * s->sz;
  s->dx = cfg->dx;
  s->dy = cfg->dy;
  s->dz = cfg->dz;
  s->dt = cfg->dt;
  s->kernel = cfg->kernel;
  // the narrow forms are the ten-coefficient medium with an FP16/BF16 copy
  s->medium = cfg->medium == DC_GB300_MEDIUM_VPZ_VSV ? DC_GB300_MEDIUM_VPZ_VSV
                                                     : DC_GB300_MEDIUM_PRECOMP;
  s->coef_form = cfg->medium == DC_GB300_MEDIUM_VPZ_VSV       ? CF_VV
                 : cfg->medium == DC_GB300_MEDIUM_PRECOMP_F16  ? CF_F16
                 : cfg->medium == DC_GB300_MEDIUM_PRECOMP_BF16 ? CF_BF16
                                                               : CF_F32;
  auto bail = [&](int code) {
    release(s);
    delete s;
    delete h;
    return code;
  };
  // Blocking stream: the legacy default stream orders with it, so callers'
  // own cudaMemcpy on data->pc etc. see the finished results.
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamDefault) != cudaSuccess)
    return bail(fail(DC_GB300_ERR_CUDA, "cudaStreamCreate failed"));
  const size_t bytes = static_cast<size_t>(s->count) * 4;
  for (int b = 0; b < 2; ++b)
    if (cudaMalloc(&s->pq[b], bytes * 2) != cudaSuccess)
      return bail(fail(DC_GB300_ERR_NOMEM, "cudaMalloc of a wavefield failed"));
  if (s->medium == DC_GB300_MEDIUM_PRECOMP) {
    if (cudaMalloc(&s->coef, bytes * DC_NCOEF) != cudaSuccess)
      return bail(fail(DC_GB300_ERR_NOMEM, "cudaMalloc of the coefficients failed"));
    if ((s->coef_form == CF_F16 || s->coef_form == CF_BF16) &&
        cudaMalloc(&s->coef16, static_cast<size_t>(s->count) * 20) != cudaSuccess)
      return bail(fail(DC_GB300_ERR_NOMEM, "cudaMalloc of the FP16 coefficients failed"));
    if (s->coef_form == CF_F16 &&
        cudaMalloc(reinterpret_cast<void **>(&s->vbase), sizeof(float4) * s->sy * s->sz) !=
            cudaSuccess)
      return bail(fail(DC_GB300_ERR_NOMEM, "cudaMalloc of the velocity bases failed"));
  } else {
    if (cudaMalloc(&s->vv, bytes * 2) != cudaSuccess)
      return bail(fail(DC_GB300_ERR_NOMEM, "cudaMalloc of vpz/vsv failed"));
  }
  if (cudaMalloc(&s->d_step, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->d_err, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->d_src_pre, 2 * sizeof(float)) != cudaSuccess)
    return bail(fail(DC_GB300_ERR_NOMEM, "cudaMalloc of counters failed"));
  for (int b = 0; b < 2; ++b)
    if (cudaMemsetAsync(s->pq[b], 0, bytes * 2, s->stream) != cudaSuccess)
      return bail(fail(DC_GB300_ERR_CUDA, "cudaMemset failed"));
  if (s->coef) cudaMemsetAsync(s->coef, 0, bytes * DC_NCOEF, s->stream);
  if (s->coef16) cudaMemsetAsync(s->coef16, 0, static_cast<size_t>(s->count) * 20, s->stream);
  if (s->vv) cudaMemsetAsync(s->vv, 0, bytes * 2, s->stream);
  cudaMemsetAsync(s->d_step, 0, sizeof(int), s->stream);
  cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream);
  cudaMemsetAsync(s->d_src_pre, 0, 2 * sizeof(float), s->stream);
  std::string err;
  if (s->kernel == DC_GB300_KERNEL_FAST && !fast_encode_maps(s, &err))
    return bail(fail(DC_GB300_ERR_CUDA, err));
  // (pp, qp) live in pair buffer 0 and (pc, qc) in pair buffer 1; the q
  // pointer is the p pointer + 1 (interleaved storage)
  h->abi.pp = reinterpret_cast<float *>(s->pq[0]);
  h->abi.qp = h->abi.pp + 1;
  h->abi.pc = reinterpret_cast<float *>(s->pq[1]);
  h->abi.qc = h->abi.pc + 1;
  refresh_abi(s);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess)
    return bail(fail(DC_GB300_ERR_CUDA, "initialisation failed"));
  *out = h;
  return DC_GB300_OK;
}

extern "C" void dc_gb300_destroy(dc_gb300_sim *h) {
  if (!h) return;
  Sim *s = h->impl;
  if (s) {
    cudaSetDevice(s->device);
    release(s);
    delete s;
  }
  delete h;
}

extern "C" dc_device_data *dc_gb300_device_data(dc_gb300_sim *h) {
  return h ? &h->abi : nullptr;
}

extern "C" dc_gb300_sim *dc_gb300_from_device_data(dc_device_data *d) {
  return reinterpret_cast<dc_gb300_sim *>(d);
}

extern "C" long dc_gb300_device_pitch(const dc_gb300_sim *h) {
  return h && h->impl ? static_cast<long>(h->impl->pitch) : 0;
}

extern "C" void *dc_gb300_stream(dc_gb300_sim *h) {
  return h && h->impl ? static_cast<void *>(h->impl->stream) : nullptr;
}

extern "C" long dc_gb300_kernel_launches(const dc_gb300_sim *h) {
  return h && h->impl ? static_cast<long>(h->impl->launches) : 0;
}

extern "C" long dc_gb300_steps_done(const dc_gb300_sim *h) {
  return h && h->impl ? static_cast<long>(h->impl->steps_done) : 0;
}

// dc_precomp_vars order -> DevCoef
constexpr int kRefOrder[10] = {DC_CXX, DC_CYY, DC_CZZ, DC_CXY, DC_CYZ,
                               DC_CXZ, DC_V2PX, DC_V2PZ, DC_V2SZ, DC_V2PN};

extern "C" int dc_gb300_set_precomp(dc_gb300_sim *h, const dc_precomp_vars *host) {
  Sim *s = impl(h);
  if (!s || !host) return fail(DC_GB300_ERR_ARG, "null argument");
  if (!s->coef) return fail(DC_GB300_ERR_STATE, "simulation uses the vpz/vsv medium form");
  const float *src[10] = {host->ch1dxx, host->ch1dyy, host->ch1dzz, host->ch1dxy,
                          host->ch1dyz, host->ch1dxz, host->v2px,   host->v2pz,
                          host->v2sz,   host->v2pn};
  for (const float *p : src)
    if (!p) return fail(DC_GB300_ERR_ARG, "a coefficient array is null");
  DCG_TRY(cudaSetDevice(s->device));
  const long long n = s->sx * s->sy * s->sz;
  CoefSources views{};
  bool direct = true;
  for (int k = 0; k < 10; ++k) direct = direct && (views.p[k] = direct_view(src[k], s->device));
  if (direct) {  // one pass, reading the caller's arrays in place
    DCG_TRY(launch_coef_gather(s->stream, s->coef, views, s->sx, s->sy, s->sz, s->pitch,
                               s->count));
    DCG_TRY(cudaStreamSynchronize(s->stream));
    s->coef16_stale = true;
    return DC_GB300_OK;
  }
  float *stage = nullptr;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n, s->stream));
  for (int k = 0; k < 10; ++k) {
    DCG_TRY(cudaMemcpyAsync(stage, src[k], sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
    DCG_TRY(launch_coef_component(s->stream, s->coef, stage, kRefOrder[k], s->sx, s->sy, s->sz,
                                  s->pitch, s->count, true));
  }
  DCG_TRY(cudaFreeAsync(stage, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  s->coef16_stale = true;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_set_vpz_vsv(dc_gb300_sim *h, const float *vpz, const float *vsv) {
  Sim *s = impl(h);
  if (!s || !vpz || !vsv) return fail(DC_GB300_ERR_ARG, "null argument");
  if (!s->vv) return fail(DC_GB300_ERR_STATE, "simulation uses the ten-coefficient medium form");
  DCG_TRY(cudaSetDevice(s->device));
  const long long n = s->sx * s->sy * s->sz;
  const float *dv = direct_view(vpz, s->device), *ds = direct_view(vsv, s->device);
  if (dv && ds) {
    DCG_TRY(launch_pack(s->stream, reinterpret_cast<float2 *>(s->vv), dv, ds, s->sx, s->sy,
                        s->sz, s->pitch));
    DCG_TRY(cudaStreamSynchronize(s->stream));
    return DC_GB300_OK;
  }
  float *stage = nullptr;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n * 2, s->stream));
  DCG_TRY(cudaMemcpyAsync(stage, vpz, sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
  DCG_TRY(cudaMemcpyAsync(stage + n, vsv, sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
  DCG_TRY(launch_pack(s->stream, reinterpret_cast<float2 *>(s->vv), stage, stage + n, s->sx,
                      s->sy, s->sz, s->pitch));
  DCG_TRY(cudaFreeAsync(stage, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_get_precomp(dc_gb300_sim *h, const dc_precomp_vars *host) {
  Sim *s = impl(h);
  if (!s || !host) return fail(DC_GB300_ERR_ARG, "null argument");
  if (!s->coef) return fail(DC_GB300_ERR_STATE, "simulation uses the vpz/vsv medium form");
  float *dst[10] = {host->ch1dxx, host->ch1dyy, host->ch1dzz, host->ch1dxy, host->ch1dyz,
                    host->ch1dxz, host->v2px,   host->v2pz,   host->v2sz,   host->v2pn};
  DCG_TRY(cudaSetDevice(s->device));
  const long long n = s->sx * s->sy * s->sz;
  float *stage = nullptr;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n, s->stream));
  for (int k = 0; k < 10; ++k) {
    if (!dst[k]) continue;
    DCG_TRY(launch_coef_component(s->stream, s->coef, stage, kRefOrder[k], s->sx, s->sy, s->sz,
                                  s->pitch, s->count, false));
    DCG_TRY(cudaMemcpyAsync(dst[k], stage, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream));
  }
  DCG_TRY(cudaFreeAsync(stage, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_get_vpz_vsv(dc_gb300_sim *h, float *vpz, float *vsv) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null argument");
  if (!s->vv) return fail(DC_GB300_ERR_STATE, "simulation uses the ten-coefficient medium form");
  DCG_TRY(cudaSetDevice(s->device));
  const long long n = s->sx * s->sy * s->sz;
  float *stage = nullptr;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n * 2, s->stream));
  DCG_TRY(launch_unpack(s->stream, reinterpret_cast<const float2 *>(s->vv), stage, stage + n,
                        s->sx, s->sy, s->sz, s->pitch));
  if (vpz) DCG_TRY(cudaMemcpyAsync(vpz, stage, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream));
  if (vsv)
    DCG_TRY(cudaMemcpyAsync(vsv, stage + n, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream));
  DCG_TRY(cudaFreeAsync(stage, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

namespace {
// GPU FP64 precompute from dense host anisotropy arrays into `grouped`, a
// dense grouped coefficient block of n points (coef_index with count = n).
int precompute_dense(cudaStream_t st, int dev, const dc_anisotropy_t *a, long long n,
                     float *grouped) {
  const float *src[6] = {a->theta, a->phi, a->vsv, a->vpz, a->epsilon, a->delta};
  for (const float *p : src)
    if (!p) return fail(DC_GB300_ERR_ARG, "an anisotropy array is null");
  const float *v[6];
  bool direct = true;
  for (int k = 0; k < 6; ++k) direct = direct && (v[k] = direct_view(src[k], dev));
  if (direct) {
    DCG_TRY(launch_precomp(st, v[0], v[1], v[2], v[3], v[4], v[5], grouped, n, n));
    return DC_GB300_OK;
  }
  float *d_in = nullptr;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d_in), sizeof(float) * n * 6, st));
  for (int k = 0; k < 6; ++k)
    DCG_TRY(cudaMemcpyAsync(d_in + k * n, src[k], sizeof(float) * n,
                            cudaMemcpyHostToDevice, st));
  DCG_TRY(launch_precomp(st, d_in, d_in + n, d_in + 2 * n, d_in + 3 * n, d_in + 4 * n,
                         d_in + 5 * n, grouped, n, n));
  DCG_TRY(cudaFreeAsync(d_in, st));
  return DC_GB300_OK;
}

// Refreshes the 16-bit copy of the medium when the fast kernel reads it:
// FP16 with fixed-point angle terms and per-row velocity bases, or BF16 with
// the velocity terms scaled by 2^-vexp so their maximum stays below 2^14.
int refresh_narrow(Sim *s) {
  if (!(s->coef_form == CF_F16 || s->coef_form == CF_BF16) || !s->coef16_stale)
    return DC_GB300_OK;
  if (s->coef_form == CF_F16) {
    DCG_TRY(launch_coef_rowref(s->stream, s->coef, s->coef16, s->vbase, s->sx, s->sy, s->sz,
                               s->pitch, s->count));
    DCG_TRY(cudaStreamSynchronize(s->stream));
    s->vexp = 0;
    s->coef16_stale = false;
    drop_graphs(s);
    ++s->config_version;
    return DC_GB300_OK;
  }
  unsigned int *d_max = nullptr;
  unsigned int bits = 0;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d_max), sizeof(unsigned int), s->stream));
  DCG_TRY(cudaMemsetAsync(d_max, 0, sizeof(unsigned int), s->stream));
  DCG_TRY(launch_coef_vmax(s->stream, s->coef, s->count, d_max));
  DCG_TRY(cudaMemcpyAsync(&bits, d_max, sizeof(bits), cudaMemcpyDeviceToHost, s->stream));
  DCG_TRY(cudaFreeAsync(d_max, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  float vmax;
  std::memcpy(&vmax, &bits, sizeof(vmax));
  int e = 0;
  if (vmax > 0.0f && std::isfinite(vmax)) {
    std::frexp(vmax, &e);  // vmax < 2^e
    e -= 14;
  }
  s->vexp = e;
  DCG_TRY(launch_coef_narrow(s->stream, s->coef, s->coef16, s->coef_form, s->vexp, s->count));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  s->coef16_stale = false;
  drop_graphs(s);  // dt^2 in the captured parameters depends on vexp
  ++s->config_version;
  return DC_GB300_OK;
}
}  // namespace

extern "C" int dc_gb300_set_anisotropy(dc_gb300_sim *h, const dc_anisotropy_t *host) {
  Sim *s = impl(h);
  if (!s || !host) return fail(DC_GB300_ERR_ARG, "null argument");
  DCG_TRY(cudaSetDevice(s->device));
  const long long n = s->sx * s->sy * s->sz;
  if (s->vv) {
    if (!host->vpz || !host->vsv) return fail(DC_GB300_ERR_ARG, "vpz/vsv null");
    int rc = dc_gb300_set_vpz_vsv(h, host->vpz, host->vsv);
    if (rc != DC_GB300_OK) return rc;
  }
  if (s->coef) {
    float *grouped = nullptr;
    DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&grouped), sizeof(float) * n * DC_NCOEF,
                            s->stream));
    int rc = precompute_dense(s->stream, s->device, host, n, grouped);
    if (rc != DC_GB300_OK) return rc;
    DCG_TRY(launch_coef_repitch(s->stream, s->coef, grouped, s->sx, s->sy, s->sz, s->pitch,
                                s->count));
    DCG_TRY(cudaFreeAsync(grouped, s->stream));
    s->coef16_stale = true;
  }
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_generate_layered(dc_gb300_sim *h, const dc_gb300_layered_spec *spec) {
  Sim *s = impl(h);
  if (!s || !spec) return fail(DC_GB300_ERR_ARG, "null argument");
  if (spec->nlayers < 1 || spec->nlayers > DC_GB300_MAX_LAYERS ||
      spec->n_noise < 0 || spec->n_noise > DC_GB300_MAX_FEATURES ||
      spec->n_theta < 0 || spec->n_theta > DC_GB300_MAX_FEATURES ||
      spec->n_phi < 0 || spec->n_phi > DC_GB300_MAX_FEATURES || !(spec->sigma_ratio > 0))
    return fail(DC_GB300_ERR_ARG, "invalid layered-medium spec");
  DCG_TRY(cudaSetDevice(s->device));
  ++s->launches;
  DCG_TRY(launch_layered(s->stream, *spec, s->coef, s->vv, s->sx, s->sy, s->sz, s->pitch,
                         s->count));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  s->coef16_stale = true;
  return DC_GB300_OK;
}

extern "C" void dc_gb300_reference_medium_constants(int absorb, float out[6]);

extern "C" int dc_gb300_generate_reference(dc_gb300_sim *h, long nx, long ny, long nz,
                                           long absorb, unsigned int seed) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  if (nx < 1 || ny < 1 || nz < 1 || absorb < 1 || s->sx != nx + 2 * absorb + 8 ||
      s->sy != ny + 2 * absorb + 8 || s->sz != nz + 2 * absorb + 8)
    return fail(DC_GB300_ERR_ARG, "sizes must be n + 2*absorb + 8 per axis, absorb >= 1");
  DCG_TRY(cudaSetDevice(s->device));
  float consts[6];
  dc_gb300_reference_medium_constants(static_cast<int>(absorb), consts);
  const int n[3] = {static_cast<int>(nx), static_cast<int>(ny), static_cast<int>(nz)};
  ++s->launches;
  DCG_TRY(launch_reference_medium(s->stream, n, static_cast<int>(absorb), seed, consts, s->coef,
                                  s->vv, s->pitch, s->count));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  s->coef16_stale = true;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_set_fields(dc_gb300_sim *h, const float *pp, const float *pc,
                                   const float *qp, const float *qc) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  DCG_TRY(cudaSetDevice(s->device));
  int cur = -1, prev = -1;
  if (!roles(s, &cur, &prev)) return fail(DC_GB300_ERR_STATE, "field pointers rearranged");
  const long long n = s->sx * s->sy * s->sz;
  const float *src[2][2] = {{pp, qp}, {pc, qc}};
  const int dst[2] = {prev, cur};
  bool direct = true;
  const float *view[2][2];
  for (int k = 0; k < 2; ++k)
    for (int c = 0; c < 2; ++c) {
      view[k][c] = direct_view(src[k][c], s->device);
      direct = direct && (!src[k][c] || view[k][c]);
    }
  float *stage = nullptr;
  if (direct) {  // pack straight from the caller's arrays
    for (int k = 0; k < 2; ++k) {
      DCG_TRY(cudaMemsetAsync(s->pq[dst[k]], 0, sizeof(float2) * s->count, s->stream));
      DCG_TRY(launch_pack(s->stream, s->pq[dst[k]], view[k][0], view[k][1], s->sx, s->sy,
                          s->sz, s->pitch));
    }
  } else {
    DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n * 2, s->stream));
  }
  for (int k = 0; k < 2 && !direct; ++k) {
    const float *dp = nullptr, *dq = nullptr;
    if (src[k][0]) {
      DCG_TRY(cudaMemcpyAsync(stage, src[k][0], sizeof(float) * n, cudaMemcpyHostToDevice,
                              s->stream));
      dp = stage;
    }
    if (src[k][1]) {
      DCG_TRY(cudaMemcpyAsync(stage + n, src[k][1], sizeof(float) * n, cudaMemcpyHostToDevice,
                              s->stream));
      dq = stage + n;
    }
    // the pitch padding stays zero: clear, then pack the dense arrays
    DCG_TRY(cudaMemsetAsync(s->pq[dst[k]], 0, sizeof(float2) * s->count, s->stream));
    DCG_TRY(launch_pack(s->stream, s->pq[dst[k]], dp, dq, s->sx, s->sy, s->sz, s->pitch));
  }
  if (stage) DCG_TRY(cudaFreeAsync(stage, s->stream));
  DCG_TRY(cudaMemsetAsync(s->d_step, 0, sizeof(int), s->stream));
  if (s->d_energy) DCG_TRY(cudaMemsetAsync(s->d_energy, 0, sizeof(double) * s->energy_cap, s->stream));
  if (s->d_traces)
    DCG_TRY(cudaMemsetAsync(s->d_traces, 0, sizeof(float) * s->trace_cap * s->nrec, s->stream));
  s->steps_done = 0;
  s->src_applied_step = -1;
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_get_fields(dc_gb300_sim *h, float *pp, float *pc, float *qp,
                                   float *qc) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  DCG_TRY(cudaSetDevice(s->device));
  int cur = -1, prev = -1;
  if (!roles(s, &cur, &prev)) return fail(DC_GB300_ERR_STATE, "field pointers rearranged");
  const long long n = s->sx * s->sy * s->sz;
  float *dst[2][2] = {{pp, qp}, {pc, qc}};
  const int src[2] = {prev, cur};
  bool direct = true;
  float *view[2][2];
  for (int k = 0; k < 2; ++k)
    for (int c = 0; c < 2; ++c) {
      view[k][c] = direct_view(dst[k][c], s->device);
      direct = direct && (!dst[k][c] || view[k][c]);
    }
  float *stage = nullptr;
  if (direct) {  // unpack straight into the caller's arrays
    for (int k = 0; k < 2; ++k)
      if (dst[k][0] || dst[k][1])
        DCG_TRY(launch_unpack(s->stream, s->pq[src[k]], view[k][0], view[k][1], s->sx, s->sy,
                              s->sz, s->pitch));
  } else {
    DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n * 2, s->stream));
  }
  for (int k = 0; k < 2 && !direct; ++k) {
    if (!dst[k][0] && !dst[k][1]) continue;
    DCG_TRY(launch_unpack(s->stream, s->pq[src[k]], stage, stage + n, s->sx, s->sy, s->sz,
                          s->pitch));
    if (dst[k][0])
      DCG_TRY(cudaMemcpyAsync(dst[k][0], stage, sizeof(float) * n, cudaMemcpyDeviceToHost,
                              s->stream));
    if (dst[k][1])
      DCG_TRY(cudaMemcpyAsync(dst[k][1], stage + n, sizeof(float) * n, cudaMemcpyDeviceToHost,
                              s->stream));
  }
  if (stage) DCG_TRY(cudaFreeAsync(stage, s->stream));
  float pre[2] = {0.f, 0.f};
  const bool patch = source_pending(s) && (pc || qc);
  if (patch)
    DCG_TRY(cudaMemcpyAsync(pre, s->d_src_pre, sizeof(pre), cudaMemcpyDeviceToHost, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  if (patch) {
    const long long i = source_dense(s);
    if (pc) pc[i] = pre[0];
    if (qc) qc[i] = pre[1];
  }
  return DC_GB300_OK;
}

namespace {
constexpr char kCkptMagic[8] = {'D', 'C', 'G', 'B', '3', '0', '0', 'C'};
struct CkptHeader {
  char magic[8];
  uint32_t version, reserved;
  int64_t sx, sy, sz, steps_done, src_applied, pad;
};
static_assert(sizeof(CkptHeader) == 64, "checkpoint header is 64 bytes");
}  // namespace

extern "C" int dc_gb300_save_checkpoint(dc_gb300_sim *h, const char *path) {
  Sim *s = impl(h);
  if (!s || !path) return fail(DC_GB300_ERR_ARG, "null argument");
  DCG_TRY(cudaSetDevice(s->device));
  int cur = -1, prev = -1;
  if (!roles(s, &cur, &prev)) return fail(DC_GB300_ERR_STATE, "field pointers rearranged");
  const long long n = s->sx * s->sy * s->sz;
  std::vector<float> host(static_cast<size_t>(n) * 2);
  float *stage = nullptr;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n * 2, s->stream));
  FILE *f = std::fopen(path, "wb");
  if (!f) {
    cudaFreeAsync(stage, s->stream);
    return fail(DC_GB300_ERR_ARG, std::string("cannot open ") + path);
  }
  CkptHeader hd{};
  std::memcpy(hd.magic, kCkptMagic, 8);
  hd.version = 1;
  hd.sx = s->sx;
  hd.sy = s->sy;
  hd.sz = s->sz;
  hd.steps_done = s->steps_done;
  hd.src_applied = 0;  // the file holds the reference's state (no pending source)
  float pre[2] = {0.f, 0.f};
  const bool patch = source_pending(s);
  if (patch) {
    DCG_TRY(cudaMemcpyAsync(pre, s->d_src_pre, sizeof(pre), cudaMemcpyDeviceToHost, s->stream));
    DCG_TRY(cudaStreamSynchronize(s->stream));
  }
  bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1;
  for (int b : {prev, cur}) {
    if (!ok) break;
    cudaError_t e = launch_unpack(s->stream, s->pq[b], stage, stage + n, s->sx, s->sy, s->sz,
                                  s->pitch);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(host.data(), stage, sizeof(float) * n * 2, cudaMemcpyDeviceToHost,
                          s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
      std::fclose(f);
      cudaFreeAsync(stage, s->stream);
      return fail(DC_GB300_ERR_CUDA, cudaGetErrorString(e));
    }
    if (patch && b == cur) {
      const long long i = source_dense(s);
      host[i] = pre[0];
      host[n + i] = pre[1];
    }
    ok = std::fwrite(host.data(), sizeof(float), host.size(), f) == host.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  DCG_TRY(cudaFreeAsync(stage, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  if (!ok) return fail(DC_GB300_ERR_ARG, std::string("write failed: ") + path);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_load_checkpoint(dc_gb300_sim *h, const char *path) {
  Sim *s = impl(h);
  if (!s || !path) return fail(DC_GB300_ERR_ARG, "null argument");
  DCG_TRY(cudaSetDevice(s->device));
  int cur = -1, prev = -1;
  if (!roles(s, &cur, &prev)) return fail(DC_GB300_ERR_STATE, "field pointers rearranged");
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(DC_GB300_ERR_ARG, std::string("cannot open ") + path);
  CkptHeader hd{};
  if (std::fread(&hd, sizeof(hd), 1, f) != 1 || std::memcmp(hd.magic, kCkptMagic, 8) != 0 ||
      hd.version != 1) {
    std::fclose(f);
    return fail(DC_GB300_ERR_ARG, "not a dc_gb300 checkpoint");
  }
  if (hd.sx != s->sx || hd.sy != s->sy || hd.sz != s->sz || hd.steps_done < 0 ||
      hd.steps_done > (1LL << 30)) {
    std::fclose(f);
    return fail(DC_GB300_ERR_ARG, "checkpoint sizes differ from the simulation's");
  }
  const long long n = s->sx * s->sy * s->sz;
  std::vector<float> host(static_cast<size_t>(n) * 2);
  float *stage = nullptr;
  DCG_TRY(cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n * 2, s->stream));
  for (int b : {prev, cur}) {
    if (std::fread(host.data(), sizeof(float), host.size(), f) != host.size()) {
      std::fclose(f);
      cudaFreeAsync(stage, s->stream);
      return fail(DC_GB300_ERR_ARG, "truncated checkpoint");
    }
    cudaError_t e = cudaMemcpyAsync(stage, host.data(), sizeof(float) * n * 2,
                                    cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(s->pq[b], 0, sizeof(float2) * s->count, s->stream);
    if (e == cudaSuccess)
      e = launch_pack(s->stream, s->pq[b], stage, stage + n, s->sx, s->sy, s->sz, s->pitch);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
      std::fclose(f);
      cudaFreeAsync(stage, s->stream);
      return fail(DC_GB300_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  std::fclose(f);
  DCG_TRY(cudaFreeAsync(stage, s->stream));
  const int step = static_cast<int>(hd.steps_done);
  DCG_TRY(cudaMemcpyAsync(s->d_step, &step, sizeof(int), cudaMemcpyHostToDevice, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  s->steps_done = hd.steps_done;
  s->src_applied_step = hd.src_applied ? hd.steps_done : -1;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_set_source(dc_gb300_sim *h, long index, const float *amp, int count) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  DCG_TRY(cudaSetDevice(s->device));
  DCG_TRY(settle_source(s));  // the old source's pending amplitude comes out first
  drop_graphs(s);
  ++s->config_version;
  if (index < 0) {
    s->src_gi = -1;
    s->src_x = s->src_y = s->src_z = -1;
    return DC_GB300_OK;
  }
  const long long n = s->sx * s->sy * s->sz;
  if (index >= n || count < 0 || (count > 0 && !amp))
    return fail(DC_GB300_ERR_ARG, "source index or amplitudes invalid");
  const long long x = index % s->sx, y = (index / s->sx) % s->sy, z = index / (s->sx * s->sy);
  if (x < 4 || x >= s->sx - 4 || y < 4 || y >= s->sy - 4 || z < 4 || z >= s->sz - 4)
    return fail(DC_GB300_ERR_ARG, "the source must lie in the updated region [4, s-4)^3");
  if (count > s->src_count || !s->d_src) {
    cudaFree(s->d_src);
    s->d_src = nullptr;
    DCG_TRY(cudaMalloc(&s->d_src, sizeof(float) * std::max(count, 1)));
  }
  if (count > 0)
    DCG_TRY(cudaMemcpyAsync(s->d_src, amp, sizeof(float) * count, cudaMemcpyHostToDevice,
                            s->stream));
  s->src_count = count;
  s->src_x = static_cast<int>(x);
  s->src_y = static_cast<int>(y);
  s->src_z = static_cast<int>(z);
  s->src_gi = z * s->plane + y * s->pitch + x;
  s->src_applied_step = -1;
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_set_sponge(dc_gb300_sim *h, const float *gx, const float *gy,
                                   const float *gz) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  DCG_TRY(cudaSetDevice(s->device));
  drop_graphs(s);
  ++s->config_version;
  if (!gx || !gy || !gz) {
    s->has_sponge = false;
    return DC_GB300_OK;
  }
  if (!s->sponge)
    DCG_TRY(cudaMalloc(&s->sponge, sizeof(float) * (s->sx + s->sy + s->sz)));
  DCG_TRY(cudaMemcpyAsync(s->sponge, gx, sizeof(float) * s->sx, cudaMemcpyHostToDevice, s->stream));
  DCG_TRY(cudaMemcpyAsync(s->sponge + s->sx, gy, sizeof(float) * s->sy, cudaMemcpyHostToDevice,
                          s->stream));
  DCG_TRY(cudaMemcpyAsync(s->sponge + s->sx + s->sy, gz, sizeof(float) * s->sz,
                          cudaMemcpyHostToDevice, s->stream));
  s->has_sponge = true;
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_set_learned_layer(dc_gb300_sim *h, const dc_gb300_mlp *mlp,
                                          int layer) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  if (layer < 0 || layer > DC_GB300_MLP_DEPTHS)
    return fail(DC_GB300_ERR_ARG, "layer width must lie in [0, DC_GB300_MLP_DEPTHS]");
  if (layer > 0 && !mlp) return fail(DC_GB300_ERR_ARG, "null MLP");
  if (layer > 0 && (s->sx < 2 * layer + 16 || s->sy < 2 * layer + 16 || s->sz < 2 * layer + 16))
    return fail(DC_GB300_ERR_ARG, "the interior must keep at least 8 cells per axis");
  DCG_TRY(cudaSetDevice(s->device));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  drop_graphs(s);
  ++s->config_version;
  free_layer(s);
  if (layer == 0) return DC_GB300_OK;
  const std::vector<int4> cells = layer_cells(s->sx, s->sy, s->sz, layer);
  const LayerPlan plan = layer_plan(s->sx, s->sy, s->sz, layer);
  const long long n = static_cast<long long>(cells.size());
  const long long nl = static_cast<long long>(plan.lines.size());
  const long long ne = static_cast<long long>(plan.edge.size());
  DCG_TRY(cudaMalloc(&s->d_lb_cells, sizeof(int4) * n));
  DCG_TRY(cudaMalloc(&s->d_lb_corr, sizeof(float2) * n));
  DCG_TRY(cudaMalloc(&s->d_lb_lines, sizeof(int4) * std::max(nl, 1LL)));
  DCG_TRY(cudaMalloc(&s->d_lb_edge, sizeof(int4) * std::max(ne, 1LL)));
  DCG_TRY(cudaMemcpyAsync(s->d_lb_cells, cells.data(), sizeof(int4) * n, cudaMemcpyHostToDevice,
                          s->stream));
  if (nl > 0)
    DCG_TRY(cudaMemcpyAsync(s->d_lb_lines, plan.lines.data(), sizeof(int4) * nl,
                            cudaMemcpyHostToDevice, s->stream));
  if (ne > 0)
    DCG_TRY(cudaMemcpyAsync(s->d_lb_edge, plan.edge.data(), sizeof(int4) * ne,
                            cudaMemcpyHostToDevice, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  s->lb_cells = n;
  s->lb_lines = nl;
  s->lb_edge = ne;
  s->lb_layer = layer;
  s->lb_params = dc_gb300_mlp_device_params(mlp);
  return DC_GB300_OK;
}

extern "C" int dc_gb300_lb_sample(dc_gb300_sim *hw, dc_gb300_sim *ht, const long offset[3],
                                  int layer, float *samples, float *targets, long long cap,
                                  long long *count) {
  Sim *w = impl(hw), *t = impl(ht);
  if (!w || !t || !offset || !samples || !targets || !count)
    return fail(DC_GB300_ERR_ARG, "null argument");
  if (w->device != t->device) return fail(DC_GB300_ERR_ARG, "simulations on different devices");
  if (layer < 1 || layer > DC_GB300_MLP_DEPTHS)
    return fail(DC_GB300_ERR_ARG, "layer width must lie in [1, DC_GB300_MLP_DEPTHS]");
  if (offset[0] < 0 || offset[1] < 0 || offset[2] < 0 || offset[0] + t->sx > w->sx ||
      offset[1] + t->sy > w->sy || offset[2] + t->sz > w->sz)
    return fail(DC_GB300_ERR_ARG, "the thin box must lie inside the wide box");
  if (t->lb_cells > 0 || t->src_gi >= 0)
    return fail(DC_GB300_ERR_STATE, "the thin simulation must have no learned layer or source");
  DCG_TRY(cudaSetDevice(w->device));
  const std::vector<int4> cells = layer_cells(t->sx, t->sy, t->sz, layer);
  const long long n = static_cast<long long>(cells.size());
  if (n > cap) return fail(DC_GB300_ERR_ARG, "sample capacity too small");
  int wc = -1, wp = -1, tc = -1, tp = -1;
  if (!roles(w, &wc, &wp) || !roles(t, &tc, &tp))
    return fail(DC_GB300_ERR_STATE, "field pointers rearranged");
  const int off[3] = {static_cast<int>(offset[0]), static_cast<int>(offset[1]),
                      static_cast<int>(offset[2])};
  // both simulations run on their own streams: order the work explicitly
  DCG_TRY(cudaStreamSynchronize(w->stream));
  DCG_TRY(cudaStreamSynchronize(t->stream));
  // thin <- crop of the wide fields (as stored, i.e. with the wide source's
  // pending injection, which the wide step consumes identically)
  t->launches += 2;
  DCG_TRY(launch_crop(t->stream, t->pq[tc], t->sx, t->sy, t->sz, t->pitch, w->pq[wc], w->pitch,
                      w->plane, off));
  DCG_TRY(launch_crop(t->stream, t->pq[tp], t->sx, t->sy, t->sz, t->pitch, w->pq[wp], w->pitch,
                      w->plane, off));
  int rc = dc_gb300_run(ht, 1);
  if (rc != DC_GB300_OK) return rc;
  rc = dc_gb300_run(hw, 1);
  if (rc != DC_GB300_OK) return rc;
  DCG_TRY(cudaStreamSynchronize(w->stream));
  int4 *d_cells = nullptr;
  DCG_TRY(cudaMalloc(&d_cells, sizeof(int4) * n));
  cudaError_t e = cudaMemcpyAsync(d_cells, cells.data(), sizeof(int4) * n,
                                  cudaMemcpyHostToDevice, t->stream);
  // after the thin step: new field in buffer tp, time t in tc; wide t+1 in wp
  if (e == cudaSuccess)
    e = launch_lb_sample(t->stream, d_cells, n, t->pq[tp], t->pq[tc], t->pitch, t->plane,
                         w->pq[wp], w->pitch, w->plane, off, samples, targets);
  if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
  cudaFree(d_cells);
  if (e != cudaSuccess) return fail(DC_GB300_ERR_CUDA, std::string("lb_sample: ") + cudaGetErrorString(e));
  ++t->launches;
  *count = n;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_lb_rollout(dc_gb300_sim *hw, dc_gb300_sim *ht, const long offset[3],
                                   int steps, float *samples, float *targets, long long cap,
                                   long long *count) {
  Sim *w = impl(hw), *t = impl(ht);
  if (!w || !t || !offset || !samples || !targets || !count)
    return fail(DC_GB300_ERR_ARG, "null argument");
  if (w->device != t->device) return fail(DC_GB300_ERR_ARG, "simulations on different devices");
  if (t->lb_cells <= 0) return fail(DC_GB300_ERR_STATE, "the thin simulation has no learned layer");
  if (t->src_gi >= 0) return fail(DC_GB300_ERR_STATE, "the thin simulation must have no source");
  if (steps < 1) return fail(DC_GB300_ERR_ARG, "steps must be positive");
  if (offset[0] < 0 || offset[1] < 0 || offset[2] < 0 || offset[0] + t->sx > w->sx ||
      offset[1] + t->sy > w->sy || offset[2] + t->sz > w->sz)
    return fail(DC_GB300_ERR_ARG, "the thin box must lie inside the wide box");
  const long long n = t->lb_cells;
  if (n * steps > cap) return fail(DC_GB300_ERR_ARG, "sample capacity too small");
  DCG_TRY(cudaSetDevice(w->device));
  int wc = -1, wp = -1, tc = -1, tp = -1;
  if (!roles(w, &wc, &wp) || !roles(t, &tc, &tp))
    return fail(DC_GB300_ERR_STATE, "field pointers rearranged");
  const int off[3] = {static_cast<int>(offset[0]), static_cast<int>(offset[1]),
                      static_cast<int>(offset[2])};
  DCG_TRY(cudaStreamSynchronize(w->stream));
  DCG_TRY(cudaStreamSynchronize(t->stream));
  t->launches += 2;
  DCG_TRY(launch_crop(t->stream, t->pq[tc], t->sx, t->sy, t->sz, t->pitch, w->pq[wc], w->pitch,
                      w->plane, off));
  DCG_TRY(launch_crop(t->stream, t->pq[tp], t->sx, t->sy, t->sz, t->pitch, w->pq[wp], w->pitch,
                      w->plane, off));
  int rc = DC_GB300_OK;
  for (int j = 0; j < steps && rc == DC_GB300_OK; ++j) {
    float *rows = samples + static_cast<long long>(j) * n * 33;
    t->lb_rec = rows;
    rc = dc_gb300_run(ht, 1);
    t->lb_rec = nullptr;
    if (rc != DC_GB300_OK) break;
    DCG_TRY(cudaStreamSynchronize(t->stream));
    rc = dc_gb300_run(hw, 1);
    if (rc != DC_GB300_OK) break;
    roles(w, &wc, &wp);  // the new wide field is now the current one
    ++w->launches;
    DCG_TRY(launch_lb_target(w->stream, t->d_lb_cells, n, rows, w->pq[wc], w->pitch, w->plane,
                             off, targets + static_cast<long long>(j) * n * 2));
    DCG_TRY(cudaStreamSynchronize(w->stream));
  }
  if (rc != DC_GB300_OK) return rc;
  *count = n * steps;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_set_receivers(dc_gb300_sim *h, const long *index, int count,
                                      int max_steps) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  DCG_TRY(cudaSetDevice(s->device));
  drop_graphs(s);
  ++s->config_version;
  cudaFree(s->d_rec_col);
  cudaFree(s->d_rec_z);
  cudaFree(s->d_rec_r);
  cudaFree(s->d_traces);
  s->d_rec_col = nullptr;
  s->d_rec_z = s->d_rec_r = nullptr;
  s->d_traces = nullptr;
  s->nrec = 0;
  s->trace_cap = 0;
  if (count <= 0) return DC_GB300_OK;
  if (!index || max_steps <= 0) return fail(DC_GB300_ERR_ARG, "receivers invalid");
  // receivers sorted by column, then depth; each column gets its run
  struct Rec {
    long long col;
    int z, r;
  };
  std::vector<Rec> recs(count);
  for (int r = 0; r < count; ++r) {
    const long long i = index[r];
    const long long x = i % s->sx, y = (i / s->sx) % s->sy, z = i / (s->sx * s->sy);
    if (i < 0 || z >= s->sz || x < 4 || x >= s->sx - 4 || y < 4 || y >= s->sy - 4 || z < 4 ||
        z >= s->sz - 4)
      return fail(DC_GB300_ERR_ARG, "receivers must lie in the updated region [4, s-4)^3");
    recs[r] = Rec{y * s->sx + x, static_cast<int>(z), r};
  }
  std::sort(recs.begin(), recs.end(), [](const Rec &a, const Rec &b) {
    return a.col != b.col ? a.col < b.col : (a.z != b.z ? a.z < b.z : a.r < b.r);
  });
  std::vector<int2> col(static_cast<size_t>(s->sx * s->sy), make_int2(0, 0));
  std::vector<int> rz(count), rr(count);
  for (int k = 0; k < count; ++k) {
    int2 &c = col[recs[k].col];
    if (c.y == 0) c.x = k;
    ++c.y;
    rz[k] = recs[k].z;
    rr[k] = recs[k].r;
  }
  DCG_TRY(cudaMalloc(&s->d_rec_col, sizeof(int2) * col.size()));
  DCG_TRY(cudaMalloc(&s->d_rec_z, sizeof(int) * count));
  DCG_TRY(cudaMalloc(&s->d_rec_r, sizeof(int) * count));
  DCG_TRY(cudaMalloc(&s->d_traces, sizeof(float) * static_cast<size_t>(count) * max_steps));
  DCG_TRY(cudaMemcpyAsync(s->d_rec_col, col.data(), sizeof(int2) * col.size(),
                          cudaMemcpyHostToDevice, s->stream));
  DCG_TRY(cudaMemcpyAsync(s->d_rec_z, rz.data(), sizeof(int) * count, cudaMemcpyHostToDevice,
                          s->stream));
  DCG_TRY(cudaMemcpyAsync(s->d_rec_r, rr.data(), sizeof(int) * count, cudaMemcpyHostToDevice,
                          s->stream));
  DCG_TRY(cudaMemsetAsync(s->d_traces, 0, sizeof(float) * static_cast<size_t>(count) * max_steps,
                          s->stream));
  s->nrec = count;
  s->trace_cap = max_steps;
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_get_traces(dc_gb300_sim *h, float *out, int steps) {
  Sim *s = impl(h);
  if (!s || !out) return fail(DC_GB300_ERR_ARG, "null argument");
  if (steps < 0 || steps > s->trace_cap) return fail(DC_GB300_ERR_ARG, "steps beyond capacity");
  DCG_TRY(cudaSetDevice(s->device));
  DCG_TRY(cudaMemcpyAsync(out, s->d_traces, sizeof(float) * static_cast<size_t>(steps) * s->nrec,
                          cudaMemcpyDeviceToHost, s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_enable_energy(dc_gb300_sim *h, int max_steps) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  DCG_TRY(cudaSetDevice(s->device));
  drop_graphs(s);
  ++s->config_version;
  cudaFree(s->d_energy);
  s->d_energy = nullptr;
  s->energy_cap = 0;
  if (max_steps <= 0) return DC_GB300_OK;
  DCG_TRY(cudaMalloc(&s->d_energy, sizeof(double) * max_steps));
  DCG_TRY(cudaMemsetAsync(s->d_energy, 0, sizeof(double) * max_steps, s->stream));
  s->energy_cap = max_steps;
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_get_energy(dc_gb300_sim *h, double *out, int steps) {
  Sim *s = impl(h);
  if (!s || !out) return fail(DC_GB300_ERR_ARG, "null argument");
  if (steps < 0 || steps > s->energy_cap) return fail(DC_GB300_ERR_ARG, "steps beyond capacity");
  DCG_TRY(cudaSetDevice(s->device));
  DCG_TRY(cudaMemcpyAsync(out, s->d_energy, sizeof(double) * steps, cudaMemcpyDeviceToHost,
                          s->stream));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return DC_GB300_OK;
}

namespace {

// Captures kGraphChunk steps (+ the step-counter advance) into a graph.
int capture_chunk(Sim *s, cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  DCG_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  const dc_device_data saved = s->handle->abi;
  const long long saved_launches = s->launches;
  cudaError_t e = cudaSuccess;
  for (int j = 0; j < kGraphChunk && e == cudaSuccess; ++j) e = queue_step(s, j);
  if (e == cudaSuccess) e = launch_advance_step(s->stream, s->d_step, kGraphChunk);
  cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
  // capture only recorded the work: restore the roles and counters
  s->handle->abi = saved;
  s->launches = saved_launches;
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(DC_GB300_ERR_CUDA, std::string("graph capture failed: ") +
                                       cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return fail(DC_GB300_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return DC_GB300_OK;
}

}  // namespace

extern "C" int dc_gb300_run(dc_gb300_sim *h, int steps) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  if (steps < 0) return fail(DC_GB300_ERR_ARG, "negative step count");
  if (steps == 0) return DC_GB300_OK;
  DCG_TRY(cudaSetDevice(s->device));
  int cur0 = -1, prev0 = -1;
  if (!roles(s, &cur0, &prev0)) return fail(DC_GB300_ERR_STATE, "field pointers rearranged");
  if (s->kernel == DC_GB300_KERNEL_FAST) {
    const int rc = refresh_narrow(s);
    if (rc != DC_GB300_OK) return rc;
  }
  if (s->energy_cap > 0 && s->steps_done + steps > s->energy_cap)
    return fail(DC_GB300_ERR_ARG, "run exceeds the energy capacity");
  if (s->nrec > 0 && s->steps_done + steps > s->trace_cap)
    return fail(DC_GB300_ERR_ARG, "run exceeds the trace capacity");
  // The source of the first step of this run goes in before the stencil
  // (src/worker.c:467-470); later ones are fused into the previous store.
  if (s->src_gi >= 0 && s->src_applied_step != s->steps_done) {
    ++s->launches;
    DCG_TRY(launch_add_source(s->stream, reinterpret_cast<float2 *>(h->abi.pc), s->src_gi,
                              s->d_src, s->src_count, s->d_step, 0));
  }
  int left = steps;
  while (left >= kGraphChunk) {
    int cur = -1, prev = -1;
    roles(s, &cur, &prev);
    const int slot = cur;  // graphs are keyed by the buffer holding pc
    if (!s->graph[slot] || s->graph_version[slot] != s->config_version ||
        s->graph_pc[slot] != cur) {
      if (s->graph[slot]) cudaGraphExecDestroy(s->graph[slot]);
      s->graph[slot] = nullptr;
      int rc = capture_chunk(s, &s->graph[slot]);
      if (rc != DC_GB300_OK) return rc;
      s->graph_version[slot] = s->config_version;
      s->graph_pc[slot] = cur;
    }
    DCG_TRY(cudaGraphLaunch(s->graph[slot], s->stream));
    s->launches += kGraphChunk * launches_per_step(s) + 1;
    // kGraphChunk is even: the roles are back where they started
    left -= kGraphChunk;
    s->steps_done += kGraphChunk;
  }
  for (int j = 0; j < left; ++j) DCG_TRY(queue_step(s, j));
  if (left > 0) {
    ++s->launches;
    DCG_TRY(launch_advance_step(s->stream, s->d_step, left));
    s->steps_done += left;
  }
  if (s->src_gi >= 0) s->src_applied_step = s->steps_done;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_synchronize(dc_gb300_sim *h) {
  Sim *s = impl(h);
  if (!s) return fail(DC_GB300_ERR_ARG, "null simulation");
  DCG_TRY(cudaSetDevice(s->device));
  DCG_TRY(cudaStreamSynchronize(s->stream));
  return check_err_word(s);
}

extern "C" int dc_gb300_propagate_box(dc_gb300_sim *h, const size_t start[3],
                                      const size_t end[3]) {
  Sim *s = impl(h);
  if (!s || !start || !end) return fail(DC_GB300_ERR_ARG, "null argument");
  const long long lim[3] = {s->sx, s->sy, s->sz};
  long long b0[3], b1[3];
  for (int d = 0; d < 3; ++d) {
    if (end[d] <= start[d]) return DC_GB300_OK;  // empty box: nothing to do
    b0[d] = static_cast<long long>(start[d]);
    b1[d] = static_cast<long long>(end[d]);
    if (b0[d] < 4 || b1[d] > lim[d] - 4)
      return fail(DC_GB300_ERR_ARG, "box outside the updatable region [4, size-4)");
  }
  int cur = -1, prev = -1;
  if (!roles(s, &cur, &prev))
    return fail(DC_GB300_ERR_STATE, "field pointers do not belong to this simulation");
  DCG_TRY(cudaSetDevice(s->device));
  if (s->kernel == DC_GB300_KERNEL_FAST) {
    const int rc = refresh_narrow(s);
    if (rc != DC_GB300_OK) return rc;
  }
  StepParams p = make_params(s, b0, b1, s->dx, s->dy, s->dz, s->dt);
  DCG_TRY(launch_pass(s, p));
  return DC_GB300_OK;
}

// ===========================================================================
// The reference's device-data and propagate entry points
// (include/device_data.h, include/propagate.h)
// ===========================================================================

extern "C" dc_device_data *dc_device_data_init(dc_process_t *process) {
  if (!process) {
    set_error("null process");
    abi_die("dc_device_data_init");
  }
  dc_gb300_config cfg{};
  cfg.sx = static_cast<long>(process->sizes[0]);
  cfg.sy = static_cast<long>(process->sizes[1]);
  cfg.sz = static_cast<long>(process->sizes[2]);
  cfg.dx = process->dx;
  cfg.dy = process->dy;
  cfg.dz = process->dz;
  cfg.dt = process->dt;
  cfg.kernel = env_is("DC_GB300_KERNEL", "exact") ? DC_GB300_KERNEL_EXACT : DC_GB300_KERNEL_FAST;
  cfg.medium = env_is("DC_GB300_MEDIUM", "vpz_vsv")        ? DC_GB300_MEDIUM_VPZ_VSV
               : env_is("DC_GB300_MEDIUM", "precomp_f16")  ? DC_GB300_MEDIUM_PRECOMP_F16
               : env_is("DC_GB300_MEDIUM", "precomp_bf16") ? DC_GB300_MEDIUM_PRECOMP_BF16
                                                          : DC_GB300_MEDIUM_PRECOMP;
  const char *dev = std::getenv("DC_GB300_DEVICE");
  cfg.device = dev ? std::atoi(dev) : 0;
  // dt etc. may be left 0 by callers that pass them to dc_propagate only
  if (!(cfg.dx > 0)) cfg.dx = 1;
  if (!(cfg.dy > 0)) cfg.dy = 1;
  if (!(cfg.dz > 0)) cfg.dz = 1;
  if (!(cfg.dt > 0)) cfg.dt = 1;
  dc_gb300_sim *h = nullptr;
  if (dc_gb300_create(&cfg, &h) != DC_GB300_OK) abi_die("dc_device_data_init");
  int rc = DC_GB300_OK;
  if (cfg.medium != DC_GB300_MEDIUM_VPZ_VSV) {
    if (process->precomp_vars.ch1dxx)
      rc = dc_gb300_set_precomp(h, &process->precomp_vars);
    else
      rc = dc_gb300_set_anisotropy(h, &process->anisotropy_vars);
  } else {
    rc = dc_gb300_set_vpz_vsv(h, process->anisotropy_vars.vpz, process->anisotropy_vars.vsv);
  }
  if (rc == DC_GB300_OK)
    rc = dc_gb300_set_fields(h, process->pp, process->pc, process->qp, process->qc);
  if (rc != DC_GB300_OK) {
    const std::string msg = g_err;
    dc_gb300_destroy(h);
    set_error(msg);
    abi_die("dc_device_data_init");
  }
  return &h->abi;
}

extern "C" void dc_device_data_free(dc_device_data *data) {
  dc_gb300_destroy(dc_gb300_from_device_data(data));
}

extern "C" void dc_device_data_get_results(dc_process_t *process, dc_device_data *data) {
  dc_gb300_sim *h = dc_gb300_from_device_data(data);
  if (!process || !h) {
    set_error("null argument");
    abi_die("dc_device_data_get_results");
  }
  if (dc_gb300_synchronize(h) != DC_GB300_OK ||
      dc_gb300_get_fields(h, nullptr, process->pc, nullptr, process->qc) != DC_GB300_OK)
    abi_die("dc_device_data_get_results");
}

extern "C" void dc_device_swap_arrays(dc_device_data *data) {
  // src/device_data.cu:119-129
  std::swap(data->pp, data->pc);
  std::swap(data->qp, data->qc);
}

extern "C" void dc_device_add_source(dc_device_data *data, size_t index, float source) {
  dc_gb300_sim *h = dc_gb300_from_device_data(data);
  Sim *s = impl(h);
  const long long n = s->sx * s->sy * s->sz;
  if (static_cast<long long>(index) >= n) {
    set_error("source index out of range");
    abi_die("dc_device_add_source");
  }
  const long long i = static_cast<long long>(index);
  const long long x = i % s->sx, y = (i / s->sx) % s->sy, z = i / (s->sx * s->sy);
  int cur = -1, prev = -1;
  if (!roles(s, &cur, &prev)) {
    set_error("field pointers rearranged");
    abi_die("dc_device_add_source");
  }
  ++s->launches;
  cudaError_t e = launch_add_value(s->stream, s->pq[cur], z * s->plane + y * s->pitch + x,
                                   source);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    abi_die("dc_device_add_source");
  }
}

extern "C" void dc_propagate(const size_t start_coords[3], const size_t end_coords[3],
                             const size_t sizes[3], const int *, const int *,
                             dc_device_data *data, const float dx, const float dy,
                             const float dz, const float dt) {
  dc_gb300_sim *h = dc_gb300_from_device_data(data);
  Sim *s = impl(h);
  if (!s || !sizes || static_cast<long long>(sizes[0]) != s->sx ||
      static_cast<long long>(sizes[1]) != s->sy || static_cast<long long>(sizes[2]) != s->sz) {
    set_error("sizes differ from the ones given to dc_device_data_init");
    abi_die("dc_propagate");
  }
  // the step sizes come with every call, as in the reference
  s->dx = dx;
  s->dy = dy;
  s->dz = dz;
  s->dt = dt;
  if (dc_gb300_propagate_box(h, start_coords, end_coords) != DC_GB300_OK)
    abi_die("dc_propagate");
}

namespace {
void halo_copy(dc_device_data *data, float *host, const size_t start[3], const size_t end[3],
               const size_t sizes[3], float *dev, bool to_host, const char *where) {
  Sim *s = impl(dc_gb300_from_device_data(data));
  if (!s || !host || !dev || !start || !end || !sizes) {
    set_error("null argument");
    abi_die(where);
  }
  const long long lim[3] = {s->sx, s->sy, s->sz};
  for (int d = 0; d < 3; ++d)
    if (end[d] < start[d] || static_cast<long long>(end[d]) > lim[d] ||
        static_cast<long long>(sizes[d]) != lim[d]) {
      set_error("box outside the array or sizes differ");
      abi_die(where);
    }
  int comp = 0;
  const int b = component_of(s, dev, &comp);
  if (b < 0) {
    set_error("array does not belong to this simulation");
    abi_die(where);
  }
  const long long b0[3] = {static_cast<long long>(start[0]), static_cast<long long>(start[1]),
                           static_cast<long long>(start[2])};
  const long long b1[3] = {static_cast<long long>(end[0]), static_cast<long long>(end[1]),
                           static_cast<long long>(end[2])};
  const long long n = (b1[0] - b0[0]) * (b1[1] - b0[1]) * (b1[2] - b0[2]);
  if (n == 0) return;
  float *stage = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n, s->stream);
  if (e == cudaSuccess && !to_host)
    e = cudaMemcpyAsync(stage, host, sizeof(float) * n, cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess)
    e = launch_box_copy(s->stream, s->pq[b], comp, stage, b0, b1, s->pitch, s->plane, to_host);
  if (e == cudaSuccess && to_host)
    e = cudaMemcpyAsync(host, stage, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream);
  if (stage) cudaFreeAsync(stage, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    abi_die(where);
  }
}
}  // namespace

extern "C" void dc_device_extract_halo_face(dc_device_data *data, float *buffer,
                                            const size_t start_coords[3],
                                            const size_t end_coords[3], const size_t sizes[3],
                                            const float *from_array) {
  halo_copy(data, buffer, start_coords, end_coords, sizes, const_cast<float *>(from_array), true,
            "dc_device_extract_halo_face");
}

extern "C" void dc_device_insert_halo_face(dc_device_data *data, const float *buffer,
                                           const size_t start_coords[3],
                                           const size_t end_coords[3], const size_t sizes[3],
                                           float *to_array) {
  halo_copy(data, const_cast<float *>(buffer), start_coords, end_coords, sizes, to_array, false,
            "dc_device_insert_halo_face");
}

// dc_compute_precomp_vars on the GPU (FP64 trig), returned as host arrays.
extern "C" dc_precomp_vars dc_compute_precomp_vars(int sx, int sy, int sz,
                                                   dc_anisotropy_t anisotropy) {
  dc_precomp_vars v{};
  const long long n = static_cast<long long>(sx) * sy * sz;
  float **dst[10] = {&v.ch1dxx, &v.ch1dyy, &v.ch1dzz, &v.ch1dxy, &v.ch1dyz,
                     &v.ch1dxz, &v.v2px,   &v.v2pz,   &v.v2sz,   &v.v2pn};
  for (float **d : dst) {
    *d = static_cast<float *>(std::malloc(sizeof(float) * std::max<long long>(n, 1)));
    if (!*d) {
      set_error("OOM in dc_compute_precomp_vars");
      abi_die("dc_compute_precomp_vars");
    }
  }
  if (n == 0) return v;
  cudaStream_t st = nullptr;
  float *grouped = nullptr, *stage = nullptr;
  if (cudaStreamCreate(&st) != cudaSuccess ||
      cudaMallocAsync(reinterpret_cast<void **>(&grouped), sizeof(float) * n * DC_NCOEF, st) !=
          cudaSuccess ||
      cudaMallocAsync(reinterpret_cast<void **>(&stage), sizeof(float) * n, st) != cudaSuccess) {
    set_error("CUDA set-up failed in dc_compute_precomp_vars");
    abi_die("dc_compute_precomp_vars");
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      precompute_dense(st, dev, &anisotropy, n, grouped) != DC_GB300_OK)
    abi_die("dc_compute_precomp_vars");
  for (int k = 0; k < 10; ++k)
    if (launch_coef_component(st, grouped, stage, kRefOrder[k], sx, sy, sz, sx, n, false) !=
            cudaSuccess ||
        cudaMemcpyAsync(*dst[k], stage, sizeof(float) * n, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess) {
      set_error("copy-back failed in dc_compute_precomp_vars");
      abi_die("dc_compute_precomp_vars");
    }
  cudaFreeAsync(grouped, st);
  cudaFreeAsync(stage, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    set_error("dc_compute_precomp_vars kernel failed");
    abi_die("dc_compute_precomp_vars");
  }
  cudaStreamDestroy(st);
  return v;
}

// ---------------------------------------------------------------------------
// The exact stencil over caller-owned device buffers, with no device
// allocation at all.
//
// Some callers cannot call cudaMalloc: applications that own every byte of
// device memory themselves (a pre-sized pool, buffers registered once with a
// communication library) and time loops that must not allocate between
// steps.  dc_gb300_exact_steps_noalloc serves them: the wavefields and the
// medium are the caller's device buffers, and the only other memory the
// kernel needs -- the per-step energy accumulators and the step counter --
// is the file-scope array below, a fixed 33 KB per device.
namespace {

// Largest number of steps one call may run: one double energy accumulator
// per step.
constexpr int kNoAllocMaxSteps = 4096;
constexpr size_t kEnergyBytes = sizeof(double) * kNoAllocMaxSteps;
constexpr size_t kScratchBytes = kEnergyBytes + 256;  // + step counter

// Shared by every call on a device; keeps the last call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array, looked up once per device with that
// device current.
int scratch_for(int dev, void **ptr) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return dcg::fail(DC_GB300_ERR_CUDA,
                  std::string("cudaGetSymbolAddress(no-allocation scratch): ") +
                      cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *ptr = g_scratch_ptr[dev];
  return DC_GB300_OK;
}

int run_steps(const dc_gb300_config *cfg, int dev, float *pairs[2], const float *medium,
              int steps, double *energy, cudaStream_t stream) {
  void *scratch = nullptr;
  const int rc = scratch_for(dev, &scratch);
  if (rc != DC_GB300_OK) return rc;
  double *e_dev = static_cast<double *>(scratch);
  int *step_dev = reinterpret_cast<int *>(static_cast<unsigned char *>(scratch) + kEnergyBytes);

#define NOALLOC_TRY(call)                                                     \
  do {                                                                        \
    const cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess)                                                    \
      return dcg::fail(DC_GB300_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

  // the accumulators of this call and the step counter start at zero
  NOALLOC_TRY(cudaMemsetAsync(e_dev, 0, sizeof(double) * steps, stream));
  NOALLOC_TRY(cudaMemsetAsync(step_dev, 0, sizeof(int), stream));

  // A host-only description of the caller's buffers, enough for the
  // library's own parameter set-up and exact-kernel launcher.
  dc_gb300_sim handle{};
  dcg::Sim sim;
  sim.handle = &handle;
  handle.impl = &sim;
  sim.device = dev;
  sim.sx = cfg->sx;
  sim.sy = cfg->sy;
  sim.sz = cfg->sz;
  sim.pitch = (static_cast<long long>(cfg->sx) + 3) / 4 * 4;
  sim.plane = sim.pitch * cfg->sy;
  sim.count = sim.plane * cfg->sz;
  sim.kernel = DC_GB300_KERNEL_EXACT;
  sim.medium = cfg->medium;
  sim.stream = stream;
  if (cfg->medium == DC_GB300_MEDIUM_PRECOMP)
    sim.coef = const_cast<float *>(medium);
  else
    sim.vv = const_cast<float *>(medium);
  sim.d_step = step_dev;

  const long long b0[3] = {4, 4, 4};
  const long long b1[3] = {cfg->sx - 4, cfg->sy - 4, cfg->sz - 4};
  for (int j = 0; j < steps; ++j) {
    handle.abi.pp = pairs[0];
    handle.abi.qp = pairs[0] + 1;
    handle.abi.pc = pairs[1];
    handle.abi.qc = pairs[1] + 1;
    dcg::StepParams prm = dcg::make_params(&sim, b0, b1, cfg->dx, cfg->dy, cfg->dz, cfg->dt);
    prm.energy = energy ? e_dev : nullptr;
    prm.energy_cap = steps;
    prm.step_offset = j;
    NOALLOC_TRY(dcg::launch_exact(&sim, prm));
    float *t = pairs[0];  // the new field was written over the previous one
    pairs[0] = pairs[1];
    pairs[1] = t;
  }
  if (energy)
    NOALLOC_TRY(cudaMemcpyAsync(energy, e_dev, sizeof(double) * steps, cudaMemcpyDeviceToHost,
                                stream));
  NOALLOC_TRY(cudaStreamSynchronize(stream));
#undef NOALLOC_TRY
  return DC_GB300_OK;
}

}  // namespace

extern "C" int dc_gb300_exact_steps_noalloc(const dc_gb300_config *cfg, float *pairs[2],
                                            const float *medium, int steps, double *energy,
                                            void *stream) {
  if (!cfg || !pairs || !pairs[0] || !pairs[1] || !medium)
    return dcg::fail(DC_GB300_ERR_ARG, "null argument");
  if (steps < 0) return dcg::fail(DC_GB300_ERR_ARG, "negative step count");
  if (steps > kNoAllocMaxSteps)
    return dcg::fail(DC_GB300_ERR_ARG,
                "dc_gb300_exact_steps_noalloc: " + std::to_string(steps) +
                    " steps exceed the no-allocation scratch maximum of " +
                    std::to_string(kNoAllocMaxSteps) + " steps per call");
  if (cfg->sx < 9 || cfg->sy < 9 || cfg->sz < 9)
    return dcg::fail(DC_GB300_ERR_ARG, "every padded size must be at least 9");
  if (cfg->sx > (1 << 30) || cfg->sy > (1 << 30) || cfg->sz > (1 << 30))
    return dcg::fail(DC_GB300_ERR_ARG, "size too large");
  if (cfg->kernel != DC_GB300_KERNEL_EXACT)
    return dcg::fail(DC_GB300_ERR_ARG, "dc_gb300_exact_steps_noalloc runs the exact kernel only");
  if (cfg->medium != DC_GB300_MEDIUM_PRECOMP && cfg->medium != DC_GB300_MEDIUM_VPZ_VSV)
    return dcg::fail(DC_GB300_ERR_ARG,
                "dc_gb300_exact_steps_noalloc takes the precomp or vpz/vsv medium form");
  if (!(cfg->dx > 0 && cfg->dy > 0 && cfg->dz > 0 && cfg->dt > 0))
    return dcg::fail(DC_GB300_ERR_ARG, "dx, dy, dz and dt must be positive");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return dcg::fail(DC_GB300_ERR_DEVICE, "no CUDA device");
  int dev = cfg->device;
  int prev_dev = 0;
  if (cudaGetDevice(&prev_dev) != cudaSuccess) return dcg::fail(DC_GB300_ERR_CUDA, "cudaGetDevice");
  if (dev < 0) dev = prev_dev;
  if (dev >= ndev || dev >= kMaxDevices)
    return dcg::fail(DC_GB300_ERR_DEVICE, "device ordinal out of range");
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3)
    return dcg::fail(DC_GB300_ERR_DEVICE, "this build targets sm_103a");
  if (cudaSetDevice(dev) != cudaSuccess) return dcg::fail(DC_GB300_ERR_CUDA, "cudaSetDevice");
  // every call synchronises its stream and reads the energy back, neither
  // of which a capture allows: refuse before touching the capture
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess ||
      cap != cudaStreamCaptureStatusNone) {
    cudaSetDevice(prev_dev);
    return dcg::fail(DC_GB300_ERR_ARG,
                     "dc_gb300_exact_steps_noalloc cannot run on a capturing stream");
  }
  const int rc = run_steps(cfg, dev, pairs, medium, steps, energy,
                           static_cast<cudaStream_t>(stream));
  cudaSetDevice(prev_dev);
  return rc;
}
