// dc_aux.cu -- small kernels around the stencil: source injection, receiver
// gather, step counter, the FP64 medium precompute and the seeded layered
// medium generator; plus tensor-map encoding.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "dc_internal.h"

namespace dcg {
namespace {

__global__ void add_source_kernel(float2 *cur, long long gi, const float *table,
                                  int count, const int *d_step,
                                  int step_offset) {
  // src/device_data.cu:131-139 with the amplitude looked up on the device
  const int step = *d_step + step_offset;
  const float s = (step >= 0 && step < count) ? table[step] : 0.0f;
  float2 v = cur[gi];
  v.x = __fadd_rn(v.x, s);
  v.y = __fadd_rn(v.y, s);
  cur[gi] = v;
}

__global__ void add_value_kernel(float2 *cur, long long gi, float s) {
  float2 v = cur[gi];
  v.x = __fadd_rn(v.x, s);
  v.y = __fadd_rn(v.y, s);
  cur[gi] = v;
}

__global__ void gather_kernel(const float2 *f, const long long *idx, int n,
                              float *traces, int cap, const int *d_step,
                              int step_offset, long long src_gi,
                              const float *src_pre) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int step = *d_step + step_offset;
  if (r >= n || step < 0 || step >= cap) return;
  const long long i = idx[r];
  // the source point already holds the next step's source: record the value
  // the stencil produced, as the reference sees it after the swap
  traces[static_cast<long long>(step) * n + r] =
      (i == src_gi && src_pre) ? src_pre[0] : f[i].x;
}

__global__ void pack_kernel(float2 *dst, const float *p, const float *q,
                            long long sx, long long sy, long long n,
                            long long pitch) {
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; d < n;
       d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = d % sx, yz = d / sx;
    dst[yz * pitch + x] = make_float2(p ? p[d] : 0.0f, q ? q[d] : 0.0f);
  }
}

__global__ void unpack_kernel(const float2 *src, float *p, float *q, long long sx,
                              long long sy, long long n, long long pitch) {
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; d < n;
       d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = d % sx, yz = d / sx;
    const float2 v = src[yz * pitch + x];
    if (p) p[d] = v.x;
    if (q) q[d] = v.y;
  }
}

__global__ void box_copy_kernel(float2 *pairs, int comp, float *dense, long long bx,
                                long long by, long long bz, long long wx, long long wy,
                                long long n, long long pitch, long long plane,
                                bool to_dense) {
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; d < n;
       d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = d % wx, y = (d / wx) % wy, z = d / (wx * wy);
    float *e = reinterpret_cast<float *>(pairs + (bz + z) * plane + (by + y) * pitch + bx + x) + comp;
    if (to_dense)
      dense[d] = *e;
    else
      *e = dense[d];
  }
}

__global__ void advance_kernel(int *d_step, int by) { *d_step += by; }

// src/precomp.c:85-105 on the GPU: libm-style double trig rounded to float,
// float products (no contraction), v2px/v2pn scaled in double.
__device__ __forceinline__ void precomp_point(float theta, float phi,
                                              float vsv, float vpz, float eps,
                                              float delta, float out[10]) {
  const float st = static_cast<float>(sin(static_cast<double>(theta)));
  const float ct = static_cast<float>(cos(static_cast<double>(theta)));
  const float s2t = static_cast<float>(sin(__dmul_rn(2.0, static_cast<double>(theta))));
  const float sp = static_cast<float>(sin(static_cast<double>(phi)));
  const float cp = static_cast<float>(cos(static_cast<double>(phi)));
  const float s2p = static_cast<float>(sin(__dmul_rn(2.0, static_cast<double>(phi))));
  out[DC_CXX] = __fmul_rn(__fmul_rn(__fmul_rn(st, st), cp), cp);
  out[DC_CYY] = __fmul_rn(__fmul_rn(__fmul_rn(st, st), sp), sp);
  out[DC_CZZ] = __fmul_rn(ct, ct);
  out[DC_CXY] = __fmul_rn(__fmul_rn(st, st), s2p);
  out[DC_CYZ] = __fmul_rn(s2t, sp);
  out[DC_CXZ] = __fmul_rn(s2t, cp);
  const float v2sz = __fmul_rn(vsv, vsv);
  const float v2pz = __fmul_rn(vpz, vpz);
  out[DC_V2SZ] = v2sz;
  out[DC_V2PZ] = v2pz;
  out[DC_V2PX] = static_cast<float>(__dmul_rn(
      static_cast<double>(v2pz), __dadd_rn(1.0, __dmul_rn(2.0, static_cast<double>(eps)))));
  out[DC_V2PN] = static_cast<float>(__dmul_rn(
      static_cast<double>(v2pz), __dadd_rn(1.0, __dmul_rn(2.0, static_cast<double>(delta)))));
}

// Dense input arrays (n points) -> coefficient block at the same dense
// index (the caller repacks to the pitched layout).
__global__ void precomp_kernel(const float *theta, const float *phi,
                               const float *vsv, const float *vpz,
                               const float *eps, const float *delta,
                               float *coef, long long count, long long n) {
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
       d < n; d += static_cast<long long>(gridDim.x) * blockDim.x) {
    float out[10];
    precomp_point(theta[d], phi[d], vsv[d], vpz[d], eps[d], delta[d], out);
#pragma unroll
    for (int k = 0; k < 10; ++k) coef[k * count + d] = out[k];
  }
}

// Random-Fourier-feature Gaussian field: sqrt(2/m) * sum cos(k.r + ph).
__device__ __forceinline__ double rff(const float (*k)[4], int m, double x,
                                      double y, double z) {
  double s = 0.0;
  for (int j = 0; j < m; ++j)
    s += cos(static_cast<double>(k[j][0]) * x + static_cast<double>(k[j][1]) * y +
             static_cast<double>(k[j][2]) * z + static_cast<double>(k[j][3]));
  return m > 0 ? s * sqrt(2.0 / m) : 0.0;
}

__global__ void layered_kernel(const dc_gb300_layered_spec spec_v, float *coef,
                               float *vv, long long sx, long long sy,
                               long long sz, long long pitch,
                               long long count) {
  const dc_gb300_layered_spec *spec = &spec_v;  // read from parameter space
  const long long n = sx * sy * sz;
  const long long plane = pitch * sy;
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
       d < n; d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = d % sx, y = (d / sx) % sy, z = d / (sx * sy);
    const double gx = static_cast<double>(spec->ox + x);
    const double gy = static_cast<double>(spec->oy + y);
    const double gz = static_cast<double>(spec->oz + z);
    int l = 0;
    while (l + 1 < spec->nlayers && gz >= spec->layer_top[l + 1]) ++l;
    const double fn = rff(spec->k_noise, spec->n_noise, gx, gy, gz);
    const double ft = rff(spec->k_theta, spec->n_theta, gx, gy, gz);
    const double fp = rff(spec->k_phi, spec->n_phi, gx, gy, gz);
    // Gaussian -> uniform marginal through the normal CDF
    const double ut = 0.5 * erfc(-ft * 0.70710678118654752440);
    const double up = 0.5 * erfc(-fp * 0.70710678118654752440);
    const float vp = static_cast<float>(static_cast<double>(spec->vp[l]) *
                                        (1.0 + static_cast<double>(spec->vp_noise) * fn));
    const float theta = static_cast<float>(spec->theta_lo + (spec->theta_hi - spec->theta_lo) * ut);
    const float phi = static_cast<float>(spec->phi_lo + (spec->phi_hi - spec->phi_lo) * up);
    const float e = spec->epsilon[l], dl = spec->delta[l];
    const float vs = __fmul_rn(vp, sqrtf(__fdiv_rn(fabsf(__fsub_rn(e, dl)), spec->sigma_ratio)));
    const long long pi = z * plane + y * pitch + x;
    if (coef) {
      float out[10];
      precomp_point(theta, phi, vs, vp, e, dl, out);
#pragma unroll
      for (int k = 0; k < 10; ++k) coef[k * count + pi] = out[k];
    }
    if (vv) {
      vv[pi] = vp;
      vv[count + pi] = vs;
    }
  }
}

}  // namespace

cudaError_t launch_add_source(cudaStream_t st, float2 *cur, long long gi,
                              const float *table, int count, const int *d_step,
                              int step_offset) {
  add_source_kernel<<<1, 1, 0, st>>>(cur, gi, table, count, d_step, step_offset);
  return cudaGetLastError();
}

cudaError_t launch_add_value(cudaStream_t st, float2 *cur, long long gi, float value) {
  add_value_kernel<<<1, 1, 0, st>>>(cur, gi, value);
  return cudaGetLastError();
}

cudaError_t launch_gather(cudaStream_t st, const float2 *f, const long long *idx, int n,
                          float *traces, int cap, const int *d_step, int step_offset,
                          long long src_gi, const float *src_pre) {
  gather_kernel<<<(n + 127) / 128, 128, 0, st>>>(f, idx, n, traces, cap, d_step,
                                                 step_offset, src_gi, src_pre);
  return cudaGetLastError();
}

namespace {
int grid_for(long long n) {
  return static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)));
}
}  // namespace

cudaError_t launch_pack(cudaStream_t st, float2 *dst, const float *p, const float *q,
                        long long sx, long long sy, long long sz, long long pitch) {
  const long long n = sx * sy * sz;
  pack_kernel<<<grid_for(n), 256, 0, st>>>(dst, p, q, sx, sy, n, pitch);
  return cudaGetLastError();
}

cudaError_t launch_unpack(cudaStream_t st, const float2 *src, float *p, float *q,
                          long long sx, long long sy, long long sz, long long pitch) {
  const long long n = sx * sy * sz;
  unpack_kernel<<<grid_for(n), 256, 0, st>>>(src, p, q, sx, sy, n, pitch);
  return cudaGetLastError();
}

cudaError_t launch_box_copy(cudaStream_t st, float2 *pairs, int comp, float *dense,
                            const long long b0[3], const long long b1[3], long long pitch,
                            long long plane, bool to_dense) {
  const long long wx = b1[0] - b0[0], wy = b1[1] - b0[1], wz = b1[2] - b0[2];
  const long long n = wx * wy * wz;
  if (n <= 0) return cudaSuccess;
  box_copy_kernel<<<grid_for(n), 256, 0, st>>>(pairs, comp, dense, b0[0], b0[1], b0[2], wx, wy,
                                               n, pitch, plane, to_dense);
  return cudaGetLastError();
}

cudaError_t launch_advance_step(cudaStream_t st, int *d_step, int by) {
  advance_kernel<<<1, 1, 0, st>>>(d_step, by);
  return cudaGetLastError();
}

cudaError_t launch_precomp(cudaStream_t st, const float *theta,
                           const float *phi, const float *vsv,
                           const float *vpz, const float *eps,
                           const float *delta, float *coef, long long count,
                           long long n) {
  const int blocks = static_cast<int>(std::min<long long>((n + 255) / 256, 152 * 16));
  precomp_kernel<<<blocks, 256, 0, st>>>(theta, phi, vsv, vpz, eps, delta, coef, count, n);
  return cudaGetLastError();
}

cudaError_t launch_layered(cudaStream_t st, const dc_gb300_layered_spec &spec,
                           float *coef, float *vv, long long sx, long long sy,
                           long long sz, long long pitch, long long count) {
  const long long n = sx * sy * sz;
  const int blocks = static_cast<int>(std::min<long long>((n + 255) / 256, 152 * 32));
  layered_kernel<<<blocks, 256, 0, st>>>(spec, coef, vv, sx, sy, sz, pitch, count);
  return cudaGetLastError();
}

bool encode_tiled(CUtensorMap *map, const void *base, int rank,
                  const uint64_t *dims, const uint64_t *strides_bytes,
                  const uint32_t *box, std::string *err, bool pairs) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  static cudaError_t lookup_err = cudaSuccess;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    lookup_err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                  cudaEnableDefault, &q);
    if (lookup_err == cudaSuccess && q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  if (!fn) {
    *err = "cuTensorMapEncodeTiled entry point unavailable";
    return false;
  }
  cuuint32_t elem_strides[5] = {1, 1, 1, 1, 1};
  // (p, q) pairs travel as opaque 8-byte elements
  const CUtensorMapDataType dt =
      pairs ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  CUresult r = fn(map, dt, rank, const_cast<void *>(base),
                  dims, strides_bytes, box, elem_strides, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d)", static_cast<int>(r));
    *err = buf;
    return false;
  }
  return true;
}

}  // namespace dcg
