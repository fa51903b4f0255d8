// dc_aux.cu -- small kernels around the stencil: source injection, receiver
// gather, step counter, the FP64 medium precompute and the seeded layered
// medium generator; plus tensor-map encoding.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <cstdint>

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
    for (int k = 0; k < 10; ++k) coef[coef_index(k, d, count)] = out[k];
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
      for (int k = 0; k < 10; ++k) coef[coef_index(k, pi, count)] = out[k];
    }
    if (vv) {
      vv[2 * pi] = vp;
      vv[2 * pi + 1] = vs;
    }
  }
}

// ---- the reference medium on the GPU ------------------------------------
// glibc's rand_r (stdlib/rand_r.c, glibc 2.39 here) advances the linear
// congruential generator x -> 1103515245 x + 12345 (mod 2^32) three times per
// call and returns bits 16..26, then 16..25 twice, of the three states,
// concatenated (11 + 10 + 10 bits).  The reference's boundary sweep
// (src/boundary.c:25-35) makes exactly one call per shell cell in global
// z, y, x order, so the generator state before a cell's call is the seed
// advanced by 3 * (number of shell cells before it), reached here by affine
// skip-ahead instead of a serial sweep.
struct Affine {
  uint32_t a, c;  // x -> a x + c (mod 2^32)
};

__host__ __device__ __forceinline__ Affine compose(Affine f, Affine g) {  // f(g(x))
  return Affine{f.a * g.a, f.a * g.c + f.c};
}

__host__ __device__ __forceinline__ Affine lcg_pow(unsigned long long k) {
  Affine r{1u, 0u}, b{1103515245u, 12345u};
  while (k) {
    if (k & 1ull) r = compose(b, r);
    b = compose(b, b);
    k >>= 1;
  }
  return r;
}

__device__ __forceinline__ int rand_r_from(uint32_t state) {
  uint32_t next = state * 1103515245u + 12345u;
  int result = static_cast<int>((next >> 16) % 2048u);
  next = next * 1103515245u + 12345u;
  result = (result << 10) ^ static_cast<int>((next >> 16) % 1024u);
  next = next * 1103515245u + 12345u;
  result = (result << 10) ^ static_cast<int>((next >> 16) % 1024u);
  return result;
}

struct RefMedium {
  int g[3];              // cube sizes (one partition at the origin)
  int lo[3], hi[3];      // shell box, inclusive, clipped to the cube
  int ilo[3], ihi[3];    // interior box, inclusive
  int first_in[3], bord_len, n[3];
  uint32_t seed;
  float frac, max_p, max_s;            // src/boundary.c:27-31
  float vpz0, vsv0, eps0, delta0, theta0, phi0;  // src/precomp.c:156-169
};

__device__ __forceinline__ long long cnt_below(int v, int lo, int hi) {
  // integers in [lo, hi] that are < v
  if (hi < lo) return 0;
  const long long c = static_cast<long long>(v) - lo;
  return c < 0 ? 0 : (c > hi - lo + 1 ? hi - lo + 1 : c);
}

__device__ __forceinline__ bool in_range(int v, int lo, int hi) { return v >= lo && v <= hi; }

// Shell cells strictly before (x, y, z) in the z, y, x sweep.
__device__ long long shell_rank(const RefMedium &m, int x, int y, int z) {
  const long long nbx = m.hi[0] >= m.lo[0] ? m.hi[0] - m.lo[0] + 1 : 0;
  const long long nby = m.hi[1] >= m.lo[1] ? m.hi[1] - m.lo[1] + 1 : 0;
  const long long nix = m.ihi[0] >= m.ilo[0] ? m.ihi[0] - m.ilo[0] + 1 : 0;
  const long long niy = m.ihi[1] >= m.ilo[1] ? m.ihi[1] - m.ilo[1] + 1 : 0;
  long long r = cnt_below(z, m.lo[2], m.hi[2]) * nbx * nby -
                cnt_below(z, m.ilo[2], m.ihi[2]) * nix * niy;
  if (in_range(z, m.lo[2], m.hi[2])) {
    const bool iz = in_range(z, m.ilo[2], m.ihi[2]);
    r += cnt_below(y, m.lo[1], m.hi[1]) * nbx - (iz ? cnt_below(y, m.ilo[1], m.ihi[1]) * nix : 0);
    if (in_range(y, m.lo[1], m.hi[1]))
      r += cnt_below(x, m.lo[0], m.hi[0]) -
           ((iz && in_range(y, m.ilo[1], m.ihi[1])) ? cnt_below(x, m.ilo[0], m.ihi[0]) : 0);
  }
  return r;
}

__device__ __forceinline__ int shell_dist(int g, int first_in, int bord_len, int n) {
  if (g > bord_len + n) return g - bord_len - n;
  if (g < first_in) return first_in - g;
  return 0;
}

__global__ void reference_medium_kernel(const RefMedium m, float *coef, float *vv,
                                        long long pitch, long long count) {
  const long long sx = m.g[0], sy = m.g[1], sz = m.g[2];
  const long long n = sx * sy * sz;
  const long long plane = pitch * sy;
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; d < n;
       d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(d % sx), y = static_cast<int>((d / sx) % sy),
              z = static_cast<int>(d / (sx * sy));
    float vpz = m.vpz0, vsv = m.vsv0;
    const bool inside = in_range(x, m.ilo[0], m.ihi[0]) && in_range(y, m.ilo[1], m.ihi[1]) &&
                        in_range(z, m.ilo[2], m.ihi[2]);
    if (!inside) {
      const bool shell = in_range(x, m.lo[0], m.hi[0]) && in_range(y, m.lo[1], m.hi[1]) &&
                         in_range(z, m.lo[2], m.hi[2]);
      if (shell) {
        const Affine f = lcg_pow(3ull * static_cast<unsigned long long>(shell_rank(m, x, y, z)));
        const int rv = rand_r_from(f.a * m.seed + f.c);
        const float r = __fdiv_rn(__int2float_rn(rv), 2147483648.0f);  // RAND_MAX as float
        int dist = shell_dist(y, m.first_in[1], m.bord_len, m.n[1]);
        const int dz = shell_dist(z, m.first_in[2], m.bord_len, m.n[2]);
        const int dx = shell_dist(x, m.first_in[0], m.bord_len, m.n[0]);
        dist = dist > dz ? dist : dz;
        dist = dist > dx ? dist : dx;
        const float w = __fmul_rn(__int2float_rn(dist), m.frac);
        const float omw = __fsub_rn(1.0f, w);
        vpz = __fadd_rn(__fmul_rn(m.max_p, omw), __fmul_rn(__fmul_rn(m.max_p, r), w));
        vsv = __fadd_rn(__fmul_rn(m.max_s, omw), __fmul_rn(__fmul_rn(m.max_s, r), w));
      } else {
        vpz = 0.0f;
        vsv = 0.0f;
      }
    }
    const long long pi = static_cast<long long>(z) * plane + static_cast<long long>(y) * pitch + x;
    if (coef) {
      float out[10];
      precomp_point(m.theta0, m.phi0, vsv, vpz, m.eps0, m.delta0, out);
#pragma unroll
      for (int k = 0; k < 10; ++k) coef[coef_index(k, pi, count)] = out[k];
    }
    if (vv) {
      vv[2 * pi] = vpz;
      vv[2 * pi + 1] = vsv;
    }
  }
}

// One coefficient (DevCoef k): dense array <-> grouped pitched layout.
__global__ void coef_component_kernel(float *coef, float *dense, int k, long long sx,
                                      long long n, long long pitch, long long count,
                                      bool to_grouped) {
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; d < n;
       d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = d % sx, yz = d / sx;
    float *g = coef + coef_index(k, yz * pitch + x, count);
    if (to_grouped)
      *g = dense[d];
    else
      dense[d] = *g;
  }
}

// Ten dense arrays in reference order (ch1dxx, ch1dyy, ch1dzz, ch1dxy,
// ch1dyz, ch1dxz, v2px, v2pz, v2sz, v2pn) -> the three groups (cxx, cyy,
// cxy, czz), (cxz, cyz, v2px, v2pz), (v2sz, v2pn) at the pitched index.
// Reads are coalesced per array; one vector store per group.
__global__ void coef_gather_kernel(float *coef, const CoefSources src, long long sx,
                                   long long n, long long pitch, long long count) {
  float4 *g0 = reinterpret_cast<float4 *>(coef);
  float4 *g1 = reinterpret_cast<float4 *>(coef + 4 * count);
  float2 *g2 = reinterpret_cast<float2 *>(coef + 8 * count);
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; d < n;
       d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = d % sx, i = (d / sx) * pitch + x;
    g0[i] = make_float4(src.p[0][d], src.p[1][d], src.p[3][d], src.p[2][d]);
    g1[i] = make_float4(src.p[5][d], src.p[4][d], src.p[6][d], src.p[7][d]);
    g2[i] = make_float2(src.p[8][d], src.p[9][d]);
  }
}

// max |v| over the four velocity terms, as float bits (non-negative floats
// order like their bit patterns)
__global__ void coef_vmax_kernel(const float *coef, long long count, unsigned int *out) {
  unsigned int m = 0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float4 g1 = reinterpret_cast<const float4 *>(coef + 4 * count)[i];
    const float2 g2 = reinterpret_cast<const float2 *>(coef + 8 * count)[i];
    const float v = fmaxf(fmaxf(fabsf(g1.z), fabsf(g1.w)), fmaxf(fabsf(g2.x), fabsf(g2.y)));
    m = max(m, __float_as_uint(v));
  }
  for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void coef_repitch_kernel(float *coef, const float *gd, long long sx, long long sy,
                                    long long n, long long pitch, long long count) {
  for (long long d = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; d < n;
       d += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = d % sx, yz = d / sx;
    const long long pi = yz * pitch + x;
#pragma unroll
    for (int k = 0; k < 10; ++k) coef[coef_index(k, pi, count)] = gd[coef_index(k, d, n)];
  }
}

template <typename H2>
__device__ __forceinline__ H2 to_h2(float a, float b);
template <>
__device__ __forceinline__ __nv_bfloat162 to_h2<__nv_bfloat162>(float a, float b) {
  return __floats2bfloat162_rn(a, b);
}

template <typename H2>
__global__ void coef_narrow_kernel(const float *coef, H2 *hl, H2 *ho1, H2 *ho2, float vscale,
                                   long long count) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float4 g0 = reinterpret_cast<const float4 *>(coef)[i];
    const float4 g1 = reinterpret_cast<const float4 *>(coef + 4 * count)[i];
    const float2 g2 = reinterpret_cast<const float2 *>(coef + 8 * count)[i];
    hl[2 * i + 0] = to_h2<H2>(g0.x, g0.y);                     // cxx, cyy
    hl[2 * i + 1] = to_h2<H2>(g0.z, g0.w);                     // cxy, czz
    ho1[2 * i + 0] = to_h2<H2>(g1.x, g1.y);                    // cxz, cyz
    ho1[2 * i + 1] = to_h2<H2>(g1.z * vscale, g1.w * vscale);  // v2px, v2pz
    ho2[i] = to_h2<H2>(g2.x * vscale, g2.y * vscale);          // v2sz, v2pn
  }
}

// 16-bit fixed point of an angle term (|c| <= 1): q = c x 2^15, round to
// nearest even, clamped to [-32768, 32767], stored biased as q + 32768; two
// values per word (first in the low half).
__device__ __forceinline__ uint32_t pack_fixed(float a, float b) {
  const int qa = max(-32768, min(32767, __float2int_rn(a * 32768.0f)));
  const int qb = max(-32768, min(32767, __float2int_rn(b * 32768.0f)));
  return static_cast<uint32_t>(qa + 32768) | (static_cast<uint32_t>(qb + 32768) << 16);
}

// FP16 ratio of a velocity term to its row base.
__device__ __forceinline__ float vratio(float v, float b) {
  return b != 0.0f ? __fsub_rn(__fdiv_rn(v, b), 1.0f) : 0.0f;
}

__device__ __forceinline__ uint32_t pack_half(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// One warp per medium row: the midrange of the row's non-zero values of
// each velocity term is its base; then every point of the row (padding
// included) is encoded.
__global__ void coef_rowref_kernel(const float *coef, uint32_t *hl, uint32_t *ho1,
                                   uint32_t *ho2, float4 *vbase, long long rows, long long sx,
                                   long long pitch, long long count) {
  const float4 *g0 = reinterpret_cast<const float4 *>(coef);
  const float4 *g1 = reinterpret_cast<const float4 *>(coef + 4 * count);
  const float2 *g2 = reinterpret_cast<const float2 *>(coef + 8 * count);
  const int lane = threadIdx.x & 31;
  const long long nwarps = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  for (long long r = (blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x) >> 5;
       r < rows; r += nwarps) {
    const long long row = r * pitch;
    float mn[4], mx[4];
    for (int k = 0; k < 4; ++k) {
      mn[k] = INFINITY;
      mx[k] = -INFINITY;
    }
    for (long long x = lane; x < sx; x += 32) {
      const float4 a = g1[row + x];
      const float2 b = g2[row + x];
      const float v[4] = {a.z, a.w, b.x, b.y};
      for (int k = 0; k < 4; ++k)
        if (v[k] != 0.0f) {
          mn[k] = fminf(mn[k], v[k]);
          mx[k] = fmaxf(mx[k], v[k]);
        }
    }
    float bs[4];
    for (int k = 0; k < 4; ++k) {
      for (int off = 16; off > 0; off >>= 1) {
        mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
        mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
      }
      bs[k] = mn[k] <= mx[k] ? 0.5f * (mn[k] + mx[k]) : 0.0f;
    }
    if (lane == 0) vbase[r] = make_float4(bs[0], bs[1], bs[2], bs[3]);
    for (long long x = lane; x < pitch; x += 32) {
      const long long i = row + x;
      const float4 c0 = g0[i], c1 = g1[i];
      const float2 c2 = g2[i];
      hl[2 * i] = pack_fixed(c0.x, c0.y);      // cxx, cyy
      hl[2 * i + 1] = pack_fixed(c0.z, c0.w);  // cxy, czz
      ho1[2 * i] = pack_fixed(c1.x, c1.y);     // cxz, cyz
      ho1[2 * i + 1] = pack_half(vratio(c1.z, bs[0]), vratio(c1.w, bs[1]));  // v2px, v2pz
      ho2[i] = pack_half(vratio(c2.x, bs[2]), vratio(c2.y, bs[3]));          // v2sz, v2pn
    }
  }
}

}  // namespace

cudaError_t launch_coef_rowref(cudaStream_t st, const float *coef, void *coef16, float4 *vbase,
                               long long sx, long long sy, long long sz, long long pitch,
                               long long count) {
  const long long rows = sy * sz;
  const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((rows + 7) / 8, 152 * 32)));
  uint32_t *h = static_cast<uint32_t *>(coef16);
  coef_rowref_kernel<<<blocks, 256, 0, st>>>(coef, h, h + 2 * count, h + 4 * count, vbase, rows,
                                             sx, pitch, count);
  return cudaGetLastError();
}

cudaError_t launch_coef_component(cudaStream_t st, float *coef, float *dense, int k,
                                  long long sx, long long sy, long long sz, long long pitch,
                                  long long count, bool to_grouped) {
  const long long n = sx * sy * sz;
  const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)));
  coef_component_kernel<<<blocks, 256, 0, st>>>(coef, dense, k, sx, n, pitch, count, to_grouped);
  return cudaGetLastError();
}

cudaError_t launch_coef_vmax(cudaStream_t st, const float *coef, long long count,
                             unsigned int *out) {
  const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((count + 255) / 256, 152 * 16)));
  coef_vmax_kernel<<<blocks, 256, 0, st>>>(coef, count, out);
  return cudaGetLastError();
}

cudaError_t launch_coef_gather(cudaStream_t st, float *coef, const CoefSources &src,
                               long long sx, long long sy, long long sz, long long pitch,
                               long long count) {
  const long long n = sx * sy * sz;
  const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)));
  coef_gather_kernel<<<blocks, 256, 0, st>>>(coef, src, sx, n, pitch, count);
  return cudaGetLastError();
}

cudaError_t launch_coef_repitch(cudaStream_t st, float *coef, const float *grouped_dense,
                                long long sx, long long sy, long long sz, long long pitch,
                                long long count) {
  const long long n = sx * sy * sz;
  const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)));
  coef_repitch_kernel<<<blocks, 256, 0, st>>>(coef, grouped_dense, sx, sy, n, pitch, count);
  return cudaGetLastError();
}

cudaError_t launch_coef_narrow(cudaStream_t st, const float *coef, void *coef16, int form,
                               int vexp, long long count) {
  const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((count + 255) / 256, 152 * 32)));
  const float vscale = ldexpf(1.0f, -vexp);
  // layout: [count] x 8 B (cxx, cyy, cxy, czz), [count] x 8 B (cxz, cyz,
  // v2px, v2pz), [count] x 4 B (v2sz, v2pn); the FP16 form has its own
  // encoding (launch_coef_rowref)
  if (form != CF_BF16) return cudaErrorInvalidValue;
  __nv_bfloat162 *h = static_cast<__nv_bfloat162 *>(coef16);
  coef_narrow_kernel<__nv_bfloat162><<<blocks, 256, 0, st>>>(coef, h, h + 2 * count,
                                                             h + 4 * count, vscale, count);
  return cudaGetLastError();
}

cudaError_t launch_reference_medium(cudaStream_t st, const int n[3], int absorb,
                                    unsigned int seed, const float consts[6], float *coef,
                                    float *vv, long long pitch, long long count) {
  RefMedium m{};
  const int bord = 4;  // STENCIL (include/definitions.h:4)
  m.bord_len = bord + absorb - 1;
  for (int d = 0; d < 3; ++d) {
    m.n[d] = n[d];
    m.g[d] = n[d] + 2 * absorb + 2 * bord;  // src/main.c:94-99
    m.first_in[d] = m.bord_len + 1;
    m.ilo[d] = m.first_in[d];
    m.ihi[d] = std::min(m.bord_len + n[d], m.g[d] - 1);
    m.lo[d] = bord;
    m.hi[d] = std::min(2 * m.bord_len + n[d], m.g[d] - 1);
  }
  m.seed = seed;
  m.frac = consts[0];
  m.max_p = consts[1];
  m.max_s = consts[2];
  m.vpz0 = 3000.0f;
  m.vsv0 = consts[3];
  m.eps0 = 0.24f;
  m.delta0 = 0.1f;
  m.theta0 = consts[4];
  m.phi0 = consts[5];
  const long long total = static_cast<long long>(m.g[0]) * m.g[1] * m.g[2];
  const int blocks = static_cast<int>(std::min<long long>((total + 255) / 256, 152 * 32));
  reference_medium_kernel<<<blocks, 256, 0, st>>>(m, coef, vv, pitch, count);
  return cudaGetLastError();
}

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
                  const uint32_t *box, std::string *err, CUtensorMapDataType dt) {
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
