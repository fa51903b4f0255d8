// dc_learned.cu -- the learned thin absorbing layer.
//
// A thin layer of L cells (L <= DC_GB300_MLP_DEPTHS) between the physical
// interior and the 4-cell halo replaces the wide sponge.  After every
// stencil pass, each of the layer's 4 outer cells -- those whose stencils
// reach into the zero halo -- gets a correction (dp, dq) predicted by a
// small MLP from the cells along its boundary normal (the inner L - 4 cells
// are updated by the stencil alone):
//
//   features  the cell and the 7 cells inward along the normal, p and q, at
//             t+1 (the stencil's output) and t: 8 x 2 x 2 = 32 values
//   scale     r = rms of the 32 features; the network sees x / r and its
//             output is multiplied by r (the correction is homogeneous of
//             degree 1 in the wavefield, like a linear absorbing condition)
//   network   32 -> 32 -> 32 -> 2, GELU (tanh form), BF16 weights and
//             activations, FP32 accumulation; the first hidden layer's bias
//             depends on the cell's depth in the layer (0 = next to the
//             interior).  Inference runs on the tensor cores (mma.sync
//             m16n8k16 BF16, activations kept in registers between layers);
//             training on CUDA cores.
//
// The normal of an edge or corner cell is the axis along which it lies
// deepest in the layer (lowest axis on ties).
//
// Training (teacher forcing): a wide simulation, whose margins keep every
// reflection out of the region of interest for the whole run, supplies the
// truth.  At a sampled step its fields (t and t-1) are cropped to the thin
// box (zero halo), stepped once by the thin simulation, and every layer cell
// yields a sample (features of the thin step) and a target (wide field at
// t+1 minus the thin step).  The loss is sum |r * y - target|^2 / sum r^2
// over a minibatch; gradients run through the BF16 roundings unchanged;
// Adam updates FP32 master weights.  Every kernel here is this project's own.
//
// The reference has no learned boundary; it absorbs with its random
// velocity boundary (src/boundary.c:7-104).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "dc_internal.h"

namespace dcg {
namespace {

constexpr int kIn = DC_GB300_MLP_IN, kHid = DC_GB300_MLP_HIDDEN, kOut = DC_GB300_MLP_OUT;
constexpr int kDepths = DC_GB300_MLP_DEPTHS;
constexpr int kStride = kIn + 1;  // sample row: 32 features + depth
constexpr int OFF_W1 = 0;                         // [kHid][kIn]
constexpr int OFF_B1 = OFF_W1 + kHid * kIn;       // [kDepths][kHid]
constexpr int OFF_W2 = OFF_B1 + kDepths * kHid;   // [kHid][kHid]
constexpr int OFF_B2 = OFF_W2 + kHid * kHid;      // [kHid]
constexpr int OFF_W3 = OFF_B2 + kHid;             // [kOut][kHid]
constexpr int OFF_B3 = OFF_W3 + kOut * kHid;      // [kOut]
constexpr int kParams = OFF_B3 + kOut;
static_assert(kParams == DC_GB300_MLP_PARAMS, "parameter count");
constexpr int kWin = 8;  // cells along the normal
constexpr int kCorrected = 4;  // outer layer cells corrected by the network

__device__ __forceinline__ bool is_weight(int p) {
  return (p >= OFF_W1 && p < OFF_B1) || (p >= OFF_W2 && p < OFF_B2) || (p >= OFF_W3 && p < OFF_B3);
}

__device__ __forceinline__ float bf16r(float v) {
  return __bfloat162float(__float2bfloat16_rn(v));
}

// GELU in its tanh form (Hendrycks & Gimpel 2016):
//   gelu(a) = a/2 (1 + tanh(c0 (a + c1 a^3))), c0 = sqrt(2/pi), c1 = 0.044715,
// with the hardware tanh (tanh.approx.f32, one MUFU operation), the same in
// training and inference.
constexpr float kGeluC0 = 0.7978845608028654f, kGeluC1 = 0.044715f;

__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// u = a (c0 + c0 c1 a^2); gelu = h + h tanh(u), h = a / 2.  The scalar and
// the packed (two values, FFMA2/FMUL2) forms round identically.
constexpr float kGeluC01 = kGeluC0 * kGeluC1;

__device__ __forceinline__ float gelu(float a) {
  const float u = fmaf(a * a, kGeluC01, kGeluC0) * a;
  const float h = 0.5f * a;
  return fmaf(h, tanh_hw(u), h);
}

__device__ __forceinline__ float2 gelu2(float2 a) {
  const float2 t = __ffma2_rn(__fmul2_rn(a, a), make_float2(kGeluC01, kGeluC01),
                              make_float2(kGeluC0, kGeluC0));
  const float2 u = __fmul2_rn(t, a);
  const float2 th = make_float2(tanh_hw(u.x), tanh_hw(u.y));
  const float2 h = __fmul2_rn(a, make_float2(0.5f, 0.5f));
  return __ffma2_rn(h, th, h);
}

__device__ __forceinline__ float gelu_grad(float a) {
  const float a2 = a * a;
  const float th = tanh_hw(fmaf(a2, kGeluC01, kGeluC0) * a);
  const float du = kGeluC0 * fmaf(3.0f * kGeluC1, a2, 1.0f);
  return 0.5f * (1.0f + th) + 0.5f * a * (1.0f - th * th) * du;
}

// Copies the compute parameters into shared memory.
__device__ __forceinline__ void load_params(float *sw, const float *wc) {
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) sw[i] = wc[i];
}

// ---------------------------------------------------------------------------
// Training: gradient of sum_i |r_i y_i - t_i|^2 over a set of samples.
// 128 samples per CTA pass; per-sample activations and deltas live in
// shared memory so the weight gradients are small block GEMMs over the
// 128 samples.  `sampled` = 0: samples [0, count); 1: `count` samples
// drawn with replacement from [0, n) by hashing `seed`.
constexpr int kTB = 128;
constexpr int kRow = 33;  // padded row (no bank conflicts)
constexpr int SM_W = 0;
constexpr int SM_XH = SM_W + kParams;
constexpr int SM_A1 = SM_XH + kTB * kRow;   // a1, then delta1
constexpr int SM_H1 = SM_A1 + kTB * kRow;
constexpr int SM_A2 = SM_H1 + kTB * kRow;   // a2, then delta2
constexpr int SM_H2 = SM_A2 + kTB * kRow;
constexpr int SM_DY = SM_H2 + kTB * kRow;   // [kTB][2]
constexpr int SM_DEP = SM_DY + kTB * 2;     // int
constexpr int SM_FLOATS = SM_DEP + kTB;
constexpr size_t kGradSmem = sizeof(float) * SM_FLOATS;

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void __launch_bounds__(kTB) mlp_grad_kernel(const float *__restrict__ wc,
                                                       const float *__restrict__ xs,
                                                       const float *__restrict__ ts, long long n,
                                                       long long count, unsigned long long seed,
                                                       int sampled, float *grad, double *acc) {
  extern __shared__ float sm[];
  float *sw = sm + SM_W;
  float *XH = sm + SM_XH, *A1 = sm + SM_A1, *H1 = sm + SM_H1, *A2 = sm + SM_A2, *H2 = sm + SM_H2;
  float *DY = sm + SM_DY;
  int *DEP = reinterpret_cast<int *>(sm + SM_DEP);
  load_params(sw, wc);
  const int t = threadIdx.x;
  // per-thread gradient accumulators: W1 (8), W2 (8), b1 (kDepths*kHid/128),
  // W3 / b2 / b3 (first threads)
  float gW1[8], gW2[8], gB1[kDepths * kHid / kTB];
  float gW3 = 0.f, gB2 = 0.f, gB3 = 0.f;
#pragma unroll
  for (int m = 0; m < 8; ++m) gW1[m] = gW2[m] = 0.f;
#pragma unroll
  for (int m = 0; m < kDepths * kHid / kTB; ++m) gB1[m] = 0.f;
  double l_err = 0.0, l_w = 0.0;
  __syncthreads();
  for (long long base = static_cast<long long>(blockIdx.x) * kTB; base < count;
       base += static_cast<long long>(gridDim.x) * kTB) {
    const long long j = base + t;
    bool live = j < count;
    long long i = j;
    if (live && sampled) i = static_cast<long long>(mix64(seed ^ (static_cast<unsigned long long>(j) * 0x2545F4914F6CDD1Dull)) % static_cast<unsigned long long>(n));
    float x[kIn];
    int depth = 0;
    float r = 0.f;
    if (live) {
      const float *row = xs + i * kStride;
#pragma unroll
      for (int k = 0; k < kIn; ++k) x[k] = row[k];
      depth = min(max(static_cast<int>(row[kIn]), 0), kDepths - 1);
      float ss = 0.f;
#pragma unroll
      for (int k = 0; k < kIn; ++k) ss = fmaf(x[k], x[k], ss);
      r = sqrtf(ss * (1.0f / kIn));
      live = r > 0.f;
    }
    float *xh = XH + t * kRow, *a1 = A1 + t * kRow, *h1 = H1 + t * kRow;
    float *a2 = A2 + t * kRow, *h2 = H2 + t * kRow;
    DEP[t] = depth;
    if (!live) {
      for (int k = 0; k < kRow; ++k) xh[k] = a1[k] = h1[k] = a2[k] = h2[k] = 0.f;
      DY[2 * t] = DY[2 * t + 1] = 0.f;
    } else {
      const float inv = 1.0f / r;
      for (int k = 0; k < kIn; ++k) xh[k] = bf16r(x[k] * inv);
      for (int o = 0; o < kHid; ++o) {
        float a = sw[OFF_B1 + depth * kHid + o];
        const float *w = sw + OFF_W1 + o * kIn;
        for (int k = 0; k < kIn; ++k) a = fmaf(w[k], xh[k], a);
        a1[o] = a;
        h1[o] = bf16r(gelu(a));
      }
      for (int o = 0; o < kHid; ++o) {
        float a = sw[OFF_B2 + o];
        const float *w = sw + OFF_W2 + o * kHid;
        for (int k = 0; k < kHid; ++k) a = fmaf(w[k], h1[k], a);
        a2[o] = a;
        h2[o] = bf16r(gelu(a));
      }
      float dy[kOut];
      for (int jj = 0; jj < kOut; ++jj) {
        float a = sw[OFF_B3 + jj];
        const float *w = sw + OFF_W3 + jj * kHid;
        for (int k = 0; k < kHid; ++k) a = fmaf(w[k], h2[k], a);
        const float e = r * a - ts[i * kOut + jj];
        l_err += static_cast<double>(e) * e;
        dy[jj] = 2.0f * r * e;
        DY[2 * t + jj] = dy[jj];
      }
      l_w += static_cast<double>(r) * r;
      // delta2 = (W3^T dy) * gelu'(a2), stored over a2
      for (int o = 0; o < kHid; ++o) {
        float d = 0.f;
        for (int jj = 0; jj < kOut; ++jj) d = fmaf(sw[OFF_W3 + jj * kHid + o], dy[jj], d);
        a2[o] = d * gelu_grad(a2[o]);
      }
      // delta1 = (W2^T delta2) * gelu'(a1), stored over a1
      for (int k = 0; k < kHid; ++k) {
        float d = 0.f;
        for (int o = 0; o < kHid; ++o) d = fmaf(sw[OFF_W2 + o * kHid + k], a2[o], d);
        a1[k] = d * gelu_grad(a1[k]);
      }
    }
    __syncthreads();
    // weight gradients: sums over the 128 samples of this pass
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int e = t + kTB * m, o = e >> 5, k = e & 31;
      float s1 = 0.f, s2 = 0.f;
      for (int s = 0; s < kTB; ++s) {
        s1 = fmaf(A1[s * kRow + o], XH[s * kRow + k], s1);
        s2 = fmaf(A2[s * kRow + o], H1[s * kRow + k], s2);
      }
      gW1[m] += s1;
      gW2[m] += s2;
    }
#pragma unroll
    for (int m = 0; m < kDepths * kHid / kTB; ++m) {
      const int e = t + kTB * m, dd = e / kHid, o = e % kHid;
      float s1 = 0.f;
      for (int s = 0; s < kTB; ++s)
        if (DEP[s] == dd) s1 += A1[s * kRow + o];
      gB1[m] += s1;
    }
    if (t < kOut * kHid) {
      const int jj = t / kHid, o = t % kHid;
      float s3 = 0.f;
      for (int s = 0; s < kTB; ++s) s3 = fmaf(DY[2 * s + jj], H2[s * kRow + o], s3);
      gW3 += s3;
    }
    if (t < kHid) {
      float s2 = 0.f;
      for (int s = 0; s < kTB; ++s) s2 += A2[s * kRow + t];
      gB2 += s2;
    }
    if (t < kOut) {
      float s3 = 0.f;
      for (int s = 0; s < kTB; ++s) s3 += DY[2 * s + t];
      gB3 += s3;
    }
    __syncthreads();
  }
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    atomicAdd(&grad[OFF_W1 + t + kTB * m], gW1[m]);
    atomicAdd(&grad[OFF_W2 + t + kTB * m], gW2[m]);
  }
#pragma unroll
  for (int m = 0; m < kDepths * kHid / kTB; ++m) atomicAdd(&grad[OFF_B1 + t + kTB * m], gB1[m]);
  if (t < kOut * kHid) atomicAdd(&grad[OFF_W3 + t], gW3);
  if (t < kHid) atomicAdd(&grad[OFF_B2 + t], gB2);
  if (t < kOut) atomicAdd(&grad[OFF_B3 + t], gB3);
  // loss sums
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    l_err += __shfl_down_sync(0xffffffffu, l_err, off);
    l_w += __shfl_down_sync(0xffffffffu, l_w, off);
  }
  if ((t & 31) == 0) {
    atomicAdd(&acc[0], l_err);
    atomicAdd(&acc[1], l_w);
  }
}

// Adam step on the FP32 master weights with the gradient of the mean loss
// (grad / sum r^2); refreshes the compute copy (weights rounded to BF16),
// clears the gradient and the loss sums, and records the loss.
__global__ void mlp_adam_kernel(float *master, float *wc, float *m1, float *m2, float *grad,
                                double *acc, float lr, float b1, float b2, float eps, int step,
                                float *loss_hist, int hist_index) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const double w = acc[1];
  if (p < kParams) {
    const float g = w > 0.0 ? static_cast<float>(grad[p] / w) : 0.0f;
    const float a = b1 * m1[p] + (1.0f - b1) * g;
    const float v = b2 * m2[p] + (1.0f - b2) * g * g;
    m1[p] = a;
    m2[p] = v;
    const float ah = a / (1.0f - powf(b1, static_cast<float>(step)));
    const float vh = v / (1.0f - powf(b2, static_cast<float>(step)));
    const float nw = master[p] - lr * ah / (sqrtf(vh) + eps);
    master[p] = nw;
    wc[p] = is_weight(p) ? bf16r(nw) : nw;
    grad[p] = 0.0f;
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0 && loss_hist)
    loss_hist[hist_index] = w > 0.0 ? static_cast<float>(acc[0] / w) : 0.0f;
}

__global__ void mlp_clear_acc_kernel(double *acc) {
  if (threadIdx.x < 2) acc[threadIdx.x] = 0.0;
}

// Compute copy of a parameter vector.
__global__ void mlp_round_kernel(const float *master, float *wc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kParams) wc[p] = is_weight(p) ? bf16r(master[p]) : master[p];
}

// ---------------------------------------------------------------------------
// Layer cells: int4 {x, y, z, meta}, meta = axis | side << 2 | depth << 3
// (side 1 = the high end of the axis).

// The 32 features of cell c from the new (t+1) and current (t) pair
// buffers; returns the depth.
__device__ __forceinline__ int gather(const int4 c, const float2 *nw, const float2 *cur,
                                      long long pitch, long long plane, float x[kIn]) {
  const int axis = c.w & 3, side = (c.w >> 2) & 1, depth = c.w >> 3;
  const long long stride = axis == 0 ? 1 : axis == 1 ? pitch : plane;
  const long long step = side ? -stride : stride;  // inward
  long long g = static_cast<long long>(c.z) * plane + static_cast<long long>(c.y) * pitch + c.x;
#pragma unroll
  for (int k = 0; k < kWin; ++k) {
    const float2 a = nw[g], b = cur[g];
    x[k] = a.x;
    x[kWin + k] = a.y;
    x[2 * kWin + k] = b.x;
    x[3 * kWin + k] = b.y;
    g += step;
  }
  return depth;
}

// ---------------------------------------------------------------------------
// Inference on the tensor cores.  One warp evaluates 16 cells per pass with
// mma.sync.m16n8k16 (BF16 operands, FP32 accumulation).  Lane (g = lane/4,
// t = lane%4) holds rows g and g+8 -- two cells -- and, per cell, the
// features of window positions 2t and 2t+1: exactly its A-fragment elements
// of the first layer (feature order p(t+1)[0..7], q(t+1)[0..7], p(t)[0..7],
// q(t)[0..7]).  Each layer's accumulator fragments are the next layer's A
// fragments, so the activations never leave registers; the weights are
// loaded once per warp as B fragments.

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// GELU of a layer's accumulator fragments, packed into the next layer's A
// fragments (k-chunk kk = n-tiles 2kk and 2kk+1).
__device__ __forceinline__ void gelu_to_a(const float acc[4][4], uint32_t a[2][4]) {
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float2 g0 = gelu2(make_float2(acc[2 * kk + h][0], acc[2 * kk + h][1]));
      const float2 g1 = gelu2(make_float2(acc[2 * kk + h][2], acc[2 * kk + h][3]));
      a[kk][2 * h] = pack_bf16(g0.x, g0.y);
      a[kk][2 * h + 1] = pack_bf16(g1.x, g1.y);
    }
  }
}

// Feature sources: load(r, t, f) fills f = {p1[2t], p1[2t+1], q1[2t],
// q1[2t+1], p0[2t], p0[2t+1], q0[2t], q0[2t+1]} of cell / sample r (p1, q1
// at t+1, p0, q0 at t) and returns its depth.
struct RowSrc {  // sample rows [n][33]
  const float *rows;
  __device__ __forceinline__ int load(long long r, int t, float f[8]) const {
    const float *row = rows + r * kStride;
    f[0] = row[2 * t];
    f[1] = row[2 * t + 1];
    f[2] = row[kWin + 2 * t];
    f[3] = row[kWin + 2 * t + 1];
    f[4] = row[2 * kWin + 2 * t];
    f[5] = row[2 * kWin + 2 * t + 1];
    f[6] = row[3 * kWin + 2 * t];
    f[7] = row[3 * kWin + 2 * t + 1];
    return min(max(static_cast<int>(row[kIn]), 0), kDepths - 1);
  }
};

__device__ __forceinline__ int load_cell(int4 c, const float2 *nw, const float2 *cur,
                                         long long pitch, long long plane, int t, float f[8],
                                         float *rec) {
  const int axis = c.w & 3, side = (c.w >> 2) & 1, depth = (c.w >> 3) & 31;
  const long long stride = axis == 0 ? 1 : axis == 1 ? pitch : plane;
  const long long step = side ? -stride : stride;  // inward
  const long long g = static_cast<long long>(c.z) * plane + static_cast<long long>(c.y) * pitch +
                      c.x + step * (2 * t);
  const float2 a0 = nw[g], a1 = nw[g + step], b0 = cur[g], b1 = cur[g + step];
  f[0] = a0.x;
  f[1] = a1.x;
  f[2] = a0.y;
  f[3] = a1.y;
  f[4] = b0.x;
  f[5] = b1.x;
  f[6] = b0.y;
  f[7] = b1.y;
  if (rec) {  // rollout training: the sample row of this cell
    rec[2 * t] = f[0];
    rec[2 * t + 1] = f[1];
    rec[kWin + 2 * t] = f[2];
    rec[kWin + 2 * t + 1] = f[3];
    rec[2 * kWin + 2 * t] = f[4];
    rec[2 * kWin + 2 * t + 1] = f[5];
    rec[3 * kWin + 2 * t] = f[6];
    rec[3 * kWin + 2 * t + 1] = f[7];
    if (t == 0) rec[kIn] = static_cast<float>(depth);
  }
  return depth;
}

struct CellSrc {  // the layer cells of one simulation
  const int4 *cells;
  const float2 *nw, *cur;
  long long pitch, plane;
  float *rec;
  __device__ __forceinline__ int load(long long r, int t, float f[8]) const {
    return load_cell(cells[r], nw, cur, pitch, plane, t, f, rec ? rec + r * kStride : nullptr);
  }
};

struct BatchCellSrc {  // the layer cells of every shot of a batch
  const int4 *cells;
  const LbShot *shots;
  int cur_buf;
  __device__ __forceinline__ int load(long long r, int t, float f[8]) const {
    int4 c = cells[r];
    const LbShot &sh = shots[c.w >> 8];
    c.w &= 0xff;
    return load_cell(c, sh.pq[1 - cur_buf], sh.pq[cur_buf], sh.pitch, sh.plane, t, f, nullptr);
  }
};

// The weights' B fragments live in shared memory (one 8-byte entry per
// lane and 16 x 8 block, read with one LDS.64 per MMA), which keeps the
// kernels under 64 registers: eight 4-warp CTAs per SM hide the gathers'
// latency.
struct NetSmem {
  float b1[kDepths * kHid], b2[kHid], b3[kOut];
  uint2 w1[2][4][32], w2[2][4][32], w3[2][32];
};

// Stages the biases and the weights' B fragments; ends with __syncthreads.
__device__ __forceinline__ void stage_net(const float *__restrict__ wc, NetSmem &sm) {
  for (int i = threadIdx.x; i < kDepths * kHid; i += blockDim.x) sm.b1[i] = wc[OFF_B1 + i];
  if (threadIdx.x < kHid) sm.b2[threadIdx.x] = wc[OFF_B2 + threadIdx.x];
  if (threadIdx.x < kOut) sm.b3[threadIdx.x] = wc[OFF_B3 + threadIdx.x];
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  if (threadIdx.x < 32) {
    // B fragments: B[k][n] = W[n][k] of each 16 x 8 (k x n) block
#pragma unroll
    for (int kk = 0; kk < 2; ++kk) {
      const int k0 = kk * 16 + 2 * t;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const float *r1 = wc + OFF_W1 + (nt * 8 + g) * kIn;
        const float *r2 = wc + OFF_W2 + (nt * 8 + g) * kHid;
        sm.w1[kk][nt][lane] = make_uint2(pack_bf16(r1[k0], r1[k0 + 1]),
                                         pack_bf16(r1[k0 + 8], r1[k0 + 9]));
        sm.w2[kk][nt][lane] = make_uint2(pack_bf16(r2[k0], r2[k0 + 1]),
                                         pack_bf16(r2[k0 + 8], r2[k0 + 9]));
      }
      const float *r3 = wc + OFF_W3 + min(g, kOut - 1) * kHid;
      sm.w3[kk][lane] = g < kOut ? make_uint2(pack_bf16(r3[k0], r3[k0 + 1]),
                                              pack_bf16(r3[k0 + 8], r3[k0 + 9]))
                                 : make_uint2(0u, 0u);
    }
  }
  __syncthreads();
}

// The network over the 16 rows of one warp pass: lane (g, t) brings the
// features f0 of row g and f1 of row g + 8 (window positions 2t, 2t + 1, in
// the order of the sample-row loader) and their depths.  Returns false,
// warp-uniformly, when all 16 rows are silent (no correction anywhere);
// otherwise the lanes with t == 0 hold the corrections r * y of row g in
// (rr0 * y[0], rr0 * y[1]) and of row g + 8 in (rr1 * y[2], rr1 * y[3]).
__device__ __forceinline__ bool net16(const NetSmem &sm, const float f0[8], const float f1[8],
                                      int d0, int d1, float &rr0, float &rr1, float y[4]) {
  const int lane = threadIdx.x & 31, t = lane & 3;
  // rms of each row's 32 features (spread over the 4 lanes of a quad)
  float s0 = 0.f, s1 = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    s0 = fmaf(f0[k], f0[k], s0);
    s1 = fmaf(f1[k], f1[k], s1);
  }
  s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
  s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
  if (__all_sync(0xffffffffu, s0 == 0.f && s1 == 0.f)) return false;
  rr0 = sqrtf(s0 * (1.0f / kIn));
  rr1 = sqrtf(s1 * (1.0f / kIn));
  const float i0 = rr0 > 0.f ? 1.0f / rr0 : 0.f, i1 = rr1 > 0.f ? 1.0f / rr1 : 0.f;
  uint32_t a[2][4];
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
    a[kk][0] = pack_bf16(f0[4 * kk] * i0, f0[4 * kk + 1] * i0);
    a[kk][1] = pack_bf16(f1[4 * kk] * i1, f1[4 * kk + 1] * i1);
    a[kk][2] = pack_bf16(f0[4 * kk + 2] * i0, f0[4 * kk + 3] * i0);
    a[kk][3] = pack_bf16(f1[4 * kk + 2] * i1, f1[4 * kk + 3] * i1);
  }
  float acc[4][4];
  // layer 1 (bias per depth)
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    const int c = nt * 8 + 2 * t;
    acc[nt][0] = sm.b1[d0 * kHid + c];
    acc[nt][1] = sm.b1[d0 * kHid + c + 1];
    acc[nt][2] = sm.b1[d1 * kHid + c];
    acc[nt][3] = sm.b1[d1 * kHid + c + 1];
    const uint2 b0 = sm.w1[0][nt][lane], b1 = sm.w1[1][nt][lane];
    mma_bf16(acc[nt], a[0], b0.x, b0.y);
    mma_bf16(acc[nt], a[1], b1.x, b1.y);
  }
  gelu_to_a(acc, a);
  // layer 2
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    const int c = nt * 8 + 2 * t;
    acc[nt][0] = acc[nt][2] = sm.b2[c];
    acc[nt][1] = acc[nt][3] = sm.b2[c + 1];
    const uint2 b0 = sm.w2[0][nt][lane], b1 = sm.w2[1][nt][lane];
    mma_bf16(acc[nt], a[0], b0.x, b0.y);
    mma_bf16(acc[nt], a[1], b1.x, b1.y);
  }
  gelu_to_a(acc, a);
  // layer 3: outputs in columns 0 and 1, held by the lanes with t == 0
  y[0] = y[2] = t == 0 ? sm.b3[0] : 0.f;
  y[1] = y[3] = t == 0 ? sm.b3[1] : 0.f;
  const uint2 b0 = sm.w3[0][lane], b1 = sm.w3[1][lane];
  mma_bf16(y, a[0], b0.x, b0.y);
  mma_bf16(y, a[1], b1.x, b1.y);
  return true;
}

// One correction per cell or sample row, written to out (zeros for silent
// rows): the training-side and recorded-rollout evaluation.
template <class Src>
__global__ void __launch_bounds__(128, 8) lb_tc_kernel(const float *__restrict__ wc, Src src,
                                                       long long n, float2 *out) {
  __shared__ NetSmem sm;
  stage_net(wc, sm);
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  for (long long base = warp * 16; base < n; base += nwarps * 16) {
    const long long r0 = base + g, r1 = base + g + 8;
    float f0[8], f1[8];
    int d0 = 0, d1 = 0;
    if (r0 < n) {
      d0 = src.load(r0, t, f0);
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) f0[k] = 0.f;
    }
    if (r1 < n) {
      d1 = src.load(r1, t, f1);
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) f1[k] = 0.f;
    }
    float rr0 = 0.f, rr1 = 0.f, y[4];
    const bool live = net16(sm, f0, f1, d0, d1, rr0, rr1, y);
    if (t == 0) {
      if (r0 < n) out[r0] = live ? make_float2(rr0 * y[0], rr0 * y[1]) : make_float2(0.f, 0.f);
      if (r1 < n) out[r1] = live ? make_float2(rr1 * y[2], rr1 * y[3]) : make_float2(0.f, 0.f);
    }
  }
}

// ---------------------------------------------------------------------------
// Fused in-step correction of the face lines.  A face line is the kLine
// corrected cells of one boundary normal (outermost first) whose tangential
// coordinates lie far enough inside the other two axes' interiors that no
// other line's cell is in its windows and no other cell's window reaches it
// (layer_plan below); its kLine windows span kLineCells distinct cells.  One
// warp takes 4 lines -- the 16 rows of one MMA pass: it gathers the 4 x
// kLineCells cells of both time levels once into shared memory, evaluates
// the network and adds each correction in place.  Every value a warp reads
// was read before it writes, and no other warp touches its lines, so the
// result is bit-identical to the two-pass form (lb_tc_kernel then
// lb_add_kernel) while reading each cell once instead of up to 8 times.
constexpr int kLine = kCorrected;               // corrected cells per line
constexpr int kLineCells = kLine + kWin - 1;    // cells the line's windows span
constexpr int kLineWarp = 16 / kLine;           // lines per warp pass
constexpr int kGather = 2 * kLineCells * kLineWarp;  // float2 loads per warp pass
constexpr int kGatherPerLane = (kGather + 31) / 32;
static_assert(16 % kLine == 0 && 32 % kLineWarp == 0, "line packing of the MMA rows");

struct LinePtr {
  float2 *nw;         // the line's outermost cell in the new field
  const float2 *cur;  // ... in the current field
  long long step;     // inward stride
};

__device__ __forceinline__ long long inward_step(int code, long long pitch, long long plane) {
  const int axis = code & 3, side = (code >> 2) & 1;
  const long long stride = axis == 0 ? 1 : axis == 1 ? pitch : plane;
  return side ? -stride : stride;
}

struct LineSrc {  // the face lines of one simulation
  const int4 *lines;
  float2 *nw;
  const float2 *cur;
  long long pitch, plane;
  __device__ __forceinline__ LinePtr at(const int4 c) const {
    const long long g = static_cast<long long>(c.z) * plane + static_cast<long long>(c.y) * pitch + c.x;
    return LinePtr{nw + g, cur + g, inward_step(c.w, pitch, plane)};
  }
};

struct BatchLineSrc {  // the face lines of every shot of a batch
  const int4 *lines;
  const LbShot *shots;
  int cur_buf;
  __device__ __forceinline__ LinePtr at(const int4 c) const {
    const LbShot &sh = shots[c.w >> 8];
    const long long g = static_cast<long long>(c.z) * sh.plane +
                        static_cast<long long>(c.y) * sh.pitch + c.x;
    return LinePtr{sh.pq[1 - cur_buf] + g, sh.pq[cur_buf] + g,
                   inward_step(c.w, sh.pitch, sh.plane)};
  }
};

// Asynchronous 8-byte copy global -> shared (zero fill when !valid; gsrc
// must still be a mapped address).
__device__ __forceinline__ void cp_async8(void *sdst, const void *gsrc, bool valid) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(sdst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(gsrc),
               "r"(valid ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait0() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Each warp keeps one pass's copies in flight while the network runs on
// the previous one: at the top of pass p it waits for the group that
// brought pass p's cells and pass p+1's line entries, then queues pass
// p+1's cells (addresses from those entries) and pass p+2's entries.
// Cells and entries are double-buffered in shared memory; nothing waits on
// a global load issued in the same pass.
template <class Src>
__global__ void __launch_bounds__(128, 8) lb_line_kernel(const float *__restrict__ wc, Src src,
                                                         long long nlines, int layer) {
  __shared__ NetSmem sm;
  // per warp and buffer: [field][cell][line] (field 0 = new, 1 = current),
  // the lines' table entries, and their new-field pointers and strides
  __shared__ __align__(16) float2 sl[4][2][2][kLineCells][kLineWarp];
  __shared__ __align__(16) int4 sent[4][2][kLineWarp];
  __shared__ float2 *snw[4][2][kLineWarp];
  __shared__ long long sst[4][2][kLineWarp];
  stage_net(wc, sm);
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  const long long stride = nwarps * kLineWarp;
  // rows g and g + 8: position j of lines la and lb
  const int j = g % kLine, la = g / kLine, lb = la + 8 / kLine;
  const int depth = layer - 1 - j;
  const int ml = lane % kLineWarp;  // the line this lane copies (32 is a multiple of 4)
  const float2 *dummy = reinterpret_cast<const float2 *>(wc);
  // queues the table entries of the pass at `base` into entry buffer `buf`
  auto fetch_entries = [&](long long base, int buf) {
    if (lane < kLineWarp) {
      const bool v = base + lane < nlines;
      const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(&sent[w][buf][lane]));
      const void *from = v ? static_cast<const void *>(src.lines + base + lane)
                           : static_cast<const void *>(wc);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(from),
                   "r"(v ? 16 : 0)
                   : "memory");
    }
  };
  // queues the cells of the pass at `base` (entries in buffer `buf`) into
  // cell buffer `buf`
  auto fetch_cells = [&](long long base, int buf) {
    const bool mv = base + ml < nlines;
    LinePtr lp{nullptr, nullptr, 0};
    if (mv) lp = src.at(sent[w][buf][ml]);
    if (lane < kLineWarp) {
      snw[w][buf][lane] = lp.nw;
      sst[w][buf][lane] = lp.step;
    }
#pragma unroll
    for (int k = 0; k < kGatherPerLane; ++k) {
      const int i = lane + 32 * k;
      const int fld = i / (kLineCells * kLineWarp), c = (i / kLineWarp) % kLineCells;
      if (i < kGather)
        cp_async8(&sl[w][buf][fld][c][ml], mv ? (fld ? lp.cur : lp.nw) + c * lp.step : dummy,
                  mv);
    }
  };
  long long base = warp * kLineWarp;
  if (base < nlines) {
    fetch_entries(base, 0);
    cp_async_commit();
    cp_async_wait0();
    __syncwarp();
    fetch_cells(base, 0);
    fetch_entries(base + stride, 1);
  }
  cp_async_commit();
  for (int buf = 0; base < nlines; base += stride, buf ^= 1) {
    cp_async_wait0();  // this pass's cells and the next pass's entries have landed
    __syncwarp();
    if (base + stride < nlines) {
      fetch_cells(base + stride, buf ^ 1);
      fetch_entries(base + 2 * stride, buf);
    }
    cp_async_commit();
    float2(*ls)[kLineCells][kLineWarp] = sl[w][buf];
    float f0[8], f1[8];
    {
      const int c0 = j + 2 * t, c1 = c0 + 1;
      const float2 a0 = ls[0][c0][la], a1 = ls[0][c1][la];
      const float2 b0 = ls[1][c0][la], b1 = ls[1][c1][la];
      f0[0] = a0.x, f0[1] = a1.x, f0[2] = a0.y, f0[3] = a1.y;
      f0[4] = b0.x, f0[5] = b1.x, f0[6] = b0.y, f0[7] = b1.y;
      const float2 e0 = ls[0][c0][lb], e1 = ls[0][c1][lb];
      const float2 h0 = ls[1][c0][lb], h1 = ls[1][c1][lb];
      f1[0] = e0.x, f1[1] = e1.x, f1[2] = e0.y, f1[3] = e1.y;
      f1[4] = h0.x, f1[5] = h1.x, f1[6] = h0.y, f1[7] = h1.y;
    }
    float rr0 = 0.f, rr1 = 0.f, y[4];
    if (net16(sm, f0, f1, depth, depth, rr0, rr1, y) && t == 0) {
      // new value = stencil output + correction, rounded as the two-pass form
      if (base + la < nlines) {
        const float2 v = ls[0][j][la];
        snw[w][buf][la][j * sst[w][buf][la]] = make_float2(
            __fadd_rn(v.x, __fmul_rn(rr0, y[0])), __fadd_rn(v.y, __fmul_rn(rr0, y[1])));
      }
      if (base + lb < nlines) {
        const float2 v = ls[0][j][lb];
        snw[w][buf][lb][j * sst[w][buf][lb]] = make_float2(
            __fadd_rn(v.x, __fmul_rn(rr1, y[2])), __fadd_rn(v.y, __fmul_rn(rr1, y[3])));
      }
    }
    __syncwarp();  // the pass after next overwrites this buffer
  }
}

__global__ void lb_add_batch_kernel(const int4 *__restrict__ cells, long long n,
                                    const LbShot *__restrict__ shots, int cur_buf,
                                    const float2 *__restrict__ corr) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int4 c = cells[i];
    const LbShot sh = shots[c.w >> 8];
    float2 *nw = sh.pq[1 - cur_buf];
    const long long g = static_cast<long long>(c.z) * sh.plane +
                        static_cast<long long>(c.y) * sh.pitch + c.x;
    const float2 d = corr[i], v = nw[g];
    nw[g] = make_float2(v.x + d.x, v.y + d.y);
  }
}

__global__ void lb_add_kernel(const int4 *__restrict__ cells, long long n, float2 *nw,
                              const float2 *__restrict__ corr, long long pitch, long long plane) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int4 c = cells[i];
    const long long g = static_cast<long long>(c.z) * plane + static_cast<long long>(c.y) * pitch + c.x;
    const float2 d = corr[i], v = nw[g];
    nw[g] = make_float2(v.x + d.x, v.y + d.y);
  }
}

// Training samples of the thin box: features from its step and targets
// from the wide field (offset into the wide box).
__global__ void lb_sample_kernel(const int4 *__restrict__ cells, long long n, const float2 *nw,
                                 const float2 *cur, long long pitch, long long plane,
                                 const float2 *wide, long long wpitch, long long wplane, int ox,
                                 int oy, int oz, float *xs, float *ts) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int4 c = cells[i];
    float x[kIn];
    const int depth = gather(c, nw, cur, pitch, plane, x);
    float *row = xs + i * kStride;
#pragma unroll
    for (int k = 0; k < kIn; ++k) row[k] = x[k];
    row[kIn] = static_cast<float>(depth);
    const long long g = static_cast<long long>(c.z) * plane + static_cast<long long>(c.y) * pitch + c.x;
    const long long w = static_cast<long long>(c.z + oz) * wplane +
                        static_cast<long long>(c.y + oy) * wpitch + (c.x + ox);
    const float2 tv = wide[w], sv = nw[g];
    ts[i * kOut] = tv.x - sv.x;
    ts[i * kOut + 1] = tv.y - sv.y;
  }
}

// Rollout targets: wide field at t+1 minus the thin stencil's output, which
// is features 0 (p) and 8 (q) of each recorded row.
__global__ void lb_target_kernel(const int4 *__restrict__ cells, long long n,
                                 const float *__restrict__ rows, const float2 *wide,
                                 long long wpitch, long long wplane, int ox, int oy, int oz,
                                 float *ts) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int4 c = cells[i];
    const long long w = static_cast<long long>(c.z + oz) * wplane +
                        static_cast<long long>(c.y + oy) * wpitch + (c.x + ox);
    const float2 tv = wide[w];
    ts[i * kOut] = tv.x - rows[i * kStride];
    ts[i * kOut + 1] = tv.y - rows[i * kStride + kWin];
  }
}

// Thin box <- wide box at (ox, oy, oz), zero outside [4, s-4)^3.
__global__ void crop_kernel(float2 *dst, long long sx, long long sy, long long sz,
                            long long pitch, const float2 *src, long long wpitch,
                            long long wplane, int ox, int oy, int oz) {
  const long long n = sx * sy * sz;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long x = i % sx, y = (i / sx) % sy, z = i / (sx * sy);
    float2 v = make_float2(0.f, 0.f);
    if (x >= 4 && x < sx - 4 && y >= 4 && y < sy - 4 && z >= 4 && z < sz - 4)
      v = src[(z + oz) * wplane + (y + oy) * wpitch + (x + ox)];
    dst[(z * sy + y) * pitch + x] = v;
  }
}

// The face-line pass: at most one wave of its 8 CTAs per SM (each stages
// the weights once and loops over its passes).
int line_grid(long long nl) {
  return static_cast<int>(std::max<long long>(1, std::min<long long>((nl + 15) / 16, 152 * 8)));
}

int grid_for(long long n, int per_block) {
  return static_cast<int>(std::max<long long>(1, std::min<long long>((n + per_block - 1) / per_block, 152 * 16)));
}

}  // namespace

// ---------------------------------------------------------------------------
std::vector<int4> layer_cells(long long sx, long long sy, long long sz, int layer) {
  std::vector<int4> out;
  const long long s[3] = {sx, sy, sz};
  auto depth_on = [&](int a, long long c, int *side) -> int {
    const long long lo = 4 + layer, hi = s[a] - 4 - layer;
    if (c < lo) {
      *side = 0;
      return static_cast<int>(lo - 1 - c);
    }
    if (c >= hi) {
      *side = 1;
      return static_cast<int>(c - hi);
    }
    return -1;
  };
  for (long long z = 4; z < sz - 4; ++z)
    for (long long y = 4; y < sy - 4; ++y) {
      int sdz = 0, sdy = 0;
      const int dz = depth_on(2, z, &sdz), dy = depth_on(1, y, &sdy);
      const bool band = dz < 0 && dy < 0;  // only the two x slabs are in the layer
      for (long long x = 4; x < sx - 4; ++x) {
        if (band && x == 4 + layer) x = sx - 4 - layer;  // skip the interior
        int sdx = 0;
        const int dx = depth_on(0, x, &sdx);
        int axis = -1, depth = -1, side = 0;
        if (dx > depth) { axis = 0; depth = dx; side = sdx; }
        if (dy > depth) { axis = 1; depth = dy; side = sdy; }
        if (dz > depth) { axis = 2; depth = dz; side = sdz; }
        // only the outer cells, whose stencils reach into the halo, are
        // corrected; the inner ones are updated by the stencil alone
        if (axis < 0 || depth < layer - kCorrected) continue;
        out.push_back(make_int4(static_cast<int>(x), static_cast<int>(y), static_cast<int>(z),
                                axis | side << 2 | depth << 3));
      }
    }
  return out;
}

cudaError_t launch_lb_step(cudaStream_t st, const float *wc, const int4 *cells, long long n,
                           float2 *nw, const float2 *cur, long long pitch, long long plane,
                           float2 *corr, float *rec) {
  lb_tc_kernel<CellSrc><<<grid_for(n, 64), 128, 0, st>>>(
      wc, CellSrc{cells, nw, cur, pitch, plane, rec}, n, corr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  lb_add_kernel<<<grid_for(n, 256), 256, 0, st>>>(cells, n, nw, corr, pitch, plane);
  return cudaGetLastError();
}

cudaError_t launch_lb_batch_step(cudaStream_t st, const float *wc, const int4 *cells,
                                 long long n, const LbShot *shots, int cur_buf, float2 *corr) {
  lb_tc_kernel<BatchCellSrc><<<grid_for(n, 64), 128, 0, st>>>(
      wc, BatchCellSrc{cells, shots, cur_buf}, n, corr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  lb_add_batch_kernel<<<grid_for(n, 256), 256, 0, st>>>(cells, n, shots, cur_buf, corr);
  return cudaGetLastError();
}

// Splits the corrected cells into face lines (entries for the outermost
// cell, meta = axis | side << 2) and the remaining edge cells (layer_cells
// entries).  The windows of the least deep corrected cells reach m cells
// past the layer into the interior; a line is a face line when both of its
// tangential coordinates lie at least m + 1 cells inside the other axes'
// interiors.  Then (a) every cell a face line reads has those tangential
// coordinates, so it is the line's own or an interior cell, and (b) no edge
// cell's window reaches a face line's cell: a window along the line's axis
// keeps the edge cell's tangential coordinates, and one along another axis
// stays within m cells of that axis' layer.  So the face lines and the edge
// cells can be corrected independently.
LayerPlan layer_plan(long long sx, long long sy, long long sz, int layer) {
  LayerPlan plan;
  const std::vector<int4> cells = layer_cells(sx, sy, sz, layer);
  if (layer < kCorrected) {
    plan.edge = cells;
    return plan;
  }
  const int m = std::max(0, kWin - 1 - (layer - kCorrected));
  const long long s[3] = {sx, sy, sz};
  auto inside = [&](int a, long long c) {
    return c >= 4 + layer + m && c < s[a] - 4 - layer - m;
  };
  for (const int4 &c : cells) {
    const int axis = c.w & 3, depth = (c.w >> 3) & 31;
    const long long p[3] = {c.x, c.y, c.z};
    const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
    if (!(inside(a1, p[a1]) && inside(a2, p[a2])))
      plan.edge.push_back(c);
    else if (depth == layer - 1)
      plan.lines.push_back(make_int4(c.x, c.y, c.z, c.w & 7));
  }
  return plan;
}

cudaError_t launch_lb_fused(cudaStream_t st, const float *wc, int layer, const int4 *lines,
                            long long nl, const int4 *edge, long long ne, float2 *nw,
                            const float2 *cur, long long pitch, long long plane, float2 *corr) {
  if (nl > 0) {
    lb_line_kernel<LineSrc><<<line_grid(nl), 128, 0, st>>>(
        wc, LineSrc{lines, nw, cur, pitch, plane}, nl, layer);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (ne > 0) return launch_lb_step(st, wc, edge, ne, nw, cur, pitch, plane, corr, nullptr);
  return cudaSuccess;
}

cudaError_t launch_lb_batch_fused(cudaStream_t st, const float *wc, int layer, const int4 *lines,
                                  long long nl, const int4 *edge, long long ne,
                                  const LbShot *shots, int cur_buf, float2 *corr) {
  if (nl > 0) {
    lb_line_kernel<BatchLineSrc><<<line_grid(nl), 128, 0, st>>>(
        wc, BatchLineSrc{lines, shots, cur_buf}, nl, layer);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (ne > 0) return launch_lb_batch_step(st, wc, edge, ne, shots, cur_buf, corr);
  return cudaSuccess;
}

cudaError_t launch_lb_sample(cudaStream_t st, const int4 *cells, long long n, const float2 *nw,
                             const float2 *cur, long long pitch, long long plane,
                             const float2 *wide, long long wpitch, long long wplane,
                             const int off[3], float *xs, float *ts) {
  lb_sample_kernel<<<grid_for(n, 256), 256, 0, st>>>(cells, n, nw, cur, pitch, plane, wide,
                                                     wpitch, wplane, off[0], off[1], off[2], xs,
                                                     ts);
  return cudaGetLastError();
}

cudaError_t launch_lb_target(cudaStream_t st, const int4 *cells, long long n, const float *rows,
                             const float2 *wide, long long wpitch, long long wplane,
                             const int off[3], float *ts) {
  lb_target_kernel<<<grid_for(n, 256), 256, 0, st>>>(cells, n, rows, wide, wpitch, wplane,
                                                     off[0], off[1], off[2], ts);
  return cudaGetLastError();
}

cudaError_t launch_crop(cudaStream_t st, float2 *dst, long long sx, long long sy, long long sz,
                        long long pitch, const float2 *src, long long wpitch, long long wplane,
                        const int off[3]) {
  crop_kernel<<<grid_for(sx * sy * sz, 256), 256, 0, st>>>(dst, sx, sy, sz, pitch, src, wpitch,
                                                           wplane, off[0], off[1], off[2]);
  return cudaGetLastError();
}

}  // namespace dcg

// ===========================================================================
// C ABI
// ===========================================================================
struct dc_gb300_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float *master = nullptr, *wc = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr;
  double *acc = nullptr;
  int adam_step = 0;
};

namespace {

int fail(int code, const std::string &msg) {
  dcg::set_error(msg);
  return code;
}

#define LB_TRY(call)                                                                 \
  do {                                                                               \
    const cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                           \
      return fail(DC_GB300_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void release(dc_gb300_mlp *m) {
  cudaFree(m->master);
  cudaFree(m->wc);
  cudaFree(m->m1);
  cudaFree(m->m2);
  cudaFree(m->grad);
  cudaFree(m->acc);
  if (m->stream) cudaStreamDestroy(m->stream);
}

}  // namespace

extern "C" int dc_gb300_mlp_create(int device, dc_gb300_mlp **out) {
  if (!out) return fail(DC_GB300_ERR_ARG, "null argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(DC_GB300_ERR_DEVICE, "no CUDA device");
  int dev = device;
  if (dev < 0) LB_TRY(cudaGetDevice(&dev));
  if (dev >= ndev) return fail(DC_GB300_ERR_DEVICE, "device ordinal out of range");
  LB_TRY(cudaSetDevice(dev));
  auto *m = new dc_gb300_mlp();
  m->device = dev;
  const size_t pb = sizeof(float) * dcg::kParams;
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&m->master, pb) != cudaSuccess || cudaMalloc(&m->wc, pb) != cudaSuccess ||
      cudaMalloc(&m->m1, pb) != cudaSuccess || cudaMalloc(&m->m2, pb) != cudaSuccess ||
      cudaMalloc(&m->grad, pb) != cudaSuccess ||
      cudaMalloc(&m->acc, 2 * sizeof(double)) != cudaSuccess) {
    release(m);
    delete m;
    return fail(DC_GB300_ERR_NOMEM, "MLP buffers");
  }
  cudaMemsetAsync(m->master, 0, pb, m->stream);
  cudaMemsetAsync(m->wc, 0, pb, m->stream);
  cudaMemsetAsync(m->m1, 0, pb, m->stream);
  cudaMemsetAsync(m->m2, 0, pb, m->stream);
  cudaMemsetAsync(m->grad, 0, pb, m->stream);
  cudaMemsetAsync(m->acc, 0, 2 * sizeof(double), m->stream);
  if (cudaStreamSynchronize(m->stream) != cudaSuccess) {
    release(m);
    delete m;
    return fail(DC_GB300_ERR_CUDA, "MLP set-up");
  }
  *out = m;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_mlp_destroy(dc_gb300_mlp *m) {
  if (!m) return DC_GB300_OK;
  cudaSetDevice(m->device);
  release(m);
  delete m;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_mlp_set_params(dc_gb300_mlp *m, const float *params) {
  if (!m || !params) return fail(DC_GB300_ERR_ARG, "null argument");
  LB_TRY(cudaSetDevice(m->device));
  const size_t pb = sizeof(float) * dcg::kParams;
  LB_TRY(cudaMemcpyAsync(m->master, params, pb, cudaMemcpyHostToDevice, m->stream));
  dcg::mlp_round_kernel<<<(dcg::kParams + 255) / 256, 256, 0, m->stream>>>(m->master, m->wc);
  LB_TRY(cudaGetLastError());
  LB_TRY(cudaMemsetAsync(m->m1, 0, pb, m->stream));
  LB_TRY(cudaMemsetAsync(m->m2, 0, pb, m->stream));
  LB_TRY(cudaMemsetAsync(m->grad, 0, pb, m->stream));
  LB_TRY(cudaStreamSynchronize(m->stream));
  m->adam_step = 0;
  return DC_GB300_OK;
}

extern "C" int dc_gb300_mlp_init(dc_gb300_mlp *m, unsigned int seed) {
  if (!m) return fail(DC_GB300_ERR_ARG, "null argument");
  std::vector<float> p(dcg::kParams, 0.0f);
  std::mt19937 rng(seed);
  auto fill = [&](int off, int rows, int cols, float gain) {
    const float sd = gain / std::sqrt(static_cast<float>(cols));
    std::normal_distribution<float> nd(0.0f, sd);
    for (int i = 0; i < rows * cols; ++i) p[off + i] = nd(rng);
  };
  fill(dcg::OFF_W1, dcg::kHid, dcg::kIn, 1.0f);
  fill(dcg::OFF_W2, dcg::kHid, dcg::kHid, 1.0f);
  fill(dcg::OFF_W3, dcg::kOut, dcg::kHid, 0.01f);  // corrections start near zero
  return dc_gb300_mlp_set_params(m, p.data());
}

extern "C" int dc_gb300_mlp_get_params(dc_gb300_mlp *m, float *params) {
  if (!m || !params) return fail(DC_GB300_ERR_ARG, "null argument");
  LB_TRY(cudaSetDevice(m->device));
  LB_TRY(cudaMemcpyAsync(params, m->master, sizeof(float) * dcg::kParams, cudaMemcpyDeviceToHost,
                         m->stream));
  LB_TRY(cudaStreamSynchronize(m->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_mlp_forward(dc_gb300_mlp *m, const float *samples, long long n,
                                    float *out) {
  if (!m || (n > 0 && (!samples || !out))) return fail(DC_GB300_ERR_ARG, "null argument");
  if (n <= 0) return DC_GB300_OK;
  LB_TRY(cudaSetDevice(m->device));
  dcg::lb_tc_kernel<dcg::RowSrc><<<dcg::grid_for(n, 64), 128, 0, m->stream>>>(
      m->wc, dcg::RowSrc{samples}, n, reinterpret_cast<float2 *>(out));
  LB_TRY(cudaGetLastError());
  LB_TRY(cudaStreamSynchronize(m->stream));
  return DC_GB300_OK;
}

extern "C" int dc_gb300_mlp_gradient(dc_gb300_mlp *m, const float *samples, const float *targets,
                                     long long n, float *grad, double *loss) {
  if (!m || !samples || !targets || !grad || n <= 0)
    return fail(DC_GB300_ERR_ARG, "invalid argument");
  LB_TRY(cudaSetDevice(m->device));
  LB_TRY(cudaFuncSetAttribute(dcg::mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(dcg::kGradSmem)));
  LB_TRY(cudaMemsetAsync(m->grad, 0, sizeof(float) * dcg::kParams, m->stream));
  LB_TRY(cudaMemsetAsync(m->acc, 0, 2 * sizeof(double), m->stream));
  dcg::mlp_grad_kernel<<<dcg::grid_for(n, dcg::kTB), dcg::kTB, dcg::kGradSmem, m->stream>>>(
      m->wc, samples, targets, n, n, 0ull, 0, m->grad, m->acc);
  LB_TRY(cudaGetLastError());
  double acc[2];
  LB_TRY(cudaMemcpyAsync(grad, m->grad, sizeof(float) * dcg::kParams, cudaMemcpyDeviceToHost,
                         m->stream));
  LB_TRY(cudaMemcpyAsync(acc, m->acc, sizeof(acc), cudaMemcpyDeviceToHost, m->stream));
  LB_TRY(cudaMemsetAsync(m->grad, 0, sizeof(float) * dcg::kParams, m->stream));
  LB_TRY(cudaStreamSynchronize(m->stream));
  if (loss) {
    loss[0] = acc[0];
    loss[1] = acc[1];
  }
  return DC_GB300_OK;
}

extern "C" int dc_gb300_mlp_train(dc_gb300_mlp *m, const float *samples, const float *targets,
                                  long long n, int steps, int batch, float lr,
                                  unsigned long long seed, float *loss_hist) {
  if (!m || !samples || !targets || n <= 0 || steps < 0 || batch < 1 || !(lr > 0))
    return fail(DC_GB300_ERR_ARG, "invalid argument");
  LB_TRY(cudaSetDevice(m->device));
  LB_TRY(cudaFuncSetAttribute(dcg::mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(dcg::kGradSmem)));
  float *d_hist = nullptr;
  if (loss_hist && steps > 0) LB_TRY(cudaMalloc(&d_hist, sizeof(float) * steps));
  LB_TRY(cudaMemsetAsync(m->grad, 0, sizeof(float) * dcg::kParams, m->stream));
  dcg::mlp_clear_acc_kernel<<<1, 32, 0, m->stream>>>(m->acc);
  cudaError_t e = cudaGetLastError();
  const int blocks = dcg::grid_for(batch, dcg::kTB);
  for (int s = 0; s < steps && e == cudaSuccess; ++s) {
    dcg::mlp_grad_kernel<<<blocks, dcg::kTB, dcg::kGradSmem, m->stream>>>(
        m->wc, samples, targets, n, batch, seed + 0x9E3779B97F4A7C15ull * (m->adam_step + 1), 1,
        m->grad, m->acc);
    ++m->adam_step;
    dcg::mlp_adam_kernel<<<(dcg::kParams + 255) / 256, 256, 0, m->stream>>>(
        m->master, m->wc, m->m1, m->m2, m->grad, m->acc, lr, 0.9f, 0.999f, 1e-8f, m->adam_step,
        d_hist, s);
    dcg::mlp_clear_acc_kernel<<<1, 32, 0, m->stream>>>(m->acc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && d_hist)
    e = cudaMemcpyAsync(loss_hist, d_hist, sizeof(float) * steps, cudaMemcpyDeviceToHost,
                        m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(d_hist);
  if (e != cudaSuccess) return fail(DC_GB300_ERR_CUDA, std::string("MLP training: ") + cudaGetErrorString(e));
  return DC_GB300_OK;
}

extern "C" long long dc_gb300_layer_cells(long sx, long sy, long sz, int layer, int *cells,
                                         long long cap) {
  if (layer < 1 || layer > DC_GB300_MLP_DEPTHS || sx < 2 * layer + 16 || sy < 2 * layer + 16 ||
      sz < 2 * layer + 16) {
    fail(DC_GB300_ERR_ARG, "invalid layer geometry");
    return -1;
  }
  const std::vector<int4> v = dcg::layer_cells(sx, sy, sz, layer);
  const long long n = static_cast<long long>(v.size());
  if (cells)
    for (long long i = 0; i < std::min(n, cap); ++i) {
      cells[4 * i] = v[i].x;
      cells[4 * i + 1] = v[i].y;
      cells[4 * i + 2] = v[i].z;
      cells[4 * i + 3] = v[i].w;
    }
  return n;
}

extern "C" int dc_gb300_layer_plan(long sx, long sy, long sz, int layer, int *lines,
                                   long long lines_cap, int *edge, long long edge_cap,
                                   long long *n_lines, long long *n_edge) {
  if (!n_lines || !n_edge) return fail(DC_GB300_ERR_ARG, "null count");
  if (layer < 1 || layer > DC_GB300_MLP_DEPTHS || sx < 2 * layer + 16 || sy < 2 * layer + 16 ||
      sz < 2 * layer + 16)
    return fail(DC_GB300_ERR_ARG, "invalid layer geometry");
  const dcg::LayerPlan p = dcg::layer_plan(sx, sy, sz, layer);
  auto put = [](const std::vector<int4> &v, int *out, long long cap) {
    if (!out) return;
    for (long long i = 0; i < std::min(static_cast<long long>(v.size()), cap); ++i) {
      out[4 * i] = v[i].x;
      out[4 * i + 1] = v[i].y;
      out[4 * i + 2] = v[i].z;
      out[4 * i + 3] = v[i].w;
    }
  };
  put(p.lines, lines, lines_cap);
  put(p.edge, edge, edge_cap);
  *n_lines = static_cast<long long>(p.lines.size());
  *n_edge = static_cast<long long>(p.edge.size());
  return DC_GB300_OK;
}

extern "C" const float *dc_gb300_mlp_device_params(const dc_gb300_mlp *m) {
  return m ? m->wc : nullptr;
}
