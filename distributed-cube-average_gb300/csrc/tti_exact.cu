// tti_exact.cu -- the bit-exact sm_103a Fletcher TTI time step.
//
// Same update as the fast kernel, but every floating-point operation is the
// reference's, in the reference's order, with explicit round-to-nearest
// intrinsics so that nothing is contracted into an FMA:
//   der2      include/derivatives.h:47-54   (9-point second derivative)
//   derCross  include/derivatives.h:56-91   (64-point direct cross sum)
//   update    include/sample_compute.h:106-185 (sample_compute) or
//             include/sample_compute.h:21-102  (sample_compute_optimized,
//             the vpz/vsv medium form with constant angles).
// Results are bit-identical to the reference's OpenMP path built without
// FMA contraction (and to its CUDA arithmetic executed the same way).
//
// Data path: a CTA owns a 32 x 4 column tile and sweeps a chunk of z.  The
// stencil reads go through the read-only data cache as (p, q) pairs (217
// 8-byte loads per point), so this kernel is bound by L1 bandwidth, not
// HBM.  It is the parity anchor, not the throughput path.
#include "dc_internal.h"

namespace dcg {
namespace {

// Second-derivative weights K0..K4 and the cross weights L_a*L_b rounded
// once, in the order of include/derivatives.h:58-89.
__device__ __forceinline__ constexpr float kw(int k) {
  return k == 0 ? static_cast<float>(-205.0 / 72.0)
         : k == 1 ? static_cast<float>(8.0 / 5.0)
         : k == 2 ? static_cast<float>(-1.0 / 5.0)
         : k == 3 ? static_cast<float>(8.0 / 315.0)
                  : static_cast<float>(-1.0 / 560.0);
}
__device__ __forceinline__ constexpr double lw(int a) {
  return a == 1 ? 4.0 / 5.0 : a == 2 ? -1.0 / 5.0 : a == 3 ? 4.0 / 105.0 : -1.0 / 280.0;
}
__device__ __forceinline__ constexpr int pair_a(int g) {
  return g < 4 ? 1 : g < 7 ? 2 : g < 9 ? 3 : 4;
}
__device__ __forceinline__ constexpr int pair_b(int g) {
  return g < 4 ? g + 1 : g < 7 ? g - 2 : g < 9 ? g - 4 : 4;
}

struct H12 {
  float h1, h2;
};

// der2 (include/derivatives.h:47-54) and derCross (:56-91) of p and q
// together: one 8-byte load of a (p, q) pair feeds both fields, and each
// field's arithmetic is the reference's, term by term and in its order.
__device__ __forceinline__ float2 ldp(const float2 *__restrict__ f, long long i) {
  return __ldg(f + i);
}

__device__ __forceinline__ float2 der2_x2(const float2 *__restrict__ f, long long i, long long s,
                                          float inv) {
  const float2 c = ldp(f, i);
  float2 a = make_float2(__fmul_rn(kw(0), c.x), __fmul_rn(kw(0), c.y));
#pragma unroll
  for (int k = 1; k <= 4; ++k) {
    const float2 u = ldp(f, i + k * s), v = ldp(f, i - k * s);
    a.x = __fadd_rn(a.x, __fmul_rn(kw(k), __fadd_rn(u.x, v.x)));
    a.y = __fadd_rn(a.y, __fmul_rn(kw(k), __fadd_rn(u.y, v.y)));
  }
  return make_float2(__fmul_rn(a.x, inv), __fmul_rn(a.y, inv));
}

__device__ __forceinline__ float2 cross_x2(const float2 *__restrict__ f, long long i,
                                           long long s1, long long s2, float inv) {
  float2 total = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int g = 0; g < 10; ++g) {
    const long long a = pair_a(g), b = pair_b(g);
    const float2 v0 = ldp(f, i + a * s2 + b * s1), v1 = ldp(f, i + a * s2 - b * s1);
    const float2 v2 = ldp(f, i - a * s2 + b * s1), v3 = ldp(f, i - a * s2 - b * s1);
    float2 acc;
    acc.x = __fadd_rn(__fsub_rn(__fsub_rn(v0.x, v1.x), v2.x), v3.x);
    acc.y = __fadd_rn(__fsub_rn(__fsub_rn(v0.y, v1.y), v2.y), v3.y);
    if (a != b) {
      const float2 w0 = ldp(f, i + b * s2 + a * s1), w1 = ldp(f, i + b * s2 - a * s1);
      const float2 w2 = ldp(f, i - b * s2 + a * s1), w3 = ldp(f, i - b * s2 - a * s1);
      acc.x = __fadd_rn(__fsub_rn(__fsub_rn(__fadd_rn(acc.x, w0.x), w1.x), w2.x), w3.x);
      acc.y = __fadd_rn(__fsub_rn(__fsub_rn(__fadd_rn(acc.y, w0.y), w1.y), w2.y), w3.y);
    }
    const float w = static_cast<float>(lw(pair_a(g)) * lw(pair_b(g)));
    const float2 term = make_float2(__fmul_rn(w, acc.x), __fmul_rn(w, acc.y));
    total = g == 0 ? term
                   : make_float2(__fadd_rn(total.x, term.x), __fadd_rn(total.y, term.y));
  }
  return make_float2(__fmul_rn(total.x, inv), __fmul_rn(total.y, inv));
}

// h1 / h2 of p (.x) and q (.y) from pair-buffer strides (sX = 1).
__device__ __forceinline__ void hterms2(const float2 *__restrict__ f, long long i, long long sY,
                                        long long sZ, const StepParams &prm, float cxx,
                                        float cyy, float czz, float cxy, float cyz, float cxz,
                                        H12 *hp, H12 *hq) {
  const float2 fxx = der2_x2(f, i, 1, prm.dxxinv);
  const float2 fyy = der2_x2(f, i, sY, prm.dyyinv);
  const float2 fzz = der2_x2(f, i, sZ, prm.dzzinv);
  const float2 fxy = cross_x2(f, i, 1, sY, prm.dxyinv);
  const float2 fyz = cross_x2(f, i, sY, sZ, prm.dyzinv);
  const float2 fxz = cross_x2(f, i, 1, sZ, prm.dxzinv);
  const float xx[2] = {fxx.x, fxx.y}, yy[2] = {fyy.x, fyy.y}, zz[2] = {fzz.x, fzz.y};
  const float xy[2] = {fxy.x, fxy.y}, yz[2] = {fyz.x, fyz.y}, xz[2] = {fxz.x, fxz.y};
  H12 *out[2] = {hp, hq};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    float h1 = __fmul_rn(cxx, xx[c]);
    h1 = __fadd_rn(h1, __fmul_rn(cyy, yy[c]));
    h1 = __fadd_rn(h1, __fmul_rn(czz, zz[c]));
    h1 = __fadd_rn(h1, __fmul_rn(cxy, xy[c]));
    h1 = __fadd_rn(h1, __fmul_rn(cxz, xz[c]));
    h1 = __fadd_rn(h1, __fmul_rn(cyz, yz[c]));
    out[c]->h1 = h1;
    out[c]->h2 = __fsub_rn(__fadd_rn(__fadd_rn(xx[c], yy[c]), zz[c]), h1);
  }
}


template <int MEDIUM, bool SPONGE>
__global__ void __launch_bounds__(128)
    exact_kernel(const StepParams prm) {
  const int gx = prm.x0 + static_cast<int>(blockIdx.x * 32 + threadIdx.x);
  const int gy = prm.y0 + static_cast<int>(blockIdx.y * 4 + threadIdx.y);
  if (gx >= prm.x1 || gy >= prm.y1) return;
  const int zb = prm.z0 + static_cast<int>(blockIdx.z) * prm.zchunk;
  const int ze = min(zb + prm.zchunk, prm.z1);
  const long long sY = prm.pitch, sZ = prm.plane;
  float e_acc = 0.f;
  int rk = 0, rend = 0, rnext = -1;  // receivers of this column
  if (prm.rec_col) {
    const int2 e = prm.rec_col[gy * prm.col_stride + gx];
    rk = e.x;
    rend = e.x + e.y;
    while (rk < rend && prm.rec_z[rk] < zb) ++rk;
    rnext = rk < rend ? prm.rec_z[rk] : -1;
  }
  for (int z = zb; z < ze; ++z) {
    const long long i = static_cast<long long>(z) * sZ +
                        static_cast<long long>(gy) * sY + gx;
    float cxx, cyy, czz, cxy, cyz, cxz, v2px, v2pz, v2sz, v2pn;
    if (MEDIUM == DC_GB300_MEDIUM_PRECOMP) {
      const long long n = prm.count;
      const float4 g0 = __ldg(reinterpret_cast<const float4 *>(prm.coef) + i);
      const float4 g1 = __ldg(reinterpret_cast<const float4 *>(prm.coef + 4 * n) + i);
      const float2 g2 = __ldg(reinterpret_cast<const float2 *>(prm.coef + 8 * n) + i);
      cxx = g0.x;
      cyy = g0.y;
      cxy = g0.z;
      czz = g0.w;
      cxz = g1.x;
      cyz = g1.y;
      v2px = g1.z;
      v2pz = g1.w;
      v2sz = g2.x;
      v2pn = g2.y;
    } else {
      // include/sample_compute.h:9-18 and :51-54
      const float2 v = __ldg(reinterpret_cast<const float2 *>(prm.vv) + i);
      const float vp = v.x, vs = v.y;
      cxx = 0.1459632909f;
      cyy = 0.3540367091f;
      czz = 0.5f;
      cxy = 0.4546487134f;
      cyz = 0.8414709848f;
      cxz = 0.5403023059f;
      v2pz = __fmul_rn(vp, vp);
      v2sz = __fmul_rn(vs, vs);
      v2px = __fmul_rn(v2pz, 1.48f);
      v2pn = __fmul_rn(v2pz, 1.2f);
    }
    H12 hp, hq;
    hterms2(prm.cur, i, sY, sZ, prm, cxx, cyy, czz, cxy, cyz, cxz, &hp, &hq);
    const float h1pmq = __fsub_rn(hp.h1, hq.h1);
    const float h2pmq = __fsub_rn(hp.h2, hq.h2);
    const float rhsp = __fadd_rn(
        __fadd_rn(__fmul_rn(v2px, hp.h2), __fmul_rn(v2pz, hq.h1)),
        __fmul_rn(v2sz, h1pmq));
    const float rhsq = __fsub_rn(
        __fadd_rn(__fmul_rn(v2pn, hp.h2), __fmul_rn(v2pz, hq.h1)),
        __fmul_rn(v2sz, h2pmq));
    const float2 cv = prm.cur[i];
    const float pc = cv.x, qc = cv.y;
    const float2 pv = prm.prev[i];
    const float ppo = pv.x, qpo = pv.y;
    const float tp = __fmul_rn(__fmul_rn(rhsp, prm.dt), prm.dt);
    const float tq = __fmul_rn(__fmul_rn(rhsq, prm.dt), prm.dt);
    float np, nq;
    if (SPONGE) {
      const float g = __fmul_rn(__fmul_rn(prm.sponge[gx], prm.sponge[prm.sponge_oy + gy]),
                                prm.sponge[prm.sponge_oz + z]);
      np = __fmul_rn(__fadd_rn(__fsub_rn(__fmul_rn(2.0f, pc), __fmul_rn(g, ppo)), tp), g);
      nq = __fmul_rn(__fadd_rn(__fsub_rn(__fmul_rn(2.0f, qc), __fmul_rn(g, qpo)), tq), g);
      if (g == 1.0f) {  // interior: the reference's own expression
        np = __fadd_rn(__fsub_rn(__fmul_rn(2.0f, pc), ppo), tp);
        nq = __fadd_rn(__fsub_rn(__fmul_rn(2.0f, qc), qpo), tq);
      }
    } else {
      np = __fadd_rn(__fsub_rn(__fmul_rn(2.0f, pc), ppo), tp);
      nq = __fadd_rn(__fsub_rn(__fmul_rn(2.0f, qc), qpo), tq);
    }
    if (prm.energy) e_acc = fmaf(np, np, fmaf(nq, nq, e_acc));
    if (z == rnext) {
      const int step = *prm.d_step + prm.step_offset;
      do {
        if (step >= 0 && step < prm.trace_cap)
          prm.traces[static_cast<long long>(step) * prm.nrec + prm.rec_r[rk]] = np;
        ++rk;
      } while (rk < rend && prm.rec_z[rk] == z);
      rnext = rk < rend ? prm.rec_z[rk] : -1;
    }
    if (gx == prm.src_x && gy == prm.src_y && z == prm.src_z) {
      const int step = *prm.d_step + prm.step_offset;
      const float sv = step + 1 < prm.src_count ? prm.src_table[step + 1] : 0.0f;
      prm.src_pre[0] = np;
      prm.src_pre[1] = nq;
      np = __fadd_rn(np, sv);
      nq = __fadd_rn(nq, sv);
    }
    prm.prev[i] = make_float2(np, nq);
  }
  if (prm.energy) {
    double e = static_cast<double>(e_acc);
    // threads of a CTA that returned early contribute nothing; reduce
    // within the warp of the active ones
    const unsigned mask = __activemask();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o = __shfl_down_sync(mask, e, off);
      if ((threadIdx.x + off) < 32 && ((mask >> (threadIdx.x + off)) & 1u)) e += o;
    }
    if (threadIdx.x == 0) {
      const int step = *prm.d_step + prm.step_offset;
      if (step >= 0 && step < prm.energy_cap) atomicAdd(&prm.energy[step], e);
    }
  }
}

template <int MEDIUM, bool SPONGE>
cudaError_t launch_exact_t(Sim *sim, const StepParams &prm) {
  const int nx = prm.x1 - prm.x0, ny = prm.y1 - prm.y0, nz = prm.z1 - prm.z0;
  dim3 grid((nx + 31) / 32, (ny + 3) / 4, (nz + prm.zchunk - 1) / prm.zchunk);
  exact_kernel<MEDIUM, SPONGE><<<grid, dim3(32, 4), 0, sim->stream>>>(prm);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_exact(Sim *sim, const StepParams &prm) {
  const bool sp = prm.sponge != nullptr;
  if (sim->medium == DC_GB300_MEDIUM_PRECOMP)
    return sp ? launch_exact_t<DC_GB300_MEDIUM_PRECOMP, true>(sim, prm)
              : launch_exact_t<DC_GB300_MEDIUM_PRECOMP, false>(sim, prm);
  return sp ? launch_exact_t<DC_GB300_MEDIUM_VPZ_VSV, true>(sim, prm)
            : launch_exact_t<DC_GB300_MEDIUM_VPZ_VSV, false>(sim, prm);
}

}  // namespace dcg
