// tti_exact.cu -- the bit-exact sm_103a Fletcher TTI time step.
//
// Same update as the fast kernel, but every floating-point operation is the
// reference's, in the reference's order, with explicit round-to-nearest
// intrinsics so that nothing is contracted into an FMA:
//   der2      include/derivatives.h:47-54   (9-point second derivative)
//   derCross  include/derivatives.h:56-91   (64-point direct cross sum)
//   update    include/sample_compute.h:229-275 (sample_compute) or
//             include/sample_compute.h:51-101  (sample_compute_optimized,
//             the vpz/vsv medium form with constant angles).
// Results are bit-identical to the reference's OpenMP path built without
// FMA contraction (and to its CUDA arithmetic executed the same way).
//
// Data path: a CTA owns a 32 x 4 column tile and sweeps a chunk of z.  The
// stencil reads go through the read-only data cache; each point reads 434
// stencil values, so this kernel is bound by L1 bandwidth, not HBM.  It is
// the parity anchor, not the throughput path.
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

__device__ __forceinline__ float der2_x(const float *__restrict__ p,
                                        long long i, long long s, float inv) {
  float a = __fmul_rn(kw(0), __ldg(p + i));
  a = __fadd_rn(a, __fmul_rn(kw(1), __fadd_rn(__ldg(p + i + s), __ldg(p + i - s))));
  a = __fadd_rn(a, __fmul_rn(kw(2), __fadd_rn(__ldg(p + i + 2 * s), __ldg(p + i - 2 * s))));
  a = __fadd_rn(a, __fmul_rn(kw(3), __fadd_rn(__ldg(p + i + 3 * s), __ldg(p + i - 3 * s))));
  a = __fadd_rn(a, __fmul_rn(kw(4), __fadd_rn(__ldg(p + i + 4 * s), __ldg(p + i - 4 * s))));
  return __fmul_rn(a, inv);
}

__device__ __forceinline__ float cross_x(const float *__restrict__ p,
                                         long long i, long long s1,
                                         long long s2, float inv) {
  float total = 0.0f;
#pragma unroll
  for (int g = 0; g < 10; ++g) {
    const long long a = pair_a(g), b = pair_b(g);
    float acc = __ldg(p + i + a * s2 + b * s1);
    acc = __fsub_rn(acc, __ldg(p + i + a * s2 - b * s1));
    acc = __fsub_rn(acc, __ldg(p + i - a * s2 + b * s1));
    acc = __fadd_rn(acc, __ldg(p + i - a * s2 - b * s1));
    if (a != b) {
      acc = __fadd_rn(acc, __ldg(p + i + b * s2 + a * s1));
      acc = __fsub_rn(acc, __ldg(p + i + b * s2 - a * s1));
      acc = __fsub_rn(acc, __ldg(p + i - b * s2 + a * s1));
      acc = __fadd_rn(acc, __ldg(p + i - b * s2 - a * s1));
    }
    const float w = static_cast<float>(lw(pair_a(g)) * lw(pair_b(g)));
    const float term = __fmul_rn(w, acc);
    total = g == 0 ? term : __fadd_rn(total, term);
  }
  return __fmul_rn(total, inv);
}

struct H12 {
  float h1, h2;
};

// `f` points at one component of a pair buffer: element strides are doubled
// (sX = 2, sY = 2*pitch, sZ = 2*plane, i = 2*index).
__device__ __forceinline__ H12 hterms(const float *__restrict__ f, long long i,
                                      long long sX, long long sY, long long sZ,
                                      const StepParams &prm, float cxx,
                                      float cyy, float czz, float cxy,
                                      float cyz, float cxz) {
  const float fxx = der2_x(f, i, sX, prm.dxxinv);
  const float fyy = der2_x(f, i, sY, prm.dyyinv);
  const float fzz = der2_x(f, i, sZ, prm.dzzinv);
  const float fxy = cross_x(f, i, sX, sY, prm.dxyinv);
  const float fyz = cross_x(f, i, sY, sZ, prm.dyzinv);
  const float fxz = cross_x(f, i, sX, sZ, prm.dxzinv);
  float h1 = __fmul_rn(cxx, fxx);
  h1 = __fadd_rn(h1, __fmul_rn(cyy, fyy));
  h1 = __fadd_rn(h1, __fmul_rn(czz, fzz));
  h1 = __fadd_rn(h1, __fmul_rn(cxy, fxy));
  h1 = __fadd_rn(h1, __fmul_rn(cxz, fxz));
  h1 = __fadd_rn(h1, __fmul_rn(cyz, fyz));
  const float h2 = __fsub_rn(__fadd_rn(__fadd_rn(fxx, fyy), fzz), h1);
  return H12{h1, h2};
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
    const float *pcf = reinterpret_cast<const float *>(prm.cur);
    const H12 hp = hterms(pcf, 2 * i, 2, 2 * sY, 2 * sZ, prm, cxx, cyy, czz, cxy, cyz, cxz);
    const H12 hq = hterms(pcf + 1, 2 * i, 2, 2 * sY, 2 * sZ, prm, cxx, cyy, czz, cxy, cyz, cxz);
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
