// tti_fast.cu -- the fast sm_103a Fletcher TTI time step.
//
// One pass updates p and q (the coupled pseudo-acoustic TTI system of the
// reference, include/sample_compute.h:105-185) for every point of a box.
//
// Work decomposition: a CTA owns a TX x TY column tile in (x, y) and sweeps
// a chunk of output planes along z.  For the leading plane k it receives,
// by TMA into a NSTAGE-deep shared-memory ring:
//   * the p and q planes k with a 4-cell halo in x and y,
//   * cxx, cyy, cxy at plane k   (in-plane coefficients),
//   * the other seven coefficients and pp, qp at the output plane z = k - 4.
// Each thread owns one (x, y) column and keeps, in registers, a 9-deep queue
// per field of the centre value, the unscaled first x-derivative and the
// unscaled first y-derivative.  The cross derivatives are evaluated in their
// separable form: with the 8th-order first-derivative weights L1..L4, the
// reference's 64-point derCross (include/derivatives.h:56-91) equals
// D_a(D_b p) because its weights are L_ab = L_a * L_b.  So
//   d2p/dxdy  = D_x of the y-derivative plane (shared memory, per plane),
//   d2p/dxdz  = D_z of the x-derivative queue (registers),
//   d2p/dydz  = D_z of the y-derivative queue (registers),
// and the in-plane part of H1/H2 is formed at the leading plane and delayed
// four planes in registers.  Rounding differs from the reference's direct
// sums (see the exact kernel for bit-identical results).
//
// Algorithmic (compulsory) DRAM traffic per point-update: read pc, qc, pp,
// qp and ten coefficients, write pp and qp: 64 bytes (32 bytes for the
// vpz/vsv medium form).
#include <cstdio>
#include <cstdlib>

#include "dc_internal.h"
#include "dc_ptx.cuh"

namespace dcg {
namespace {

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per TMA wait

constexpr int align128(int b) { return (b + 127) / 128 * 128; }

template <int TX, int TY, int NSTAGE, int MEDIUM>
struct FastLayout {
  static constexpr int HX = TX + 2 * kHalo;
  static constexpr int HY = TY + 2 * kHalo;
  static constexpr int NT = TX * TY;
  static constexpr int NCA = MEDIUM == DC_GB300_MEDIUM_PRECOMP ? 3 : 0;
  static constexpr int NCB = MEDIUM == DC_GB300_MEDIUM_PRECOMP ? 7 : 2;
  // a halo plane of (p, q) pairs, HY rows of HX pairs
  static constexpr int HALO_BYTES = align128(HX * HY * 8);
  static constexpr int TILE4 = NT * 4;  // one coefficient tile (128-B multiple)
  static constexpr int OFF_H = 0;
  static constexpr int OFF_CA = HALO_BYTES;
  static constexpr int OFF_CB = OFF_CA + NCA * TILE4;
  static constexpr int OFF_OWN = OFF_CB + NCB * TILE4;  // (pp, qp) pairs
  static constexpr int STAGE_BYTES = OFF_OWN + NT * 8;
  static constexpr int DY_BYTES = align128(TY * HX * 8);  // (dy p, dy q) pairs
  static constexpr int OFF_DY = NSTAGE * STAGE_BYTES;     // 3 buffers
  // per-thread ring of the delayed in-plane terms (A_p, A_q, B_p, B_q) of
  // the last 9 planes
  static constexpr int OFF_AB = OFF_DY + 3 * DY_BYTES;
  static constexpr int OFF_BAR = OFF_AB + 9 * NT * 16;
  static constexpr int SMEM_BYTES = OFF_BAR + NSTAGE * 8;
  static constexpr uint32_t TX_HALO = HX * HY * 8u;
  static constexpr uint32_t TX_CA = NCA * NT * 4u;
  static constexpr uint32_t TX_OUT = NCB * NT * 4u + NT * 8u;
  static_assert(TX % 32 == 0, "a warp spans one tile row");
  static_assert(8 * TY <= NT, "halo-column work fits the CTA");
  static_assert(NSTAGE == 3, "stage index u % 3 is a compile-time constant");
};

// Packed FP32 pair arithmetic (one instruction updates p and q).
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// Second derivative of a (p, q) pair with pre-scaled weights w[0..4]
// (K_i / da^2), summed as two independent chains for instruction-level
// parallelism.
__device__ __forceinline__ float2 d2(const float *w, float2 c, float2 m1, float2 p1,
                                     float2 m2, float2 p2, float2 m3, float2 p3,
                                     float2 m4, float2 p4) {
  const float2 s1 = add2(m1, p1), s2 = add2(m2, p2), s3 = add2(m3, p3), s4 = add2(m4, p4);
  float2 t0 = fma2(bc(w[1]), s1, mul2(bc(w[0]), c));
  const float2 t1 = fma2(bc(w[3]), s3, mul2(bc(w[2]), s2));
  t0 = fma2(bc(w[4]), s4, t0);
  return add2(t0, t1);
}

// First derivative of a (p, q) pair with weights w[0..3] (L_i / da).
__device__ __forceinline__ float2 d1(const float *w, float2 m1, float2 p1, float2 m2,
                                     float2 p2, float2 m3, float2 p3, float2 m4, float2 p4) {
  const float2 n = bc(-1.0f);
  const float2 e1 = fma2(n, m1, p1), e2 = fma2(n, m2, p2), e3 = fma2(n, m3, p3),
               e4 = fma2(n, m4, p4);
  const float2 t0 = fma2(bc(w[2]), e3, mul2(bc(w[0]), e1));
  const float2 t1 = fma2(bc(w[3]), e4, mul2(bc(w[1]), e2));
  return add2(t0, t1);
}

// Constant-angle factors of the reference CUDA backend
// (include/sample_compute.h:9-18).
constexpr float kCxx = 0.1459632909f, kCyy = 0.3540367091f, kCzz = 0.5f;
constexpr float kCxy = 0.4546487134f, kCyz = 0.8414709848f;
constexpr float kCxz = 0.5403023059f;
constexpr float kV2pxFactor = 1.48f, kV2pnFactor = 1.2f;

template <int TX, int TY, int MEDIUM, bool SPONGE, bool ISO>
__global__ void __launch_bounds__(TX *TY, (TX * TY <= 256) ? 2 : 1)
    fast_kernel(const __grid_constant__ CUtensorMap tm_cur,
                const __grid_constant__ CUtensorMap tm_prev,
                const __grid_constant__ CUtensorMap tm_ca,
                const __grid_constant__ CUtensorMap tm_cb,
                const __grid_constant__ StepParams prm) {
  constexpr int NSTAGE = 3;
  using Lay = FastLayout<TX, TY, NSTAGE, MEDIUM>;
  constexpr int HX = Lay::HX;
  constexpr int NT = Lay::NT;
  // equal spacing on all axes: one set of weights serves x, y and z
  const float *w2x = prm.w2x, *w1x = prm.w1x;
  const float *w2y = ISO ? prm.w2x : prm.w2y, *w1y = ISO ? prm.w1x : prm.w1y;
  const float *w2z = ISO ? prm.w2x : prm.w2z, *w1z = ISO ? prm.w1x : prm.w1z;
  // No static shared memory in this kernel: the dynamic window starts at
  // the CTA's shared base, so this alignment holds and every access below
  // is a shared-space access at a compile-time offset.
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + Lay::OFF_BAR);

  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int x0 = prm.tile_x0 + static_cast<int>(blockIdx.x) * TX;
  const int y0 = prm.tile_y0 + static_cast<int>(blockIdx.y) * TY;
  const int zb = prm.z0 + static_cast<int>(blockIdx.z) * prm.zchunk;
  const int ze = min(zb + prm.zchunk, prm.z1);
  const int n_it = ze - zb + 2 * kHalo;
  const int gx = x0 + tx, gy = y0 + ty;
  const bool active =
      gx >= prm.x0 && gx < prm.x1 && gy >= prm.y0 && gy < prm.y1;

  // TMA destinations must be 128-byte aligned; refuse to run otherwise
  // (CTA-uniform, before any copy is issued).
  if (smem_u32(smem) & 127u) {
    if (tid == 0) atomicOr(prm.err, kErrAlign);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
    mbar_init_fence();
    prefetch_tensormap(&tm_cur);
    prefetch_tensormap(&tm_prev);
    prefetch_tensormap(&tm_cb);
    if (MEDIUM == DC_GB300_MEDIUM_PRECOMP) prefetch_tensormap(&tm_ca);
  }
  __syncthreads();

  // Producer: one elected thread fills stage j % 3 for iteration j.
  auto issue = [&](int j) {
    const int s = j % NSTAGE;
    unsigned char *st = smem + s * Lay::STAGE_BYTES;
    const int k = zb - kHalo + j;
    const bool want_ca = Lay::NCA > 0 && j >= kHalo && j < n_it - kHalo;
    const bool want_out = j >= 2 * kHalo;
    const uint32_t bytes = Lay::TX_HALO + (want_ca ? Lay::TX_CA : 0u) +
                           (want_out ? Lay::TX_OUT : 0u);
    mbar_arrive_expect_tx(&bars[s], bytes);
    tma_load_3d(st + Lay::OFF_H, &tm_cur, x0 - kHalo, y0 - kHalo, k, &bars[s]);
    if (want_ca) tma_load_4d(st + Lay::OFF_CA, &tm_ca, x0, y0, k, 0, &bars[s]);
    if (want_out) {
      tma_load_4d(st + Lay::OFF_CB, &tm_cb, x0, y0, k - kHalo,
                  MEDIUM == DC_GB300_MEDIUM_PRECOMP ? 3 : 0, &bars[s]);
      tma_load_3d(st + Lay::OFF_OWN, &tm_prev, x0, y0, k - kHalo, &bars[s]);
    }
  };

  if (tid == 0)
    for (int j = 0; j < NSTAGE - 1 && j < n_it; ++j) issue(j);

  // Register queues of (p, q) pairs indexed by plane mod 9 (compile-time
  // after unrolling): centre value, x- and y-derivative, and the delayed
  // in-plane parts A (of H1) and B (of the Laplacian).
  float2 cq[9], dxq[9], dyq[9];
  float4 *abr = reinterpret_cast<float4 *>(smem + Lay::OFF_AB);
  float2 e_acc = make_float2(0.f, 0.f);
  int abort_it = -1;

  // inactive threads of edge tiles may sit past the array: no profile read
  const float gxy = (SPONGE && active)
                        ? prm.sponge[gx] * prm.sponge[prm.sponge_oy + gy]
                        : 1.0f;
  const bool src_col = active && gx == prm.src_x && gy == prm.src_y;
  // receivers of this column at or below the first output plane
  int rk = 0, rend = 0, rnext = -1;
  if (prm.rec_col && active) {
    const int2 e = prm.rec_col[gy * prm.col_stride + gx];
    rk = e.x;
    rend = e.x + e.y;
    while (rk < rend && prm.rec_z[rk] < zb) ++rk;
    rnext = rk < rend ? prm.rec_z[rk] : -1;
  }
  const int c0 = (ty + kHalo) * HX + tx + kHalo;  // centre in a halo plane
  const int od = ty * HX + tx + kHalo;            // centre in a dy plane
  const int ot = ty * TX + tx;                    // centre in a tile
  // global position of this column at the first output plane (advanced by
  // one plane per output; never dereferenced for inactive threads)
  float2 *out = prm.prev + (static_cast<long long>(zb) * prm.plane +
                            static_cast<long long>(gy) * prm.pitch + gx);

  uint32_t mpar = 0;  // parity of the outer (9-plane) iteration
  for (int it0 = 0; it0 < n_it; it0 += 9, mpar ^= 1u) {
#pragma unroll
    for (int u = 0; u < 9; ++u) {
      const int it = it0 + u;
      if (it < n_it) {  // CTA-uniform
        // stage u % 3; its use count is it / 3 = 3 * (it0 / 9) + u / 3
        unsigned char *st = smem + (u % 3) * Lay::STAGE_BYTES;
        const bool ok = mbar_wait_bounded(&bars[u % 3],
                                          mpar ^ static_cast<uint32_t>((u / 3) & 1),
                                          kWaitLimitNs);
        const float2 *h = reinterpret_cast<const float2 *>(st + Lay::OFF_H);
        float2 *dyb = reinterpret_cast<float2 *>(smem + Lay::OFF_DY + (u % 3) * Lay::DY_BYTES);

        // ---- leading plane k: centre, x/y second and first derivatives
        float2 xx, yy;
        {
          const float2 c = h[c0];
          const float2 xm1 = h[c0 - 1], xp1 = h[c0 + 1], xm2 = h[c0 - 2],
                       xp2 = h[c0 + 2], xm3 = h[c0 - 3], xp3 = h[c0 + 3],
                       xm4 = h[c0 - 4], xp4 = h[c0 + 4];
          const float2 ym1 = h[c0 - HX], yp1 = h[c0 + HX],
                       ym2 = h[c0 - 2 * HX], yp2 = h[c0 + 2 * HX],
                       ym3 = h[c0 - 3 * HX], yp3 = h[c0 + 3 * HX],
                       ym4 = h[c0 - 4 * HX], yp4 = h[c0 + 4 * HX];
          xx = d2(w2x, c, xm1, xp1, xm2, xp2, xm3, xp3, xm4, xp4);
          yy = d2(w2y, c, ym1, yp1, ym2, yp2, ym3, yp3, ym4, yp4);
          cq[u] = c;
          dxq[u] = d1(w1x, xm1, xp1, xm2, xp2, xm3, xp3, xm4, xp4);
          dyq[u] = d1(w1y, ym1, yp1, ym2, yp2, ym3, yp3, ym4, yp4);
          dyb[od] = dyq[u];
        }
        // y-derivatives of the 4 + 4 halo columns (needed by d2/dxdy)
        if (tid < 8 * TY) {
          const int hc = tid & 7, hy = tid >> 3;
          const int hx = hc < 4 ? hc : TX + hc;
          const int o = (hy + kHalo) * HX + hx;
          dyb[hy * HX + hx] =
              d1(w1y, h[o - HX], h[o + HX], h[o - 2 * HX], h[o + 2 * HX],
                 h[o - 3 * HX], h[o + 3 * HX], h[o - 4 * HX], h[o + 4 * HX]);
        }
        if (__syncthreads_or(!ok)) {
          abort_it = it;
          goto done;
        }
        // The stage read in iteration it-1 is free: refill it.
        if (tid == 0 && it + NSTAGE - 1 < n_it) issue(it + NSTAGE - 1);

        // ---- in-plane part of H1 and of the Laplacian at plane k
        if (it >= kHalo && it < n_it - kHalo) {
          const float2 xy = d1(w1x, dyb[od - 1], dyb[od + 1], dyb[od - 2],
                               dyb[od + 2], dyb[od - 3], dyb[od + 3], dyb[od - 4],
                               dyb[od + 4]);
          float cxx, cyy, cxy;
          if (MEDIUM == DC_GB300_MEDIUM_PRECOMP) {
            const float *ca = reinterpret_cast<const float *>(st + Lay::OFF_CA);
            cxx = ca[ot];
            cyy = ca[NT + ot];
            cxy = ca[2 * NT + ot];
          } else {
            cxx = kCxx;
            cyy = kCyy;
            cxy = kCxy;
          }
          const float2 av = fma2(bc(cxy), xy, fma2(bc(cyy), yy, mul2(bc(cxx), xx)));
          const float2 bv = add2(xx, yy);
          abr[u * NT + ot] = make_float4(av.x, av.y, bv.x, bv.y);
        }

        // ---- output plane z = k - 4
        if (it >= 2 * kHalo) {
          // ring slots of planes z-4 .. z+4 (u is a compile-time constant)
          const int m4 = (u + 1) % 9, m3 = (u + 2) % 9, m2 = (u + 3) % 9,
                    m1 = (u + 4) % 9, c = (u + 5) % 9, p1 = (u + 6) % 9,
                    p2 = (u + 7) % 9, p3 = (u + 8) % 9, p4 = u;
          const float4 ab = abr[c * NT + ot];  // A, B of plane z (own column)
          const float2 zz = d2(w2z, cq[c], cq[m1], cq[p1], cq[m2], cq[p2], cq[m3],
                               cq[p3], cq[m4], cq[p4]);
          const float2 xz = d1(w1z, dxq[m1], dxq[p1], dxq[m2], dxq[p2],
                               dxq[m3], dxq[p3], dxq[m4], dxq[p4]);
          const float2 yz = d1(w1z, dyq[m1], dyq[p1], dyq[m2], dyq[p2],
                               dyq[m3], dyq[p3], dyq[m4], dyq[p4]);
          const float *cb = reinterpret_cast<const float *>(st + Lay::OFF_CB);
          const float2 *own = reinterpret_cast<const float2 *>(st + Lay::OFF_OWN);
          float czz, cxz, cyz, v2px, v2pz, v2sz, v2pn;
          if (MEDIUM == DC_GB300_MEDIUM_PRECOMP) {
            czz = cb[0 * NT + ot];
            cxz = cb[1 * NT + ot];
            cyz = cb[2 * NT + ot];
            v2px = cb[3 * NT + ot];
            v2pz = cb[4 * NT + ot];
            v2sz = cb[5 * NT + ot];
            v2pn = cb[6 * NT + ot];
          } else {
            const float vp = cb[ot], vs = cb[NT + ot];
            czz = kCzz;
            cxz = kCxz;
            cyz = kCyz;
            v2pz = vp * vp;
            v2sz = vs * vs;
            v2px = v2pz * kV2pxFactor;
            v2pn = v2pz * kV2pnFactor;
          }
          // (h1p, h1q) and (h2p, h2q)
          const float2 h1 = fma2(bc(cyz), yz,
                                 fma2(bc(cxz), xz, fma2(bc(czz), zz, make_float2(ab.x, ab.y))));
          const float2 h2 = fma2(bc(-1.0f), h1, add2(make_float2(ab.z, ab.w), zz));
          const float rhsp = fmaf(v2sz, h1.x - h1.y, fmaf(v2pz, h1.y, v2px * h2.x));
          const float rhsq = fmaf(-v2sz, h2.x - h2.y, fmaf(v2pz, h1.y, v2pn * h2.x));
          const float2 rhs = make_float2(rhsp, rhsq);
          const float2 pv = own[ot];
          const float2 cc = add2(cq[c], cq[c]);  // 2 * current
          float2 nv;
          if (SPONGE) {
            const int z = zb + it - 2 * kHalo;
            const float g = gxy * prm.sponge[prm.sponge_oz + z];
            nv = mul2(fma2(rhs, bc(prm.dt2), fma2(bc(-g), pv, cc)), bc(g));
          } else {
            nv = fma2(rhs, bc(prm.dt2), fma2(bc(-1.0f), pv, cc));
          }
          if (active) {
            if (prm.energy) e_acc = fma2(nv, nv, e_acc);
            const int z = zb + it - 2 * kHalo;
            if (z == rnext) {
              const int step = *prm.d_step + prm.step_offset;
              do {
                if (step >= 0 && step < prm.trace_cap)
                  prm.traces[static_cast<long long>(step) * prm.nrec + prm.rec_r[rk]] = nv.x;
                ++rk;
              } while (rk < rend && prm.rec_z[rk] == z);
              rnext = rk < rend ? prm.rec_z[rk] : -1;
            }
            if (src_col && z == prm.src_z) {
              const int step = *prm.d_step + prm.step_offset;
              const float sv =
                  step + 1 < prm.src_count ? prm.src_table[step + 1] : 0.0f;
              prm.src_pre[0] = nv.x;
              prm.src_pre[1] = nv.y;
              nv.x += sv;
              nv.y += sv;
            }
            *out = nv;
          }
          out += prm.plane;
        }
      }
    }
  }
done:
  if (abort_it >= 0) {
    // A TMA wait timed out: record it, give the copies still in flight a
    // bounded chance to land, and leave without touching the outputs.
    if (tid == 0) {
      atomicOr(prm.err, kErrTimeout);
      const int last = min(n_it, abort_it + NSTAGE - 1);
      for (int j = abort_it; j < last; ++j)
        mbar_wait_bounded(&bars[j % NSTAGE],
                          static_cast<uint32_t>(j / NSTAGE) & 1u, kWaitLimitNs);
    }
    return;
  }
  if (prm.energy) {
    // CTA reduction of the float partials in double, one atomic per CTA.
    double e = static_cast<double>(e_acc.x) + static_cast<double>(e_acc.y);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) e += __shfl_down_sync(0xffffffffu, e, off);
    double *red = reinterpret_cast<double *>(smem + Lay::OFF_DY);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = e;
    __syncthreads();
    if (tid == 0) {
      double tot = 0.0;
      for (int w = 0; w < NT / 32; ++w) tot += red[w];
      const int step = *prm.d_step + prm.step_offset;
      if (step >= 0 && step < prm.energy_cap) atomicAdd(&prm.energy[step], tot);
    }
  }
}

// Compiled tile shapes: TX = 32 (one warp per tile row) and TY = 8, 12 or
// 16 rows (256, 384 or 512 threads), a 3-stage TMA ring.
constexpr int kTX = 32, kStages = 3;

template <int TY, int MEDIUM, bool SPONGE, bool ISO>
cudaError_t launch_fast_t(Sim *sim, const StepParams &prm, int cur_buf, int prev_buf) {
  using Lay = FastLayout<kTX, TY, kStages, MEDIUM>;
  auto kern = fast_kernel<kTX, TY, MEDIUM, SPONGE, ISO>;
  const int nx = prm.x1 - prm.tile_x0, ny = prm.y1 - prm.tile_y0;
  const int nz = prm.z1 - prm.z0;
  dim3 grid((nx + kTX - 1) / kTX, (ny + TY - 1) / TY, (nz + prm.zchunk - 1) / prm.zchunk);
  kern<<<grid, kTX * TY, Lay::SMEM_BYTES, sim->stream>>>(
      sim->tm_halo[cur_buf], sim->tm_own[prev_buf], sim->tm_ca, sim->tm_cb, prm);
  return cudaGetLastError();
}

template <int TY, int MEDIUM>
cudaError_t set_smem_attr_all() {
  using Lay = FastLayout<kTX, TY, kStages, MEDIUM>;
  cudaError_t e = cudaSuccess;
  const int b = Lay::SMEM_BYTES;
  const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, MEDIUM, false, false>, attr, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, MEDIUM, false, true>, attr, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, MEDIUM, true, false>, attr, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, MEDIUM, true, true>, attr, b);
  return e;
}

template <int TY>
cudaError_t launch_ty(Sim *sim, const StepParams &prm, int cur, int prev) {
  const bool sp = prm.sponge != nullptr;
  const bool iso = sim->dx == sim->dy && sim->dy == sim->dz;
  constexpr int P = DC_GB300_MEDIUM_PRECOMP, V = DC_GB300_MEDIUM_VPZ_VSV;
  if (sim->medium == P) {
    if (sp) return iso ? launch_fast_t<TY, P, true, true>(sim, prm, cur, prev)
                       : launch_fast_t<TY, P, true, false>(sim, prm, cur, prev);
    return iso ? launch_fast_t<TY, P, false, true>(sim, prm, cur, prev)
               : launch_fast_t<TY, P, false, false>(sim, prm, cur, prev);
  }
  if (sp) return iso ? launch_fast_t<TY, V, true, true>(sim, prm, cur, prev)
                     : launch_fast_t<TY, V, true, false>(sim, prm, cur, prev);
  return iso ? launch_fast_t<TY, V, false, true>(sim, prm, cur, prev)
             : launch_fast_t<TY, V, false, false>(sim, prm, cur, prev);
}

// 32 x 8 tiles with two CTAs per SM measured fastest on GB300 (616^3 cube:
// 2.83 ms per step vs 3.09 ms for 32 x 16 and 3.44 ms for 32 x 12);
// DC_GB300_FAST_TY=12|16 selects the others.
int chosen_ty() {
  const char *e = std::getenv("DC_GB300_FAST_TY");
  const int v = e ? std::atoi(e) : 0;
  return (v == 12 || v == 16) ? v : 8;
}

}  // namespace

FastShape fast_shape(const Sim *sim) {
  // z-chunk: enough CTAs for several waves over 152 SMs while keeping the
  // 8-plane warm-up of each chunk small.
  const int ty = sim->maps_ty ? sim->maps_ty : chosen_ty();
  const long long tiles = ((sim->sx - 8 + kTX - 1) / kTX + 1) *
                          ((sim->sy - 8 + ty - 1) / ty);
  const long long nzc = sim->sz - 8;
  long long chunks = (4 * 152 + tiles - 1) / tiles;
  long long zc = (nzc + chunks - 1) / chunks;
  if (zc < 32) zc = 32;
  if (zc > nzc) zc = nzc;
  return FastShape{kTX, ty, static_cast<int>(zc)};
}

bool fast_encode_maps(Sim *sim, std::string *err) {
  // dynamic shared memory above 48 KB must be enabled per kernel and device
  // (done here, before any stream capture)
  const int kTY = chosen_ty();
  cudaError_t ae;
  if (kTY == 8)
    ae = sim->medium == DC_GB300_MEDIUM_PRECOMP ? set_smem_attr_all<8, DC_GB300_MEDIUM_PRECOMP>()
                                                : set_smem_attr_all<8, DC_GB300_MEDIUM_VPZ_VSV>();
  else if (kTY == 12)
    ae = sim->medium == DC_GB300_MEDIUM_PRECOMP ? set_smem_attr_all<12, DC_GB300_MEDIUM_PRECOMP>()
                                                : set_smem_attr_all<12, DC_GB300_MEDIUM_VPZ_VSV>();
  else
    ae = sim->medium == DC_GB300_MEDIUM_PRECOMP ? set_smem_attr_all<16, DC_GB300_MEDIUM_PRECOMP>()
                                                : set_smem_attr_all<16, DC_GB300_MEDIUM_VPZ_VSV>();
  if (ae != cudaSuccess) {
    *err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(ae);
    return false;
  }
  const uint64_t dims3[3] = {static_cast<uint64_t>(sim->sx),
                             static_cast<uint64_t>(sim->sy),
                             static_cast<uint64_t>(sim->sz)};
  // (p, q) pair buffers: 8-byte elements
  const uint64_t str_pq[2] = {static_cast<uint64_t>(sim->pitch) * 8,
                              static_cast<uint64_t>(sim->plane) * 8};
  const uint32_t box_halo[3] = {kTX + 8, kTY + 8, 1};
  const uint32_t box_own[3] = {kTX, kTY, 1};
  for (int b = 0; b < 2; ++b) {
    if (!encode_tiled(&sim->tm_halo[b], sim->pq[b], 3, dims3, str_pq, box_halo, err, true))
      return false;
    if (!encode_tiled(&sim->tm_own[b], sim->pq[b], 3, dims3, str_pq, box_own, err, true))
      return false;
  }
  // coefficient arrays: 4-byte elements
  const uint64_t str3[2] = {static_cast<uint64_t>(sim->pitch) * 4,
                            static_cast<uint64_t>(sim->plane) * 4};
  const uint64_t str4[3] = {str3[0], str3[1],
                            static_cast<uint64_t>(sim->count) * 4};
  if (sim->medium == DC_GB300_MEDIUM_PRECOMP) {
    const uint64_t dims4[4] = {dims3[0], dims3[1], dims3[2], DC_NCOEF};
    const uint32_t box_a[4] = {kTX, kTY, 1, 3};
    const uint32_t box_b[4] = {kTX, kTY, 1, 7};
    if (!encode_tiled(&sim->tm_ca, sim->coef, 4, dims4, str4, box_a, err)) return false;
    if (!encode_tiled(&sim->tm_cb, sim->coef, 4, dims4, str4, box_b, err)) return false;
  } else {
    const uint64_t dims4[4] = {dims3[0], dims3[1], dims3[2], 2};
    const uint32_t box_b[4] = {kTX, kTY, 1, 2};
    if (!encode_tiled(&sim->tm_cb, sim->vv, 4, dims4, str4, box_b, err)) return false;
    sim->tm_ca = sim->tm_cb;  // unused by this medium form
  }
  sim->maps_tx = kTX;
  sim->maps_ty = kTY;
  return true;
}

cudaError_t launch_fast(Sim *sim, const StepParams &prm, int cur_buf, int prev_buf) {
  if (sim->maps_ty == 8) return launch_ty<8>(sim, prm, cur_buf, prev_buf);
  if (sim->maps_ty == 12) return launch_ty<12>(sim, prm, cur_buf, prev_buf);
  return launch_ty<16>(sim, prm, cur_buf, prev_buf);
}

}  // namespace dcg
