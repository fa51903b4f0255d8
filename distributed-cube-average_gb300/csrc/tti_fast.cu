// tti_fast.cu -- the fast sm_103a Fletcher TTI time step.
//
// One pass updates p and q (the coupled pseudo-acoustic TTI system of the
// reference, include/sample_compute.h:105-185) for every point of a box.
//
// Work decomposition: a CTA owns a 32 x TY column tile in (x, y) and sweeps
// a chunk of output planes along z.  For the leading plane k it receives,
// by TMA into a 3-deep shared-memory ring:
//   * the (p, q) pairs of plane k with a 4-cell halo in x and y and the
//     in-plane coefficient group (cxx, cyy, cxy, czz) of plane k,
//   * the other coefficients and the (pp, qp) tile of the output plane
//     z = k - 4.
// Each thread owns one (x, y) column and keeps, in registers, 9-deep queues
// of (p, q) pairs: the centre value, the x-derivative and the y-derivative.
// The cross derivatives are evaluated in their separable form: with the
// 8th-order first-derivative weights L1..L4 the reference's 64-point
// derCross (include/derivatives.h:56-91) has weights L_ab = L_a * L_b, so it
// equals D_a(D_b p):
//   d2/dxdy = D_x of a shared-memory plane of the y-derivative,
//   d2/dxdz = D_z of the x-derivative queue,
//   d2/dydz = D_z of the y-derivative queue.
// The in-plane part of H1 (cxx d2/dx2 + cyy d2/dy2 + cxy d2/dxdy), the
// in-plane Laplacian and czz of plane k wait four planes in a per-thread
// shared-memory ring (9 slots, indexed by the compile-time plane number)
// until plane k is the output plane.
//
// The sweep of one column tile is `sweep_column`; `fast_kernel` runs one
// tile per CTA over one box, `batch_kernel` runs persistent CTAs over the
// tiles of many boxes (shots) cropped out of one shared medium.
// Rounding differs from the reference's direct sums (the exact kernel is
// bit-identical).
//
// p and q are processed as pairs with packed f32x2 arithmetic (FFMA2,
// FADD2, FMUL2): one instruction updates both fields.
//
// Medium forms (CoefForm): CF_F32 reads the grouped FP32 coefficients
// (40 B/point); CF_VV reads (vpz, vsv) with the reference CUDA backend's
// constant angles (8 B/point); CF_F16 / CF_BF16 read a 20 B/point copy in
// FP16 / BF16 (the mixed-precision form), converted to FP32 on load -- all
// arithmetic stays FP32.
//
// Compulsory DRAM traffic per point-update: read (pc,qc) 8 B, (pp,qp) 8 B and
// the medium, write (pp,qp) 8 B: 64 B (CF_F32), 32 B (CF_VV), 44 B (CF_F16,
// CF_BF16).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "dc_internal.h"
#include "dc_ptx.cuh"

namespace dcg {
namespace {

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per TMA wait

constexpr int align128(int b) { return (b + 127) / 128 * 128; }

template <int CF>
struct CoefBytes {
  // bytes per point of each coefficient group: L (cxx, cyy, cxy, czz) is
  // read at the leading plane, O1 and O2 (the rest) at the output plane
  static constexpr int L = CF == CF_F32 ? 16 : CF == CF_VV ? 0 : 8;
  static constexpr int O1 = CF == CF_F32 ? 16 : 8;  // VV: (vpz, vsv)
  static constexpr int O2 = CF == CF_F32 ? 8 : CF == CF_VV ? 0 : 4;
};

template <int TX, int TY, int CF, int NS = 3>
struct FastLayout {
  using CB = CoefBytes<CF>;
  static constexpr int HX = TX + 2 * kHalo;
  static constexpr int HY = TY + 2 * kHalo;
  static constexpr int NT = TX * TY;
  // TMA ring depth: 3, or 4 for large FP32 ten-coefficient boxes (their
  // 17 KB stages land late when the whole GPU streams from DRAM; see
  // fast_encode_maps)
  static constexpr int NSTAGE = NS;
  static_assert(NS == 3 || NS == 4, "ring depth");
  static constexpr int HALO_BYTES = align128(HX * HY * 8);  // (p, q) pairs
  static constexpr int OFF_H = 0;
  static constexpr int OFF_L = HALO_BYTES;
  static constexpr int OFF_O1 = OFF_L + NT * CB::L;
  static constexpr int OFF_O2 = OFF_O1 + NT * CB::O1;
  static constexpr int OFF_OWN = align128(OFF_O2 + NT * CB::O2);  // (pp, qp) pairs
  // FP16 form: the velocity bases of the tile's TY rows at the output plane
  static constexpr int VB = CF == CF_F16 ? 16 : 0;
  static constexpr int OFF_VB = align128(OFF_OWN + NT * 8);
  static constexpr int STAGE_BYTES = align128(OFF_VB + TY * VB);
  static constexpr int DY_BYTES = align128(TY * HX * 8);      // y-derivative plane
  static constexpr int OFF_DY = NSTAGE * STAGE_BYTES;         // 3 buffers
  // per-thread ring of the delayed in-plane terms of the last 9 planes:
  // (A_p, A_q, B_p, B_q) and czz
  // delayed in-plane terms: 9 slots indexed by the compile-time plane
  // number of the 9-plane unrolled body, or -- where the fourth TMA stage
  // needs the room for two CTAs per SM -- the 5 slots the 4-plane delay
  // needs, indexed at run time
  static constexpr int RING = NSTAGE == 4 ? 5 : 9;
  static_assert(RING == 9 || RING == 5, "ring slots");
  static constexpr int OFF_RA = OFF_DY + 3 * DY_BYTES;
  static constexpr int OFF_RZ = OFF_RA + RING * NT * 16;
  static constexpr int OFF_BAR = OFF_RZ + RING * NT * 4;
  static constexpr int SMEM_BYTES = OFF_BAR + NSTAGE * 8;
  static constexpr uint32_t TX_HALO = HX * HY * 8u;
  static constexpr uint32_t TX_LEAD = NT * CB::L;
  static constexpr uint32_t TX_OUT = NT * (CB::O1 + CB::O2) + NT * 8u + TY * VB;
  static_assert(TX % 32 == 0, "a warp spans one tile row");
  static_assert(8 * TY <= NT, "halo-column work fits the CTA");
};

// Packed FP32 pair arithmetic (one instruction updates p and q).
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// Second derivative of a (p, q) pair with pre-scaled weights w[0..4]
// (K_i / da^2), summed as two independent chains.
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

// With equal spacing on all axes the stencil uses the unscaled 8th-order
// weights (K_i for the second derivative, L_i for the first) as
// compile-time constants and applies 1/d^2 once, in dt2_iso: every term of
// the update is a second derivative, so the scale factors out of the sum.
constexpr float kK0 = -205.0f / 72.0f, kK1 = 8.0f / 5.0f, kK2 = -1.0f / 5.0f,
                kK3 = 8.0f / 315.0f, kK4 = -1.0f / 560.0f;
constexpr float kL1 = 4.0f / 5.0f, kL2 = -1.0f / 5.0f, kL3 = 4.0f / 105.0f,
                kL4 = -1.0f / 280.0f;

// Two forms of each derivative with the constant weights: two FMA chains
// summed at the end (shorter dependency chains), or one chain (one
// instruction fewer).  The FP16/BF16 sweeps run 2 % faster with the second
// (64-shot FP16 batch: 32.57 vs 33.19 ms); the FP32-medium sweep, nearer its
// memory bound, gains nothing from it and keeps the first.
template <bool CHAIN>
__device__ __forceinline__ float2 d2k(float2 c, float2 m1, float2 p1, float2 m2, float2 p2,
                                      float2 m3, float2 p3, float2 m4, float2 p4) {
  const float2 s1 = add2(m1, p1), s2 = add2(m2, p2), s3 = add2(m3, p3), s4 = add2(m4, p4);
  if (CHAIN) {
    float2 t = fma2(bc(kK1), s1, mul2(bc(kK0), c));
    t = fma2(bc(kK2), s2, t);
    t = fma2(bc(kK3), s3, t);
    return fma2(bc(kK4), s4, t);
  }
  float2 t0 = fma2(bc(kK1), s1, mul2(bc(kK0), c));
  const float2 t1 = fma2(bc(kK3), s3, mul2(bc(kK2), s2));
  t0 = fma2(bc(kK4), s4, t0);
  return add2(t0, t1);
}

template <bool CHAIN>
__device__ __forceinline__ float2 d1k(float2 m1, float2 p1, float2 m2, float2 p2, float2 m3,
                                      float2 p3, float2 m4, float2 p4) {
  const float2 n = bc(-1.0f);
  const float2 e1 = fma2(n, m1, p1), e2 = fma2(n, m2, p2), e3 = fma2(n, m3, p3),
               e4 = fma2(n, m4, p4);
  if (CHAIN) {
    float2 t = fma2(bc(kL2), e2, mul2(bc(kL1), e1));
    t = fma2(bc(kL3), e3, t);
    return fma2(bc(kL4), e4, t);
  }
  const float2 t0 = fma2(bc(kL3), e3, mul2(bc(kL1), e1));
  const float2 t1 = fma2(bc(kL4), e4, mul2(bc(kL2), e2));
  return add2(t0, t1);
}

// Second / first derivative with the runtime weights w, or with the
// unscaled constants when ISO.
template <bool ISO, bool CHAIN>
__device__ __forceinline__ float2 d2s(const float *w, float2 c, float2 m1, float2 p1, float2 m2,
                                      float2 p2, float2 m3, float2 p3, float2 m4, float2 p4) {
  return ISO ? d2k<CHAIN>(c, m1, p1, m2, p2, m3, p3, m4, p4)
             : d2(w, c, m1, p1, m2, p2, m3, p3, m4, p4);
}
template <bool ISO, bool CHAIN>
__device__ __forceinline__ float2 d1s(const float *w, float2 m1, float2 p1, float2 m2, float2 p2,
                                      float2 m3, float2 p3, float2 m4, float2 p4) {
  return ISO ? d1k<CHAIN>(m1, p1, m2, p2, m3, p3, m4, p4)
             : d1(w, m1, p1, m2, p2, m3, p3, m4, p4);
}

// Constant-angle factors of the reference CUDA backend
// (include/sample_compute.h:9-18).
constexpr float kCxx = 0.1459632909f, kCyy = 0.3540367091f, kCzz = 0.5f;
constexpr float kCxy = 0.4546487134f, kCyz = 0.8414709848f;
constexpr float kCxz = 0.5403023059f;
constexpr float kV2pxFactor = 1.48f, kV2pnFactor = 1.2f;

struct Medium {
  float cxx, cyy, cxy, czz, cxz, cyz, v2px, v2pz, v2sz, v2pn;
};

__device__ __forceinline__ float2 h2f(uint32_t v, bool bf16) {
  if (bf16) {  // bfloat16 -> float: the 16 bits are the float's high half
    return make_float2(__uint_as_float(v << 16), __uint_as_float(v & 0xffff0000u));
  }
  __half2 h;
  *reinterpret_cast<uint32_t *>(&h) = v;
  return __half22float2(h);
}

// Two 16-bit fixed-point values (low half first, each stored biased by
// 2^15) as exact floats: a byte permutation places each half in the low
// mantissa bits of 2^23, and one packed subtraction of 2^23 + 2^15 removes
// both offsets.  The values come out scaled by 2^15; the sweep unscales H1
// once.
__device__ __forceinline__ float2 fx2f(uint32_t w) {
  const uint32_t lo = __byte_perm(w, 0x4b000000u, 0x7610);
  const uint32_t hi = __byte_perm(w, 0x4b000000u, 0x7632);
  return __fadd2_rn(make_float2(__uint_as_float(lo), __uint_as_float(hi)),
                    make_float2(-8421376.0f, -8421376.0f));
}

// Scale of the angle terms as the kernel reads them (1 / 2^15 for the
// fixed-point FP16 form, applied to H1).
template <int CF>
constexpr float kChUnscale = CF == CF_F16 ? 1.0f / 32768.0f : 1.0f;

// (cxx, cyy, cxy, czz) of the thread's point at the leading plane.
template <int CF>
__device__ __forceinline__ float4 load_lead(const unsigned char *l, int ot) {
  if (CF == CF_F32) return reinterpret_cast<const float4 *>(l)[ot];
  if (CF == CF_VV) return make_float4(kCxx, kCyy, kCxy, kCzz);
  const uint2 h = reinterpret_cast<const uint2 *>(l)[ot];
  const float2 a = CF == CF_F16 ? fx2f(h.x) : h2f(h.x, true);
  const float2 b = CF == CF_F16 ? fx2f(h.y) : h2f(h.y, true);
  return make_float4(a.x, a.y, b.x, b.y);
}

// (cxz, cyz, v2px, v2pz, v2sz, v2pn) of the thread's point at the output
// plane.
struct OutMedium {
  float cxz, cyz, v2px, v2pz, v2sz, v2pn;
};

template <int CF>
__device__ __forceinline__ OutMedium load_out(const unsigned char *o1, const unsigned char *o2,
                                              int ot, float4 vb) {
  if (CF == CF_F32) {
    const float4 g1 = reinterpret_cast<const float4 *>(o1)[ot];
    const float2 g2 = reinterpret_cast<const float2 *>(o2)[ot];
    return OutMedium{g1.x, g1.y, g1.z, g1.w, g2.x, g2.y};
  }
  if (CF == CF_VV) {
    // include/sample_compute.h:51-54
    const float2 v = reinterpret_cast<const float2 *>(o1)[ot];
    const float v2pz = v.x * v.x;
    return OutMedium{kCxz, kCyz, v2pz * kV2pxFactor, v2pz, v.y * v.y, v2pz * kV2pnFactor};
  }
  const uint2 h = reinterpret_cast<const uint2 *>(o1)[ot];
  const uint32_t h2 = reinterpret_cast<const uint32_t *>(o2)[ot];
  if (CF == CF_F16) {
    // fixed-point cxz, cyz (x 2^15); velocity v = b + b * d from the row's
    // bases vb and the FP16 ratios d
    const float2 a = fx2f(h.x), b = h2f(h.y, false), c = h2f(h2, false);
    return OutMedium{a.x, a.y, fmaf(vb.x, b.x, vb.x), fmaf(vb.y, b.y, vb.y),
                     fmaf(vb.z, c.x, vb.z), fmaf(vb.w, c.y, vb.w)};
  }
  const float2 a = h2f(h.x, true), b = h2f(h.y, true), c = h2f(h2, true);
  return OutMedium{a.x, a.y, b.x, b.y, c.x, c.y};
}

// Sweeps the column tile at (x0, y0) over the output planes [zb, ze) of the
// box in prm, with the CTA's shared memory `smem` (128-byte aligned).  The
// FD weights, dt2 and the energy output are read from `cw`, the parameters
// shared by every box of the launch (kept at fixed constant-bank offsets so
// they feed the arithmetic directly).
// Returns false if a TMA wait timed out: the error word is set and the
// copies in flight have been given a bounded chance to land.
template <int TX, int TY, int CF, bool SPONGE, bool ISO, int NS>
__device__ __forceinline__ bool sweep_column(const CUtensorMap *tm_cur,
                                             const CUtensorMap *tm_prev,
                                             const CUtensorMap *tm_l,
                                             const CUtensorMap *tm_o1,
                                             const CUtensorMap *tm_o2,
                                             const CUtensorMap *tm_vb, const StepParams &prm,
                                             const StepParams &cw, const int x0, const int y0, const int zb,
                                             const int ze, unsigned char *smem) {
  using Lay = FastLayout<TX, TY, CF, NS>;
  using CB = CoefBytes<CF>;
  constexpr int NSTAGE = Lay::NSTAGE;
  constexpr int HX = Lay::HX;
  constexpr int NT = Lay::NT;
  // single-chain derivatives for the narrow-coefficient sweeps (see d2k)
  constexpr bool CHAIN = CF == CF_F16 || CF == CF_BF16;
  // equal spacing on all axes: one set of weights serves x, y and z
  const float *w2x = cw.w2x, *w1x = cw.w1x;
  const float *w2y = ISO ? cw.w2x : cw.w2y, *w1y = ISO ? cw.w1x : cw.w1y;
  const float *w2z = ISO ? cw.w2x : cw.w2z, *w1z = ISO ? cw.w1x : cw.w1z;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + Lay::OFF_BAR);

  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int n_it = ze - zb + 2 * kHalo;
  const int gx = x0 + tx, gy = y0 + ty;
  const bool active =
      gx >= prm.x0 && gx < prm.x1 && gy >= prm.y0 && gy < prm.y1;
  // medium coordinates of the tile
  const int mx0 = x0 + prm.mox, my0 = y0 + prm.moy;

  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
    mbar_init_fence();
    prefetch_tensormap(tm_cur);
    prefetch_tensormap(tm_prev);
    if (CB::L) prefetch_tensormap(tm_l);
    prefetch_tensormap(tm_o1);
    if (CB::O2) prefetch_tensormap(tm_o2);
    if (Lay::VB) prefetch_tensormap(tm_vb);
  }
  __syncthreads();

  // Producer: one elected thread fills stage j % 3 for iteration j.
  auto issue = [&](int j) {
    const int s = j % NSTAGE;
    unsigned char *st = smem + s * Lay::STAGE_BYTES;
    const int k = zb - kHalo + j;
    const bool want_lead = CB::L > 0 && j >= kHalo && j < n_it - kHalo;
    const bool want_out = j >= 2 * kHalo;
    mbar_arrive_expect_tx(&bars[s], Lay::TX_HALO + (want_lead ? Lay::TX_LEAD : 0u) +
                                        (want_out ? Lay::TX_OUT : 0u));
    tma_load_3d(st + Lay::OFF_H, tm_cur, x0 - kHalo, y0 - kHalo, k, &bars[s]);
    // 16-byte groups are mapped as two 8-byte elements per point (x
    // coordinate 2 * x: one 512-byte row per tile row), 8- and 4-byte groups
    // as one element per point
    constexpr int XL = CB::L == 16 ? 2 : 1, XO = CB::O1 == 16 ? 2 : 1;
    if (want_lead) tma_load_3d(st + Lay::OFF_L, tm_l, XL * mx0, my0, k + prm.moz, &bars[s]);
    if (want_out) {
      const int z = k - kHalo;
      const int mz = z + prm.moz;
      tma_load_3d(st + Lay::OFF_O1, tm_o1, XO * mx0, my0, mz, &bars[s]);
      if (CB::O2) tma_load_3d(st + Lay::OFF_O2, tm_o2, mx0, my0, mz, &bars[s]);
      // FP16 form: rows my0 .. my0 + TY - 1 of the bases (two 8-byte
      // elements per row)
      if (Lay::VB) tma_load_2d(st + Lay::OFF_VB, tm_vb, 2 * my0, mz, &bars[s]);
      tma_load_3d(st + Lay::OFF_OWN, tm_prev, x0, y0, z, &bars[s]);
    }
  };

  if (tid == 0)
    for (int j = 0; j < NSTAGE - 1 && j < n_it; ++j) issue(j);

  // Register queues of (p, q) pairs indexed by plane mod 9 (compile-time
  // after unrolling): centre value, x- and y-derivative.
  float2 cq[9], dxq[9], dyq[9];
  float2 e_acc = make_float2(0.f, 0.f);
  int abort_it = -1;
  float4 *ring_ab = reinterpret_cast<float4 *>(smem + Lay::OFF_RA);
  float *ring_czz = reinterpret_cast<float *>(smem + Lay::OFF_RZ);
  constexpr int RING = Lay::RING;
  int rw = 0;  // 5-slot ring: the slot of this iteration (it % 5)
  // stage and parity of this iteration when the ring depth does not divide
  // the 9-plane body (compile-time otherwise)
  constexpr bool kStaticStage = 9 % NSTAGE == 0;
  int stg = 0;
  uint32_t sph = 0;

  // inactive threads of edge tiles may sit past the array: no profile read
  const float gxy = (SPONGE && active)
                        ? prm.sponge[gx] * prm.sponge[prm.sponge_oy + gy]
                        : 1.0f;
  float gzv = SPONGE ? prm.sponge[prm.sponge_oz + zb] : 1.0f;  // next output plane
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
  // next plane where this column records or injects something
  int ev = (src_col && prm.src_z >= zb) ? min(rnext < 0 ? 1 << 30 : rnext, prm.src_z)
                                        : (rnext < 0 ? 1 << 30 : rnext);
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
        // stage it % NSTAGE; with NSTAGE dividing 9 its use count is
        // it / NSTAGE = (9 / NSTAGE) * (it0 / 9) + u / NSTAGE
        const int sidx = kStaticStage ? u % NSTAGE : stg;
        const uint32_t spar =
            kStaticStage
                ? (((9 / NSTAGE) & 1 ? mpar : 0u) ^ static_cast<uint32_t>((u / NSTAGE) & 1))
                : sph;
        unsigned char *st = smem + sidx * Lay::STAGE_BYTES;
        const bool ok = mbar_wait_bounded(&bars[sidx], spar, kWaitLimitNs);
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
          xx = d2s<ISO, CHAIN>(w2x, c, xm1, xp1, xm2, xp2, xm3, xp3, xm4, xp4);
          yy = d2s<ISO, CHAIN>(w2y, c, ym1, yp1, ym2, yp2, ym3, yp3, ym4, yp4);
          cq[u] = c;
          dxq[u] = d1s<ISO, CHAIN>(w1x, xm1, xp1, xm2, xp2, xm3, xp3, xm4, xp4);
          dyq[u] = d1s<ISO, CHAIN>(w1y, ym1, yp1, ym2, yp2, ym3, yp3, ym4, yp4);
          dyb[od] = dyq[u];
        }
        // y-derivatives of the 4 + 4 halo columns (needed by d2/dxdy)
        if (tid < 8 * TY) {
          const int hc = tid & 7, hy = tid >> 3;
          const int hx = hc < 4 ? hc : TX + hc;
          const int o = (hy + kHalo) * HX + hx;
          dyb[hy * HX + hx] =
              d1s<ISO, CHAIN>(w1y, h[o - HX], h[o + HX], h[o - 2 * HX], h[o + 2 * HX],
                 h[o - 3 * HX], h[o + 3 * HX], h[o - 4 * HX], h[o + 4 * HX]);
        }
        if (__syncthreads_or(!ok)) {
          abort_it = it;
          goto done;
        }
        // The stage read in iteration it-1 is free: refill it.
        if (tid == 0 && it + NSTAGE - 1 < n_it) issue(it + NSTAGE - 1);

        // ---- in-plane part of H1 (A) and of the Laplacian (B) at plane k;
        // they wait in ring slot u for 4 planes
        if (it >= kHalo && it < n_it - kHalo) {
          const float2 xy = d1s<ISO, CHAIN>(w1x, dyb[od - 1], dyb[od + 1], dyb[od - 2], dyb[od + 2],
                               dyb[od - 3], dyb[od + 3], dyb[od - 4], dyb[od + 4]);
          const float4 lc = load_lead<CF>(st + Lay::OFF_L, ot);  // cxx, cyy, cxy, czz
          const float2 av = fma2(bc(lc.z), xy, fma2(bc(lc.y), yy, mul2(bc(lc.x), xx)));
          const float2 bv = add2(xx, yy);
          const int sw = RING == 9 ? u : rw;
          ring_ab[sw * NT + ot] = make_float4(av.x, av.y, bv.x, bv.y);
          ring_czz[sw * NT + ot] = lc.w;
        }

        // ---- output plane z = k - 4
        if (it >= 2 * kHalo) {
          // ring slots of planes z-4 .. z+4 (u is a compile-time constant)
          const int m4 = (u + 1) % 9, m3 = (u + 2) % 9, m2 = (u + 3) % 9,
                    m1 = (u + 4) % 9, c = (u + 5) % 9, p1 = (u + 6) % 9,
                    p2 = (u + 7) % 9, p3 = (u + 8) % 9, p4 = u;
          // slot of plane z = k - 4, written four iterations ago
          const int sr = RING == 9 ? c : (rw == 4 ? 0 : rw + 1);
          const float4 ab = ring_ab[sr * NT + ot];  // A, B of plane z
          const float czz = ring_czz[sr * NT + ot];
          const float2 zz = d2s<ISO, CHAIN>(w2z, cq[c], cq[m1], cq[p1], cq[m2], cq[p2], cq[m3],
                               cq[p3], cq[m4], cq[p4]);
          const float2 xz = d1s<ISO, CHAIN>(w1z, dxq[m1], dxq[p1], dxq[m2], dxq[p2],
                               dxq[m3], dxq[p3], dxq[m4], dxq[p4]);
          const float2 yz = d1s<ISO, CHAIN>(w1z, dyq[m1], dyq[p1], dyq[m2], dyq[p2],
                               dyq[m3], dyq[p3], dyq[m4], dyq[p4]);
          // FP16 form: the velocity bases of this thread's row (a broadcast
          // read: one row per warp)
          const float4 vb = Lay::VB ? reinterpret_cast<const float4 *>(st + Lay::OFF_VB)[ty]
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
          const OutMedium md = load_out<CF>(st + Lay::OFF_O1, st + Lay::OFF_O2, ot, vb);
          // H1 = sum c * d2 over the six second derivatives; the Laplacian
          // (H1 + H2) = xx + yy + zz
          float2 h1 =
              fma2(bc(md.cyz), yz, fma2(bc(md.cxz), xz, fma2(bc(czz), zz, make_float2(ab.x, ab.y))));
          if (CF == CF_F16) h1 = mul2(h1, bc(kChUnscale<CF>));
          const float2 h2 = fma2(bc(-1.0f), h1, add2(make_float2(ab.z, ab.w), zz));
          const float rhsp = fmaf(md.v2sz, h1.x - h1.y, fmaf(md.v2pz, h1.y, md.v2px * h2.x));
          const float rhsq = fmaf(-md.v2sz, h2.x - h2.y, fmaf(md.v2pz, h1.y, md.v2pn * h2.x));
          const float2 rhs = make_float2(rhsp, rhsq);
          const float2 pv = reinterpret_cast<const float2 *>(st + Lay::OFF_OWN)[ot];
          const float2 cc = add2(cq[c], cq[c]);  // 2 * current
          float2 nv;
          if (SPONGE) {
            const float g = gxy * gzv;
            nv = mul2(fma2(rhs, bc(ISO ? cw.dt2_iso : cw.dt2), fma2(bc(-g), pv, cc)), bc(g));
          } else {
            nv = fma2(rhs, bc(ISO ? cw.dt2_iso : cw.dt2), fma2(bc(-1.0f), pv, cc));
          }
          const int z = zb + it - 2 * kHalo;
          if (SPONGE && z + 1 < ze) gzv = prm.sponge[prm.sponge_oz + z + 1];
          if (active) {
            if (cw.energy) e_acc = fma2(nv, nv, e_acc);
            if (z == ev) {  // a receiver and/or the source sits at this point
              const int step = *prm.d_step + prm.step_offset;
              while (z == rnext) {
                if (step >= 0 && step < prm.trace_cap)
                  prm.traces[static_cast<long long>(step) * prm.nrec + prm.rec_r[rk]] = nv.x;
                ++rk;
                rnext = rk < rend ? prm.rec_z[rk] : -1;
              }
              if (src_col && z == prm.src_z) {
                const float sv =
                    step + 1 < prm.src_count ? prm.src_table[step + 1] : 0.0f;
                prm.src_pre[0] = nv.x;
                prm.src_pre[1] = nv.y;
                nv.x += sv;
                nv.y += sv;
              }
              const int nr = rnext < 0 ? 1 << 30 : rnext;
              ev = (src_col && prm.src_z > z) ? min(nr, prm.src_z) : nr;
            }
            *out = nv;
          }
          out += prm.plane;
        }
        if (RING != 9) rw = rw == 4 ? 0 : rw + 1;
        if (!kStaticStage && ++stg == NSTAGE) {
          stg = 0;
          sph ^= 1u;
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
    return false;
  }
  if (cw.energy) {
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
      if (step >= 0 && step < cw.energy_cap) atomicAdd(&cw.energy[step], tot);
    }
  }
  // every copy of this column has landed and been read: release the
  // barriers so the CTA can initialise them again for its next column
  __syncthreads();
  if (tid == 0)
    for (int s = 0; s < NSTAGE; ++s) mbar_inval(&bars[s]);
  return true;
}

// CTAs per SM the register allocation must allow: two of 256 threads, one
// of 512.
template <int NT>
constexpr int kMinBlocks = NT <= 256 ? 2 : 1;

// No static shared memory in these kernels: the dynamic window starts at
// the CTA's shared base, so the 1024-byte alignment holds and every access
// is a shared-space access.  TMA destinations must be 128-byte aligned; the
// kernels refuse to run otherwise (CTA-uniform, before any copy is issued).

// One pass over a box: CTA (bx, by, bz) sweeps tile (bx, by), z-chunk bz.
template <int TX, int TY, int CF, bool SPONGE, bool ISO, int NS>
__global__ void __launch_bounds__(TX *TY, kMinBlocks<TX * TY>)
    fast_kernel(const __grid_constant__ CUtensorMap tm_cur,
                const __grid_constant__ CUtensorMap tm_prev,
                const __grid_constant__ CUtensorMap tm_l,
                const __grid_constant__ CUtensorMap tm_o1,
                const __grid_constant__ CUtensorMap tm_o2,
                const __grid_constant__ CUtensorMap tm_vb,
                const __grid_constant__ StepParams prm) {
  extern __shared__ __align__(1024) unsigned char smem[];
  if (smem_u32(smem) & 127u) {
    if (threadIdx.x == 0) atomicOr(prm.err, kErrAlign);
    return;
  }
  const int x0 = prm.tile_x0 + static_cast<int>(blockIdx.x) * TX;
  const int y0 = prm.tile_y0 + static_cast<int>(blockIdx.y) * TY;
  const int zb = prm.z0 + static_cast<int>(blockIdx.z) * prm.zchunk;
  const int ze = min(zb + prm.zchunk, prm.z1);
  sweep_column<TX, TY, CF, SPONGE, ISO, NS>(&tm_cur, &tm_prev, &tm_l, &tm_o1, &tm_o2, &tm_vb,
                                            prm, prm, x0, y0, zb, ze, smem);
}

// One step of a batch of shots: persistent CTAs stride over the work items
// (shot by shot: x tile fastest, then y tile, then z-chunk).  The shot of an
// item is found from the per-shot prefix counts, so every index here is
// CTA-uniform.
template <int TX, int TY, int CF, bool SPONGE, bool ISO>
__global__ void __launch_bounds__(TX *TY, kMinBlocks<TX * TY>)
    batch_kernel(const __grid_constant__ BatchLaunch bl) {
  extern __shared__ __align__(1024) unsigned char smem[];
  if (smem_u32(smem) & 127u) {
    if (threadIdx.x == 0) atomicOr(bl.err, kErrAlign);
    return;
  }
  for (int slot = blockIdx.x; slot < bl.n_items; slot += gridDim.x) {
    const int item = bl.order ? bl.order[slot] : slot;
    int s = 0;
    while (s + 1 < bl.nshots && bl.item_prefix[s + 1] <= item) ++s;
    const StepParams &prm = bl.shot[s];
    int local = item - bl.item_prefix[s];
    const int ix = local % bl.tiles_x[s];
    local /= bl.tiles_x[s];
    const int iy = local % bl.tiles_y[s];
    const int iz = local / bl.tiles_y[s];
    const int x0 = prm.tile_x0 + ix * TX, y0 = prm.tile_y0 + iy * TY;
    const int zb = prm.z0 + iz * prm.zchunk;
    const int ze = min(zb + prm.zchunk, prm.z1);
    const CUtensorMap *m = bl.maps + 4 * s;
    // weights, dt2 and energy (none) are the same in every shot: read them
    // from shot 0 at fixed offsets
    if (!sweep_column<TX, TY, CF, SPONGE, ISO, 3>(m + bl.cur_buf, m + 2 + (1 - bl.cur_buf),
                                             &bl.tm_l, &bl.tm_o1, &bl.tm_o2, &bl.tm_vb, prm,
                                             bl.shot[0],
                                             x0, y0, zb, ze, smem))
      return;
  }
}

// Compiled tile shapes: TX = 32 (one warp per tile row) and TY = 8 or 16
// rows (256 or 512 threads); a 3-stage TMA ring, or 4 stages for large
// FP32 boxes.
constexpr int kTX = 32;

template <int TY, int CF, bool SPONGE, bool ISO, int NS>
cudaError_t launch_fast_t(Sim *sim, const StepParams &prm, int cur_buf, int prev_buf) {
  using Lay = FastLayout<kTX, TY, CF, NS>;
  auto kern = fast_kernel<kTX, TY, CF, SPONGE, ISO, NS>;
  const int nx = prm.x1 - prm.tile_x0, ny = prm.y1 - prm.tile_y0;
  const int nz = prm.z1 - prm.z0;
  dim3 grid((nx + kTX - 1) / kTX, (ny + TY - 1) / TY, (nz + prm.zchunk - 1) / prm.zchunk);
  kern<<<grid, kTX * TY, Lay::SMEM_BYTES, sim->stream>>>(
      sim->tm_halo[cur_buf], sim->tm_own[prev_buf], sim->tm_c[0], sim->tm_c[1], sim->tm_c[2],
      sim->tm_c[3], prm);  // tm_c: L, O1, O2, row bases
  return cudaGetLastError();
}

template <int TY, int CF, int NS>
cudaError_t set_smem_attr_ns() {
  using Lay = FastLayout<kTX, TY, CF, NS>;
  cudaError_t e = cudaSuccess;
  const int b = Lay::SMEM_BYTES;
  const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, CF, false, false, NS>, attr, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, CF, false, true, NS>, attr, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, CF, true, false, NS>, attr, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fast_kernel<kTX, TY, CF, true, true, NS>, attr, b);
  return e;
}

template <int TY, int CF>
cudaError_t set_smem_attr_all() {
  cudaError_t e = set_smem_attr_ns<TY, CF, 3>();
  if constexpr (CF == CF_F32)
    if (e == cudaSuccess) e = set_smem_attr_ns<TY, CF, 4>();
  return e;
}

template <int TY, int CF, int NS>
cudaError_t launch_cf_ns(Sim *sim, const StepParams &prm, int cur, int prev) {
  const bool sp = prm.sponge != nullptr;
  const bool iso = sim->dx == sim->dy && sim->dy == sim->dz;
  if (sp)
    return iso ? launch_fast_t<TY, CF, true, true, NS>(sim, prm, cur, prev)
               : launch_fast_t<TY, CF, true, false, NS>(sim, prm, cur, prev);
  return iso ? launch_fast_t<TY, CF, false, true, NS>(sim, prm, cur, prev)
             : launch_fast_t<TY, CF, false, false, NS>(sim, prm, cur, prev);
}

template <int TY, int CF>
cudaError_t launch_cf(Sim *sim, const StepParams &prm, int cur, int prev) {
  if constexpr (CF == CF_F32)
    if (sim->deep_ring) return launch_cf_ns<TY, CF, 4>(sim, prm, cur, prev);
  return launch_cf_ns<TY, CF, 3>(sim, prm, cur, prev);
}

template <int TY>
cudaError_t launch_ty(Sim *sim, const StepParams &prm, int cur, int prev) {
  switch (sim->coef_form) {
    case CF_VV: return launch_cf<TY, CF_VV>(sim, prm, cur, prev);
    case CF_F16: return launch_cf<TY, CF_F16>(sim, prm, cur, prev);
    case CF_BF16: return launch_cf<TY, CF_BF16>(sim, prm, cur, prev);
    default: return launch_cf<TY, CF_F32>(sim, prm, cur, prev);
  }
}

template <int TY>
cudaError_t set_attrs(int form) {
  switch (form) {
    case CF_VV: return set_smem_attr_all<TY, CF_VV>();
    case CF_F16: return set_smem_attr_all<TY, CF_F16>();
    case CF_BF16: return set_smem_attr_all<TY, CF_BF16>();
    default: return set_smem_attr_all<TY, CF_F32>();
  }
}

// 32 x 8 tiles with two CTAs per SM measured fastest on GB300 (616^3 cube:
// 2.83 ms per step vs 3.09 ms for 32 x 16; 32 x 6 with three CTAs per SM
// was slower still: 2.93 ms FP32, 2.68 ms FP16 against 2.56 ms).
// DC_GB300_FAST_TY=16 selects 32 x 16.
int chosen_ty(int) {
  const char *e = std::getenv("DC_GB300_FAST_TY");
  const int v = e ? std::atoi(e) : 0;
  return v == 16 ? 16 : 8;
}

template <typename F>
auto by_ty(int ty, F &&f) {
  if (ty == 16) return f(std::integral_constant<int, 16>{});
  return f(std::integral_constant<int, 8>{});
}

}  // namespace

// z-chunk of a pass: a CTA sweeping zc output planes streams zc + 8 leading
// planes (the 8-plane warm-up of the z queues), and the CTAs run in waves of
// `fast_slots`, a partly filled last wave taking about as long as a full
// one.  So the pass costs ~ ceil(tiles * chunks / slots) * (zc + 8) plane
// sweeps; the chunk count (1..8, chunks of at least 32 planes) minimising it
// is taken, the smaller on ties.  Measured on cubes of 200^3 to 616^3 (FP32,
// 32 x 8 tiles, 304 slots) this choice is within 1.2 % of the fastest of
// 1..8 chunks everywhere; one chunk per column, wherever that left the last
// wave nearly empty, was up to 18 % slower (408^3: 0.969 vs 0.822 ms).
// DC_GB300_FAST_ZCHUNKS=<n> forces n chunks.
FastShape fast_shape(const Sim *sim, long long nx, long long ny, long long nz) {
  const int ty = sim->maps_ty ? sim->maps_ty : chosen_ty(sim->coef_form);
  if (nz < 1) return FastShape{kTX, ty, 1};
  const long long tiles = std::max(1ll, (nx + kTX - 1) / kTX) * std::max(1ll, (ny + ty - 1) / ty);
  const long long slots = sim->fast_slots > 0 ? sim->fast_slots : 2 * 152;
  long long best_zc = nz, best_cost = -1;
  for (long long c = 1; c <= 8; ++c) {
    const long long zc = (nz + c - 1) / c;
    if (c > 1 && zc < 32) break;
    const long long chunks = (nz + zc - 1) / zc;
    const long long cost = (tiles * chunks + slots - 1) / slots * (zc + 8);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best_zc = zc;
    }
  }
  if (const char *e = std::getenv("DC_GB300_FAST_ZCHUNKS")) {
    const long long c = std::max(1, std::atoi(e));
    best_zc = (nz + c - 1) / c;
  }
  return FastShape{kTX, ty, static_cast<int>(best_zc)};
}

int fast_default_ty(int form) { return chosen_ty(form); }

bool fast_encode_pair_maps(const float2 *buf, long long sx, long long sy, long long sz,
                           long long pitch, int ty, CUtensorMap *halo, CUtensorMap *own,
                           std::string *err) {
  const uint64_t dims3[3] = {static_cast<uint64_t>(sx), static_cast<uint64_t>(sy),
                             static_cast<uint64_t>(sz)};
  // (p, q) pair buffers: 8-byte elements
  const uint64_t str8[2] = {static_cast<uint64_t>(pitch) * 8,
                            static_cast<uint64_t>(pitch * sy) * 8};
  const uint32_t box_halo[3] = {kTX + 8, static_cast<uint32_t>(ty) + 8, 1};
  const uint32_t box_tile[3] = {kTX, static_cast<uint32_t>(ty), 1};
  const auto U64 = CU_TENSOR_MAP_DATA_TYPE_UINT64;
  return encode_tiled(halo, buf, 3, dims3, str8, box_halo, err, U64) &&
         encode_tiled(own, buf, 3, dims3, str8, box_tile, err, U64);
}

bool fast_encode_medium_maps(int form, const float *coef, const void *coef16, const float *vv,
                             const float4 *vbase, long long sx, long long sy, long long sz,
                             long long pitch, long long count, int ty, CUtensorMap out[4],
                             std::string *err) {
  const uint64_t X = sx, Y = sy, Z = sz, P = pitch, PL = pitch * sy;
  const uint64_t dims3[3] = {X, Y, Z};
  const uint64_t str8[2] = {P * 8, PL * 8};
  const uint64_t str4[2] = {P * 4, PL * 4};
  const uint32_t box_tile[3] = {kTX, static_cast<uint32_t>(ty), 1};
  // 16-byte coefficient groups: two 8-byte elements per point, so a tile
  // row is one 512-byte box row (a box whose innermost extent is a single
  // 16-byte group makes the copy engine walk 32 x TY rows of 16 bytes)
  const uint64_t dims16[3] = {2 * X, Y, Z};
  const uint64_t str16[2] = {P * 16, PL * 16};
  const uint32_t box16[3] = {2 * kTX, static_cast<uint32_t>(ty), 1};
  const auto U64 = CU_TENSOR_MAP_DATA_TYPE_UINT64, U32 = CU_TENSOR_MAP_DATA_TYPE_UINT32;
  const long long cnt = count;
  // out[0] = L (cxx, cyy, cxy, czz), out[1] = O1, out[2] = O2, out[3] = the
  // FP16 form's row bases
  bool ok = false;
  switch (form) {
    case CF_F32: {
      const char *c = reinterpret_cast<const char *>(coef);
      ok = encode_tiled(&out[0], c, 3, dims16, str16, box16, err, U64) &&
           encode_tiled(&out[1], c + cnt * 16, 3, dims16, str16, box16, err, U64) &&
           encode_tiled(&out[2], c + cnt * 32, 3, dims3, str8, box_tile, err, U64);
      break;
    }
    case CF_VV:
      ok = encode_tiled(&out[1], vv, 3, dims3, str8, box_tile, err, U64);
      out[0] = out[2] = out[1];  // unused
      break;
    default: {  // CF_F16, CF_BF16: 8-byte L, 8-byte O1, 4-byte O2
      const char *h = static_cast<const char *>(coef16);
      ok = encode_tiled(&out[0], h, 3, dims3, str8, box_tile, err, U64) &&
           encode_tiled(&out[1], h + cnt * 8, 3, dims3, str8, box_tile, err, U64) &&
           encode_tiled(&out[2], h + cnt * 16, 3, dims3, str4, box_tile, err, U32);
    }
  }
  if (!ok) return false;
  if (form != CF_F16) {
    out[3] = out[2];  // unused
    return true;
  }
  // row bases: [sz][sy] float4 as a 2-D tensor of 8-byte elements, x = 2 y
  const uint64_t dims_vb[2] = {2 * Y, Z};
  const uint64_t str_vb[1] = {Y * 16};
  const uint32_t box_vb[2] = {2 * static_cast<uint32_t>(ty), 1};
  return encode_tiled(&out[3], vbase, 2, dims_vb, str_vb, box_vb, err, U64);
}

// The 4-stage ring pays off on large FP32 boxes, where the whole GPU
// streams from DRAM over long sweeps (616^3: 2.690 ms per step against
// 2.739 ms), and costs on small ones (the run-time ring indices add 10 %
// instructions; 304^3: 411 against 371 us).  DC_GB300_FAST_STAGES=3|4
// overrides the choice.
constexpr long long kDeepRingPoints = 96ll << 20;

bool deep_ring_for(const Sim *sim) {
  if (sim->coef_form != CF_F32) return false;
  const char *e = std::getenv("DC_GB300_FAST_STAGES");
  if (e && std::atoi(e) == 3) return false;
  if (e && std::atoi(e) == 4) return true;
  return (sim->sx - 8) * (sim->sy - 8) * (sim->sz - 8) >= kDeepRingPoints;
}

namespace {

// CTAs of the fast sweep one SM holds at once (the sponge, equal-spacing
// instance; the others differ by a few registers, well inside the limit).
template <int TY, int CF, int NS>
int fast_occupancy() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &n, fast_kernel<kTX, TY, CF, true, true, NS>, kTX * TY,
          FastLayout<kTX, TY, CF, NS>::SMEM_BYTES) != cudaSuccess)
    return 0;
  return n;
}

template <int TY, int CF>
int fast_occupancy_cf(bool deep) {
  if constexpr (CF == CF_F32)
    if (deep) return fast_occupancy<TY, CF, 4>();
  return fast_occupancy<TY, CF, 3>();
}

template <int TY>
int fast_occupancy_ty(int form, bool deep) {
  switch (form) {
    case CF_VV: return fast_occupancy_cf<TY, CF_VV>(deep);
    case CF_F16: return fast_occupancy_cf<TY, CF_F16>(deep);
    case CF_BF16: return fast_occupancy_cf<TY, CF_BF16>(deep);
    default: return fast_occupancy_cf<TY, CF_F32>(deep);
  }
}

}  // namespace

bool fast_encode_maps(Sim *sim, std::string *err) {
  sim->deep_ring = deep_ring_for(sim);
  // dynamic shared memory above 48 KB must be enabled per kernel and device
  // (done here, before any stream capture)
  const int kTY = chosen_ty(sim->coef_form);
  cudaError_t ae = by_ty(kTY, [&](auto t) { return set_attrs<decltype(t)::value>(sim->coef_form); });
  if (ae != cudaSuccess) {
    *err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(ae);
    return false;
  }
  for (int b = 0; b < 2; ++b)
    if (!fast_encode_pair_maps(sim->pq[b], sim->sx, sim->sy, sim->sz, sim->pitch, kTY,
                               &sim->tm_halo[b], &sim->tm_own[b], err))
      return false;
  if (!fast_encode_medium_maps(sim->coef_form, sim->coef, sim->coef16, sim->vv, sim->vbase,
                               sim->sx, sim->sy, sim->sz, sim->pitch, sim->count, kTY, sim->tm_c,
                               err))
    return false;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sim->device) != cudaSuccess)
    sms = 0;
  const int per_sm =
      by_ty(kTY, [&](auto t) { return fast_occupancy_ty<decltype(t)::value>(sim->coef_form, sim->deep_ring); });
  sim->fast_slots = sms > 0 && per_sm > 0 ? sms * per_sm : 0;
  cudaGetLastError();  // a failed occupancy query leaves the fallback slot count
  sim->maps_tx = kTX;
  sim->maps_ty = kTY;
  return true;
}

namespace {

// Batch kernel variants: every coefficient form and spacing with the
// sponge; without it (all shots' profiles are 1, e.g. learned layers) for
// equal spacing and the FP32 / FP16 / BF16 forms.
template <int CF>
constexpr bool kNoSpongeForm = CF == CF_F32 || CF == CF_F16 || CF == CF_BF16;

template <int TY, int CF, bool SPONGE, bool ISO>
cudaError_t batch_attr() {
  return cudaFuncSetAttribute(batch_kernel<kTX, TY, CF, SPONGE, ISO>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              FastLayout<kTX, TY, CF>::SMEM_BYTES);
}

template <int TY, int CF>
cudaError_t batch_attr_cf() {
  cudaError_t e = batch_attr<TY, CF, true, false>();
  if (e == cudaSuccess) e = batch_attr<TY, CF, true, true>();
  if constexpr (kNoSpongeForm<CF>)
    if (e == cudaSuccess) e = batch_attr<TY, CF, false, true>();
  return e;
}

template <int TY>
cudaError_t batch_attr_ty(int form) {
  switch (form) {
    case CF_F16: return batch_attr_cf<TY, CF_F16>();
    case CF_BF16: return batch_attr_cf<TY, CF_BF16>();
    case CF_VV: return batch_attr_cf<TY, CF_VV>();
    default: return batch_attr_cf<TY, CF_F32>();
  }
}

template <int TY, int CF, bool SPONGE, bool ISO>
int batch_occ() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<kTX, TY, CF, SPONGE, ISO>,
                                                    kTX * TY,
                                                    FastLayout<kTX, TY, CF>::SMEM_BYTES) !=
      cudaSuccess)
    return 0;
  return n;
}

template <int TY, int CF>
int batch_occ_cf(bool iso, bool sponge) {
  if constexpr (kNoSpongeForm<CF>)
    if (iso && !sponge) return batch_occ<TY, CF, false, true>();
  return iso ? batch_occ<TY, CF, true, true>() : batch_occ<TY, CF, true, false>();
}

template <int TY>
int batch_occ_ty(int form, bool iso, bool sponge) {
  switch (form) {
    case CF_F16: return batch_occ_cf<TY, CF_F16>(iso, sponge);
    case CF_BF16: return batch_occ_cf<TY, CF_BF16>(iso, sponge);
    case CF_VV: return batch_occ_cf<TY, CF_VV>(iso, sponge);
    default: return batch_occ_cf<TY, CF_F32>(iso, sponge);
  }
}

template <int TY, int CF>
cudaError_t launch_batch_cf(cudaStream_t st, const BatchLaunch &bl, bool iso, bool sponge,
                            int blocks) {
  const int smem = FastLayout<kTX, TY, CF>::SMEM_BYTES;
  bool done = false;
  if constexpr (kNoSpongeForm<CF>)
    if (iso && !sponge) {
      batch_kernel<kTX, TY, CF, false, true><<<blocks, kTX * TY, smem, st>>>(bl);
      done = true;
    }
  if (!done) {
    if (iso)
      batch_kernel<kTX, TY, CF, true, true><<<blocks, kTX * TY, smem, st>>>(bl);
    else
      batch_kernel<kTX, TY, CF, true, false><<<blocks, kTX * TY, smem, st>>>(bl);
  }
  return cudaGetLastError();
}

template <int TY>
cudaError_t launch_batch_ty(cudaStream_t st, const BatchLaunch &bl, int form, bool iso,
                            bool sponge, int blocks) {
  switch (form) {
    case CF_F16: return launch_batch_cf<TY, CF_F16>(st, bl, iso, sponge, blocks);
    case CF_BF16: return launch_batch_cf<TY, CF_BF16>(st, bl, iso, sponge, blocks);
    case CF_VV: return launch_batch_cf<TY, CF_VV>(st, bl, iso, sponge, blocks);
    default: return launch_batch_cf<TY, CF_F32>(st, bl, iso, sponge, blocks);
  }
}

}  // namespace

bool fast_tile_rows_valid(int ty, int) { return ty == 8 || ty == 16; }

cudaError_t batch_prepare(int ty, int form) {
  return by_ty(ty, [&](auto t) { return batch_attr_ty<decltype(t)::value>(form); });
}

int batch_blocks_per_sm(int ty, int form, bool iso, bool sponge) {
  return by_ty(ty, [&](auto t) { return batch_occ_ty<decltype(t)::value>(form, iso, sponge); });
}

cudaError_t launch_batch(cudaStream_t st, const BatchLaunch &bl, int ty, int form, bool iso,
                         bool sponge, int blocks) {
  return by_ty(ty, [&](auto t) {
    return launch_batch_ty<decltype(t)::value>(st, bl, form, iso, sponge, blocks);
  });
}

cudaError_t launch_fast(Sim *sim, const StepParams &prm, int cur_buf, int prev_buf) {
  return by_ty(sim->maps_ty, [&](auto t) {
    return launch_ty<decltype(t)::value>(sim, prm, cur_buf, prev_buf);
  });
}

}  // namespace dcg
