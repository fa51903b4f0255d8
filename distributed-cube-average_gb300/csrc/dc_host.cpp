// dc_host.cpp -- host-side set-up entry points of the reference ABI
// (default medium, random velocity boundary, source wavelet) and the
// library's own parameterised source and sponge profile.
//
// Compiled with -ffp-contract=off: these functions must round exactly as
// the reference's host C does (an FMA would change the last bit).
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "dc_gb300.h"

namespace {

[[noreturn]] void oom(const char *what) {
  std::fprintf(stderr, "[dc_gb300] OOM: could not allocate memory for %s\n", what);
  std::exit(1);
}

float *alloc(long long n, const char *what) {
  float *p = static_cast<float *>(std::malloc(sizeof(float) * (n > 0 ? n : 1)));
  if (!p) oom(what);
  return p;
}

// Distance into the absorbing shell along one axis (src/boundary.c:57-89).
int shell_dist(int g, int first_in, int bord_len, int n) {
  if (g > bord_len + n) return g - bord_len - n;
  if (g < first_in) return first_in - g;
  return 0;
}

// Ricker-type wavelet of src/calculate_source.c:10-17 with the cut-off
// frequency as a parameter; the constants are pi^3, 2*sqrt(pi), 3*sqrt(pi)
// (src/calculate_source.c:6-8), and tf, fc, expo are stored in float.
float source_sample(float dt, int it, double fcut) {
  const double pi_cube = 31.00627668029982017537;
  const double two_sqrt_pi = 3.54490770181103205458;
  const double three_sqrt_pi = 5.31736155271654808184;
  const float tf = two_sqrt_pi / fcut;
  const float fc = fcut / three_sqrt_pi;
  const float fct = fc * (static_cast<float>(it) * dt - tf);
  const float expo = pi_cube * fct * fct;
  return (1.0f - 2.0f * expo) * expf(-expo);
}

}  // namespace

extern "C" dc_anisotropy_t dc_compute_anisotropy_vars(int sx, int sy, int sz) {
  // src/precomp.c:110-171: vpz 3000, eps 0.24, delta 0.1, phi 1 rad,
  // theta atanf(1); vsv by the SIGMA = 0.75 rule (division in double).
  const long long n = static_cast<long long>(sx) * sy * sz;
  dc_anisotropy_t a;
  a.vpz = alloc(n, "vpz");
  a.vsv = alloc(n, "vsv");
  a.epsilon = alloc(n, "epsilon");
  a.delta = alloc(n, "delta");
  a.phi = alloc(n, "phi");
  a.theta = alloc(n, "theta");
  const float theta = atanf(1.0f);
  for (long long i = 0; i < n; ++i) {
    a.vpz[i] = 3000.0;
    a.epsilon[i] = 0.24;
    a.delta[i] = 0.1;
    a.phi[i] = 1.0;
    a.theta[i] = theta;
    a.vsv[i] = a.vpz[i] * sqrtf(fabsf(a.epsilon[i] - a.delta[i]) / 0.75);
  }
  return a;
}

extern "C" void dc_free_anisotropy_vars(dc_anisotropy_t *a) {
  if (!a) return;
  std::free(a->theta);
  std::free(a->phi);
  std::free(a->vsv);
  std::free(a->vpz);
  std::free(a->epsilon);
  std::free(a->delta);
  a->theta = a->phi = a->vsv = a->vpz = a->epsilon = a->delta = nullptr;
}

extern "C" void dc_free_precomp_vars(dc_precomp_vars *v) {
  if (!v) return;
  float **f[10] = {&v->ch1dxx, &v->ch1dyy, &v->ch1dzz, &v->ch1dxy, &v->ch1dyz,
                   &v->ch1dxz, &v->v2px,   &v->v2pz,   &v->v2sz,   &v->v2pn};
  for (float **p : f) {
    std::free(*p);
    *p = nullptr;
  }
}

extern "C" void randomVelocityBoundaryPartition(int local_sx, int local_sy, int local_sz,
                                                int global_sx, int global_sy, int global_sz,
                                                int start_x, int start_y, int start_z, int nx,
                                                int ny, int nz, int bord, int absorb,
                                                float *vpz, float *vsv, unsigned int *seed) {
  // src/boundary.c:7-104.  Every shell cell of the global cube draws one
  // rand_r value in z,y,x order -- also the ones outside this partition --
  // so that all partitions agree on the sequence.  The ramp goes from the
  // interior value to a random fraction of the maximum over `absorb` cells;
  // cells outside the shell and the interior are zeroed.
  const int bord_len = bord + absorb - 1;
  const int first_in = bord_len + 1;
  const float frac = 1.0f / static_cast<float>(absorb);
  const float max_p = 3000.0f;
  const float max_s = max_p * sqrtf(fabsf(0.24f - 0.1f) / 0.75f);
  const int end_x = start_x + local_sx, end_y = start_y + local_sy, end_z = start_z + local_sz;
  for (int gz = 0; gz < global_sz; ++gz)
    for (int gy = 0; gy < global_sy; ++gy)
      for (int gx = 0; gx < global_sx; ++gx) {
        const bool inside = gz >= first_in && gz <= bord_len + nz && gy >= first_in &&
                            gy <= bord_len + ny && gx >= first_in && gx <= bord_len + nx;
        if (inside) continue;
        const bool in_shell = gz >= bord && gz <= 2 * bord_len + nz && gy >= bord &&
                              gy <= 2 * bord_len + ny && gx >= bord && gx <= 2 * bord_len + nx;
        const bool mine = gx >= start_x && gx < end_x && gy >= start_y && gy < end_y &&
                          gz >= start_z && gz < end_z;
        const long long i = static_cast<long long>(gx - start_x) +
                            static_cast<long long>(gy - start_y) * local_sx +
                            static_cast<long long>(gz - start_z) * local_sx * local_sy;
        if (in_shell) {
          const float r = static_cast<float>(rand_r(seed)) / static_cast<float>(RAND_MAX);
          if (!mine) continue;
          int d = shell_dist(gy, first_in, bord_len, ny);
          const int dz = shell_dist(gz, first_in, bord_len, nz);
          const int dx = shell_dist(gx, first_in, bord_len, nx);
          d = d > dz ? d : dz;
          d = d > dx ? d : dx;
          const float w = static_cast<float>(d) * frac;
          vpz[i] = max_p * (1.0f - w) + max_p * r * w;
          vsv[i] = max_s * (1.0f - w) + max_s * r * w;
        } else if (mine) {
          vpz[i] = 0.0f;
          vsv[i] = 0.0f;
        }
      }
}

// Float constants of the reference medium, computed with the reference's
// own expressions (src/boundary.c:27-31, src/precomp.c:156-169) so that the
// GPU generator starts from identical values.
extern "C" void dc_gb300_reference_medium_constants(int absorb, float out[6]) {
  out[0] = 1.0f / static_cast<float>(absorb);           // frac
  out[1] = 3000.0f;                                     // max_p
  out[2] = out[1] * sqrtf(fabsf(0.24f - 0.1f) / 0.75f);  // max_s (float division)
  const float vpz = 3000.0;
  const float eps = 0.24, delta = 0.1;
  out[3] = vpz * sqrtf(fabsf(eps - delta) / 0.75);      // default vsv (double division)
  out[4] = atanf(1.0);                                  // theta
  out[5] = 1.0;                                         // phi
}

extern "C" float dc_calculate_source(float dt, int it) {
  return source_sample(dt, it, 40.0);  // FCUT = 40 (src/calculate_source.c:5)
}

extern "C" float dc_gb300_source(float dt, int it, double fcut) {
  return source_sample(dt, it, fcut);
}

extern "C" void dc_gb300_sponge_profile(long s, long a, double kappa, float *g) {
  // Cells into the absorbing shell: d = 1 at the cell next to the physical
  // interior up to d = a at the halo; g = exp(-(kappa*d/a)^2); g = 1 in the
  // interior and in the 4-cell halo.
  for (long i = 0; i < s; ++i) {
    long d = 0;
    if (a > 0 && i >= 4 && i < s - 4) {
      const long lo = (4 + a) - i, hi = i - (s - 5 - a);
      d = lo > d ? lo : d;
      d = hi > d ? hi : d;
    }
    const double t = a > 0 ? kappa * static_cast<double>(d) / static_cast<double>(a) : 0.0;
    g[i] = static_cast<float>(std::exp(-t * t));
  }
}
