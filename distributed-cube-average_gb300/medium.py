"""Seeded media and workload geometry for the propagator.

* ``layered_spec`` draws the random parameters of the layered model (numpy
  PCG64, seed stated by the caller) into the ``dc_gb300_layered_spec`` that
  the GPU generator evaluates (dc_gb300_generate_layered).
* ``layered_fields`` evaluates the same model on the host (numpy, double)
  for small grids and crops, so tests can check the GPU generator.
* ``homogeneous`` builds constant media such as the reference default.

The layered model: ``nlayers`` horizontal layers of equal thickness over the
model depth, P velocity per layer drawn U(vp_lo, vp_hi) and sorted to
increase with depth, times (1 + vp_noise * n(r)); epsilon per layer U(0,
0.3), delta per layer U(0, epsilon); theta and phi smooth fields whose
marginals are uniform on their ranges; vsv by the SIGMA rule of the
reference (vsv = vp * sqrt(|eps - delta| / 0.75), include/precomp.h:3 and
src/precomp.c:165-167).  n(r) and the angle fields are Gaussian random
fields with a Gaussian covariance, generated by random Fourier features:
f(r) = sqrt(2/m) * sum_j cos(k_j . r + ph_j) with k_j ~ N(0, I / l^2) and
ph_j ~ U(0, 2 pi).  A white noise smoothed by a Gaussian filter of width
sigma cells has a Gaussian covariance of length l = sigma * sqrt(2), which
is what is drawn here.  The angle fields pass through the normal CDF so that
their marginals are uniform.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import LayeredSpec, MAX_FEATURES, MAX_LAYERS

SIGMA = 0.75  # include/precomp.h:3


def _rff(rng: np.random.Generator, m: int, sigma_cells: float) -> np.ndarray:
    ell = sigma_cells * math.sqrt(2.0)
    k = rng.normal(0.0, 1.0 / ell, size=(m, 3))
    ph = rng.uniform(0.0, 2.0 * math.pi, size=(m, 1))
    return np.concatenate([k, ph], axis=1).astype(np.float32)


def layered_spec(seed: int, model_sizes, nlayers: int = 12, vp_range=(1500.0, 4500.0),
                 vp_noise: float = 0.02, noise_sigma: float = 2.0, angle_sigma: float = 20.0,
                 theta_range=(-math.pi / 3, math.pi / 3), phi_range=(0.0, 2.0 * math.pi),
                 n_noise: int = 64, n_theta: int = 32, n_phi: int = 32,
                 origin=(0, 0, 0)) -> LayeredSpec:
    """Draws the layered model for a global cube of ``model_sizes`` (x, y, z,
    padded).  ``origin`` places the array evaluated by the generator inside
    that cube (crops)."""
    if not (1 <= nlayers <= MAX_LAYERS):
        raise ValueError("nlayers out of range")
    if max(n_noise, n_theta, n_phi) > MAX_FEATURES:
        raise ValueError("too many features")
    rng = np.random.Generator(np.random.PCG64(seed))
    vp = np.sort(rng.uniform(vp_range[0], vp_range[1], nlayers))
    eps = rng.uniform(0.0, 0.3, nlayers)
    delta = rng.uniform(0.0, 1.0, nlayers) * eps
    k_noise = _rff(rng, n_noise, noise_sigma)
    k_theta = _rff(rng, n_theta, angle_sigma)
    k_phi = _rff(rng, n_phi, angle_sigma)
    spec = LayeredSpec()
    spec.nlayers = nlayers
    depth = float(model_sizes[2])
    for l in range(nlayers):
        spec.layer_top[l] = np.float32(l * depth / nlayers)
        spec.vp[l] = vp[l]
        spec.epsilon[l] = eps[l]
        spec.delta[l] = delta[l]
    spec.vp_noise = vp_noise
    spec.theta_lo, spec.theta_hi = theta_range
    spec.phi_lo, spec.phi_hi = phi_range
    spec.sigma_ratio = SIGMA
    spec.n_noise, spec.n_theta, spec.n_phi = n_noise, n_theta, n_phi
    for dst, src in ((spec.k_noise, k_noise), (spec.k_theta, k_theta), (spec.k_phi, k_phi)):
        for j in range(src.shape[0]):
            for c in range(4):
                dst[j][c] = src[j, c]
    spec.ox, spec.oy, spec.oz = (int(v) for v in origin)
    return spec


def with_origin(spec: LayeredSpec, origin) -> LayeredSpec:
    """A copy of ``spec`` evaluated at another origin (a crop)."""
    import ctypes
    out = LayeredSpec()
    ctypes.memmove(ctypes.addressof(out), ctypes.addressof(spec), ctypes.sizeof(spec))
    out.ox, out.oy, out.oz = (int(v) for v in origin)
    return out


def _spec_arrays(spec: LayeredSpec):
    def feats(arr, m):
        return np.array([[arr[j][c] for c in range(4)] for j in range(m)], np.float32).astype(np.float64)
    return (feats(spec.k_noise, spec.n_noise), feats(spec.k_theta, spec.n_theta),
            feats(spec.k_phi, spec.n_phi))


def _field(feat: np.ndarray, gx, gy, gz) -> np.ndarray:
    m = feat.shape[0]
    if m == 0:
        return np.zeros(np.broadcast(gx, gy, gz).shape)
    s = np.zeros(np.broadcast(gx, gy, gz).shape)
    for j in range(m):
        s += np.cos(feat[j, 0] * gx + feat[j, 1] * gy + feat[j, 2] * gz + feat[j, 3])
    return s * math.sqrt(2.0 / m)


def layered_fields(spec: LayeredSpec, sizes) -> dict:
    """Host evaluation of the GPU generator (dc_aux.cu:layered_kernel) on an
    array of ``sizes`` (x, y, z) placed at the spec's origin.  Returns the
    anisotropy arrays (float32, shape (sz, sy, sx))."""
    from scipy.special import erfc
    sx, sy, sz = sizes
    gz, gy, gx = np.meshgrid(np.arange(sz, dtype=np.float64) + spec.oz,
                             np.arange(sy, dtype=np.float64) + spec.oy,
                             np.arange(sx, dtype=np.float64) + spec.ox, indexing="ij")
    kn, kt, kp = _spec_arrays(spec)
    fn = _field(kn, gx, gy, gz)
    ft = _field(kt, gx, gy, gz)
    fp = _field(kp, gx, gy, gz)
    ut = 0.5 * erfc(-ft * 0.70710678118654752440)
    up = 0.5 * erfc(-fp * 0.70710678118654752440)
    tops = np.array([spec.layer_top[l] for l in range(spec.nlayers)], np.float32).astype(np.float64)
    layer = np.clip(np.searchsorted(tops, gz[:, 0, 0], side="right") - 1, 0, spec.nlayers - 1)
    layer = np.broadcast_to(layer[:, None, None], gz.shape)
    vp_l = np.array([spec.vp[l] for l in range(spec.nlayers)], np.float32).astype(np.float64)
    eps_l = np.array([spec.epsilon[l] for l in range(spec.nlayers)], np.float32)
    del_l = np.array([spec.delta[l] for l in range(spec.nlayers)], np.float32)
    vp = (vp_l[layer] * (1.0 + float(np.float32(spec.vp_noise)) * fn)).astype(np.float32)
    t_lo, t_hi = float(np.float32(spec.theta_lo)), float(np.float32(spec.theta_hi))
    p_lo, p_hi = float(np.float32(spec.phi_lo)), float(np.float32(spec.phi_hi))
    theta = (t_lo + (t_hi - t_lo) * ut).astype(np.float32)
    phi = (p_lo + (p_hi - p_lo) * up).astype(np.float32)
    eps = eps_l[layer].astype(np.float32)
    delta = del_l[layer].astype(np.float32)
    ratio = np.float32(spec.sigma_ratio)
    vs = (vp * np.sqrt(np.abs(eps - delta) / ratio, dtype=np.float32)).astype(np.float32)
    return {"theta": theta, "phi": phi, "vsv": vs, "vpz": vp, "epsilon": eps, "delta": delta}


def homogeneous(sizes, vp=3000.0, epsilon=0.24, delta=0.10, theta=math.pi / 4, phi=math.pi / 6,
                vs=0.0) -> dict:
    """Constant medium (float32 arrays of shape (sz, sy, sx))."""
    sx, sy, sz = sizes
    shape = (sz, sy, sx)
    mk = lambda v: np.full(shape, np.float32(v), np.float32)  # noqa: E731
    return {"theta": mk(theta), "phi": mk(phi), "vsv": mk(vs), "vpz": mk(vp),
            "epsilon": mk(epsilon), "delta": mk(delta)}


@dataclass(frozen=True)
class Geometry:
    """Padded cube of the reference CLI: s = n + 2a + 8 per axis
    (src/main.c:94-99); the updated (compute) region is [4, s-4)."""
    n: tuple
    absorb: int

    @property
    def sizes(self):
        return tuple(int(v) + 2 * self.absorb + 8 for v in self.n)

    @property
    def shape(self):
        sx, sy, sz = self.sizes
        return (sz, sy, sx)

    def index(self, x, y, z) -> int:
        sx, sy, _ = self.sizes
        return int(x + y * sx + z * sx * sy)

    @property
    def centre_index(self) -> int:
        """Source position of the reference: the global centre s//2
        (src/coordinator.c:11-16)."""
        sx, sy, sz = self.sizes
        return self.index(sx // 2, sy // 2, sz // 2)

    @property
    def compute_points(self) -> int:
        """Point-updates per step: the compute region (s-8)^3, absorbing
        shell included, halo excluded (src/main.c:207-214)."""
        sx, sy, sz = self.sizes
        return (sx - 8) * (sy - 8) * (sz - 8)

    def interior_to_global(self, x, y, z):
        o = 4 + self.absorb
        return (x + o, y + o, z + o)


def receiver_line(geom: Geometry, count: int, depth: int):
    """``count`` receivers along x through the centre in y, at interior
    depth ``depth`` (global z = 4 + absorb + depth), spread evenly over the
    interior x range.  Returns linear indices."""
    sx, sy, _ = geom.sizes
    nx = geom.n[0]
    xs = np.linspace(0, nx - 1, count).round().astype(int)
    o = 4 + geom.absorb
    return np.array([geom.index(o + x, sy // 2, o + depth) for x in xs], np.int64)
