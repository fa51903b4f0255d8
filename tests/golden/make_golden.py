"""Generates the golden fixtures in this directory from the reference's own
sources (compiled here by oracle/build_oracle.py into oracle/_ref/libref.so).

Run from the repository root where the reference checkout exists:

    python tests/golden/make_golden.py

Fixtures (float32 unless stated):

* ``default_rvb.npz`` -- the reference default medium (src/precomp.c:156-169)
  with its random velocity boundary (src/boundary.c:7-104, seed 0) on a
  ragged cube (interior 12 x 10 x 9, absorption 3: sizes 26 x 24 x 23),
  40 steps of dt = 1e-3, dx = dy = dz = 12.5, source at the centre with
  FCUT = 40.  Holds the medium after the boundary (vpz, vsv), its ten
  precomputed coefficients, the source amplitudes and the final pc/qc of the
  OpenMP path (``omp_pc``, ``omp_qc``) and of the CUDA backend's arithmetic
  executed on the host (``cuda_pc``, ``cuda_qc``).
* ``hetero.npz`` -- a random heterogeneous anisotropic medium (numpy PCG64
  seed 7) on sizes 20 x 19 x 18, its coefficients from the reference's
  dc_compute_precomp_vars, and 30 steps of the OpenMP path.
* ``source.npz`` -- dc_calculate_source(dt, it) for it < 2001 and dt in
  {1e-3, 8e-4, 1e-6}.
* ``rvb_partitions.npz`` -- randomVelocityBoundaryPartition for a 2 x 1 x 2
  partitioning of a 22 x 20 x 21 cube (absorption 3), each partition's
  vpz/vsv and the seed after the call.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle.oracle import Geometry, Reference, reference_medium  # noqa: E402


def default_rvb(ref: Reference) -> dict:
    geom = Geometry((12, 10, 9), 3)
    aniso, coef = reference_medium(ref, geom, seed=0)
    steps, dt, d = 40, 1e-3, (12.5, 12.5, 12.5)
    src = np.array([ref.source(dt, i) for i in range(steps)], np.float32)
    z = lambda: np.zeros(geom.shape, np.float32)  # noqa: E731
    omp_pc, omp_qc = ref.run(0, geom.sizes, d, dt, steps, z(), z(), z(), z(), coef=coef,
                             src_index=geom.source_index, src=src)
    cu_pc, cu_qc = ref.run(1, geom.sizes, d, dt, steps, z(), z(), z(), z(), vpz=aniso["vpz"],
                           vsv=aniso["vsv"], src_index=geom.source_index, src=src)
    out = dict(sizes=np.array(geom.sizes), n=np.array(geom.n), absorb=np.array(geom.absorb),
               steps=np.array(steps), dt=np.array(dt, np.float32), d=np.array(d, np.float32),
               src_index=np.array(geom.source_index), src=src, vpz=aniso["vpz"],
               vsv=aniso["vsv"], omp_pc=omp_pc, omp_qc=omp_qc, cuda_pc=cu_pc, cuda_qc=cu_qc)
    for k, c in enumerate(coef):
        out[f"coef{k}"] = c
    return out


def hetero(ref: Reference) -> dict:
    sizes = (20, 19, 18)
    shape = (sizes[2], sizes[1], sizes[0])
    rng = np.random.Generator(np.random.PCG64(7))
    vp = rng.uniform(1800.0, 3200.0, shape).astype(np.float32)
    eps = rng.uniform(0.0, 0.3, shape).astype(np.float32)
    delta = (rng.uniform(0.0, 1.0, shape) * eps).astype(np.float32)
    aniso = {
        "vpz": vp,
        "epsilon": eps,
        "delta": delta,
        "theta": rng.uniform(-1.0, 1.0, shape).astype(np.float32),
        "phi": rng.uniform(0.0, 6.28, shape).astype(np.float32),
    }
    aniso["vsv"] = (vp * np.sqrt(np.abs(eps - delta) / np.float32(0.75))).astype(np.float32)
    coef = ref.precomp(aniso)
    steps, dt, d = 30, 1e-3, (12.5, 12.5, 12.5)
    src = np.array([ref.source(dt, i) for i in range(steps)], np.float32)
    src_index = sizes[0] // 2 + (sizes[1] // 2) * sizes[0] + (sizes[2] // 2) * sizes[0] * sizes[1]
    z = lambda: np.zeros(shape, np.float32)  # noqa: E731
    pc, qc = ref.run(0, sizes, d, dt, steps, z(), z(), z(), z(), coef=coef, src_index=src_index,
                     src=src)
    out = dict(sizes=np.array(sizes), steps=np.array(steps), dt=np.array(dt, np.float32),
               d=np.array(d, np.float32), src_index=np.array(src_index), src=src,
               omp_pc=pc, omp_qc=qc)
    for k, v in aniso.items():
        out["a_" + k] = v
    for k, c in enumerate(coef):
        out[f"coef{k}"] = c
    return out


def source(ref: Reference) -> dict:
    out = {}
    for tag, dt in (("1e-3", 1e-3), ("8e-4", 8e-4), ("1e-6", 1e-6)):
        out["dt_" + tag] = np.array([ref.source(dt, i) for i in range(2001)], np.float32)
    return out


def rvb_partitions(ref: Reference) -> dict:
    n, absorb = (6, 4, 5), 3
    glob = tuple(v + 2 * absorb + 8 for v in n)
    out = {"glob": np.array(glob), "n": np.array(n), "absorb": np.array(absorb)}
    px = [(0, 11), (11, glob[0] - 11)]
    pz = [(0, 10), (10, glob[2] - 10)]
    k = 0
    for zs, zl in pz:
        for xs, xl in px:
            local = (xl, glob[1], zl)
            shape = (zl, glob[1], xl)
            vpz = np.full(shape, 3000.0, np.float32)
            vsv = np.full(shape, 1296.0, np.float32)
            seed = ref.random_velocity_boundary(local, glob, (xs, 0, zs), n, 4, absorb, vpz, vsv, 0)
            out[f"p{k}_start"] = np.array((xs, 0, zs))
            out[f"p{k}_local"] = np.array(local)
            out[f"p{k}_vpz"] = vpz
            out[f"p{k}_vsv"] = vsv
            out[f"p{k}_seed"] = np.array(seed, np.uint64)
            k += 1
    out["parts"] = np.array(k)
    return out


def main() -> None:
    ref = Reference()
    for name, fn in (("default_rvb", default_rvb), ("hetero", hetero), ("source", source),
                     ("rvb_partitions", rvb_partitions)):
        data = fn(ref)
        np.savez_compressed(HERE / f"{name}.npz", **data)
        print(name, (HERE / f"{name}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
