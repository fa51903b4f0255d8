"""Parity against the reference's own CUDA path, run on the same GPU.

The reference's ``src/cuda_propagate.cu`` and ``src/device_data.cu`` are
compiled by nvcc for sm_103a with the reference's CUDA flags
(``oracle/build_oracle.py`` -> ``oracle/_ref/librefcuda.so``) and driven by
the reference's one-rank loop (``oracle/ref_driver.c``: the source, the
seven boxes of ``src/worker.c:321-402`` through ``dc_propagate``, the
swap).  The medium is the reference's default medium with its random
velocity boundary, generated by the reference's own ``src/precomp.c`` and
``src/boundary.c`` in the same library, on the config-1 geometry (64^3
interior + 16-cell boundary, 104^3 padded), with the reference's source
(``src/calculate_source.c``).

nvcc contracts multiply-adds inside ``sample_compute_optimized``, so no
kernel with another operation order can be bit-identical to it.  Gates
(relative L2 over the whole field): <= 1e-5 after 100 steps and <= 1e-4
after 500 steps, for the fast and the exact kernel.  The distance between
the reference's CUDA and OpenMP paths on the same medium is printed for
context.

Skipped where the reference sources are neither checked out nor staged, or
nvcc is missing.
"""
import numpy as np
import pytest

from oracle.oracle import Geometry, Reference, rel_l2

pytestmark = pytest.mark.gpu

DT = 1e-3
D = (12.5, 12.5, 12.5)
STEPS = (100, 500)


@pytest.fixture(scope="module")
def refcuda():
    try:
        return Reference("cuda")
    except FileNotFoundError as e:
        pytest.skip(str(e))


@pytest.fixture(scope="module")
def case(refcuda):
    geom = Geometry((64, 64, 64), 16)
    sx, sy, sz = geom.sizes
    aniso = refcuda.default_anisotropy(geom.shape)
    refcuda.random_velocity_boundary((sx, sy, sz), (sx, sy, sz), (0, 0, 0), geom.n, 4,
                                     geom.absorb, aniso["vpz"], aniso["vsv"], 0)
    src = np.array([refcuda.source(DT, it) for it in range(max(STEPS))], np.float32)
    outs = {}
    for steps in STEPS:
        z = [np.zeros(geom.shape, np.float32) for _ in range(4)]
        outs[steps] = refcuda.run(0, geom.sizes, D, DT, steps, *z, vpz=aniso["vpz"],
                                  vsv=aniso["vsv"], src_index=geom.source_index, src=src)
    return geom, aniso, src, outs


def _ours(dc, geom, aniso, src, steps, kernel):
    with dc.Simulation(geom.sizes, D, DT, kernel=kernel, medium=dc.MEDIUM_VPZ_VSV,
                       device=0) as sim:
        sim.set_vpz_vsv(aniso["vpz"], aniso["vsv"])
        sim.set_fields()
        sim.set_source(geom.source_index, src)
        sim.run(steps)
        sim.synchronize()
        f = sim.get_fields()
    return f["pc"], f["qc"]


def test_reference_cuda_path_runs(case):
    _, _, _, outs = case
    for pc, qc in outs.values():
        assert np.isfinite(pc).all() and np.isfinite(qc).all()
        assert np.abs(pc).max() > 0


@pytest.mark.parametrize("steps,tol", [(100, 1e-5), (500, 1e-4)])
@pytest.mark.parametrize("kernel", ["fast", "exact"])
def test_matches_reference_cuda_path(dc, case, kernel, steps, tol):
    geom, aniso, src, outs = case
    k = dc.KERNEL_FAST if kernel == "fast" else dc.KERNEL_EXACT
    pc, qc = _ours(dc, geom, aniso, src, steps, k)
    rpc, rqc = outs[steps]
    ep, eq = rel_l2(pc, rpc), rel_l2(qc, rqc)
    print(f"{kernel} kernel vs reference CUDA path, {steps} steps: "
          f"rel L2 p {ep:.3e}, q {eq:.3e}")
    assert ep <= tol and eq <= tol


def test_reference_cuda_vs_reference_openmp(case):
    """Context: the reference's two backends on the same medium (the OpenMP
    path reads the ten precomputed arrays, the CUDA path constant angles)."""
    try:
        pin = Reference("pin")
    except FileNotFoundError as e:
        pytest.skip(str(e))
    geom, aniso, src, outs = case
    coef = pin.precomp(aniso)
    steps = STEPS[0]
    z = [np.zeros(geom.shape, np.float32) for _ in range(4)]
    pc, qc = pin.run(0, geom.sizes, D, DT, steps, *z, coef=coef,
                     src_index=geom.source_index, src=src)
    e = rel_l2(pc, outs[steps][0])
    print(f"reference CUDA vs reference OpenMP, {steps} steps: rel L2 p {e:.3e}")
    assert e <= 1e-4
