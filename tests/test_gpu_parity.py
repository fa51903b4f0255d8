"""GPU parity: the CUDA path, through the C ABI, against the reference's own
outputs (golden fixtures) and the CPU oracle.

Tolerances (relative L2 over the whole array):
* exact kernel: 0 -- bit-identical to the reference's OpenMP path and to the
  reference CUDA backend's arithmetic;
* fast kernel: 1e-5 where the reference's own FP32 result is within 2.3e-6
  of FP64 (<= 100 steps at the config-1 geometry), 1e-4 against the OpenMP
  path at 500 steps; and its distance to the FP64 oracle may exceed the
  reference's own by at most 50 %.
"""
import os
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import (KIND_F32, KIND_F32_REFCUDA, KIND_F64, Geometry, reference_medium,
                           rel_l2)

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def zeros(shape, dtype=np.float32):
    return [np.zeros(shape, dtype) for _ in range(4)]


def run_sim(dc, sizes, d, dt, steps, kernel, medium, coef=None, vpz=None, vsv=None,
            src_index=-1, src=None, sponge=None, fields=None):
    with dc.Simulation(sizes, d, dt, kernel=kernel, medium=medium, device=0) as sim:
        if medium == dc.MEDIUM_PRECOMP:
            sim.set_precomp(coef)
        else:
            sim.set_vpz_vsv(vpz, vsv)
        sim.set_fields(*(fields or (None,) * 4))
        if src_index >= 0:
            sim.set_source(src_index, src)
        if sponge is not None:
            sim.set_sponge(*sponge)
        sim.run(steps)
        sim.synchronize()
        return sim.get_fields()


def test_smoke():
    import __graft_entry__ as ge
    ge.smoke()


@pytest.mark.parametrize("medium,key", [(0, "omp"), (1, "cuda")])
def test_exact_kernel_bit_identical_to_reference(dc, medium, key):
    g = load("default_rvb")
    sizes = tuple(int(v) for v in g["sizes"])
    coef = [g[f"coef{k}"] for k in range(10)]
    out = run_sim(dc, sizes, tuple(g["d"]), float(g["dt"]), int(g["steps"]), dc.KERNEL_EXACT,
                  medium, coef=coef, vpz=g["vpz"], vsv=g["vsv"], src_index=int(g["src_index"]),
                  src=g["src"])
    assert np.array_equal(out["pc"], g[f"{key}_pc"])
    assert np.array_equal(out["qc"], g[f"{key}_qc"])


@pytest.mark.parametrize("medium,key", [(0, "omp"), (1, "cuda")])
def test_fast_kernel_matches_reference(dc, medium, key):
    g = load("default_rvb")
    sizes = tuple(int(v) for v in g["sizes"])
    coef = [g[f"coef{k}"] for k in range(10)]
    out = run_sim(dc, sizes, tuple(g["d"]), float(g["dt"]), int(g["steps"]), dc.KERNEL_FAST,
                  medium, coef=coef, vpz=g["vpz"], vsv=g["vsv"], src_index=int(g["src_index"]),
                  src=g["src"])
    assert rel_l2(out["pc"], g[f"{key}_pc"]) <= 1e-5
    assert rel_l2(out["qc"], g[f"{key}_qc"]) <= 1e-5


@pytest.mark.parametrize("kernel,tol", [(1, 0.0), (0, 1e-5)])
def test_heterogeneous_medium(dc, kernel, tol):
    g = load("hetero")
    sizes = tuple(int(v) for v in g["sizes"])
    coef = [g[f"coef{k}"] for k in range(10)]
    out = run_sim(dc, sizes, tuple(g["d"]), float(g["dt"]), int(g["steps"]), kernel, 0,
                  coef=coef, src_index=int(g["src_index"]), src=g["src"])
    assert rel_l2(out["pc"], g["omp_pc"]) <= tol
    assert rel_l2(out["qc"], g["omp_qc"]) <= tol


def _worker_loop(dc, process, steps, sizes, d, dt, src_index):
    """The one-rank time loop of src/worker.c:466-511 through the ABI,
    including the 7-region split of src/worker.c:321-402."""
    data = dc.device_data_init(process)
    r = 4
    sx, sy, sz = sizes
    boxes = []
    for side in range(2):
        boxes.append(((r if side == 0 else sx - 2 * r, r, r),
                      (2 * r if side == 0 else sx - r, sy - r, sz - r)))
    for side in range(2):
        boxes.append(((2 * r, r if side == 0 else sy - 2 * r, r),
                      (sx - 2 * r, 2 * r if side == 0 else sy - r, sz - r)))
    for side in range(2):
        boxes.append(((2 * r, 2 * r, r if side == 0 else sz - 2 * r),
                      (sx - 2 * r, sy - 2 * r, 2 * r if side == 0 else sz - r)))
    boxes.append(((2 * r,) * 3, (sx - 2 * r, sy - 2 * r, sz - 2 * r)))
    for it in range(steps):
        dc.device_add_source(data, src_index, dc.calculate_source(dt, it))
        for b0, b1 in boxes:
            dc.propagate(b0, b1, sizes, data, *d, dt)
        dc.device_swap_arrays(data)
    dc.device_data_get_results(process, data)
    dc.device_data_free(data)
    return process.field("pc"), process.field("qc")


@pytest.mark.parametrize("kernel", ["exact", "fast"])
def test_reference_abi_worker_loop(dc, kernel, monkeypatch):
    g = load("default_rvb")
    sizes = tuple(int(v) for v in g["sizes"])
    d, dt, steps = tuple(float(v) for v in g["d"]), float(g["dt"]), int(g["steps"])
    coef = [g[f"coef{k}"] for k in range(10)]
    monkeypatch.setenv("DC_GB300_KERNEL", kernel)
    proc = dc.Process(sizes, d, dt, precomp=coef, source_index=int(g["src_index"]))
    pc, qc = _worker_loop(dc, proc, steps, sizes, d, dt, int(g["src_index"]))
    if kernel == "exact":
        assert np.array_equal(pc, g["omp_pc"]) and np.array_equal(qc, g["omp_qc"])
    else:
        assert rel_l2(pc, g["omp_pc"]) <= 1e-5 and rel_l2(qc, g["omp_qc"]) <= 1e-5


def test_abi_medium_from_anisotropy_uses_gpu_precompute(dc, monkeypatch):
    """dc_device_data_init with only anisotropy arrays: the coefficients are
    computed on the GPU in FP64 and must equal the reference's host
    precompute."""
    g = load("hetero")
    sizes = tuple(int(v) for v in g["sizes"])
    aniso = {k[2:]: v for k, v in g.items() if k.startswith("a_")}
    gpu_coef = dc.compute_precomp_vars(sizes, aniso)
    for k in range(10):
        assert np.array_equal(gpu_coef[k], g[f"coef{k}"]), k
    monkeypatch.setenv("DC_GB300_KERNEL", "exact")
    d, dt, steps = tuple(float(v) for v in g["d"]), float(g["dt"]), int(g["steps"])
    proc = dc.Process(sizes, d, dt, anisotropy=aniso, source_index=int(g["src_index"]))
    pc, qc = _worker_loop(dc, proc, steps, sizes, d, dt, int(g["src_index"]))
    assert np.array_equal(pc, g["omp_pc"]) and np.array_equal(qc, g["omp_qc"])


def test_graph_replay_equals_single_launches(dc, port):
    """> 64 steps go through captured graphs; the result must not depend on
    how the steps were grouped into run() calls."""
    geom = Geometry((20, 18, 16), 6)
    aniso, coef = reference_medium(port, geom)
    src = port.source_table(1e-3, 150)
    outs = []
    for chunks in ((150,), (3, 64, 1, 70, 12), (1,) * 10 + (140,)):
        with dc.Simulation(geom.sizes, (12.5,) * 3, 1e-3, kernel=dc.KERNEL_FAST, device=0) as sim:
            sim.set_precomp(coef)
            sim.set_fields()
            sim.set_source(geom.source_index, src)
            for c in chunks:
                sim.run(c)
            sim.synchronize()
            assert sim.steps_done == 150
            outs.append(sim.get_fields())
    for o in outs[1:]:
        for k in ("pp", "pc", "qp", "qc"):
            assert np.array_equal(o[k], outs[0][k]), k


def test_config1_geometry_against_oracle(dc, port):
    """Config-1 geometry (64^3 interior, 16-cell absorbing shell: 104^3),
    reference default medium + random boundary, dt = 1 ms.  100 steps: fast
    within 1e-5 of both reference arithmetics; exact bit-identical."""
    geom = Geometry((64, 64, 64), 16)
    aniso, coef = reference_medium(port, geom)
    steps, dt, d = 100, 1e-3, (12.5, 12.5, 12.5)
    src = port.source_table(dt, steps)
    s = geom.source_index
    omp = port.run(KIND_F32, geom.sizes, d, dt, steps, *zeros(geom.shape), coef=coef,
                   src_index=s, src=src)
    cuda = port.run(KIND_F32_REFCUDA, geom.sizes, d, dt, steps, *zeros(geom.shape),
                    vpz=aniso["vpz"], vsv=aniso["vsv"], src_index=s, src=src)
    fast = run_sim(dc, geom.sizes, d, dt, steps, dc.KERNEL_FAST, 0, coef=coef, src_index=s,
                   src=src)
    assert rel_l2(fast["pc"], omp.pc) <= 1e-5 and rel_l2(fast["qc"], omp.qc) <= 1e-5
    fast_v = run_sim(dc, geom.sizes, d, dt, steps, dc.KERNEL_FAST, 1, vpz=aniso["vpz"],
                     vsv=aniso["vsv"], src_index=s, src=src)
    assert rel_l2(fast_v["pc"], cuda.pc) <= 1e-5 and rel_l2(fast_v["qc"], cuda.qc) <= 1e-5
    exact = run_sim(dc, geom.sizes, d, dt, steps, dc.KERNEL_EXACT, 0, coef=coef, src_index=s,
                    src=src)
    assert np.array_equal(exact["pc"], omp.pc) and np.array_equal(exact["qc"], omp.qc)


def test_config1_500_steps_within_fp32_noise(dc, port):
    """500 steps (the config's length): fast within 1e-4 of the OpenMP path,
    and no further from the FP64 oracle than 1.5x the reference's own FP32
    distance."""
    geom = Geometry((64, 64, 64), 16)
    aniso, coef = reference_medium(port, geom)
    steps, dt, d = 500, 1e-3, (12.5, 12.5, 12.5)
    src = port.source_table(dt, steps)
    s = geom.source_index
    omp = port.run(KIND_F32, geom.sizes, d, dt, steps, *zeros(geom.shape), coef=coef,
                   src_index=s, src=src)
    f64 = port.run(KIND_F64, geom.sizes, d, dt, steps, *zeros(geom.shape, np.float64),
                   coef=coef, src_index=s, src=src)
    fast = run_sim(dc, geom.sizes, d, dt, steps, dc.KERNEL_FAST, 0, coef=coef, src_index=s,
                   src=src)
    assert rel_l2(fast["pc"], omp.pc) <= 1e-4
    ref_err = rel_l2(omp.pc, f64.pc)
    assert rel_l2(fast["pc"], f64.pc) <= 1.5 * ref_err + 1e-7


def test_config1_homogeneous_workload(dc, port):
    """The config-1 workload itself: 64^3 interior + 16-cell sponge,
    homogeneous vp 3000, epsilon 0.24, delta 0.10, theta pi/4, phi pi/6,
    vs 0, 15 Hz Ricker (FCUT 45) at the centre, dt 1 ms, 500 steps, final p
    and a 64-receiver line at interior depth 8.  Exact: bit-identical to
    the oracle's reference arithmetic (fields and traces); fast: 1e-4 of it
    and no further from FP64 than 1.5x the reference's own FP32 distance."""
    from dc_gb300 import medium
    geom = Geometry((64, 64, 64), 16)
    coef = port.precomp(medium.homogeneous(geom.sizes))
    steps, dt, d = 500, 1e-3, (12.5, 12.5, 12.5)
    src = port.source_table(dt, steps + 1, 45.0)
    sponge = [port.sponge_profile(s, geom.absorb, 0.35) for s in geom.sizes]
    rec = medium.receiver_line(medium.Geometry(geom.n, geom.absorb), 64, 8)
    s = geom.source_index  # the centre s // 2
    common = dict(coef=coef, src_index=s, src=src, sponge=sponge, rec=rec)
    ref = port.run(KIND_F32, geom.sizes, d, dt, steps, *zeros(geom.shape), **common)
    f64 = port.run(KIND_F64, geom.sizes, d, dt, steps, *zeros(geom.shape, np.float64), **common)
    out = {}
    for kernel in (dc.KERNEL_EXACT, dc.KERNEL_FAST):
        with dc.Simulation(geom.sizes, d, dt, kernel=kernel, device=0) as sim:
            sim.set_precomp(coef)
            sim.set_fields()
            sim.set_source(s, src)
            sim.set_sponge(*sponge)
            sim.set_receivers(rec, steps)
            sim.run(steps)
            sim.synchronize()
            out[kernel] = (sim.get_fields(), sim.traces(steps))
    ex, ex_tr = out[dc.KERNEL_EXACT]
    assert np.array_equal(ex["pc"], ref.pc) and np.array_equal(ex["qc"], ref.qc)
    assert np.array_equal(ex_tr, ref.traces.astype(np.float32))
    fa, fa_tr = out[dc.KERNEL_FAST]
    assert rel_l2(fa["pc"], ref.pc) <= 1e-4 and rel_l2(fa_tr, ref.traces) <= 1e-4
    ref_err = rel_l2(ref.pc, f64.pc)
    assert rel_l2(fa["pc"], f64.pc) <= 1.5 * ref_err + 1e-7
    assert np.abs(fa_tr).max() > 0


def test_ragged_and_tiny_cubes(dc, port):
    """Sizes that are not multiples of 4 (pitched rows), of the 32 x 16
    tile, and cubes below the 16-cell threshold of the reference's region
    split."""
    for n, absorb, steps in (((3, 5, 2), 1, 12), ((37, 21, 19), 2, 25), ((1, 1, 1), 0, 5)):
        geom = Geometry(n, absorb)
        aniso, coef = reference_medium(port, geom)
        rng = np.random.Generator(np.random.PCG64(11))
        init = [rng.standard_normal(geom.shape).astype(np.float32) for _ in range(4)]
        d, dt = (10.0, 12.0, 14.0), 5e-4
        src = port.source_table(dt, steps)
        ref = port.run(KIND_F32, geom.sizes, d, dt, steps, *[a.copy() for a in init], coef=coef,
                       src_index=geom.source_index, src=src)
        for kernel in (dc.KERNEL_EXACT, dc.KERNEL_FAST):
            out = run_sim(dc, geom.sizes, d, dt, steps, kernel, 0, coef=coef,
                          src_index=geom.source_index, src=src, fields=init)
            tol = 0.0 if kernel == dc.KERNEL_EXACT else 1e-5
            for k, r in (("pc", ref.pc), ("qc", ref.qc), ("pp", ref.pp), ("qp", ref.qp)):
                assert rel_l2(out[k], r) <= tol, (n, kernel, k)
            # the 4-cell halo is never written
            sx, sy, sz = geom.sizes
            halo = np.ones(geom.shape, bool)
            halo[4:sz - 4, 4:sy - 4, 4:sx - 4] = False
            assert np.array_equal(out["pc"][halo], ref.pc[halo])


@pytest.mark.parametrize("kernel", [1, 0])
def test_sponge_against_oracle(dc, port, kernel):
    geom = Geometry((24, 20, 18), 8)
    aniso, coef = reference_medium(port, geom)
    sponge = [port.sponge_profile(s, geom.absorb, 0.35) for s in geom.sizes]
    steps, dt, d = 60, 1e-3, (12.5,) * 3
    src = port.source_table(dt, steps, 45.0)
    ref = port.run(KIND_F32, geom.sizes, d, dt, steps, *zeros(geom.shape), coef=coef,
                   src_index=geom.source_index, src=src, sponge=sponge)
    out = run_sim(dc, geom.sizes, d, dt, steps, kernel, 0, coef=coef,
                  src_index=geom.source_index, src=src, sponge=sponge)
    tol = 0.0 if kernel == 1 else 1e-5
    assert rel_l2(out["pc"], ref.pc) <= tol and rel_l2(out["qc"], ref.qc) <= tol


@pytest.mark.parametrize("kernel", [1, 0])
def test_receivers_and_energy(dc, port, kernel):
    geom = Geometry((30, 26, 22), 5)
    aniso, coef = reference_medium(port, geom)
    steps, dt, d = 90, 1e-3, (12.5,) * 3
    src = port.source_table(dt, steps)
    sx, sy, sz = geom.sizes
    rec = [geom.index(x, sy // 2, 10) for x in range(4, sx - 4, 3)] + [geom.source_index]
    ref = port.run(KIND_F32, geom.sizes, d, dt, steps, *zeros(geom.shape), coef=coef,
                   src_index=geom.source_index, src=src, rec=rec, energy=True)
    with dc.Simulation(geom.sizes, d, dt, kernel=kernel, device=0) as sim:
        sim.set_precomp(coef)
        sim.set_fields()
        sim.set_source(geom.source_index, src)
        sim.set_receivers(rec, steps)
        sim.enable_energy(steps)
        sim.run(steps)
        sim.synchronize()
        tr = sim.traces(steps)
        en = sim.energy(steps)
    if kernel == 1:
        assert np.array_equal(tr, ref.traces.astype(np.float32))
    else:
        assert rel_l2(tr, ref.traces) <= 1e-5
    assert np.allclose(en, ref.energy, rtol=1e-5, atol=0)


def test_propagate_box_bounds_are_checked(dc):
    with dc.Simulation((20, 20, 20), device=0) as sim:
        with pytest.raises(dc.DcError) as e:
            sim.propagate_box((3, 4, 4), (10, 10, 10))
        assert e.value.code == dc.ERR_ARG
        with pytest.raises(dc.DcError):
            sim.propagate_box((4, 4, 4), (17, 10, 10))
        sim.propagate_box((4, 4, 4), (4, 10, 10))  # empty box: no-op
        with pytest.raises(dc.DcError):
            sim.set_source(0, [1.0])  # in the halo


def test_halo_face_roundtrip(dc):
    sizes = (21, 18, 17)
    proc = dc.Process(sizes, (1.0, 1.0, 1.0), 1e-3,
                      anisotropy=dc.compute_anisotropy_vars(sizes))
    data = dc.device_data_init(proc)
    view = dc.device_view(data)
    rng = np.random.Generator(np.random.PCG64(2))
    start, end = (4, 3, 5), (17, 9, 8)
    buf = rng.standard_normal((3, 6, 13)).astype(np.float32)
    dc.insert_halo_face(data, buf, start, end, sizes, view.pp)
    back = dc.extract_halo_face(data, start, end, sizes, view.pp)
    assert np.array_equal(back, buf)
    dc.device_data_free(data)


@pytest.mark.parametrize("n,absorb,seed", [((12, 10, 9), 3, 0), ((40, 7, 19), 5, 123),
                                           ((64, 64, 64), 16, 0)])
def test_reference_medium_generated_on_gpu(dc, port, n, absorb, seed):
    """Default anisotropy + random velocity boundary (glibc rand_r sequence
    replayed by skip-ahead) + FP64 precompute, all on the GPU, against the
    host restatement pinned to the reference."""
    geom = Geometry(n, absorb)
    aniso, coef = reference_medium(port, geom, seed=seed)
    with dc.Simulation(geom.sizes, device=0) as sim:
        sim.generate_reference(n, absorb, seed)
        got = sim.get_precomp()
    for k in range(10):
        assert np.array_equal(got[k], coef[k]), k
    with dc.Simulation(geom.sizes, device=0, medium=dc.MEDIUM_VPZ_VSV) as sim:
        sim.generate_reference(n, absorb, seed)
        vpz, vsv = sim.get_vpz_vsv()
    assert np.array_equal(vpz, aniso["vpz"]) and np.array_equal(vsv, aniso["vsv"])


@pytest.mark.parametrize("kernel", [1, 0])
def test_receiver_columns_and_duplicates(dc, port, kernel):
    """Several receivers in one column (a vertical array, spanning the
    kernel's z-chunks), duplicated indices and scattered points."""
    geom = Geometry((20, 18, 70), 4)
    aniso, coef = reference_medium(port, geom)
    steps, dt = 40, 1e-3
    src = port.source_table(dt, steps)
    sx, sy, sz = geom.sizes
    cx, cy = sx // 2 + 2, sy // 2 - 1
    rec = [geom.index(cx, cy, z) for z in range(4, sz - 4, 5)]
    rec += [rec[3], geom.index(5, 6, 7), geom.index(sx - 5, sy - 5, sz - 5), geom.source_index]
    ref = port.run(KIND_F32, geom.sizes, (12.5,) * 3, dt, steps, *zeros(geom.shape), coef=coef,
                   src_index=geom.source_index, src=src, rec=rec)
    with dc.Simulation(geom.sizes, (12.5,) * 3, dt, kernel=kernel, device=0) as sim:
        sim.set_precomp(coef)
        sim.set_fields()
        sim.set_source(geom.source_index, src)
        sim.set_receivers(rec, steps)
        sim.run(steps)
        sim.synchronize()
        tr = sim.traces(steps)
    if kernel == 1:
        assert np.array_equal(tr, ref.traces.astype(np.float32))
    else:
        assert rel_l2(tr, ref.traces) <= 1e-5


@pytest.mark.parametrize("kernel", [1, 0])
def test_observed_state_excludes_next_source(dc, port, kernel):
    """The next step's amplitude is fused into the store, yet get_fields after
    run(N) is the reference's state after N steps even when the amplitude
    table is longer; replacing the source between runs keeps that too."""
    geom = Geometry((16, 14, 12), 3)
    aniso, coef = reference_medium(port, geom)
    dt = 1e-3
    long_src = port.source_table(dt, 200)
    other = geom.index(geom.sizes[0] // 2 - 3, geom.sizes[1] // 2, geom.sizes[2] // 2 + 2)
    # oracle: 30 steps with the centre source, then 25 with `other`
    z = zeros(geom.shape)
    ref1 = port.run(KIND_F32, geom.sizes, (12.5,) * 3, dt, 30, *z, coef=coef,
                    src_index=geom.source_index, src=long_src)
    src2 = np.concatenate([np.zeros(30, np.float32), long_src[30:55]])
    # continue from ref1's state: pp<-ref1.pp etc. (o_run leaves pc = current)
    ref2 = port.run(KIND_F32, geom.sizes, (12.5,) * 3, dt, 25, ref1.pp.copy(), ref1.pc.copy(),
                    ref1.qp.copy(), ref1.qc.copy(), coef=coef, src_index=other,
                    src=long_src[30:55])
    tol = 0.0 if kernel == 1 else 1e-5
    with dc.Simulation(geom.sizes, (12.5,) * 3, dt, kernel=kernel, device=0) as sim:
        sim.set_precomp(coef)
        sim.set_fields()
        sim.set_source(geom.source_index, long_src)
        sim.run(30)
        sim.synchronize()
        f = sim.get_fields()
        assert rel_l2(f["pc"], ref1.pc) <= tol and rel_l2(f["qc"], ref1.qc) <= tol
        assert rel_l2(f["pp"], ref1.pp) <= tol
        sim.set_source(other, src2)
        sim.run(25)
        sim.synchronize()
        f = sim.get_fields()
        assert rel_l2(f["pc"], ref2.pc) <= tol and rel_l2(f["qc"], ref2.qc) <= tol


def test_fast_ring_depth_bit_identical(dc, monkeypatch):
    """The FP32 sweep's 4-stage TMA ring (chosen for large boxes) gives the
    same bits as the 3-stage ring: only the pipelining differs."""
    g = load("hetero")
    sizes = tuple(int(v) for v in g["sizes"])
    coef = [g[f"coef{k}"] for k in range(10)]
    out = {}
    for ns in ("3", "4"):
        monkeypatch.setenv("DC_GB300_FAST_STAGES", ns)
        out[ns] = run_sim(dc, sizes, tuple(g["d"]), float(g["dt"]), int(g["steps"]),
                          dc.KERNEL_FAST, 0, coef=coef, src_index=int(g["src_index"]),
                          src=g["src"])
    for k in ("pp", "pc", "qp", "qc"):
        assert np.array_equal(out["3"][k], out["4"][k]), k
    assert rel_l2(out["4"]["pc"], g["omp_pc"]) <= 1e-5


@pytest.mark.parametrize("stages,case", [("3", "cube"), ("4", "cube"), ("3", "ragged")])
def test_fast_zchunks_bit_identical(dc, port, monkeypatch, stages, case):
    """Splitting each column's z sweep into chunks (the count the wave model
    picks, or any forced count) changes which CTA computes a plane, not how:
    on the config-1 geometry (104^3, 96 updated planes) and on a ragged box
    with unequal spacings (run-time weights) the fields are the same bits
    for the default and for 1, 2, 3 and 5 chunks."""
    if case == "cube":
        geom, steps, dt, d = Geometry((64, 64, 64), 16), 40, 1e-3, (12.5, 12.5, 12.5)
    else:
        geom, steps, dt, d = Geometry((37, 29, 53), 8), 40, 5e-4, (12.5, 10.0, 15.0)
    aniso, coef = reference_medium(port, geom)
    src = port.source_table(dt, steps)
    monkeypatch.setenv("DC_GB300_FAST_STAGES", stages)
    out = {}
    for chunks in (None, "1", "2", "3", "5"):
        if chunks is None:
            monkeypatch.delenv("DC_GB300_FAST_ZCHUNKS", raising=False)
        else:
            monkeypatch.setenv("DC_GB300_FAST_ZCHUNKS", chunks)
        out[chunks] = run_sim(dc, geom.sizes, d, dt, steps, dc.KERNEL_FAST, 0, coef=coef,
                              src_index=geom.source_index, src=src)
    assert np.isfinite(out[None]["pc"]).all() and np.abs(out[None]["pc"]).max() > 0
    for chunks in ("1", "2", "3", "5"):
        for k in ("pp", "pc", "qp", "qc"):
            assert np.array_equal(out[None][k], out[chunks][k]), (chunks, k)
