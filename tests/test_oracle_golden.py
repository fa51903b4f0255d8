"""The oracle (oracle/dc_oracle.c) against the reference's own outputs.

The golden fixtures were produced by the reference's sources (see
tests/golden/make_golden.py); equality is bit for bit.  Where the reference
checkout is present, the oracle is also compared live against the reference
build on fresh random cases.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import (KIND_F32, KIND_F32_REFCUDA, KIND_F64, Geometry, reference_medium,
                           rel_l2)

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def zeros(shape, dtype=np.float32):
    return [np.zeros(shape, dtype) for _ in range(4)]


def test_source_matches_reference(port):
    g = load("source")
    for tag, dt in (("1e-3", 1e-3), ("8e-4", 8e-4), ("1e-6", 1e-6)):
        mine = np.array([port.source(dt, i) for i in range(2001)], np.float32)
        assert np.array_equal(mine, g["dt_" + tag])


def test_default_medium_and_boundary_match_reference(port):
    g = load("default_rvb")
    geom = Geometry(tuple(g["n"]), int(g["absorb"]))
    aniso, coef = reference_medium(port, geom, seed=0)
    assert np.array_equal(aniso["vpz"], g["vpz"])
    assert np.array_equal(aniso["vsv"], g["vsv"])
    for k in range(10):
        assert np.array_equal(coef[k], g[f"coef{k}"]), k


@pytest.mark.parametrize("kind,key", [(KIND_F32, "omp"), (KIND_F32_REFCUDA, "cuda")])
def test_propagation_bit_exact(port, kind, key):
    g = load("default_rvb")
    sizes = tuple(int(v) for v in g["sizes"])
    shape = (sizes[2], sizes[1], sizes[0])
    coef = [g[f"coef{k}"] for k in range(10)]
    res = port.run(kind, sizes, tuple(g["d"]), float(g["dt"]), int(g["steps"]), *zeros(shape),
                   coef=coef, vpz=g["vpz"], vsv=g["vsv"], src_index=int(g["src_index"]),
                   src=g["src"])
    assert np.array_equal(res.pc, g[f"{key}_pc"])
    assert np.array_equal(res.qc, g[f"{key}_qc"])
    assert np.abs(res.pc).max() > 1e-3  # the wave actually propagated


def test_heterogeneous_bit_exact(port):
    g = load("hetero")
    sizes = tuple(int(v) for v in g["sizes"])
    shape = (sizes[2], sizes[1], sizes[0])
    aniso = {k[2:]: v for k, v in g.items() if k.startswith("a_")}
    coef = port.precomp(aniso)
    for k in range(10):
        assert np.array_equal(coef[k], g[f"coef{k}"]), k
    res = port.run(KIND_F32, sizes, tuple(g["d"]), float(g["dt"]), int(g["steps"]), *zeros(shape),
                   coef=coef, src_index=int(g["src_index"]), src=g["src"])
    assert np.array_equal(res.pc, g["omp_pc"])
    assert np.array_equal(res.qc, g["omp_qc"])


def test_partitioned_boundary_matches_reference(port):
    g = load("rvb_partitions")
    glob = tuple(int(v) for v in g["glob"])
    n = tuple(int(v) for v in g["n"])
    for k in range(int(g["parts"])):
        local = tuple(int(v) for v in g[f"p{k}_local"])
        start = tuple(int(v) for v in g[f"p{k}_start"])
        shape = (local[2], local[1], local[0])
        vpz = np.full(shape, 3000.0, np.float32)
        vsv = np.full(shape, 1296.0, np.float32)
        seed = port.random_velocity_boundary(local, glob, start, n, 4, int(g["absorb"]), vpz, vsv)
        assert np.array_equal(vpz, g[f"p{k}_vpz"])
        assert np.array_equal(vsv, g[f"p{k}_vsv"])
        assert seed == int(g[f"p{k}_seed"])


def test_box_split_is_irrelevant(port):
    """Updating [4,s-4)^3 in one box or in the reference's 7 regions
    (src/worker.c:321-402) gives identical fields: points are independent
    within a step."""
    geom = Geometry((13, 11, 10), 2)
    aniso, coef = reference_medium(port, geom)
    rng = np.random.Generator(np.random.PCG64(3))
    pc = rng.standard_normal(geom.shape).astype(np.float32)
    qc = rng.standard_normal(geom.shape).astype(np.float32)
    pp = rng.standard_normal(geom.shape).astype(np.float32)
    qp = rng.standard_normal(geom.shape).astype(np.float32)
    d, dt = (10.0, 11.0, 12.0), 1e-3
    sx, sy, sz = geom.sizes
    one_p, one_q = pp.copy(), qp.copy()
    port.step(KIND_F32, geom.sizes, (4, 4, 4), (sx - 4, sy - 4, sz - 4), d, dt, pc, qc, one_p, one_q,
              coef=coef)
    split_p, split_q = pp.copy(), qp.copy()
    r = 4
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
    for b0, b1 in boxes:
        port.step(KIND_F32, geom.sizes, b0, b1, d, dt, pc, qc, split_p, split_q, coef=coef)
    assert np.array_equal(one_p, split_p) and np.array_equal(one_q, split_q)


def test_box_outside_compute_region_rejected(port):
    geom = Geometry((5, 5, 5), 1)
    f = np.zeros(geom.shape, np.float32)
    with pytest.raises(ValueError):
        port.step(KIND_F32, geom.sizes, (3, 4, 4), (6, 6, 6), (1, 1, 1), 1e-3, f, f, f.copy(),
                  f.copy(), coef=[f] * 10)


def test_fp64_oracle_close_to_fp32(port):
    g = load("default_rvb")
    sizes = tuple(int(v) for v in g["sizes"])
    shape = (sizes[2], sizes[1], sizes[0])
    coef = [g[f"coef{k}"] for k in range(10)]
    res = port.run(KIND_F64, sizes, tuple(g["d"]), float(g["dt"]), int(g["steps"]),
                   *zeros(shape, np.float64), coef=coef, src_index=int(g["src_index"]),
                   src=g["src"])
    assert rel_l2(g["omp_pc"], res.pc) < 1e-5


def test_oracle_matches_live_reference(port, reference):
    """Fresh seeds against the reference build (skipped without it)."""
    for seed, n, absorb, steps in ((1, (9, 8, 7), 2, 25), (5, (14, 6, 11), 4, 18)):
        geom = Geometry(n, absorb)
        a_ref, c_ref = reference_medium(reference, geom, seed=seed)
        a_me, c_me = reference_medium(port, geom, seed=seed)
        assert all(np.array_equal(x, y) for x, y in zip(c_ref, c_me))
        rng = np.random.Generator(np.random.PCG64(seed))
        init = [rng.standard_normal(geom.shape).astype(np.float32) * 1e-3 for _ in range(4)]
        src = np.array([reference.source(8e-4, i) for i in range(steps)], np.float32)
        for kind in (0, 1):
            rpc, rqc = reference.run(kind, geom.sizes, (12.5, 12.5, 12.5), 8e-4, steps,
                                     *[a.copy() for a in init], coef=c_ref, vpz=a_ref["vpz"],
                                     vsv=a_ref["vsv"], src_index=geom.source_index, src=src)
            res = port.run(kind, geom.sizes, (12.5, 12.5, 12.5), 8e-4, steps,
                           *[a.copy() for a in init], coef=c_me, vpz=a_me["vpz"],
                           vsv=a_me["vsv"], src_index=geom.source_index, src=src)
            assert np.array_equal(rpc, res.pc) and np.array_equal(rqc, res.qc)
