"""dc_gb300_exact_steps_noalloc: the exact stencil over caller-owned device
buffers, for callers that cannot allocate device memory themselves (their
memory is all owned up front, or their time loop must not allocate).
Checked through the C ABI on two calls in a row, for both medium forms and
with and without the energy output:

* against the simulation entry points (dc_gb300_run with the exact kernel),
  within the tolerance of the parity tests (relative L2 <= 1e-5 for the
  fields, relative difference <= 1e-5 for each step's energy);
* against the CPU oracle running the reference arithmetic, bit for bit (the
  exact kernel keeps the reference's operation order);
* free device memory (cudaMemGetInfo) is the same before and after a call.

The file is named so that pytest collects it last; it also passes alone in a
fresh process, where its first call does the per-device scratch set-up."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
TOL = 1e-5

# reference coefficient order (include/precomp.h:6-26) -> grouped lanes
# (cxx, cyy, cxy, czz | cxz, cyz, v2px, v2pz | v2sz, v2pn)
_REF_TO_LANE = {0: (0, 0), 1: (0, 1), 2: (0, 3), 3: (0, 2), 4: (1, 1), 5: (1, 0),
                6: (1, 2), 7: (1, 3), 8: (2, 0), 9: (2, 1)}


def _pitched(a, pitch):
    sz, sy, sx = a.shape
    out = np.zeros((sz, sy, pitch), a.dtype)
    out[:, :, :sx] = a
    return out


def _grouped(coef, pitch):
    sz, sy, _ = coef[0].shape
    count = sz * sy * pitch
    g0 = np.zeros((count, 4), np.float32)
    g1 = np.zeros((count, 4), np.float32)
    g2 = np.zeros((count, 2), np.float32)
    groups = (g0, g1, g2)
    for k, (grp, lane) in _REF_TO_LANE.items():
        groups[grp][:, lane] = _pitched(coef[k], pitch).reshape(-1)
    return np.concatenate([g0.reshape(-1), g1.reshape(-1), g2.reshape(-1)])


def _pairs(p, q, pitch):
    return np.stack([_pitched(p, pitch), _pitched(q, pitch)], axis=-1).reshape(-1)


def _unpair(buf, shape, pitch):
    sz, sy, sx = shape
    a = buf.reshape(sz, sy, pitch, 2)[:, :, :sx, :]
    return np.ascontiguousarray(a[..., 0]), np.ascontiguousarray(a[..., 1])


def _config(dc, sizes, d, dt, medium):
    return dc.Config(sizes[0], sizes[1], sizes[2], d[0], d[1], d[2], dt, dc.KERNEL_EXACT,
                     medium, 0)


def _fields(shape, seed=7):
    rng = np.random.default_rng(seed)
    fields = [rng.standard_normal(shape).astype(np.float32) for _ in range(4)]
    for f in fields:  # the 4-cell halo stays zero, as in the reference
        f[:4], f[-4:], f[:, :4], f[:, -4:], f[:, :, :4], f[:, :, -4:] = 0, 0, 0, 0, 0, 0
    return fields


def _inputs(medium: str):
    """Sizes, spacing, dt, the medium (ten coefficients or (vpz, vsv)) and
    random initial fields: the golden heterogeneous medium for the
    coefficient form, the golden default medium with its random velocity
    boundary for the vpz/vsv form."""
    g = dict(np.load(GOLDEN / ("hetero.npz" if medium == "precomp" else "default_rvb.npz")))
    sizes = tuple(int(v) for v in g["sizes"])
    shape = (sizes[2], sizes[1], sizes[0])
    med = ([g[f"coef{k}"] for k in range(10)] if medium == "precomp"
           else (g["vpz"], g["vsv"]))
    return sizes, tuple(float(v) for v in g["d"]), float(g["dt"]), med, _fields(shape)


@pytest.mark.parametrize("with_energy", [True, False])
@pytest.mark.parametrize("medium", ["precomp", "vpz_vsv"])
def test_noalloc_matches_simulation_and_oracle_on_two_calls(dc, port, medium, with_energy):
    torch = pytest.importorskip("torch")
    from oracle.oracle import KIND_F32, KIND_F32_REFCUDA
    sizes, d, dt, med, (pp, pc, qp, qc) = _inputs(medium)
    form = dc.MEDIUM_PRECOMP if medium == "precomp" else dc.MEDIUM_VPZ_VSV
    n = 12
    # existing entry points: a simulation running 2n steps with energy
    with dc.Simulation(sizes, d, dt, kernel=dc.KERNEL_EXACT, medium=form, device=0) as sim:
        if medium == "precomp":
            sim.set_precomp(med)
        else:
            sim.set_vpz_vsv(*med)
        sim.set_fields(pp, pc, qp, qc)
        sim.enable_energy(2 * n)
        sim.run(n)
        sim.synchronize()
        want = [sim.get_fields()]
        sim.run(n)
        sim.synchronize()
        want.append(sim.get_fields())
        want_e = sim.energy(2 * n)
    # the CPU oracle with the reference arithmetic, n steps at a time
    kind = KIND_F32 if medium == "precomp" else KIND_F32_REFCUDA
    o = [a.copy() for a in (pp, pc, qp, qc)]
    oracle = []
    for _ in range(2):
        r = port.run(kind, sizes, d, dt, n, *o, coef=med if medium == "precomp" else None,
                     vpz=None if medium == "precomp" else med[0],
                     vsv=None if medium == "precomp" else med[1], energy=True)
        oracle.append(r)
        o = [r.pp.copy(), r.pc.copy(), r.qp.copy(), r.qc.copy()]

    # caller-owned device buffers (allocated here by the test, not by the
    # entry point)
    pitch = (sizes[0] + 3) // 4 * 4
    shape = (sizes[2], sizes[1], sizes[0])
    dev = torch.device("cuda", 0)
    prev = torch.from_numpy(_pairs(pp, qp, pitch)).to(dev)
    cur = torch.from_numpy(_pairs(pc, qc, pitch)).to(dev)
    host_medium = _grouped(med, pitch) if medium == "precomp" else _pairs(*med, pitch)
    medium_dev = torch.from_numpy(host_medium).to(dev)
    torch.cuda.synchronize()
    by_ptr = {prev.data_ptr(): prev, cur.data_ptr(): cur}
    cfg = _config(dc, sizes, d, dt, form)
    pairs = (C.c_void_p * 2)(prev.data_ptr(), cur.data_ptr())
    lib = dc.lib()
    for call in range(2):
        energy = np.zeros(n, np.float64) if with_energy else None
        free_before = torch.cuda.mem_get_info(0)[0]
        rc = lib.dc_gb300_exact_steps_noalloc(
            C.byref(cfg), pairs, C.c_void_p(medium_dev.data_ptr()), n,
            energy.ctypes.data_as(C.POINTER(C.c_double)) if with_energy else None, None)
        assert rc == 0, lib.dc_gb300_last_error().decode()
        assert torch.cuda.mem_get_info(0)[0] == free_before, "device memory changed"
        newest = by_ptr[pairs[1]].cpu().numpy()
        before = by_ptr[pairs[0]].cpu().numpy()
        p_new, q_new = _unpair(newest, shape, pitch)
        p_old, q_old = _unpair(before, shape, pitch)
        w = want[call]
        assert rel_l2(p_new, w["pc"]) <= TOL and rel_l2(q_new, w["qc"]) <= TOL
        assert rel_l2(p_old, w["pp"]) <= TOL and rel_l2(q_old, w["qp"]) <= TOL
        r = oracle[call]
        assert np.array_equal(p_new, r.pc) and np.array_equal(q_new, r.qc)
        assert np.array_equal(p_old, r.pp) and np.array_equal(q_old, r.qp)
        if with_energy:
            ref_e = want_e[call * n:(call + 1) * n]
            assert np.all(ref_e > 0)
            assert np.max(np.abs(energy - ref_e) / ref_e) <= TOL
            assert np.max(np.abs(energy - r.energy) / r.energy) <= TOL


def test_noalloc_rejects_steps_beyond_scratch(dc):
    sizes, d, dt, _, _ = _inputs("precomp")
    cfg = _config(dc, sizes, d, dt, dc.MEDIUM_PRECOMP)
    dummy = (C.c_void_p * 2)(16, 32)  # never dereferenced: the count is checked first
    lib = dc.lib()
    rc = lib.dc_gb300_exact_steps_noalloc(C.byref(cfg), dummy, C.c_void_p(48), 4097, None, None)
    assert rc == dc.ERR_ARG
    msg = lib.dc_gb300_last_error().decode()
    assert "4096" in msg and "maximum" in msg


def test_noalloc_refuses_capturing_stream(dc):
    """A call on a stream under capture fails with DC_GB300_ERR_ARG before it
    issues any work, and the caller's capture stays valid."""
    torch = pytest.importorskip("torch")
    sizes, d, dt, _, _ = _inputs("precomp")
    cfg = _config(dc, sizes, d, dt, dc.MEDIUM_PRECOMP)
    dummy = (C.c_void_p * 2)(16, 32)  # never dereferenced: the capture is checked first
    lib = dc.lib()
    x = torch.zeros(1, device="cuda:0")
    stream = torch.cuda.Stream(device=0)
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        graph.capture_begin()
        try:
            x.add_(1.0)
            rc = lib.dc_gb300_exact_steps_noalloc(C.byref(cfg), dummy, C.c_void_p(48), 1, None,
                                                  C.c_void_p(stream.cuda_stream))
        finally:
            graph.capture_end()
    assert rc == dc.ERR_ARG
    assert "capturing" in lib.dc_gb300_last_error().decode()
    graph.replay()
    torch.cuda.synchronize()
    assert float(x.item()) == 1.0
