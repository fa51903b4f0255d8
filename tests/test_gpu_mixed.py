"""The mixed-precision medium forms (DC_GB300_MEDIUM_PRECOMP_F16 / _BF16):
the fast kernel reads a 16-bit copy of the ten coefficients, computes in
FP32 and keeps FP32 wavefields.  The FP16 form stores the angle terms as
16-bit fixed point and the velocity terms as FP16 ratios to a per-row FP32
base; the BF16 form rounds all ten to BF16 (velocity terms scaled by
2^-vexp).

* Against the oracle run on identically rounded coefficients the result must
  agree to FP32 reordering noise (rel. L2 <= 1e-5): the kernel adds no error
  beyond the storage rounding.
* Against the FP64 oracle on the exact coefficients, on a 64^3 + 16 layered
  medium after 300 steps of dt = 0.8 ms, FP16 storage meets the accuracy bar
  of relative L2 <= 1e-3 with room to spare (the CPU emulation of the same
  encoding stays at 3.9e-4 after 1500 steps).  BF16 storage does not: its 8
  mantissa bits on the four velocity terms alone cost 4.4e-3 (all ten
  coefficients 4.7e-3); the test pins that it stays within (1e-3, 1e-2] so
  that the miss is stated, not hidden behind a loose bound.
"""
import numpy as np
import pytest

from oracle.oracle import KIND_F32, KIND_F64, Geometry, narrow_medium, rel_l2

pytestmark = pytest.mark.gpu


def narrowed(coef, fmt):
    """Coefficients as the fast kernel sees them (oracle.narrow_medium)."""
    return narrow_medium(coef, fmt)


@pytest.fixture(scope="module")
def layered_case(dc, port):
    from dc_gb300 import medium
    geom = Geometry((64, 64, 64), 16)
    spec = medium.layered_spec(7, geom.sizes)
    aniso = medium.layered_fields(spec, geom.sizes)
    coef = port.precomp(aniso)
    steps, dt = 300, 0.8e-3
    src = port.source_table(dt, steps, 60.0)
    sponge = [port.sponge_profile(s, 16, 0.35) for s in geom.sizes]
    s_idx = geom.index(geom.sizes[0] // 2, geom.sizes[1] // 2, 4 + 16 + 20)
    z64 = [np.zeros(geom.shape, np.float64) for _ in range(4)]
    f64 = port.run(KIND_F64, geom.sizes, (12.5,) * 3, dt, steps, *z64, coef=coef,
                   src_index=s_idx, src=src, sponge=sponge)
    return geom, coef, steps, dt, src, sponge, s_idx, f64


BAR = 1e-3  # relative L2 against the FP64 oracle


@pytest.mark.parametrize("fmt,medium_form", [("f16", 2), ("bf16", 3)])
def test_mixed_precision_medium(dc, port, layered_case, fmt, medium_form):
    geom, coef, steps, dt, src, sponge, s_idx, f64 = layered_case
    with dc.Simulation(geom.sizes, (12.5,) * 3, dt, kernel=dc.KERNEL_FAST, medium=medium_form,
                       device=0) as sim:
        sim.set_precomp(coef)
        sim.set_fields()
        sim.set_source(s_idx, src)
        sim.set_sponge(*sponge)
        sim.run(steps)
        sim.synchronize()
        out = sim.get_fields()
    z = [np.zeros(geom.shape, np.float32) for _ in range(4)]
    emu = port.run(KIND_F32, geom.sizes, (12.5,) * 3, dt, steps, *z, coef=narrowed(coef, fmt),
                   src_index=s_idx, src=src, sponge=sponge)
    assert rel_l2(out["pc"], emu.pc) <= 1e-5 and rel_l2(out["qc"], emu.qc) <= 1e-5
    err = rel_l2(out["pc"], f64.pc)
    print(f"{fmt}: rel L2 vs FP64 oracle after {steps} steps = {err:.3e}")
    if fmt == "f16":
        assert err <= BAR
    else:  # BF16 misses the bar (see the module docstring)
        assert BAR < err <= 1e-2


def test_mixed_precision_keeps_fp32_for_exact_kernel(dc, port, layered_case):
    """The exact kernel ignores the narrow copy and stays bit-identical."""
    geom, coef, steps, dt, src, sponge, s_idx, f64 = layered_case
    n = 40
    with dc.Simulation(geom.sizes, (12.5,) * 3, dt, kernel=dc.KERNEL_EXACT,
                       medium=dc.MEDIUM_PRECOMP_F16, device=0) as sim:
        sim.set_precomp(coef)
        sim.set_fields()
        sim.set_source(s_idx, src)
        sim.run(n)
        sim.synchronize()
        out = sim.get_fields()
    z = [np.zeros(geom.shape, np.float32) for _ in range(4)]
    ref = port.run(KIND_F32, geom.sizes, (12.5,) * 3, dt, n, *z, coef=coef, src_index=s_idx,
                   src=src)
    assert np.array_equal(out["pc"], ref.pc)


@pytest.mark.parametrize("medium_form", [0, 2, 3])
def test_tile_rows_sixteen_bit_identical(dc, layered_case, monkeypatch, medium_form):
    """DC_GB300_FAST_TY=16 (32 x 16 tiles) gives the same bits as the default
    32 x 8 tiles on the FP32, FP16 and BF16 coefficient forms."""
    geom, coef, steps, dt, src, sponge, s_idx, f64 = layered_case
    n = 60
    out = {}
    for ty in ("8", "16"):
        monkeypatch.setenv("DC_GB300_FAST_TY", ty)
        with dc.Simulation(geom.sizes, (12.5,) * 3, dt, kernel=dc.KERNEL_FAST,
                           medium=medium_form, device=0) as sim:
            sim.set_precomp(coef)
            sim.set_fields()
            sim.set_source(s_idx, src)
            sim.set_sponge(*sponge)
            sim.run(n)
            sim.synchronize()
            out[ty] = sim.get_fields()
    for k in ("pp", "pc", "qp", "qc"):
        assert np.array_equal(out["8"][k], out["16"][k]), k


@pytest.mark.parametrize("medium_form", [0, 2, 3])
def test_zchunks_bit_identical_narrow_media(dc, layered_case, monkeypatch, medium_form):
    """z-chunks on the FP32, FP16 and BF16 coefficient forms: 1, 2, 3 and 5
    chunks per column (each chunk's first output plane loads its own row
    bases and delay-ring warm-up) give the same bits as the default count."""
    geom, coef, steps, dt, src, sponge, s_idx, f64 = layered_case
    n = 40
    out = {}
    for chunks in (None, "1", "2", "3", "5"):
        if chunks is None:
            monkeypatch.delenv("DC_GB300_FAST_ZCHUNKS", raising=False)
        else:
            monkeypatch.setenv("DC_GB300_FAST_ZCHUNKS", chunks)
        with dc.Simulation(geom.sizes, (12.5,) * 3, dt, kernel=dc.KERNEL_FAST,
                           medium=medium_form, device=0) as sim:
            sim.set_precomp(coef)
            sim.set_fields()
            sim.set_source(s_idx, src)
            sim.set_sponge(*sponge)
            sim.run(n)
            sim.synchronize()
            out[chunks] = sim.get_fields()
    for chunks in ("1", "2", "3", "5"):
        for k in ("pp", "pc", "qp", "qc"):
            assert np.array_equal(out[None][k], out[chunks][k]), (chunks, k)
