"""Batched shots (dc_gb300_batch_*): boxes cropped out of one shared medium,
each with its own wavelet, sponge and receivers, advanced together by the
persistent batch kernel.

* Each shot's fields and traces are bit-identical to a single-shot
  simulation (fast kernel) over the same cropped medium, sponge, wavelet and
  receivers -- the sweep code and per-point arithmetic are shared.
* The tile shape and the z-split of the columns do not change a bit.
* Against the FP64 oracle a shot stays within the FP32 noise floor
  (rel. L2 <= 1e-5 after 70 steps).
* FP16 medium storage: within 1e-5 of the oracle run on identically encoded
  coefficients (the velocity bases are per row of the whole medium box) and
  within 1e-3 of the FP64 oracle.
* dc_gb300_batch_autotune returns one of its candidates and leaves the batch
  at step 0 with zero wavefields.
* 130 shots span several launch groups (64 shots each), and with the
  learned layer two launch chains: the shots at every group boundary match
  single-shot simulations bit for bit.
"""

import numpy as np
import pytest

from oracle.oracle import KIND_F32, KIND_F64, narrow_medium, rel_l2

pytestmark = pytest.mark.gpu

MEDIUM = (96, 88, 72)            # medium box (x, y, z)
D, DT, KAPPA, ABSORB = (12.5, 12.5, 12.5), 0.8e-3, 0.35, 8
# (sizes, origin, source, fcut): uneven boxes, x origins multiples of 4
SHOTS = [((44, 52, 40), (0, 4, 8), (20, 25, 14), 45.0),
         ((60, 40, 48), (8, 20, 0), (30, 20, 16), 60.0),
         ((37, 45, 41), (32, 12, 10), (18, 22, 12), 75.0)]
STEPS = 70                        # two 32-step graphs and 6 single steps


def receivers(sizes, src):
    sx = sizes[0]
    return [(x, src[1], 6) for x in range(5, sx - 5, 5)]


def dense_index(sizes, p):
    return p[0] + p[1] * sizes[0] + p[2] * sizes[0] * sizes[1]


def crop(a, origin, sizes):
    (ox, oy, oz), (sx, sy, sz) = origin, sizes
    return np.ascontiguousarray(a[oz:oz + sz, oy:oy + sy, ox:ox + sx])


@pytest.fixture(scope="module")
def medium_coef(dc, port):
    from dc_gb300 import medium
    spec = medium.layered_spec(11, MEDIUM)
    aniso = medium.layered_fields(spec, MEDIUM)
    return port.precomp(aniso)


def wavelet(dc, fcut, n):
    return np.array([dc.lib().dc_gb300_source(DT, i, fcut) for i in range(n)], np.float32)


def sponge(dc, sizes):
    out = []
    for s in sizes:
        g = np.empty(s, np.float32)
        dc.lib().dc_gb300_sponge_profile(s, ABSORB, KAPPA, g.ctypes.data_as(dc._fp))
        out.append(g)
    return out


def run_batch(dc, coef, steps_split=(40, 30), tiles=None, form=None, shots=SHOTS,
              persistent=True):
    form = dc.MEDIUM_PRECOMP if form is None else form
    with dc.Batch(MEDIUM, D, DT, medium=form, device=0, max_steps=STEPS + 2) as b:
        b.set_precomp(coef)
        for i, (sizes, origin, src, fcut) in enumerate(shots):
            assert b.add_shot(sizes, origin, src, fcut, ABSORB, KAPPA) == i
            b.set_receivers(i, receivers(sizes, src))
        if tiles:
            b.set_tiles(*tiles)
        b.set_grid(persistent)
        for n in steps_split:
            b.run(n)
        b.synchronize()
        assert b.steps_done == STEPS
        out = [(b.get_fields(i), b.traces(i, STEPS)) for i in range(len(shots))]
        assert b.points == sum((s[0][0] - 8) * (s[0][1] - 8) * (s[0][2] - 8) for s in shots)
        return out


@pytest.fixture(scope="module")
def batch_f32(dc, medium_coef):
    return run_batch(dc, medium_coef)


@pytest.mark.parametrize("shot", range(len(SHOTS)))
def test_batch_shot_bit_identical_to_single_simulation(dc, medium_coef, batch_f32, shot):
    sizes, origin, src, fcut = SHOTS[shot]
    coef = [crop(c, origin, sizes) for c in medium_coef]
    rec = [dense_index(sizes, r) for r in receivers(sizes, src)]
    with dc.Simulation(sizes, D, DT, kernel=dc.KERNEL_FAST, medium=dc.MEDIUM_PRECOMP,
                       device=0) as sim:
        sim.set_precomp(coef)
        sim.set_fields()
        sim.set_source(dense_index(sizes, src), wavelet(dc, fcut, STEPS + 3))
        sim.set_sponge(*sponge(dc, sizes))
        sim.set_receivers(rec, STEPS)
        sim.run(STEPS)
        sim.synchronize()
        want = sim.get_fields()
        want_tr = sim.traces(STEPS)
    got, got_tr = batch_f32[shot]
    for k in ("pp", "pc", "qp", "qc"):
        assert np.array_equal(got[k], want[k]), k
    assert np.array_equal(got_tr, want_tr)
    assert np.abs(got["pc"]).max() > 0


@pytest.mark.parametrize("persistent", [True, False])
def test_batch_tiles_do_not_change_results(dc, medium_coef, batch_f32, persistent):
    other = run_batch(dc, medium_coef, steps_split=(STEPS,), tiles=(16, 3),
                      persistent=persistent)
    for (a, ta), (b, tb) in zip(batch_f32, other):
        assert np.array_equal(a["pc"], b["pc"]) and np.array_equal(a["qc"], b["qc"])
        assert np.array_equal(ta, tb)


def test_batch_shot_against_fp64_oracle(dc, port, medium_coef, batch_f32):
    sizes, origin, src, fcut = SHOTS[0]
    coef = [crop(c, origin, sizes) for c in medium_coef]
    shape = (sizes[2], sizes[1], sizes[0])
    z = [np.zeros(shape, np.float64) for _ in range(4)]
    rec = [dense_index(sizes, r) for r in receivers(sizes, src)]
    ref = port.run(KIND_F64, sizes, D, DT, STEPS, *z, coef=coef,
                   src_index=dense_index(sizes, src), src=wavelet(dc, fcut, STEPS),
                   sponge=sponge(dc, sizes), rec=rec)
    got, tr = batch_f32[0]
    assert rel_l2(got["pc"], ref.pc) <= 1e-5
    assert rel_l2(got["qc"], ref.qc) <= 1e-5
    assert rel_l2(tr, ref.traces) <= 1e-5


def _narrow_f16(coef_box):
    """The batch's FP16 medium copy: the encoding is per row of the shared
    medium box, so it is emulated on the box and then cropped."""
    return narrow_medium(coef_box, "f16")


def test_batch_fp16_medium(dc, port, medium_coef):
    got = run_batch(dc, medium_coef, steps_split=(STEPS,), form=dc.MEDIUM_PRECOMP_F16,
                    shots=SHOTS[:1])
    sizes, origin, src, fcut = SHOTS[0]
    shape = (sizes[2], sizes[1], sizes[0])
    common = dict(src_index=dense_index(sizes, src), src=wavelet(dc, fcut, STEPS),
                  sponge=sponge(dc, sizes))
    emu_coef = [crop(c, origin, sizes) for c in _narrow_f16(medium_coef)]
    z = [np.zeros(shape, np.float32) for _ in range(4)]
    emu = port.run(KIND_F32, sizes, D, DT, STEPS, *z, coef=emu_coef, **common)
    z64 = [np.zeros(shape, np.float64) for _ in range(4)]
    f64 = port.run(KIND_F64, sizes, D, DT, STEPS, *z64,
                   coef=[crop(c, origin, sizes) for c in medium_coef], **common)
    pc = got[0][0]["pc"]
    assert rel_l2(pc, emu.pc) <= 1e-5
    err = rel_l2(pc, f64.pc)
    print(f"batched FP16 medium: rel L2 vs FP64 oracle after {STEPS} steps = {err:.3e}")
    assert err <= 1e-3


@pytest.fixture(scope="module")
def batch_f16(dc, medium_coef):
    return run_batch(dc, medium_coef, steps_split=(STEPS,), form=dc.MEDIUM_PRECOMP_F16,
                     tiles=(8, 1))


@pytest.mark.parametrize("tiles,persistent", [((16, 2), True), ((8, 3), False)])
def test_batch_fp16_tiles_do_not_change_results(dc, medium_coef, batch_f16, tiles, persistent):
    """Tile shape, z-split and grid give the same bits on the FP16 medium."""
    other = run_batch(dc, medium_coef, steps_split=(STEPS,), form=dc.MEDIUM_PRECOMP_F16,
                      tiles=tiles, persistent=persistent)
    for (a, ta), (b, tb) in zip(batch_f16, other):
        for k in ("pp", "pc", "qp", "qc"):
            assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(ta, tb)


def test_batch_rejects_bad_tile_rows(dc, medium_coef):
    with dc.Batch(MEDIUM, D, DT, device=0, max_steps=10) as b:
        with pytest.raises(dc.DcError):
            b.set_tiles(12, 1)


def test_batch_autotune(dc, medium_coef, batch_f32):
    with dc.Batch(MEDIUM, D, DT, device=0, max_steps=STEPS + 2) as b:
        b.set_precomp(medium_coef)
        for i, (sizes, origin, src, fcut) in enumerate(SHOTS):
            b.add_shot(sizes, origin, src, fcut, ABSORB, KAPPA)
            b.set_receivers(i, receivers(sizes, src))
        ty, zs, ms = b.autotune(2)
        assert ty in (8, 16) and zs in (1, 2, 4, 8) and ms > 0
        assert b.tiles() == (ty, zs) and b.steps_done == 0
        assert not np.any(b.get_fields(1)["pc"])
        b.run(STEPS)
        b.synchronize()
        for i in range(len(SHOTS)):
            assert np.array_equal(b.get_fields(i)["pc"], batch_f32[i][0]["pc"])
            assert np.array_equal(b.traces(i, STEPS), batch_f32[i][1])


def test_batch_rejects_bad_shots(dc, medium_coef):
    with dc.Batch(MEDIUM, D, DT, device=0, max_steps=10) as b:
        with pytest.raises(dc.DcError):
            b.add_shot((40, 40, 40), (2, 0, 0), (20, 20, 20))    # ox not a multiple of 4
        with pytest.raises(dc.DcError):
            b.add_shot((40, 40, 40), (60, 0, 0), (20, 20, 20))   # outside the medium
        with pytest.raises(dc.DcError):
            b.add_shot((40, 40, 40), (0, 0, 0), (2, 20, 20))     # source in the halo
        with pytest.raises(dc.DcError):
            b.run(1)                                             # no medium, no shots


def test_batch_learned_layer_matches_single_simulation(dc, medium_coef):
    """The learned thin layer applied to every shot of a batch gives each
    shot exactly what a single-shot simulation with the same layer gives."""
    from dc_gb300 import learned
    layer = 8
    params = np.load(learned.WEIGHTS)
    shots = SHOTS[:2]
    with dc.MLP(device=0, params=params) as mlp:
        with dc.Batch(MEDIUM, D, DT, device=0, max_steps=STEPS + 2) as b:
            b.set_precomp(medium_coef)
            for sizes, origin, src, fcut in shots:
                b.add_shot(sizes, origin, src, fcut, 0, 0.0)
            b.set_learned_layer(mlp, layer)
            with pytest.raises(dc.DcError):
                b.add_shot(*shots[0][:4])  # shots first, then the layer
            b.run(STEPS)
            b.synchronize()
            got = [b.get_fields(i) for i in range(len(shots))]
        for (sizes, origin, src, fcut), g in zip(shots, got):
            with dc.Simulation(sizes, D, DT, kernel=dc.KERNEL_FAST, device=0) as sim:
                sim.set_precomp([crop(c, origin, sizes) for c in medium_coef])
                sim.set_fields()
                sim.set_source(dense_index(sizes, src), wavelet(dc, fcut, STEPS + 3))
                dc.set_learned_layer(sim, mlp, layer)
                sim.run(STEPS)
                sim.synchronize()
                want = sim.get_fields()
            assert np.array_equal(g["pc"], want["pc"]) and np.array_equal(g["qc"], want["qc"])
            assert np.abs(g["pc"]).max() > 0


def test_batch_many_shots_span_launch_groups(dc, medium_coef):
    """130 small shots: the kernel parameters hold 64 shots per launch, and
    with the learned layer the batch runs as two launch chains of 65 shots
    (groups of 64 + 1 each).  The shots at every group boundary match a
    single-shot simulation bit for bit, with and without the layer."""
    from dc_gb300 import learned
    layer, steps, n = 8, 40, 130
    rng = np.random.default_rng(77)
    shots = []
    for _ in range(n):
        sizes = (32, 32, 32)
        origin = (4 * int(rng.integers(0, (MEDIUM[0] - 32) // 4 + 1)),
                  int(rng.integers(0, MEDIUM[1] - 32 + 1)), int(rng.integers(0, MEDIUM[2] - 32 + 1)))
        src = (16, 16, 14)
        shots.append((sizes, origin, src, 50.0))
    check = [0, 63, 64, 65, 128, 129]
    params = np.load(learned.WEIGHTS)
    with dc.MLP(device=0, params=params) as mlp:
        for with_layer in (False, True):
            with dc.Batch(MEDIUM, D, DT, device=0, max_steps=steps + 2) as b:
                b.set_precomp(medium_coef)
                for sizes, origin, src, fcut in shots:
                    b.add_shot(sizes, origin, src, fcut, 0 if with_layer else ABSORB,
                               0.0 if with_layer else KAPPA)
                if with_layer:
                    b.set_learned_layer(mlp, layer)
                b.run(steps)
                b.synchronize()
                got = {i: b.get_fields(i) for i in check}
            for i in check:
                sizes, origin, src, fcut = shots[i]
                with dc.Simulation(sizes, D, DT, kernel=dc.KERNEL_FAST, device=0) as sim:
                    sim.set_precomp([crop(c, origin, sizes) for c in medium_coef])
                    sim.set_fields()
                    sim.set_source(dense_index(sizes, src), wavelet(dc, fcut, steps + 3))
                    if with_layer:
                        dc.set_learned_layer(sim, mlp, layer)
                    else:
                        sim.set_sponge(*sponge(dc, sizes))
                    sim.run(steps)
                    sim.synchronize()
                    want = sim.get_fields()
                for k in ("pc", "qc", "pp", "qp"):
                    assert np.array_equal(got[i][k], want[k]), (with_layer, i, k)
                assert np.abs(got[i]["pc"]).max() > 0
