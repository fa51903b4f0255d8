"""The command-line driver (distributed-cube-average_gb300/cli/dc_gb300_main.c):
the reference's options, iteration rule, output file format and timing
lines (src/main.c, src/coordinator.c:116-219), plus checkpoint / resume."""
import math
import subprocess

import numpy as np
import pytest

from oracle.oracle import KIND_F32, Geometry, reference_medium, rel_l2


def cli(dc, *args, check=True):
    exe = dc.PKG_DIR / "dc_gb300"
    assert exe.exists(), "CLI not built"
    return subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True,
                          check=check)


BASE = ["--dx", "12.5", "--dy", "12.5", "--dz", "12.5"]


@pytest.mark.parametrize("tmax,dt", [(1e-3, 1e-6), (0.5, 1e-3), (0.03, 1e-3), (1.6, 8e-4),
                                      (0.1, 3e-4)])
def test_iteration_count_rule(dc, tmax, dt):
    """src/main.c:132: ceil of the float quotient (1e-3 / 1e-6 -> 1001)."""
    out = cli(dc, "--size-x", 8, "--size-y", 8, "--size-z", 8, *BASE, "--dt", dt, "-t", tmax,
              "-a", 2, "--print-iterations")
    expected = math.ceil(float(np.float32(tmax) / np.float32(dt)))
    assert int(out.stdout.strip()) == expected
    if (tmax, dt) == (1e-3, 1e-6):
        assert expected == 1001


def test_required_options(dc):
    r = cli(dc, "--size-x", 8, "--size-y", 8, "--size-z", 8, *BASE, "--dt", 1e-3, "-t", 0.01,
            "-a", 2, check=False)  # no --output-file
    assert r.returncode != 0
    assert "Usage" in r.stderr or "usage" in r.stderr.lower()


def oracle_run(port, n, absorb, steps, dt, sponge=None):
    geom = Geometry(n, absorb)
    aniso, coef = reference_medium(port, geom)
    src = port.source_table(dt, steps)
    z = [np.zeros(geom.shape, np.float32) for _ in range(4)]
    sp = None
    if sponge is not None:
        sp = [port.sponge_profile(s, absorb, sponge) for s in geom.sizes]
    res = port.run(KIND_F32, geom.sizes, (12.5,) * 3, dt, steps, *z, coef=coef,
                   src_index=geom.source_index, src=src, sponge=sp)
    return geom, res


def read_output(path, geom):
    data = np.fromfile(path, np.float32)
    n = geom.count
    assert data.size == 2 * n
    return data[:n].reshape(geom.shape), data[n:].reshape(geom.shape)


@pytest.mark.gpu
@pytest.mark.parametrize("loop", ["graph", "abi"])
def test_cli_output_matches_oracle(dc, port, tmp_path, loop):
    n, absorb, dt, tmax = (10, 9, 8), 3, 1e-3, 0.04
    steps = math.ceil(float(np.float32(tmax) / np.float32(dt)))
    out = tmp_path / "out.dc"
    r = cli(dc, "--size-x", n[0], "--size-y", n[1], "--size-z", n[2], *BASE, "--dt", dt,
            "-t", tmax, "-a", absorb, "-o", out, "--kernel", "exact", "--loop", loop)
    lines = r.stdout.strip().splitlines()
    assert lines[0] == "rank,total_time,msamples_per_s"
    assert lines[1].startswith("0,") and lines[2].startswith("*,")
    geom, ref = oracle_run(port, n, absorb, steps, dt)
    pc, qc = read_output(out, geom)
    sx, sy, sz = geom.sizes
    halo = np.ones(geom.shape, bool)
    halo[4:sz - 4, 4:sy - 4, 4:sx - 4] = False
    assert not pc[halo].any() and not qc[halo].any()
    assert np.array_equal(pc, ref.pc) and np.array_equal(qc, ref.qc)


@pytest.mark.gpu
def test_cli_fast_kernel_and_sponge(dc, port, tmp_path):
    n, absorb, dt, tmax = (12, 10, 9), 4, 1e-3, 0.05
    steps = math.ceil(float(np.float32(tmax) / np.float32(dt)))
    out = tmp_path / "out.dc"
    cli(dc, "--size-x", n[0], "--size-y", n[1], "--size-z", n[2], *BASE, "--dt", dt,
        "-t", tmax, "-a", absorb, "-o", out, "--boundary", "sponge", "--sponge-kappa", 0.4)
    geom, ref = oracle_run(port, n, absorb, steps, dt, sponge=0.4)
    pc, qc = read_output(out, geom)
    assert rel_l2(pc, ref.pc) <= 1e-5 and rel_l2(qc, ref.qc) <= 1e-5


@pytest.mark.gpu
def test_cli_checkpoint_resume_bit_identical(dc, tmp_path):
    n, absorb, dt = (11, 9, 10), 3, 1e-3
    args = ["--size-x", n[0], "--size-y", n[1], "--size-z", n[2], *BASE, "--dt", dt,
            "-t", 1.0, "-a", absorb]
    straight, first, resumed = tmp_path / "s.dc", tmp_path / "f.dc", tmp_path / "r.dc"
    ck = tmp_path / "state.ckpt"
    cli(dc, *args, "--steps", 70, "-o", straight)
    cli(dc, *args, "--steps", 33, "-o", first, "--checkpoint", ck)
    cli(dc, *args, "--steps", 70, "-o", resumed, "--resume", ck)
    assert np.array_equal(np.fromfile(straight, np.float32), np.fromfile(resumed, np.float32))
    assert not np.array_equal(np.fromfile(first, np.float32), np.fromfile(resumed, np.float32))


@pytest.mark.gpu
def test_checkpoint_api_roundtrip(dc, port, tmp_path):
    geom = Geometry((14, 12, 10), 3)
    aniso, coef = reference_medium(port, geom)
    src = port.source_table(1e-3, 200)
    ck = tmp_path / "c.ckpt"
    with dc.Simulation(geom.sizes, (12.5,) * 3, 1e-3, device=0) as a:
        a.set_precomp(coef)
        a.set_fields()
        a.set_source(geom.source_index, src)
        a.run(77)
        a.save_checkpoint(ck)
        a.run(66)
        a.synchronize()
        want = a.get_fields()
    with dc.Simulation(geom.sizes, (12.5,) * 3, 1e-3, device=0) as b:
        b.set_precomp(coef)
        b.set_fields()
        b.set_source(geom.source_index, src)
        b.load_checkpoint(ck)
        assert b.steps_done == 77
        b.run(66)
        b.synchronize()
        got = b.get_fields()
    for k in want:
        assert np.array_equal(want[k], got[k]), k
    with dc.Simulation((16, 16, 16), (12.5,) * 3, 1e-3, device=0) as c:
        with pytest.raises(dc.DcError):
            c.load_checkpoint(ck)  # other sizes


@pytest.mark.gpu
def test_cli_learned_boundary(dc, port, tmp_path):
    """--boundary learned: the default medium (no random velocity boundary)
    with the committed network on an 8-cell layer gives exactly what a
    simulation with the same layer gives; a bad weights file is refused."""
    from dc_gb300 import learned
    n, absorb, dt, steps = (20, 18, 16), 8, 1e-3, 60
    out = tmp_path / "out.dc"
    args = ["--size-x", n[0], "--size-y", n[1], "--size-z", n[2], *BASE, "--dt", dt,
            "-t", 1.0, "-a", absorb, "--steps", steps, "--boundary", "learned"]
    cli(dc, *args, "-o", out)
    geom = Geometry(n, absorb)
    coef = port.precomp(port.default_anisotropy(geom.shape))
    with dc.MLP(device=0, params=np.load(learned.WEIGHTS)) as mlp:
        with dc.Simulation(geom.sizes, (12.5,) * 3, dt, kernel=dc.KERNEL_FAST, device=0) as sim:
            sim.set_precomp(coef)
            sim.set_fields()
            sim.set_source(geom.source_index, dc.source_table(dt, steps + 1, 40.0))
            dc.set_learned_layer(sim, mlp, absorb)
            sim.run(steps)
            sim.synchronize()
            want = sim.get_fields()
    pc, qc = read_output(out, geom)
    assert np.array_equal(pc, want["pc"]) and np.array_equal(qc, want["qc"])
    bad = tmp_path / "bad.npy"
    np.save(bad, np.zeros(10, np.float32))
    r = cli(dc, *args, "-o", tmp_path / "x.dc", "--learned-weights", bad, check=False)
    assert r.returncode != 0 and "weights" in r.stderr
