"""Benchmark of the Fletcher TTI time step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--form plain|batched] [--medium f32|f16|bf16]

Plain workload: 512^3 interior + 48-cell absorbing shell
(616^3 padded, 608^3 = 224.8 M updated points per step), dt = 0.8 ms,
dx = dy = dz = 12.5 m, seeded 12-layer medium (numpy PCG64 seed 2026) on the
GPU, 20 Hz Ricker (FCUT = 60) at interior depth 20, 48-cell sponge.  A step
is one time step of the whole cube; K = 2000 steps is the config's length.
The working set (14 x 0.93 GB) is far larger than the 129 MB L2, so no L2
flush is needed between steps.

Metric: point-updates per second (compute region x steps / time), the
reference's MSamples/s divided by 1000 (reference src/main.c:207-214).

Our arm: ``value`` is the device-resident rate (graph-replayed steps, CUDA
events on the library's stream); ``e2e`` is the same rate through the
reference-facing C ABI with host buffers (dc_device_data_init with the
copies, dc_device_add_source + dc_propagate + dc_device_swap_arrays per
step, dc_device_data_get_results), wall clock.  ``roofline`` compares the
stencil kernel's algorithmic bytes (64 B per update) per launch time with the
measured HBM copy bandwidth; ``cpu_baseline`` times the reference's own
OpenMP path (built from its sources with its own flags) on a bounded y-slab
of the same workload.

Batched form (--form batched): 64 shots over one shared seeded medium of
768 x 768 x 512 cells (plus a 52-cell margin per side for the shots'
absorbing layers and halos: an 872 x 872 x 616 medium box), each shot a
crop of U(192, 320) x U(192, 320) x 256 interior cells around its source
(sources on an 8 x 8 surface grid with seeded jitter, depth 20, Ricker peak
U(15, 25) Hz), a 48-cell sponge per shot, FP16 medium storage, 64 receivers
per shot; tile rows, z-split and grid (persistent CTAs or one CTA per tile)
chosen by the library's autotuner.  One step advances every shot (one
launch); K defaults to 1000 steps.
``value`` is shot-point-updates per second summed over the shots.

Learned form (--form learned): a 384^3 interior with the 8-cell learned
absorbing layer (network weights from the package's data/learned_layer8.npy,
trained by dc_gb300.learned.main) against the same interior with the
48-cell sponge, K = 1500 steps, FP32, the same seeded medium generator.
``value`` is interior point-updates per second of the learned form; the
line also carries the sponge form's rate and the reflected energy of both
in a 32-cell band next to the interior's boundary against a wide run whose
reflections never return (sampled every 100 steps).

Mixed-precision form (--form mixed): 1024 x 1024 x 768 interior + 48-cell
sponge (1.084 G updated points per step), FP16 coefficient storage (BF16
with --medium bf16), FP32 arithmetic and wavefields, K = 1500 steps.

Best form (--form best): the batched workload's 64 crops with the 8-cell
learned layer instead of the 48-cell sponge and FP16 medium storage, against
the plain form (FP32, 48-cell sponge, one shot at a time through
dc_gb300_run) timed on every shot of the same layout (at most 100 steps
each: its step cost does not change).  ``value`` is
interior shot-point-updates per second (crop points x steps / time) of the
best form; the line carries the plain form's rate and the ratio.

Reference-CUDA form (--form refcuda): the reference's own GPU path
(src/cuda_propagate.cu, src/device_data.cu, nvcc sm_103a) against ours on
the same GPU and inputs (the reference's default medium and random velocity
boundary on the plain workload's geometry).

Reference arm (--impl reference): the reference's CPU implementation of the
path (src/openmp_propagate.c built with the reference's flags, all host
threads; the oracle port only where the reference's sources are absent) on
the same workload; each step is one time step of a 608 x 16 x 608 y-slab.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "TTI Gpoint-updates/s & %HBM roofline: plain vs mixed/batched/learned at stated L2"
UNIT = "Gpoint-updates/s"
N_INTERIOR, ABSORB = 512, 48
DT, DX = 0.8e-3, 12.5
FCUT = 60.0           # Ricker peak fcut/3 = 20 Hz
SRC_DEPTH = 20        # interior-relative depth of the source (cells)
MEDIUM_SEED = 2026
SPONGE_KAPPA = 0.35
BYTES_PER_UPDATE = 64  # pc,qc,pp,qp + 10 coefficients read, pp,qp written
SLAB_ROWS = 16         # CPU sample: updated y rows per step
# batched form
BATCH_MODEL = (768, 768, 512)
BATCH_PAD = ABSORB + 4  # sponge + halo around every crop
BATCH_SHOTS = 64
BATCH_DEPTH = 256
BATCH_SEED = 2027
BATCH_RECEIVERS = 64
# learned form
LEARNED_N, LEARNED_LAYER = 384, 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 2000 plain, 1000 batched)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--kernel", choices=("fast", "exact"), default="fast")
    ap.add_argument("--medium", choices=("f32", "f16", "bf16"), default="f32",
                    help="coefficient storage read by the fast kernel")
    ap.add_argument("--n", type=int, default=N_INTERIOR, help="interior cells per axis")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", choices=("plain", "mixed", "batched", "learned", "best",
                                       "refcuda"),
                    default="plain")
    ap.add_argument("--shots", type=int, default=BATCH_SHOTS)
    ap.add_argument("--model", type=int, nargs=3, default=list(BATCH_MODEL),
                    help="batched form: model sizes (x y z); smaller for profiling captures")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched form: keep the default tiles (profiling captures)")
    ap.add_argument("--learned-n", type=int, default=LEARNED_N,
                    help="learned form: interior cells per axis")
    ap.add_argument("--no-judge", action="store_true",
                    help="learned form: skip the reflected-energy judge")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="mixed/batched/best forms: skip the FP64-oracle accuracy check")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"batched": 1000, "learned": 1500, "best": 1000,
                      "mixed": 1500, "refcuda": 20}.get(args.form, 2000)
    if args.form == "mixed":
        # the mixed-precision workload: 1024 x 1024 x 768 interior + 48-cell
        # sponge, FP16 medium unless another storage is asked for
        args.nxyz = (1024, 1024, 768)
        if args.medium == "f32":
            args.medium = "f16"
        args.no_e2e = True
    else:
        args.nxyz = (args.n,) * 3
    return args


def max_over_ranks(v: float, dist, device: str) -> float:
    """Largest value over the ranks (the slowest rank's time); v itself when
    running alone."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_rate(points_per_step: int, steps: int, world: int, ms: float) -> float:
    """Whole-job rate in G updates/s: every one of the `world` ranks updated
    points_per_step points `steps` times in `ms` (the max over ranks)."""
    return points_per_step * steps * world / (ms * 1e-3) / 1e9


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(name: str):
    """DRAM bytes per point-update of the stencil kernel from the committed
    ncu summary (a line 'traffic_bytes_per_update: X'), or None."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_update:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def geometry(n):
    from dc_gb300.medium import Geometry
    return Geometry(tuple(n) if isinstance(n, (tuple, list)) else (n, n, n), ABSORB)


def shot_source(geom, rank: int) -> int:
    """Rank r runs shot r: sources step along x from the centre (weak scaling:
    one independent shot per GPU, shared medium, no exchange)."""
    sx, sy, _ = geom.sizes
    o = 4 + geom.absorb
    x = sx // 2 + (rank * 16) % max(1, geom.n[0] // 2)
    return geom.index(x, sy // 2, o + SRC_DEPTH)


def make_spec(geom):
    from dc_gb300 import medium
    return medium.layered_spec(MEDIUM_SEED, geom.sizes)


def slab_inputs(dc, port, geom, rows: int):
    """Host inputs of a CPU sample: a y-slab of the workload (full x and z
    extent, `rows` updated rows through the cube's centre) with its medium
    precomputed like the reference (src/precomp.c:85-105).  A y-slab keeps
    the reference's OpenMP loop, which is parallel over z
    (src/openmp_propagate.c:14-16), as parallel as on the whole cube."""
    from dc_gb300 import medium
    sx, sy, sz = geom.sizes
    y0 = sy // 2 - rows // 2 - 4
    spec = medium.with_origin(make_spec(geom), (0, y0, 0))
    sizes = (sx, rows + 8, sz)
    aniso = medium.layered_fields(spec, sizes)
    coef = port.precomp(aniso)
    rng = np.random.Generator(np.random.PCG64(1))
    shape = (sz, sizes[1], sx)
    fields = [(rng.standard_normal(shape) * 1e-3).astype(np.float32) for _ in range(4)]
    return sizes, coef, fields


def time_cpu_oracle(port, sizes, coef, fields, target_s: float, nthreads: int):
    """Repeated oracle-port steps over the slab until ~target_s; returns
    (updates/s, steps, seconds).  Used only where the reference's sources
    are absent."""
    from oracle.oracle import KIND_F32
    sx, sy, sz = sizes
    pc, qc, pp, qp = fields
    b0, b1 = (4, 4, 4), (sx - 4, sy - 4, sz - 4)
    pts = (sx - 8) * (sy - 8) * (sz - 8)
    t0 = time.perf_counter()
    port.step(KIND_F32, sizes, b0, b1, (DX,) * 3, DT, pc, qc, pp, qp, coef=coef, nthreads=nthreads)
    one = time.perf_counter() - t0
    reps = max(1, int(target_s / max(one, 1e-6)))
    t0 = time.perf_counter()
    for _ in range(reps):
        port.step(KIND_F32, sizes, b0, b1, (DX,) * 3, DT, pc, qc, pp, qp, coef=coef,
                  nthreads=nthreads)
    el = time.perf_counter() - t0
    return pts * reps / el, reps, el


def cpu_reference():
    """The reference's own OpenMP path built with its own flags
    (oracle/_ref/librefomp.so: src/openmp_propagate.c, -O3 -fopenmp), or
    None where its sources are absent."""
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    from oracle.oracle import Reference
    try:
        return Reference("native")
    except FileNotFoundError:
        return None


def cpu_baseline_slab(dc, geom, steps=None, target_s=12.0, warmup=1):
    """CPU baseline on a y-slab of the workload (SLAB_ROWS updated rows, full
    x and z extent): the reference's own OpenMP path through its one-rank
    loop (kind "reference"), or the oracle port where the reference's
    sources are absent (kind "port").  `steps` timed steps, or as many as
    fill ~target_s.  Returns (updates/s, info dict)."""
    from oracle.oracle import Port
    port = Port()
    ssizes, coef, fields = slab_inputs(dc, port, geom, SLAB_ROWS)
    sx, sy, sz = ssizes
    pts = (sx - 8) * (sy - 8) * (sz - 8)
    ref = cpu_reference()
    if ref is None:
        nthreads = os.cpu_count() or 1
        rate, reps, el = time_cpu_oracle(port, ssizes, coef, fields, target_s, nthreads)
        return rate, {"kind": "port", "cores": nthreads, "steps": reps, "seconds": el,
                      "what": "oracle port of src/openmp_propagate.c"}
    shape = fields[0].shape
    if warmup:
        z = [np.zeros(shape, np.float32) for _ in range(4)]
        ref.run(0, ssizes, (DX,) * 3, DT, warmup, *z, coef=coef)
    if steps is None:
        z = [np.zeros(shape, np.float32) for _ in range(4)]
        _, _, one = ref.run(0, ssizes, (DX,) * 3, DT, 1, *z, coef=coef, timed=True)
        steps = max(1, int(target_s / max(one, 1e-6)))
    z = list(fields)
    _, _, el = ref.run(0, ssizes, (DX,) * 3, DT, steps, *z, coef=coef, timed=True)
    return pts * steps / el, {"kind": "reference", "cores": ref.threads(), "steps": steps,
                              "seconds": el,
                              "what": "the reference's src/openmp_propagate.c built with its "
                                      "own flags (-O3 -fopenmp), its one-rank loop"}


# ---------------------------------------------------------------------------
# Accuracy against the FP64 CPU oracle (outside every timed region)
ACC_CROP_N = 160      # the mixed form's check: 160^3 interior + 48-cell sponge = 256^3 updated


def receiver_grid(sizes, pad: int, n_xy, nx: int = 32, ny: int = 16, depth: int = 8):
    """nx x ny receivers spread over the interior's x-y extent at interior
    depth `depth` (global z = pad + depth); linear indices."""
    sx, sy, _ = sizes
    xs = np.linspace(pad, pad + n_xy[0] - 1, nx).round().astype(np.int64)
    ys = np.linspace(pad, pad + n_xy[1] - 1, ny).round().astype(np.int64)
    z = pad + depth
    return np.array([x + y * sx + z * sx * sy for y in ys for x in xs], np.int64)


def oracle_f64(sizes, coef, steps, src_idx, src, sponge, rec):
    """The FP64 CPU oracle (oracle/dc_oracle.c, double precision, cross
    terms in separable form) over `steps` steps from zero fields."""
    from oracle.oracle import KIND_F64_SEP, Port
    port = Port()
    shape = (sizes[2], sizes[1], sizes[0])
    z = [np.zeros(shape, np.float64) for _ in range(4)]
    t0 = time.perf_counter()
    r = port.run(KIND_F64_SEP, sizes, (DX,) * 3, DT, steps, *z, coef=coef, src_index=src_idx,
                 src=src, sponge=sponge, rec=rec)
    return r, time.perf_counter() - t0


def rel(a, b) -> float:
    from oracle.oracle import rel_l2
    return rel_l2(a, b)


def gpu_box_run(dc, sizes, spec, form, steps, src_idx, src, sponge, rec, local):
    """One GPU run of a box of the seeded medium with the given coefficient
    storage; returns (pc, qc, traces, FP32 coefficients)."""
    sim = dc.Simulation(sizes, (DX,) * 3, DT, kernel=dc.KERNEL_FAST, medium=form, device=local)
    sim.generate_layered(spec)
    sim.set_fields()
    sim.set_source(src_idx, src)
    if sponge is not None:
        sim.set_sponge(*sponge)
    sim.set_receivers(rec, steps)
    sim.run(steps)
    sim.synchronize()
    f = sim.get_fields()
    tr = sim.traces(steps)
    coef = sim.get_precomp()
    sim.close()
    return f["pc"], f["qc"], tr, coef


def mixed_accuracy(dc, big_geom, form, storage: str, steps: int, local: int):
    """The mixed form's error on its own workload: a 256^3 crop of the
    1024 x 1024 x 768 run (160^3 interior + the 48-cell sponge, the same
    medium origin, source depth and number of steps, centred on the source
    horizontally) run as its own box in the narrow storage and in FP32,
    both against the FP64 CPU oracle on the same box; wavefield and a
    32 x 16 = 512-receiver grid at interior depth 8."""
    from dc_gb300 import medium
    crop = geometry(ACC_CROP_N)
    sizes = crop.sizes
    bsx, bsy, _ = big_geom.sizes
    origin = (bsx // 2 - sizes[0] // 2, bsy // 2 - sizes[1] // 2, 0)
    spec = medium.with_origin(make_spec(big_geom), origin)
    o = 4 + ABSORB
    src_idx = crop.index(sizes[0] // 2, sizes[1] // 2, o + SRC_DEPTH)
    src = dc.source_table(DT, steps + 1, FCUT)
    sponge = [dc.sponge_profile(v, ABSORB, SPONGE_KAPPA) for v in sizes]
    rec = receiver_grid(sizes, o, crop.n[:2])
    pc, qc, tr, coef = gpu_box_run(dc, sizes, spec, form, steps, src_idx, src, sponge, rec, local)
    pc32, qc32, tr32, _ = gpu_box_run(dc, sizes, spec, dc.MEDIUM_PRECOMP, steps, src_idx, src,
                                      sponge, rec, local)
    f64, osec = oracle_f64(sizes, coef, steps, src_idx, src, sponge, rec)
    return {"check": f"FP64 CPU oracle on a {sizes[0] - 8}^3 crop ({ACC_CROP_N}^3 interior + "
                     f"{ABSORB}-cell sponge) of the same run, origin {origin}, {steps} steps, "
                     f"{rec.size} receivers", "storage": storage,
            "rel_l2_p": rel(pc, f64.pc), "rel_l2_q": rel(qc, f64.qc),
            "rel_l2_traces": rel(tr, f64.traces),
            "fp32_rel_l2_p": rel(pc32, f64.pc), "fp32_rel_l2_traces": rel(tr32, f64.traces),
            "bar": 1e-3, "meets_bar": bool(rel(pc, f64.pc) <= 1e-3 and rel(tr, f64.traces) <= 1e-3),
            "oracle_seconds": osec}


def shot_coef(dc, spec_box, shot, local):
    """FP32 coefficients of a shot's crop of the shared medium (the values
    the batch reads at the crop: the medium is evaluated per point at global
    coordinates)."""
    from dc_gb300 import medium
    sim = dc.Simulation(shot["sizes"], (DX,) * 3, DT, kernel=dc.KERNEL_FAST, device=local)
    sim.generate_layered(medium.with_origin(spec_box, shot["origin"]))
    coef = sim.get_precomp()
    sim.close()
    return coef


def shot_index(sizes, xyz) -> int:
    sx, sy, _ = sizes
    return int(xyz[0] + xyz[1] * sx + xyz[2] * sx * sy)


# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    """Reference arm: the reference's own CPU implementation of the path on
    the host cores (its OpenMP backend, built from its sources with its own
    flags), one time step of a y-slab of the workload per timed step."""
    if rank != 0:
        return
    import __graft_entry__ as ge
    dc = ge.package()
    geom = geometry(args.n)
    rate, info = cpu_baseline_slab(dc, geom, steps=args.steps, warmup=args.warmup)
    value = rate / 1e9
    sx, sz = geom.sizes[0] - 8, geom.sizes[2] - 8
    sample = (f"{info['steps']} steps of the {sx}x{SLAB_ROWS}x{sz} updated slab (full x and z "
              f"extent of the {geom.sizes[0]}^3 cube, {SLAB_ROWS} rows through its centre), "
              f"{info['seconds']:.1f} s; {info['what']}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": info["seconds"] / info["steps"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered medium, numpy PCG64 seed 2026)",
        "config": {"workload": f"plain FP32 TTI, {args.n}^3 interior + {ABSORB} absorbing, "
                               f"y-slab sample of {SLAB_ROWS} rows", "global_batch": 1,
                   "seq_len": None, "parallelism": "cpu", "threads": info["cores"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"],
                         "kind": info["kind"], "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local):
    import torch
    import __graft_entry__ as ge
    dc = ge.package()
    dc.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_ms(v: float) -> float:
        return max_over_ranks(v, dist, "cuda")

    geom = geometry(args.nxyz)
    sizes = geom.sizes
    pts = geom.compute_points
    kernel = dc.KERNEL_FAST if args.kernel == "fast" else dc.KERNEL_EXACT
    total_steps = args.warmup + args.steps
    src_amp = dc.source_table(DT, total_steps + 1, FCUT)
    src_idx = shot_source(geom, rank)
    sponge = [dc.sponge_profile(s, geom.absorb, SPONGE_KAPPA) for s in sizes]

    # ---- device-resident run (value, roofline) -------------------------
    medium_form = {"f32": dc.MEDIUM_PRECOMP, "f16": dc.MEDIUM_PRECOMP_F16,
                   "bf16": dc.MEDIUM_PRECOMP_BF16}[args.medium]
    bytes_per_update = BYTES_PER_UPDATE if args.medium == "f32" else 44
    sim = dc.Simulation(sizes, (DX,) * 3, DT, kernel=kernel, medium=medium_form,
                        device=local)
    sim.generate_layered(make_spec(geom))
    sim.set_fields()
    sim.set_source(src_idx, src_amp)
    sim.set_sponge(*sponge)
    sim.run(args.warmup)
    sim.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = sim.launches
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        sim.run(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    sim.synchronize()
    launches = sim.launches - l0
    ms = ev0.elapsed_time(ev1)
    ms = max_ms(ms)
    barrier()
    value = weak_rate(pts, args.steps, world, ms)
    stencil_ms = ms / args.steps  # graph-replayed region: one stencil launch per step
    achieved = bytes_per_update * pts / (stencil_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic_pp = (profiled_traffic("tti_fast_config2.md")
                  if kernel == dc.KERNEL_FAST and args.n == N_INTERIOR and args.medium == "f32"
                  else None)
    sim.close()

    # ---- the mixed form's error against the FP64 CPU oracle ---------------
    accuracy = None
    if args.form == "mixed" and rank == 0 and not args.no_accuracy:
        accuracy = mixed_accuracy(dc, geom, medium_form, args.medium, args.steps, local)

    # ---- end to end through the reference ABI with host buffers ----------
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(dc, torch, geom, args, src_idx, kernel, local, barrier, max_ms, world)

    # ---- CPU baseline: the reference's OpenMP path on a slab (rank 0, N = 1)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, info = cpu_baseline_slab(dc, geom)
        cpu = {"value": rate / 1e9, "unit": UNIT, "cores": info["cores"], "kind": info["kind"],
               "sample": f"{info['steps']} steps of a {geom.sizes[0] - 8}x{SLAB_ROWS}x"
                         f"{geom.sizes[2] - 8} y-slab of the same workload "
                         f"({info['seconds']:.1f} s); {info['what']}"}

    if rank != 0:
        return
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 12-layer TTI medium, numpy PCG64 seed 2026, generated on GPU)",
        "config": {"workload": (f"plain FP32 TTI, {args.n}^3 interior + {ABSORB}-cell sponge, "
                                f"{geom.sizes[0]}^3 padded, dt 0.8 ms, 20 Hz Ricker")
                   if args.form == "plain" else
                   (f"mixed precision: {'x'.join(map(str, args.nxyz))} interior + "
                    f"{ABSORB}-cell sponge, {args.medium.upper()} medium storage, FP32 math "
                    f"and wavefields, dt 0.8 ms, 20 Hz Ricker; rel. L2 vs the FP64 oracle "
                    f"in config.accuracy"),
                   "form": args.form,
                   "kernel": args.kernel, "medium_storage": args.medium,
                   "points_per_step": pts, "global_batch": world,
                   "seq_len": None, "parallelism": f"shots{world}" if world > 1 else "single",
                   "l2": "inputs 13 GB >> 129 MB L2; no flush", "accuracy": accuracy},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "bytes_per_update": bytes_per_update,
                     "traffic": (traffic_pp * pts) if traffic_pp else None},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_e2e(dc, torch, geom, args, src_idx, kernel, local, barrier, max_ms, world):
    """Same workload through the reference's entry points with host
    buffers: the medium comes from pinned host arrays, the loop is
    src/worker.c's (source, propagate, swap), results come back to the
    host.  Wall clock around everything, after one untimed warm-up pass of
    the same loop."""
    sizes = geom.sizes
    sx, sy, sz = sizes
    shape = (sz, sy, sx)
    pts = geom.compute_points

    def pinned(n_floats):
        t = torch.empty(n_floats, dtype=torch.float32, pin_memory=True)
        return t, t.numpy()

    # build the host medium once (outside the timed region): generate on the
    # GPU, copy to pinned host memory
    n = sx * sy * sz
    keep = []
    coef_host = []
    for _ in dc.COEF_NAMES:
        t, a = pinned(n)
        keep.append(t)
        coef_host.append(a.reshape(shape))
    gen = dc.Simulation(sizes, (DX,) * 3, DT, kernel=kernel, device=local)
    gen.generate_layered(make_spec(geom))
    gen.get_precomp(coef_host)
    gen.close()
    fields = []
    for _ in range(4):
        t, a = pinned(n)
        a[:] = 0.0
        keep.append(t)
        fields.append(a.reshape(shape))
    os.environ["DC_GB300_KERNEL"] = args.kernel
    os.environ["DC_GB300_DEVICE"] = str(local)
    proc = dc.Process(sizes, (DX,) * 3, DT, pp=None, pc=None, qp=None, qc=None,
                      precomp=coef_host, source_index=src_idx)
    # Process copies its field arrays; point pc/qc at pinned outputs instead
    for name, arr in zip(("pp", "pc", "qp", "qc"), fields):
        proc._keep[name] = arr
        setattr(proc.proc, name, dc.fptr(arr))
    amp = [dc.source(DT, i, FCUT) for i in range(max(args.steps, args.warmup) + 1)]
    b0 = (4, 4, 4)
    b1 = (sx - 4, sy - 4, sz - 4)

    marks = {}

    def abi_run(steps):
        data = dc.device_data_init(proc)  # returns once the arrays are on the device
        marks["init"] = time.perf_counter()
        for it in range(steps):
            dc.device_add_source(data, src_idx, amp[it])
            dc.propagate(b0, b1, sizes, data, DX, DX, DX, DT)
            dc.device_swap_arrays(data)
        dc.device_data_get_results(proc, data)
        return data

    # untimed warm-up pass (first use of the path in this process), then the
    # fields it wrote back are zeroed again: the timed pass starts from the
    # same state
    dc.device_data_free(abi_run(args.warmup))
    for a in fields:
        a[:] = 0.0
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    data = abi_run(args.steps)
    el = time.perf_counter() - t0
    dc.device_data_free(data)
    init_s, local_s = marks["init"] - t0, el  # this rank's phases
    el = max_ms(el)
    h2d = 14 * sx * sy * sz * 4
    d2h = 2 * sx * sy * sz * 4
    return {"value": pts * args.steps * world / el / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
            "seconds": el,
            "phases_s": {"init_and_upload": init_s, "steps_and_read_back": local_s - init_s},
            "api": "reference C ABI (dc_device_data_init, dc_device_add_source, "
                                  "dc_propagate, dc_device_swap_arrays, "
                                  "dc_device_data_get_results), pinned host buffers"}


def batch_shots(n_shots: int, seed: int = BATCH_SEED, model=BATCH_MODEL, pad: int = BATCH_PAD):
    """Shot layout of the batched workload: sources on an 8 x 8 grid over the
    model surface with seeded jitter; each shot a crop of uneven aperture
    around its source.  Returns a list of dicts in medium-box coordinates."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mx, my, mz = model
    side = 8
    shots = []
    for k in range(n_shots):
        i, j = (k % (side * side)) % side, (k % (side * side)) // side
        sx_m = int(mx * (i + 0.5) / side + rng.uniform(-mx / side / 4, mx / side / 4))
        sy_m = int(my * (j + 0.5) / side + rng.uniform(-my / side / 4, my / side / 4))
        ax, ay = (min(int(v), m) for v, m in zip(rng.integers(192, 321, size=2), (mx, my)))
        peak = float(rng.uniform(15.0, 25.0))
        cx = min(max(sx_m - ax // 2, 0), mx - ax) // 4 * 4
        cy = min(max(sy_m - ay // 2, 0), my - ay)
        p = pad
        sizes = (ax + 2 * p, ay + 2 * p, min(BATCH_DEPTH, mz) + 2 * p)
        src = (sx_m - cx + p, sy_m - cy + p, p + SRC_DEPTH)
        rec_x = np.linspace(p, p + ax - 1, BATCH_RECEIVERS).astype(int)
        rec = [(int(x), src[1], p + 8) for x in rec_x]
        shots.append({"sizes": sizes, "origin": (cx + BATCH_PAD - p, cy + BATCH_PAD - p,
                                                 BATCH_PAD - p),
                      "src": src, "fcut": 3.0 * peak, "rec": rec,
                      "interior": ax * ay * min(BATCH_DEPTH, mz)})
    return shots


def run_batched(args, rank, world, local):
    """The batched form: all shots in one persistent, graph-captured launch
    per step.  Ranks > 0 run their own independent batch (weak scaling)."""
    import torch
    import __graft_entry__ as ge
    dc = ge.package()
    dc.build()
    from dc_gb300 import medium
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    form = {"f32": dc.MEDIUM_PRECOMP, "f16": dc.MEDIUM_PRECOMP_F16,
            "bf16": dc.MEDIUM_PRECOMP_BF16}[args.medium if args.medium != "f32" else "f16"]
    storage = "f16" if args.medium == "f32" else args.medium
    model = tuple(args.model)
    mbox = tuple(v + 2 * BATCH_PAD for v in model)
    shots = batch_shots(args.shots, BATCH_SEED + rank, model)
    total = args.warmup + args.steps
    b = dc.Batch(mbox, (DX,) * 3, DT, medium=form, device=local, max_steps=total + 1)
    b.generate_layered(medium.layered_spec(MEDIUM_SEED, mbox))
    for k, sh in enumerate(shots):
        b.add_shot(sh["sizes"], sh["origin"], sh["src"], sh["fcut"], ABSORB, SPONGE_KAPPA)
        b.set_receivers(k, sh["rec"])
    if args.no_autotune:
        (ty, zsplit), tune_ms = b.tiles(), None
    else:
        ty, zsplit, tune_ms = b.autotune(3)
    persistent = b.persistent
    pts = b.points
    b.run(args.warmup)
    b.synchronize()
    stream = torch.cuda.ExternalStream(b.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = b.launches
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        b.run(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    b.synchronize()
    launches = b.launches - l0
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    tr = b.traces(0, total)
    assert np.isfinite(tr).all()
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        # the smallest shot, as the batch computed it, against the FP64 oracle
        k = min(range(len(shots)), key=lambda i: int(np.prod(shots[i]["sizes"])))
        sh = shots[k]
        f = b.get_fields(k)
        btr = b.traces(k, total)
        coef = shot_coef(dc, medium.layered_spec(MEDIUM_SEED, mbox), sh, local)
        sizes = sh["sizes"]
        rec = np.array([shot_index(sizes, r) for r in sh["rec"]], np.int64)
        f64, osec = oracle_f64(sizes, coef, total, shot_index(sizes, sh["src"]),
                               dc.source_table(DT, total + 1, sh["fcut"]),
                               [dc.sponge_profile(v, ABSORB, SPONGE_KAPPA) for v in sizes], rec)
        accuracy = {"check": f"shot {k} of the batch (the smallest, {sizes[0]}x{sizes[1]}x"
                             f"{sizes[2]} padded) after all {total} steps against the FP64 "
                             f"CPU oracle on its crop; {rec.size} receivers",
                    "storage": storage, "rel_l2_p": rel(f["pc"], f64.pc),
                    "rel_l2_q": rel(f["qc"], f64.qc), "rel_l2_traces": rel(btr, f64.traces),
                    "bar": 1e-3,
                    "meets_bar": bool(rel(f["pc"], f64.pc) <= 1e-3 and
                                      rel(btr, f64.traces) <= 1e-3),
                    "oracle_seconds": osec}
    b.close()
    value = weak_rate(pts, args.steps, world, ms)
    bytes_per_update = 44 if storage in ("f16", "bf16") else 64
    achieved = bytes_per_update * pts / (ms / args.steps * 1e-3) / 1e9
    peak, peak_kind = peaks()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        g2 = geometry(N_INTERIOR)
        rate, info = cpu_baseline_slab(dc, g2)
        cpu = {"value": rate / 1e9, "unit": UNIT, "cores": info["cores"], "kind": info["kind"],
               "sample": f"{info['steps']} steps of a {g2.sizes[0] - 8}x{SLAB_ROWS}x"
                         f"{g2.sizes[2] - 8} y-slab of the plain workload ({info['seconds']:.1f} s; "
                         f"{info['what']}); the per-update CPU cost does not depend on the "
                         "batching"}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 12-layer TTI medium, numpy PCG64 seed 2026, generated on "
                "GPU; shot layout PCG64 seed 2027)",
        "config": {"workload": f"batched: {args.shots} shots in one launch per step "
                               f"over a shared {model[0]}x{model[1]}x"
                               f"{model[2]} medium, crops U(192,320)^2 x {BATCH_DEPTH} "
                               f"+ {ABSORB}-cell sponge, dt 0.8 ms, 15-25 Hz Ricker",
                   "form": "batched", "medium_storage": storage, "shots": args.shots,
                   "points_per_step": pts, "tiles": {"ty": ty, "zsplit": zsplit,
                                                     "persistent": persistent,
                                                     "autotune_ms_per_step": tune_ms},
                   "global_batch": args.shots * world, "seq_len": None,
                   "parallelism": f"shots{args.shots}x{world}",
                   "l2": "inputs ~76 GB >> 129 MB L2; no flush", "accuracy": accuracy},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "bytes_per_update": bytes_per_update, "traffic": None},
        "cpu_baseline": cpu,
        "e2e": None,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_learned(args, rank, world, local):
    """The learned thin layer against the 48-cell sponge on one shot."""
    import torch
    import __graft_entry__ as ge
    dc = ge.package()
    dc.build()
    from dc_gb300 import learned
    torch.cuda.set_device(local)
    n, layer = args.learned_n, LEARNED_LAYER
    st = learned.Setup(n=(n,) * 3, layer=layer, fcut=FCUT)
    total = args.warmup + args.steps
    src = (4 + layer + n // 2 + 8 * rank, 4 + layer + n // 2, 4 + layer + SRC_DEPTH)
    mlp = dc.MLP(device=local, params=np.load(learned.WEIGHTS))

    def timed(sim):
        sim.run(args.warmup)
        sim.synchronize()
        stream = torch.cuda.ExternalStream(sim.stream)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = sim.launches
        torch.cuda.synchronize()
        ev0.record(stream)
        sim.run(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        sim.synchronize()
        return ev0.elapsed_time(ev1), sim.launches - l0

    def with_source(sim, sizes, s):
        sx, sy, _ = sizes
        sim.set_source(s[0] + s[1] * sx + s[2] * sx * sy, dc.source_table(DT, total + 2, FCUT))

    thin = learned.thin_sim(st, local)
    with_source(thin, st.thin_sizes, src)
    dc.set_learned_layer(thin, mlp, layer)
    with ClockSampler(local) as clk:
        ms_l, launches = timed(thin)
    thin.close()
    a = ABSORB
    sp = dc.Simulation(st.sponge_sizes, (DX,) * 3, DT, kernel=dc.KERNEL_FAST, device=local)
    shift = st.wide_pad + layer - a
    sp.generate_layered(learned._origin_spec(st, (shift,) * 3))
    sp.set_fields()
    sp.set_sponge(*[dc.sponge_profile(v, a, SPONGE_KAPPA) for v in st.sponge_sizes])
    with_source(sp, st.sponge_sizes, tuple(c - layer + a for c in src))
    ms_s, _ = timed(sp)
    sp.close()
    interior = n ** 3
    value = interior * args.steps / (ms_l * 1e-3) / 1e9
    sponge_value = interior * args.steps / (ms_s * 1e-3) / 1e9
    refl = (None if args.no_judge else
            learned.reflected_energy(st, mlp, src, total, 100, 32, local))
    mlp.close()
    pts_l = (n + 2 * layer) ** 3
    achieved = BYTES_PER_UPDATE * pts_l / (ms_l / args.steps * 1e-3) / 1e9
    peak, peak_kind = peaks()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_l / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 12-layer TTI medium, numpy PCG64 seed 2026, generated on GPU)",
        "config": {"workload": f"learned thin layer: {n}^3 interior, {layer}-cell learned layer "
                               f"vs {ABSORB}-cell sponge, dt 0.8 ms, 20 Hz Ricker, FP32",
                   "form": "learned", "value_counts": "interior point-updates",
                   "learned": {"interior_gupd_s": value, "ms_per_step": ms_l / args.steps,
                               "compute_points": pts_l},
                   "sponge48": {"interior_gupd_s": sponge_value, "ms_per_step": ms_s / args.steps,
                                "compute_points": (n + 2 * ABSORB) ** 3},
                   "speedup_vs_sponge48": ms_s / ms_l,
                   "reflected_energy_band32": refl,
                   "global_batch": world, "seq_len": None, "parallelism": "single",
                   "l2": "inputs ~4 GB >> 129 MB L2; no flush"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "bytes_per_update": BYTES_PER_UPDATE,
                     "note": "stencil bytes over the whole learned step (stencil + network)",
                     "traffic": None},
        "cpu_baseline": None, "e2e": None, "gpu_launches": launches, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def best_accuracy(dc, b, thin, wide, spec, total: int, layer: int, local: int):
    """The best form's error on its own workload: the smallest shot, as the
    batch computed it (FP16 medium, learned thin layer), against the FP64
    CPU oracle of the same shot in the plain form's geometry (the 48-cell
    sponge), compared over the shot's interior and its receivers; the plain
    FP32 form of the same shot against the same oracle for comparison."""
    k = min(range(len(thin)), key=lambda i: int(np.prod(wide[i]["sizes"])))
    t, w = thin[k], wide[k]
    pt, pw = layer + 4, BATCH_PAD
    nx, ny = w["sizes"][0] - 2 * pw, w["sizes"][1] - 2 * pw
    nz = w["sizes"][2] - 2 * pw

    def inner(a, pad):
        return a[pad:pad + nz, pad:pad + ny, pad:pad + nx]

    f = b.get_fields(k)
    btr = b.traces(k, total)
    sizes = w["sizes"]
    coef = shot_coef(dc, spec, w, local)
    src_idx = shot_index(sizes, w["src"])
    src = dc.source_table(DT, total + 1, w["fcut"])
    sponge = [dc.sponge_profile(v, ABSORB, SPONGE_KAPPA) for v in sizes]
    rec = np.array([shot_index(sizes, r) for r in w["rec"]], np.int64)
    f64, osec = oracle_f64(sizes, coef, total, src_idx, src, sponge, rec)
    # the plain form (FP32, 48-cell sponge) of the same shot on the GPU
    sim = dc.Simulation(sizes, (DX,) * 3, DT, kernel=dc.KERNEL_FAST, device=local)
    sim.set_precomp(coef)
    sim.set_fields()
    sim.set_source(src_idx, src)
    sim.set_sponge(*sponge)
    sim.set_receivers(rec, total)
    sim.run(total)
    sim.synchronize()
    pf = sim.get_fields()
    ptr = sim.traces(total)
    sim.close()
    e_p = rel(inner(f["pc"], pt), inner(f64.pc, pw))
    e_tr = rel(btr, f64.traces)
    return {"check": f"shot {k} of the batch (the smallest: {nx}x{ny}x{nz} interior) after "
                     f"all {total} steps against the FP64 CPU oracle of the same shot with the "
                     f"{ABSORB}-cell sponge, over the interior and {rec.size} receivers",
            "rel_l2_p_interior": e_p, "rel_l2_q_interior": rel(inner(f["qc"], pt),
                                                               inner(f64.qc, pw)),
            "rel_l2_traces": e_tr,
            "plain_fp32_rel_l2_p_interior": rel(inner(pf["pc"], pw), inner(f64.pc, pw)),
            "plain_fp32_rel_l2_traces": rel(ptr, f64.traces),
            "bar": 1e-3, "meets_bar": bool(e_p <= 1e-3 and e_tr <= 1e-3),
            "oracle_seconds": osec}


def run_best(args, rank, world, local):
    """Best form (batched + FP16 medium + learned thin layer) against the
    plain form on the same shot layout."""
    import torch
    import __graft_entry__ as ge
    dc = ge.package()
    dc.build()
    from dc_gb300 import learned, medium
    torch.cuda.set_device(local)
    layer = LEARNED_LAYER
    model = tuple(args.model)
    mbox = tuple(v + 2 * BATCH_PAD for v in model)
    spec = medium.layered_spec(MEDIUM_SEED, mbox)
    total = args.warmup + args.steps
    thin = batch_shots(args.shots, BATCH_SEED + rank, model, pad=layer + 4)
    wide = batch_shots(args.shots, BATCH_SEED + rank, model)
    interior = sum(s["interior"] for s in thin)

    def timed_run(obj, steps):
        stream = torch.cuda.ExternalStream(obj.stream)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        obj.run(steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        obj.synchronize()
        return ev0.elapsed_time(ev1)

    # best form: one batch, FP16 medium, learned layer on every shot
    mlp = dc.MLP(device=local, params=np.load(learned.WEIGHTS))
    b = dc.Batch(mbox, (DX,) * 3, DT, medium=dc.MEDIUM_PRECOMP_F16, device=local,
                 max_steps=total + 1)
    b.generate_layered(spec)
    for k, sh in enumerate(thin):
        b.add_shot(sh["sizes"], sh["origin"], sh["src"], sh["fcut"], 0, 0.0)
        b.set_receivers(k, sh["rec"])
    ty, zsplit, _ = b.autotune(3)
    persistent = b.persistent
    b.set_learned_layer(mlp, layer)
    b.run(args.warmup)
    b.synchronize()
    l0 = b.launches
    with ClockSampler(local) as clk:
        ms = timed_run(b, args.steps)
    launches = b.launches - l0
    assert np.isfinite(b.traces(0, total)).all()
    compute_pts = b.points
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        accuracy = best_accuracy(dc, b, thin, wide, spec, total, layer, local)
    b.close()
    mlp.close()
    best = interior * args.steps / (ms * 1e-3) / 1e9
    # stencil bytes (FP16 medium: 44 B per updated point) over the whole step
    achieved = 44 * compute_pts / (ms / args.steps * 1e-3) / 1e9
    peak, peak_kind = peaks()
    # plain form: FP32, 48-cell sponge, one shot at a time, every shot (the
    # interior fraction of a crop depends on its aperture); its step costs
    # the same at every step, so each shot is timed over at most 100 steps
    n_plain = len(wide)
    plain_steps = min(args.steps, 100)
    plain_pts, plain_ms = 0, 0.0
    for sh in wide:
        sizes = sh["sizes"]
        sim = dc.Simulation(sizes, (DX,) * 3, DT, kernel=dc.KERNEL_FAST, device=local)
        sim.generate_layered(medium.with_origin(spec, sh["origin"]))
        sim.set_fields()
        sx, sy, _ = sizes
        x, y, z = sh["src"]
        sim.set_source(x + y * sx + z * sx * sy, dc.source_table(DT, total + 2, sh["fcut"]))
        sim.set_sponge(*[dc.sponge_profile(v, ABSORB, SPONGE_KAPPA) for v in sizes])
        sim.run(args.warmup)
        sim.synchronize()
        plain_ms += timed_run(sim, plain_steps)
        plain_pts += sh["interior"]
        sim.close()
    plain = plain_pts * plain_steps / (plain_ms * 1e-3) / 1e9
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": best, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 12-layer TTI medium, numpy PCG64 seed 2026, generated on "
                "GPU; shot layout PCG64 seed 2027)",
        "config": {"workload": f"best form: {args.shots} crops of U(192,320)^2 x {BATCH_DEPTH} "
                               f"from a {model[0]}x{model[1]}x{model[2]} medium, batched, FP16 "
                               f"medium, {layer}-cell learned layer; vs plain FP32 + "
                               f"{ABSORB}-cell sponge one shot at a time",
                   "form": "best", "value_counts": "interior shot-point-updates",
                   "shots": args.shots, "interior_points_per_step": interior,
                   "tiles": {"ty": ty, "zsplit": zsplit, "persistent": persistent},
                   "plain": {"interior_gupd_s": plain, "shots_timed": n_plain,
                             "steps_per_shot": plain_steps,
                             "ms_per_step_all_shots": plain_ms / plain_steps},
                   "speedup_vs_plain": best / plain,
                   "accuracy": accuracy,
                   "global_batch": args.shots * world, "seq_len": None,
                   "parallelism": f"shots{args.shots}x{world}",
                   "l2": "inputs ~40 GB >> 129 MB L2; no flush"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "bytes_per_update": 44,
                     "note": "stencil bytes per updated point over the whole step "
                             "(stencil + network + correction)", "traffic": None},
        "cpu_baseline": None, "e2e": None, "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_refcuda(args, rank, world, local):
    """The reference's own GPU path against ours on the same GPU and the
    same inputs: the reference's default medium with its random velocity
    boundary (vpz/vsv, constant angles: the only medium its CUDA backend
    reads) on the plain workload's geometry, the reference's source at the
    cube centre.  The reference runs its one-rank loop (seven dc_propagate
    launches per step, each synchronised, src/worker.c:321-402 and
    src/cuda_propagate.cu:32-69); ours runs the same steps as graph-replayed
    single launches of the fast kernel on the (vpz, vsv) medium (32 B per
    point-update), and once more through our library's reference ABI with
    the same seven-box loop.  Both runs start from zero fields, so their
    final fields are compared."""
    import torch
    import __graft_entry__ as ge
    from oracle.oracle import Geometry, Reference, rel_l2
    if rank != 0:
        return
    dc = ge.package()
    dc.build()
    torch.cuda.set_device(local)
    ref = Reference("cuda")
    geom = Geometry((args.n,) * 3, ABSORB)
    sizes = geom.sizes
    sx, sy, sz = sizes
    dt = 1e-3
    aniso = ref.default_anisotropy(geom.shape)
    ref.random_velocity_boundary(sizes, sizes, (0, 0, 0), geom.n, 4, ABSORB,
                                 aniso["vpz"], aniso["vsv"], 0)
    vpz, vsv = aniso["vpz"], aniso["vsv"]
    del aniso
    steps = args.steps
    src = np.array([ref.source(dt, it) for it in range(steps + args.warmup + 1)], np.float32)
    pts = geom.compute_points
    # the reference's CUDA path (its dc_device_data_init copies the host
    # arrays; the loop time excludes set-up and the read-back)
    z = [np.zeros(geom.shape, np.float32) for _ in range(4)]
    ref.run(0, sizes, (DX,) * 3, dt, args.warmup, *z, vpz=vpz, vsv=vsv,
            src_index=geom.source_index, src=src)
    z = [np.zeros(geom.shape, np.float32) for _ in range(4)]
    rpc, rqc, ref_s = ref.run(0, sizes, (DX,) * 3, dt, steps, *z, vpz=vpz, vsv=vsv,
                              src_index=geom.source_index, src=src, timed=True)
    del z
    # ours: graph-replayed fast kernel on the vpz/vsv medium
    sim = dc.Simulation(sizes, (DX,) * 3, dt, kernel=dc.KERNEL_FAST,
                        medium=dc.MEDIUM_VPZ_VSV, device=local)
    sim.set_vpz_vsv(vpz, vsv)
    sim.set_fields()
    sim.set_source(geom.source_index, src)
    sim.run(args.warmup)
    sim.set_fields()
    sim.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        sim.run(steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    sim.synchronize()
    ms = ev0.elapsed_time(ev1)
    f = sim.get_fields()
    sim.close()
    err = max(rel_l2(f["pc"], rpc), rel_l2(f["qc"], rqc))
    # ours through the reference ABI, same seven-box loop
    os.environ["DC_GB300_KERNEL"] = "fast"
    os.environ["DC_GB300_MEDIUM"] = "vpz_vsv"
    os.environ["DC_GB300_DEVICE"] = str(local)
    proc = dc.Process(sizes, (DX,) * 3, dt, anisotropy={"vpz": vpz, "vsv": vsv},
                      source_index=geom.source_index)
    data = dc.device_data_init(proc)
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
    for it in range(args.warmup):
        dc.device_add_source(data, geom.source_index, float(src[it]))
        for b0, b1 in boxes:
            dc.propagate(b0, b1, sizes, data, DX, DX, DX, dt)
        dc.device_swap_arrays(data)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(steps):
        dc.device_add_source(data, geom.source_index, float(src[it]))
        for b0, b1 in boxes:
            dc.propagate(b0, b1, sizes, data, DX, DX, DX, dt)
        dc.device_swap_arrays(data)
    dc.device_data_get_results(proc, data)
    abi_s = time.perf_counter() - t0
    dc.device_data_free(data)
    for k in ("DC_GB300_KERNEL", "DC_GB300_MEDIUM", "DC_GB300_DEVICE"):
        os.environ.pop(k, None)
    ours = pts * steps / (ms * 1e-3) / 1e9
    ref_rate = pts * steps / ref_s / 1e9
    abi_rate = pts * steps / abi_s / 1e9
    peak, peak_kind = peaks()
    achieved = 32 * pts / (ms / steps * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": ours, "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (the reference's default medium + random velocity boundary, seed 0)",
        "config": {"workload": f"reference CUDA path vs ours on one GB300: {args.n}^3 interior + "
                               f"{ABSORB}-cell random velocity boundary, {sx}^3 padded, "
                               "vpz/vsv medium (constant angles), FCUT 40 source at the centre, "
                               "dt 1 ms",
                   "form": "refcuda", "points_per_step": pts,
                   "reference_cuda": {"gupd_s": ref_rate, "ms_per_step": ref_s / steps * 1e3,
                                      "launches_per_step": 8,
                                      "what": "src/cuda_propagate.cu + src/device_data.cu, nvcc "
                                              "sm_103a, one-rank loop of src/worker.c"},
                   "ours_graph": {"gupd_s": ours, "ms_per_step": ms / steps},
                   "ours_reference_abi": {"gupd_s": abi_rate,
                                          "ms_per_step": abi_s / steps * 1e3,
                                          "note": "same seven-box loop through our dc_propagate, "
                                                  "wall clock incl. the final read-back"},
                   "speedup_vs_reference_cuda": ours / ref_rate,
                   "rel_l2_vs_reference_cuda": err,
                   "l2": "inputs 5.6 GB >> 129 MB L2; no flush"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "bytes_per_update": 32,
                     "traffic": None},
        "cpu_baseline": None, "e2e": None, "gpu_launches": steps, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    try:
        if args.form == "batched":
            run_batched(args, rank, world, local)
        elif args.form == "learned":
            run_learned(args, rank, world, local)
        elif args.form == "best":
            run_best(args, rank, world, local)
        elif args.form == "refcuda":
            run_refcuda(args, rank, world, local)
        else:
            run_ours(args, rank, world, local)
    finally:
        if world > 1:  # ranks leave the process group together
            import torch.distributed as dist
            if dist.is_initialized():
                dist.destroy_process_group()


if __name__ == "__main__":
    main()
