"""Training and judging the learned thin absorbing layer.

The layer, its network and every kernel (sample gathering, forward,
backward, Adam, in-step inference) live in the library (csrc/dc_learned.cu);
this module only arranges the runs:

* ``Setup`` describes a thin box (interior ``n`` + a ``layer``-cell learned
  layer + 4-cell halo) placed inside a wide box whose margins and 48-cell
  sponge keep reflections away from the thin box for the whole window.
* ``make_samples`` runs the wide box from random source positions and at
  every ``every``-th step gathers teacher-forced samples from the thin box
  (``dc_gb300_lb_sample``) into device arrays.
* ``make_rollout_samples`` does the same from the thin box running its own
  network for a few steps after each crop (``dc_gb300_lb_rollout``), so the
  network also learns from the states it produces itself.
* ``train`` fits an MLP to them (``dc_gb300_mlp_train``); ``fit`` chains
  teacher-forced samples, training and rounds of rollout samples.
* ``reflected_energy`` runs one shot three ways -- the thin box with or
  without the network, a box with a wide sponge -- and compares each with
  the wide run inside a band of the interior next to its boundary.

Device arrays are allocated with torch (plumbing only: no torch operator
touches the data).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import (KERNEL_FAST, MEDIUM_PRECOMP, MLP, Simulation, lb_rollout, lb_sample,
               set_learned_layer, source_table, sponge_profile)
from . import medium as _medium


@dataclass(frozen=True)
class Setup:
    n: tuple = (48, 48, 48)       # interior cells of the thin box
    layer: int = 8                # learned layer width
    thin_kappa: float = 0.0       # sponge strength inside the thin layer (0: none)
    margin: int = 48              # wide box: cells beyond the thin box, per side
    wide_absorb: int = 48         # wide box: its own sponge width
    wide_kappa: float = 0.35
    sponge_absorb: int = 48       # judge: the plain sponge of this width
    d: float = 12.5
    dt: float = 0.8e-3
    fcut: float = 60.0
    seed: int = 2026              # medium seed
    medium_args: tuple = ()       # extra layered_spec arguments, as (name, value) pairs

    @property
    def thin_sizes(self):
        return tuple(v + 2 * self.layer + 8 for v in self.n)

    @property
    def wide_pad(self):
        return self.margin + self.wide_absorb

    @property
    def wide_sizes(self):
        return tuple(v + 2 * self.wide_pad for v in self.thin_sizes)

    @property
    def offset(self):
        """Position of the thin box's point (0, 0, 0) in the wide box."""
        return (self.wide_pad,) * 3

    @property
    def sponge_sizes(self):
        return tuple(v + 2 * self.sponge_absorb + 8 for v in self.n)

    def spec(self):
        return _medium.layered_spec(self.seed, self.wide_sizes, **dict(self.medium_args))


def _origin_spec(setup: Setup, origin):
    return _medium.with_origin(setup.spec(), origin)


def _sponge(sizes, absorb, kappa):
    return [sponge_profile(s, absorb, kappa) for s in sizes]


def thin_sim(setup: Setup, device=0, kernel=KERNEL_FAST):
    """The thin box with its medium (wide-box coordinates shifted by the
    offset) and its thin-layer sponge."""
    sim = Simulation(setup.thin_sizes, (setup.d,) * 3, setup.dt, kernel=kernel,
                     medium=MEDIUM_PRECOMP, device=device)
    sim.generate_layered(_origin_spec(setup, setup.offset))
    sim.set_fields()
    if setup.thin_kappa > 0:  # a zero-strength profile is all ones: no sponge pass at all
        sim.set_sponge(*_sponge(setup.thin_sizes, setup.layer, setup.thin_kappa))
    return sim


def wide_sim(setup: Setup, src_thin, steps, device=0, kernel=KERNEL_FAST):
    """The wide box with a source at thin-box coordinates ``src_thin``."""
    sim = Simulation(setup.wide_sizes, (setup.d,) * 3, setup.dt, kernel=kernel,
                     medium=MEDIUM_PRECOMP, device=device)
    sim.generate_layered(setup.spec())
    sim.set_fields()
    sx, sy, _ = setup.wide_sizes
    x, y, z = (c + o for c, o in zip(src_thin, setup.offset))
    sim.set_source(x + y * sx + z * sx * sy, source_table(setup.dt, steps + 2, setup.fcut))
    sim.set_sponge(*_sponge(setup.wide_sizes, setup.wide_absorb, setup.wide_kappa))
    return sim


def random_sources(setup: Setup, count: int, seed: int, inset: int = 6):
    """Source positions (thin-box coordinates) drawn inside the interior."""
    rng = np.random.default_rng(seed)
    lo = 4 + setup.layer + inset
    hi = [s - 4 - setup.layer - inset for s in setup.thin_sizes]
    return [tuple(int(rng.integers(lo, h)) for h in hi) for _ in range(count)]


class SampleStore:
    """Device arrays of samples [cap][33] and targets [cap][2], filled from
    the front by the library's sample functions."""

    def __init__(self, cap: int, device=0):
        import torch
        dev = torch.device("cuda", device)
        self.xs = torch.empty((cap, 33), dtype=torch.float32, device=dev)
        self.ts = torch.empty((cap, 2), dtype=torch.float32, device=dev)
        torch.cuda.synchronize(dev)
        self.cap, self.n = cap, 0

    def ptrs(self):
        return (self.xs.data_ptr() + self.n * 33 * 4, self.ts.data_ptr() + self.n * 2 * 4,
                self.cap - self.n)


def corrected_cells(setup: Setup) -> int:
    from . import layer_cells
    return len(layer_cells(setup.thin_sizes, setup.layer))


def make_samples(setup: Setup, sources, steps: int, first: int, every: int, store: SampleStore,
                 device=0):
    """Teacher-forced samples from wide runs (every ``every``-th step from
    ``first`` on), appended to ``store``."""
    thin = thin_sim(setup, device)
    try:
        for src in sources:
            wide = wide_sim(setup, src, steps, device)
            try:
                done = 0
                for k in range(first, steps, every):
                    wide.run(k - done)
                    wide.synchronize()
                    xp, tp, cap = store.ptrs()
                    store.n += lb_sample(wide, thin, setup.offset, setup.layer, xp, tp, cap)
                    done = k + 1  # lb_sample advanced the wide run one step
            finally:
                wide.close()
    finally:
        thin.close()


def make_rollout_samples(setup: Setup, mlp: MLP, sources, steps: int, starts, seg: int,
                         store: SampleStore, device=0):
    """Rollout samples appended to ``store``: for every source and start
    step, the wide run is cropped into the thin box, which then runs
    ``seg`` steps with the network while the wide run keeps pace."""
    thin = thin_sim(setup, device)
    set_learned_layer(thin, mlp, setup.layer)
    try:
        for src in sources:
            wide = wide_sim(setup, src, steps + seg, device)
            try:
                done = 0
                for k in starts:
                    if k < done:
                        continue
                    wide.run(k - done)
                    wide.synchronize()
                    xp, tp, cap = store.ptrs()
                    store.n += lb_rollout(wide, thin, setup.offset, seg, xp, tp, cap)
                    done = k + seg
            finally:
                wide.close()
    finally:
        thin.close()


def fit(setup: Setup, mlp: MLP, sources, steps: int, rounds: int = 6, train_steps: int = 2000,
        batch: int = 8192, lr: float = 2e-3, seg: int = 16, first: int = 40, every: int = 6,
        seed: int = 1, device=0):
    """Teacher-forced samples and training, then ``rounds`` rounds of
    rollout samples from the current network added to the same set
    (dataset aggregation) and further training on all of it.  Returns the
    loss history."""
    per = corrected_cells(setup)
    teacher = len(range(first, steps, every)) * len(sources) * per
    starts = [list(range(first + (r * seg) // max(1, rounds), steps - seg, 3 * seg))
              for r in range(rounds)]
    rollout = sum(len(st) for st in starts) * seg * len(sources) * per
    store = SampleStore(teacher + rollout, device)
    make_samples(setup, sources, steps, first, every, store, device)
    hist = [train(mlp, store.xs, store.ts, store.n, train_steps, batch, lr, seed=seed,
                  decay_every=train_steps // 2)]
    for r in range(rounds):
        make_rollout_samples(setup, mlp, sources, steps, starts[r], seg, store, device)
        hist.append(train(mlp, store.xs, store.ts, store.n, train_steps, batch, lr * 0.5,
                          seed=seed + 100 + r, decay_every=train_steps // 2))
    del store
    return np.concatenate(hist)


def select(setup: Setup, seeds, sources, val_sources, steps: int, rounds: int = 6,
           band: int = 12, every: int = 20, device=0, **fit_args):
    """Trains one network per seed and keeps the one with the lowest
    reflected energy on the validation shots.  Returns (mlp or None,
    report): None when no network beats the thin layer without it -- the
    sponge is then the one to use."""
    best, best_score, report = None, None, []
    base = None
    for k, sd in enumerate(seeds):
        mlp = MLP(device=device, seed=sd)
        fit(setup, mlp, sources, steps, rounds=rounds, seed=sd, device=device, **fit_args)
        ev = [reflected_energy(setup, mlp, s, steps, every, band, device,
                               judges=("thin", "learned") if base is None else ("learned",))
              for s in val_sources]
        if base is None:
            base = sum(e["thin"] for e in ev)
        score = sum(e["learned"] for e in ev)
        report.append({"seed": sd, "val_learned": score, "val_thin": base})
        if np.isfinite(score) and (best_score is None or score < best_score):
            if best is not None:
                best.close()
            best, best_score = mlp, score
        else:
            mlp.close()
    if best is not None and not best_score < base:
        best.close()
        best = None
    return best, report


def train(mlp: MLP, xs, ts, n: int, steps: int, batch: int = 8192, lr: float = 2e-3,
          seed: int = 1, decay_every: int = 0):
    """Adam on the samples; a step-wise learning-rate decay (x 0.3 every
    ``decay_every`` steps) if given.  Returns the loss history."""
    hist = []
    left, rate = steps, lr
    chunk = decay_every if decay_every > 0 else steps
    k = 0
    while left > 0:
        m = min(chunk, left)
        hist.append(mlp.train(xs.data_ptr(), ts.data_ptr(), n, m, batch, rate, seed + k))
        left -= m
        rate *= 0.3
        k += 1
    return np.concatenate(hist) if hist else np.zeros(0, np.float32)


def _band_mask(n, band):
    """Interior cells within ``band`` of the interior's boundary."""
    nz, ny, nx = n[2], n[1], n[0]
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    dist = np.minimum.reduce([x, nx - 1 - x, y, ny - 1 - y, z, nz - 1 - z])
    return dist < band


def _interior(a, pad, n):
    return a[pad:pad + n[2], pad:pad + n[1], pad:pad + n[0]]


def reflected_energy(setup: Setup, mlp: MLP | None, src, steps: int, every: int, band: int,
                     device=0, judges=("thin", "learned", "sponge")):
    """Energy of (p - p_wide) in the interior band, summed over the sampled
    steps, relative to the energy of p_wide there.  Returns a dict for
    'thin' (thin layer without the network), 'learned' (with it, if given)
    and 'sponge' (plain sponge of setup.sponge_absorb cells)."""
    mask = _band_mask(setup.n, band)
    keys = list(range(every, steps + 1, every))
    truth = {}
    wide = wide_sim(setup, src, steps, device)
    done = 0
    for k in keys:
        wide.run(k - done)
        done = k
        wide.synchronize()
        truth[k] = _interior(wide.get_pc(), setup.wide_pad + 4 + setup.layer, setup.n).copy()
    wide.close()
    ref = sum(float(np.sum(truth[k][mask].astype(np.float64) ** 2)) for k in keys)

    def run(sim, pad):
        err, dn = 0.0, 0
        for k in keys:
            sim.run(k - dn)
            dn = k
            sim.synchronize()
            d = _interior(sim.get_pc(), pad, setup.n) - truth[k]
            err += float(np.sum(d[mask].astype(np.float64) ** 2))
        return err / ref if ref > 0 else float("nan")

    def with_source(sim, sizes, s):
        sx, sy, _ = sizes
        sim.set_source(s[0] + s[1] * sx + s[2] * sx * sy,
                       source_table(setup.dt, steps + 2, setup.fcut))

    out = {}
    for name in [j for j in judges if j in ("thin", "learned")]:
        if name == "learned" and mlp is None:
            continue
        sim = thin_sim(setup, device)
        with_source(sim, setup.thin_sizes, src)
        if name == "learned":
            set_learned_layer(sim, mlp, setup.layer)
        out[name] = run(sim, 4 + setup.layer)
        sim.close()
    if "sponge" not in judges:
        return out
    a = setup.sponge_absorb
    sim = Simulation(setup.sponge_sizes, (setup.d,) * 3, setup.dt, kernel=KERNEL_FAST,
                     medium=MEDIUM_PRECOMP, device=device)
    shift = setup.wide_pad + setup.layer - a  # sponge box origin in wide coordinates
    sim.generate_layered(_origin_spec(setup, (shift,) * 3))
    sim.set_fields()
    sim.set_sponge(*_sponge(setup.sponge_sizes, a, setup.wide_kappa))
    with_source(sim, setup.sponge_sizes, tuple(c - setup.layer + a for c in src))
    out["sponge"] = run(sim, 4 + a)
    sim.close()
    return out


WEIGHTS = __import__("pathlib").Path(__file__).resolve().parent / "data" / "learned_layer8.npy"


def main(argv=None):
    """Trains the layer's network (best of several seeds on validation
    shots) and writes its parameters:

        python -c "import __graft_entry__ as g; g.package(); \\
                   from dc_gb300 import learned; learned.main(['--out', 'w.npy'])"
    """
    import argparse
    import json
    ap = argparse.ArgumentParser(prog="learned")
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--seeds", type=int, nargs="+", default=[11, 12, 13, 14])
    ap.add_argument("--rounds", type=int, default=6)
    ap.add_argument("--seg", type=int, default=16)
    ap.add_argument("--n", type=int, default=48)
    ap.add_argument("--steps", type=int, default=320)
    args = ap.parse_args(argv)
    st = Setup(n=(args.n,) * 3, layer=8)
    mlp, report = select(st, args.seeds, random_sources(st, 4, 7), random_sources(st, 2, 55),
                         steps=args.steps, rounds=args.rounds, seg=args.seg)
    if mlp is None:
        raise SystemExit("no network beat the thin layer without it")
    np.save(args.out, mlp.params())
    mlp.close()
    print(json.dumps({"out": args.out, "setup": str(st), "selection": report}))
