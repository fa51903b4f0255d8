"""The learned layer on the CPU: the oracle's backpropagation against finite
differences, and the layer-cell geometry against a direct enumeration."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def test_oracle_gradient_matches_finite_differences():
    p = mo.init_params(3).astype(np.float64)
    s = mo.random_samples(64, 4)
    t = np.random.default_rng(5).normal(0, 1, (64, 2)) * np.sqrt(np.mean(s[:, :32] ** 2, 1))[:, None]
    g, _, _ = mo.gradient(p, s, t, rounding=False)
    rng = np.random.default_rng(6)
    idx = np.concatenate([rng.choice(np.arange(lo, hi), min(6, hi - lo), replace=False) for lo, hi in
                          ((mo.OFF_W1, mo.OFF_B1), (mo.OFF_B1, mo.OFF_B1 + 8 * 32),
                           (mo.OFF_W2, mo.OFF_B2), (mo.OFF_B2, mo.OFF_W3),
                           (mo.OFF_W3, mo.OFF_B3), (mo.OFF_B3, mo.NPARAMS))])
    for i in idx:
        h = 1e-5 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss(pp, s, t, rounding=False)[0] - mo.loss(pm, s, t, rounding=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7 * np.abs(g).max(), (i, fd, g[i])


def test_oracle_forward_is_homogeneous():
    """The correction scales with the wavefield: f(a x) = a f(x), a > 0."""
    p = mo.init_params(8)
    s = mo.random_samples(32, 9)
    s2 = s.copy()
    s2[:, :32] *= 4.0  # a power of two keeps every BF16 rounding identical
    np.testing.assert_allclose(mo.forward(p, s2), 4.0 * mo.forward(p, s), rtol=1e-12, atol=0)


def _layer_cells_direct(s, layer):
    out = {}
    for z in range(4, s[2] - 4):
        for y in range(4, s[1] - 4):
            for x in range(4, s[0] - 4):
                best = None
                for a, c in enumerate((x, y, z)):
                    lo, hi = 4 + layer, s[a] - 4 - layer
                    d = lo - 1 - c if c < lo else (c - hi if c >= hi else -1)
                    if d >= 0 and (best is None or d > best[1]):
                        best = (a, d, int(c >= hi))
                if best and best[1] >= layer - 4:
                    out[(x, y, z)] = best
    return out


def test_layer_cell_table_matches_direct_enumeration(dc):
    """The library's layer-cell table: one entry per cell of the shell, with
    the normal axis, side and depth of a direct enumeration."""
    s, layer = (28, 30, 29), 6
    want = _layer_cells_direct(s, layer)
    got = dc.layer_cells(s, layer)
    # the corrected cells: the 4 outer cells of the layer on every side
    assert len(got) == len(want) == np.prod([v - 8 for v in s]) - np.prod([v - 16 for v in s])
    for x, y, z, m in got:
        assert want[(x, y, z)] == (m & 3, m >> 3, (m >> 2) & 1)
    assert want[(4, 4, 10)] == (0, layer - 1, 0)  # tie: lowest axis


def _inward(cell, axis, side, k):
    c = list(cell)
    c[axis] += k if side == 0 else -k
    return tuple(c)


@pytest.mark.parametrize("s,layer", [((40, 38, 36), 6), ((44, 46, 45), 8), ((32, 33, 32), 8),
                                     ((30, 30, 31), 4), ((28, 29, 30), 3)])
def test_layer_plan_partitions_and_separates(dc, s, layer):
    """The step's split of the corrected cells: face lines (4 cells from the
    outermost inward, corrected in place from windows spanning 11 cells)
    and edge cells (8-cell windows, corrected through a buffer) cover every
    corrected cell once, and no line's or edge cell's window reads a cell
    that another line or the edge pass writes -- so the fused step equals
    the two-pass one."""
    cells = {(x, y, z): m for x, y, z, m in dc.layer_cells(s, layer)}
    lines, edge = dc.layer_plan(s, layer)
    if layer < 4:
        assert len(lines) == 0
    elif min(s) >= 2 * layer + 16 + 2 * (11 - layer):
        assert len(lines) > 0
    owner, line_reads = {}, []
    for i, (x, y, z, m) in enumerate(lines):
        axis, side = m & 3, (m >> 2) & 1
        for j in range(4):
            c = _inward((x, y, z), axis, side, j)
            assert cells[c] == axis | side << 2 | (layer - 1 - j) << 3
            assert c not in owner
            owner[c] = i
        line_reads.append([_inward((x, y, z), axis, side, k) for k in range(11)])
    edge_cells = {(x, y, z) for x, y, z, _ in edge}
    assert len(edge_cells) == len(edge)
    assert not edge_cells & owner.keys()
    assert edge_cells | owner.keys() == cells.keys()
    for i, reads in enumerate(line_reads):
        for c in reads:
            assert owner.get(c, i) == i and c not in edge_cells
    for x, y, z, m in edge:
        axis, side = m & 3, (m >> 2) & 1
        for k in range(8):
            assert _inward((x, y, z), axis, side, k) not in owner
