"""Host-side checks of the benchmark workloads (no GPU): the batched shot
layout and the learned-layer set-up respect the library's geometric rules
(shot boxes inside the medium box, x origins multiples of 4, sources and
receivers in the updated region, interiors of at least 8 cells)."""
import numpy as np
import pytest

import bench


@pytest.mark.parametrize("pad", [bench.BATCH_PAD, bench.LEARNED_LAYER + 4])
def test_batch_shot_layout(pad):
    mbox = tuple(v + 2 * bench.BATCH_PAD for v in bench.BATCH_MODEL)
    shots = bench.batch_shots(bench.BATCH_SHOTS, bench.BATCH_SEED, bench.BATCH_MODEL, pad=pad)
    assert len(shots) == bench.BATCH_SHOTS
    for sh in shots:
        sx, sy, sz = sh["sizes"]
        ox, oy, oz = sh["origin"]
        assert ox % 4 == 0 and min(ox, oy, oz) >= 0
        assert ox + sx <= mbox[0] and oy + sy <= mbox[1] and oz + sz <= mbox[2]
        for p in [sh["src"]] + sh["rec"]:
            assert all(4 <= c < s - 4 for c, s in zip(p, (sx, sy, sz)))
        ax, ay, az = sx - 2 * pad, sy - 2 * pad, sz - 2 * pad
        assert 192 <= ax <= 320 and 192 <= ay <= 320 and az == bench.BATCH_DEPTH
        assert sh["interior"] == ax * ay * az
        assert 45.0 <= sh["fcut"] <= 75.0
    # the thin-layer shots are the same crops as the sponge shots
    wide = bench.batch_shots(4, bench.BATCH_SEED)
    thin = bench.batch_shots(4, bench.BATCH_SEED, pad=bench.LEARNED_LAYER + 4)
    for w, t in zip(wide, thin):
        assert w["interior"] == t["interior"]
        d = bench.BATCH_PAD - bench.LEARNED_LAYER - 4
        assert tuple(a + d for a in w["origin"]) == t["origin"]


def test_learned_setup_geometry(dc):
    from dc_gb300 import learned
    st = learned.Setup(n=(48, 48, 48), layer=8)
    assert st.thin_sizes == (72, 72, 72)
    assert st.wide_sizes == tuple(v + 2 * st.wide_pad for v in st.thin_sizes)
    # the thin box sits inside the wide box; the sponge box origin is >= 0
    assert st.offset[0] + st.thin_sizes[0] <= st.wide_sizes[0]
    assert st.wide_pad + st.layer - st.sponge_absorb >= 0
    for src in learned.random_sources(st, 8, 3):
        assert all(4 + st.layer <= c < s - 4 - st.layer for c, s in zip(src, st.thin_sizes))
    n = dc.layer_cells(st.thin_sizes, st.layer)
    assert len(n) == np.prod([v - 8 for v in st.thin_sizes]) - np.prod([v - 16 for v in st.thin_sizes])
