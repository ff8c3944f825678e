"""The FMA solver's tile geometry, checked on the CPU for many frame sizes.

`solver_fma_solve_kernel` (video-stream-consistency_gb300/csrc/vsc_solver.cu:
`pl_job`, `pl_mode`, `pl_iterate`) runs 8-step rounds on 128 x 72 tiles whose
112 x 56 interiors tile the frame.  Tile (tx, ty) starts at
(112 tx - 8, 56 ty - 8); the bottom row of tiles is moved up to end on the
frame's last row (oy = h - 64) when it has an upper neighbour row and at
least 8 rows of its own.  A tile of round k waits only for its 3 x 3
neighbourhood's round k - 1, so every frame pixel a tile reads must lie in
the interior of a tile of that neighbourhood, and every frame pixel must lie
in some interior.  The edge tests without per-pixel tests (kPlLanes) rely on
rows 0, h - 2 and h - 1 sitting at fixed rows of the tile.  These rules are
restated here; the GPU tests check the kernel's results bit for bit on a
handful of sizes, these checks cover the geometry on many more.
"""
import itertools

import pytest

W_T, H_T, RING = 128, 72, 8            # tile, temporal ring (one round's steps)
IW, IH = W_T - 2 * RING, H_T - 2 * RING  # interior: 112 x 56


def tile_origin(tx, ty, w, h):
    ty_n = (h + IH - 1) // IH
    ox, oy = tx * IW - RING, ty * IH - RING
    if ty == ty_n - 1 and ty > 0 and h - ty * IH >= RING:
        oy = h - H_T + RING
    return ox, oy


def pl_mode(ox, oy, w, h):
    if ox >= 1 and oy >= 1 and ox + W_T - 1 <= w - 3 and oy + H_T - 1 <= h - 3:
        return "all"
    row0 = oy <= 0 <= oy + H_T - 1
    last2 = oy <= h - 1 and oy + H_T - 1 >= h - 2
    if w % 4 == 0 and ox % 4 == 0 and (not row0 or oy == -RING) and (not last2 or oy == h - H_T + RING):
        return "lanes"
    return "every"


SIZES = sorted(set([(w, h) for w in (4, 8, 64, 100, 128, 236, 240, 960, 1920, 3840)
                    for h in (1, 2, 17, 40, 56, 57, 61, 63, 64, 65, 72, 100, 112, 119, 120, 121, 130, 360, 540, 1080,
                              2160)]))


@pytest.mark.parametrize("w,h", SIZES)
def test_interiors_cover_the_frame_and_each_tile_reads_only_its_neighbours(w, h):
    tx_n, ty_n = (w + IW - 1) // IW, (h + IH - 1) // IH
    org = {(tx, ty): tile_origin(tx, ty, w, h) for tx in range(tx_n) for ty in range(ty_n)}

    def interior_rows(ty):
        oy = org[(0, ty)][1]
        return max(0, oy + RING), min(h, oy + RING + IH)

    def interior_cols(tx):
        ox = org[(tx, 0)][0]
        return max(0, ox + RING), min(w, ox + RING + IW)

    # rows and columns factor: check each axis
    for axis_n, span in ((ty_n, interior_rows), (tx_n, interior_cols)):
        covered = set()
        for t in range(axis_n):
            lo, hi = span(t)
            covered.update(range(lo, hi))
        assert covered == set(range(h if span is interior_rows else w))
    for (tx, ty), (ox, oy) in org.items():
        # every frame row / column the tile loads comes from a neighbour's interior
        rows = range(max(0, oy), min(h, oy + H_T))
        cols = range(max(0, ox), min(w, ox + W_T))
        nb_rows = set().union(*(range(*interior_rows(t)) for t in range(max(0, ty - 1), min(ty_n, ty + 2))))
        nb_cols = set().union(*(range(*interior_cols(t)) for t in range(max(0, tx - 1), min(tx_n, tx + 2))))
        assert set(rows) <= nb_rows, (tx, ty)
        assert set(cols) <= nb_cols, (tx, ty)
        # TMA coordinates: a tile's x origin and its interior's are multiples of 4 floats
        assert ox % 4 == 0 and (ox + RING) % 4 == 0
        # its interior lies inside what it loads, with the full ring where the frame goes on
        assert oy + RING >= 0 and oy + RING + IH <= oy + H_T


@pytest.mark.parametrize("w,h", SIZES)
def test_fixed_edge_rows_and_lanes_of_the_lane_mode(w, h):
    """kPlLanes tests column 0 at lane 2's first column (tile x origin -8),
    columns w - 2, w - 1 as the last two columns of one lane (width a multiple
    of 4), row 0 at warp 1's row 2 (oy = -8) and rows h - 2, h - 1 at warp
    10's rows 2 and 3 (oy = h - 64); a tile holding any of them elsewhere
    takes the per-pixel tests."""
    tx_n, ty_n = (w + IW - 1) // IW, (h + IH - 1) // IH
    for tx, ty in itertools.product(range(tx_n), range(ty_n)):
        ox, oy = tile_origin(tx, ty, w, h)
        if pl_mode(ox, oy, w, h) != "lanes":
            continue
        if oy <= 0 <= oy + H_T - 1:
            assert 0 - oy == 6 * 1 + 2
        for r in (h - 2, h - 1):
            if oy <= r <= oy + H_T - 1:
                assert r - oy in (6 * 10 + 2, 6 * 10 + 3)
        if ox <= 0 <= ox + W_T - 1:
            assert (0 - ox) % 4 == 0 and (0 - ox) // 4 == 2
        if ox <= w - 2 <= ox + W_T - 1:
            assert (w - 2 - ox) % 4 == 2 and (w - 1 - ox) % 4 == 3
