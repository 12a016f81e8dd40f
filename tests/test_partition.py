"""Race and bounds audit of the stencil's work partition, on the CPU.

compute-sanitizer is not available on the GPU pool, so the partition that
decides which warp touches which site is checked here instead.  The functions
below restate, line for line, the index arithmetic of
thirring2d_gb300/csrc/tg_stencil.cuh: for_warp_rows (a grid's warps over the
(strip, t) rows, the single-lattice kernels and the persistent solver),
stencil_team (a batched chain's team), and march_segment (the sites one warp
reads and writes for one segment, chunked by kMarchT rows with the edge
operands fetched by the first 2 * kMarchT lanes).  For every benchmark and test
lattice shape and for the grid shapes the launchers use, each site must be
written by exactly one (warp, lane) per pass -- two warps writing one site would
race -- and every address read must lie inside the lattice.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "thirring2d_gb300", "csrc")


def _constant(name: str, header: str) -> int:
    with open(os.path.join(CSRC, header)) as f:
        m = re.search(rf"constexpr int {name} = (\d+);", f.read())
    assert m, f"{name} not found in {header}"
    return int(m.group(1))


K_MARCH_T = _constant("kMarchT", "tg_internal.cuh")


def warp_segments_grid(nt, nx, grid, wpb):
    """for_warp_rows: yields (warp, xw, ta, tb) for every warp of the grid."""
    rows = (nx >> 5) * nt
    nw = grid * wpb
    for gw in range(nw):
        r, r1 = rows * gw // nw, rows * (gw + 1) // nw
        while r < r1:
            xw = r // nt
            ta = r - xw * nt
            tb = ta + (r1 - r) if r1 - r < nt - ta else nt
            yield gw, xw, ta, tb
            r += tb - ta


def warp_segments_team(nt, nx, nblocks, wpb):
    """stencil_team's march branch: the team's warps over the chain's rows."""
    rows = (nx >> 5) * nt
    nw = nblocks * wpb
    for w in range(nw):
        r, r1 = rows * w // nw, rows * (w + 1) // nw
        while r < r1:
            xw = r // nt
            ta = r - xw * nt
            tb = ta + (r1 - r) if r1 - r < nt - ta else nt
            yield w, xw, ta, tb
            r += tb - ta


def segment_accesses(nt, nx, xw, ta, tb):
    """march_segment: (reads, writes) site indices of one warp's segment."""
    V = nt * nx
    x0 = xw << 5
    xle = nx - 1 if x0 == 0 else x0 - 1
    xre = 0 if x0 + 32 == nx else x0 + 32
    tm = nt - 1 if ta == 0 else ta - 1
    reads, writes = [], []
    for lane in range(32):
        x = x0 + lane
        reads += [tm * nx + x, ta * nx + x]              # psi(t-1), Wt(t-1), psi(t)
    t = ta
    while t + K_MARCH_T <= tb:                           # chunks: edge operands by lanes < 2 kMarchT
        for lane in range(2 * K_MARCH_T):
            rr = t + (lane if lane < K_MARCH_T else lane - K_MARCH_T)
            reads.append(rr * nx + (xle if lane < K_MARCH_T else xre))
            if lane < K_MARCH_T:
                reads.append(rr * nx + xle)             # Wx entering column x0
        for i in range(K_MARCH_T):
            tt = t + i
            tp = 0 if tt + 1 == nt else tt + 1
            for lane in range(32):
                reads += [tp * nx + x0 + lane, tt * nx + x0 + lane]
                writes.append(tt * nx + x0 + lane)
        t += K_MARCH_T
    while t < tb:                                        # leftover rows: lanes 0 and 31 fetch their own edges
        tp = 0 if t + 1 == nt else t + 1
        for lane in range(32):
            xe = xre if lane == 31 else xle
            reads += [t * nx + xe, t * nx + xle, tp * nx + x0 + lane, t * nx + x0 + lane]
            writes.append(t * nx + x0 + lane)
        t += 1
    assert all(0 <= a < V for a in reads), "read outside the lattice"
    return writes


def audit(nt, nx, segments):
    V = nt * nx
    count = [0] * V
    for _, xw, ta, tb in segments:
        assert 0 <= xw < nx // 32 and 0 <= ta < tb <= nt
        for s in segment_accesses(nt, nx, xw, ta, tb):
            count[s] += 1
    assert min(count) == 1 and max(count) == 1, "a site written by no warp or by two"


# single-lattice kernels (kBlock-thread blocks, grids of one wave or fewer) and
# the persistent solver (152 x 512 or 304 x 256 threads); lattices whose nx is a
# multiple of 32 use the march
GRID_SHAPES = [(1, 8), (4, 16), (152, 16), (304, 8), (456, 8), (7, 8)]
SHAPES = [(32, 32), (16, 32), (36, 32), (64, 96), (8, 64), (128, 128), (96, 128), (1024, 64), (4, 32), (2, 64),
          (64, 64), (32, 96), (32, 64)]


@pytest.mark.parametrize("nt,nx", SHAPES)
def test_grid_partition_writes_each_site_once(nt, nx):
    for grid, wpb in GRID_SHAPES:
        audit(nt, nx, warp_segments_grid(nt, nx, grid, wpb))


def test_grid_partition_benchmark_lattice():
    # the 1024^2 workload on the persistent solver's two grid shapes (every
    # site, once): 2432 warps over 32768 rows
    for grid, wpb in ((152, 16), (304, 8)):
        audit(1024, 1024, warp_segments_grid(1024, 1024, grid, wpb))


@pytest.mark.parametrize("side", [32, 64, 96, 128])
def test_team_partition_writes_each_site_once(side):
    # batched chains with nx a multiple of 32: one block (4, 8 or 16 warps) or
    # a 2- or 4-block cluster of 512 threads
    for nblocks, wpb in ((1, 4), (1, 8), (1, 16), (2, 16), (4, 16), (4, 8)):
        audit(side, side, warp_segments_team(side, side, nblocks, wpb))


def test_ranges_differ_by_at_most_one_row():
    # the balance for_warp_rows promises: contiguous ranges of floor or ceil rows
    rows = 32 * 1024
    for nw in (2432, 2433, 4864):
        sizes = [rows * (w + 1) // nw - rows * w // nw for w in range(nw)]
        assert max(sizes) - min(sizes) <= 1 and sum(sizes) == rows


def fused_segment_accesses(nt, nx, xw, ta, tb):
    """march_mdagm (thirring2d_gb300/csrc/tg_fused.cuh): (reads, writes) of one
    warp's segment -- v and the links at rows ta-2 .. tb+1 of its columns, the
    operands beyond its edges, and the five v and four links of every
    recomputed edge u."""
    V = nt * nx
    x0 = xw << 5
    xle = nx - 1 if x0 == 0 else x0 - 1
    xre = 0 if x0 + 32 == nx else x0 + 32

    def wrap(t):
        assert -nt <= t < 2 * nt
        return t + nt if t < 0 else (t - nt if t >= nt else t)

    def u_at(t, c):
        tp, tm = wrap(t + 1), wrap(t - 1)
        cp, cm = (0 if c + 1 == nx else c + 1), (nx - 1 if c == 0 else c - 1)
        return [t * nx + c, tp * nx + c, tm * nx + c, t * nx + cp, t * nx + cm, t * nx + c, tm * nx + c, t * nx + c,
                t * nx + cm]

    reads, writes = [], []
    cols = [x0 + lane for lane in range(32)]
    for r in (wrap(ta - 2), wrap(ta - 1), ta, wrap(ta + 1)):    # prologue: v, Wt, Wx
        reads += [r * nx + c for c in cols]
    for r in (wrap(ta - 1), ta):                                  # prologue edges (lanes 0 and 31)
        reads += [r * nx + xle, r * nx + xre]
    t = ta
    while t + K_MARCH_T <= tb:
        for i in range(K_MARCH_T):
            reads += [wrap(t + 2 + i) * nx + c for c in cols] + [wrap(t + 1 + i) * nx + c for c in cols]
            for c in (xle, xre):
                reads.append(wrap(t + 1 + i) * nx + c)
                reads += u_at(t + i, c)
            writes += [(t + i) * nx + c for c in cols]
        t += K_MARCH_T
    while t < tb:
        reads += [wrap(t + 2) * nx + c for c in cols] + [wrap(t + 1) * nx + c for c in cols]
        for c in (xle, xre):
            reads.append(wrap(t + 1) * nx + c)
            reads += u_at(t, c)
        writes += [t * nx + c for c in cols]
        t += 1
    assert all(0 <= a < V for a in reads), "read outside the lattice"
    return writes


@pytest.mark.parametrize("nt,nx", SHAPES)
def test_fused_march_partition_writes_each_site_once(nt, nx):
    """The fused M^dag M march over the persistent solver's grid shapes: every
    site written by exactly one warp and lane per pass, every read inside the
    lattice (the halo rows and edge columns wrap)."""
    if nt < 2:
        return
    for grid, wpb in ((1, 8), (4, 16), (152, 16), (304, 8)):
        V = nt * nx
        count = [0] * V
        for _, xw, ta, tb in warp_segments_grid(nt, nx, grid, wpb):
            for s in fused_segment_accesses(nt, nx, xw, ta, tb):
                count[s] += 1
        assert min(count) == 1 and max(count) == 1
