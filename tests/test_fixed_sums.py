"""The fixed-point grid sums of the mixed persistent CG (grid_total_fx in
thirring2d_gb300/csrc/tg_pcg.cu), restated on the CPU: one 64-bit word per kind
of sum takes each block's arrival (bits 0-8), overflow flag (bits 9-17) and
block total as an integer at a power-of-two scale (bits 18-63); a block reads
the difference to the word's value at its previous use.  The fields must
decode exactly whatever the word's history (it wraps modulo 2^64), an
overflowing block must send every block to the exact path, and the scale must
come out the same from the exponent bits in every block."""
import math
import re
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = open(os.path.join(ROOT, "thirring2d_gb300", "csrc", "tg_pcg.cu")).read()


def _const(name):
    m = re.search(rf"\b{name} = ([0-9.]+)[;,]", SRC)
    assert m, name
    return float(m.group(1))


OVF_SHIFT = int(_const("kFxOvfShift"))
SUM_SHIFT = int(_const("kFxSumShift"))
MAX_GRID = int(_const("kFxMaxGrid"))
BLOCK_CAP = _const("kFxBlockCap")
MIN_BITS = int(_const("kFxMinBits"))
M64 = (1 << 64) - 1


def scale_of(total, nb):
    """FxSum::rescale: 2^(29 - (exponent(total) - floor(log2 nb)))."""
    if not (total > 0) or not math.isfinite(total):
        return None
    lt = math.frexp(total)[1] - 1          # the unbiased exponent field of a normal double
    lg = nb.bit_length() - 1
    e = min(max(29 - (lt - lg), -1000), 1000)
    return 2.0 ** e


def add_of(b, scale):
    sc = float(np.float64(np.float32(b))) * scale
    if sc >= 0.0 and sc < BLOCK_CAP:
        return (int(np.rint(sc)) << SUM_SHIFT) | 1, False
    return (1 << OVF_SHIFT) | 1, True


def decode(cur, last, nb):
    d = (cur - last) & M64
    assert d & MAX_GRID == nb
    ovf = (d >> OVF_SHIFT) & MAX_GRID
    fsum = d >> SUM_SHIFT
    return ovf, fsum


def test_layout_holds_511_blocks():
    assert MAX_GRID == 511 and OVF_SHIFT == 9 and SUM_SHIFT == 18
    assert MAX_GRID * (1 << (OVF_SHIFT)) < (1 << SUM_SHIFT)          # flags never carry into the sum
    assert MAX_GRID * BLOCK_CAP < 2.0 ** (64 - SUM_SHIFT)             # nor the sum past the word
    assert BLOCK_CAP < 2.0 ** 53                                       # block integers exact in FP64


@pytest.mark.parametrize("nb", [2, 152, 304, 511])
def test_fields_decode_exactly_across_wraps(nb):
    rng = np.random.default_rng(nb)
    word = (1 << 64) - 12345                      # a word about to wrap
    last = word
    total_prev = float(nb)
    for it in range(200):
        scale = scale_of(total_prev, nb)
        parts = rng.uniform(0.2, 1.8, nb).astype(np.float32) * np.float32(total_prev / nb)
        adds = [add_of(p, scale) for p in parts]
        for a, _ in adds:                           # any order: integer addition
            word = (word + a) & M64
        ovf, fsum = decode(word, last, nb)
        last = word
        assert ovf == 0
        exact = sum(int(np.rint(float(p) * scale)) for p in parts)
        assert fsum == exact
        total = fsum / scale
        ref = float(np.sum(parts.astype(np.float64)))
        assert abs(total - ref) <= nb * 0.5 / scale + 1e-15 * ref
        assert fsum >= nb << MIN_BITS               # a steady sum stays on the fixed-point path
        assert nb * 0.5 / fsum <= 2.0 ** -27       # and is then within 2^-27 of the block totals' sum
        total_prev = total * rng.uniform(0.5, 1.5)


def test_overflow_and_small_totals_take_the_exact_path():
    nb = 152
    scale = scale_of(1.0, nb)
    # one block 1000 times its expected share: flagged, counted, its value left out
    parts = np.full(nb, 1.0 / nb, np.float32)
    parts[7] *= 1000
    word = 0
    flags = 0
    for p in parts:
        a, f = add_of(p, scale)
        word = (word + a) & M64
        flags += f
    ovf, _ = decode(word, 0, nb)
    assert ovf == flags == 1
    # a sum 20 times below the last: too few significant bits, exact path
    parts = np.full(nb, 1.0 / nb / 20, np.float32)
    word = 0
    for p in parts:
        word = (word + add_of(p, scale)[0]) & M64
    ovf, fsum = decode(word, 0, nb)
    assert ovf == 0 and fsum < nb << MIN_BITS
    # NaN and negative totals are flagged
    assert add_of(float("nan"), scale)[1] and add_of(-1.0, scale)[1]


def test_scale_is_a_power_of_two_near_2_29_per_block():
    for total in (1e-300, 3.7e-12, 1.0, 123456.0, 5e200):
        for nb in (2, 152, 304):
            s = scale_of(total, nb)
            assert math.frexp(s)[0] == 0.5          # a power of two
            per_block = total / nb * s
            assert 2 ** 27 <= per_block < 2 ** 31 or s in (2.0 ** 1000, 2.0 ** -1000)
