"""The batched kernel's work queue (queue_front / queue_back in
thirring2d_gb300/csrc/tg_batch_impl.cuh), restated on the CPU: one 64-bit word,
front draws (the teams, atomic add) in its low half and back draws (the filler
blocks beside a cluster launch, compare-and-swap, positions at or after `lo`
only) in its high half.  Under any interleaving every queue position must be
handed out exactly once, and never one before `lo` from the back."""
import numpy as np
import pytest


def front(word, n):
    old = word[0]
    word[0] = (old + 1) & ((1 << 64) - 1)
    f, b = old & 0xFFFFFFFF, old >> 32
    return f if f + b < n else n


def back(word, n, lo, stale=None):
    # `stale`: a value read earlier (the CAS may fail on it and retry)
    old = word[0] if stale is None else stale
    for _ in range(1 << 20):
        f, b = old & 0xFFFFFFFF, old >> 32
        t = n - 1 - b
        if f + b >= n or t < lo:
            return n
        if word[0] == old:            # compare-and-swap
            word[0] = old + (1 << 32)
            return t
        old = word[0]
    return n


@pytest.mark.parametrize("n,lo,front_share", [(512, 36, 0.9), (512, 36, 0.3), (10, 0, 0.5), (10, 10, 0.5),
                                              (1, 0, 0.5), (300, 299, 0.2)])
def test_every_position_once(n, lo, front_share):
    rng = np.random.default_rng(n + lo)
    for trial in range(50):
        word = [0]
        taken = []
        front_done = back_done = False
        while not (front_done and back_done):
            use_front = (rng.random() < front_share and not front_done) or back_done
            if use_front:
                q = front(word, n)
                if q >= n:
                    front_done = True
                else:
                    taken.append(("f", q))
            else:
                stale = word[0] if rng.random() < 0.5 else None
                if stale is not None and not front_done and rng.random() < 0.5:
                    q = front(word, n)          # a team draws between the read and the CAS
                    if q >= n:
                        front_done = True
                    else:
                        taken.append(("f", q))
                q = back(word, n, lo, stale)
                if q >= n:
                    back_done = True
                else:
                    assert q >= lo
                    taken.append(("b", q))
        positions = sorted(q for _, q in taken)
        assert positions == list(range(n)), (n, lo, trial)


def test_front_alone_takes_all_in_order():
    word = [0]
    assert [front(word, 7) for _ in range(9)] == [0, 1, 2, 3, 4, 5, 6, 7, 7]
