"""Checkpoint and resume: a lattice restored from a checkpoint continues the
chain bitwise (same dH, accept decisions and field) as the lattice it was taken
from, with either random stream.  The header is checked against the lattice it
is loaded into."""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


def run(L, hp, n):
    out = []
    for _ in range(n):
        r = L.update_gauge(hp)
        assert r.status == 0
        out.append((r.dH, r.accepted, r.cg_iterations))
    return out, L.get_gauge()


@pytest.mark.parametrize("rng_kind", ["mt", "philox"])
def test_resume_is_bitwise(tg, tmp_path, rng_kind):
    rng = tg.native.RNG_MT if rng_kind == "mt" else tg.native.RNG_PHILOX
    hp = tg.hmc_params(nsteps=8, tau=0.5, rng=rng, seed=77)
    L = tg.Lattice(24, 16, 0.15, 0.6, 0.2, -1, 1)
    L.seed_mersenne(2024)
    L.set_gauge(np.random.default_rng(5).normal(0, 0.4, (24, 16, 2)))
    run(L, hp, 3)
    path = tmp_path / "state.ckpt"
    L.save(str(path))
    assert path.stat().st_size == 7560 + 24 * 16 * 2 * 8
    want, A_want = run(L, hp, 3)

    R = tg.Lattice(24, 16, 0.9, 0.1, 0.0, -1, 1)     # other couplings, field and stream: all replaced by the load
    R.seed_mersenne(1)
    R.set_gauge(np.zeros((24, 16, 2)))
    R.load(str(path))
    assert (R.params.m, R.params.g, R.params.mu) == (0.15, 0.6, 0.2)
    got, A_got = run(R, hp, 3)
    assert got == want
    assert np.array_equal(A_got, A_want)
    if rng_kind == "mt":                                # the host stream continues too
        assert np.array_equal(R.mersenne(5), L.mersenne(5))


def test_checkpoint_header_and_refusals(tg):
    L = tg.Lattice(8, 6, 0.3, 0.5, 0.1, -1, 1)
    L.seed_mersenne(9)
    A = np.random.default_rng(1).normal(size=(8, 6, 2))
    L.set_gauge(A)
    ck = L.checkpoint()
    assert ck[:8] == b"TGCKPT01"
    version, nt, nx, bc_t, bc_x = struct.unpack_from("<5i", ck, 8)
    assert (version, nt, nx, bc_t, bc_x) == (1, 8, 6, -1, 1)
    assert struct.unpack_from("<3d", ck, 40) == (0.3, 0.5, 0.1)
    assert np.array_equal(np.frombuffer(ck, "<f8", offset=7560).reshape(8, 6, 2), L.get_gauge())

    with pytest.raises(tg.native.TGError):
        tg.Lattice(8, 8, 0.3).restore(ck)                  # another size
    with pytest.raises(tg.native.TGError):
        tg.Lattice(8, 6, 0.3, 0.5, 0.1, 1, 1).restore(ck)  # another boundary condition
    with pytest.raises(tg.native.TGError):
        L.restore(ck[:-8])                                 # truncated
    with pytest.raises(tg.native.TGError):
        L.restore(b"XGCKPT01" + ck[8:])                    # not a checkpoint
    with pytest.raises(tg.native.TGError):
        L.restore(ck[:8] + struct.pack("<i", 2) + ck[12:])   # unknown version
    L.restore(ck)                                          # a good one still loads
    assert np.array_equal(L.get_gauge(), A)
    out = np.full((8, 6, 2), np.nan)                       # into a caller's buffer
    assert L.get_gauge(out) is out and np.array_equal(out, A)
    with pytest.raises(ValueError):
        L.get_gauge(np.empty((8, 6, 2), np.float32))


BATCH = [dict(nt=16, nx=16, m=0.3, g=0.5, mu=0.0, bc_t=-1, bc_x=1, seed=71),
         dict(nt=32, nx=32, m=0.2, g=0.8, mu=0.1, bc_t=-1, bc_x=-1, seed=72),
         dict(nt=24, nx=40, m=0.4, g=0.6, mu=0.0, bc_t=-1, bc_x=1, seed=73),
         dict(nt=64, nx=64, m=0.25, g=0.7, mu=0.0, bc_t=-1, bc_x=1, seed=74)]


def run_batch(tg, B, n):
    bp = tg.batch_params(nsteps=6, block=51201, cg=tg.cg_params(rel_tol=1e-10, abs_tol2=0.0, precision=1))
    out = []
    for _ in range(n):
        out.append([(r.dH, r.accepted, r.cg_iterations) for r in B.trajectory(bp)])
    return out, [B.get_gauge(i) for i in range(len(BATCH))]


def test_batch_resume_is_bitwise(tg, tmp_path):
    rng = np.random.default_rng(8)
    B = tg.Batch(BATCH)
    for i, c in enumerate(BATCH):
        B.set_gauge(i, rng.normal(0, 0.2, (c["nt"], c["nx"], 2)))
    run_batch(tg, B, 2)
    path = tmp_path / "batch.ckpt"
    B.save(str(path))
    sites = sum(c["nt"] * c["nx"] for c in BATCH)
    assert path.stat().st_size == 24 + 56 * len(BATCH) + 16 * sites
    want, A_want = run_batch(tg, B, 2)
    B.close()

    R = tg.Batch(BATCH)                          # fresh: fields 0, trajectory counters 0
    R.load(str(path))
    got, A_got = run_batch(tg, R, 2)
    assert got == want
    assert all(np.array_equal(a, b) for a, b in zip(A_got, A_want))
    ck = R.checkpoint()
    assert ck[:8] == b"TGBATCH1"
    assert struct.unpack_from("<2iq", ck, 8) == (1, len(BATCH), sites)
    assert [struct.unpack_from("<Q", ck, 24 + 56 * i + 48)[0] for i in range(len(BATCH))] == [4] * len(BATCH)
    other = [dict(c) for c in BATCH]
    other[2]["m"] = 0.41
    with pytest.raises(tg.native.TGError):
        tg.Batch(other).restore(ck)                   # another chain
    with pytest.raises(tg.native.TGError):
        tg.Batch(BATCH[:3]).restore(ck)               # another chain count
    with pytest.raises(tg.native.TGError):
        R.restore(ck[:-16])                           # truncated
    R.close()
