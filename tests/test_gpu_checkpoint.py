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
