"""Tensor-core path (DQMC_MIXED): wraps and B-chain products on the BF16 tensor
cores through exact integer slices (49 bits), submatrix Metropolis with tensor-core
block flushes, and for 128 <= N <= 768 the blocked Householder stabilization with
56-bit products; FP64 for the panels, the decisions and the ratios.

Bars: the product engine agrees with FP64 to 2^-38 of |A||B| (normwise) and is
exact on integer inputs; the mixed sweep makes the FP64 path's accept/reject
decisions and keeps max|dG| <= 1e-6 against it at every stabilization, on the same
fields and uniforms; the autotuner's pick is one of its timed candidates; walker
groups (graph branches) do not change any walker's result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300

    return dqmc_gb300


@pytest.mark.parametrize("n", [16, 37, 64, 100, 256, 300])
def test_product_engine_accuracy(dq, n):
    rng = np.random.default_rng(n)
    # rows / columns graded over many decades, like U diag(D) operands of the chain
    a = rng.standard_normal((n, n)) * np.exp(rng.uniform(-20, 20, n))[:, None]
    b = rng.standard_normal((n, n)) * np.exp(rng.uniform(-30, 30, n))[None, :]
    c = dq.product_check(a, b)
    ref = a @ b
    bound = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * n
    assert (np.abs(c - ref) <= 2.0 ** -38 * bound).all()


def test_product_engine_exact_on_integers(dq):
    rng = np.random.default_rng(7)
    n = 128
    a = rng.integers(-1000, 1000, (n, n)).astype(np.float64)
    b = rng.integers(-1000, 1000, (n, n)).astype(np.float64)
    np.testing.assert_array_equal(dq.product_check(a, b), a @ b)


def _run(dq, descs, precision, sweeps=1):
    b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=precision, trace=True)
    for w in range(len(descs)):
        b.fields_random(w)
    b.init_greens()
    out = []
    for _ in range(sweeps):
        b.trace_clear()
        b.sweep_0_to_beta(measure=True)
        b.sweep_beta_to_0(measure=True)
        out.append([(b.fields(w), b.trace(w)) for w in range(len(descs))])
    return b, out


@pytest.mark.parametrize("model,L,U,mu,beta,Lt,pace", [
    (1, 8, 4.0, -0.5, 4.0, 40, 8),     # attractive, the mixed configuration's model on 8x8
    (0, 6, 4.0, 0.0, 4.0, 80, 10),     # repulsive
    (1, 16, 4.0, -0.5, 2.0, 20, 8),    # 16x16
    (0, 12, 4.0, 0.0, 2.0, 20, 5),     # repulsive N = 144: tensor-core QR, two spins, partial panel
    (1, 12, 3.0, -0.3, 2.0, 20, 10),   # attractive N = 144
    (1, 16, 4.0, -0.5, 10.0, 100, 8),  # the mixed-precision configuration itself (beta = 10)
    (0, 17, 4.0, 0.0, 1.0, 10, 5),     # N = 289 > 256: 8 x 6-bit wrap slices, 9 x 6-bit stabilization slices
])
def test_mixed_sweep_dG_against_fp64(dq, model, L, U, mu, beta, Lt, pace):
    descs = [dq.WalkerDesc(model=model, L=L, U=U, mu=mu, beta=beta, Lt=Lt, pace=pace, seed=100 + w) for w in range(2)]
    bm, om = _run(dq, descs, dq.MIXED)
    bf, of = _run(dq, descs, dq.FP64)
    worst = 0.0
    for w in range(len(descs)):
        np.testing.assert_array_equal(om[0][w][0], of[0][w][0])  # same decisions
        worst = max(worst, float(np.abs(om[0][w][1] - of[0][w][1]).max()))
        assert bm.status(w) == 0
    assert worst <= 1e-6, worst


def test_autotuner_picks_a_timed_candidate(dq):
    """dqmc_init_greens times every (k, flush) candidate on the batch's own
    state and restores it: the pick is the fastest candidate, and the sweep that
    follows still matches the FP64 path (same decisions)."""
    descs = [dq.WalkerDesc(model=1, L=12, U=4.0, mu=-0.5, beta=2.0, Lt=20, pace=10, seed=300 + w) for w in range(3)]
    bm, om = _run(dq, descs, dq.MIXED)
    t = bm.tuning()
    cands = t["candidates"]
    assert {(c["kd"], c["tc_flush"]) for c in cands} >= {(32, 1), (32, 0), (16, 1), (16, 0), (8, 0)}
    best = min(cands, key=lambda c: c["ms_per_slice"])
    assert (t["kd"], t["tc_flush"]) == (best["kd"], best["tc_flush"])
    assert all(c["ms_per_slice"] > 0 for c in cands)
    # the products' tile shape: both shapes timed, the faster kept
    pc = t["product_candidates"]
    assert sorted(c["tile"] for c in pc) == [0, 1] and all(c["ms_per_slice"] > 0 for c in pc)
    assert t["product_tile"] == min(pc, key=lambda c: c["ms_per_slice"])["tile"]
    bf, of = _run(dq, descs, dq.FP64)
    assert {c["tc_flush"] for c in bf.tuning()["candidates"]} == {0}
    for w in range(len(descs)):
        np.testing.assert_array_equal(om[0][w][0], of[0][w][0])
        assert float(np.abs(om[0][w][1] - of[0][w][1]).max()) <= 1e-6


def test_walker_groups_give_identical_walkers(dq, monkeypatch):
    """The half-sweep of 16 tensor-core-path walkers as one branch and as four
    forked walker groups (DQMC_STREAM_GROUPS): every walker's fields, Green's
    function and observables are bitwise the same (Philox keyed by the walker's
    batch index, no work shared between walkers)."""
    descs = [dq.WalkerDesc(model=1, L=12, U=4.0, mu=-0.5, beta=2.0, Lt=20, pace=5, seed=300 + w) for w in range(16)]
    res = []
    for groups in ("1", "4"):
        monkeypatch.setenv("DQMC_STREAM_GROUPS", groups)
        b = dq.Batch(descs, rng=dq.RNG_PHILOX, precision=dq.MIXED)
        for w in range(16):
            b.fields_random(w)
        b.init_greens()
        for k in range(2):
            b.sweep_0_to_beta(measure=True)
            b.sweep_beta_to_0(measure=True)
        res.append(([b.fields(w) for w in range(16)], [b.green(w, 0) for w in range(16)],
                    b.observables_all(), [b.status(w) for w in range(16)]))
        b.close()
    (f1, g1, o1, s1), (f4, g4, o4, s4) = res
    for w in range(16):
        np.testing.assert_array_equal(f1[w], f4[w])
        np.testing.assert_array_equal(g1[w], g4[w])
        assert s1[w] == 0 and s4[w] == 0
    np.testing.assert_array_equal(o1[0], o4[0])
    np.testing.assert_array_equal(o1[1], o4[1])


def test_split_submatrix_equals_fused(dq, monkeypatch):
    """The submatrix updates split per 32-site block (a decision kernel, then a flush spread
    over several CTAs per walker) do the fused kernel's arithmetic element for element:
    with the tuner held to each kind (DQMC_METROPOLIS_KIND), fields, G and observables are
    bitwise equal after two sweep pairs, for N = 144 (two spins) and N = 289 (partial tiles)."""
    for L, model in ((12, 0), (17, 1)):
        descs = [dq.WalkerDesc(model=model, L=L, U=4.0, mu=-0.3 * model, beta=1.0, Lt=10, pace=5, seed=400 + w)
                 for w in range(3)]
        res = []
        for kind in ("2", "3"):
            monkeypatch.setenv("DQMC_METROPOLIS_KIND", kind)
            b = dq.Batch(descs, rng=dq.RNG_PHILOX, precision=dq.MIXED)
            for w in range(3):
                b.fields_random(w)
            b.init_greens()
            assert b.tuning()["tc_flush"] == int(kind)
            for _ in range(2):
                b.sweep_0_to_beta(measure=True)
                b.sweep_beta_to_0(measure=True)
            res.append(([b.fields(w) for w in range(3)], [b.green(w, s) for w in range(3) for s in (0, 1)],
                        b.observables_all(), [b.status(w) for w in range(3)]))
            b.close()
        (f2, g2, o2, s2), (f3, g3, o3, s3) = res
        assert s2 == [0, 0, 0] and s3 == [0, 0, 0]
        for a, c in zip(f2, f3):
            np.testing.assert_array_equal(a, c)
        for a, c in zip(g2, g3):
            np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(o2[0], o3[0])


@pytest.mark.parametrize("model,L", [(1, 12), (0, 17)])  # 7-slice (N = 144) and 8-slice (N = 289) products
def test_product_tile_shapes_agree(dq, monkeypatch, model, L):
    """The wrap and chain products with 128 x 32 and with 128 x 64 output tiles (the tuner
    held to each by DQMC_PRODUCT_TILE): the same decisions and G to 1e-10 after a sweep pair."""
    descs = [dq.WalkerDesc(model=model, L=L, U=4.0, mu=-0.2 * model, beta=1.0, Lt=10, pace=5, seed=450 + w)
             for w in range(2)]
    res = []
    for tile in ("0", "1"):
        monkeypatch.setenv("DQMC_PRODUCT_TILE", tile)
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=dq.MIXED)
        for w in range(2):
            b.fields_random(w)
        b.init_greens()
        assert b.tuning()["product_tile"] == int(tile)
        b.sweep_0_to_beta(measure=True)
        b.sweep_beta_to_0(measure=True)
        res.append(([b.fields(w) for w in range(2)], [b.green(w, 0) for w in range(2)], [b.status(w) for w in range(2)]))
        b.close()
    (f0, g0, s0), (f1, g1, s1) = res
    assert s0 == [0, 0] and s1 == [0, 0]
    for w in range(2):
        np.testing.assert_array_equal(f0[w], f1[w])
        assert float(np.abs(g0[w] - g1[w]).max()) <= 1e-10
