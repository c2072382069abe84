"""Failure detection without a GPU fault: a non-finite entry injected on the host into
one walker's G (dqmc_set_green) must set that walker's status word and leave the
other walkers of the batch bitwise unaffected (no trap, no wait, nothing shared)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300

    return dqmc_gb300


@pytest.mark.parametrize("hbm", [False, True])  # shared-memory and HBM FP64 paths
def test_nonfinite_green_flags_only_that_walker(dq, hbm):
    descs = [dq.WalkerDesc(model=0, L=4, U=4.0, beta=1.0, Lt=10, pace=5, seed=70 + w) for w in range(3)]
    runs = []
    for poison in (False, True):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, hbm=hbm)
        for w in range(3):
            b.fields_random(w)
        b.init_greens()
        if poison:
            g = b.green(1, 0)
            g[0, 0] = np.nan
            b.set_green(1, 0, g)
        b.sweep_0_to_beta(measure=True)
        b.sweep_beta_to_0(measure=True)
        runs.append(b)
    clean, bad = runs
    assert bad.status(1) & (1 | 4), bad.status(1)  # non-finite G or ratio
    assert clean.status(1) == 0
    for w in (0, 2):
        assert clean.status(w) == 0 and bad.status(w) == 0
        np.testing.assert_array_equal(clean.fields(w), bad.fields(w))
        for s in (0, 1):
            np.testing.assert_array_equal(clean.green(w, s), bad.green(w, s))
    for b in runs:
        b.close()


def test_bounded_wait_timeout_flags_only_that_batch(dq):
    """A bounded device wait that runs out: the tensor-core wrap and B-chain products of one
    batch are given an iteration limit of 0 for their operand waits (dqmc_set_wait_limit, a
    test hook), so every such product gives up at once, drains the copies it issued, skips
    its output and sets status bit 8 (a timed-out wait) of its walker.  Nothing faults or
    hangs; a batch created beside it, and one created after it, run normally and match the
    FP64 path (identical decisions, max |dG| <= 1e-6)."""
    descs = [dq.WalkerDesc(model=1, L=12, U=4.0, mu=-0.5, beta=2.0, Lt=20, pace=5, seed=80 + w) for w in range(2)]

    def fresh(prec, trace=False):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec, trace=trace)
        for w in range(len(descs)):
            b.fields_random(w)
        b.init_greens()
        return b

    hooked = fresh(dq.MIXED)
    beside = fresh(dq.MIXED, trace=True)
    hooked.set_wait_limit(0)
    hooked.sweep_0_to_beta(measure=True)
    hooked.synchronize()
    assert all(hooked.status(w) & 8 for w in range(len(descs))), [hooked.status(w) for w in range(len(descs))]
    hooked.set_wait_limit(-1)
    hooked.close()
    after = fresh(dq.MIXED, trace=True)
    ref = fresh(dq.FP64, trace=True)
    for b in (beside, after, ref):
        b.sweep_0_to_beta(measure=True)
        b.sweep_beta_to_0(measure=True)
    for b in (beside, after):
        for w in range(len(descs)):
            assert b.status(w) == 0
            np.testing.assert_array_equal(b.fields(w), ref.fields(w))
            assert float(np.abs(b.trace(w) - ref.trace(w)).max()) <= 1e-6
    for b in (beside, after, ref):
        b.close()
