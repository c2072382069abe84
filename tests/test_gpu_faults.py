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
