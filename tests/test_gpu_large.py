"""The large and the uneven batches on the GPU.

Large walkers: repulsive Hubbard on a 24x24 lattice (N = 576), U = 4, mu = 0,
dtau = 0.1, stabilization every 6 slices; at beta = 12 (Lt = 120) the tensor-core
path (rank-32 submatrix updates with tensor-core flushes, 48-bit wraps, blocked
Householder stabilization with 54-bit products) against the FP64 path on the same
fields and uniforms, and at beta = 1.2 (Lt = 12) the FP64 path against the oracle,
including the time-displaced half-sweep (src/dqmc_walker.cpp:424-524,
include/utils/numerical_stable.hpp:246-325) at 12 tau points.

Uneven batch: walkers of sides 6, 8, 10 and 12 (N = 36 ... 144) with |U| and beta
drawn per walker from std::mt19937_64(7) (dqmc_gb300.workloads.uneven_batch), all
in one launch sequence, tensor-core path against FP64.

Bars: identical decisions; max |dG| <= 1e-6 against FP64 at every stabilization
(tensor-core path); G, G(k,tau) sums, G(beta,0) and G(0,beta) within 1e-10
relative of the oracle (FP64 path).
"""
import numpy as np
import pytest

from test_gpu_parity import _rel_err, _run_pair

pytestmark = pytest.mark.gpu

LARGE = dict(model=0, L=24, U=4.0, mu=0.0, pace=6)


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300

    return dqmc_gb300


def _mixed_vs_fp64(dq, descs, sweeps=1):
    """Both precisions from the same seeds: per-walker identical fields after every
    pair, and max |dG| (absolute, G is O(1)) at every stabilization, in order."""
    runs = []
    for prec in (dq.MIXED, dq.FP64):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec, trace=True)
        for w in range(len(descs)):
            b.fields_random(w)
        b.init_greens()
        per = []
        for _ in range(sweeps):
            b.trace_clear()
            b.sweep_0_to_beta(measure=True)
            b.sweep_beta_to_0(measure=True)
            per.append([(b.fields(w), b.trace(w)) for w in range(len(descs))])
        runs.append((b, per))
    (bm, om), (bf, of) = runs
    ns_max = max(-(-d.Lt // d.pace) for d in descs)
    series = []
    for p in range(sweeps):
        for w, d in enumerate(descs):
            np.testing.assert_array_equal(om[p][w][0], of[p][w][0], err_msg=f"walker {w}: decisions differ")
            ns = -(-d.Lt // d.pace)
            for h in range(2):
                for i in range(ns):
                    k = h * ns_max + i
                    series.append(float(np.abs(om[p][w][1][k] - of[p][w][1][k]).max()))
    for w in range(len(descs)):
        assert bm.status(w) == 0 and bf.status(w) == 0
    return bm, bf, series


def test_large_mixed_against_fp64(dq):
    """Two 24x24 walkers at beta = 12, Lt = 120, pace 6: one forth-and-back pair."""
    descs = [dq.WalkerDesc(beta=12.0, Lt=120, seed=500 + w, **LARGE) for w in range(2)]
    bm, _, series = _mixed_vs_fp64(dq, descs)
    t = bm.tuning()
    print(f"MEASURED 24x24 beta=12 mixed vs fp64: max|dG| {max(series):.2e} over {len(series)} stabilizations; "
          f"tuner kd={t['kd']} flush={t['tc_flush']}; series {' '.join(f'{e:.1e}' for e in series)}")
    assert max(series) <= 1e-6


def test_large_fp64_against_oracle(dq, oracle_mod):
    """One 24x24 walker at beta = 1.2, Lt = 12, pace 6 against the oracle."""
    d = dq.WalkerDesc(beta=1.2, Lt=12, seed=577, **LARGE)
    errs = []
    _run_pair(dq, oracle_mod, [d], sweeps=1, errs=errs)
    print(f"MEASURED 24x24 fp64 vs oracle: max rel |dG| {max(errs):.2e}")


def test_large_dynamic_against_oracle(dq, oracle_mod):
    """The time-displaced half-sweep of a 24x24 walker at 12 tau points (every slice of
    Lt = 12) against the oracle: G(k,tau) sums, the other dynamic observables,
    G(beta,0) and G(0,beta) within 1e-10; then a backward half-sweep with updates."""
    O = oracle_mod
    O.use_scipy_lapack(False)
    d = dq.WalkerDesc(beta=1.2, Lt=12, seed=578, **LARGE)
    b = dq.Batch([d], rng=dq.RNG_MINSTD)
    r = O.Walker(model=0, L=24, U=4.0, beta=1.2, Lt=12, pace=6, stack=O.STACK_QRP)
    r.seed(578)
    b.fields_random(0)
    r.fields_random()
    b.init_greens()
    r.init()
    taus = list(range(12))
    b.sweep_dynamic(taus)
    r.sweep_dynamic(taus)
    s_dev, c_dev = b.dynamic(0)
    s_ref, c_ref = r.dynamic()
    np.testing.assert_array_equal(c_dev, c_ref)
    assert _rel_err(s_dev, s_ref) <= 1e-10, (s_dev, s_ref)
    for dv, rv in zip(b.dynamic_obs(0), r.dynamic_obs()):
        assert _rel_err(dv, rv) <= 1e-10
    errs = []
    for which in (0, 1):
        for s in (0, 1):
            errs.append(_rel_err(b.green_dynamic(0, which, s), r.green_dynamic(which, s)))
    print(f"MEASURED 24x24 dynamic vs oracle: G(beta,0)/G(0,beta) max rel err {max(errs):.2e}, "
          f"G(k,tau) {_rel_err(s_dev, s_ref):.2e}")
    assert max(errs) <= 1e-10
    b.sweep_beta_to_0(measure=False)
    r.sweep_beta_to_0()
    np.testing.assert_array_equal(b.fields(0), r.fields())
    for s in (0, 1):
        assert _rel_err(b.green(0, s), r.green(s)) <= 1e-10
    assert b.status(0) == 0


def test_large_dynamic_mixed_against_fp64(dq):
    """The time-displaced half-sweep on the tensor-core path at beta = 12 (Lt = 120,
    tau = 0, 10, ..., 110) against the FP64 path on the same fields: G(k,tau) sums
    within 1e-6 relative, then a backward half-sweep with identical decisions.

    The sums carry the configuration sign, and the initial sign sgn(det G_up det G_dn)
    from an LU of G (src/dqmc_walker.cpp:162) is rounding noise at beta = 12, where G
    has eigenvalues far below its FP64 rounding: the two precisions may start with
    opposite signs.  The sums are compared with each path's own sign divided out."""
    descs = [dq.WalkerDesc(beta=12.0, Lt=120, seed=590, **LARGE)]
    taus = list(range(0, 120, 10))
    out = []
    for prec in (dq.MIXED, dq.FP64):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec)
        b.fields_random(0)
        b.init_greens()
        b.sweep_dynamic(taus)
        s, c = b.dynamic(0)
        s = s * b.config_sign(0)  # the sign is +-1 and no flip ran yet
        b.sweep_beta_to_0(measure=False)
        out.append((s, c, b.fields(0), b.green(0, 0), b.status(0)))
        b.close()
    (sm, cm, fm, gm, stm), (sf, cf, ff, gf, stf) = out
    np.testing.assert_array_equal(cm, cf)
    np.testing.assert_array_equal(fm, ff)
    print(f"MEASURED 24x24 beta=12 dynamic mixed vs fp64: G(k,tau) rel {_rel_err(sm, sf):.2e}, "
          f"G after bwd {float(abs(gm - gf).max()):.2e}")
    assert _rel_err(sm, sf) <= 1e-6
    assert float(abs(gm - gf).max()) <= 1e-6
    assert stm == 0 and stf == 0


def test_uneven_batch_mixed_against_fp64(dq):
    """Two walkers of each side 6, 8, 10, 12 (|U| and beta from std::mt19937_64(7)) in
    one tensor-core-path batch against the FP64 batch on the same fields and uniforms."""
    from dqmc_gb300.workloads import uneven_batch

    descs = uneven_batch(dq, per_size=2)
    assert sorted({d.L for d in descs}) == [6, 8, 10, 12]
    bm, _, series = _mixed_vs_fp64(dq, descs)
    print(f"MEASURED uneven batch mixed vs fp64: max|dG| {max(series):.2e} over {len(series)} stabilizations")
    assert max(series) <= 1e-6
