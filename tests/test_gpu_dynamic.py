"""Dynamic (time-displaced) half-sweep on the GPU against the oracle.

DqmcWalker::sweep_for_dynamic_greens (src/dqmc_walker.cpp:424-524) with
measure_greens_functions (src/measure/measure_methods.cpp:278-308): the fields
stay fixed, G(t,0) and G(0,t) are propagated and recomputed stably at every
stabilization, and G(k,tau) is accumulated at the listed tau.  Bar: the plain
FP64 path agrees with the oracle within 1e-10 relative (G(k,tau) sums, G(beta,0),
G(0,beta)); the tensor-core path agrees with the FP64 path within 1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300

    return dqmc_gb300


def _close(a, b, rel=REL):
    scale = max(1.0, abs(np.asarray(b)).max())
    return abs(np.asarray(a) - np.asarray(b)).max() <= rel * scale


@pytest.mark.parametrize("model,L,mu,Lt,pace,cb", [
    (0, 9, 0.0, 20, 5, False),     # repulsive, odd side, N = 81
    (1, 10, -0.5, 24, 8, False),   # attractive, N = 100
    (0, 8, 0.0, 20, 5, True),      # checkerboard break-up, shared-memory walker (N = 64)
    (0, 10, 0.0, 20, 5, True),     # checkerboard, HBM walker (N = 100)
    (1, 6, -0.3, 16, 4, False),    # shared-memory walker (N = 36)
])
def test_dynamic_sweep_against_oracle(dq, oracle_mod, model, L, mu, Lt, pace, cb):
    """Shared-memory walkers (N <= 64) run the dynamic half-sweep on the HBM path's kernels
    and return to their own path for the backward half-sweep; checkerboard walkers take
    G(t,0) and G(0,t) through the plaquette passes (mult_B_from_left / mult_invB_from_right
    of the model's checkerboard link, src/dqmc_walker.cpp:455-466)."""
    O = oracle_mod
    O.use_scipy_lapack(False)
    d = dq.WalkerDesc(model=model, L=L, U=4.0, mu=mu, beta=2.0, Lt=Lt, pace=pace, checkerboard=cb, seed=61)
    b = dq.Batch([d], rng=dq.RNG_MINSTD)
    r = O.Walker(model=model, L=L, U=4.0, mu=mu, beta=2.0, Lt=Lt, pace=pace, checkerboard=cb, stack=O.STACK_QRP)
    r.seed(61)
    b.fields_random(0)
    r.fields_random()
    b.init_greens()
    r.init()
    taus = [0, 1, pace - 1, pace, pace + 3, Lt - 1]
    for rnd in range(2):
        f0 = b.fields(0)
        b.sweep_dynamic(taus)
        r.sweep_dynamic(taus)
        np.testing.assert_array_equal(b.fields(0), f0)  # the fields stay fixed
        s_dev, c_dev = b.dynamic(0)
        s_ref, c_ref = r.dynamic()
        np.testing.assert_array_equal(c_dev, c_ref)
        assert _close(s_dev, s_ref), (s_dev, s_ref)
        for which in (0, 1):
            for s in (0, 1):
                assert _close(b.green_dynamic(0, which, s), r.green_dynamic(which, s)), (rnd, which, s)
        for s in (0, 1):
            assert _close(b.green(0, s), r.green(s))
        assert b.status(0) == 0
        # back to t = 0 with Metropolis updates (same uniforms on both sides)
        b.sweep_beta_to_0(measure=False)
        r.sweep_beta_to_0()
        np.testing.assert_array_equal(b.fields(0), r.fields())
        for s in (0, 1):
            assert _close(b.green(0, s), r.green(s))
    assert b.wrap_error(0) < 1e-6


def test_dynamic_mixed_against_fp64(dq):
    """Tensor-core path (N = 144: tensor-core wraps and stabilization in the
    regular half-sweeps) against the FP64 path on the same fields and uniforms."""
    descs = [dq.WalkerDesc(model=1, L=12, U=4.0, mu=-0.5, beta=2.0, Lt=20, pace=5, seed=70 + w) for w in range(2)]
    taus = [0, 3, 5, 12, 19]
    out = []
    for prec in (dq.MIXED, dq.FP64):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec)
        for w in range(2):
            b.fields_random(w)
        b.init_greens()
        b.sweep_dynamic(taus)
        b.sweep_beta_to_0(measure=False)
        b.sweep_dynamic(taus)
        out.append(([b.dynamic(w)[0] for w in range(2)], [b.fields(w) for w in range(2)],
                    [b.green_dynamic(w, 0, 0) for w in range(2)], [b.status(w) for w in range(2)]))
    (sm, fm, gm, stm), (sf, ff, gf, stf) = out
    for w in range(2):
        np.testing.assert_array_equal(fm[w], ff[w])
        assert _close(sm[w], sf[w], 1e-6)
        assert abs(gm[w] - gf[w]).max() <= 1e-6
        assert stm[w] == 0 and stf[w] == 0


def test_dynamic_mixed_large_n(dq):
    """N = 289 (> 256 slice configuration) on the tensor-core path against FP64."""
    descs = [dq.WalkerDesc(model=0, L=17, U=4.0, beta=1.0, Lt=10, pace=5, seed=90)]
    taus = [0, 3, 5, 9]
    res = []
    for prec in (dq.MIXED, dq.FP64):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec)
        b.fields_random(0)
        b.init_greens()
        b.sweep_dynamic(taus)
        res.append((b.dynamic(0)[0], b.green_dynamic(0, 0, 0), b.status(0)))
    assert _close(res[0][0], res[1][0], 1e-6)
    assert abs(res[0][1] - res[1][1]).max() <= 1e-6
    assert res[0][2] == 0 and res[1][2] == 0


def test_dynamic_sweep_state_and_arguments(dq):
    d = dq.WalkerDesc(model=0, L=9, U=4.0, beta=1.0, Lt=10, pace=5, seed=1)
    b = dq.Batch([d], rng=dq.RNG_PHILOX)
    b.fields_random(0)
    with pytest.raises(dq.DqmcError):
        b.sweep_dynamic([0])          # before set-up
    b.init_greens()
    with pytest.raises(dq.DqmcError):
        b.sweep_dynamic([10])         # tau outside [0, Lt)
    b.sweep_0_to_beta()
    with pytest.raises(dq.DqmcError):
        b.sweep_dynamic([0])          # stacks at beta
    b.sweep_beta_to_0()
    b.sweep_dynamic([0, 4])
    with pytest.raises(dq.DqmcError):
        b.sweep_dynamic([0])          # stacks at beta again


@pytest.mark.parametrize("model,L,mu,Lt,pace", [
    (0, 10, 0.0, 20, 5),    # repulsive, N = 100
    (1, 10, -0.5, 24, 8),   # attractive
])
def test_dynamic_observables_against_oracle(dq, oracle_mod, model, L, mu, Lt, pace):
    """Density of states, local dynamic spin susceptibility and the superfluid-stiffness
    terms per tau (measure_methods.cpp:315-461) on the FP64 path against the oracle,
    over two dynamic half-sweeps separated by a backward half-sweep."""
    O = oracle_mod
    O.use_scipy_lapack(False)
    d = dq.WalkerDesc(model=model, L=L, U=4.0, mu=mu, beta=2.0, Lt=Lt, pace=pace, seed=17)
    b = dq.Batch([d], rng=dq.RNG_MINSTD)
    r = O.Walker(model=model, L=L, U=4.0, mu=mu, beta=2.0, Lt=Lt, pace=pace, stack=O.STACK_QRP)
    r.seed(17)
    b.fields_random(0)
    r.fields_random()
    b.init_greens()
    r.init()
    taus = [0, 1, pace - 1, pace, pace + 3, Lt - 1]
    for rnd in range(2):
        b.sweep_dynamic(taus)
        r.sweep_dynamic(taus)
        for dev, ref in zip(b.dynamic_obs(0), r.dynamic_obs()):
            assert _close(dev, ref), (rnd, dev, ref)
        assert _close(b.dynamic_r(0), r.dynamic_r())
        # G(k,tau) of the walker's momentum from the per-displacement sums
        # the M point (pi, pi) is the walker's default momentum
        assert _close(b.dynamic_greens_k(0, [(np.pi, np.pi)])[0], b.dynamic(0)[0], 1e-12)
        b.sweep_beta_to_0(measure=False)
        r.sweep_beta_to_0()
    assert b.status(0) == 0


def test_dynamic_observables_mixed_against_fp64(dq):
    """The tensor-core path (N = 144) against the FP64 path on the same fields."""
    descs = [dq.WalkerDesc(model=0, L=12, U=4.0, beta=2.0, Lt=20, pace=5, seed=80)]
    taus = [0, 2, 5, 11, 19]
    res = []
    for prec in (dq.MIXED, dq.FP64):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec)
        b.fields_random(0)
        b.init_greens()
        b.sweep_dynamic(taus)
        res.append(b.dynamic_obs(0))
    for m, f in zip(res[0], res[1]):
        assert _close(m, f, 1e-6), (m, f)
