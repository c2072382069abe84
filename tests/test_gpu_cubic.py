"""The cubic lattice on the GPU (src/lattice/cubic.cpp: N = L^3 sites, bonds to the
+x, +y, +z neighbours, k stars on the tetrahedron (0,0,0), (pi,0,0), (pi,pi,0),
(pi,pi,pi)), dense exp(-dtau K) only (dqmc_initializer.cpp:169-182).

Bars as for the square lattice: identical accept/reject decisions; G within 1e-10
(relative to max(1, |G|)) of the oracle at every stabilization and after every
half-sweep; equal-time sums, G(k,tau) sums and the dynamic observables within 1e-10;
the superfluid stiffness stays zero (a square-lattice observable,
dqmc_initializer.cpp:233-237).  The tensor-core path against FP64 on the same fields:
identical decisions and max |dG| <= 1e-6 at every stabilization.
"""
import numpy as np
import pytest

from test_gpu_large import _mixed_vs_fp64
from test_gpu_parity import _close, _run_pair

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300

    return dqmc_gb300


@pytest.mark.parametrize("model,L,mu,Lt,pace,kidx", [
    (0, 4, 0.0, 20, 5, -1),    # repulsive, N = 64: shared-memory walker, R point
    (1, 4, -0.5, 16, 4, 2),    # attractive, shared-memory walker, third k star
    (0, 5, 0.0, 20, 5, 4),     # odd side, N = 125: HBM walker
    (1, 6, -0.3, 16, 8, -1),   # N = 216
])
def test_cubic_fp64_against_oracle(dq, oracle_mod, model, L, mu, Lt, pace, kidx):
    d = dq.WalkerDesc(model=model, L=L, U=4.0, mu=mu, beta=2.0, Lt=Lt, pace=pace, momentum_index=kidx,
                      lattice=dq.CUBIC, seed=300 + L)
    assert d.N == L ** 3
    errs = []
    _run_pair(dq, oracle_mod, [d], sweeps=2, errs=errs)
    print(f"MEASURED cubic L={L} fp64 vs oracle: max rel |dG| {max(errs):.2e}")


def test_square_and_cubic_walkers_in_one_batch(dq, oracle_mod):
    """Square and cubic walkers of similar N side by side in one batch (8x8 and 4^3 on the
    shared-memory path, 11x11 and 5^3 on the HBM path) against one oracle each."""
    descs = [dq.WalkerDesc(model=0, L=8, U=4.0, beta=2.0, Lt=20, pace=5, seed=401),
             dq.WalkerDesc(model=0, L=4, U=4.0, beta=2.0, Lt=20, pace=5, lattice=dq.CUBIC, seed=402),
             dq.WalkerDesc(model=1, L=11, U=4.0, mu=-0.2, beta=2.0, Lt=20, pace=5, seed=403),
             dq.WalkerDesc(model=1, L=5, U=4.0, mu=-0.2, beta=2.0, Lt=20, pace=5, lattice=dq.CUBIC, seed=404)]
    _run_pair(dq, oracle_mod, descs, sweeps=1)


@pytest.mark.parametrize("L,Lt,pace", [(4, 16, 4), (5, 20, 5)])
def test_cubic_dynamic_against_oracle(dq, oracle_mod, L, Lt, pace):
    """The time-displaced half-sweep on the cubic lattice: G(k,tau) sums, the density of
    states and spin susceptibility, G(beta,0) and G(0,beta) within 1e-10; the stiffness
    terms zero; then a backward half-sweep with identical decisions."""
    O = oracle_mod
    O.use_scipy_lapack(False)
    d = dq.WalkerDesc(model=0, L=L, U=4.0, beta=2.0, Lt=Lt, pace=pace, lattice=dq.CUBIC, seed=450 + L)
    b = dq.Batch([d], rng=dq.RNG_MINSTD)
    r = O.Walker(model=0, L=L, U=4.0, beta=2.0, Lt=Lt, pace=pace, stack=O.STACK_QRP, lattice=O.CUBIC)
    r.seed(450 + L)
    b.fields_random(0)
    r.fields_random()
    b.init_greens()
    r.init()
    taus = [0, 1, pace - 1, pace, pace + 2, Lt - 1]
    b.sweep_dynamic(taus)
    r.sweep_dynamic(taus)
    s_dev, c_dev = b.dynamic(0)
    s_ref, c_ref = r.dynamic()
    np.testing.assert_array_equal(c_dev, c_ref)
    assert _close(s_dev, s_ref), (s_dev, s_ref)
    np.testing.assert_allclose(b.dynamic_r(0), r.dynamic_r(), rtol=1e-10, atol=1e-10)
    dos, chi, rho = b.dynamic_obs(0)
    rdos, rchi, rrho = r.dynamic_obs()
    assert _close(dos, rdos) and _close(chi, rchi)
    assert not np.any(rho) and not np.any(rrho)
    for which in (0, 1):
        for s in (0, 1):
            assert _close(b.green_dynamic(0, which, s), r.green_dynamic(which, s))
    b.sweep_beta_to_0(measure=True)
    r.sweep_beta_to_0()
    np.testing.assert_array_equal(b.fields(0), r.fields())
    for s in (0, 1):
        assert _close(b.green(0, s), r.green(s))
    assert b.status(0) == 0


@pytest.mark.parametrize("L", [6, 7])
def test_cubic_mixed_against_fp64(dq, L):
    """The tensor-core path on the cubic lattice (N = 216: 7-slice wraps; N = 343: 8-slice
    wraps and 9-slice stabilization products) against FP64 on the same fields."""
    descs = [dq.WalkerDesc(model=0, L=L, U=4.0, beta=4.0, Lt=40, pace=8, lattice=dq.CUBIC, seed=500 + L + w)
             for w in range(2)]
    _, _, series = _mixed_vs_fp64(dq, descs)
    print(f"MEASURED cubic L={L} mixed vs fp64: max|dG| {max(series):.2e} over {len(series)} stabilizations")
    assert max(series) <= 1e-6
