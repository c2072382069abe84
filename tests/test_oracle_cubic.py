"""Pins the oracle's cubic lattice (src/lattice/cubic.cpp) before it is checked against.

The reference has no tests for it.  The tables are checked against the
reference's own formulas, written out independently here (index2site,
nearest-neighbour order, displacement, k stars with their closed-form count,
Fourier factors, hopping matrix).  The walker is checked by the U = 0 known
answers: G = (1 + e^{-beta K})^-1 for both models and stack kinds, G(k, tau) =
e^{-tau e_k} / (1 + e^{-beta e_k}) with e_k = -2t(cos kx + cos ky + cos kz) + mu
for every k star, and the analytic density of states and spin susceptibility.
The stiffness, a square-lattice observable, stays zero.
"""
import math

import numpy as np
import pytest


def _site(i, L):
    """Cubic::initial_index2site_table (cubic.cpp:35-44)."""
    return i % L, (i % (L * L)) // L, i // (L * L)


def _kstars(L):
    """Cubic::initial_index2momentum_table (cubic.cpp:47-81)."""
    out = []
    for k in range(math.ceil(L / 2), L + 1):
        for i in range(k, L + 1):
            for j in range(k, i + 1):
                out.append([i / L * 2 * math.pi - math.pi, j / L * 2 * math.pi - math.pi,
                            k / L * 2 * math.pi - math.pi])
    return np.array(out)


def _hopping(L):
    N = L ** 3
    H = np.zeros((N, N))
    for i in range(N):
        x, y, z = _site(i, L)
        for j in ((x + 1) % L + L * y + L * L * z, x + L * ((y + 1) % L) + L * L * z,
                  x + L * y + L * L * ((z + 1) % L)):
            H[i, j] += 1.0
            H[j, i] += 1.0
    return H


@pytest.mark.parametrize("L", [2, 3, 4, 5])
def test_cubic_lattice_tables(oracle_mod, L):
    O = oracle_mod
    w = O.Walker(L=L, Lt=4, pace=2, lattice=O.CUBIC)
    N = L ** 3
    assert w.N == N and w.space_dim() == 3
    h = L // 2 + 1
    assert w.num_k_stars() == round(h * (h + 1) * (2 * h + 1) / 12 + h * (h + 1) / 4)  # cubic.cpp:52-53
    ks = _kstars(L)
    assert len(ks) == w.num_k_stars()
    for k in range(len(ks)):
        np.testing.assert_array_equal(w.k_star(k), ks[k])
    assert w.m_point() == len(ks) - 1  # the R point (pi, pi, pi)
    for i in range(N):
        x, y, z = _site(i, L)
        nn = [(x + 1) % L + L * y + L * L * z, x + L * ((y + 1) % L) + L * L * z,
              x + L * y + L * L * ((z + 1) % L), (x - 1 + L) % L + L * y + L * L * z,
              x + L * ((y - 1 + L) % L) + L * L * z, x + L * y + L * L * ((z - 1 + L) % L)]
        assert [w.nearest_neighbour(i, d) for d in range(6)] == nn  # cubic.cpp:84-109
        for j in range(0, N, max(1, N // 16)):
            xj, yj, zj = _site(j, L)
            d = (xj - x) % L + ((yj - y) % L) * L + ((zj - z) % L) * L * L  # cubic.cpp:112-132
            assert w.displacement(i, j) == d
    for d in range(N):
        x, y, z = _site(d, L)
        for k in range(len(ks)):
            assert w.fourier(d, k) == pytest.approx(math.cos(-x * ks[k, 0] - y * ks[k, 1] - z * ks[k, 2]), abs=1e-14)
    H = w.dense(2)
    np.testing.assert_array_equal(H, _hopping(L))  # cubic.cpp:203-219 (zero-initialised here)
    assert (H.sum(axis=1) == 6).all()


def test_cubic_rejects_checkerboard_and_bad_side(oracle_mod):
    O = oracle_mod
    with pytest.raises(ValueError):
        O.Walker(L=4, Lt=4, pace=2, lattice=O.CUBIC, checkerboard=True)  # dqmc_initializer.cpp:169-182
    with pytest.raises(ValueError):
        O.Walker(L=0, Lt=4, pace=2, lattice=O.CUBIC)
    with pytest.raises(ValueError):
        O.Walker(L=4, Lt=4, pace=2, lattice=7)


def test_square_tables_unchanged_by_the_dimension_generalisation(oracle_mod):
    """Square tables from the same code path: square.cpp:69-105 order and displacement."""
    O = oracle_mod
    L = 5
    w = O.Walker(L=L, Lt=4, pace=2)
    assert w.space_dim() == 2
    for i in range(L * L):
        x, y = i % L, i // L
        assert [w.nearest_neighbour(i, d) for d in range(4)] == [
            (x + 1) % L + L * y, x + L * ((y + 1) % L), (x - 1 + L) % L + L * y, x + L * ((y - 1 + L) % L)]
        for j in range(L * L):
            assert w.displacement(i, j) == (j % L - x) % L + ((j // L - y) % L) * L


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("stack", [0, 1])
def test_cubic_free_fermion_greens(oracle_mod, model, stack):
    O = oracle_mod
    L, mu, beta = 3, -0.3, 4.0
    w = O.Walker(model=model, L=L, U=0.0, mu=mu, beta=beta, Lt=40, pace=10, stack=stack, lattice=O.CUBIC)
    w.seed(7)
    w.fields_random()
    w.init()
    K = -_hopping(L) + mu * np.eye(L ** 3)
    ev, V = np.linalg.eigh(K)
    g_exact = V @ np.diag(1.0 / (1.0 + np.exp(-beta * ev))) @ V.T
    for s in (0, 1):
        assert abs(w.green(s) - g_exact).max() < 1e-12
    w.sweep_0_to_beta()
    w.sweep_beta_to_0()
    for s in (0, 1):
        assert abs(w.green(s) - g_exact).max() < 1e-12
    assert w.wrap_error < 1e-12


@pytest.mark.parametrize("stack", [0, 1])
def test_cubic_dynamic_free_fermions_known_answer(oracle_mod, stack):
    """G(k, tau) of every k star from the per-displacement sums, the walker's own momentum
    (the R point), D(tau), the local spin susceptibility, and a zero stiffness term."""
    O = oracle_mod
    L, mu, beta, Lt = 4, 0.3, 2.0, 20
    N = L ** 3
    w = O.Walker(model=0, L=L, U=0.0, mu=mu, beta=beta, Lt=Lt, pace=5, stack=stack, lattice=O.CUBIC)
    w.seed(5)
    w.fields_random()
    w.init()
    taus = [0, 1, 5, 7, 10, 19]
    w.sweep_dynamic(taus)
    sums, counts = w.dynamic()
    S = w.dynamic_r()
    r = np.arange(N)
    rx, ry, rz = r % L, (r % (L * L)) // L, r // (L * L)
    ks = _kstars(L)
    G = np.array([[np.cos(-(rx * kx + ry * ky + rz * kz)) @ S[t] for t in range(len(taus))] for kx, ky, kz in ks])
    np.testing.assert_allclose(G[-1], sums, atol=1e-12)
    assert (counts == 1).all()
    tt = np.array(taus) * beta / Lt
    for (kx, ky, kz), row in zip(ks, G):
        e = -2.0 * (np.cos(kx) + np.cos(ky) + np.cos(kz)) + mu
        np.testing.assert_allclose(row, np.exp(-tt * e) / (1 + np.exp(-beta * e)), atol=1e-12)
    # D(tau) = tr(e^{-tau K} G0) / N (G(beta, beta) = G0 at tau = 0); the local spin
    # susceptibility of free fermions, 0.25/N sum_i 2 (-G(0,tau)_ii G(tau,0)_ii)
    # (in the eigenbasis of K: forming e^{s K} in the site basis loses digits to e^{beta |e|})
    K = -_hopping(L) + mu * np.eye(N)
    ev, V = np.linalg.eigh(K)
    fermi = 1.0 / (1.0 + np.exp(-beta * ev))
    G0 = (V * fermi) @ V.T
    dos, chi, rho = w.dynamic_obs()
    for k, tau in enumerate(taus):
        s = beta if tau == 0 else tau * beta / Lt
        gt0 = (V * (np.exp(-s * ev) * fermi)) @ V.T                  # e^{-s K} G0
        g0t = -(V * (np.exp(-(beta - s) * ev) * fermi)) @ V.T        # -(1 - G0) e^{s K}
        assert abs(dos[k] - np.trace(G0 if tau == 0 else gt0) / N) < 1e-12
        assert abs(chi[k] - 0.25 / N * np.sum(-2 * np.diag(g0t) * np.diag(gt0))) < 1e-12
    assert (rho == 0).all()


def test_cubic_equal_time_observables_free_fermions(oracle_mod):
    """U = 0: filling 2 - tr(G_up + G_dn)/N, double occupancy, kinetic energy
    2t/N sum_i sum_{+x,+y,+z} 2 G(i, i+a) (measure_methods.cpp:77-98 over SpaceDim), and
    the momentum distribution at the walker's momentum equals the Fermi function there."""
    O = oracle_mod
    L, beta = 4, 2.0  # even L: the R point (pi, pi, pi) is a momentum of the lattice
    N = L ** 3
    w = O.Walker(model=0, L=L, U=0.0, mu=0.0, beta=beta, Lt=10, pace=5, lattice=O.CUBIC)
    w.seed(1)
    w.fields_random()
    w.init()
    w.sweep_0_to_beta()
    w.measure()
    sums, counts = w.accumulators()
    v = sums / counts
    K = -_hopping(L)
    ev, V = np.linalg.eigh(K)
    G0 = V @ np.diag(1.0 / (1.0 + np.exp(-beta * ev))) @ V.T
    assert abs(v[0] - (2 - 2 * np.trace(G0) / N)) < 1e-12
    assert abs(v[0] - 1.0) < 1e-12  # even L, mu = 0: bipartite, half filled
    assert abs(v[1] - np.mean((1 - np.diag(G0)) ** 2)) < 1e-12
    kin = 0.0
    for i in range(N):
        for d in range(3):
            kin += 2 * G0[i, w.nearest_neighbour(i, d)]
    assert abs(v[2] - 2.0 * kin / N) < 1e-12
    kR = _kstars(L)[-1]
    eR = -2.0 * np.cos(kR).sum()
    assert abs(v[3] - (1 - 1 / (1 + np.exp(-beta * eR)))) < 1e-12  # n(k) = 1 - G(k)
