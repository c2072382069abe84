"""Pins the CPU oracle before anything is checked against it.

The reference ships no unit tests or golden vectors (its test/test_main.cpp
only prints lattice indices).  The oracle is pinned by
  * known answers written from the mathematics (U = 0 Green's function,
    determinant ratios, Sherman-Morrison = fresh recomputation, UDV
    reconstruction, checkerboard algebra, lattice tables),
  * the exact uniform stream of libstdc++'s minstd_rand0 + bernoulli, and
  * a statistical comparison with the reference's only shipped run
    (example/log.out, fixture tests/golden/example_8x8.json).
"""
import multiprocessing as mp

import numpy as np
import pytest


def _minstd_uniforms(seed, n):
    m, a = 2147483647, 16807
    x = seed % m or 1
    R = 2147483646.0
    out = []
    for _ in range(n):
        x = (a * x) % m
        g1 = x
        x = (a * x) % m
        g2 = x
        s = float(g1 - 1) + float(g2 - 1) * R
        u = s / (R * R)
        out.append(u if u < 1.0 else np.nextafter(1.0, 0.0))
    return np.array(out)


def test_uniform_stream_matches_libstdcxx(oracle_mod):
    w = oracle_mod.Walker(L=2, Lt=4, pace=2)
    for seed in (1, 12345, 2**31 - 1, 0):
        w.seed(seed)
        np.testing.assert_array_equal(w.uniforms(200), _minstd_uniforms(seed, 200))


def _exact_G0(w, beta, K):
    ev, V = np.linalg.eigh(K)
    return V @ np.diag(1.0 / (1.0 + np.exp(-beta * ev))) @ V.T


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("stack", [0, 1])
def test_free_fermion_greens(oracle_mod, model, stack):
    O = oracle_mod
    w = O.Walker(model=model, L=4, U=0.0, mu=-0.3, beta=4.0, Lt=40, pace=10, stack=stack)
    w.seed(7)
    w.fields_random()
    w.init()
    K = -w.dense(2) + (-0.3) * np.eye(16)
    g_exact = _exact_G0(w, 4.0, K)
    for s in (0, 1):
        assert abs(w.green(s) - g_exact).max() < 1e-12
    w.sweep_0_to_beta()
    w.sweep_beta_to_0()
    for s in (0, 1):
        assert abs(w.green(s) - g_exact).max() < 1e-12
    assert w.wrap_error < 1e-12


def test_checkerboard_algebra(oracle_mod):
    O = oracle_mod
    w = O.Walker(L=4, U=4.0, beta=1.0, Lt=20, pace=5, checkerboard=True)
    I = np.eye(16)
    E = w.mult_expK(0, I)
    np.testing.assert_allclose(w.mult_expK(1, I), E, atol=1e-15)
    np.testing.assert_allclose(w.mult_expK(4, I), E.T, atol=1e-15)
    np.testing.assert_allclose(w.mult_expK(2, E), I, atol=1e-13)
    np.testing.assert_allclose(w.mult_expK(3, E), I, atol=1e-13)
    # the break-up approximates exp(dtau t H) to O(dtau^2) (mu = 0)
    dense = O.Walker(L=4, U=4.0, beta=1.0, Lt=20, pace=5, checkerboard=False).dense(0)
    err = abs(E - dense).max()
    assert err < 0.05 ** 2 * 2
    # plaquette in isolation: exp(dtau t h_plaq) for a 2x2 torus-free block
    assert E.shape == (16, 16)


def test_lattice_tables(oracle_mod):
    w = oracle_mod.Walker(L=6, Lt=4, pace=2)
    assert w.num_k_stars() == (3 + 1) * (3 + 2) // 2
    m = w.m_point()
    for d in range(36):
        x, y = d % 6, d // 6
        assert w.fourier(d, m) == pytest.approx((-1.0) ** (x + y), abs=1e-12)
        assert w.fourier(d, 0) == pytest.approx(1.0)
    H = w.dense(2)
    assert (H == H.T).all() and H.sum() == 4 * 36


def _chain_product(w, N, Lt, spin):
    B = np.eye(N)
    for t in range(1, Lt + 1):
        B = w.mult_B(0, B, t, spin)  # B(t) . (B(t-1) ... B(1))
    return B


def _rest_product(w, N, Lt, spin):
    """B(Lt) ... B(2)."""
    rest = np.eye(N)
    for t in range(2, Lt + 1):
        rest = w.mult_B(0, rest, t, spin)
    return rest


def _greens_slice1(w, N, Lt):
    """Equal-time G at slice 1: (1 + B(1) B(Lt)..B(2))^-1 for both spins."""
    out = []
    for spin in (+1, -1):
        B1 = w.mult_B(0, np.eye(N), 1, spin)
        out.append(np.linalg.inv(np.eye(N) + B1 @ _rest_product(w, N, Lt, spin)))
    return out


@pytest.mark.parametrize("model", [0, 1])
def test_ratio_is_determinant_ratio(oracle_mod, model):
    """get_update_ratio (repulsive_hubbard.cpp:112-124, attractive_hubbard.cpp:112-125)
    equals the weight ratio: det ratio of (1 + B(1)..B(Lt)) over spins, times
    exp(2 alpha s) for the attractive decoupling's bosonic factor."""
    O = oracle_mod
    N, Lt = 4, 8
    w = O.Walker(model=model, L=2, U=3.0, mu=0.2, beta=1.0, Lt=Lt, pace=4)
    w.seed(3)
    w.fields_random()
    i = 2
    f = w.fields()
    dets = []
    for flip in (False, True):
        ff = f.copy()
        if flip:
            ff[0, i] *= -1
        w.set_fields(ff)
        d = 1.0
        for spin in (+1, -1):
            B = w.mult_B(0, np.eye(N), 1, spin) @ _rest_product(w, N, Lt, spin)
            d *= np.linalg.det(np.eye(N) + B)
        dets.append(d)
    w.set_fields(f)
    g = _greens_slice1(w, N, Lt)
    for s in (0, 1):
        w.set_green(s, g[s])
    expected = dets[1] / dets[0]
    if model == O.ATTRACTIVE:
        expected *= np.exp(2 * w.alpha * f[0, i])
    assert w.ratio(0, i) == pytest.approx(expected, rel=1e-10)


@pytest.mark.parametrize("model", [0, 1])
def test_sherman_morrison_equals_fresh(oracle_mod, model):
    """update_greens_function (repulsive_hubbard.cpp:127-155) vs recomputation."""
    O = oracle_mod
    N, Lt = 4, 6
    w = O.Walker(model=model, L=2, U=4.0, beta=1.2, Lt=Lt, pace=3)
    w.seed(11)
    w.fields_random()
    f = w.fields()
    g_old = _greens_slice1(w, N, Lt)
    for s in (0, 1):
        w.set_green(s, g_old[s])
    i = 1
    w.update_greens(0, i)
    f2 = f.copy()
    f2[0, i] *= -1
    w.set_fields(f2)
    g_new = _greens_slice1(w, N, Lt)
    for s in (0, 1):
        np.testing.assert_allclose(w.green(s), g_new[s], atol=1e-11)


def test_udv_factorisations(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(5)
    n = 12
    scales = np.exp(np.linspace(-20, 20, n))
    A = rng.standard_normal((n, n)) @ np.diag(scales) @ rng.standard_normal((n, n))
    u, s, v = O.svd(A)
    assert np.all(np.diff(s) <= 0)
    np.testing.assert_allclose(u.T @ u, np.eye(n), atol=1e-13)
    np.testing.assert_allclose(v.T @ v, np.eye(n), atol=1e-13)
    np.testing.assert_allclose(u @ np.diag(s) @ v.T, A, rtol=0, atol=1e-12 * abs(A).max())
    U, D, T = O.qrp_udt(A)
    np.testing.assert_allclose(U.T @ U, np.eye(n), atol=1e-13)
    np.testing.assert_allclose(U @ np.diag(D) @ T, A, rtol=0, atol=1e-12 * abs(A).max())
    assert np.all(D > 0)
    # (1 + U D T)^-1 from the stable assembly, on a spread where numpy's
    # plain inverse is itself accurate
    A2 = rng.standard_normal((n, n)) @ np.diag(np.exp(np.linspace(-4, 4, n))) @ rng.standard_normal((n, n))
    U2, D2, T2 = O.qrp_udt(A2)
    G = O.greens_from_udv(U2, D2, T2)
    assert abs(G - np.linalg.inv(np.eye(n) + A2)).max() < 1e-11


def test_svd_and_qrp_stacks_agree(oracle_mod):
    """Reference SVD stack and the device QRP stack give the same walker."""
    O = oracle_mod
    ws = []
    for stack in (O.STACK_SVD, O.STACK_QRP):
        w = O.Walker(model=0, L=4, U=4.0, beta=4.0, Lt=80, pace=10, stack=stack)
        w.seed(12345)
        w.fields_random()
        w.init()
        w.trace(True)
        for _ in range(2):
            w.sweep_0_to_beta()
            w.sweep_beta_to_0()
        ws.append(w)
    np.testing.assert_array_equal(ws[0].fields(), ws[1].fields())
    ta, tb = ws[0].trace_get(), ws[1].trace_get()
    assert ta.shape == tb.shape and ta.shape[0] == 2 * 2 * 8
    assert abs(ta - tb).max() < 1e-10


# ---- time-displaced Green's functions (sweep_for_dynamic_greens) ----------------

@pytest.mark.parametrize("stack", [0, 1])
def test_dynamic_free_fermions_known_answer(oracle_mod, stack):
    """U = 0: G(k, tau) = exp(-tau e_k) / (1 + exp(-beta e_k)), e_k = -2t(cos kx + cos ky) + mu;
    the M point (pi, pi) gives e = 4t + mu."""
    O = oracle_mod
    mu, beta, Lt = 0.3, 2.0, 20
    w = O.Walker(model=0, L=4, U=0.0, mu=mu, beta=beta, Lt=Lt, pace=5, stack=stack)
    w.seed(5)
    w.fields_random()
    w.init()
    taus = [0, 1, 5, 7, 10, 19]
    w.sweep_dynamic(taus)
    sums, counts = w.dynamic()
    e = 4.0 + mu
    for tau, s, c in zip(taus, sums, counts):
        assert c == 1
        assert abs(s - np.exp(-tau * beta / Lt * e) / (1 + np.exp(-beta * e))) < 1e-12
    assert w.wrap_error < 1e-12


@pytest.mark.parametrize("stack", [0, 1])
@pytest.mark.parametrize("model", [0, 1])
def test_dynamic_greens_at_beta_equal_direct_formula(oracle_mod, stack, model):
    """After the dynamic sweep G(beta, 0) = (1 + B)^-1 B and G(0, beta) = -(1 + B)^-1 with
    B = B(beta) ... B(1) of the spin (interacting, fixed fields)."""
    O = oracle_mod
    w = O.Walker(model=model, L=4, U=4.0, mu=-0.2 if model else 0.0, beta=2.0, Lt=20, pace=5, stack=stack)
    w.seed(3)
    w.fields_random()
    w.init()
    N = 16
    B = [np.eye(N), np.eye(N)]
    for t in range(1, 21):
        for s, sg in ((0, +1), (1, -1)):
            m = np.asfortranarray(np.eye(N))
            O.lib().orc_mult_B(w.h, 0, O._dp(m), t, sg)
            B[s] = m @ B[s]
    w.sweep_dynamic([3])
    for s in (0, 1):
        assert abs(w.green_dynamic(0, s) - np.linalg.solve(np.eye(N) + B[s], B[s])).max() < 1e-10
        assert abs(w.green_dynamic(1, s) + np.linalg.inv(np.eye(N) + B[s])).max() < 1e-10
    assert w.wrap_error < 1e-9


def test_dynamic_stacks_agree_and_alternate(oracle_mod):
    """Both stack kinds give the same G(k, tau); dynamic and backward half-sweeps alternate."""
    O = oracle_mod
    res = []
    for stack in (O.STACK_SVD, O.STACK_QRP):
        w = O.Walker(model=1, L=4, U=4.0, mu=-0.5, beta=4.0, Lt=40, pace=8, stack=stack)
        w.seed(11)
        w.fields_random()
        w.init()
        taus = [0, 4, 8, 13, 39]
        for _ in range(2):
            w.sweep_dynamic(taus)
            w.sweep_beta_to_0()
        res.append((w.dynamic()[0], w.wrap_error))
        with pytest.raises(RuntimeError):
            w.sweep_0_to_beta()
            w.sweep_dynamic(taus)  # stacks no longer at t = 0
    assert abs(res[0][0] - res[1][0]).max() < 1e-10
    assert res[0][1] < 1e-9 and res[1][1] < 1e-9


def _pin_chain(args):
    import os
    import sys

    root = args[0]
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle as O

    O.use_scipy_lapack(True)
    seed, fields, warm, nbins, binsize = args[1:]
    w = O.Walker(model=O.ATTRACTIVE, L=8, U=4.0, beta=8.0, Lt=160, pace=10)
    w.seed(seed)
    w.set_fields(fields)
    w.init()
    for _ in range(warm):
        w.sweep_0_to_beta()
        w.sweep_beta_to_0()
    bins = []
    for _ in range(nbins):
        for _ in range(binsize):
            w.sweep_0_to_beta()
            w.measure()
            w.sweep_beta_to_0()
            w.measure()
        bins.append(w.write_bin())
    return np.array(bins), w.wrap_error


@pytest.mark.slow
def test_statistical_pin_against_reference_example(oracle_mod, example_fixture):
    """Oracle vs example/log.out:44-55 (attractive 8x8, beta=8, from fields.out)."""
    import os

    O = oracle_mod
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    jobs = [(root, 500 + k, example_fixture["fields"], 6, 3, 12) for k in range(8)]
    with mp.get_context("spawn").Pool(8) as pool:
        res = pool.map(_pin_chain, jobs)
    bins = np.concatenate([r[0] for r in res])
    mean, err = O.analyse(bins)
    for k, name in enumerate(O.OBS_NAMES):
        ref, ref_err = example_fixture["observables"][name]
        sigma = np.hypot(err[k], ref_err)
        if sigma == 0:
            assert mean[k] == pytest.approx(ref)
        else:
            # bins of one chain are autocorrelated, so allow 4 combined sigma
            assert abs(mean[k] - ref) < 4 * sigma, (name, mean[k], err[k], ref, ref_err)
    wrap = max(r[1] for r in res)
    assert 1e-11 < wrap < 1e-6  # published maximum wrap error 1.085e-8


def _free_fermion_dynamic_obs(L, t, mu, beta, Lt, taus):
    """U = 0 restatement of measure_methods.cpp:315-461 with the analytic Green's functions
    G0 = (1 + e^{-beta K})^-1, G(tau,0) = e^{-tau K} G0, G(0,tau) = -(1 - G0) e^{tau K},
    G(tau,tau) = G0 (the reference's index Lt-1 at tau = 0: G(beta,0), G(0,beta))."""
    N = L * L
    H = np.zeros((N, N))
    for i in range(N):
        x, y = i % L, i // L
        for j in ((x + 1) % L + L * y, x + L * ((y + 1) % L)):
            H[i, j] += 1.0
            H[j, i] += 1.0
    K = -t * H + mu * np.eye(N)
    ev, U = np.linalg.eigh(K)
    ex = lambda s: (U * np.exp(s * ev)) @ U.T
    I = np.eye(N)
    G0 = np.linalg.inv(I + ex(-beta))
    dt = beta / Lt
    kx1 = ((L + 1) // 2 + 1) / L * 2 * np.pi - np.pi
    cf = np.cos(-np.arange(L) * kx1)
    nn = [(i % L + 1) % L + L * (i // L) for i in range(N)]
    out = []
    for tau in taus:
        s = beta if tau == 0 else tau * dt
        gtt, g00 = G0, G0
        gt0 = ex(-s) @ G0
        g0t = -(I - G0) @ ex(s)
        dos = np.trace(G0 if tau == 0 else gt0) / N
        chi = sum(0.25 / N * (2 * (1 - gtt[i, i]) * (1 - g00[i, i]) - 2 * g0t[i, i] * gt0[i, i]
                              - 2 * (1 - gtt[i, i]) * (1 - g00[i, i])) for i in range(N))
        rho = 0.0
        for i in range(N):
            ipx = nn[i]
            for j in range(N):
                jpx = nn[j]
                rx, ry = (j % L - i % L) % L, (j // L - i // L) % L
                ff = cf[rx] - cf[ry]
                rho += t * t * ff * (
                    -(2 * (gtt[j, jpx] - gtt[jpx, j])) * (2 * (g00[i, ipx] - g00[ipx, i]))
                    + 2 * (-g0t[ipx, jpx] * gt0[j, i] + g0t[i, jpx] * gt0[j, ipx]
                           + g0t[ipx, j] * gt0[jpx, i] - g0t[i, j] * gt0[jpx, ipx]))
        out.append((dos, chi, 0.25 * rho / N ** 2))
    return np.array(out)


@pytest.mark.parametrize("stack", [0, 1])
def test_dynamic_observables_free_fermions_known_answer(oracle_mod, stack):
    """U = 0: density of states, local dynamic spin susceptibility and the stiffness terms
    of the oracle's dynamic half-sweep equal the analytic free-fermion values."""
    O = oracle_mod
    L, mu, beta, Lt = 4, 0.3, 2.0, 20
    w = O.Walker(model=0, L=L, U=0.0, mu=mu, beta=beta, Lt=Lt, pace=5, stack=stack)
    w.seed(5)
    w.fields_random()
    w.init()
    taus = [0, 1, 5, 7, 10, 19]
    w.sweep_dynamic(taus)
    dos, chi, rho = w.dynamic_obs()
    ref = _free_fermion_dynamic_obs(L, 1.0, mu, beta, Lt, taus)
    np.testing.assert_allclose(dos, ref[:, 0], atol=1e-12)
    np.testing.assert_allclose(chi, ref[:, 1], atol=1e-12)
    np.testing.assert_allclose(rho, ref[:, 2], atol=1e-12)
    # particle-hole symmetric point: D(tau) = D(beta - tau), chi(tau) = chi(beta - tau)
    w0 = O.Walker(model=0, L=L, U=0.0, mu=0.0, beta=beta, Lt=Lt, pace=5, stack=stack)
    w0.seed(5)
    w0.fields_random()
    w0.init()
    w0.sweep_dynamic([1, 19, 0])
    d0, c0, _ = w0.dynamic_obs()
    assert abs(d0[0] - d0[1]) < 1e-12 and abs(c0[0] - c0[1]) < 1e-12
    assert abs(d0[2] - 0.5) < 1e-12 and abs(c0[2] - 0.125) < 1e-12  # half filling, U = 0


def test_dynamic_displacement_sums_give_g_of_every_k(oracle_mod):
    """The per-displacement sums reproduce G(k, tau) of the walker's momentum and, at
    U = 0, exp(-tau e_k) / (1 + exp(-beta e_k)) for every k star."""
    O = oracle_mod
    L, mu, beta, Lt = 4, 0.3, 2.0, 20
    w = O.Walker(model=0, L=L, U=0.0, mu=mu, beta=beta, Lt=Lt, pace=5, stack=1)
    w.seed(5)
    w.fields_random()
    w.init()
    taus = [0, 1, 5, 7, 10, 19]
    w.sweep_dynamic(taus)
    S = w.dynamic_r()
    sums, _ = w.dynamic()
    r = np.arange(L * L)
    rx, ry = r % L, r // L
    ks = [(i / L * 2 * np.pi - np.pi, j / L * 2 * np.pi - np.pi)
          for i in range(L // 2, L + 1) for j in range(L // 2, i + 1)]
    G = np.array([[np.cos(-(rx * kx + ry * ky)) @ S[t] for t in range(len(taus))] for kx, ky in ks])
    np.testing.assert_allclose(G[-1], sums, atol=1e-12)  # the M point, the walker's momentum
    for (kx, ky), row in zip(ks, G):
        e = -2.0 * (np.cos(kx) + np.cos(ky)) + mu
        np.testing.assert_allclose(row, np.exp(-np.array(taus) * beta / Lt * e) / (1 + np.exp(-beta * e)), atol=1e-12)


def _pin_chain_dynamic(args):
    import os
    import sys

    root = args[0]
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle as O

    O.use_scipy_lapack(True)
    seed, fields, warm, nbins, binsize, taus, kstars = args[1:]
    w = O.Walker(model=O.ATTRACTIVE, L=8, U=4.0, beta=8.0, Lt=160, pace=10)
    w.seed(seed)
    w.set_fields(fields)
    w.init()
    for _ in range(warm):
        w.sweep_0_to_beta()
        w.sweep_beta_to_0()
    alltau = list(range(160))
    r = np.arange(64)
    rx, ry = r % 8, r // 8
    ff = np.array([[np.cos(-(rx * kx + ry * ky))] for kx, ky in kstars])[:, 0, :]  # [k][r]
    prev = None
    out = {"dos": [], "dss": [], "greens": []}
    for _ in range(nbins):
        sg = 0.0
        for _ in range(binsize):
            w.sweep_dynamic(alltau)
            sg += w.sign
            w.sweep_beta_to_0()
        d, c, _ = w.dynamic_obs()
        S = w.dynamic_r()
        cur = (d.copy(), c.copy(), S.copy())
        if prev is not None:
            d, c, S = d - prev[0], c - prev[1], S - prev[2]
        prev = cur
        norm = binsize * (sg / binsize)  # MeasureHandler::normalize_stats with the dynamic sign
        out["dos"].append(d[taus] / norm)
        out["dss"].append(c[taus] / norm)
        out["greens"].append((ff @ S.T)[:, taus] / norm)
    return {k: np.array(v) for k, v in out.items()}


@pytest.mark.slow
def test_statistical_pin_dynamic_against_reference_example(oracle_mod, example_fixture):
    """Oracle dynamic observables vs the reference's example/output/dos.out, dss.out and
    greens.out (attractive 8x8, beta = 8, warm-started from fields.out)."""
    import os

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    dyn = example_fixture["dynamic"]
    taus = dyn["taus"]
    L = 8
    ks_all = [(i / L * 2 * np.pi - np.pi, j / L * 2 * np.pi - np.pi)
              for i in range(L // 2, L + 1) for j in range(L // 2, i + 1)]
    kstars = [ks_all[k] for k in dyn["greens_kstars"]]
    jobs = [(root, 900 + k, example_fixture["fields"], 4, 3, 8, taus, kstars) for k in range(8)]
    with mp.get_context("spawn").Pool(8) as pool:
        res = pool.map(_pin_chain_dynamic, jobs)

    def check(name, bins, ref):
        bins = np.concatenate(bins)
        mean = bins.mean(axis=0)
        err = np.sqrt(np.maximum((bins ** 2).mean(axis=0) - mean ** 2, 0)) / np.sqrt(len(bins) - 1)
        ref = np.array(ref)
        sigma = np.hypot(err, ref[..., 1])
        # bins of one chain are autocorrelated: allow 5 combined sigma
        bad = np.abs(mean - ref[..., 0]) > 5 * sigma
        assert not bad.any(), (name, mean[bad], err[bad], ref[..., 0][bad], ref[..., 1][bad])

    check("density_of_states", [r["dos"] for r in res], dyn["density_of_states"])
    check("dynamic_spin_susceptibility", [r["dss"] for r in res], dyn["dynamic_spin_susceptibility"])
    check("greens_functions", [r["greens"] for r in res], dyn["greens_functions"])
