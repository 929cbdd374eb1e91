"""CPU tests of the oracle: closed-form and quadrature pins of the STO overlap,
matrix invariants, and the Taylor restatement against the exact propagator."""
import math

import numpy as np
import pytest

from dynemol_gb300 import systems


def two_atom(sym_a, sym_b, vec):
    s = systems.EHTSystem([sym_a, sym_b], np.array([[0.0, 0.0, 0.0], list(vec)]), np.zeros(2, np.int32),
                          np.ones(2, bool), np.ones(2, bool))
    return s.build_basis()


def test_h2_overlap_closed_form(oracle_mod):
    """1s-1s, equal exponents: S = exp(-p)(1 + p + p^2/3), p = zeta R."""
    for vec in ([0.3, 0.4, 0.5], [0.0, 0.0, 0.74], [1.2, -0.7, 0.1], [0.0, 2.5, 0.0]):
        h2 = two_atom("H", "H", vec)
        S = oracle_mod.overlap(h2)
        p = h2.ao_zeta[0, 0] * np.linalg.norm(vec)
        assert S[0, 1] == pytest.approx(math.exp(-p) * (1 + p + p * p / 3), abs=2e-15)


def _sto(n, zeta, r):
    return (2 * zeta) ** (n + 0.5) / math.sqrt(math.factorial(2 * n)) * r ** (n - 1) * np.exp(-zeta * r)


def _quad_overlap(fa, fb, R):
    """Two-centre overlap by Gauss-Legendre quadrature in prolate spheroidal
    coordinates (A at z = -R/2, B at z = +R/2, a(mu, nu) density)."""
    from numpy.polynomial.legendre import leggauss
    xm, wm = leggauss(200)
    xn, wn = leggauss(200)
    # mu in [1, inf): mu = 1 + t/(1-t), t in [0,1)
    t = 0.5 * (xm + 1.0)
    mu = 1.0 + t / (1.0 - t)
    dmu = 0.5 * wm / (1.0 - t) ** 2
    nu = xn
    MU, NU = np.meshgrid(mu, nu, indexing="ij")
    ra = 0.5 * R * (MU + NU)
    rb = 0.5 * R * (MU - NU)
    cos_a = (1.0 + MU * NU) / (MU + NU)        # angle at A measured along +z (towards B)
    cos_b = (MU * NU - 1.0) / (MU - NU)        # angle at B measured along +z
    jac = (R / 2.0) ** 3 * (MU * MU - NU * NU) * 2.0 * np.pi
    val = fa(ra, cos_a) * fb(rb, cos_b) * jac
    return float(np.einsum("i,j,ij->", dmu, wn, val))


def test_ch_overlaps_vs_quadrature(oracle_mod):
    """C 2s / 2p(sigma) with H 1s against direct numerical integration."""
    R = 1.09
    ch = two_atom("C", "H", [0.0, 0.0, R])  # H on +z of C
    S = oracle_mod.overlap(ch)
    zc = ch.ao_zeta[0, 0]
    zh = ch.ao_zeta[4, 0]
    y00 = 1.0 / math.sqrt(4 * math.pi)
    y10 = math.sqrt(3.0 / (4 * math.pi))
    s2s1s = _quad_overlap(lambda r, c: _sto(2, zc, r) * y00, lambda r, c: _sto(1, zh, r) * y00, R)
    p2s1s = _quad_overlap(lambda r, c: _sto(2, zc, r) * y10 * c, lambda r, c: _sto(1, zh, r) * y00, R)
    assert S[0, 4] == pytest.approx(s2s1s, rel=1e-9)
    # p_z (m = 0) on C pointing at the H: positive overlap
    assert S[2, 4] == pytest.approx(p2s1s, rel=1e-9)
    # p_x, p_y are orthogonal to the bond
    assert abs(S[1, 4]) < 1e-15 and abs(S[3, 4]) < 1e-15


def test_cc_pi_sigma_vs_quadrature(oracle_mod):
    """C-C along z: p_z p_z (sigma) and p_x p_x (pi)."""
    R = 1.42
    cc = two_atom("C", "C", [0.0, 0.0, R])
    S = oracle_mod.overlap(cc)
    z = cc.ao_zeta[0, 0]
    y10 = math.sqrt(3.0 / (4 * math.pi))
    sig = _quad_overlap(lambda r, c: _sto(2, z, r) * y10 * c, lambda r, c: _sto(2, z, r) * y10 * c, R)
    # pi: p_x p_x = (3/4pi) sin^2 ... average over azimuth: 1/2 sin_a sin_b
    pi = _quad_overlap(lambda r, c: _sto(2, z, r) * y10 * np.sqrt(np.clip(1 - c * c, 0, None)),
                       lambda r, c: _sto(2, z, r) * y10 * np.sqrt(np.clip(1 - c * c, 0, None)), R) * 0.5
    assert S[2, 6] == pytest.approx(sig, rel=1e-8)
    assert S[3, 7] == pytest.approx(pi, rel=1e-8)
    assert S[1, 5] == pytest.approx(pi, rel=1e-8)


def test_rotation_invariance(oracle_mod):
    """|S| block invariants are independent of the bond direction."""
    base = oracle_mod.overlap(two_atom("C", "O", [0.0, 0.0, 1.3]))
    rng = np.random.default_rng(0)
    for _ in range(5):
        v = rng.normal(size=3)
        v *= 1.3 / np.linalg.norm(v)
        S = oracle_mod.overlap(two_atom("C", "O", v))
        blk, b0 = S[:4, 4:], base[:4, 4:]
        assert np.linalg.svd(blk, compute_uv=False) == pytest.approx(np.linalg.svd(b0, compute_uv=False), abs=1e-14)
        assert S[0, 4] == pytest.approx(base[0, 4], abs=1e-15)


def test_matrix_invariants(oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    assert np.array_equal(S, S.T) and np.array_equal(h, h.T)
    assert np.all(S.diagonal() == 1.0)
    assert np.linalg.eigvalsh(S).min() > 0.0
    assert np.allclose(h.diagonal(), flake.ao_ip)
    # cutoff: atoms further than 12 A apart do not couple
    d = np.linalg.norm(flake.coords[flake.ao_atom][:, None] - flake.coords[flake.ao_atom][None], axis=2)
    assert np.all(S[d > 12.0] == 0.0)
    Si = oracle_mod.sy_invert(S)
    assert np.abs(Si @ S - np.eye(flake.nao)).max() < 1e-12
    Hp = oracle_mod.h_prime(Si, h)
    assert np.abs(S @ Hp - h).max() < 1e-11


def test_wolfsberg_helmholz(oracle_mod):
    """Off-diagonal X_ij for C 2s - H 1s (hamiltonians.f:48-61)."""
    ch = two_atom("C", "H", [0.0, 0.0, 1.09])
    S = oracle_mod.overlap(ch)
    h = oracle_mod.huckel(ch, S)
    ipi, ipj = -21.4, -13.6
    c3 = ((ipi - ipj) / (ipi + ipj)) ** 2
    keff = 1.75 + c3 + c3 * c3 * (1 - 1.75)
    assert h[0, 4] == pytest.approx(keff * (ipi + ipj) / 2 * S[0, 4], rel=1e-15)


def test_initial_states(oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    homo = systems.fermi_state(flake, np.arange(20))
    assert homo == 40
    bra, ket = oracle_mod.initial_states(flake, S, homo + 1, homo)
    for p in range(2):
        assert np.vdot(ket[:, p], S @ ket[:, p]).real == pytest.approx(1.0, abs=1e-12)
        pops = oracle_mod.populations(flake, bra[:, p], ket[:, p])
        assert pops[0] == pytest.approx(1.0, abs=1e-12) and pops[-1] == pytest.approx(1.0, abs=1e-12)


def test_taylor_vs_exact(oracle_mod, flake):
    """The Taylor restatement at tolerance 1e-12 tracks the exact propagator."""
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    step = oracle_mod.ReferenceStep(flake, bra, ket, dt=1e-4, tol=1e-12, norm_tol=1e-12, nthreads=4)
    ex = oracle_mod.ExactPropagator(S, h)
    for _ in range(5):
        pops = step.step()
    ref = oracle_mod.exact_populations(flake, S, ex.ket(ket, step.t))
    assert np.abs(pops - ref).max() < 1e-10
    # norm conservation (Taylor.f:103-104)
    for p in range(2):
        assert abs(abs(np.vdot(step.bra[:, p], step.ket[:, p])) - 1.0) < 1e-11


def test_taylor_default_tolerance(oracle_mod, flake):
    """At the reference's 1e-8 thresholds the error stays at that level."""
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    step = oracle_mod.ReferenceStep(flake, bra, ket, dt=1e-4, nthreads=4)
    ex = oracle_mod.ExactPropagator(S, h)
    for _ in range(3):
        pops = step.step()
    ref = oracle_mod.exact_populations(flake, S, ex.ket(ket, step.t))
    assert np.abs(pops - ref).max() < 1e-7
    assert step.stats[0].gemv_terms > 0 and step.stats[1].gemv_terms > 0


def test_two_level_rabi(oracle_mod):
    """Orthogonal two-level system: populations follow cos^2(V t / hbar)."""
    V = 0.5  # eV
    Hp = np.array([[0.0, V], [V, 0.0]], order="F")
    bra = np.array([1.0 + 0j, 0.0])
    ket = bra.copy()
    t_max = 2e-3
    b, k, _, _, st = oracle_mod.propagate(Hp, bra, ket, 0.0, t_max, t_max / oracle_mod.H_BAR, tol=1e-13,
                                          norm_tol=1e-13)
    p0 = (np.conj(k[0]) * b[0]).real
    assert p0 == pytest.approx(math.cos(V * t_max / oracle_mod.H_BAR) ** 2, abs=1e-11)


def test_no_convergence_is_bounded(oracle_mod):
    Hp = np.full((3, 3), np.nan, order="F")
    v = np.array([1.0 + 0j, 0, 0])
    _, _, _, _, st = oracle_mod.propagate(Hp, v, v, 0.0, 1e-4, 0.15, max_conv_calls=5)
    assert st.status == 1 and st.conv_calls == 5


def test_pulay_forces_h2_closed_form(oracle_mod):
    """Two H 1s STOs (equal zeta): S(R) = e^{-zR}(1 + zR + (zR)^2/3); with
    kernel(0, 1) = kernel(1, 0) = 1 the force on atom 0 is
    2 e2N (-dS/dx_0) and on atom 1 its negative."""
    sysm = two_atom("H", "H", [0.74, 0.21, -0.13])
    X = sysm.coords
    kern = np.array([[0.0, 1.0], [1.0, 0.0]])
    f = oracle_mod.pulay_forces(sysm, kern, delta=1e-5)
    z = sysm.ao_zeta[0, 0]
    R = np.linalg.norm(X[1] - X[0])
    dS_dR = -z * np.exp(-z * R) * (1 + z * R + (z * R) ** 2 / 3) + np.exp(-z * R) * (z + 2 * z * z * R / 3)
    dS_dx0 = dS_dR * (X[0] - X[1]) / R
    ref0 = 2 * 1.602176565e-9 * (-dS_dx0)
    assert np.abs(f[0] - ref0).max() < 1e-8 * np.abs(ref0).max()
    assert np.abs(f[0] + f[1]).max() < 1e-20


def test_huckel_with_fields_zero_field_is_huckel(oracle_mod):
    """With zero dipole matrix and zero fields the field Hamiltonian is the plain
    Wolfsberg-Helmholz h of the oracle's C restatement."""
    from dynemol_gb300 import systems
    c = systems.cubic_cluster(n_atoms=12, seed=3)
    S = oracle_mod.overlap(c)
    h0 = oracle_mod.huckel(c, S)
    hf = oracle_mod.huckel_with_fields(c, S, np.zeros((c.nao, c.nao, 3)), np.zeros((c.natoms, c.natoms, 4)))
    assert np.abs(hf - h0).max() < 1e-14 * np.abs(h0).max()


def test_huckel_with_fields_uniform_potential(oracle_mod):
    """A uniform potential phi (DP_1 = phi, no field) shifts every off-diagonal
    element with |S_ij| > 1e-7 by -phi S_ij."""
    from dynemol_gb300 import systems
    c = systems.cubic_cluster(n_atoms=12, seed=3)
    S = oracle_mod.overlap(c)
    dp4 = np.zeros((c.natoms, c.natoms, 4))
    dp4[:, :, 0] = 0.37
    hf = oracle_mod.huckel_with_fields(c, S, np.zeros((c.nao, c.nao, 3)), dp4)
    h0 = oracle_mod.huckel(c, S)
    off = ~np.eye(c.nao, dtype=bool) & (np.abs(S) > 1e-7)
    assert np.abs((hf - h0)[off] + 0.37 * S[off]).max() < 1e-13
