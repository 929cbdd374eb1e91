"""GPU parity tests: libelhlprop.so (through its C ABI) against the oracle.

Tolerances: S, h and the initial states to 1e-12 absolute (same FP64
arithmetic, different operation order / FMA contraction); H' = S^-1 h to 1e-10
relative (Cholesky solve vs Bunch-Kaufman inverse, cond(S) ~ 20); populations
within 1e-10 with both sides run at Taylor tolerance 1e-12, within 5e-8 at the
reference's own 1e-8 thresholds."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cluster_small():
    return systems.cubic_cluster(n_atoms=64, seed=7)


def test_build_sh_matches_oracle(elhl, oracle_mod, flake, cluster_small):
    for sysm in (flake, cluster_small):
        tr = elhl.Trajectory(sysm)
        S, h, Hp = tr.matrices()
        So = oracle_mod.overlap(sysm)
        ho = oracle_mod.huckel(sysm, So)
        assert np.abs(S - So).max() < 1e-13
        assert np.abs(h - ho).max() < 1e-11
        Hpo = oracle_mod.h_prime(oracle_mod.sy_invert(So), ho)
        assert np.abs(Hp - Hpo).max() < 1e-10 * np.abs(Hpo).max()
        tr.close()


def test_fmo_initial_states(elhl, oracle_mod, flake):
    tr = elhl.Trajectory(flake)
    tr.init_fmo(41, 40)
    b, k = tr.get_psi()
    S = oracle_mod.overlap(flake)
    bo, ko = oracle_mod.initial_states(flake, S, 41, 40)
    assert np.abs(k - ko).max() < 1e-10
    assert np.abs(b - bo).max() < 1e-10
    tr.close()


def _oracle_run(oracle_mod, sysm, nsteps, coords=None, **kw):
    S = oracle_mod.overlap(sysm, coords[0] if coords is not None else None)
    bra, ket = oracle_mod.initial_states(sysm, S, 41, 40)
    st = oracle_mod.ReferenceStep(sysm, bra, ket, dt=1e-4, nthreads=4, **kw)
    pops = [st.step(None if coords is None else coords[i]) for i in range(nsteps)]
    return np.stack([p.T for p in pops]), st, bra, ket


def test_fixed_nuclei_propagation_tight(elhl, oracle_mod, flake):
    """Config-1 system, 10 steps of 0.1 fs, Taylor tolerance 1e-12 on both sides."""
    po, st, bra, ket = _oracle_run(oracle_mod, flake, 10, tol=1e-12, norm_tol=1e-12)
    tr = elhl.Trajectory(flake, dt=1e-4, tol=1e-12, norm_tol=1e-12)
    tr.set_psi(bra, ket)
    pg = tr.step(None, nsteps=10)
    assert np.abs(pg - po).max() < 1e-10
    b, k = tr.get_psi()
    assert np.abs(k - st.ket).max() < 1e-9
    tr.close()


def test_fixed_nuclei_reference_tolerance(elhl, oracle_mod, flake):
    """At the reference's 1e-8 thresholds the tau sequence matches the oracle."""
    po, st, bra, ket = _oracle_run(oracle_mod, flake, 5)
    tr = elhl.Trajectory(flake, dt=1e-4)
    tr.set_psi(bra, ket)
    pg = tr.step(None, nsteps=5)
    assert np.abs(pg - po).max() < 5e-8
    s = tr.stats()
    assert list(s.save_tau) == pytest.approx(list(st.save_tau), rel=1e-12)
    tr.close()


def test_one_step_at_a_time_equals_multi_step(elhl, oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    a = elhl.Trajectory(flake, dt=1e-4)
    a.set_psi(bra, ket)
    pa = a.step(None, nsteps=4)
    b = elhl.Trajectory(flake, dt=1e-4)
    b.set_psi(bra, ket)
    pb = np.concatenate([b.step(None, nsteps=1) for _ in range(4)])
    assert np.array_equal(pa, pb)
    a.close(); b.close()


def test_moving_nuclei(elhl, oracle_mod, cluster_small):
    """Per-step rebuild of S, h, H' from perturbed coordinates."""
    base = cluster_small.coords
    coords = np.stack([systems.perturbed_coords(base, i, seed=3) for i in range(4)])
    po, st, bra, ket = _oracle_run(oracle_mod, cluster_small, 3, coords=coords[1:], tol=1e-12, norm_tol=1e-12)
    tr = elhl.Trajectory(cluster_small, coords=coords[1], dt=1e-4, tol=1e-12, norm_tol=1e-12)
    tr.set_psi(bra, ket)
    pg = tr.step(coords[1:], nsteps=3)
    assert np.abs(pg - po).max() < 1e-10
    tr.close()


def test_dropin_propagationelhl(elhl, oracle_mod, flake):
    """propagationelhl_gpucaller_ against the oracle for one particle and step."""
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    Si = oracle_mod.sy_invert(S)
    Hpo = oracle_mod.h_prime(Si, h)
    tau = 1e-4 / oracle_mod.H_BAR
    bo, ko, _, sto, _ = oracle_mod.propagate(Hpo, bra[:, 0], ket[:, 0], 0.0, 1e-4, tau)
    pb = np.ascontiguousarray(bra[:, 0])
    pk = np.ascontiguousarray(ket[:, 0])
    Hp, ao_bra, pb, pk, st = elhl.propagationelhl_gpucaller(S, h, pb, pk, 0.0, 1e-4, tau)
    assert np.abs(Hp - Hpo).max() < 1e-10 * np.abs(Hpo).max()
    assert st == pytest.approx(sto, rel=1e-12)
    assert np.abs(pk - ko).max() < 1e-8 and np.abs(pb - bo).max() < 1e-8
    assert np.abs(ao_bra - Si @ pb).max() < 1e-10


def test_dropin_propagation_single(elhl, oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    Hpo = oracle_mod.h_prime(oracle_mod.sy_invert(S), h)
    tau = 1e-4 / oracle_mod.H_BAR
    bo, ko, _, sto, _ = oracle_mod.propagate(Hpo, bra[:, 1], ket[:, 1], 0.0, 1e-4, tau)
    pb = np.ascontiguousarray(bra[:, 1])
    pk = np.ascontiguousarray(ket[:, 1])
    pb, pk, st = elhl.propagation_gpucaller(Hpo, pb, pk, 0.0, 1e-4, tau)
    assert st == pytest.approx(sto, rel=1e-12)
    assert np.abs(pk - ko).max() < 1e-8


@pytest.mark.parametrize("sym,vec", [("H", [0.0, 0.0, 0.9]), ("C", [0.3, 1.1, 0.4])])
def test_tiny_systems(elhl, oracle_mod, sym, vec):
    """N = 2 and N = 8: fewer rows than CTAs."""
    s = systems.EHTSystem([sym, sym], np.array([[0.0, 0, 0], vec]), np.array([0, 1], np.int32),
                          np.array([True, False]), np.array([True, False])).build_basis()
    S = oracle_mod.overlap(s)
    h = oracle_mod.huckel(s, S)
    Hpo = oracle_mod.h_prime(oracle_mod.sy_invert(S), h)
    v = np.zeros(s.nao, np.complex128)
    v[0] = 1.0
    bra = (S @ v).astype(np.complex128)
    tau = 1e-4 / oracle_mod.H_BAR
    bo, ko, _, sto, _ = oracle_mod.propagate(Hpo, bra, v, 0.0, 1e-4, tau)
    pb, pk, st = elhl.propagation_gpucaller(Hpo, bra.copy(), v.copy(), 0.0, 1e-4, tau)
    assert np.abs(pk - ko).max() < 1e-9


def test_not_positive_definite(elhl):
    S = np.array([[1.0, 2.0], [2.0, 1.0]], order="F")
    h = np.eye(2, order="F")
    v = np.array([1.0 + 0j, 0.0])
    with pytest.raises(elhl.ElhlError) as e:
        elhl.propagationelhl_gpucaller(S, h, v.copy(), v.copy(), 0.0, 1e-4, 0.15)
    assert e.value.status == elhl.ERR_NOT_PD


def test_nan_hamiltonian_reports_no_convergence(elhl):
    Hp = np.full((4, 4), np.nan, order="F")
    v = np.zeros(4, np.complex128)
    v[0] = 1.0
    with pytest.raises(elhl.ElhlError) as e:
        elhl.propagation_gpucaller(Hp, v.copy(), v.copy(), 0.0, 1e-4, 0.15)
    assert e.value.status == elhl.ERR_NO_CONVERGENCE


def test_bad_arguments(elhl, flake):
    with pytest.raises(elhl.ElhlError) as e:
        elhl.propagation_gpucaller(np.zeros((0, 0), order="F"), np.zeros(0, np.complex128),
                                   np.zeros(0, np.complex128), 0.0, 1e-4, 0.1)
    assert e.value.status == elhl.ERR_BAD_ARG
    with pytest.raises(ValueError):
        tr = elhl.Trajectory(flake)
        tr.step(np.zeros(5), nsteps=1)


@pytest.mark.parametrize("method", [0, 1])
def test_energies_match_oracle(elhl, oracle_mod, flake, method):
    """QuasiParticleEnergies after 3 steps, Taylor and Chebyshev trajectories."""
    S = oracle_mod.overlap(flake)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    ref = oracle_mod.ReferenceStep(flake, bra, ket, dt=1e-4, tol=1e-12, norm_tol=1e-12, nthreads=4)
    for _ in range(3):
        ref.step()
    Eo = ref.energies()
    kw = dict(dt=1e-4, tol=1e-12, norm_tol=1e-12) if method == 0 else dict(
        dt=1e-4, method=elhl.METHOD_CHEBYSHEV, ncols=4, cheb_tol=1e-14)
    tr = elhl.Trajectory(flake, **kw)
    tr.set_psi(bra, ket)
    tr.step(None, nsteps=3)
    E = tr.energies()
    tr.close()
    assert np.abs(E - Eo).max() < 1e-9


def test_ehrenfest_kernels(elhl, oracle_mod, flake):
    """ehrenfestkernel_gpu_ / ehrenfestkernel2_gpu_ against the oracle (FP64 DGEMM, 1e-10 relative)."""
    rng = np.random.default_rng(4)
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    Hp = oracle_mod.h_prime(oracle_mod.sy_invert(S), h)
    X = rng.normal(size=Hp.shape)
    A = rng.normal(size=Hp.shape)
    K = elhl.ehrenfest_kernel(Hp, X, A=A)
    Ko = oracle_mod.ehrenfest_kernel(Hp, X, A=A)
    assert np.abs(K - Ko).max() < 1e-10 * np.abs(Ko).max()
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    K2 = elhl.ehrenfest_kernel(Hp, X, bra=bra, ket=ket)
    K2o = oracle_mod.ehrenfest_kernel(Hp, X, bra=bra, ket=ket)
    assert np.abs(K2 - K2o).max() < 1e-10 * np.abs(K2o).max()
