"""GPU tests of the Ehrenfest force pieces: the kernel K = X o A - H' A
(ehrenfestkernel[2]_gpu_) and the Pulay overlap-derivative forces
(elhl_ehrenfest_forces) against the oracle."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cluster():
    return systems.cubic_cluster(n_atoms=24, seed=21)


def _kernel(rng, n):
    return rng.normal(size=(n, n))


def test_pulay_forces_match_oracle(elhl, oracle_mod, cluster):
    """delta = 1e-5: both sides difference the same S blocks; relative 1e-9."""
    K = _kernel(np.random.default_rng(1), cluster.nao)
    f = elhl.ehrenfest_forces(cluster, K, delta=1e-5)
    fo = oracle_mod.pulay_forces(cluster, K, delta=1e-5)
    scale = np.abs(fo).max()
    assert scale > 0
    assert np.abs(f - fo).max() < 1e-9 * scale
    assert np.abs(f.sum(0)).max() < 1e-12 * scale  # action = reaction


def test_pulay_forces_reference_delta(elhl, oracle_mod, cluster):
    """The reference's delta = 1e-8 Angstrom: S round-off (~1e-16) over 2 delta
    limits agreement to ~1e-7 of the largest force; tested at 1e-5."""
    K = _kernel(np.random.default_rng(2), cluster.nao)
    f = elhl.ehrenfest_forces(cluster, K)
    fo = oracle_mod.pulay_forces(cluster, K, delta=1e-8)
    fo5 = oracle_mod.pulay_forces(cluster, K, delta=1e-5)
    scale = np.abs(fo5).max()
    assert np.abs(f - fo).max() < 1e-5 * scale
    assert np.abs(f - fo5).max() < 1e-5 * scale


def test_forces_from_propagated_state(elhl, oracle_mod, flake):
    """The reference's chain on the flake: A = sym(rho) from the propagated bra/ket,
    K = X o A - H' A, then the Pulay forces (parity with the oracle chain)."""
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    Hp = oracle_mod.h_prime(oracle_mod.sy_invert(S), h)
    X = np.where(np.abs(S) > 0, h / np.where(S == 0, 1, S), 0.0)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    Kg = elhl.ehrenfest_kernel(Hp, X, bra=bra, ket=ket)
    Ko = oracle_mod.ehrenfest_kernel(Hp, X, bra=bra, ket=ket)
    assert np.abs(Kg - Ko).max() < 1e-10 * np.abs(Ko).max()
    sub = systems.EHTSystem(flake.symbols[:30], flake.coords[:30].copy(), flake.fragment[:30].copy(),
                            flake.el_atoms[:30].copy(), flake.hl_atoms[:30].copy()).build_basis()
    n = sub.nao
    f = elhl.ehrenfest_forces(sub, Ko[:n, :n], delta=1e-5)
    fo = oracle_mod.pulay_forces(sub, Ko[:n, :n], delta=1e-5)
    assert np.abs(f - fo).max() < 1e-9 * np.abs(fo).max()


def test_huckel_with_fields_matches_oracle(elhl, oracle_mod, cluster):
    """elhl_huckel_with_fields against the oracle with random dipole matrix and
    pair fields (the same IEEE operations: 1e-13 relative)."""
    rng = np.random.default_rng(7)
    S = oracle_mod.overlap(cluster)
    dp_ao = rng.normal(size=(cluster.nao, cluster.nao, 3))
    dp4 = rng.normal(size=(cluster.natoms, cluster.natoms, 4))
    h = elhl.huckel_with_fields(cluster, S, dp_ao, dp4)
    ho = oracle_mod.huckel_with_fields(cluster, S, dp_ao, dp4)
    assert np.abs(h - ho).max() < 1e-13 * np.abs(ho).max()
