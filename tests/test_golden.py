"""The oracle against its committed golden fixtures (tests/golden/, written by
tests/golden/make_golden.py).

The reference ships no golden vectors and cannot be run here, so these pins are
twofold: the oracle must reproduce its own committed outputs (any change to the
restatement that moves a number fails), and its Taylor populations must agree
with the exact generalized-eigenbasis propagator (ElHl_schroedinger.f:131-147)
over the config-1 run.  CPU only, a few seconds."""
import dataclasses
import os

import numpy as np
import pytest

from dynemol_gb300 import systems

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    path = os.path.join(GOLD, name)
    if not os.path.exists(path):
        pytest.fail(f"golden fixture {name} is missing: run tests/golden/make_golden.py")
    return np.load(path)


def test_small_matrices_reproduced(oracle_mod):
    g = _load("small16.npz")
    cl = systems.cubic_cluster(n_atoms=16, seed=11, frag_atoms=6)
    coords = np.stack([systems.perturbed_coords(cl.coords, i, seed=11) for i in range(4)])
    assert np.array_equal(coords, g["coords"])
    S = oracle_mod.overlap(cl, coords[0])
    h = oracle_mod.huckel(cl, S)
    Sinv = oracle_mod.sy_invert(S)
    assert np.abs(S - g["S"]).max() < 1e-15
    assert np.abs(h - g["h"]).max() < 1e-13
    assert np.abs(Sinv - g["Sinv"]).max() < 1e-12
    assert np.abs(oracle_mod.h_prime(Sinv, h) - g["Hp"]).max() < 1e-11


def test_small_moving_steps_reproduced(oracle_mod):
    g = _load("small16.npz")
    cl = systems.cubic_cluster(n_atoms=16, seed=11, frag_atoms=6)
    coords = g["coords"]
    S = oracle_mod.overlap(cl, coords[0])
    homo = int(g["homo"])
    bra, ket = oracle_mod.initial_states(dataclasses.replace(cl, coords=coords[0]), S, homo + 1, homo)
    assert np.abs(ket - g["ket0"]).max() < 1e-13 and np.abs(bra - g["bra0"]).max() < 1e-13
    ref = oracle_mod.ReferenceStep(cl, bra, ket, dt=float(g["dt"]), tol=float(g["tol"]), norm_tol=float(g["tol"]),
                                   nthreads=2)
    pops = np.stack([ref.step(coords[1 + i]).T for i in range(3)])
    assert np.abs(pops - g["pops"]).max() < 1e-12
    assert np.abs(ref.ket - g["ket3"]).max() < 1e-11


def test_flake_taylor_reproduced(oracle_mod, flake):
    g = _load("flake.npz")
    homo = systems.fermi_state(flake, np.arange(20))
    assert homo == int(g["homo"])
    S = oracle_mod.overlap(flake)
    bra, ket = oracle_mod.initial_states(flake, S, homo + 1, homo)
    ref = oracle_mod.ReferenceStep(flake, bra, ket, dt=float(g["dt"]), tol=float(g["tol"]), norm_tol=float(g["tol"]))
    for _ in range(5):
        p = ref.step().T
    assert np.abs(p - g["taylor5"]).max() < 1e-12


def test_flake_exact_reproduced(oracle_mod, flake):
    g = _load("flake.npz")
    homo = int(g["homo"])
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    bra, ket = oracle_mod.initial_states(flake, S, homo + 1, homo)
    ex = oracle_mod.ExactPropagator(S, h)
    assert np.abs(ex.E - g["eig"]).max() < 1e-10
    for n in (200, 2000):
        p = oracle_mod.exact_populations(flake, S, ex.ket(ket, n * float(g["dt"]))).T
        assert np.abs(p - g[f"exact{n}"]).max() < 1e-11


def test_flake_taylor_against_exact_over_200_steps():
    """The committed Taylor run (tolerance 1e-12) and the exact propagator agree
    to 1e-10 after 200 steps: the oracle is accurate well past the tests' bar."""
    g = _load("flake.npz")
    assert np.abs(g["taylor200"] - g["exact200"]).max() < 1e-10
    # populations are conserved: fragments sum to the total, total = 1
    for key in ("taylor200", "exact200", "exact2000"):
        p = g[key]
        assert np.abs(p[:, :-1].sum(axis=1) - p[:, -1]).max() < 1e-12
        assert np.abs(p[:, -1] - 1.0).max() < 1e-10


def test_cluster1200_fixture_consistent():
    """Config 2 (N = 3720, 2 moving-nuclei steps): fragments sum to the total and
    the reference's bra/ket norm is held to its 1e-12 tolerance per step."""
    g = _load("cluster1200.npz")
    p = g["pops"]
    assert p.shape[:2] == (2, 2)
    assert np.abs(p[:, :, :-1].sum(axis=2) - p[:, :, -1]).max() < 1e-12
    assert np.abs(p[:, :, -1] - 1.0).max() < 1e-9
