"""GPU tests of batched Chebyshev propagation: trajectories of uneven size
advanced by one launch per nuclear step give the same result as each
trajectory alone (FP64: 1e-12; FP32: 1e-6) and match the oracle."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix():
    sizes = [(24, 11), (64, 7), (40, 5), (90, 3), (32, 13)]
    return [systems.cubic_cluster(n_atoms=n, seed=s) for n, s in sizes]


def _alone(elhl, sysm, nsteps, prec):
    tr = elhl.Trajectory(sysm, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=2, cheb_tol=1e-14)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    tr.init_fmo(homo + 1, homo)
    pops = tr.step(None, nsteps=nsteps)
    tr.close()
    return pops


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-6)])
def test_batch_equals_alone(elhl, mix, prec, tol):
    b = elhl.Batch(mix, dt=1e-4, precision=prec, ncols=2, cheb_tol=1e-14)
    b.init_fmo()
    pops = b.step(4)
    st = b.stats()
    assert st.prop_launches == 4
    for i, sysm in enumerate(mix):
        alone = _alone(elhl, sysm, 4, prec)
        assert np.abs(pops[:, i] - alone).max() < tol
    b.close()


def test_batch_member_vs_exact(elhl, oracle_mod, mix):
    b = elhl.Batch(mix, dt=1e-4, precision=0, ncols=2, cheb_tol=1e-14)
    b.init_fmo()
    b.compact()
    pops = b.step(3)
    for i in (0, 3):
        sysm = mix[i]
        S = oracle_mod.overlap(sysm)
        homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
        bra, ket = oracle_mod.initial_states(sysm, S, homo + 1, homo)
        h = oracle_mod.huckel(sysm, S)
        ex = oracle_mod.ExactPropagator(S, h)
        ref = oracle_mod.exact_populations(sysm, S, ex.ket(ket, 3e-4)).T
        assert np.abs(pops[-1, i] - ref).max() < 1e-10
    b.close()


def test_ensemble_columns(elhl, oracle_mod):
    """nparticles = 6 fragment MOs propagated as one trajectory."""
    sysm = systems.cubic_cluster(n_atoms=40, seed=5)
    tr = elhl.Trajectory(sysm, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=0, ncols=6, nparticles=6,
                         cheb_tol=1e-14)
    states = [3, 8, 15, 22, 30, 41]
    tr.init_fmo_states(states)
    pops = tr.step(None, nsteps=2)
    S = oracle_mod.overlap(sysm)
    h = oracle_mod.huckel(sysm, S)
    ex = oracle_mod.ExactPropagator(S, h)
    for c, st in enumerate(states):
        ket0, _ = oracle_mod.fragment_mo(sysm, "E", st)
        ref = oracle_mod.exact_populations(sysm, S, ex.ket(ket0.astype(complex), 2e-4))
        assert np.abs(pops[-1, c] - ref).max() < 1e-10
    tr.close()
