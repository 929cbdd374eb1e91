"""Norm and convergence control of the Chebyshev path (the counterpart of the
Taylor path's |<bra|ket>| - norm_ref test, Taylor.f:103-114, and its tau
retries, Taylor.f:65-70).

The failure is made on the host: `lanczos_guard` < 0 shrinks the spectral
interval so that part of the spectrum falls outside [-1, 1] and the truncated
expansion is wrong.  Every test must see the retry or the error, never a
silently wrong answer.  On the config-1 flake a guard of -0.3 leaves 40 % of
the spectrum inside the interval (per-step norm drift about 2e-3); widening by
half the width twice covers 90 % and brings the drift to about 1e-12.  A guard
of -0.44 (12 %) still drifts by about 1e-4 after three widenings."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


def _exact(oracle_mod, sysm, ket0, t):
    S = oracle_mod.overlap(sysm)
    h = oracle_mod.huckel(sysm, S)
    ex = oracle_mod.ExactPropagator(S, h)
    return oracle_mod.exact_populations(sysm, S, ex.ket(ket0, t)).T


def _traj(elhl, sysm, prec, **kw):
    tr = elhl.Trajectory(sysm, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=2, cheb_tol=1e-14,
                         **kw)
    tr.init_fmo(41, 40)
    return tr


def test_fp64_shrunk_interval_is_redone(elhl, oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    _, ket = oracle_mod.initial_states(flake, S, 41, 40)
    tr = _traj(elhl, flake, elhl.PREC_FP64, lanczos_guard=-0.3)
    pops = tr.step(None, nsteps=5)
    st = tr.stats()
    tr.close()
    assert st.cheb_retries >= 1
    assert st.norm_drift < 1e-8
    assert np.abs(pops[-1] - _exact(oracle_mod, flake, ket, 5e-4)).max() < 1e-9


def test_fp64_shrunk_interval_without_retries_fails(elhl, flake):
    tr = _traj(elhl, flake, elhl.PREC_FP64, lanczos_guard=-0.3, cheb_max_retries=0)
    with pytest.raises(elhl.ElhlError) as e:
        tr.step(None, nsteps=3)
    st = tr.stats()
    tr.close()
    assert e.value.status == elhl.ERR_NO_CONVERGENCE
    assert st.norm_drift > 1e-8


def test_fp32_drift_beyond_renormalisation_fails(elhl, oracle_mod, flake):
    """Reduced precision renormalises every step; the drift before that is
    checked first (tolerance 1e-4), so a diverging expansion is reported."""
    tr = _traj(elhl, flake, elhl.PREC_FP32, lanczos_guard=-0.44)
    with pytest.raises(elhl.ElhlError) as e:
        tr.step(None, nsteps=2)
    tr.close()
    assert e.value.status == elhl.ERR_NO_CONVERGENCE
    # with more retries allowed the interval grows until the step is accepted
    S = oracle_mod.overlap(flake)
    _, ket = oracle_mod.initial_states(flake, S, 41, 40)
    tr = _traj(elhl, flake, elhl.PREC_FP32, lanczos_guard=-0.44, cheb_max_retries=8)
    pops = tr.step(None, nsteps=2)
    st = tr.stats()
    tr.close()
    assert st.cheb_retries >= 4
    assert np.abs(pops[-1] - _exact(oracle_mod, flake, ket, 2e-4)).max() < 1e-5


def test_moving_nuclei_shrunk_interval_is_redone(elhl, oracle_mod):
    sysm = systems.cubic_cluster(n_atoms=64, seed=7)
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=3) for i in range(3)])
    S0 = oracle_mod.overlap(sysm, coords[0])
    bra, ket = oracle_mod.initial_states(sysm, S0, 41, 40)
    ref = oracle_mod.ReferenceStep(sysm, bra, ket, dt=5e-4, tol=1e-12, norm_tol=1e-12, nthreads=4)
    rp = np.stack([ref.step(coords[1 + i]).T for i in range(2)])
    tr = elhl.Trajectory(sysm, coords=coords[0], dt=5e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64,
                         ncols=4, cheb_tol=1e-14, lanczos_guard=-0.3)
    tr.set_psi(bra, ket)
    pops = tr.step(coords[1:], nsteps=2)
    st = tr.stats()
    tr.close()
    assert st.cheb_retries >= 2  # the bounds are recomputed (and shrunk) at every rebuild
    assert np.abs(pops - rp).max() < 1e-9


def test_batch_member_divergence_fails_the_step(elhl):
    mix = [systems.cubic_cluster(n_atoms=40, seed=31), systems.cubic_cluster(n_atoms=56, seed=32)]
    b = elhl.Batch(mix, dt=1e-4, precision=elhl.PREC_FP32, ncols=2, cheb_tol=1e-12, lanczos_guard=-0.44)
    b.init_fmo()
    with pytest.raises(elhl.ElhlError) as e:
        b.step(1)
    st = b.stats()
    b.close()
    assert e.value.status == elhl.ERR_NO_CONVERGENCE
    assert st.norm_drift > 1e-4


def test_server_request_divergence_is_reported(elhl):
    sysm = systems.cubic_cluster(n_atoms=40, seed=33)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    sv = elhl.Server(4e9, dt=1e-4, precision=elhl.PREC_FP32, cheb_tol=1e-12, lanczos_guard=-0.44)
    rid = sv.submit(sysm, 3, [homo + 1, homo])
    for _ in range(10):
        sv.step()
        if rid in sv.poll():
            break
    with pytest.raises(elhl.ElhlError) as e:
        sv.result(rid)
    sv.close()
    assert e.value.status == elhl.ERR_NO_CONVERGENCE


def test_grid_barrier_timeout_is_reported(elhl, flake):
    """A CTA that leaves the propagation launch before its first grid barrier
    (the test hook) leaves the others waiting until their limit (0.2 s here):
    the call returns ELHL_ERR_TIMEOUT, and the device stays usable."""
    tr = _traj(elhl, flake, elhl.PREC_FP64)
    tr.step(None, nsteps=1)
    elhl.debug_barrier(0.2, 5)
    try:
        with pytest.raises(elhl.ElhlError) as e:
            tr.step(None, nsteps=1)
    finally:
        elhl.debug_barrier(0.0, -1)
    tr.close()
    assert e.value.status == elhl.ERR_TIMEOUT
    tr = _traj(elhl, flake, elhl.PREC_FP64)  # a fresh launch on the same context succeeds
    pops = tr.step(None, nsteps=2)
    tr.close()
    assert np.isfinite(pops).all() and abs(pops[-1, 0, -1] - 1.0) < 1e-10
