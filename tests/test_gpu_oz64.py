"""GPU tests of ELHL_PREC_OZ64: the FP64 Chebyshev propagation with every
operator product computed exactly on the tensor cores from BF16 slices
(dynemol_gb300/csrc/ozaki.cu).  It is an FP64 path, so it is held to the FP64
bars: 1e-10 in populations against the exact propagator and the Taylor oracle,
and it must agree with the FP64-pipe propagation to round-off."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


def _exact(oracle_mod, sysm, ket0, t):
    S = oracle_mod.overlap(sysm)
    h = oracle_mod.huckel(sysm, S)
    ex = oracle_mod.ExactPropagator(S, h)
    return oracle_mod.exact_populations(sysm, S, ex.ket(ket0, t)).T


def test_oz64_fixed_nuclei_vs_exact(elhl, oracle_mod, flake):
    """Config-1 flake (N = 450), explicit operator (one grid phase per order), 20 steps."""
    S = oracle_mod.overlap(flake)
    _, ket = oracle_mod.initial_states(flake, S, 41, 40)
    tr = elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_OZ64, ncols=2,
                         cheb_tol=1e-14)
    tr.init_fmo(41, 40)
    pops = tr.step(None, nsteps=20)
    st = tr.stats()
    tr.close()
    ref = _exact(oracle_mod, flake, ket, 20 * 1e-4)
    assert np.abs(pops[-1] - ref).max() < 1e-10
    assert st.orders > 0 and st.norm_drift < 1e-10


def test_oz64_fixed_nuclei_matches_fp64(elhl, flake):
    """Bra and ket columns (ncols = 4): OZ64 and the FP64 pipe agree to round-off."""
    out = {}
    for prec in (elhl.PREC_FP64, elhl.PREC_OZ64):
        tr = elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=4, cheb_tol=1e-14)
        tr.init_fmo(41, 40)
        pops = tr.step(None, nsteps=10)
        b, k = tr.get_psi()
        tr.close()
        out[prec] = (pops, b, k)
    p0, b0, k0 = out[elhl.PREC_FP64]
    p1, b1, k1 = out[elhl.PREC_OZ64]
    assert np.abs(p1 - p0).max() < 1e-12
    assert np.abs(k1 - k0).max() < 1e-11 and np.abs(b1 - b0).max() < 1e-11


def test_oz64_moving_nuclei_vs_taylor_oracle(elhl, oracle_mod):
    """Moving nuclei with H~ = G h G^T formed every step on the tensor cores (one
    grid phase per order), bra and ket carried through geometry changes, against
    the reference's Taylor step driver at tolerance 1e-12."""
    sysm = systems.cubic_cluster(n_atoms=64, seed=7)
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=3) for i in range(4)])
    S0 = oracle_mod.overlap(sysm, coords[1])
    bra, ket = oracle_mod.initial_states(sysm, S0, 41, 40)
    ref = oracle_mod.ReferenceStep(sysm, bra, ket, dt=5e-4, tol=1e-12, norm_tol=1e-12, nthreads=4)
    rp = np.stack([ref.step(coords[1 + i]).T for i in range(3)])
    tr = elhl.Trajectory(sysm, coords=coords[1], dt=5e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_OZ64,
                         ncols=4, cheb_tol=1e-14)
    tr.set_psi(bra, ket)
    pops = tr.step(coords[1:], nsteps=3)
    st = tr.stats()
    tr.close()
    assert np.abs(pops - rp).max() < 1e-10
    assert st.phases == 1


@pytest.mark.parametrize("n_atoms", [600, 300])
def test_oz64_moving_nuclei_matches_fp64(elhl, n_atoms):
    """N = 1860 (15 row tiles, 68 rows in the last: several segments per tile,
    partial last tile and block) and N = 930 (8 row tiles, 34 rows in the last:
    its diagonal tile has one 64-K block and no second transposed half), two
    moving-nuclei steps: OZ64 against the FP64 pipe."""
    sysm = systems.cubic_cluster(n_atoms=n_atoms, seed=11)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=5) for i in range(3)])
    out = {}
    for prec in (elhl.PREC_FP64, elhl.PREC_OZ64):
        tr = elhl.Trajectory(sysm, coords=coords[0], dt=5e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=4,
                             cheb_tol=1e-14)
        tr.init_fmo(homo + 1, homo)
        pops = tr.step(coords[1:], nsteps=2)
        b, k = tr.get_psi()
        tr.close()
        out[prec] = (pops, b, k)
    p0, b0, k0 = out[elhl.PREC_FP64]
    p1, b1, k1 = out[elhl.PREC_OZ64]
    assert np.abs(p1 - p0).max() < 1e-12
    assert np.abs(k1 - k0).max() < 1e-10 and np.abs(b1 - b0).max() < 1e-10


def test_oz64_unsupported_forms(elhl, flake):
    """More than 4 columns, batches and servers stay on the other precisions."""
    with pytest.raises(elhl.ElhlError):
        elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_OZ64, ncols=8,
                        nparticles=8)
    with pytest.raises(elhl.ElhlError):
        elhl.Server(1e9, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_OZ64)


def test_oz64_stalled_cta_is_reported(elhl, flake):
    """A CTA that leaves the OZ64 propagation launch at once (the test hook) never
    reaches the grid barrier, so the others' waits run out at the 0.2 s limit and
    the call returns ELHL_ERR_TIMEOUT; a fresh launch on the same context then
    succeeds."""
    kw = dict(dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_OZ64, ncols=2, cheb_tol=1e-14)
    tr = elhl.Trajectory(flake, **kw)
    tr.init_fmo(41, 40)
    tr.step(None, nsteps=1)
    elhl.debug_barrier(0.2, 0)
    try:
        with pytest.raises(elhl.ElhlError) as e:
            tr.step(None, nsteps=1)
    finally:
        elhl.debug_barrier(0.0, -1)
    tr.close()
    assert e.value.status == elhl.ERR_TIMEOUT
    tr = elhl.Trajectory(flake, **kw)
    tr.init_fmo(41, 40)
    pops = tr.step(None, nsteps=2)
    tr.close()
    assert np.isfinite(pops).all() and abs(pops[-1, 0, -1] - 1.0) < 1e-10
