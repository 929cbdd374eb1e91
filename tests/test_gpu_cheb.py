"""GPU tests of the Chebyshev propagator (symmetrised H~ = L^-1 h L^-T).

FP64: the same exact propagator as the reference's Taylor series, so parity
with the oracle and with the exact eigenbasis propagator is tested at 1e-10 in
populations.  FP32: reduced precision; its error against the exact propagator
is bounded by 1e-5 after 20 steps (the measured value is reported by
bench.py)."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


def _exact(oracle_mod, sysm, ket0, t):
    S = oracle_mod.overlap(sysm)
    h = oracle_mod.huckel(sysm, S)
    ex = oracle_mod.ExactPropagator(S, h)
    return oracle_mod.exact_populations(sysm, S, ex.ket(ket0, t)).T


def _cheb(elhl, sysm, nsteps, prec, ncols, dt=1e-4):
    tr = elhl.Trajectory(sysm, dt=dt, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=ncols, cheb_tol=1e-14)
    tr.init_fmo(41, 40)
    pops = tr.step(None, nsteps=nsteps)
    b, k = tr.get_psi()
    st = tr.stats()
    tr.close()
    return pops, b, k, st


def test_cheb_fp64_fixed_nuclei_vs_exact(elhl, oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    pops, b, k, st = _cheb(elhl, flake, 20, elhl.PREC_FP64, 2)
    ref = _exact(oracle_mod, flake, ket, 20 * 1e-4)
    assert np.abs(pops[-1] - ref).max() < 1e-10
    assert st.orders > 0


def test_cheb_fp64_bra_columns_equal_ket_only(elhl, flake):
    p2, b2, k2, _ = _cheb(elhl, flake, 5, elhl.PREC_FP64, 2)
    p4, b4, k4, _ = _cheb(elhl, flake, 5, elhl.PREC_FP64, 4)
    assert np.abs(p2 - p4).max() < 1e-12
    assert np.abs(k2 - k4).max() < 1e-11 and np.abs(b2 - b4).max() < 1e-11


def test_cheb_fp64_vs_taylor_oracle(elhl, oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    ref = oracle_mod.ReferenceStep(flake, bra, ket, dt=1e-4, tol=1e-12, norm_tol=1e-12, nthreads=4)
    rp = np.stack([ref.step().T for _ in range(5)])
    pops, b, k, _ = _cheb(elhl, flake, 5, elhl.PREC_FP64, 4)
    assert np.abs(pops - rp).max() < 1e-10
    assert np.abs(k - ref.ket).max() < 1e-9 and np.abs(b - ref.bra).max() < 1e-9


def test_cheb_fp64_moving_nuclei_vs_taylor_oracle(elhl, oracle_mod):
    """Bra and ket carried through geometry changes (ncols = 4) as the reference does."""
    sysm = systems.cubic_cluster(n_atoms=64, seed=7)
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=3) for i in range(4)])
    S0 = oracle_mod.overlap(sysm, coords[1])
    bra, ket = oracle_mod.initial_states(sysm, S0, 41, 40)
    ref = oracle_mod.ReferenceStep(sysm, bra, ket, dt=5e-4, tol=1e-12, norm_tol=1e-12, nthreads=4)
    rp = np.stack([ref.step(coords[1 + i]).T for i in range(3)])
    tr = elhl.Trajectory(sysm, coords=coords[1], dt=5e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64,
                         ncols=4, cheb_tol=1e-14)
    tr.set_psi(bra, ket)
    pops = tr.step(coords[1:], nsteps=3)
    tr.close()
    assert np.abs(pops - rp).max() < 1e-9


@pytest.mark.parametrize("prec_name,tol", [("fp64", 1e-11), ("fp32", 5e-6)])
def test_implicit_operator_matches_explicit(elhl, flake, prec_name, tol):
    """Steps given coordinates run the implicit operator G (h/b) G^T (three phases
    per order; G = L^-1 by the recursive Cholesky-with-inverse in FP64, its large
    products on the tensor cores in FP32); fixed-nuclei steps run the explicit H~.  Same
    geometry, same result; fixed steps after moving ones keep the implicit form."""
    prec = {"fp64": elhl.PREC_FP64, "fp32": elhl.PREC_FP32}[prec_name]
    kw = dict(dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=4, cheb_tol=1e-14)
    tr = elhl.Trajectory(flake, **kw)
    tr.init_fmo(41, 40)
    p_ex = tr.step(None, nsteps=4)
    b_ex, k_ex = tr.get_psi()
    tr.close()
    tr = elhl.Trajectory(flake, coords=flake.coords, **kw)
    tr.init_fmo(41, 40)
    c = np.stack([flake.coords] * 2)
    p_im = np.concatenate([tr.step(c, nsteps=2), tr.step(None, nsteps=2)])
    b_im, k_im = tr.get_psi()
    tr.close()
    assert np.abs(p_im - p_ex).max() < tol
    assert np.abs(k_im - k_ex).max() < 10 * tol and np.abs(b_im - b_ex).max() < 10 * tol


def test_implicit_operator_cluster_vs_exact(elhl, oracle_mod):
    """N = 1860 (600-atom cluster): every CTA owns two row chunks of the implicit
    plan; populations after two steps through the moving-nuclei path (unchanged
    geometry) against the exact generalized-eigenbasis propagator."""
    sysm = systems.cubic_cluster(n_atoms=600, seed=11)
    S = oracle_mod.overlap(sysm)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    tr = elhl.Trajectory(sysm, coords=sysm.coords, dt=2e-4, method=elhl.METHOD_CHEBYSHEV,
                         precision=elhl.PREC_FP64, ncols=4, cheb_tol=1e-14)
    tr.init_fmo(homo + 1, homo)
    pops = tr.step(np.stack([sysm.coords] * 2), nsteps=2)
    tr.close()
    ket0, _ = oracle_mod.fragment_mo(sysm, "E", homo + 1)
    ref = _exact(oracle_mod, sysm, np.column_stack([ket0, oracle_mod.fragment_mo(sysm, "H", homo)[0]]).astype(complex),
                 4e-4)
    assert np.abs(pops[-1] - ref).max() < 1e-9
    assert np.abs(pops[:, :, -1] - 1.0).max() < 1e-11


def test_cheb_fp32_error_bound(elhl, oracle_mod, flake):
    S = oracle_mod.overlap(flake)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    pops, b, k, st = _cheb(elhl, flake, 20, elhl.PREC_FP32, 2)
    ref = _exact(oracle_mod, flake, ket, 20 * 1e-4)
    err = np.abs(pops[-1] - ref).max()
    assert err < 1e-5, err
    # renormalisation after every step keeps the total population from drifting:
    # each step's (pre-renormalisation) total is within one step's FP32 error of 1
    assert np.abs(pops[:, :, -1] - 1.0).max() < 1e-6


def test_cheb_rejects_bad_config(elhl, flake):
    with pytest.raises(elhl.ElhlError) as e:
        elhl.Trajectory(flake, method=elhl.METHOD_CHEBYSHEV, ncols=3)
    assert e.value.status == elhl.ERR_UNSUPPORTED


@pytest.mark.parametrize("ncols", [32, 64])
def test_bf16x3_tensor_gemm_column_blocks(elhl, ncols):
    """The tcgen05 GEMM with 2m = 64 and 128 (N = 2170, partial 128-row tile at the
    end, K split): populations within 1e-6 of FP64 over 3 steps."""
    sysm = systems.cubic_cluster(n_atoms=700, seed=9)
    states = list(range(1, ncols + 1))
    out = {}
    for prec in (elhl.PREC_FP64, elhl.PREC_BF16X3):
        tr = elhl.Trajectory(sysm, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=ncols,
                             nparticles=ncols, cheb_tol=1e-12)
        tr.init_fmo_states(states)
        out[prec] = tr.step(None, nsteps=3)
        tr.close()
    err = np.abs(out[elhl.PREC_BF16X3] - out[elhl.PREC_FP64])
    assert err[:, :, :-1].max() < 1e-6
    assert err[:, :, -1].max() < 2e-6


@pytest.mark.parametrize("prec_name", ["fp32", "bf16x3"])
def test_gemm_regime_matches_fp64(elhl, oracle_mod, prec_name):
    """N = 2170 with 16 ket columns: H~.Psi runs as one cuBLAS GEMM per order
    (CUDA graph per step).  Fragment populations within 1e-6 of the FP64 path
    and of the exact propagator over 4 steps.  The per-step total (before the
    next step's renormalisation) is held to 2e-6: cuBLAS sums each output over
    N = 2170 terms in one FP32 chain (measured 1.3e-6 at 8 columns; the row
    kernel's tree sums give 2.7e-7)."""
    prec32 = {"fp32": elhl.PREC_FP32, "bf16x3": elhl.PREC_BF16X3}[prec_name]
    tol = 1e-6
    sysm = systems.cubic_cluster(n_atoms=700, seed=9)
    assert sysm.nao >= 2048
    states = list(range(22, 54, 2))
    out = {}
    for prec in (elhl.PREC_FP64, prec32):
        tr = elhl.Trajectory(sysm, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=16,
                             nparticles=16, cheb_tol=1e-14)
        tr.init_fmo_states(states)
        out[prec] = tr.step(None, nsteps=4)
        if prec == prec32:
            assert tr.stats().tile_cols == 0  # GEMM regime
        tr.close()
    err = np.abs(out[prec32] - out[elhl.PREC_FP64])
    assert err[:, :, :-1].max() < tol
    assert err[:, :, -1].max() < 2 * tol
    S = oracle_mod.overlap(sysm)
    h = oracle_mod.huckel(sysm, S)
    ex = oracle_mod.ExactPropagator(S, h)
    for c, st in enumerate(states[:3]):
        ket0, _ = oracle_mod.fragment_mo(sysm, "E", st)
        ref = oracle_mod.exact_populations(sysm, S, ex.ket(ket0.astype(complex), 4e-4))
        assert np.abs(out[elhl.PREC_FP64][-1, c] - ref).max() < 1e-10
        assert np.abs(out[prec32][-1, c, :-1] - ref[:-1]).max() < tol


def test_df64_fixed_nuclei_vs_exact(elhl, oracle_mod, flake):
    """DF64 (FP32 pairs on the FP32 pipes, implicit operator) on the flake: 20 steps
    against the exact propagator at the FP64 bar, 1e-10."""
    S = oracle_mod.overlap(flake)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    pops, b, k, st = _cheb(elhl, flake, 20, elhl.PREC_DF64, 2)
    ref = _exact(oracle_mod, flake, ket, 20 * 1e-4)
    assert np.abs(pops[-1] - ref).max() < 1e-10
    assert st.phases == 3


def test_df64_moving_nuclei_vs_taylor_oracle(elhl, oracle_mod):
    """DF64 with moving nuclei, bra and ket carried (ncols = 4): the reference's
    Taylor step driver at tolerance 1e-12, populations to 1e-9."""
    sysm = systems.cubic_cluster(n_atoms=64, seed=7)
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=3) for i in range(4)])
    S0 = oracle_mod.overlap(sysm, coords[1])
    bra, ket = oracle_mod.initial_states(sysm, S0, 41, 40)
    ref = oracle_mod.ReferenceStep(sysm, bra, ket, dt=5e-4, tol=1e-12, norm_tol=1e-12, nthreads=4)
    rp = np.stack([ref.step(coords[1 + i]).T for i in range(3)])
    tr = elhl.Trajectory(sysm, coords=coords[1], dt=5e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_DF64,
                         ncols=4, cheb_tol=1e-14)
    tr.set_psi(bra, ket)
    pops = tr.step(coords[1:], nsteps=3)
    tr.close()
    assert np.abs(pops - rp).max() < 1e-9


def test_df64_cluster_vs_exact(elhl, oracle_mod):
    """DF64 at N = 1860 (two row chunks per CTA) against the exact propagator, 1e-9."""
    sysm = systems.cubic_cluster(n_atoms=600, seed=11)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    tr = elhl.Trajectory(sysm, coords=sysm.coords, dt=2e-4, method=elhl.METHOD_CHEBYSHEV,
                         precision=elhl.PREC_DF64, ncols=4, cheb_tol=1e-14)
    tr.init_fmo(homo + 1, homo)
    pops = tr.step(np.stack([sysm.coords] * 2), nsteps=2)
    tr.close()
    ket0, _ = oracle_mod.fragment_mo(sysm, "E", homo + 1)
    ref = _exact(oracle_mod, sysm, np.column_stack([ket0, oracle_mod.fragment_mo(sysm, "H", homo)[0]]).astype(complex),
                 4e-4)
    assert np.abs(pops[-1] - ref).max() < 1e-9


@pytest.mark.parametrize("n_atoms,nao", [(20, 62), (64, 199), (150, 465), (600, 1860)])
@pytest.mark.parametrize("prec_name,tol", [("fp64", 1e-12), ("df64", 1e-12), ("fp32", 1e-12), ("oz64", 1e-12)])
def test_rebuild_factor_and_inverse(elhl, prec_name, tol, n_atoms, nao):
    """The moving-nuclei rebuild's factorisations: FP64 the recursive
    Cholesky-with-inverse on the FP64 pipe, OZ64 the same recursion with its
    products of 320 or more rows on the tensor cores (exact slices), and DF64 and
    FP32 the same FP64 recursion as OZ64.
    N = 62 is one leaf; 199 and 465 keep every product below the 320-row cut
    (FP64 pipe); 1860 slices its top-level products and has a short last
    64-row leaf.
    L L^T = S, G L = I, L against numpy's Cholesky of the same S, both factors
    lower triangular."""
    prec = {"fp64": elhl.PREC_FP64, "df64": elhl.PREC_DF64, "fp32": elhl.PREC_FP32, "oz64": elhl.PREC_OZ64}[prec_name]
    sysm = systems.cubic_cluster(n_atoms=n_atoms, seed=11)
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=5) for i in range(2)])
    tr = elhl.Trajectory(sysm, coords=coords[0], dt=2e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=4,
                         cheb_tol=1e-12)
    rng = np.random.default_rng(n_atoms)
    psi = rng.standard_normal((nao, 2)) + 1j * rng.standard_normal((nao, 2))
    psi /= np.linalg.norm(psi, axis=0)
    tr.set_psi(psi, psi)  # any state: only the factors are checked
    tr.step(coords[1:], nsteps=1)
    S, _, _ = tr.matrices()
    L, G = tr.factor()
    tr.close()
    assert S.shape == (nao, nao)
    assert np.abs(np.triu(L, 1)).max() == 0.0 and np.abs(np.triu(G, 1)).max() == 0.0
    assert np.abs(L @ L.T - S).max() < tol
    assert np.abs(G @ L - np.eye(S.shape[0])).max() < 10 * tol
    assert np.abs(L - np.linalg.cholesky(S)).max() < 10 * tol


def test_kernel_launch_counter(elhl, flake):
    """The library counts its own kernel launches (bench.py's gpu_launches)."""
    n0 = elhl.kernel_launches()
    tr = elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64, ncols=2)
    tr.init_fmo(41, 40)
    n1 = elhl.kernel_launches()
    tr.step(None, nsteps=3)
    n2 = elhl.kernel_launches()
    tr.close()
    assert n1 > n0 and n2 > n1


@pytest.mark.parametrize("prec_name,moving", [("fp64", False), ("fp64", True), ("oz64", True), ("fp32", True),
                                              ("fp32", False)])
def test_spectral_interval_encloses_the_spectrum(elhl, prec_name, moving):
    """The FP64 Lanczos bounds (one cooperative launch, lanczos.cu) of the explicit
    H~ (fixed nuclei; OZ64 moving nuclei) and of the implicit G h G^T (moving
    nuclei): [emin, emax] holds every generalised eigenvalue of (h, S) of the
    current geometry and is no wider than the 1 % guards plus 3 % of the width."""
    import scipy.linalg
    prec = {"fp64": elhl.PREC_FP64, "fp32": elhl.PREC_FP32, "oz64": elhl.PREC_OZ64}[prec_name]
    sysm = systems.cubic_cluster(n_atoms=150, seed=3)
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=2) for i in range(3)])
    tr = elhl.Trajectory(sysm, coords=coords[0] if moving else None, dt=2e-4, method=elhl.METHOD_CHEBYSHEV,
                         precision=prec, ncols=4 if moving else 2, cheb_tol=1e-12)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    tr.init_fmo(homo + 1, homo)
    tr.step(coords[1:] if moving else None, nsteps=2)
    st = tr.stats()
    S, h, _ = tr.matrices()
    tr.close()
    lam = scipy.linalg.eigh(h, S, eigvals_only=True)
    width = lam[-1] - lam[0]
    assert st.emin <= lam[0] and st.emax >= lam[-1]
    assert st.emin >= lam[0] - 0.04 * width and st.emax <= lam[-1] + 0.04 * width


def test_fp32_diagonal_correction_mix_member(elhl):
    """A member of the trajectory mix (95-atom cluster, N = 296) over 200 fixed-nuclei
    steps of 0.1 fs: FP32 Hs with the rounding residual of its diagonal added back in
    the row kernel stays within 1e-6 of FP64 in every fragment population at every
    step (the served mix measured 4.9e-7 at the end for this member, 1.19e-6 without
    the correction).  Rounding the whole Hs to FP32 moves it by 9.6e-7 even with
    exact propagators (numpy replay): the diagonal, the largest entries, carries
    most of that."""
    sysm = systems.cubic_cluster(n_atoms=95, seed=5)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    out = {}
    for prec in (elhl.PREC_FP64, elhl.PREC_FP32):
        tr = elhl.Trajectory(sysm, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=2, cheb_tol=1e-12)
        tr.init_fmo(homo + 1, homo)
        out[prec] = tr.step(None, nsteps=200)
        tr.close()
    assert np.abs(out[elhl.PREC_FP32] - out[elhl.PREC_FP64]).max() < 1e-6
