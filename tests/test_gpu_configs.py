"""GPU tests at the sizes of the precision and batching workloads, through
size-independent properties and independent paths:

* config 3 (C/H sheet, N = 8192, 64 complex columns): FP32 and BF16X3 (the
  tensor-core GEMM) against FP64 per step within 1e-6 in populations, FP64
  unitary to 1e-10 per step, and FP64 Chebyshev against the FP64 Taylor path
  (the drop-in's method, independent kernels) within 1e-10;
* config 4 (uneven C/H/O trajectories of N near 3,000): two members batched
  against their solo runs (1e-12) and against the exact generalized-eigenbasis
  propagator (ElHl_schroedinger.f:131-147) within 1e-10; FP32 batch within 1e-6
  of FP64."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sheet():
    s = systems.honeycomb_sheet(8192)
    assert s.nao == 8192
    return s


def test_config3_reduced_precision_vs_fp64(elhl, sheet):
    nf = int(sum(sheet.atom_nao[a] for a in sheet.fragment_atoms("E")))
    states = (systems.SplitMix64(3).permutation(nf)[:64] + 1).tolist()
    pops = {}
    for name, prec in (("fp64", elhl.PREC_FP64), ("fp32", elhl.PREC_FP32), ("bf16x3", elhl.PREC_BF16X3)):
        tr = elhl.Trajectory(sheet, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=64, nparticles=64,
                             cheb_tol=1e-12)
        tr.init_fmo_states(states)
        pops[name] = tr.step(None, nsteps=3)
        st = tr.stats()
        tr.close()
        if name == "fp64":
            assert st.norm_drift < 1e-10
        else:
            assert st.norm_drift < 1e-4
    for name in ("fp32", "bf16x3"):
        err = np.abs(pops[name] - pops["fp64"])
        assert err[:, :, :-1].max() < 1e-6, name  # fragment populations, every step
        assert err[:, :, -1].max() < 2e-6, name    # totals (renormalised to the target each step)


def test_config3_chebyshev_vs_taylor_fp64(elhl, sheet):
    homo = systems.fermi_state(sheet, sheet.fragment_atoms("E"))
    tr = elhl.Trajectory(sheet, dt=1e-4, tol=1e-12, norm_tol=1e-12)
    tr.init_fmo(homo + 1, homo)
    pt = tr.step(None, nsteps=1)
    tr.close()
    tr = elhl.Trajectory(sheet, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64, ncols=4,
                         cheb_tol=1e-14)
    tr.init_fmo(homo + 1, homo)
    pc = tr.step(None, nsteps=1)
    tr.close()
    assert np.abs(pc - pt).max() < 1e-10


def test_config4_members_batched_vs_solo_and_exact(elhl, oracle_mod):
    mix = [systems.cubic_cluster(n_atoms=968, seed=41), systems.cubic_cluster(n_atoms=940, seed=42)]
    assert all(2800 <= s.nao <= 3100 for s in mix)
    kw = dict(dt=1e-4, ncols=2, cheb_tol=1e-14)
    b = elhl.Batch(mix, precision=elhl.PREC_FP64, **kw)
    b.init_fmo()
    pb = b.step(5)
    b.close()
    b = elhl.Batch(mix, precision=elhl.PREC_FP32, **kw)
    b.init_fmo()
    p32 = b.step(5)
    b.close()
    assert np.abs(p32 - pb).max() < 1e-6
    for i, sysm in enumerate(mix):
        homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
        tr = elhl.Trajectory(sysm, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64, **kw)
        tr.init_fmo(homo + 1, homo)
        ps = tr.step(None, nsteps=5)
        tr.close()
        assert np.abs(pb[:, i] - ps).max() < 1e-12
        S = oracle_mod.overlap(sysm)
        h = oracle_mod.huckel(sysm, S)
        _, ket = oracle_mod.initial_states(sysm, S, homo + 1, homo)
        ex = oracle_mod.ExactPropagator(S, h)
        ref = oracle_mod.exact_populations(sysm, S, ex.ket(ket, 5e-4)).T
        assert np.abs(pb[-1, i] - ref).max() < 1e-10
