"""GPU path against the committed golden fixtures (tests/golden/), at the
workloads' full sizes: the config-1 flake over the config's 2,000 steps and the
config-2 cluster (N = 3720) with moving nuclei.  The fixtures hold the oracle's
outputs (Taylor restatement of Taylor.f at tolerance 1e-12, and the exact
generalized-eigenbasis propagator of ElHl_schroedinger.f:131-147), so these
tests compare the CUDA path with the oracle without running the oracle here.
Bar: populations within 1e-10 (FP64, DF64 and OZ64)."""
import os

import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


def test_small_matrices_vs_golden(elhl):
    """S, h and H' = S^-1 h built on the device (Taylor drop-in path)."""
    g = _load("small16.npz")
    cl = systems.cubic_cluster(n_atoms=16, seed=11, frag_atoms=6)
    tr = elhl.Trajectory(cl, coords=g["coords"][0], dt=5e-4)
    S, h, Hp = tr.matrices()
    tr.close()
    assert np.abs(S - g["S"]).max() < 1e-13
    assert np.abs(h - g["h"]).max() < 1e-11
    assert np.abs(Hp - g["Hp"]).max() < 1e-10 * np.abs(g["Hp"]).max()


@pytest.mark.parametrize("method,prec", [("taylor", "fp64"), ("cheb", "fp64"), ("cheb", "df64"), ("cheb", "oz64")])
def test_small_moving_nuclei_vs_golden(elhl, method, prec):
    g = _load("small16.npz")
    cl = systems.cubic_cluster(n_atoms=16, seed=11, frag_atoms=6)
    coords = g["coords"]
    homo = int(g["homo"])
    kw = dict(dt=float(g["dt"]), tol=1e-12, norm_tol=1e-12)
    if method == "cheb":
        kw.update(method=elhl.METHOD_CHEBYSHEV,
                  precision={"fp64": elhl.PREC_FP64, "df64": elhl.PREC_DF64, "oz64": elhl.PREC_OZ64}[prec],
                  ncols=4, cheb_tol=1e-14)
    tr = elhl.Trajectory(cl, coords=coords[0], **kw)
    tr.init_fmo(homo + 1, homo)
    pops = tr.step(coords[1:], nsteps=3)
    tr.close()
    assert np.abs(pops - g["pops"]).max() < 1e-10


def test_flake_taylor_200_steps_vs_golden(elhl, flake):
    """The drop-in's method (adaptive-tau Taylor) over 200 config-1 steps."""
    g = _load("flake.npz")
    homo = int(g["homo"])
    tr = elhl.Trajectory(flake, dt=1e-4, tol=1e-12, norm_tol=1e-12)
    tr.init_fmo(homo + 1, homo)
    pops = tr.step(None, nsteps=200)
    tr.close()
    assert np.abs(pops[4] - g["taylor5"]).max() < 1e-10
    assert np.abs(pops[19] - g["taylor20"]).max() < 1e-10
    assert np.abs(pops[199] - g["taylor200"]).max() < 1e-10


@pytest.mark.parametrize("prec", ["fp64", "df64", "oz64"])
def test_flake_chebyshev_2000_steps_vs_golden(elhl, flake, prec):
    """Config 1 in full: 2,000 fixed-nuclei steps at dt 0.1 fs against the exact
    propagator (and the Taylor oracle at step 200).  DF64 runs the implicit
    operator G (h/b) G^T, FP64 and OZ64 (products on the tensor cores) the
    explicit H~."""
    g = _load("flake.npz")
    homo = int(g["homo"])
    p = {"fp64": elhl.PREC_FP64, "df64": elhl.PREC_DF64, "oz64": elhl.PREC_OZ64}[prec]
    tr = elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=p, ncols=4, cheb_tol=1e-14)
    tr.init_fmo(homo + 1, homo)
    pops = tr.step(None, nsteps=2000)
    st = tr.stats()
    tr.close()
    assert np.abs(pops[199] - g["exact200"]).max() < 1e-10
    assert np.abs(pops[199] - g["taylor200"]).max() < 1e-10
    assert np.abs(pops[1999] - g["exact2000"]).max() < 1e-10
    assert st.norm_drift < 1e-10  # per-step unitarity held throughout


@pytest.mark.parametrize("prec", ["fp64", "df64", "oz64"])
def test_cluster1200_moving_nuclei_vs_golden(elhl, prec):
    """Config 2 at its size (1,200 atoms, N = 3720): two moving-nuclei steps
    (S, h, the factor and its inverse rebuilt each step) against the Taylor
    oracle's populations."""
    g = _load("cluster1200.npz")
    cl = systems.cubic_cluster(n_atoms=1200, seed=2)
    assert cl.nao == 3720
    coords = np.stack([systems.perturbed_coords(cl.coords, i, sigma=0.02, seed=2) for i in range(3)])
    homo = int(g["homo"])
    p = {"fp64": elhl.PREC_FP64, "df64": elhl.PREC_DF64, "oz64": elhl.PREC_OZ64}[prec]
    tr = elhl.Trajectory(cl, coords=coords[0], dt=float(g["dt"]), method=elhl.METHOD_CHEBYSHEV, precision=p,
                         ncols=4, cheb_tol=1e-14)
    tr.init_fmo(homo + 1, homo)
    pops = tr.step(coords[1:], nsteps=2)
    _, ket = tr.get_psi()
    tr.close()
    assert np.abs(pops - g["pops"]).max() < 1e-10
    assert np.abs(np.abs(ket) - g["ket2_abs"]).max() < 1e-8
