"""Generate the golden fixtures of tests/golden/ from the oracle.

The reference (Fortran + MKL + MPI + MAGMA) cannot be built or run here and
ships no golden vectors of its own, so these fixtures are the oracle's outputs
on the seeded workloads, committed so that

  * CPU tests pin the oracle against regressions (a change to the restatement
    that moves any of these numbers fails), and
  * GPU tests compare the CUDA path with oracle results at the workloads' full
    sizes without running the oracle on the GPU host (config 2 takes minutes
    of host time per step).

Each fixture states what produced it.  Run from the repository root:

    python tests/golden/make_golden.py [small] [flake] [cluster1200]

The oracle runs at Taylor tolerance 1e-12 (error and norm), well below the
1e-10 population bar of the tests; the exact fixed-nuclei propagator
(generalized eigenbasis, ElHl_schroedinger.f:131-147) gives the flake's long-time
populations.
"""
from __future__ import annotations

import dataclasses
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dynemol_gb300 import systems  # noqa: E402
from oracle import oracle  # noqa: E402

TOL = 1e-12


def small():
    """16-atom C/H/O cluster (seed 11): S, h, S^-1, H' at the initial geometry
    and per-step populations of 3 moving-nuclei steps (dt 0.5 fs)."""
    cl = systems.cubic_cluster(n_atoms=16, seed=11, frag_atoms=6)
    coords = np.stack([systems.perturbed_coords(cl.coords, i, seed=11) for i in range(4)])
    S = oracle.overlap(cl, coords[0])
    h = oracle.huckel(cl, S)
    Sinv = oracle.sy_invert(S)
    Hp = oracle.h_prime(Sinv, h)
    homo = systems.fermi_state(cl, np.arange(6))
    # fragment MOs at the initial geometry, as a trajectory created there computes them
    bra, ket = oracle.initial_states(dataclasses.replace(cl, coords=coords[0]), S, homo + 1, homo)
    ref = oracle.ReferenceStep(cl, bra, ket, dt=5e-4, tol=TOL, norm_tol=TOL, nthreads=2)
    pops = np.stack([ref.step(coords[1 + i]).T for i in range(3)])
    np.savez_compressed(os.path.join(HERE, "small16.npz"), coords=coords, S=S, h=h, Sinv=Sinv, Hp=Hp,
                        homo=homo, bra0=bra, ket0=ket, pops=pops, bra3=ref.bra, ket3=ref.ket,
                        save_tau=ref.save_tau, dt=5e-4, tol=TOL,
                        note="oracle: cubic_cluster(16, seed=11, frag_atoms=6), perturbed_coords seed 11, "
                             "fragment LUMO/HOMO, 3 moving-nuclei steps at dt 0.5 fs")


def flake():
    """Config 1: C100H50 flake, fragment = first 20 atoms, el = LUMO, hl = HOMO,
    fixed nuclei, dt 0.1 fs.  Taylor oracle populations after 5, 20 and 200
    steps; exact-propagator populations after 200 and 2000 steps."""
    fl = systems.honeycomb_flake()
    homo = systems.fermi_state(fl, np.arange(20))
    S = oracle.overlap(fl)
    h = oracle.huckel(fl, S)
    bra, ket = oracle.initial_states(fl, S, homo + 1, homo)
    ex = oracle.ExactPropagator(S, h)
    exact = {n: oracle.exact_populations(fl, S, ex.ket(ket, n * 1e-4)).T for n in (200, 2000)}
    ref = oracle.ReferenceStep(fl, bra, ket, dt=1e-4, tol=TOL, norm_tol=TOL)
    taylor = {}
    t0 = time.time()
    for i in range(1, 201):
        p = ref.step().T
        if i in (5, 20, 200):
            taylor[i] = p
            print(f"  flake step {i}: {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, "flake.npz"), homo=homo, eig=ex.E,
                        ket0_norm=np.linalg.norm(ket, axis=0),
                        taylor5=taylor[5], taylor20=taylor[20], taylor200=taylor[200],
                        exact200=exact[200], exact2000=exact[2000], dt=1e-4, tol=TOL,
                        note="oracle: honeycomb_flake(), fragment LUMO/HOMO of atoms 0-19, fixed nuclei, dt 0.1 fs; "
                             "taylorK = ReferenceStep populations after K steps [particle][fragment..., total]; "
                             "exactK = generalized-eigenbasis propagator at t = K dt")


def cluster1200():
    """Config 2: 1,200-atom C/H/O cluster (seed 2, N = 3720), moving nuclei
    (perturbed_coords seed 2, steps 0, 1, 2), dt 0.5 fs: populations after each
    of 2 steps from the geometry of step 0."""
    cl = systems.cubic_cluster(n_atoms=1200, seed=2)
    coords = np.stack([systems.perturbed_coords(cl.coords, i, sigma=0.02, seed=2) for i in range(3)])
    homo = systems.fermi_state(cl, np.arange(20))
    S0 = oracle.overlap(cl, coords[0])
    bra, ket = oracle.initial_states(dataclasses.replace(cl, coords=coords[0]), S0, homo + 1, homo)
    ref = oracle.ReferenceStep(cl, bra, ket, dt=5e-4, tol=TOL, norm_tol=TOL)
    pops = []
    t0 = time.time()
    for i in range(2):
        pops.append(ref.step(coords[1 + i]).T)
        print(f"  cluster1200 step {i + 1}: {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, "cluster1200.npz"), homo=homo, pops=np.stack(pops),
                        ket2_abs=np.abs(ref.ket), save_tau=ref.save_tau, dt=5e-4, tol=TOL,
                        note="oracle: cubic_cluster(1200, seed=2), N = 3720, initial geometry perturbed_coords(step 0), "
                             "steps at perturbed_coords(steps 1, 2), sigma 0.02 A, seed 2; fragment LUMO/HOMO of "
                             "atoms 0-19 at the step-0 geometry; populations [step][particle][fragment..., total]")


if __name__ == "__main__":
    oracle.build()
    which = sys.argv[1:] or ["small", "flake", "cluster1200"]
    for name in which:
        t = time.time()
        globals()[name]()
        print(f"{name}: {time.time() - t:.0f} s", flush=True)
