"""The oracle: CPU restatement of Dynemol's ElHl_Chebyshev propagation path.

TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py import this module as the checker; the product library
(dynemol_gb300, libelhlprop.so) never does.

What lives where:
* oracle/elhl_oracle.c (compiled to oracle/liborc.so by `build()`):
  STO overlap S (SOLAP/ROTAR), Hueckel h, the Taylor propagator, populations.
* here, with scipy's LAPACK:
  - S^-1 by Bunch-Kaufman dsytrf + dsytri then symmetrised (cpu_syInvert,
    GPU_Interface.cpp:936-947; Matrix_Symmetrize, Matrix_math.f:126-177);
  - H' = S^-1 h by dsymm (syMultiply, Matrix_math.f:79-121);
  - initial states: fragment generalized eigenproblem by dsygvd, MO embedded in
    the full basis (eigen_FMO / projector('AO'), FMO.f:260-350) with
    Psi_ket = C, Psi_bra = S C (ElHl_Chebyshev.f:119-129);
  - the per-nuclear-step driver (ElHl_Chebyshev, ElHl_Chebyshev.f:148-291);
  - the exact fixed-nuclei propagator psi(t) = U exp(-iEt/hbar) U^T S psi(0)
    from dsygvd (Simple_dynamics, ElHl_schroedinger.f:131-147; qdynamics.f:104-182),
    an independent pin of the Taylor restatement.

Parity: the reference ships no tests or golden vectors, so this oracle is pinned
by the exact propagator, closed-form STO overlaps and conservation laws
(tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
H_BAR = 6.58264e-4  # eV ps, constants_m.f:23

_lib = None


def build(force: bool = False) -> str:
    """Compile the C restatement (plain gcc, OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "elhl_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
               "-Wall", "-o", LIB_PATH, src, "-lm"]
        subprocess.check_call(cmd)
    return LIB_PATH


class _Basis(ctypes.Structure):
    _fields_ = [("nao", ctypes.c_int), ("natoms", ctypes.c_int),
                ("atom_ao0", ctypes.c_void_p), ("atom_nao", ctypes.c_void_p),
                ("coord", ctypes.c_void_p), ("ao_n", ctypes.c_void_p), ("ao_l", ctypes.c_void_p),
                ("ao_m", ctypes.c_void_p), ("ao_nzeta", ctypes.c_void_p), ("ao_zeta", ctypes.c_void_p),
                ("ao_coef", ctypes.c_void_p), ("ao_ip", ctypes.c_void_p), ("ao_kwh", ctypes.c_void_p),
                ("ao_vshift", ctypes.c_void_p)]


class PropStats(ctypes.Structure):
    _fields_ = [("gemv_terms", ctypes.c_longlong), ("conv_calls", ctypes.c_int),
                ("substeps", ctypes.c_int), ("status", ctypes.c_int)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.orc_solap.argtypes = [ci, ci, cd, ci, ci, cd, cd, vp]
        L.orc_overlap.argtypes = [ctypes.POINTER(_Basis), cd, vp, ci]
        L.orc_huckel.argtypes = [ctypes.POINTER(_Basis), vp, vp]
        L.orc_huckel.restype = None
        L.orc_propagation.argtypes = [ci, vp, vp, vp, cd, cd, vp, vp, cd, cd, ci, ci, ctypes.POINTER(PropStats)]
        L.orc_dzgemv.argtypes = [ci, ci, vp, vp, vp, vp, ci]
        L.orc_dzgemv.restype = None
        L.orc_populations.argtypes = [ci, vp, ci, vp, vp, vp]
        L.orc_populations.restype = None
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _basis_struct(sys, coords=None):
    coords = np.ascontiguousarray(sys.coords if coords is None else coords, np.float64)
    keep = [coords, sys.atom_ao0, sys.atom_nao, sys.ao_n, sys.ao_l, sys.ao_m, sys.ao_nzeta,
            sys.ao_zeta, sys.ao_coef, sys.ao_ip, sys.ao_kwh, sys.ao_vshift]
    b = _Basis(sys.nao, sys.natoms, _p(sys.atom_ao0), _p(sys.atom_nao), _p(coords), _p(sys.ao_n),
               _p(sys.ao_l), _p(sys.ao_m), _p(sys.ao_nzeta), _p(sys.ao_zeta), _p(sys.ao_coef),
               _p(sys.ao_ip), _p(sys.ao_kwh), _p(sys.ao_vshift))
    return b, keep


# ------------------------------------------------------------------ matrices
def solap(na, la, za, nb, lb, zb, R):
    out = np.zeros(6)
    rc = lib().orc_solap(na, la, za, nb, lb, zb, R, _p(out))
    if rc:
        raise ValueError("solap: unsupported quantum numbers")
    return out[: min(la, lb) + 1]


def overlap(sys, coords=None, cutoff=12.0, nthreads=0) -> np.ndarray:
    """S (N x N, column-major storage == numpy Fortran order)."""
    b, keep = _basis_struct(sys, coords)
    S = np.zeros((sys.nao, sys.nao), order="F")
    if lib().orc_overlap(ctypes.byref(b), cutoff, _p(S), nthreads):
        raise ValueError("overlap: unsupported basis")
    return S


def huckel(sys, S) -> np.ndarray:
    b, keep = _basis_struct(sys)
    S = np.asfortranarray(S)
    h = np.zeros_like(S, order="F")
    lib().orc_huckel(ctypes.byref(b), _p(S), _p(h))
    return h


def sy_invert(S) -> np.ndarray:
    """S^-1 via dsytrf + dsytri ('U') then copy upper to lower."""
    from scipy.linalg import lapack
    a = np.array(S, order="F", dtype=np.float64, copy=True)
    lu, ipiv, info = lapack.dsytrf(a, lower=0)
    if info != 0:
        raise np.linalg.LinAlgError(f"dsytrf info={info}")
    inv, info = lapack.dsytri(lu, ipiv, lower=0)
    if info != 0:
        raise np.linalg.LinAlgError(f"dsytri info={info}")
    iu = np.triu_indices(inv.shape[0], 1)
    inv[(iu[1], iu[0])] = inv[iu]
    return np.asfortranarray(inv)


def h_prime(S_inv, h) -> np.ndarray:
    """H' = S^-1 h via dsymm (left, upper)."""
    from scipy.linalg import blas
    return np.asfortranarray(blas.dsymm(1.0, S_inv, h, side=0, lower=0))


# ------------------------------------------------------------------ initial state
def fragment_mo(sys, which: str, orbital: int):
    """Embedded fragment MO C (length N, zeros outside the fragment), C^T S_f C = 1.

    orbital is 1-based (the reference's electron_state / hole_state)."""
    from scipy.linalg import eigh
    atoms = sys.fragment_atoms(which)
    sub = _subsystem(sys, atoms)
    Sf = overlap(sub)
    hf = huckel(sub, Sf)
    e, Q = eigh(hf, Sf, driver="gvd")
    c = Q[:, orbital - 1]
    # eigenvector sign is arbitrary in LAPACK; fix it (largest |component| positive)
    if c[np.argmax(np.abs(c))] < 0:
        c = -c
    full = np.zeros(sys.nao)
    aos = np.concatenate([np.arange(sys.atom_ao0[a], sys.atom_ao0[a] + sys.atom_nao[a]) for a in atoms])
    full[aos] = c
    return full, e


def _subsystem(sys, atoms):
    from dynemol_gb300.systems import EHTSystem
    sub = EHTSystem([sys.symbols[i] for i in atoms], sys.coords[atoms].copy(), sys.fragment[atoms].copy(),
                    sys.el_atoms[atoms].copy(), sys.hl_atoms[atoms].copy())
    return sub.build_basis()


def initial_states(sys, S, electron_state: int, hole_state: int):
    """Psi_bra (N,2), Psi_ket (N,2) complex: column 0 electron, 1 hole."""
    ce, _ = fragment_mo(sys, "E", electron_state)
    ch, _ = fragment_mo(sys, "H", hole_state)
    C = np.column_stack([ce, ch])
    psi_ket = C.astype(np.complex128)
    psi_bra = (S.T @ C).astype(np.complex128)  # bra_x_op(Psi_bra, AO_bra, S) = S^T C
    return np.asfortranarray(psi_bra), np.asfortranarray(psi_ket)


# ------------------------------------------------------------------ propagation
def propagate(Hp, bra, ket, t_init, t_max, tau, tol=1e-8, norm_tol=1e-8, max_conv_calls=100000, nthreads=0):
    """Taylor Propagation of one particle. Returns (bra, ket, tau_after, save_tau, stats)."""
    Hp = np.asfortranarray(Hp, dtype=np.float64)
    N = Hp.shape[0]
    b = np.ascontiguousarray(bra, dtype=np.complex128).copy()
    k = np.ascontiguousarray(ket, dtype=np.complex128).copy()
    t = np.array([tau], np.float64)
    st = np.array([0.0])
    stats = PropStats()
    rc = lib().orc_propagation(N, _p(Hp), _p(b), _p(k), float(t_init), float(t_max), _p(t), _p(st),
                               tol, norm_tol, max_conv_calls, nthreads, ctypes.byref(stats))
    if rc < 0:
        raise MemoryError("orc_propagation")
    return b, k, float(t[0]), float(st[0]), stats


def populations(sys, psi_bra, psi_ket) -> np.ndarray:
    """(nfrag+1) populations of one particle (pop_Slater over fragments + total)."""
    pop = np.zeros(sys.nfrag + 1)
    lib().orc_populations(sys.nao, _p(sys.ao_frag), sys.nfrag,
                          _p(np.ascontiguousarray(psi_bra, np.complex128)),
                          _p(np.ascontiguousarray(psi_ket, np.complex128)), _p(pop))
    return pop


class ReferenceStep:
    """Per-nuclear-step driver restating ElHl_Chebyshev (ElHl_Chebyshev.f:148-291).

    Holds Psi_bra/Psi_ket (N,2), save_tau(2) and first_call_.  The electron and
    the hole are propagated concurrently on two halves of the host threads,
    mirroring the reference's two MPI ranks.  `hole_tau_quirk` reproduces the
    CPU path's hole rank that never clears first_call_ (it always restarts at
    tau_max, ElHl_Chebyshev.f:237 vs :287)."""

    def __init__(self, sys, psi_bra, psi_ket, dt, frame_step=1, tol=1e-8, norm_tol=1e-8,
                 nthreads=0, hole_tau_quirk=False, cutoff=12.0):
        self.sys = sys
        self.bra = np.array(psi_bra, dtype=np.complex128, order="F")
        self.ket = np.array(psi_ket, dtype=np.complex128, order="F")
        self.dt = dt
        self.frame_step = frame_step
        self.tol, self.norm_tol = tol, norm_tol
        self.nthreads = nthreads if nthreads > 0 else (os.cpu_count() or 1)
        self.first = True
        self.save_tau = np.zeros(2)
        self.hole_quirk = hole_tau_quirk
        self.cutoff = cutoff
        self.t = 0.0
        self.it = 1
        self.last_coords = None
        self.S = self.h = self.S_inv = self.Hp = None
        self.stats = [None, None]

    def rebuild(self, coords):
        self.S = overlap(self.sys, coords, self.cutoff, self.nthreads)
        self.h = huckel(self.sys, self.S)
        self.S_inv = sy_invert(self.S)
        self.Hp = h_prime(self.S_inv, self.h)

    def step(self, coords=None):
        """One nuclear step; coords None keeps the nuclei fixed (S, h, H' rebuilt
        all the same, as the reference does)."""
        coords = self.sys.coords if coords is None else coords
        self.it += 1
        t_init = self.t
        t_max = self.dt * self.frame_step * (self.it - 1)
        tau_max = self.dt / H_BAR
        taus = []
        for p in range(2):
            first = self.first or (p == 1 and self.hole_quirk)
            tau = tau_max if first else self.save_tau[p] * 1.15
            taus.append(tau_max if tau > tau_max else tau)
        self.rebuild(coords)
        out = [None, None]
        half = max(1, self.nthreads // 2)

        def run(p):
            out[p] = propagate(self.Hp, self.bra[:, p], self.ket[:, p], t_init, t_max, taus[p],
                               self.tol, self.norm_tol, nthreads=half)

        th = [threading.Thread(target=run, args=(p,)) for p in range(2)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        for p in range(2):
            b, k, _, st, stats = out[p]
            if stats.status:
                raise RuntimeError("oracle propagation did not converge")
            self.bra[:, p] = b
            self.ket[:, p] = k
            self.save_tau[p] = st
            self.stats[p] = stats
        self.t = t_init + self.dt * self.frame_step
        self.first = False
        return self.populations()

    def populations(self):
        return np.stack([populations(self.sys, self.bra[:, p], self.ket[:, p]) for p in range(2)], 1)

    def ao_bra(self):
        """AO_bra = conj(S^-1 Psi_bra) (ElHl_Chebyshev.f:274-275)."""
        return np.conj(self.S_inv @ self.bra)

    def energies(self):
        """sum_ij AO_bra_i h_ij AO_ket_j per particle (QuasiParticleEnergies,
        ElHl_Chebyshev.f:329-371, evaluated with the Hueckel h)."""
        ab = self.ao_bra()
        return np.array([ab[:, p] @ (self.h @ self.ket[:, p]) for p in range(2)])


# ------------------------------------------------------------------ exact pin
class ExactPropagator:
    """Fixed-nuclei exact propagation in the generalized eigenbasis (dsygvd):
    psi(t) = U exp(-i E t / hbar) U^T S psi(0), U^T S U = 1."""

    def __init__(self, S, h):
        from scipy.linalg import eigh
        self.E, self.U = eigh(h, S, driver="gvd")
        self.S = S

    def ket(self, psi0, t):
        c = self.U.T @ (self.S @ psi0)
        return self.U @ (np.exp(-1j * self.E * t / H_BAR)[:, None] * c if c.ndim == 2 else
                         np.exp(-1j * self.E * t / H_BAR) * c)


def exact_populations(sys, S, psi_ket_t):
    """Populations from a ket alone, with bra = S ket."""
    bra = S @ psi_ket_t
    if psi_ket_t.ndim == 1:
        return populations(sys, bra, psi_ket_t)
    return np.stack([populations(sys, bra[:, p], psi_ket_t[:, p]) for p in range(psi_ket_t.shape[1])], 1)


# ------------------------------------------------------------------ Ehrenfest pieces
def ehrenfest_kernel(H, X, A=None, bra=None, ket=None):
    """K = X o A - H A (hadamard_minus after the DGEMM, Taylor_gpu.cpp:776-781); with
    bra/ket (N x 2): A = (rho + rho^T)/2, rho_ij = Re(ket_j1 bra_i1) - Re(ket_j2 bra_i2)
    (calculate_rho_kernel / calculate_A, Chebyshev_gpu_kernels.cu:394-455)."""
    if A is None:
        rho = np.real(np.outer(bra[:, 0], ket[:, 0])) - np.real(np.outer(bra[:, 1], ket[:, 1]))
        A = 0.5 * (rho + rho.T)
    return X * A - H @ A


def pulay_forces(sys, kernel, coords=None, delta=1e-8, cutoff=12.0):
    """Ehrenfest (Hellmann-Feynman-Pulay) forces, natoms x 3 in N (Ehrenfest and
    Diabatic_Ehrenfest, diabatic-Ehren.f:163-230 and :100-150): per atom K and
    direction, S rebuilt with K displaced by +-delta (PULAY_OVERLAP,
    overlap_D.f:314-463, here the whole S), grad_S = (S_fwd - S_bck) / (2 delta)
    over the columns of K, F_K(L) = -sum_{j in L, i in K} grad_S(j, i) kernel(i, j)
    for the atoms L > K closer than the cutoff (preprocess, :316-324), and
    force(a) = 2 e2N (sum_{L > a} F_a(L) - sum_{K < a} F_K(a))."""
    X = np.array(sys.coords if coords is None else coords, np.float64)
    nat = sys.natoms
    F = np.zeros((nat, nat, 3))
    aos = [np.arange(sys.atom_ao0[a], sys.atom_ao0[a] + sys.atom_nao[a]) for a in range(nat)]
    for K in range(nat):
        for xyz in range(3):
            Xf = X.copy(); Xf[K, xyz] += delta
            Xb = X.copy(); Xb[K, xyz] -= delta
            Sf = overlap(sys, Xf, cutoff=cutoff)
            Sb = overlap(sys, Xb, cutoff=cutoff)
            for L in range(K + 1, nat):
                if not np.sqrt(((X[K] - X[L]) ** 2).sum()) < cutoff:
                    continue
                g = (Sf[np.ix_(aos[L], aos[K])] - Sb[np.ix_(aos[L], aos[K])]) / (2.0 * delta)
                F[K, L, xyz] = -(g * kernel[np.ix_(aos[K], aos[L])].T).sum()
    force = np.zeros((nat, 3))
    for a in range(nat):
        force[a] = F[a, a + 1:].sum(0) - F[:a, a].sum(0)
    return 2.0 * 1.602176565e-9 * force


def huckel_with_fields(sys, S, dp_ao, dp4, coords=None, cutoff=12.0):
    """Extended-Hueckel h with environment fields, the EnvField_ case of
    even_more_extended_Huckel / Huckel_with_FIELDS (hamiltonians.f:69-264):
    for AOs i of atom a > b and j of atom b within the cutoff,
    h_ij = X_ij S_ij - [S_ij DP_1 + (mu_ij - (r0 - R_a) S_ij) . DP_2..4] when |S_ij| > low_prec
    (1e-7, constants_m.f:26), h_ji = h_ij; h_ii = IP + V_shift."""
    X = np.array(sys.coords if coords is None else coords, np.float64)
    n = sys.nao
    h = np.zeros((n, n), order="F")
    for i in range(n):
        h[i, i] = sys.ao_ip[i] + sys.ao_vshift[i]
    for b in range(sys.natoms):
        for a in range(b + 1, sys.natoms):
            if np.sqrt(((X[b] - X[a]) ** 2).sum()) > cutoff:
                continue
            Ri = X[a]
            r0 = (X[a] + X[b]) / 2.0
            DP = dp4[a, b, :]
            for jb in range(sys.atom_nao[b]):
                j = sys.atom_ao0[b] + jb
                for ja in range(sys.atom_nao[a]):
                    i = sys.atom_ao0[a] + ja
                    s = S[i, j]
                    c1 = sys.ao_ip[i] - sys.ao_ip[j]
                    c2 = sys.ao_ip[i] + sys.ao_ip[j]
                    c3 = (c1 / c2) * (c1 / c2)
                    c4 = (sys.ao_vshift[i] + sys.ao_vshift[j]) * 0.5
                    k = (sys.ao_kwh[i] + sys.ao_kwh[j]) * 0.5
                    keff = k + c3 + c3 * c3 * (1.0 - k)
                    v = (keff * c2 * 0.5 + c4) * s
                    if abs(s) > 1e-7:
                        vec = dp_ao[i, j, :] - (r0 - Ri) * s
                        v = v - (s * DP[0] + (vec[0] * DP[1] + vec[1] * DP[2] + vec[2] * DP[3]))
                    h[i, j] = v
                    h[j, i] = v
    return h
