"""Python mirror of the C ABI of libelhlprop.so (include/elhl_prop.h).

Two layers, matching the library:

* the drop-in symbols with the reference's by-reference calling convention:
  ``propagationelhl_gpucaller`` (Taylor_gpu.cpp:634-736) and
  ``propagation_gpucaller`` (Taylor_gpu.cpp:295-330), plus ``gpu_init`` /
  ``gpu_finalize`` / ``gpu_pin`` / ``gpu_unpin`` (GPU_Interface.cpp:226-302);
* :class:`Trajectory`, the device-resident electron-hole trajectory whose
  ``step`` is one or more calls of ElHl_Chebyshev (ElHl_Chebyshev.f:148-291).

The library must be built (``dynemol_gb300.build.build()``); loading fails
loudly otherwise -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libelhlprop.so")

# status codes (elhl_prop.h)
OK, ERR_BAD_ARG, ERR_NO_CONVERGENCE, ERR_TIMEOUT, ERR_OOM, ERR_CUDA, ERR_NOT_PD, ERR_NO_DEVICE, ERR_UNSUPPORTED = range(9)
METHOD_TAYLOR_REF, METHOD_CHEBYSHEV = 0, 1
PREC_FP64, PREC_FP32, PREC_BF16X3, PREC_DF64, PREC_OZ64 = 0, 1, 2, 3, 4

EXPORTED_SYMBOLS = (
    "gpu_init_", "gpu_finalize_", "gpu_pin_", "gpu_unpin_", "propagation_gpucaller_", "ehrenfestkernel_gpu_",
    "ehrenfestkernel2_gpu_", "elhl_ehrenfest_forces", "elhl_huckel_with_fields",
    "propagationelhl_gpucaller_", "elhl_last_status", "elhl_status_string", "elhl_traj_config_default",
    "elhl_traj_create", "elhl_traj_destroy", "elhl_traj_init_fmo", "elhl_traj_init_fmo_states", "elhl_traj_set_psi", "elhl_traj_get_psi", "elhl_traj_step",
    "elhl_traj_step_device", "elhl_traj_energies", "elhl_traj_get_matrices", "elhl_traj_get_factor", "elhl_traj_get_stats", "elhl_traj_snapshot", "elhl_traj_restore", "elhl_device_count",
    "elhl_sm_count", "elhl_set_stream", "elhl_debug_barrier", "elhl_kernel_launches", "elhl_propagate_fixed_scratch", "elhl_bessel_j",
    "elhl_chebyshev_coefficients", "elhl_batch_create", "elhl_batch_size", "elhl_batch_member",
    "elhl_batch_compact", "elhl_batch_step", "elhl_batch_get_stats", "elhl_batch_destroy",
    "elhl_server_create", "elhl_server_submit", "elhl_server_step", "elhl_server_poll", "elhl_server_result",
    "elhl_server_destroy", "elhl_server_snapshot", "elhl_server_submit_restart",
)


class ElhlError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {status_string(status)} (status {status})")


class BasisDesc(ctypes.Structure):
    _fields_ = [("natoms", ctypes.c_int), ("nao", ctypes.c_int)] + [
        (n, ctypes.c_void_p) for n in ("atom_ao0", "atom_nao", "ao_n", "ao_l", "ao_m", "ao_nzeta", "ao_zeta",
                                       "ao_coef", "ao_ip", "ao_kwh", "ao_vshift", "ao_frag")] + [("nfrag", ctypes.c_int)]


class TrajConfig(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("precision", ctypes.c_int), ("dt", ctypes.c_double),
                ("frame_step", ctypes.c_int), ("tol", ctypes.c_double), ("norm_tol", ctypes.c_double),
                ("cheb_tol", ctypes.c_double), ("cutoff", ctypes.c_double), ("max_conv_calls", ctypes.c_int),
                ("ncols", ctypes.c_int), ("nparticles", ctypes.c_int), ("cheb_norm_tol", ctypes.c_double),
                ("cheb_max_retries", ctypes.c_int), ("lanczos_guard", ctypes.c_double)]


class TrajStats(ctypes.Structure):
    _fields_ = [("orders", ctypes.c_longlong), ("conv_calls", ctypes.c_longlong), ("substeps", ctypes.c_longlong),
                ("save_tau", ctypes.c_double * 2), ("t", ctypes.c_double), ("it", ctypes.c_int),
                ("status", ctypes.c_int), ("prop_ms", ctypes.c_double), ("rebuild_ms", ctypes.c_double),
                ("prop_launches", ctypes.c_int), ("rebuild_count", ctypes.c_int), ("tile_cols", ctypes.c_int),
                ("phases", ctypes.c_int), ("sh_ms", ctypes.c_double), ("factor_ms", ctypes.c_double),
                ("inverse_ms", ctypes.c_double), ("cheb_retries", ctypes.c_int), ("norm_drift", ctypes.c_double),
                ("emin", ctypes.c_double), ("emax", ctypes.c_double)]


class Request(ctypes.Structure):
    _fields_ = [("basis", ctypes.POINTER(BasisDesc)), ("coords", ctypes.c_void_p), ("nsteps", ctypes.c_int),
                ("nparticles", ctypes.c_int), ("n_frag_atoms", ctypes.c_int), ("frag_atoms", ctypes.c_void_p),
                ("states", ctypes.c_void_p)]


_lib = None


def load(path: str = LIB_PATH):
    """Load libelhlprop.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run dynemol_gb300.build.build() (no CPU fallback exists)")
    L = ctypes.CDLL(path)
    vp, ip, dp, ci = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_int
    L.gpu_init_.argtypes = [ip, ip]
    L.gpu_init_.restype = None
    L.gpu_finalize_.argtypes = []
    L.gpu_finalize_.restype = None
    L.gpu_pin_.argtypes = [vp, ip]
    L.gpu_pin_.restype = None
    L.gpu_unpin_.argtypes = [vp]
    L.gpu_unpin_.restype = None
    L.propagation_gpucaller_.argtypes = [ip, dp, dp, dp, dp, vp, vp, vp]
    L.propagation_gpucaller_.restype = None
    L.propagationelhl_gpucaller_.argtypes = [ip, vp, vp, vp, vp, vp, vp, vp, dp, dp, dp, dp]
    L.propagationelhl_gpucaller_.restype = None
    L.ehrenfestkernel_gpu_.argtypes = [ip, vp, vp, vp, vp]
    L.ehrenfestkernel_gpu_.restype = None
    L.ehrenfestkernel2_gpu_.argtypes = [ip, vp, vp, vp, vp, vp]
    L.ehrenfestkernel2_gpu_.restype = None
    L.elhl_ehrenfest_forces.argtypes = [ctypes.POINTER(BasisDesc), vp, vp, ctypes.c_double, ctypes.c_double, vp]
    L.elhl_ehrenfest_forces.restype = ci
    L.elhl_huckel_with_fields.argtypes = [ctypes.POINTER(BasisDesc), vp, vp, vp, vp, ctypes.c_double, vp]
    L.elhl_huckel_with_fields.restype = ci
    L.elhl_last_status.restype = ci
    L.elhl_status_string.argtypes = [ci]
    L.elhl_status_string.restype = ctypes.c_char_p
    L.elhl_traj_config_default.argtypes = [ctypes.POINTER(TrajConfig)]
    L.elhl_traj_config_default.restype = None
    L.elhl_traj_create.argtypes = [ctypes.POINTER(BasisDesc), vp, ctypes.POINTER(TrajConfig), ctypes.POINTER(vp)]
    L.elhl_traj_destroy.argtypes = [vp]
    L.elhl_traj_init_fmo.argtypes = [vp, ci, vp, ci, ci, vp, ci]
    L.elhl_traj_init_fmo_states.argtypes = [vp, ci, vp, ci, vp]
    L.elhl_traj_set_psi.argtypes = [vp, vp, vp]
    L.elhl_traj_get_psi.argtypes = [vp, vp, vp]
    L.elhl_traj_step.argtypes = [vp, vp, ci, vp]
    L.elhl_traj_step_device.argtypes = [vp, vp, ci, vp]
    L.elhl_traj_get_matrices.argtypes = [vp, vp, vp, vp]
    L.elhl_traj_get_factor.argtypes = [vp, vp, vp]
    L.elhl_traj_energies.argtypes = [vp, vp]
    L.elhl_traj_get_stats.argtypes = [vp, ctypes.POINTER(TrajStats)]
    L.elhl_traj_snapshot.argtypes = [vp, ctypes.c_char_p]
    L.elhl_traj_restore.argtypes = [vp, ctypes.c_char_p]
    L.elhl_device_count.restype = ci
    L.elhl_sm_count.restype = ci
    L.elhl_set_stream.argtypes = [vp]
    L.elhl_debug_barrier.argtypes = [ctypes.c_double, ci]
    L.elhl_kernel_launches.argtypes = []
    L.elhl_kernel_launches.restype = ctypes.c_longlong
    L.elhl_propagate_fixed_scratch.argtypes = [ci, vp, ci, vp, vp, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, dp, vp]
    L.elhl_bessel_j.argtypes = [ctypes.c_double, ci, vp]
    L.elhl_chebyshev_coefficients.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                              ci, vp, vp, ip]
    L.elhl_batch_create.argtypes = [ci, vp, vp, ctypes.POINTER(TrajConfig), ctypes.POINTER(vp)]
    L.elhl_batch_size.argtypes = [vp]
    L.elhl_batch_member.argtypes = [vp, ci]
    L.elhl_batch_member.restype = vp
    L.elhl_batch_compact.argtypes = [vp]
    L.elhl_batch_step.argtypes = [vp, ci, vp]
    L.elhl_batch_get_stats.argtypes = [vp, ctypes.POINTER(TrajStats)]
    L.elhl_batch_destroy.argtypes = [vp]
    L.elhl_server_create.argtypes = [ctypes.c_double, ctypes.POINTER(TrajConfig), ctypes.POINTER(vp)]
    L.elhl_server_submit.argtypes = [vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_longlong)]
    L.elhl_server_step.argtypes = [vp, ip, ip]
    L.elhl_server_poll.argtypes = [vp, vp, ci, ip]
    L.elhl_server_result.argtypes = [vp, ctypes.c_longlong, vp, vp, vp]
    L.elhl_server_snapshot.argtypes = [vp, ctypes.c_longlong, ctypes.c_char_p]
    L.elhl_server_submit_restart.argtypes = [vp, ctypes.POINTER(Request), ctypes.c_char_p,
                                             ctypes.POINTER(ctypes.c_longlong)]
    L.elhl_server_destroy.argtypes = [vp]
    for s in EXPORTED_SYMBOLS:
        getattr(L, s)
    _lib = L
    return L


def status_string(status: int) -> str:
    return load().elhl_status_string(int(status)).decode()


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _check(rc: int, where: str):
    if rc != OK:
        raise ElhlError(rc, where)


# ---------------------------------------------------------------- drop-in
def gpu_init(myid: int = 0, procs_per_dev: int = 1):
    L = load()
    L.gpu_init_(ctypes.byref(ctypes.c_int(myid)), ctypes.byref(ctypes.c_int(procs_per_dev)))
    _check(L.elhl_last_status(), "gpu_init_")


def gpu_finalize():
    load().gpu_finalize_()


def gpu_pin(arr: np.ndarray):
    L = load()
    L.gpu_pin_(_p(arr), ctypes.byref(ctypes.c_int(arr.nbytes)))
    _check(L.elhl_last_status(), "gpu_pin_")


def gpu_unpin(arr: np.ndarray):
    L = load()
    L.gpu_unpin_(_p(arr))
    _check(L.elhl_last_status(), "gpu_unpin_")


def propagationelhl_gpucaller(S, h, psi_bra, psi_ket, t_init, t_max, tau):
    """One particle, one nuclear step, reference semantics.

    Returns (H', AO_bra, psi_bra, psi_ket, save_tau); psi arrays are updated in place."""
    L = load()
    N = S.shape[0]
    S = np.asfortranarray(S, np.float64)
    h = np.asfortranarray(h, np.float64)
    Hp = np.zeros((N, N), order="F")
    ao_bra = np.zeros(N, np.complex128)
    ao_ket = np.zeros(N, np.complex128)
    assert psi_bra.dtype == np.complex128 and psi_bra.flags.c_contiguous
    assert psi_ket.dtype == np.complex128 and psi_ket.flags.c_contiguous
    tau_c, st = ctypes.c_double(tau), ctypes.c_double(0.0)
    L.propagationelhl_gpucaller_(ctypes.byref(ctypes.c_int(N)), _p(S), _p(h), _p(Hp), _p(ao_bra), _p(ao_ket),
                                 _p(psi_bra), _p(psi_ket), ctypes.byref(ctypes.c_double(t_init)),
                                 ctypes.byref(ctypes.c_double(t_max)), ctypes.byref(tau_c), ctypes.byref(st))
    _check(L.elhl_last_status(), "propagationelhl_gpucaller_")
    return Hp, ao_bra, psi_bra, psi_ket, st.value


def propagation_gpucaller(Hp, psi_bra, psi_ket, t_init, t_max, tau):
    L = load()
    N = Hp.shape[0]
    Hp = np.asfortranarray(Hp, np.float64)
    tau_c, st = ctypes.c_double(tau), ctypes.c_double(0.0)
    L.propagation_gpucaller_(ctypes.byref(ctypes.c_int(N)), ctypes.byref(tau_c), ctypes.byref(st),
                             ctypes.byref(ctypes.c_double(t_init)), ctypes.byref(ctypes.c_double(t_max)),
                             _p(psi_bra), _p(psi_ket), _p(Hp))
    _check(L.elhl_last_status(), "propagation_gpucaller_")
    return psi_bra, psi_ket, st.value


def ehrenfest_kernel(H, X, A=None, bra=None, ket=None) -> np.ndarray:
    """K = X o A - H A (ehrenfestkernel_gpu_), or with A from bra/ket (N x 2,
    ehrenfestkernel2_gpu_)."""
    L = load()
    N = H.shape[0]
    H = np.asfortranarray(H, np.float64)
    X = np.asfortranarray(X, np.float64)
    K = np.zeros((N, N), order="F")
    n = ctypes.byref(ctypes.c_int(N))
    if A is not None:
        A = np.asfortranarray(A, np.float64)
        L.ehrenfestkernel_gpu_(n, _p(H), _p(A), _p(X), _p(K))
    else:
        b = np.asfortranarray(bra, np.complex128)
        k = np.asfortranarray(ket, np.complex128)
        L.ehrenfestkernel2_gpu_(n, _p(b), _p(k), _p(H), _p(X), _p(K))
    _check(L.elhl_last_status(), "ehrenfestkernel_gpu_")
    return K


def ehrenfest_forces(system, kernel, coords=None, delta: float = 1e-8, cutoff: float = 12.0) -> np.ndarray:
    """Ehrenfest (Hellmann-Feynman-Pulay) forces, natoms x 3, in N (elhl_ehrenfest_forces)."""
    L = load()
    desc, keep = _basis_desc(system)
    c = np.ascontiguousarray(system.coords if coords is None else coords, np.float64)
    K = np.asfortranarray(kernel, np.float64)
    out = np.zeros((system.natoms, 3))
    _check(L.elhl_ehrenfest_forces(ctypes.byref(desc), _p(c), _p(K), delta, cutoff, _p(out)), "elhl_ehrenfest_forces")
    return out


def huckel_with_fields(system, S, dp_ao, dp4, coords=None, cutoff: float = 12.0) -> np.ndarray:
    """h with environment fields (elhl_huckel_with_fields); dp_ao N x N x 3, dp4 natoms x natoms x 4."""
    L = load()
    desc, keep = _basis_desc(system)
    c = np.ascontiguousarray(system.coords if coords is None else coords, np.float64)
    S = np.asfortranarray(S, np.float64)
    dp = np.asfortranarray(dp_ao, np.float64)
    d4 = np.asfortranarray(dp4, np.float64)
    h = np.zeros((system.nao, system.nao), order="F")
    _check(L.elhl_huckel_with_fields(ctypes.byref(desc), _p(c), _p(S), _p(dp), _p(d4), cutoff, _p(h)),
           "elhl_huckel_with_fields")
    return h


# ---------------------------------------------------------------- trajectories
def default_config(**kw) -> TrajConfig:
    c = TrajConfig()
    load().elhl_traj_config_default(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _basis_desc(system):
    keep = [system.atom_ao0, system.atom_nao, system.ao_n, system.ao_l, system.ao_m, system.ao_nzeta,
            system.ao_zeta, system.ao_coef, system.ao_ip, system.ao_kwh, system.ao_vshift, system.ao_frag]
    return BasisDesc(system.natoms, system.nao, *[_p(a) for a in keep], system.nfrag), keep


class Trajectory:
    """Device-resident electron-hole trajectory (S, h, H', Psi live in HBM)."""

    @classmethod
    def borrowed(cls, system, handle):
        """Wrap a handle owned elsewhere (a batch member); close() does not free it."""
        self = cls.__new__(cls)
        self.sys, self.handle, self.N, self.P, self._owned = system, handle, system.nao, 2, False
        return self

    def __init__(self, system, coords=None, config: TrajConfig | None = None, **cfg_kw):
        self._owned = True
        L = load()
        self.sys = system
        self._keep = [system.atom_ao0, system.atom_nao, system.ao_n, system.ao_l, system.ao_m, system.ao_nzeta,
                      system.ao_zeta, system.ao_coef, system.ao_ip, system.ao_kwh, system.ao_vshift, system.ao_frag]
        self.desc = BasisDesc(system.natoms, system.nao, *[_p(a) for a in self._keep], system.nfrag)
        self.config = config if config is not None else default_config(**cfg_kw)
        c = np.ascontiguousarray(system.coords if coords is None else coords, np.float64)
        h = ctypes.c_void_p()
        _check(L.elhl_traj_create(ctypes.byref(self.desc), _p(c), ctypes.byref(self.config), ctypes.byref(h)),
               "elhl_traj_create")
        self.handle = h
        self.N = system.nao
        self.P = int(self.config.nparticles)

    def close(self):
        if getattr(self, "handle", None) and getattr(self, "_owned", True):
            load().elhl_traj_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_fmo(self, electron_state: int, hole_state: int):
        """Initial electron / hole states from the El / Hl fragment MOs (1-based)."""
        el = np.ascontiguousarray(self.sys.fragment_atoms("E"), np.int32)
        hl = np.ascontiguousarray(self.sys.fragment_atoms("H"), np.int32)
        _check(load().elhl_traj_init_fmo(self.handle, len(el), _p(el), electron_state, len(hl), _p(hl), hole_state),
               "elhl_traj_init_fmo")

    def init_fmo_states(self, states, which: str = "E"):
        """Chebyshev ensembles: column c = fragment MO states[c] (1-based)."""
        at = np.ascontiguousarray(self.sys.fragment_atoms(which), np.int32)
        st = np.ascontiguousarray(states, np.int32)
        _check(load().elhl_traj_init_fmo_states(self.handle, len(at), _p(at), len(st), _p(st)),
               "elhl_traj_init_fmo_states")

    def set_psi(self, psi_bra, psi_ket):
        b = np.asfortranarray(psi_bra, np.complex128)
        k = np.asfortranarray(psi_ket, np.complex128)
        _check(load().elhl_traj_set_psi(self.handle, _p(b), _p(k)), "elhl_traj_set_psi")

    def get_psi(self):
        b = np.zeros((self.N, self.P), np.complex128, order="F")
        k = np.zeros((self.N, self.P), np.complex128, order="F")
        _check(load().elhl_traj_get_psi(self.handle, _p(b), _p(k)), "elhl_traj_get_psi")
        return b, k

    def step(self, coords=None, nsteps: int = 1, want_pops: bool = True):
        """nsteps nuclear steps; coords None = fixed nuclei, else (nsteps, natoms, 3).
        Returns populations (nsteps, P, nfrag+1) or None."""
        pops = np.zeros((nsteps, self.P, self.sys.nfrag + 1)) if want_pops else None
        c = None if coords is None else np.ascontiguousarray(coords, np.float64)
        if c is not None and c.size != nsteps * self.sys.natoms * 3:
            raise ValueError("coords must hold nsteps * natoms * 3 values")
        _check(load().elhl_traj_step(self.handle, _p(c), nsteps, _p(pops)), "elhl_traj_step")
        return pops

    def step_device(self, d_coords_ptr: int, nsteps: int, d_pops_ptr: int):
        """Device-pointer variant (pointers as integers)."""
        _check(load().elhl_traj_step_device(self.handle, ctypes.c_void_p(d_coords_ptr), nsteps,
                                            ctypes.c_void_p(d_pops_ptr)), "elhl_traj_step_device")

    def energies(self) -> np.ndarray:
        """Complex wavepacket energy per particle (eV)."""
        E = np.zeros(self.P, np.complex128)
        _check(load().elhl_traj_energies(self.handle, _p(E)), "elhl_traj_energies")
        return E

    def matrices(self):
        N = self.N
        S, h, Hp = (np.zeros((N, N), order="F") for _ in range(3))
        _check(load().elhl_traj_get_matrices(self.handle, _p(S), _p(h), _p(Hp)), "elhl_traj_get_matrices")
        return S, h, Hp

    def factor(self, with_inverse: bool = True):
        """Cholesky factor L of S and (after a step with coordinates) G = L^-1, host copies."""
        N = self.N
        L = np.zeros((N, N), order="F")
        G = np.zeros((N, N), order="F") if with_inverse else None
        _check(load().elhl_traj_get_factor(self.handle, _p(L), _p(G) if G is not None else None),
               "elhl_traj_get_factor")
        return L, G

    def stats(self) -> TrajStats:
        st = TrajStats()
        _check(load().elhl_traj_get_stats(self.handle, ctypes.byref(st)), "elhl_traj_get_stats")
        return st

    def snapshot(self, path: str):
        """Checkpoint in the reference's Security_copy.dat layout (plus the resume record)."""
        _check(load().elhl_traj_snapshot(self.handle, os.fsencode(path)), "elhl_traj_snapshot")

    def restore(self, path: str):
        """Resume from a checkpoint written by snapshot() (or by the reference)."""
        _check(load().elhl_traj_restore(self.handle, os.fsencode(path)), "elhl_traj_restore")


FIXED_SCRATCH_MAX_N = 4096


def propagate_fixed_scratch(n: int, d_H: int, ld: int, d_psi_bra: int, d_psi_ket: int, t_init: float, t_max: float,
                            tau: float, stream: int | None = None) -> float:
    """Allocation-free one-particle propagation on device buffers (integer device
    pointers); for callers that cannot allocate device memory.  Returns save_tau."""
    st = ctypes.c_double(0.0)
    _check(load().elhl_propagate_fixed_scratch(n, ctypes.c_void_p(d_H), ld, ctypes.c_void_p(d_psi_bra),
                                               ctypes.c_void_p(d_psi_ket), t_init, t_max, tau, ctypes.byref(st),
                                               ctypes.c_void_p(stream) if stream else None),
           "elhl_propagate_fixed_scratch")
    return st.value


def bessel_j(beta: float, kmax: int) -> np.ndarray:
    """J_0..J_kmax(beta) (host code of the library, no GPU needed)."""
    J = np.zeros(kmax + 1)
    _check(load().elhl_bessel_j(beta, kmax, _p(J)), "elhl_bessel_j")
    return J


def chebyshev_coefficients(dt: float, emin: float, emax: float, tol: float = 1e-12, kcap: int = 4000):
    """Complex c_k of exp(-i dt H / hbar) on [emin, emax] (host code)."""
    cre, cim = np.zeros(kcap + 1), np.zeros(kcap + 1)
    K = ctypes.c_int(0)
    _check(load().elhl_chebyshev_coefficients(dt, emin, emax, tol, kcap, _p(cre), _p(cim), ctypes.byref(K)),
           "elhl_chebyshev_coefficients")
    return cre[: K.value + 1] + 1j * cim[: K.value + 1]


def kernel_launches() -> int:
    """Kernels of this library launched so far in this process (library calls such as cuBLAS not counted)."""
    return int(load().elhl_kernel_launches())


def set_stream(stream_handle: int | None):
    """Route library work to a caller stream (integer cudaStream_t) or back to its own (None)."""
    _check(load().elhl_set_stream(ctypes.c_void_p(stream_handle) if stream_handle else None), "elhl_set_stream")


def debug_barrier(limit_s: float = 0.0, exit_cta: int = -1):
    """Failure-detection test hook: grid-barrier limit (s, <= 0: default) and a
    CTA of the next propagation launch that leaves before its first barrier."""
    _check(load().elhl_debug_barrier(float(limit_s), int(exit_cta)), "elhl_debug_barrier")


class Batch:
    """Many Chebyshev trajectories advanced by one launch per nuclear step."""

    def __init__(self, systems_list, coords_list=None, **cfg_kw):
        L = load()
        cfg_kw.setdefault("method", METHOD_CHEBYSHEV)
        self.config = default_config(**cfg_kw)
        self.systems = list(systems_list)
        descs = (BasisDesc * len(self.systems))()
        self._keep = []
        cptrs = (ctypes.c_void_p * len(self.systems))()
        for i, sysm in enumerate(self.systems):
            d, keep = _basis_desc(sysm)
            descs[i] = d
            c = np.ascontiguousarray(sysm.coords if coords_list is None else coords_list[i], np.float64)
            self._keep += keep + [c]
            cptrs[i] = c.ctypes.data
        self._descs, self._cptrs = descs, cptrs
        h = ctypes.c_void_p()
        _check(L.elhl_batch_create(len(self.systems), ctypes.cast(descs, ctypes.c_void_p),
                                   ctypes.cast(cptrs, ctypes.c_void_p), ctypes.byref(self.config), ctypes.byref(h)),
               "elhl_batch_create")
        self.handle = h
        self.members = [Trajectory.borrowed(sysm, ctypes.c_void_p(L.elhl_batch_member(h, i)))
                        for i, sysm in enumerate(self.systems)]

    def init_fmo(self, electron_state=None, hole_state=None):
        """Fragment-MO initial states; default LUMO / HOMO of each member's fragment."""
        from dynemol_gb300.systems import fermi_state
        for tr, sysm in zip(self.members, self.systems):
            homo = fermi_state(sysm, sysm.fragment_atoms("E"))
            tr.init_fmo(electron_state or homo + 1, hole_state or homo)

    def compact(self):
        _check(load().elhl_batch_compact(self.handle), "elhl_batch_compact")

    def step(self, nsteps: int = 1, want_pops: bool = True):
        nf1 = self.systems[0].nfrag + 1
        pops = np.zeros((nsteps, len(self.systems), int(self.config.nparticles), nf1)) if want_pops else None
        _check(load().elhl_batch_step(self.handle, nsteps, _p(pops)), "elhl_batch_step")
        return pops

    def stats(self) -> TrajStats:
        st = TrajStats()
        _check(load().elhl_batch_get_stats(self.handle, ctypes.byref(st)), "elhl_batch_get_stats")
        return st

    def close(self):
        if getattr(self, "handle", None):
            load().elhl_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching propagation server (fixed-nuclei Chebyshev requests)."""

    def __init__(self, hbm_budget_bytes: float, **cfg_kw):
        cfg_kw.setdefault("method", METHOD_CHEBYSHEV)
        self.config = default_config(**cfg_kw)
        h = ctypes.c_void_p()
        _check(load().elhl_server_create(float(hbm_budget_bytes), ctypes.byref(self.config), ctypes.byref(h)),
               "elhl_server_create")
        self.handle = h
        self.meta = {}

    def submit(self, system, nsteps: int, states, which: str = "E", coords=None, restart: str | None = None) -> int:
        """Queue a request; `restart`: resume from a checkpoint (snapshot()) and run nsteps more steps."""
        desc, keep = _basis_desc(system)
        c = np.ascontiguousarray(system.coords if coords is None else coords, np.float64)
        at = np.ascontiguousarray(system.fragment_atoms(which), np.int32)
        st = np.ascontiguousarray(states, np.int32)
        req = Request(ctypes.pointer(desc), _p(c), nsteps, len(st), len(at), _p(at), _p(st))
        rid = ctypes.c_longlong(0)
        if restart is None:
            _check(load().elhl_server_submit(self.handle, ctypes.byref(req), ctypes.byref(rid)), "elhl_server_submit")
        else:
            _check(load().elhl_server_submit_restart(self.handle, ctypes.byref(req), os.fsencode(restart),
                                                     ctypes.byref(rid)), "elhl_server_submit_restart")
        self.meta[rid.value] = (system, len(st))
        return rid.value

    def snapshot(self, rid: int, path: str):
        """Checkpoint of an admitted request."""
        _check(load().elhl_server_snapshot(self.handle, rid, os.fsencode(path)), "elhl_server_snapshot")

    def step(self):
        a, p = ctypes.c_int(0), ctypes.c_int(0)
        _check(load().elhl_server_step(self.handle, ctypes.byref(a), ctypes.byref(p)), "elhl_server_step")
        return a.value, p.value

    def poll(self, max_n: int = 1024):
        ids = np.zeros(max_n, np.int64)
        n = ctypes.c_int(0)
        _check(load().elhl_server_poll(self.handle, _p(ids), max_n, ctypes.byref(n)), "elhl_server_poll")
        return [int(x) for x in ids[: n.value]]

    def result(self, rid: int):
        """(populations (P, nfrag+1), kets (N, P), times {submit, admit, done})."""
        system, P = self.meta.pop(rid)
        pops = np.zeros((P, system.nfrag + 1))
        psi = np.zeros((system.nao, P), np.complex128, order="F")
        times = np.zeros(3)
        _check(load().elhl_server_result(self.handle, rid, _p(pops), _p(psi), _p(times)), "elhl_server_result")
        return pops, psi, times

    def close(self):
        if getattr(self, "handle", None):
            load().elhl_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_count() -> int:
    return int(load().elhl_device_count())
