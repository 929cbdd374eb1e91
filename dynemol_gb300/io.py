"""On-disk formats of the reference's Chebyshev slice driver.

* survival / wavepacket-energy dumps written by dump_Qdyn (Taylor.f:244-285):
  ``dyn.trunk/{el,hl}_survival.dat`` with a numbered header line
  (FORMAT(A,I9,14I10)), a label line (FORMAT(/15A10)) and one line per step
  (FORMAT(F11.6,14F10.5): time in ps, fragment populations, total), and
  ``{el,hl}_wp_energy.dat`` lines (FORMAT(3F12.6): time, Re E, Im E);
* the checkpoint of Security_Copy_Cheb / Restart_State_Cheb
  (backup.f:329-445): a Fortran sequential unformatted file with 4-byte
  record markers holding frame (optional), it, t, basis size, particle count,
  tag count, the two-character particle tags, per particle the interleaved
  (DUAL_bra, DUAL_ket) and (AO_bra, AO_ket) pairs, and the Net_Charge record
  (which the reference writes as the whole array repeated once per atom).

These let a device-resident run resume from, and hand results to, the
reference's own post-processing.
"""
from __future__ import annotations

import os
import struct

import numpy as np


def _fmt_f(x: float, w: int, d: int) -> str:
    s = f"{x:{w}.{d}f}"
    return s if len(s) <= w else "*" * w


class SurvivalWriter:
    """dump_Qdyn equivalent for one particle tag ("el" or "hl")."""

    def __init__(self, directory: str, tag: str, fragments):
        self.dir = directory
        self.tag = tag
        self.fragments = list(fragments)
        os.makedirs(directory, exist_ok=True)
        self.surv = os.path.join(directory, f"{tag}_survival.dat")
        self.erg = os.path.join(directory, f"{tag}_wp_energy.dat")
        nf = len(self.fragments)
        with open(self.surv, "w") as f:
            cols = [nf_ + 1 for nf_ in range(nf + 2)]
            f.write("#" + f"{cols[0]:9d}" + "".join(f"{c:10d}" for c in cols[1:]) + "\n")
            f.write("\n" + "".join(f"{s:>10s}" for s in ["#"] + self.fragments + ["total"]) + "\n")
        open(self.erg, "w").close()

    def write(self, t: float, pops, energy: complex | None = None):
        """pops: fragment populations followed by the total."""
        with open(self.surv, "a") as f:
            f.write(_fmt_f(t, 11, 6) + "".join(_fmt_f(p, 10, 5) for p in pops) + "\n")
        if energy is not None:
            with open(self.erg, "a") as f:
                f.write(_fmt_f(t, 12, 6) + _fmt_f(energy.real, 12, 6) + _fmt_f(energy.imag, 12, 6) + "\n")


def read_survival(path: str) -> np.ndarray:
    rows = []
    for line in open(path):
        if line.startswith("#") or not line.strip() or line.strip().startswith("#"):
            continue
        rows.append([float(x) for x in line.split()])
    return np.array(rows)


# ---------------------------------------------------------------- checkpoint
def _record(f, payload: bytes):
    n = struct.pack("<i", len(payload))
    f.write(n + payload + n)


def _read_record(f) -> bytes:
    head = f.read(4)
    if len(head) < 4:
        raise EOFError
    (n,) = struct.unpack("<i", head)
    data = f.read(n)
    (m,) = struct.unpack("<i", f.read(4))
    if m != n:
        raise ValueError("corrupt record markers")
    return data


def net_charge(dual_bra, dual_ket, ao_atom, natoms) -> np.ndarray:
    """Net_Charge(atom) = sum_n sign_n |sum_{i in atom} bra_i ket_i|, sign = [-1 el, +1 hl]
    (Populations_mtx, data_output.f:129-134)."""
    q = np.zeros(natoms)
    signs = [-1.0, 1.0]
    for n in range(dual_bra.shape[1]):
        prod = dual_bra[:, n] * dual_ket[:, n]
        for a in range(natoms):
            q[a] += signs[n % 2] * abs(prod[ao_atom == a].sum())
    return q


def write_checkpoint(path: str, it: int, t: float, dual_bra, dual_ket, ao_bra, ao_ket, tags=("el", "hl"),
                     charges=None, frame: int | None = None):
    """Security_Copy_Cheb layout (backup.f:367-390)."""
    N, P = ao_bra.shape
    with open(path, "wb") as f:
        if frame is not None:
            _record(f, struct.pack("<i", frame))
        _record(f, struct.pack("<i", it))
        _record(f, struct.pack("<d", t))
        _record(f, struct.pack("<i", N))
        _record(f, struct.pack("<i", P))
        _record(f, struct.pack("<i", len(tags)))
        _record(f, "".join(f"{s:2.2s}" for s in tags).encode())
        for j in range(P):
            pair = np.empty(2 * N, np.complex128)
            pair[0::2], pair[1::2] = dual_bra[:, j], dual_ket[:, j]
            _record(f, pair.tobytes())
            pair[0::2], pair[1::2] = ao_bra[:, j], ao_ket[:, j]
            _record(f, pair.tobytes())
        q = np.zeros(0) if charges is None else np.asarray(charges, np.float64)
        _record(f, np.tile(q, len(q)).tobytes())


def read_checkpoint(path: str, with_frame: bool = False) -> dict:
    """Restart_State_Cheb (backup.f:399-445)."""
    out = {}
    with open(path, "rb") as f:
        if with_frame:
            (out["frame"],) = struct.unpack("<i", _read_record(f))
        (out["it"],) = struct.unpack("<i", _read_record(f))
        (out["t"],) = struct.unpack("<d", _read_record(f))
        (N,) = struct.unpack("<i", _read_record(f))
        (P,) = struct.unpack("<i", _read_record(f))
        (ntag,) = struct.unpack("<i", _read_record(f))
        raw = _read_record(f).decode()
        out["tags"] = [raw[2 * i: 2 * i + 2] for i in range(ntag)]
        for k in ("dual_bra", "dual_ket", "ao_bra", "ao_ket"):
            out[k] = np.zeros((N, P), np.complex128, order="F")
        for j in range(P):
            pair = np.frombuffer(_read_record(f), np.complex128)
            out["dual_bra"][:, j], out["dual_ket"][:, j] = pair[0::2], pair[1::2]
            pair = np.frombuffer(_read_record(f), np.complex128)
            out["ao_bra"][:, j], out["ao_ket"][:, j] = pair[0::2], pair[1::2]
        q = np.frombuffer(_read_record(f), np.float64)
        n = int(round(np.sqrt(len(q)))) if len(q) else 0
        out["net_charge"] = q[:n].copy()
    return out


def state_from_checkpoint(ck: dict):
    """(Psi_bra, Psi_ket) for resuming: Psi_bra = DUAL_ket, Psi_ket = AO_ket
    (preprocess_from_restart, ElHl_Chebyshev.f:396-397)."""
    return np.asfortranarray(ck["dual_ket"]), np.asfortranarray(ck["ao_ket"])


def checkpoint_from_state(psi_bra, psi_ket, ao_bra_conj):
    """DUAL_bra = conj(Psi_ket), DUAL_ket = Psi_bra, AO_bra = conj(S^-1 Psi_bra) (given),
    AO_ket = Psi_ket (ElHl_Chebyshev.f:270-276)."""
    return np.conj(psi_ket), psi_bra, ao_bra_conj, psi_ket
