"""Seeded synthetic EHT systems for the electron-hole propagator.

Geometries are generated here (no external data): a honeycomb carbon flake with
hydrogen-terminated edges and a jittered cubic C/H/O cluster, plus the STO
basis built from the extended-Hueckel parameter table.

* EHT parameters restate the H, C and O rows of ``my_eht_parameters.dat:1,9-10,13-14``
  with the reference's unit conversion and truncation (``EHT_input.f:79-91``):
  zeta / a_Bohr, then zeta and coef truncated to 1e-4.
* AO order per atom is l = 0..AngMax, m = -l..l (``Basis_Builder``,
  ``structure.f:256-298``); k_WH = 1.75 for every atom (``babel.f:120``),
  V_shift = 0.
* Random numbers: splitmix64 -> 53-bit uniforms -> Box-Muller normals, so the
  same seed yields the same geometry on every machine.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

A_BOHR = 0.52917720859  # constants_m.f:21
H_BAR = 6.58264e-4      # eV ps, constants_m.f:23
CUTOFF_ANGS = 12.0      # constants_m.f:34
K_WH = 1.75             # babel.f:120

# symbol: (AtNo, Nvalen, [(n, l, IP eV, zeta a0^-1)]) -- my_eht_parameters.dat rows
_EHT_TABLE = {
    "H": (1, 1, [(1, 0, -13.600, 1.3000)]),
    "C": (6, 4, [(2, 0, -21.400, 1.6250), (2, 1, -11.400, 1.6250)]),
    "O": (8, 6, [(2, 0, -32.300, 2.2750), (2, 1, -14.800, 2.2750)]),
}
SYMBOLS = ("H", "C", "O")


def _trunc4(x: float) -> float:
    """int(x*1e4)*1e-4 as in EHT_input.f:84-91."""
    return float(int(x * 1.0e4)) * 1.0e-4


def eht_shells(symbol: str):
    """[(n, l, IP, zeta_angs, coef)] after the reference's conversion."""
    atno, nval, shells = _EHT_TABLE[symbol]
    out = []
    for n, l, ip, zeta in shells:
        z = _trunc4(zeta / A_BOHR)
        out.append((n, l, ip, z, _trunc4(1.0)))
    return out


def n_valence(symbol: str) -> int:
    return _EHT_TABLE[symbol][1]


# ---------------------------------------------------------------- RNG
_M64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 generator (Steele, Lea, Flood 2014) with Box-Muller normals."""

    def __init__(self, seed: int):
        self.state = seed & _M64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self, n: int) -> np.ndarray:
        """n doubles in (0, 1): (top 53 bits + 0.5) / 2^53."""
        out = np.empty(n)
        for i in range(n):
            out[i] = ((self.next_u64() >> 11) + 0.5) / 9007199254740992.0
        return out

    def normal(self, n: int) -> np.ndarray:
        m = (n + 1) // 2
        u1 = self.uniform(m)
        u2 = self.uniform(m)
        r = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([r * np.cos(2.0 * np.pi * u2), r * np.sin(2.0 * np.pi * u2)])
        return z[:n]

    def permutation(self, n: int) -> np.ndarray:
        """Fisher-Yates with the generator's integers."""
        p = np.arange(n)
        for i in range(n - 1, 0, -1):
            j = self.next_u64() % (i + 1)
            p[i], p[j] = p[j], p[i]
        return p


# ---------------------------------------------------------------- systems
@dataclass
class EHTSystem:
    """Atoms + AO basis of one trajectory (the STO_basis fields the path uses)."""

    symbols: list
    coords: np.ndarray            # (natoms, 3) Angstrom
    fragment: np.ndarray          # (natoms,) int fragment id (0 = donor "D")
    el_atoms: np.ndarray          # (natoms,) bool, El flag
    hl_atoms: np.ndarray          # (natoms,) bool, Hl flag
    nfrag: int = 2
    # basis (filled by build_basis)
    atom_ao0: np.ndarray = field(default=None)
    atom_nao: np.ndarray = field(default=None)
    ao_atom: np.ndarray = field(default=None)
    ao_n: np.ndarray = field(default=None)
    ao_l: np.ndarray = field(default=None)
    ao_m: np.ndarray = field(default=None)
    ao_nzeta: np.ndarray = field(default=None)
    ao_zeta: np.ndarray = field(default=None)   # (nao, 2)
    ao_coef: np.ndarray = field(default=None)   # (nao, 2)
    ao_ip: np.ndarray = field(default=None)
    ao_kwh: np.ndarray = field(default=None)
    ao_vshift: np.ndarray = field(default=None)
    ao_frag: np.ndarray = field(default=None)

    @property
    def natoms(self) -> int:
        return len(self.symbols)

    @property
    def nao(self) -> int:
        return int(self.ao_n.shape[0])

    def build_basis(self) -> "EHTSystem":
        rows = []
        ao0, nao = [], []
        for ia, s in enumerate(self.symbols):
            ao0.append(len(rows))
            for n, l, ip, z, c in eht_shells(s):
                for m in range(-l, l + 1):
                    rows.append((ia, n, l, m, 1, z, 0.0, c, 0.0, ip, K_WH, 0.0, int(self.fragment[ia])))
            nao.append(len(rows) - ao0[-1])
        r = list(zip(*rows))
        self.atom_ao0 = np.asarray(ao0, np.int32)
        self.atom_nao = np.asarray(nao, np.int32)
        self.ao_atom = np.asarray(r[0], np.int32)
        self.ao_n = np.asarray(r[1], np.int32)
        self.ao_l = np.asarray(r[2], np.int32)
        self.ao_m = np.asarray(r[3], np.int32)
        self.ao_nzeta = np.asarray(r[4], np.int32)
        self.ao_zeta = np.ascontiguousarray(np.stack([r[5], r[6]], 1), np.float64)
        self.ao_coef = np.ascontiguousarray(np.stack([r[7], r[8]], 1), np.float64)
        self.ao_ip = np.asarray(r[9], np.float64)
        self.ao_kwh = np.asarray(r[10], np.float64)
        self.ao_vshift = np.asarray(r[11], np.float64)
        self.ao_frag = np.asarray(r[12], np.int32)
        self.coords = np.ascontiguousarray(self.coords, np.float64)
        return self

    def fragment_atoms(self, which: str) -> np.ndarray:
        return np.nonzero(self.el_atoms if which == "E" else self.hl_atoms)[0]


# Hexagon cells (i, j) of the 26-ring benzenoid used for the flake: a 22-ring
# acene strip (row 0) carrying two 2-ring bumps on row 1 (two pyrene-like
# units).  Counted on the bond graph when the flake is built: 100 C, 50
# two-coordinated C (one H each), closest H-H pair 1.75 A.
FLAKE_CELLS = tuple((i, 0) for i in range(22)) + ((5, 1), (6, 1), (15, 1), (16, 1))


def _benzenoid_carbons(cells, bond):
    """Distinct vertices of the fused hexagons at lattice cells (i, j)."""
    a1 = np.array([np.sqrt(3.0) * bond, 0.0])
    a2 = np.array([np.sqrt(3.0) / 2.0 * bond, 1.5 * bond])
    ang = np.deg2rad(30.0 + 60.0 * np.arange(6))
    hexv = bond * np.column_stack([np.cos(ang), np.sin(ang)])
    verts = {}
    for i, j in cells:
        for v in hexv + (i * a1 + j * a2):
            verts.setdefault((int(round(v[0] * 1000)), int(round(v[1] * 1000))), v)
    return np.array(list(verts.values()))


def honeycomb_flake(n_c: int = 100, n_h: int = 50, bond: float = 1.42, ch: float = 1.09,
                    jitter: float = 0.03, seed: int = 1, frag_atoms: int = 20) -> EHTSystem:
    """Hydrogen-terminated graphene flake, C100H50 (FLAKE_CELLS benzenoid).

    Each two-coordinated C gets one H at `ch` along the outward bisector; all
    atoms are then jittered by N(0, jitter^2) per coordinate (z included).
    Atom order: C sorted by (x, y), then H in the order of their carbons.  The
    first `frag_atoms` atoms form the donor fragment (El = Hl = True)."""
    sel = _benzenoid_carbons(FLAKE_CELLS, bond)
    order = np.lexsort((np.round(sel[:, 1], 6), np.round(sel[:, 0], 6)))
    sel = sel[order]
    d = np.linalg.norm(sel[:, None, :] - sel[None, :, :], axis=2)
    nb = (d > 0.1) & (d < bond * 1.1)
    deg = nb.sum(1)
    if len(sel) != n_c or int((deg == 2).sum()) != n_h or (deg < 2).any():
        raise ValueError("FLAKE_CELLS does not give the requested C/H counts")
    c_xyz = np.column_stack([sel, np.zeros(len(sel))])
    h_xyz = []
    for i in range(len(sel)):
        if nb[i].sum() == 2:
            v = (sel[nb[i]] - sel[i]).sum(0)
            u = -v / np.linalg.norm(v)
            h_xyz.append([sel[i, 0] + ch * u[0], sel[i, 1] + ch * u[1], 0.0])
    coords = np.vstack([c_xyz, np.array(h_xyz)])
    rng = SplitMix64(seed)
    coords = coords + jitter * rng.normal(coords.size).reshape(coords.shape)
    symbols = ["C"] * n_c + ["H"] * len(h_xyz)
    nat = len(symbols)
    frag = np.ones(nat, np.int32)
    frag[:frag_atoms] = 0
    el = np.zeros(nat, bool)
    el[:frag_atoms] = True
    return EHTSystem(symbols, coords, frag, el, el.copy()).build_basis()


def cubic_cluster(n_atoms: int = 1200, spacing: float = 1.4, frac=(0.6, 0.3, 0.1), jitter: float = 0.02,
                  seed: int = 2, frag_atoms: int = 20) -> EHTSystem:
    """Disordered C/H/O cluster on a jittered simple-cubic lattice.

    Sites fill a near-cubic box in (x, y, z) order; element labels are a seeded
    permutation of round(frac * n_atoms) C, H and O; the first `frag_atoms`
    atoms form the donor fragment."""
    side = int(np.ceil(n_atoms ** (1.0 / 3.0)))
    idx = np.arange(n_atoms)
    lattice = np.column_stack([idx % side, (idx // side) % side, idx // (side * side)]).astype(np.float64) * spacing
    rng = SplitMix64(seed)
    n_c = int(round(frac[0] * n_atoms))
    n_h = int(round(frac[1] * n_atoms))
    n_o = n_atoms - n_c - n_h
    labels = np.array(["C"] * n_c + ["H"] * n_h + ["O"] * n_o)[rng.permutation(n_atoms)]
    coords = lattice + jitter * rng.normal(3 * n_atoms).reshape(n_atoms, 3)
    frag = np.ones(n_atoms, np.int32)
    frag[:frag_atoms] = 0
    el = np.zeros(n_atoms, bool)
    el[:frag_atoms] = True
    return EHTSystem(list(labels), coords, frag, el, el.copy()).build_basis()


def perturbed_coords(base: np.ndarray, step: int, sigma: float = 0.02, seed: int = 2) -> np.ndarray:
    """Coordinates of nuclear step `step`: base + N(0, sigma^2), fresh per step."""
    rng = SplitMix64((seed * 1_000_003 + step * 7919) & _M64)
    return base + sigma * rng.normal(base.size).reshape(base.shape)


def fermi_state(sys: EHTSystem, atoms: np.ndarray) -> int:
    """HOMO index (1-based) of a fragment: sum(Nvalen)/2 + mod(sum, 2) (FMO.f:332)."""
    tot = sum(n_valence(sys.symbols[i]) for i in atoms)
    return tot // 2 + tot % 2


# target_nao -> (nx, ny, trim): rectangle of nx x ny 4-atom cells, first `trim`
# sites dropped; (11, 48, 0) gives 2014 C + 136 H = 8192 AOs.  Other sizes are
# found by the scan in honeycomb_sheet and cached here.
SHEET_WINDOWS = {8192: (11, 48, 0)}


def honeycomb_sheet(target_nao: int = 8192, bond: float = 1.42, ch: float = 1.09, jitter: float = 0.03,
                    seed: int = 3, frag_atoms: int = 20) -> EHTSystem:
    """Hydrogen-terminated rectangular graphene patch with exactly `target_nao`
    AOs (4 per C, 1 per H): the config-1 construction at larger size.

    A deterministic scan over rectangular windows of the sheet keeps carbons
    with at least two carbon neighbours; every carbon with two neighbours gets
    one H along the outward bisector.  The first `frag_atoms` carbons (sorted by
    x, y) form the donor fragment."""
    a = bond
    cell = np.array([3.0 * a, np.sqrt(3.0) * a])
    basis = np.array([[0.0, 0.0], [a, 0.0], [1.5 * a, np.sqrt(3.0) / 2 * a], [2.5 * a, np.sqrt(3.0) / 2 * a]])

    def patch(nx, ny, trim):
        from scipy.spatial import cKDTree
        pts = (np.stack(np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij"), -1).reshape(-1, 1, 2) * cell
               + basis[None]).reshape(-1, 2)
        pts = pts[trim:] if trim else pts
        while True:  # prune carbons with fewer than two carbon neighbours
            pairs = np.array(sorted(cKDTree(pts).query_pairs(1.1 * a)), dtype=np.int64).reshape(-1, 2)
            deg = np.bincount(pairs.ravel(), minlength=len(pts))
            if (deg >= 2).all():
                nb = [[] for _ in range(len(pts))]
                for i, j in pairs:
                    nb[i].append(j)
                    nb[j].append(i)
                return pts, nb, deg
            pts = pts[deg >= 2]

    found = None
    # windows known to give the workload sizes (found by the scan below)
    candidates = [SHEET_WINDOWS[target_nao]] if target_nao in SHEET_WINDOWS else [
        (nx, ny, trim) for nx in range(2, 40) for ny in range(2, 60)
        if 0.6 * target_nao <= 16 * nx * ny <= 1.05 * target_nao for trim in range(0, 24)]
    for nx, ny, trim in candidates:
        pts, nb, deg = patch(nx, ny, trim)
        if 4 * len(pts) + int((deg == 2).sum()) == target_nao:
            found = (pts, nb, deg)
            SHEET_WINDOWS[target_nao] = (nx, ny, trim)
            break
    if found is None:
        raise ValueError("no sheet with the requested AO count")
    pts, nb, deg = found
    order = np.lexsort((np.round(pts[:, 1], 6), np.round(pts[:, 0], 6)))
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    pts = pts[order]
    nb = [sorted(inv[j] for j in nb[i]) for i in order]
    h_xyz = []
    for i in range(len(pts)):
        if len(nb[i]) == 2:
            v = (pts[nb[i]] - pts[i]).sum(0)
            u = -v / np.linalg.norm(v)
            h_xyz.append([pts[i, 0] + ch * u[0], pts[i, 1] + ch * u[1], 0.0])
    coords = np.vstack([np.column_stack([pts, np.zeros(len(pts))]), np.array(h_xyz)])
    rng = SplitMix64(seed)
    coords = coords + jitter * rng.normal(coords.size).reshape(coords.shape)
    symbols = ["C"] * len(pts) + ["H"] * len(h_xyz)
    nat = len(symbols)
    frag = np.ones(nat, np.int32)
    frag[:frag_atoms] = 0
    el = np.zeros(nat, bool)
    el[:frag_atoms] = True
    return EHTSystem(symbols, coords, frag, el, el.copy()).build_basis()
