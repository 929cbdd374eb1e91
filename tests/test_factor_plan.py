"""Host replays of the rebuild's index arithmetic, checked on the CPU before any
GPU run:

* the block plan of the recursive Cholesky-with-inverse (chol_inv64 in
  dynemol_gb300/csrc/elhl_api.cu, checked up front by chol_inv_fits): every leaf is a diagonal block of at most 64 rows, the leaves
  tile the matrix, and no off-diagonal block exceeds the ld x N workspace the
  factor allocates; a numpy replay of the same splits reproduces L and L^-1;
* dgemm64's work units (dynemol_gb300/csrc/dgemm.cu): the output tile size it
  picks (64, 32 or 16 rows) and the k range each (tile, k-chunk) unit reads, for
  every tile size and triangular flag, with the constants read from the source;
  the replayed masked product must equal the triangular product, the chunks
  must cover each tile's k tiles exactly once, and every partial tile must have
  its slot in the workspace."""

import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
API = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "elhl_api.cu")).read()
DG = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "dgemm.cu")).read()
HDR = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "elhl_internal.cuh")).read()
LEAF = 64  # leaf_rows(): 64-row diagonal blocks (factor.cu)


def _const(src, name):
    m = re.search(r"\b%s = (\d+)" % name, src)
    assert m, name
    return int(m.group(1))


MAX_TILE, BK = _const(DG, "kMaxTile"), _const(DG, "kBK")
MAX_PARTIALS, UNITS_PER_SLOT = _const(DG, "kMaxPartials"), _const(DG, "kUnitsPerSlot")
# resident CTAs on a GB300 (152 SMs) for 64-, 32- and 16-row tiles: 3 per SM at 256
# threads and 64-68 registers, 8 per SM at 32 registers and 9-17 KB
SLOTS = {64: 3 * 152, 32: 8 * 152, 16: 8 * 152}
TRI_A, TRI_B, TRI_BT, TRI_LC, TRI_AT = (_const(HDR, n) for n in ("kTriA", "kTriB", "kTriBt", "kTriLowerC", "kTriAt"))


def ru(x, m):
    return (x + m - 1) // m * m


def chol_plan(n, ld):
    need, leaves = 0, []

    def rec(a, m):
        nonlocal need
        if m <= LEAF:
            leaves.append((a, m))
            return
        n1 = ru(m // 2, LEAF)
        assert 0 < n1 < m
        need = max(need, ld * n1)
        rec(a, n1)
        rec(a + n1, m - n1)

    rec(0, n)
    return need, leaves


@pytest.mark.parametrize("n", list(range(1, 600)) + list(range(600, 4097, 7)) + [2170, 3720, 8192, 16384])
def test_plan_fits_the_workspace(n):
    assert "chol_inv_fits(n, ld, (size_t)ld * N)" in API  # the FP64 factor's check, workspace ld x N
    ld = ru(n, 32)
    need, leaves = chol_plan(n, ld)
    assert need <= ld * n, (n, need)
    pos = 0
    for a, m in leaves:  # leaves tile [0, n) with aligned blocks of at most 64 rows
        assert a == pos and a % LEAF == 0 and 0 < m <= LEAF
        pos += m
    assert pos == n


def _chol_inv(S):
    n = S.shape[0]
    A, G = np.tril(S).copy(), np.zeros_like(S)

    def rec(a, m):
        i = slice(a, a + m)
        if m <= LEAF:
            Lb = np.linalg.cholesky(A[i, i] + np.tril(A[i, i], -1).T)
            A[i, i], G[i, i] = Lb, np.linalg.inv(Lb)
            return
        n1 = ru(m // 2, LEAF)
        i1, i2 = slice(a, a + n1), slice(a + n1, a + m)
        rec(a, n1)
        A[i2, i1] = A[i2, i1] @ G[i1, i1].T
        A[i2, i2] -= np.tril(A[i2, i1] @ A[i2, i1].T)
        rec(a + n1, m - n1)
        G[i2, i1] = -G[i2, i2] @ (A[i2, i1] @ G[i1, i1])

    rec(0, n)
    return np.tril(A), np.tril(G)


@pytest.mark.parametrize("n", [1, 63, 64, 65, 130, 300, 513, 700, 1100])
def test_plan_computes_the_factors(n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, n))
    S = X @ X.T / n + np.eye(n)
    L = np.linalg.cholesky(S)
    L2, G2 = _chol_inv(S)
    assert np.abs(L2 - L).max() < 1e-12
    assert np.abs(G2 - np.linalg.inv(L)).max() < 1e-12


def _select(m, n, k):
    """dgemm64's tile size: the largest at most twice the narrow side whose (tile,
    k tile) units number at least half of kUnitsPerSlot per resident CTA, else 16
    rows (dgemm.cu, host side)."""
    assert "if (bm <= 2 * std::min(m, n) && 2 * units >= (long long)kUnitsPerSlot * g_slots[v]) break;" in DG
    kt = max(1, (k + BK - 1) // BK)
    for v, bm in enumerate((64, 32)):
        units = ((m + bm - 1) // bm) * ((n + bm - 1) // bm) * kt
        if bm <= 2 * min(m, n) and 2 * units >= UNITS_PER_SLOT * SLOTS[bm]:
            return bm
    return 16


def _chunking(tiles, k, slots, bm):
    """dgemm64's k tiles per work unit and units per tile (dgemm.cu, host side)."""
    max_part = MAX_PARTIALS * (MAX_TILE // bm) ** 2  # partial tiles of bm x bm in the workspace
    kt = max(1, (k + BK - 1) // BK)
    chunk = (tiles * kt + UNITS_PER_SLOT * slots - 1) // (UNITS_PER_SLOT * slots)
    chunk = max(1, min(chunk, kt))
    while chunk < kt and tiles * ((kt + chunk - 1) // chunk) > max_part:
        chunk *= 2
    chunk = min(chunk, kt)
    nchunk = (kt + chunk - 1) // chunk
    assert nchunk == 1 or tiles * nchunk <= max_part
    return chunk, nchunk, max_part


def _dgemm_replay(m, n, k, A, B, ta, tb, tri, bm, slots):
    """C = op(A) op(B) accumulated unit by unit over the k ranges the kernel reads."""
    BM = BN = bm
    opA = A.T if ta else A
    opB = B.T if tb else B
    gx, gy = (m + BM - 1) // BM, (n + BN - 1) // BN
    chunk, nchunk, max_part = _chunking(gx * gy, k, slots, bm)
    C = np.zeros((m, n))
    seen = set()
    for u in range(gx * gy * nchunk):
        t, ch = divmod(u, nchunk)
        bx0, by0 = t % gx, t // gx
        bx = gx - 1 - bx0 if tri & TRI_A else bx0
        by = gy - 1 - by0 if tri & TRI_BT else by0
        i0, j0 = bx * BM, by * BN
        if (tri & TRI_LC) and i0 + BM <= j0:
            continue
        klo, khi = 0, k
        if tri & TRI_A:
            khi = min(khi, i0 + BM)
        if tri & TRI_AT:
            klo = max(klo, i0)
        if tri & TRI_B:
            klo = max(klo, j0)
        if tri & TRI_BT:
            khi = min(khi, j0 + BN)
        nkt = (khi - klo + BK - 1) // BK if khi > klo else 0
        nch = max(1, (nkt + chunk - 1) // chunk)
        if ch >= nch:
            continue
        assert nch == 1 or (by * gx + bx) * nchunk + ch < max_part  # partial slot in the workspace
        assert nch == 1 or by * gx + bx < MAX_PARTIALS * 16  # arrival counter of the tile
        kt0, kt1 = ch * chunk, min(nkt, ch * chunk + chunk)
        lo, hi = klo + kt0 * BK, min(khi, klo + kt1 * BK)
        for k0 in range(lo, hi, BK):
            kk = np.arange(k0, min(k0 + BK, k))  # whole k tiles, masked only at k (as the kernel loads)
            for x in kk:
                assert (bx, by, x) not in seen  # no k index twice in one tile
                seen.add((bx, by, x))
            ii = np.arange(i0, min(i0 + BM, m))
            jj = np.arange(j0, min(j0 + BN, n))
            a = opA[np.ix_(ii, kk)].copy()
            b = opB[np.ix_(kk, jj)].copy()
            gi, gk = np.meshgrid(ii, kk, indexing="ij")
            if tri & TRI_A:
                a[gk > gi] = 0.0
            if tri & TRI_AT:
                a[gk < gi] = 0.0
            gk2, gj = np.meshgrid(kk, jj, indexing="ij")
            if tri & TRI_B:
                b[gk2 < gj] = 0.0
            if tri & TRI_BT:
                b[gk2 > gj] = 0.0
            C[np.ix_(ii, jj)] += a @ b
    return C


@pytest.mark.parametrize("m,n,k", [(200, 200, 200), (130, 70, 130), (64, 2, 64), (3, 5, 7), (190, 190, 61),
                                   (700, 640, 900)])
@pytest.mark.parametrize("case", ["none", "A", "At", "B", "Bt", "Bt_lowerC"])
@pytest.mark.parametrize("bm", [64, 32, 16])
def test_dgemm_tiles_cover_the_triangular_products(m, n, k, case, bm):
    rng = np.random.default_rng(m * 7 + n + k)
    ta = case == "At"
    tb = case.startswith("Bt")
    A = rng.standard_normal((k, m) if ta else (m, k))
    B = rng.standard_normal((n, k) if tb else (k, n))
    tri = {"none": 0, "A": TRI_A, "At": TRI_AT, "B": TRI_B, "Bt": TRI_BT, "Bt_lowerC": TRI_BT | TRI_LC}[case]
    # the triangular operand's stored zero side holds garbage, which the kernel must ignore
    opA, opB = (A.T if ta else A), (B.T if tb else B)
    if tri & TRI_A:
        ref_a = np.tril(opA)
    elif tri & TRI_AT:
        ref_a = np.triu(opA)
    else:
        ref_a = opA
    if tri & TRI_B:
        ref_b = np.tril(opB)
    elif tri & TRI_BT:
        ref_b = np.triu(opB)
    else:
        ref_b = opB
    C = _dgemm_replay(m, n, k, A, B, ta, tb, tri, bm, slots=8)  # few slots: many chunks per tile
    ref = ref_a @ ref_b
    if tri & TRI_LC:  # only tiles reaching the diagonal are written; compare the lower triangle
        mask = np.tril(np.ones((m, n), bool))
        assert np.abs((C - ref)[mask]).max() < 1e-10
    else:
        assert np.abs(C - ref).max() < 1e-10


CHEB = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "cheb.cu")).read()
CBLOCK, YROWS = _const(CHEB, "kBlock"), _const(CHEB, "kYRows")
SMEM_LIMIT = 200 * 1024
PART_BYTES = 16 * 64 * 8


def _jwin(ld, mg, c2):
    """The launcher's window (explicit Hs) when the whole vector does not fit."""
    if PART_BYTES + ld * mg * c2 <= SMEM_LIMIT:
        return 0
    return ((SMEM_LIMIT - PART_BYTES - YROWS * mg * c2) // (mg * c2)) & ~31


@pytest.mark.parametrize("n,mg,c2,krt", [(15553, 4, 8, 8), (15553, 1, 8, 8), (9000, 2, 8, 8), (4000, 4, 16, 2),
                                          (12001, 4, 16, 2), (3000, 4, 8, 8)])
def test_windowed_rows_cover_the_matrix_once(n, mg, c2, krt):
    """order_rows + rows_gemv (cheb.cu) with the vector staged in windows: every
    (row, j) of a segment is summed exactly once, every 16-byte vector stays in
    its window, and the window and partial-sum arrays fit the shared memory."""
    assert "rows_gemv<T, MG, 0>(reinterpret_cast<const T *>(pb.H), ld, s_v, r0, r1, s_part, acc_epi, jw0, jw1)" in CHEB
    ld = ru(n, 32)
    jwin = _jwin(ld, mg, c2)
    warps = CBLOCK // 32
    ve = 16 // (c2 // 2)  # elements per 16-byte load
    if jwin:
        assert PART_BYTES + jwin * mg * c2 + YROWS * mg * c2 <= SMEM_LIMIT and jwin % 32 == 0
    for row0, row1 in [(0, 37), (n - 700, n), (1000, 1000 + YROWS + 5)]:
        row1 = min(row1, n)
        count = np.zeros((row1 - row0, ld), np.int32)
        blocks = [(r, min(row1, r + YROWS)) for r in range(row0, row1, YROWS)] if jwin else [(row0, row1)]
        for r0, r1 in blocks:
            assert r1 - r0 <= YROWS or not jwin
            windows = [(w, min(ld, w + jwin)) for w in range(0, ld, jwin)] if jwin else [(0, ld)]
            for jw0, jw1 in windows:
                rows = r1 - r0
                WR = 1
                while WR < warps and WR * krt < rows:
                    WR <<= 1
                WJ = warps // WR
                for base in range(r0, r1, krt * WR):
                    jlo, jhi = max(jw0, 0), min(jw1, ld)
                    jchunk = ((jhi - jlo + WJ - 1) // WJ + 31) // 32 * 32
                    for wr in range(WR):
                        rr0 = base + krt * wr
                        nr = min(krt, r1 - rr0)
                        if nr <= 0:
                            continue
                        for wj in range(WJ):
                            j0 = jlo + wj * jchunk
                            j1 = min(jhi, j0 + jchunk)
                            for jv in range(j0, j1, ve):  # one lane's vector: [jv, jv + ve)
                                assert jv + ve <= j1 and jv - jw0 >= 0 and jv + ve - jw0 <= jwin + (0 if jwin else ld)
                            if j1 > j0:
                                count[rr0 - row0:rr0 - row0 + nr, j0:j1] += 1
        assert (count == 1).all(), (n, mg, row0, row1)


@pytest.mark.parametrize("tiles,k", [(484, 1408), (841, 1920), (16384, 8192), (4, 64), (64, 480), (3000, 16384),
                                     (65536, 4096)])
@pytest.mark.parametrize("bm", [64, 32, 16])
def test_dgemm_chunking_bounds(tiles, k, bm):
    chunk, nchunk, max_part = _chunking(tiles, k, SLOTS[bm], bm)
    assert chunk >= 1 and nchunk >= 1 and (nchunk == 1 or tiles * nchunk <= max_part)


@pytest.mark.parametrize("m,n,k,bm", [(64, 64, 64, 16), (128, 128, 128, 16), (256, 256, 256, 16), (512, 512, 512, 64),
                                      (3720, 3720, 3720, 64), (3720, 2, 3720, 16), (1920, 24, 1920, 32),
                                      (3720, 40, 3720, 64)])
def test_dgemm_tile_choice(m, n, k, bm):
    """Small products take small tiles so that their units reach most SMs."""
    assert _select(m, n, k) == bm
    gx, gy = (m + bm - 1) // bm, (n + bm - 1) // bm
    _, nchunk, _ = _chunking(gx * gy, k, SLOTS[bm], bm)
    assert gx * gy * nchunk >= min(152, gx * gy * max(1, (k + BK - 1) // BK))
