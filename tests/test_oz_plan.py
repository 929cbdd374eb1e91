"""Host replays of the tensor-core FP64 arithmetic of ELHL_PREC_OZ64 (the
propagation in dynemol_gb300/csrc/ozaki.cu, the factorisation products in
dynemol_gb300/csrc/ozgemm.cu), checked on the CPU before any GPU run:

* the block schedule (oz_schedule): every 128 x 64 block of the operator is
  given to exactly one CTA, CTAs differ by at most one block, a row tile's
  segments are numbered in K order and their partial slots fit the partial
  buffer, and every half of a 64-row chunk (4 of its 8 columns) has one CTA
  designated for its epilogue;
* the arithmetic: operands cut into 7 slices of 8 bits on power-of-two scales
  exactly as the kernels do (slice7: one rounding to a 64-bit integer, then
  balanced base-256 digits; operator rows one scale each, vector columns one
  per 64-row chunk), the slice products of one weight s_a + s_b accumulated
  together per 64-K block, where every sum of absolute products must stay at or
  below 2^24 (so that the tensor cores' FP32 accumulation is exact), the weights <= 6 folded exactly into
  two 64-bit integers and the chunks added as integers in the frame of the
  column's largest chunk scale; the result must agree with the exact
  (rational) product to within an FP64 dot product's rounding bound plus the
  slices' own truncation (2^-54.5 of the row and column scales per k),
  including rows and columns of very different scales;
* the products' weight sums (ozgemm: all slice pairs of one weight share an
  accumulator over a 64-K block) against the same 2^24 bound, and their fold
  into two 64-bit integers.
The constants are read from the kernel sources."""

import os
import re
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OZ = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "ozaki.cu")).read()


def _const(name):
    m = re.search(r"\b%s = (\d+)" % name, OZ)
    assert m, name
    return int(m.group(1))


S, TILE, KB = _const("kS"), _const("kTileM"), _const("kKB")
CHUNK = 64  # rows of a vector sharing one scale per column (one 64-K block)
GRID = 152


def schedule(n, grid):
    """oz_schedule: (segments, seg_begin, part_base, part_count); a segment is (rt, kb0, kb1, slot)."""
    nkb, ntiles = -(-n // KB), -(-n // TILE)
    total = nkb * ntiles
    segs, begin, count = [], [0], [0] * ntiles
    for b in range(grid):
        u0, u1 = total * b // grid, total * (b + 1) // grid
        while u0 < u1:
            rt = u0 // nkb
            end = min(u1, (rt + 1) * nkb)
            segs.append((rt, u0 - rt * nkb, end - rt * nkb, count[rt]))
            count[rt] += 1
            u0 = end
        begin.append(len(segs))
    base = [0] * ntiles
    for t in range(1, ntiles):
        base[t] = base[t - 1] + count[t - 1]
    return segs, begin, base, count


def test_schedule_source_matches_replay():
    """The replay follows the source's block ranges (guard against drift)."""
    assert "const long long total = (long long)nkb * ntiles;" in OZ
    assert "long long u0 = total * b / grid;" in OZ
    assert "const int rt = (int)(u0 / nkb);" in OZ


@pytest.mark.parametrize("n", [1, 2, 8, 63, 64, 65, 127, 128, 129, 450, 1000, 1860, 2170, 3720, 4096, 8192, 16384])
def test_schedule_covers_blocks_once(n):
    """Every 128 x 64 block of the operator (rows and K below n) goes to exactly
    one CTA, CTAs differ by at most one block, a row tile's segments are
    numbered in K order, partial slots fit the buffer, and every half of a
    64-row chunk (4 of its 8 columns) has one designated CTA, floor(q grid /
    halves)."""
    segs, begin, base, count = schedule(n, GRID)
    nkb, ntiles = -(-n // KB), -(-n // TILE)
    seen = np.zeros((ntiles, nkb), dtype=int)
    for rt, k0, k1, slot in segs:
        assert 0 <= rt < ntiles and 0 <= k0 < k1 <= nkb
        seen[rt, k0:k1] += 1
    assert np.all(seen == 1)
    per_cta = [sum(s[2] - s[1] for s in segs[begin[b]:begin[b + 1]]) for b in range(GRID)]
    assert max(per_cta) - min(per_cta) <= 1
    for rt in range(ntiles):
        mine = sorted([s for s in segs if s[0] == rt], key=lambda s: s[3])
        assert [s[3] for s in mine] == list(range(count[rt]))
        assert all(mine[i][2] == mine[i + 1][1] for i in range(len(mine) - 1))
        assert base[rt] + count[rt] <= len(segs)
    assert len(segs) <= GRID + ntiles
    nhc = 4 * ntiles  # half-chunks: 64 rows x 4 columns
    designated = [list(range(-(-b * nhc // GRID), -(-(b + 1) * nhc // GRID))) for b in range(GRID)]
    assert sorted(q for d in designated for q in d) == list(range(nhc))
    assert all(q * GRID // nhc == b for b, d in enumerate(designated) for q in d)
    assert "const int nhc = 4 * ntiles, G = gridDim.x;" in OZ


def scale_exp(mx):
    """The kernel's scale_exp: e with |x| < 2^e from the biased exponent (0 for 0)."""
    if not mx > 0.0:
        return 0
    return int((np.float64(mx).view(np.int64) >> 52) & 0x7FF) - 1022


def slices(x, e):
    """x (1-D) on scale 2^e cut as slice7 (tc_ptx.cuh) does: T = rint(x 2^-e 2^56) as a
    64-bit integer (the kernel rounds on the bits; test_slice7_bits_round_like_rint),
    then balanced base-256 digits from the bottom."""
    T = np.rint(x * np.ldexp(1.0, -e) * 2.0 ** 56).astype(np.int64)
    out = [None] * S
    for s in range(S - 1, 0, -1):
        d = ((T + 128) & 255) - 128
        out[s] = d
        T = (T - d) >> 8
    out[0] = T
    return np.array(out, dtype=np.float64)  # [S][len]


def test_slice7_source_matches_replay():
    src = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "tc_ptx.cuh")).read()
    assert "const int sh = (be ? be : 1) - 1075 + 56 - e;" in src  # T = rint(x 2^(56 - e)) from the bits
    assert "T = (long long)(q + ((rem > half || (rem == half && (q & 1))) ? 1ull : 0ull));" in src  # half to even
    assert "const int d = (int)(((T + 128) & 255) - 128);" in src
    assert "T = (T - d) >> 8;" in src


def slice7_bits(x, e):
    """slice7's rounding of x 2^(56 - e) done on the bits as the kernel does (Python ints)."""
    b = int(np.float64(x).view(np.uint64))
    be = (b >> 52) & 0x7FF
    m = (b & ((1 << 52) - 1)) | ((1 << 52) if be else 0)
    sh = (be if be else 1) - 1075 + 56 - e
    if sh >= 0:
        T = m << sh
    elif sh > -64:
        k = -sh
        q, rem, half = m >> k, m & ((1 << k) - 1), 1 << (k - 1)
        T = q + (1 if (rem > half or (rem == half and (q & 1))) else 0)
    else:
        T = 0
    return -T if b >> 63 else T


def test_slice7_bits_round_like_rint():
    """The integer rounding equals rint(x 2^(56 - e)) for normal, tiny and subnormal
    values, ties included."""
    rng = np.random.default_rng(3)
    xs = list(rng.standard_normal(2000) * np.exp(rng.uniform(-40, 3, 2000)))
    xs += [0.0, -0.0, 5e-324, -7e-320, 2.0 ** -1022, 1.5 * 2.0 ** -60, 2.5 * 2.0 ** -56, 3.5 * 2.0 ** -56]
    for x in xs:
        e = scale_exp(abs(x)) if x != 0 else 0
        for ee in (e, e + 3):
            want = round(Fraction(float(x)) * Fraction(2) ** (56 - ee))  # half to even
            assert slice7_bits(x, ee) == want, (x, ee)


def oz_product(A, X):
    """y = A X as oz_cheb_kernel computes it: row scales for A, one scale per
    64-row chunk and column for X (the producing epilogue's chunk); per 64-K block
    all pairs of weight d = a + b <= 6 share one accumulator, folded exactly into
    H (weights d <= 2) and L (d >= 3) over the chunk's blocks; T = 2^32 H + L is
    added, shifted down to the frame of the column's
    largest chunk exponent E (floor), into one integer; y = 2^(E - 64) x that
    integer x the row scale."""
    m, K = A.shape
    nc = X.shape[1]
    er = [scale_exp(np.abs(A[i]).max()) for i in range(m)]
    As = np.stack([slices(A[i], er[i]) for i in range(m)], axis=1).astype(np.int64)  # [S][m][K]
    assert np.abs(As[0]).max() <= 256 and np.abs(As[1:]).max() <= 128
    chunks = []
    for g0 in range(0, K, CHUNK):
        g = slice(g0, min(K, g0 + CHUNK))
        mx = [np.abs(X[g, c]).max() for c in range(nc)]
        ec = [scale_exp(v) for v in mx]
        Xs = np.stack([slices(X[g, c], ec[c]) for c in range(nc)], axis=2).astype(np.int64)  # [S][chunk][c]
        assert np.abs(Xs[0]).max() <= 256 and np.abs(Xs[1:]).max() <= 128
        chunks.append((g, ec, mx, Xs))
    E = [max([ch[1][c] for ch in chunks if ch[2][c] > 0], default=0) for c in range(nc)]
    y = np.zeros((m, nc))
    for i in range(m):
        for c in range(nc):
            acc128 = 0
            for g, ec, mx, Xs in chunks:
                H = Lo = 0
                for b0 in range(0, g.stop - g.start, KB):  # one TMEM accumulation per 64-K block
                    kk = slice(b0, b0 + KB)
                    for d in range(S):  # all pairs of weight d share one accumulator
                        terms = [As[a, i, g][kk] * Xs[d - a, kk, c] for a in range(d + 1)]
                        assert sum(int(np.abs(t).sum()) for t in terms) <= 1 << 24  # exact FP32 accumulation
                        acc = sum(int(t.sum()) for t in terms)
                        if d <= 2:
                            H += acc << (8 * (2 - d))
                        else:
                            Lo += acc << (8 * (S - 1 - d))
                assert abs(H) < 1 << 62 and abs(Lo) < 1 << 62
                T = (H << 32) + Lo
                assert abs(T) < 1 << 76
                acc128 += T >> max(0, E[c] - ec[c])
            assert abs(acc128) < 1 << 126
            y[i, c] = float(Fraction(acc128) * Fraction(2) ** (E[c] - 64 + er[i]))
    return y


def oz_bound(A, X, groups=1):
    """FP64 rounding of the group sums, (groups + 1) 2^-53 sum |a| |x|, plus what the
    slices leave out: per k at most 2^-54.5 of the row and column scales 2^(e_r +
    e_c) (residuals below 2^-57 of each scale, dropped products of weight d >= 7)."""
    er = np.array([scale_exp(np.abs(A[i]).max()) for i in range(A.shape[0])], dtype=float)
    ec = np.array([scale_exp(np.abs(X[:, c]).max()) for c in range(X.shape[1])], dtype=float)
    return ((np.abs(A) @ np.abs(X)) * (groups + 1) * 2.0 ** -53 + A.shape[1] * 2.0 ** (er[:, None] + ec[None, :] - 54)
            + 1e-300)


def exact_product(A, X):
    return np.array([[float(sum(Fraction(float(A[i, k])) * Fraction(float(X[k, c])) for k in range(A.shape[1])))
                      for c in range(X.shape[1])] for i in range(A.shape[0])])


def test_slice_product_matches_exact_product():
    rng = np.random.default_rng(7)
    m, K = 6, 700  # six 128-row chunks of X, the last partial
    A = rng.standard_normal((m, K)) * np.exp(rng.uniform(-12, 2, (m, K)))  # wide dynamic range per row
    A[1] *= 1e-9   # a tiny row
    A[2, ::7] = 0.0
    X = rng.standard_normal((K, 8))
    X[:, 3] *= 1e-12  # a tiny column
    X[:, 5] = 0.0     # an unused column
    y = oz_product(A, X)
    ref = exact_product(A, X)
    assert np.all(np.abs(y - ref) <= oz_bound(A, X, groups=-(-K // CHUNK)))
    assert np.all(y[:, 5] == 0.0)


OZG = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "ozgemm.cu")).read()


def test_gemm_constants_match_source():
    assert re.search(r"\bkS = (\d+)", OZG).group(1) == str(S)
    assert "constexpr int kTM = 128, kTN = 32, kKB = 64;" in OZG
    assert "if (d <= 2) H[c] += x * (1ll << (8 * (2 - d)));" in OZG
    assert "else L[c] += x * (1ll << (8 * (kS - 1 - d)));" in OZG


def test_gemm_weight_sums_are_exact_and_fold_to_the_product():
    """ozgemm: per 64-K block the products of equal weight d = a + b share one FP32
    accumulator; every such sum of absolute products must stay at or below 2^24,
    the folds H (d <= 2) and L (d >= 3) must stay inside int64 over all blocks, and
    2^-64 (2^32 H + L) times the scales must agree with the exact product.  The
    lower-triangular masks of kTriA / kTriBt are applied as the slicing does."""
    rng = np.random.default_rng(11)
    m, n, k = 5, 4, 300
    A = rng.standard_normal((m, k)) * np.exp(rng.uniform(-10, 3, (m, k)))
    B = rng.standard_normal((k, n))
    B[:, 2] *= 1e-7
    A[np.arange(m)[:, None] < np.arange(k)[None, :] - 200] = 0.0  # zero upper band, as a triangular operand
    er = [scale_exp(np.abs(A[i]).max()) for i in range(m)]
    ec = [scale_exp(np.abs(B[:, j]).max()) for j in range(n)]
    As = np.stack([slices(A[i], er[i]) for i in range(m)], axis=1).astype(np.int64)     # [S][m][k]
    Bs = np.stack([slices(B[:, j], ec[j]) for j in range(n)], axis=2).astype(np.int64)  # [S][k][n]
    out = np.zeros((m, n))
    for i in range(m):
        for j in range(n):
            H = L = 0
            for k0 in range(0, k, KB):
                g = slice(k0, k0 + KB)
                for d in range(S):
                    terms = [As[a, i, g] * Bs[d - a, g, j] for a in range(d + 1)]
                    assert sum(int(np.abs(t).sum()) for t in terms) <= 1 << 24
                    acc = sum(int(t.sum()) for t in terms)
                    if d <= 2:
                        H += acc << (8 * (2 - d))
                    else:
                        L += acc << (8 * (S - 1 - d))
                assert abs(H) < 1 << 62 and abs(L) < 1 << 62
            out[i, j] = float(Fraction((H << 32) + L, 1 << 64) * Fraction(2) ** (er[i] + ec[j]))
    ref = exact_product(A, B)
    assert np.all(np.abs(out - ref) <= oz_bound(A, B))


def i128_to_double(v):
    """The kernel's rounding of a 128-bit integer to FP64: its magnitude from three
    positive parts (high word, two 32-bit halves of the low word), two roundings."""
    m = abs(v)
    hi, lo = m >> 64, m & ((1 << 64) - 1)
    assert hi < 1 << 52
    d = float(hi) * 2.0 ** 64 + (float(lo >> 32) * 2.0 ** 32 + float(lo & 0xFFFFFFFF))
    return -d if v < 0 else d


def test_partial_sums_round_to_fp64():
    """The exact 128-bit sum of a row tile's partials rounds to within 2 ulp,
    negative sums included (rounding the magnitude avoids the cancellation of a
    two's complement high word -1 against a large low word)."""
    src = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "ozaki.cu")).read()
    assert "fma(u52_to_double(s.lo >> 32), 0x1p32, u52_to_double(s.lo & 0xffffffffull))" in src
    rng = np.random.default_rng(5)
    for trial in range(4000):
        nseg = int(rng.integers(1, 9))
        parts = [int(rng.integers(-2 ** 62, 2 ** 62)) * int(rng.integers(1, 2 ** 28)) >> int(rng.integers(0, 60))
                 for _ in range(nseg)]
        total = sum(parts)
        assert abs(total) < 2 ** 116
        d = i128_to_double(total)
        assert abs(Fraction(d) - total) <= 2 * abs(Fraction(total)) * Fraction(1, 2 ** 53)


def _gemm_kblocks(m, n, k, tri, bx, by):
    """ozgemm_kernel's K blocks [kb0, kb1) for output tile (bx, by) (128 x 32)."""
    TM, TN, KBK = 128, 32, 64
    i0, j0 = bx * TM, by * TN
    klo, khi = 0, k
    if tri & 1:    # kTriA
        khi = min(khi, i0 + TM)
    if tri & 16:   # kTriAt
        klo = max(klo, i0)
    if tri & 2:    # kTriB
        klo = max(klo, j0)
    if tri & 4:    # kTriBt
        khi = min(khi, j0 + TN)
    kb0 = klo // KBK
    kb1 = -(-khi // KBK) if khi > klo else kb0
    return kb0, kb1


def _read_range(mask, tile, k, r):
    """The slicing kernels' read_range: the K range a row's output tile reads."""
    t0 = r // tile * tile
    lo = t0 // 64 * 64 if mask == 2 else 0
    hi = -(-min(k, t0 + tile) // 64) * 64 if mask == 1 else 1 << 30
    return lo, hi


def test_slicing_covers_every_k_block_the_product_reads():
    """The slicing kernels skip a triangular operand's 32-column tiles outside
    read_range; every K block ozgemm_kernel loads for an output tile must lie
    inside the range of every row of both operand tiles (op(A): 128 rows, op(B)^T:
    32 rows), for each triangular flag and ragged sizes."""
    src = OZG
    assert "lo = v.mask == 2 ? t0 / kKB * kKB : 0;" in src
    assert "hi = v.mask == 1 ? (min(v.k, t0 + v.tile) + kKB - 1) / kKB * kKB : 1 << 30;" in src
    assert "if (g.tri & kTriA) khi = min(khi, i0 + kTM);" in src
    assert "if (g.tri & kTriBt) khi = min(khi, j0 + kTN);" in src
    masks = {0: (0, 0), 1: (1, 0), 16: (2, 0), 2: (0, 2), 4: (0, 1), 1 | 4: (1, 1), 16 | 2: (2, 2)}
    for (m, n, k) in [(320, 320, 320), (448, 1000, 1920), (1800, 1920, 1920), (1000, 333, 777), (130, 97, 64)]:
        for tri, (ma, mb) in masks.items():
            for bx in range(-(-m // 128)):
                for by in range(-(-n // 32)):
                    kb0, kb1 = _gemm_kblocks(m, n, k, tri, bx, by)
                    if kb1 <= kb0:
                        continue
                    K0, K1 = 64 * kb0, 64 * kb1
                    for r in range(bx * 128, min(m, bx * 128 + 128), 32):
                        lo, hi = _read_range(ma, 128, k, r)
                        assert lo <= K0 and K1 <= hi, ("A", m, n, k, tri, bx, r)
                    for r in range(by * 32, min(n, by * 32 + 32), 32):
                        lo, hi = _read_range(mb, 32, k, r)
                        assert lo <= K0 and K1 <= hi, ("B", m, n, k, tri, by, r)


def test_half_chunk_epilogue_covers_the_chunk_once():
    """The chunk epilogue runs in two halves of 4 columns on different CTAs:
    thread t of half c owns row t & 63 and columns 4 c + 2 (t >> 6) + {0, 1}
    (one complex column); together the halves own every (row, column) of the
    64 x 8 chunk once, and their 16-byte copies of slots 1-7 cover the tile's
    rows 8 (b + 1) + column without overlap and never touch the zero slots 0, 8."""
    assert "return EpiThread{t, t & 63, t >> 6, 64 * h + (t & 63), 4 * c + 2 * (t >> 6)};" in OZ
    assert "const int o = (8 * (1 + q / 32) + 4 * half + (q / 8) % 4) * 128 + (q % 8) * 16;" in OZ
    assert "constexpr int kPieces = kS * 4 * 8;" in OZ
    own = np.zeros((64, 8), dtype=int)
    for c in range(2):
        for t in range(128):
            r, col = t & 63, 4 * c + 2 * (t >> 6)
            own[r, col] += 1
            own[r, col + 1] += 1
            assert col // 2 == 2 * c + (t >> 6)  # the complex column the thread accumulates
    assert np.all(own == 1)
    tile = np.zeros(9 * 8 * 128, dtype=int)  # 9 slots x 8 rows x 128 bytes
    for half in range(2):
        for q in range(S * 4 * 8):
            o = (8 * (1 + q // 32) + 4 * half + (q // 8) % 4) * 128 + (q % 8) * 16
            tile[o:o + 16] += 1
    rows = tile.reshape(9 * 8, 128)
    assert np.all(rows[8:64] == 1)                   # slots 1-7: every byte copied once
    assert np.all(rows[:8] == 0) and np.all(rows[64:] == 0)  # the zero slots are never written
