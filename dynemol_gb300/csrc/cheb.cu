// Batched Chebyshev propagation on the symmetrised Hamiltonian.
//
// For S = L L^T, S^-1 h = L^-T H~ L^T with H~ = L^-1 h L^-T symmetric, so
//   ket:  psi(t) = L^-T exp(-i H~ t/hbar) L^T psi(0)
//   bra:  bra(t) = L exp(-i H~ t/hbar) L^-1 bra(0)
// (the reference's bra update with H'^T, Taylor.f:94, is exp(-i h S^-1 t) =
// L exp(-i H~ t) L^-1).  The transformed columns phi = L^T psi and
// chi = L^-1 bra are propagated with the Chebyshev expansion of
// exp(-i tau H~) (Tal-Ezer & Kosloff 1984) on Hs = (H~ - a)/b, spectrum in [-1, 1]:
//   v_0 = phi, v_1 = Hs v_0, v_{k+1} = 2 Hs v_k - v_{k-1},   phi' = sum_k c_k v_k.
//
// One cooperative launch advances every problem of a batch (trajectories of
// different N and order counts) by one nuclear step.  Each CTA owns fixed row
// segments (balanced by matrix elements on the host).  Per order it stages the
// previous vector of a column group in shared memory; warps form a WR x WJ
// grid over (8-row tiles, slices of j); every warp accumulates 8 rows x MG
// complex columns in registers (Hs symmetric: row i is the contiguous column i),
// partial sums meet in shared memory in a fixed order, and the epilogue
// applies the recurrence and adds c_k v_k to the FP64 accumulator.  A bounded
// grid barrier separates orders.
//   T = double : FP64 products;  T = float : FP32 Hs and vectors,
//   FP64 coefficients and accumulation.
#include <type_traits>

#include "df64.cuh"
#include "elhl_internal.cuh"
#include "grid_sync.cuh"

namespace elhl {
namespace {

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

constexpr int kBlock = 512;
constexpr int kWarps = kBlock / 32;
constexpr int kYRows = 512;  // rows per block of window partial sums (explicit Hs, large bases)
// rows per warp tile: FP32 reuses each staged x over 8 rows (shared-memory
// bandwidth); FP64 is bound by its FMA pipe, so 2-row tiles keep the per-CTA
// row counts (about N / 152) from wasting FMAs on partial tiles
template <typename T> struct RowTile;
template <> struct RowTile<double> { static constexpr int value = 2; };
template <> struct RowTile<float> { static constexpr int value = 8; };

template <typename T> struct Vec16;  // 16-byte vector of T
template <> struct Vec16<double> { using type = double2; };
template <> struct Vec16<float> { using type = float4; };
__device__ __forceinline__ double lane_elem(const double2 &v, int u) { return u == 0 ? v.x : v.y; }
__device__ __forceinline__ float lane_elem(const float4 &v, int u) {
    return u == 0 ? v.x : u == 1 ? v.y : u == 2 ? v.z : v.w;
}

__device__ __forceinline__ double2 ldcg2(const double2 *p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg2(const float2 *p) { return __ldcg(p); }

// Warp sums of NV values (NV = 4 ... 32) per lane: plain butterflies over the
// lane bits >= log2(NV), then a transposed butterfly over the low bits; lane l
// returns the warp sum of v[l % NV].
template <typename T, int NV>
__device__ __forceinline__ T warp_sums(T (&v)[NV], int lane) {
#pragma unroll
    for (int o = 16; o >= NV; o >>= 1)
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
#pragma unroll
    for (int o = NV / 2; o > 0; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const T send = upper ? v[i] : v[i + o];
            const T keep = upper ? v[i + o] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0];
}

// y_i = sum_j M(j, i) x_j for the rows [row0, row1) of one segment, MG complex
// columns x staged in shared memory (s_v[j*MG + c]); M is column-major with
// leading dimension ld (column i = row i of M^T).  Calls epi(i, c, yr, yi).
// TRI = 0: full columns; 1: column i is zero above row i (M = L^-1, j >= i);
// 2: column i is zero below row i (M = L^T or L^-T, j <= i).  The j range of a
// super-tile is cut to its non-zero part (widened to multiples of 32; the
// stored zeros inside it are read as they are).  Rows past row1 in a warp's
// 8-row tile issue no loads and no FMAs.
template <typename T, int MG, int TRI, typename Epi>
__device__ void rows_gemv(const T *M, int ld, const typename Vec2<T>::type *s_v, int row0, int row1, T *s_part,
                          Epi &epi, int jw0 = 0, int jw1 = 1 << 30) {
    using T2 = typename Vec2<T>::type;
    constexpr int kRT = RowTile<T>::value;
    constexpr int NV = kRT * MG * 2;   // accumulators per lane (4 ... 64)
    constexpr int NW = NV < 32 ? NV : 32;
    constexpr int NB = NV / NW;        // warp-sum batches
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rows = row1 - row0;
    int WR = 1;
    while (WR < kWarps && WR * kRT < rows) WR <<= 1;
    const int WJ = kWarps / WR;
    const int wr = warp / WJ, wj = warp % WJ;
    for (int base = row0; base < row1; base += kRT * WR) {
        const int tile_end = min(row1, base + kRT * WR);
        // j window [jw0, jw1) (multiples of 32; s_v holds x from row jw0 on)
        const int jlo = max(jw0, TRI == 1 ? (base & ~31) : 0);
        const int jhi = min(jw1, TRI == 2 ? min(ld, (tile_end + 31) & ~31) : ld);
        const int jchunk = ((jhi - jlo + WJ - 1) / WJ + 31) / 32 * 32;
        const int j0 = jlo + wj * jchunk, j1 = min(jhi, j0 + jchunk);
        const int r0 = base + kRT * wr;
        const int nr = min(kRT, row1 - r0);  // rows of this warp's tile (<= 0: none)
        T acc[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = T(0);
        const T *cols[kRT];
#pragma unroll
        for (int r = 0; r < kRT; ++r) cols[r] = M + (size_t)min(r0 + r, row1 - 1) * ld;
        // 16-byte loads: VE consecutive j per lane, 512 B per row per warp
        // instruction; full tiles run without per-row predicates, and warps whose
        // tile lies past row1 skip the sweep (a warp-uniform branch: no FMAs
        // issued).  j0, j1 and ld are multiples of 32, so a vector never crosses j1.
        constexpr int VE = 16 / (int)sizeof(T);
        using TV = typename Vec16<T>::type;
        auto sweep = [&](auto full) {
            constexpr bool kFull = decltype(full)::value;
            for (int jv = j0 + VE * lane; jv < j1; jv += 32 * VE) {
                TV hv[kRT];
#pragma unroll
                for (int r = 0; r < kRT; ++r)
                    hv[r] = (kFull || r < nr) ? *reinterpret_cast<const TV *>(cols[r] + jv) : TV{};
#pragma unroll
                for (int u = 0; u < VE; ++u) {
                    T2 x[MG];
#pragma unroll
                    for (int c = 0; c < MG; ++c) x[c] = s_v[(jv - jw0 + u) * MG + c];
#pragma unroll
                    for (int r = 0; r < kRT; ++r) {
                        if (kFull || r < nr) {
                            const T h = lane_elem(hv[r], u);
#pragma unroll
                            for (int c = 0; c < MG; ++c) {
                                acc[(r * MG + c) * 2 + 0] = fma(h, x[c].x, acc[(r * MG + c) * 2 + 0]);
                                acc[(r * MG + c) * 2 + 1] = fma(h, x[c].y, acc[(r * MG + c) * 2 + 1]);
                            }
                        }
                    }
                }
            }
        };
        if (nr == kRT)
            sweep(std::true_type{});
        else if (nr > 0)
            sweep(std::false_type{});
        // warp sums -> shared memory, layout s_part[wj][wr][NV]
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            T tmp[NW];
#pragma unroll
            for (int q = 0; q < NW; ++q) tmp[q] = acc[b * NW + q];
            const T sm = warp_sums<T, NW>(tmp, lane);
            if (lane < NW) s_part[((size_t)wj * WR + wr) * NV + b * NW + lane] = sm;
        }
        __syncthreads();
        // epilogue: one thread per (row, column) of the super-tile, fixed-order sum over j slices
        for (int t = tid; t < WR * kRT * MG; t += kBlock) {
            const int wrr = t / (kRT * MG), rem = t % (kRT * MG);
            const int r = rem / MG, c = rem % MG;
            const int i = base + kRT * wrr + r;
            if (i >= row1) continue;
            T yr = T(0), yi = T(0);
            for (int w = 0; w < WJ; ++w) {
                yr += s_part[((size_t)w * WR + wrr) * NV + (r * MG + c) * 2 + 0];
                yi += s_part[((size_t)w * WR + wrr) * NV + (r * MG + c) * 2 + 1];
            }
            epi(i, c, yr, yi);
        }
        __syncthreads();
    }
}

// (a + b) + c rounded once for |c| far below ulp(a + b): TwoSum gives a + b = t + e
// exactly, then t + (e + c)
__device__ __forceinline__ float two_sum_plus(float a, float b, float c) {
    const float t = __fadd_rn(a, b);
    const float z = __fsub_rn(t, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(t, z)), __fsub_rn(b, z));
    return __fadd_rn(t, __fadd_rn(e, c));
}

// epilogue of one order: recurrence + FP64 accumulation of c_k v_k
template <typename T, int MG>
struct OrderEpi {
    using T2 = typename Vec2<T>::type;
    const T2 *vprev2;
    T2 *vout;
    double2 *acc;
    int k, m, g;
    double cre, cim;
    const T2 *vprev1;  // implicit operator: y -= shift v_{k-1}; nullptr for an explicit Hs
    T shift;
    // explicit FP32 Hs: the part of its diagonal that FP32 rounding dropped, added
    // back as y_i += dcorr_i v_{k-1,i} before v is rounded once (nullptr: none).
    // FP32 only, error-free: with (t, e) = TwoSum(2 y, -v_{k-2}), v = t + (e + 2 dcorr v_{k-1})
    // is 2 y + 2 dcorr v_{k-1} - v_{k-2} rounded once (the small terms are far below
    // t's ulp, so their own roundings do not reach the result)
    const float *dcorr;
    const T2 *vdiag;   // v_{k-1}
    __device__ void operator()(int i, int c, T yr, T yi) {
        if constexpr (std::is_same<T, float>::value) {
            if (dcorr) {
                const T2 p = ldcg2(vdiag + (size_t)i * MG + c);
                const float d = __ldg(dcorr + i);
                const float dr = __fmul_rn(d, p.x), di = __fmul_rn(d, p.y);
                T2 v;
                if (k == 1) {
                    v.x = __fadd_rn(yr, dr);
                    v.y = __fadd_rn(yi, di);
                } else {
                    const T2 w2 = ldcg2(vprev2 + (size_t)i * MG + c);
                    v.x = two_sum_plus(__fmul_rn(2.f, yr), -w2.x, __fmul_rn(2.f, dr));
                    v.y = two_sum_plus(__fmul_rn(2.f, yi), -w2.y, __fmul_rn(2.f, di));
                }
                vout[(size_t)i * MG + c] = v;
                const size_t ao = (size_t)i * m + g * MG + c;
                double2 a = acc[ao];
                const double vr = (double)v.x, vi = (double)v.y;
                a.x += cre * vr - cim * vi;
                a.y += cre * vi + cim * vr;
                acc[ao] = a;
                return;
            }
        }
        if (vprev1) {
            const T2 p = ldcg2(vprev1 + (size_t)i * MG + c);
            yr -= shift * p.x;
            yi -= shift * p.y;
        }
        T2 v;
        if (k == 1) {
            v.x = yr;
            v.y = yi;
        } else {
            const T2 w2 = ldcg2(vprev2 + (size_t)i * MG + c);
            v.x = T(2) * yr - w2.x;
            v.y = T(2) * yi - w2.y;
        }
        vout[(size_t)i * MG + c] = v;
        const size_t ao = (size_t)i * m + g * MG + c;
        double2 a = acc[ao];
        const double vr = (double)v.x, vi = (double)v.y;
        a.x += cre * vr - cim * vi;
        a.y += cre * vi + cim * vr;
        acc[ao] = a;
    }
};

// partial sums of a j window: s_y[(i - r0) * MG + c] += (yr, yi)
template <typename T, int MG>
struct AccEpi {
    typename Vec2<T>::type *s_y;
    int r0;
    __device__ void operator()(int i, int c, T yr, T yi) {
        auto &y = s_y[(size_t)(i - r0) * MG + c];
        y.x += yr;
        y.y += yi;
    }
};

// one order k >= 1 for the rows of segment sg, column group g (MG columns);
// jwin > 0: the previous vector is staged in windows of jwin rows
template <typename T, int MG>
__device__ void order_rows(const ChebProblem &pb, const ChebSegment &sg, int k, int g, int parity,
                           typename Vec2<T>::type *s_v, T *s_part, double cre, double cim, int jwin,
                           typename Vec2<T>::type *s_y) {
    using T2 = typename Vec2<T>::type;
    const int tid = threadIdx.x;
    const int ld = pb.ld, m = pb.m;
    T2 *vbuf = reinterpret_cast<T2 *>(pb.vbuf);
    const size_t gstride = (size_t)pb.ldv * MG;         // one column group
    const size_t bstride = gstride * (m / MG);          // one of the three vector buffers
    const T2 *vprev = vbuf + (size_t)((k + 2) % 3) * bstride + g * gstride;   // v_{k-1}
    OrderEpi<T, MG> epi{vbuf + (size_t)((k + 1) % 3) * bstride + g * gstride,
                        vbuf + (size_t)(k % 3) * bstride + g * gstride,
                        pb.col[parity ^ 1], k, m, g, cre, cim, nullptr, T(0), pb.dcorr, vprev};
    if (jwin == 0 || ld <= jwin) {  // the whole previous vector in shared memory
        __syncthreads();
        for (int q = tid; q < ld * MG; q += kBlock) s_v[q] = ldcg2(vprev + q);  // padding rows are zero
        __syncthreads();
        rows_gemv<T, MG, 0>(reinterpret_cast<const T *>(pb.H), ld, s_v, sg.row0, sg.row1, s_part, epi);
        return;
    }
    // A basis too large for the whole vector: stage it in windows of jwin rows;
    // each row's partial sums accumulate over the windows in shared memory (s_y,
    // one writer per entry per window), and the order's epilogue runs once after
    // the last window, in row blocks of kYRows.
    for (int r0 = sg.row0; r0 < sg.row1; r0 += kYRows) {
        const int r1 = min(sg.row1, r0 + kYRows);
        __syncthreads();
        for (int q = tid; q < (r1 - r0) * MG; q += kBlock) s_y[q] = T2{T(0), T(0)};
        for (int jw0 = 0; jw0 < ld; jw0 += jwin) {
            const int jw1 = min(ld, jw0 + jwin);
            __syncthreads();
            for (int q = tid; q < (jw1 - jw0) * MG; q += kBlock) s_v[q] = ldcg2(vprev + (size_t)jw0 * MG + q);
            __syncthreads();
            AccEpi<T, MG> acc_epi{s_y, r0};
            rows_gemv<T, MG, 0>(reinterpret_cast<const T *>(pb.H), ld, s_v, r0, r1, s_part, acc_epi, jw0, jw1);
        }
        __syncthreads();
        for (int q = tid; q < (r1 - r0) * MG; q += kBlock) epi(r0 + q / MG, q % MG, s_y[q].x, s_y[q].y);
    }
}

template <typename T, int MG>
struct StoreEpi {
    typename Vec2<T>::type *dst;  // one column group [ldv][MG]
    __device__ void operator()(int i, int c, T yr, T yi) {
        typename Vec2<T>::type v;
        v.x = yr;
        v.y = yi;
        dst[(size_t)i * MG + c] = v;
    }
};

// Phase ph of order k >= 1 of an implicit problem, column group g, over the
// CTA's segments [s0, s1): 0: w = G^T v_{k-1};  1: y = (h/b) w;
// 2: v_k from G y - shift v_{k-1} (recurrence + accumulation).  The staged
// vector is shared by all of the CTA's segments.
template <typename T, int MG>
__device__ void implicit_phase(const ChebLaunch &L, const ChebProblem &pb, int s0, int s1, int k, int ph, int g,
                               typename Vec2<T>::type *s_v, T *s_part, double cre, double cim) {
    using T2 = typename Vec2<T>::type;
    const int ld = pb.ld, m = pb.m;
    T2 *vbuf = reinterpret_cast<T2 *>(pb.vbuf);
    T2 *wb = reinterpret_cast<T2 *>(pb.wb);
    const size_t gstride = (size_t)pb.ldv * MG;
    const size_t bstride = gstride * (m / MG);
    const T2 *vprev = vbuf + (size_t)((k + 2) % 3) * bstride + g * gstride;  // v_{k-1}
    const T2 *src = ph == 0 ? vprev : wb + (size_t)(ph - 1) * bstride + g * gstride;
    const ChebSegment *segs = L.segs;
    if (ph == 1 && L.segs_full) {  // the full phase has its own even row split
        segs = L.segs_full;
        s0 = L.seg_full_begin[blockIdx.x];
        s1 = L.seg_full_begin[blockIdx.x + 1];
    }
    if (s0 >= s1) return;
    __syncthreads();
    for (int q = threadIdx.x; q < ld * MG; q += kBlock) s_v[q] = ldcg2(src + q);  // padding rows are zero
    __syncthreads();
    for (int s = s0; s < s1; ++s) {
        const ChebSegment sg = segs[s];
        if (ph == 0) {
            StoreEpi<T, MG> epi{wb + g * gstride};
            rows_gemv<T, MG, 1>(reinterpret_cast<const T *>(pb.G), ld, s_v, sg.row0, sg.row1, s_part, epi);
        } else if (ph == 1) {
            StoreEpi<T, MG> epi{wb + bstride + g * gstride};
            rows_gemv<T, MG, 0>(reinterpret_cast<const T *>(pb.H), ld, s_v, sg.row0, sg.row1, s_part, epi);
        } else {
            OrderEpi<T, MG> epi{vbuf + (size_t)((k + 1) % 3) * bstride + g * gstride,
                                vbuf + (size_t)(k % 3) * bstride + g * gstride,
                                pb.col[L.parity ^ 1], k, m, g, cre, cim, vprev, (T)pb.shift, nullptr, nullptr};
            rows_gemv<T, MG, 2>(reinterpret_cast<const T *>(pb.Gt), ld, s_v, sg.row0, sg.row1, s_part, epi);
        }
    }
}

// order 0: v_0 = s phi (rounded to T), acc = c_0 s phi (FP64); s = renormalisation factor
template <typename T, int MG>
__device__ void order_zero(const ChebProblem &pb, const ChebSegment &sg, int parity) {
    using T2 = typename Vec2<T>::type;
    T2 *v0 = reinterpret_cast<T2 *>(pb.vbuf);
    const int m = pb.m;
    const size_t gstride = (size_t)pb.ldv * MG;
    const double cre = pb.coef[0].x, cim = pb.coef[0].y;
    const double2 *phi = pb.col[parity];
    double2 *acc = pb.col[parity ^ 1];
    for (int q = threadIdx.x; q < (sg.row1 - sg.row0) * m; q += kBlock) {
        const int i = sg.row0 + q / m, col = q % m;
        const int g = col / MG, c = col % MG;
        const size_t o = (size_t)i * m + col;
        double2 p = phi[o];
        if (pb.scale) {
            const double sc = pb.scale[col % pb.P];
            p.x *= sc;
            p.y *= sc;
        }
        T2 v;
        v.x = (T)p.x;
        v.y = (T)p.y;
        v0[g * gstride + (size_t)i * MG + c] = v;
        acc[o] = make_double2(cre * p.x - cim * p.y, cre * p.y + cim * p.x);
    }
}

template <typename T, int MG>
__global__ void __launch_bounds__(kBlock, 1) cheb_kernel(ChebLaunch L) {
    using T2 = typename Vec2<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *s_part = reinterpret_cast<T *>(smem_raw);
    T2 *s_v = reinterpret_cast<T2 *>(smem_raw + kCheb_part_bytes);
    const int G = gridDim.x;
    const int s0 = L.seg_begin[blockIdx.x], s1 = L.seg_begin[blockIdx.x + 1];
    const unsigned long long bar_ns = L.barrier_ns ? L.barrier_ns : kBarrierNs;
    if ((int)blockIdx.x + 1 == L.exit_cta1) return;  // test hook: the other CTAs' barrier waits run out
    for (int k = 0; k <= L.kmax; ++k) {
        const int nph = k == 0 ? 1 : L.nphase;
        for (int ph = 0; ph < nph; ++ph) {
            if (L.nphase == 3) {  // one implicit problem
                const ChebProblem &pb = L.probs[0];
                if (k == 0) {
                    for (int s = s0; s < s1; ++s) order_zero<T, MG>(pb, L.segs[s], L.parity);
                } else if (k <= pb.K) {
                    const double cre = pb.coef[k].x, cim = pb.coef[k].y;
                    for (int g = 0; g < pb.m / MG; ++g)
                        implicit_phase<T, MG>(L, pb, s0, s1, k, ph, g, s_v, s_part, cre, cim);
                }
            } else {
                for (int s = s0; s < s1; ++s) {
                    const ChebSegment sg = L.segs[s];
                    const ChebProblem &pb = L.probs[sg.prob];
                    if (k > pb.K) continue;
                    if (k == 0) {
                        order_zero<T, MG>(pb, sg, L.parity);
                    } else {
                        const double cre = pb.coef[k].x, cim = pb.coef[k].y;
                        for (int g = 0; g < pb.m / MG; ++g)
                            order_rows<T, MG>(pb, sg, k, g, L.parity, s_v, s_part, cre, cim, L.jwin,
                                              s_v + (size_t)L.jwin * MG);
                    }
                }
            }
            if (!grid_barrier(L.bar_count, G, L.error, bar_ns)) return;
        }
    }
}

// ---- read-out: psi = L^-T phi (A = L^-1), bra = L chi (B = L^T), population partials
template <typename T, int MG>
struct ReadEpi {
    double2 *out;
    int P, c0;  // out column base
    __device__ void operator()(int i, int c, T yr, T yi) {
        out[(size_t)i * P + c0 + c] = make_double2((double)yr, (double)yi);
    }
};

template <typename T, int MG>
__global__ void __launch_bounds__(kBlock, 1) readout_kernel(ChebLaunch L) {
    using T2 = typename Vec2<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *s_part = reinterpret_cast<T *>(smem_raw);
    T2 *s_v = reinterpret_cast<T2 *>(smem_raw + kCheb_part_bytes);
    __shared__ double s_pop[kBlock];
    const int tid = threadIdx.x;
    const int s0 = L.seg_begin[blockIdx.x], s1 = L.seg_begin[blockIdx.x + 1];
    for (int s = s0; s < s1; ++s) {
        const ChebSegment sg = L.segs[s];
        const ChebProblem &pb = L.probs[sg.prob];
        if (!pb.A) continue;
        const int ld = pb.ld, m = pb.m, P = pb.P;
        const double2 *cols = pb.col[L.parity ^ 1];  // the step's propagated columns
        for (int pass = 0; pass < 2; ++pass) {       // 0: psi from ket columns, 1: bra
            const T *M = reinterpret_cast<const T *>(pass == 0 ? pb.A : pb.B);
            const int src0 = (pass == 1 && m == 2 * P) ? P : 0;
            double2 *out = pass == 0 ? pb.psi : pb.bra;
            for (int g = 0; g < P / MG; ++g) {
                __syncthreads();
                for (int q = tid; q < ld * MG; q += kBlock) {
                    const int j = q / MG, c = q % MG;
                    const double2 v = j < pb.N ? __ldcg(cols + (size_t)j * m + src0 + g * MG + c) : make_double2(0, 0);
                    T2 t;
                    t.x = (T)v.x;
                    t.y = (T)v.y;
                    s_v[q] = t;
                }
                __syncthreads();
                ReadEpi<T, MG> epi{out, P, g * MG};
                if (pass == 0)
                    rows_gemv<T, MG, 1>(M, ld, s_v, sg.row0, sg.row1, s_part, epi);  // A = L^-1: j >= i
                else
                    rows_gemv<T, MG, 2>(M, ld, s_v, sg.row0, sg.row1, s_part, epi);  // B = L^T: j <= i
            }
        }
        __syncthreads();
        // population partials of this segment: Re conj(psi_ip) bra_ip per (column, fragment)
        const int nf = min(pb.nfrag, kMaxFrag);
        double *dst = L.seg_pops + (size_t)s * kMaxCols * (kMaxFrag + 1);
        for (int p = 0; p < P; ++p) {
            for (int f = 0; f <= nf; ++f) {
                double a = 0.0;
                for (int i = sg.row0 + tid; i < sg.row1; i += kBlock) {
                    const bool in = (f == nf) || (pb.ao_frag && pb.ao_frag[i] == f);
                    if (in) {
                        const double2 x = pb.psi[(size_t)i * P + p], y = pb.bra[(size_t)i * P + p];
                        a += x.x * y.x + x.y * y.y;
                    }
                }
                s_pop[tid] = a;
                __syncthreads();
                for (int o = kBlock / 2; o > 0; o >>= 1) {
                    if (tid < o) s_pop[tid] += s_pop[tid + o];
                    __syncthreads();
                }
                if (tid == 0) dst[p * (kMaxFrag + 1) + f] = s_pop[0];
                __syncthreads();
            }
        }
    }
}

// one block per problem: sum its segments' partials in order -> populations of
// this step.  Reduced precision: the renormalisation factor s = sqrt(target /
// total) for the next step, with the total from the propagated columns in FP64
// (pb.ntot; a total from the read-out, whose matrices are in the launch
// precision, carries about 1e-7 of noise that renormalising every step would
// turn into a random walk of the norm), and the populations reported are those
// of the renormalised state the trajectory carries on with (each times s^2).
__global__ void reduce_pops_kernel(ChebLaunch L, int nprob) {
    const int q = blockIdx.x;
    if (q >= nprob) return;
    const ChebProblem &pb = L.probs[q];
    if (!pb.A) return;
    const int nf = min(pb.nfrag, kMaxFrag), P = pb.P;
    __shared__ double s2[kMaxCols];  // population factor s^2 per particle
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        double tot = 0.0;
        if (pb.ntot) {
            tot = pb.ntot[p];  // FP64 from the propagated columns, not the read-out in the launch precision
        } else {
            for (int s = L.prob_seg0[q]; s < L.prob_seg0[q + 1]; ++s)
                tot += L.seg_pops[(size_t)s * kMaxCols * (kMaxFrag + 1) + p * (kMaxFrag + 1) + nf];
        }
        const double tgt = pb.target ? pb.target[p] : 0.0;
        const bool rn = pb.scale_out && tot > 0.0 && tgt > 0.0;
        if (pb.scale_out) pb.scale_out[p] = rn ? sqrt(tgt / tot) : 1.0;
        s2[p] = rn ? tgt / tot : 1.0;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < P * (nf + 1); t += blockDim.x) {
        const int p = t / (nf + 1), f = t % (nf + 1);
        double a = 0.0;
        for (int s = L.prob_seg0[q]; s < L.prob_seg0[q + 1]; ++s)
            a += L.seg_pops[(size_t)s * kMaxCols * (kMaxFrag + 1) + p * (kMaxFrag + 1) + f];
        if (L.pops) L.pops[pb.pops_off + p * (pb.nfrag + 1) + (f == nf ? pb.nfrag : f)] = a * s2[p];
    }
}

// ============================ double-float (DF64) ================================
// GB300's FP64 pipe runs at 1/58 of its FP32 rate.  ELHL_PREC_DF64 keeps the
// operator and the series vectors as unevaluated sums hi + lo of two FP32
// numbers (48-bit significands, about 4e-15 relative) and evaluates the
// products on the FP32 pipes: Dekker's exact product error by FMA and Knuth's
// TwoSum for the running sums (df64.cuh).  Sums leave the row loop in FP64; the recurrence and
// the accumulation of c_k v_k are FP64 as in the other precisions.  Implicit
// operator only (G, h/b and G^T stored as float2 = (hi, lo)).

__device__ __forceinline__ float4 df_split2(double re, double im) {
    const float2 a = df_split(re), b = df_split(im);
    return make_float4(a.x, a.y, b.x, b.y);
}

// warp sums of NV FP32-pair values (NV = 4 ... 32), all on the FP32 pipe: plain
// butterflies over the lane bits >= log2(NV), then a transposed butterfly; lane l
// returns the warp sum of value l % NV
template <int NV>
__device__ __forceinline__ float2 df_warp_sums(float (&h)[NV], float (&l)[NV], int lane) {
#pragma unroll
    for (int o = 16; o >= NV; o >>= 1)
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const float oh = __shfl_xor_sync(0xffffffffu, h[i], o), ol = __shfl_xor_sync(0xffffffffu, l[i], o);
            df_add(h[i], l[i], oh, ol);
        }
#pragma unroll
    for (int o = NV / 2; o > 0; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const float sh = upper ? h[i] : h[i + o], sl = upper ? l[i] : l[i + o];
            float kh = upper ? h[i + o] : h[i], kl = upper ? l[i + o] : l[i];
            const float rh = __shfl_xor_sync(0xffffffffu, sh, o), rl = __shfl_xor_sync(0xffffffffu, sl, o);
            df_add(kh, kl, rh, rl);
            h[i] = kh;
            l[i] = kl;
        }
    }
    return make_float2(h[0], l[0]);
}

// rows_gemv for DF64: y_i = sum_j M(j, i) x_j, M float2 (hi, lo) column-major,
// x staged as float4 (re hi, re lo, im hi, im lo); calls epi(i, c, yr, yi) with
// FP64 sums.  Same tiling, triangular ranges and warp sums as rows_gemv.
template <int MG, int TRI, typename Epi>
__device__ void rows_gemv_df(const float2 *M, int ld, const float4 *s_v, int row0, int row1, float2 *s_part,
                             Epi &epi) {
    // rows per warp tile: 8 for one staged column (4 KB of matrix loads in flight per
    // warp), 4 for two or four (register budget of the hi/lo accumulators)
    constexpr int kRT = MG == 1 ? 8 : 4;
    constexpr int NV = kRT * MG * 2;      // sums per lane (16 ... 32)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rows = row1 - row0;
    int WR = 1;
    while (WR < kWarps && WR * kRT < rows) WR <<= 1;
    const int WJ = kWarps / WR;
    const int wr = warp / WJ, wj = warp % WJ;
    for (int base = row0; base < row1; base += kRT * WR) {
        const int tile_end = min(row1, base + kRT * WR);
        const int jlo = TRI == 1 ? (base & ~31) : 0;
        const int jhi = TRI == 2 ? min(ld, (tile_end + 31) & ~31) : ld;
        const int jchunk = ((jhi - jlo + WJ - 1) / WJ + 31) / 32 * 32;
        const int j0 = jlo + wj * jchunk, j1 = min(jhi, j0 + jchunk);
        const int r0 = base + kRT * wr;
        const int nr = min(kRT, row1 - r0);
        float ah[NV], al[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) ah[q] = al[q] = 0.f;
        const float2 *cols[kRT];
#pragma unroll
        for (int r = 0; r < kRT; ++r) cols[r] = M + (size_t)min(r0 + r, row1 - 1) * ld;
        // 16-byte loads: two (hi, lo) elements per lane, 512 B per row per warp instruction
        auto sweep = [&](auto full) {
            constexpr bool kFull = decltype(full)::value;
            for (int jv = j0 + 2 * lane; jv < j1; jv += 64) {
                float4 hv[kRT];
#pragma unroll
                for (int r = 0; r < kRT; ++r)
                    hv[r] = (kFull || r < nr) ? *reinterpret_cast<const float4 *>(cols[r] + jv)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    float4 x[MG];
#pragma unroll
                    for (int c = 0; c < MG; ++c) x[c] = s_v[(jv + u) * MG + c];
#pragma unroll
                    for (int r = 0; r < kRT; ++r) {
                        if (kFull || r < nr) {
                            const float hh = u ? hv[r].z : hv[r].x, hl = u ? hv[r].w : hv[r].y;
#pragma unroll
                            for (int c = 0; c < MG; ++c) {
                                const int k = (r * MG + c) * 2;
                                df_fma(ah[k], al[k], hh, hl, x[c].x, x[c].y);
                                df_fma(ah[k + 1], al[k + 1], hh, hl, x[c].z, x[c].w);
                            }
                        }
                    }
                }
            }
        };
        if (nr == kRT)
            sweep(std::true_type{});
        else if (nr > 0)
            sweep(std::false_type{});
        // warp sums in FP32 pairs (no FP64 instruction in the tile), then the
        // fixed-order sum over the WJ slices; FP64 only for the tile's outputs
        constexpr int NW = NV < 32 ? NV : 32;
#pragma unroll
        for (int b = 0; b < NV / NW; ++b) {
            float th[NW], tl[NW];
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                th[q] = ah[b * NW + q];
                tl[q] = al[b * NW + q];
            }
            const float2 sm = df_warp_sums<NW>(th, tl, lane);
            if (lane < NW) s_part[((size_t)wj * WR + wr) * NV + b * NW + lane] = sm;
        }
        __syncthreads();
        for (int t = tid; t < WR * kRT * MG; t += kBlock) {
            const int wrr = t / (kRT * MG), rem = t % (kRT * MG);
            const int r = rem / MG, c = rem % MG;
            const int i = base + kRT * wrr + r;
            if (i >= row1) continue;
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int w = 0; w < WJ; ++w) {
                const float2 a = s_part[((size_t)w * WR + wrr) * NV + (r * MG + c) * 2 + 0];
                const float2 b = s_part[((size_t)w * WR + wrr) * NV + (r * MG + c) * 2 + 1];
                df_add(rh, rl, a.x, a.y);
                df_add(ih, il, b.x, b.y);
            }
            epi(i, c, (double)rh + (double)rl, (double)ih + (double)il);
        }
        __syncthreads();
    }
}

template <int MG>
struct StoreEpiDF {
    float4 *dst;
    __device__ void operator()(int i, int c, double yr, double yi) { dst[(size_t)i * MG + c] = df_split2(yr, yi); }
};

// recurrence in FP64: y -= shift v_{k-1}; v_k = 2 y - v_{k-2} (v_1 = y), stored as
// DF64; acc += c_k v_k
template <int MG>
struct OrderEpiDF {
    const float4 *vprev2;
    float4 *vout;
    double2 *acc;
    int k, m, g;
    double cre, cim;
    const float4 *vprev1;
    double shift;
    __device__ void operator()(int i, int c, double yr, double yi) {
        const float4 p = __ldcg(vprev1 + (size_t)i * MG + c);
        yr -= shift * ((double)p.x + (double)p.y);
        yi -= shift * ((double)p.z + (double)p.w);
        double vr = yr, vi = yi;
        if (k > 1) {
            const float4 w = __ldcg(vprev2 + (size_t)i * MG + c);
            vr = 2.0 * yr - ((double)w.x + (double)w.y);
            vi = 2.0 * yi - ((double)w.z + (double)w.w);
        }
        vout[(size_t)i * MG + c] = df_split2(vr, vi);
        const size_t ao = (size_t)i * m + g * MG + c;
        double2 a = acc[ao];
        a.x += cre * vr - cim * vi;
        a.y += cre * vi + cim * vr;
        acc[ao] = a;
    }
};

template <int MG>
__device__ void order_zero_df(const ChebProblem &pb, const ChebSegment &sg, int parity) {
    float4 *v0 = reinterpret_cast<float4 *>(pb.vbuf);
    const int m = pb.m;
    const size_t gstride = (size_t)pb.ldv * MG;
    const double cre = pb.coef[0].x, cim = pb.coef[0].y;
    const double2 *phi = pb.col[parity];
    double2 *acc = pb.col[parity ^ 1];
    for (int q = threadIdx.x; q < (sg.row1 - sg.row0) * m; q += kBlock) {
        const int i = sg.row0 + q / m, col = q % m;
        const int g = col / MG, c = col % MG;
        const size_t o = (size_t)i * m + col;
        double2 p = phi[o];
        if (pb.scale) {
            const double sc = pb.scale[col % pb.P];
            p.x *= sc;
            p.y *= sc;
        }
        v0[g * gstride + (size_t)i * MG + c] = df_split2(p.x, p.y);
        acc[o] = make_double2(cre * p.x - cim * p.y, cre * p.y + cim * p.x);
    }
}

template <int MG>
__device__ void implicit_phase_df(const ChebLaunch &L, const ChebProblem &pb, int s0, int s1, int k, int ph, int g,
                                  float4 *s_v, float2 *s_part, double cre, double cim) {
    const int ld = pb.ld, m = pb.m;
    float4 *vbuf = reinterpret_cast<float4 *>(pb.vbuf);
    float4 *wb = reinterpret_cast<float4 *>(pb.wb);
    const size_t gstride = (size_t)pb.ldv * MG;
    const size_t bstride = gstride * (m / MG);
    const float4 *vprev = vbuf + (size_t)((k + 2) % 3) * bstride + g * gstride;
    const float4 *src = ph == 0 ? vprev : wb + (size_t)(ph - 1) * bstride + g * gstride;
    const ChebSegment *segs = L.segs;
    if (ph == 1 && L.segs_full) {  // the full phase has its own even row split
        segs = L.segs_full;
        s0 = L.seg_full_begin[blockIdx.x];
        s1 = L.seg_full_begin[blockIdx.x + 1];
    }
    if (s0 >= s1) return;
    __syncthreads();
    for (int q = threadIdx.x; q < ld * MG; q += kBlock) s_v[q] = __ldcg(src + q);
    __syncthreads();
    for (int s = s0; s < s1; ++s) {
        const ChebSegment sg = segs[s];
        if (ph == 0) {
            StoreEpiDF<MG> epi{wb + g * gstride};
            rows_gemv_df<MG, 1>(reinterpret_cast<const float2 *>(pb.G), ld, s_v, sg.row0, sg.row1, s_part, epi);
        } else if (ph == 1) {
            StoreEpiDF<MG> epi{wb + bstride + g * gstride};
            rows_gemv_df<MG, 0>(reinterpret_cast<const float2 *>(pb.H), ld, s_v, sg.row0, sg.row1, s_part, epi);
        } else {
            OrderEpiDF<MG> epi{vbuf + (size_t)((k + 1) % 3) * bstride + g * gstride,
                               vbuf + (size_t)(k % 3) * bstride + g * gstride,
                               pb.col[L.parity ^ 1], k, m, g, cre, cim, vprev, pb.shift};
            rows_gemv_df<MG, 2>(reinterpret_cast<const float2 *>(pb.Gt), ld, s_v, sg.row0, sg.row1, s_part, epi);
        }
    }
}

// one launch per step, implicit operator (one problem, three phases per order)
template <int MG>
__global__ void __launch_bounds__(kBlock, 1) cheb_df_kernel(ChebLaunch L) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *s_part = reinterpret_cast<float2 *>(smem_raw);
    float4 *s_v = reinterpret_cast<float4 *>(smem_raw + kCheb_part_bytes);
    const int G = gridDim.x;
    const int s0 = L.seg_begin[blockIdx.x], s1 = L.seg_begin[blockIdx.x + 1];
    const ChebProblem &pb = L.probs[0];
    const unsigned long long bar_ns = L.barrier_ns ? L.barrier_ns : kBarrierNs;
    if ((int)blockIdx.x + 1 == L.exit_cta1) return;  // test hook: the other CTAs' barrier waits run out
    for (int k = 0; k <= L.kmax; ++k) {
        const int nph = k == 0 ? 1 : 3;
        for (int ph = 0; ph < nph; ++ph) {
            if (k == 0) {
                for (int s = s0; s < s1; ++s) order_zero_df<MG>(pb, L.segs[s], L.parity);
            } else if (k <= pb.K) {
                const double cre = pb.coef[k].x, cim = pb.coef[k].y;
                for (int g = 0; g < pb.m / MG; ++g)
                    implicit_phase_df<MG>(L, pb, s0, s1, k, ph, g, s_v, s_part, cre, cim);
            }
            if (!grid_barrier(L.bar_count, G, L.error, bar_ns)) return;
        }
    }
}

template <int MG>
cudaError_t launch_df(const ChebLaunch &L, cudaStream_t st) {
    if (L.nphase != 3) return cudaErrorInvalidValue;  // implicit operator only
    auto kern = cheb_df_kernel<MG>;
    const size_t smem = kCheb_part_bytes + (size_t)L.max_ld * MG * sizeof(float4);
    if (smem > kCheb_smem_limit) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    ChebLaunch copy = L;
    void *args[] = {&copy};
    e = cudaLaunchCooperativeKernel((const void *)kern, dim3(L.grid), dim3(kBlock), args, smem, st);
    count_launch();
    return e;
}

template <typename T, int MG>
cudaError_t launch_t(const ChebLaunch &L, cudaStream_t st) {
    auto kern = cheb_kernel<T, MG>;
    constexpr size_t c2 = sizeof(typename Vec2<T>::type);
    size_t smem = kCheb_part_bytes + (size_t)L.max_ld * MG * c2;
    ChebLaunch copy = L;
    copy.jwin = 0;
    if (smem > kCheb_smem_limit && L.nphase == 1) {  // explicit Hs: stage the vector in windows
        const size_t ybytes = (size_t)kYRows * MG * c2;
        copy.jwin = (int)(((kCheb_smem_limit - kCheb_part_bytes - ybytes) / (MG * c2)) & ~(size_t)31);
        smem = kCheb_part_bytes + (size_t)copy.jwin * MG * c2 + ybytes;
    }
    if (smem > kCheb_smem_limit) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void *args[] = {&copy};
    e = cudaLaunchCooperativeKernel((const void *)kern, dim3(L.grid), dim3(kBlock), args, smem, st);
    count_launch();
    return e;
}

template <typename T, int MG>
cudaError_t launch_readout_t(const ChebLaunch &L, int nprob, cudaStream_t st) {
    auto kern = readout_kernel<T, MG>;
    const size_t smem = kCheb_part_bytes + (size_t)L.max_ld * MG * sizeof(typename Vec2<T>::type);
    if (smem > kCheb_smem_limit) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<L.grid, kBlock, smem, st>>>(L);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce_pops_kernel<<<nprob, 128, 0, st>>>(L, nprob);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_readout(const ChebLaunch &L, int nprob, int precision, int mg, cudaStream_t st) {
    if (precision == ELHL_PREC_FP64) {
        switch (mg) {
            case 1: return launch_readout_t<double, 1>(L, nprob, st);
            case 2: return launch_readout_t<double, 2>(L, nprob, st);
            case 4: return launch_readout_t<double, 4>(L, nprob, st);
        }
    } else {
        switch (mg) {
            case 1: return launch_readout_t<float, 1>(L, nprob, st);
            case 2: return launch_readout_t<float, 2>(L, nprob, st);
            case 4: return launch_readout_t<float, 4>(L, nprob, st);
        }
    }
    return cudaErrorInvalidValue;
}

int cheb_block() { return kBlock; }

int cheb_group_size(int precision, int m, int max_ld, bool windowed) {
    // the largest of 4, 2, 1 staged columns that divides m and fits in shared
    // memory (windowed: the explicit propagation stages the vector in windows)
    const size_t c2 = (precision == ELHL_PREC_FP64 || precision == ELHL_PREC_DF64) ? sizeof(double2) : sizeof(float2);
    for (int mg : {4, 2, 1})
        if (m % mg == 0 && (windowed || kCheb_part_bytes + (size_t)max_ld * mg * c2 <= kCheb_smem_limit)) return mg;
    return 0;
}

cudaError_t launch_cheb(const ChebLaunch &L, int precision, int mg, cudaStream_t st) {
    if (precision == ELHL_PREC_DF64) {
        switch (mg) {
            case 1: return launch_df<1>(L, st);
            case 2: return launch_df<2>(L, st);
            case 4: return launch_df<4>(L, st);
        }
        return cudaErrorInvalidValue;
    }
    if (precision == ELHL_PREC_FP64) {
        switch (mg) {
            case 1: return launch_t<double, 1>(L, st);
            case 2: return launch_t<double, 2>(L, st);
            case 4: return launch_t<double, 4>(L, st);
        }
    } else {
        switch (mg) {
            case 1: return launch_t<float, 1>(L, st);
            case 2: return launch_t<float, 2>(L, st);
            case 4: return launch_t<float, 4>(L, st);
        }
    }
    return cudaErrorInvalidValue;
}

int cheb_grid_size(int *grid_out) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    *grid_out = sms;
    return 0;
}

}  // namespace elhl
