// Persistent FP64 engine for the reference's adaptive-tau Taylor propagator.
//
// Semantics follow Taylor.f:35-239 (Propagation, Convergence, coefficient,
// isConverged) with bra propagated by H'^T and ket by H' (bra_x_op / op_x_ket,
// Matrix_math.f:225-301), for one or two particles (electron, hole) at once.
// In multi-step mode the kernel also runs the step driver of ElHl_Chebyshev
// (ElHl_Chebyshev.f:174-187, :267) for fixed nuclei and records populations
// (pop_Slater, data_output.f:242-262) after every step.
//
// Execution model: one cooperative launch, one CTA per SM.  Each CTA owns a
// contiguous block of rows; one "round" = one expansion order for every
// active particle:
//   phase A  each CTA computes its rows of H'^T.bra and H'.ket (H' read from
//            L2/HBM), the epilogue forms the scaled term, the partial sum and
//            per-CTA partials (max |delta|, <bra|ket>, populations);
//   barrier  bounded grid barrier (gives up after kBarrierNs and reports
//            ELHL_ERR_TIMEOUT instead of hanging);
//   phase B  every CTA reduces the per-CTA partials in the same fixed order and
//            advances an identical copy of the per-particle state machine, so
//            all CTAs take the same branch with no host round trip.
// Vectors live in kSlots slots per particle; "Psi = new" and the term/partial-
// sum rotation are slot renames, never copies.
#include <cooperative_groups.h>

#include "elhl_internal.cuh"
#include "grid_sync.cuh"

namespace elhl {
namespace {

constexpr int RC = 4;            // rows per register chunk
constexpr int PMAX = 2;          // particles per launch
constexpr int PW = 16;           // partial record width (doubles)

enum Phase { PH_NORM = 0, PH_CONV = 1, PH_MAIN = 2, PH_DONE = 3 };

struct Ctrl {
    int phase, first, k, kmax;
    int psi, src, old, out_term, out_acc;
    int conv_calls, conv_step, substeps, status;
    long long orders;
    double tau, t, norm_ref, save_tau;
    double cre[kOrder], cim[kOrder];
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// coefficient(tau): c_1 = 1, c_k = -i c_{k-1} tau/(k-1) (Taylor.f:224-239), 0-based storage
__device__ void set_coefficients(Ctrl &c) {
    c.cre[0] = 1.0;
    c.cim[0] = 0.0;
    for (int k = 1; k < kOrder; ++k) {
        const double f = c.tau / k;
        c.cre[k] = c.cim[k - 1] * f;
        c.cim[k] = -c.cre[k - 1] * f;
    }
}

__device__ void pick_out_slots(Ctrl &c) {
    int found = 0;
    for (int s = 0; s < kSlots && found < 2; ++s) {
        if (s == c.psi || s == c.src || s == c.old) continue;
        if (found == 0) c.out_term = s; else c.out_acc = s;
        ++found;
    }
}

__device__ void start_conv(Ctrl &c, int max_calls) {
    if (c.conv_step >= max_calls) {
        c.status = ELHL_ERR_NO_CONVERGENCE;
        c.phase = PH_DONE;
        return;
    }
    c.conv_calls++;
    c.conv_step++;
    set_coefficients(c);
    c.kmax = kOrder;  // 1-based: first k >= 2 with |c_k| < 1e-16 (Taylor.f:165-171)
    for (int k = 2; k <= kOrder; ++k)
        if (hypot(c.cre[k - 1], c.cim[k - 1]) < 1.0e-16) {
            c.kmax = k;
            break;
        }
    c.src = c.psi;
    c.old = c.psi;
    c.k = 2;
    c.phase = PH_CONV;
    pick_out_slots(c);
}

__device__ void start_main(Ctrl &c) {
    c.src = c.psi;
    c.old = c.psi;
    c.k = 2;
    c.phase = PH_MAIN;
    pick_out_slots(c);
}

// After an accepted convergence sub-step (Taylor.f:71-78 first time, :116-121 later).
__device__ void after_accept(Ctrl &c, double t_init, double t_max) {
    c.substeps++;
    if (c.first) {
        c.save_tau = c.tau;
        c.t = t_init + c.tau * kHbar;
        c.first = 0;
    } else {
        c.t = c.t + (c.tau * kHbar);
    }
    if (t_max - c.t < c.tau * kHbar) {
        c.tau = (t_max - c.t) / kHbar;
        set_coefficients(c);
    }
    if (c.t < t_max) start_main(c); else c.phase = PH_DONE;
}

__global__ void __launch_bounds__(kTaylorBlock, 1) taylor_kernel(TaylorLaunch L) {
    __shared__ Ctrl ctrl[PMAX];
    __shared__ double red[kTaylorBlock / 32][PMAX * RC * 4];
    __shared__ double part[PMAX][RC][4];   // per (particle, chunk row) running partials
    __shared__ double cta_rec[PMAX][PW];
    __shared__ int s_step, s_it;
    __shared__ double s_tinit, s_tmax;

    const int G = gridDim.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int N = L.N, ld = L.ld, ldv = L.ldv, P = L.nparticles;
    const int rows = (N + G - 1) / G;
    const int r0 = min(N, blockIdx.x * rows), r1 = min(N, r0 + rows);
    const int nf = L.nfrag < kMaxFrag ? L.nfrag : kMaxFrag;

    auto vec = [&](int p, int slot, int which) -> double2 * {
        return L.slots + ((size_t)(p * kSlots + slot) * 2 + which) * ldv;
    };

    if (tid == 0) {
        s_step = 0;
        s_it = L.it0;
        s_tinit = L.t_init;
        s_tmax = L.t_max;
        for (int p = 0; p < P; ++p) {
            Ctrl &c = ctrl[p];
            c.phase = PH_NORM;
            c.first = 1;
            c.psi = 0; c.src = 0; c.old = 0; c.out_term = 1; c.out_acc = 2;
            c.conv_calls = 0; c.conv_step = 0; c.substeps = 0; c.status = ELHL_OK; c.orders = 0;
            c.tau = L.part[p].tau_in;
            c.t = L.t_init;
            c.save_tau = 0.0;
        }
    }
    __syncthreads();

    int parity = 0;
    for (;;) {
        // ------------------------------------------------ phase A
        bool any_gemv = false;
        for (int p = 0; p < P; ++p) any_gemv |= (ctrl[p].phase == PH_CONV || ctrl[p].phase == PH_MAIN);

        // norm / population partials on own rows (particles in PH_NORM)
        if (tid < PMAX * PW) (&cta_rec[0][0])[tid] = 0.0;
        __syncthreads();
        if (tid < P && ctrl[tid].phase == PH_NORM) {
            const int p = tid;
            const double2 *b = vec(p, ctrl[p].psi, 0), *k = vec(p, ctrl[p].psi, 1);
            double dre = 0.0, dim = 0.0, pops[kMaxFrag + 1];
            for (int f = 0; f <= kMaxFrag; ++f) pops[f] = 0.0;
            for (int i = r0; i < r1; ++i) {
                const double2 bi = __ldcg(b + i), ki = __ldcg(k + i);
                dre += bi.x * ki.x + bi.y * ki.y;  // conj(bra) ket
                dim += bi.x * ki.y - bi.y * ki.x;
                const double v = ki.x * bi.x + ki.y * bi.y;  // Re conj(ket) bra
                if (L.ao_frag) {
                    const int f = L.ao_frag[i];
                    if (f >= 0 && f < nf) pops[f] += v;
                }
                pops[kMaxFrag] += v;
            }
            cta_rec[p][2] = dre;
            cta_rec[p][3] = dim;
            for (int f = 0; f <= kMaxFrag; ++f) cta_rec[p][4 + f] = pops[f];
        }

        if (any_gemv) {
            if (tid < PMAX * RC * 4) (&part[0][0][0])[tid] = 0.0;
            __syncthreads();
            double2 rr[PMAX];
            bool act[PMAX];
            for (int p = 0; p < PMAX; ++p) {
                act[p] = p < P && (ctrl[p].phase == PH_CONV || ctrl[p].phase == PH_MAIN);
                if (act[p]) {
                    const Ctrl &c = ctrl[p];
                    // r = c_k / c_{k-1} (Taylor.f:93); both pure real or pure imaginary multiples
                    const double ar = c.cre[c.k - 1], ai = c.cim[c.k - 1];
                    const double br = c.cre[c.k - 2], bi = c.cim[c.k - 2];
                    const double d = br * br + bi * bi;
                    rr[p] = make_double2((ar * br + ai * bi) / d, (ai * br - ar * bi) / d);
                }
            }
            for (int c0 = r0; c0 < r1; c0 += RC) {
                const int nr = min(RC, r1 - c0);
                double acc[PMAX][RC][4];
#pragma unroll
                for (int p = 0; p < PMAX; ++p)
#pragma unroll
                    for (int r = 0; r < RC; ++r)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[p][r][q] = 0.0;
                const double2 *xb[PMAX], *xk[PMAX];
                for (int p = 0; p < PMAX; ++p) {
                    xb[p] = act[p] ? vec(p, ctrl[p].src, 0) : nullptr;
                    xk[p] = act[p] ? vec(p, ctrl[p].src, 1) : nullptr;
                }
                for (int j = tid; j < N; j += kTaylorBlock) {
                    double hk[RC], hb[RC];
#pragma unroll
                    for (int r = 0; r < RC; ++r) {
                        const int i = c0 + (r < nr ? r : 0);
                        hk[r] = L.H[(size_t)j * ld + i];   // H'(i, j): row block (ket)
                        hb[r] = L.H[(size_t)i * ld + j];   // H'(j, i): column block (bra, H'^T)
                    }
#pragma unroll
                    for (int p = 0; p < PMAX; ++p) {
                        if (!act[p]) continue;
                        // vectors written by other CTAs: L2 loads (L1 is not coherent across SMs)
                        const double2 vk = __ldcg(xk[p] + j), vb = __ldcg(xb[p] + j);
#pragma unroll
                        for (int r = 0; r < RC; ++r) {
                            acc[p][r][0] = fma(hk[r], vk.x, acc[p][r][0]);
                            acc[p][r][1] = fma(hk[r], vk.y, acc[p][r][1]);
                            acc[p][r][2] = fma(hb[r], vb.x, acc[p][r][2]);
                            acc[p][r][3] = fma(hb[r], vb.y, acc[p][r][3]);
                        }
                    }
                }
                // block reduction of the 32 accumulators: transposed butterfly, after
                // which lane l holds the warp sum of accumulator l (31 shuffles + adds
                // per lane instead of 5 per accumulator), then a fixed-order sum over warps
                static_assert(PMAX * RC * 4 == 32, "one accumulator per lane");
                double v[32];
#pragma unroll
                for (int p = 0; p < PMAX; ++p)
#pragma unroll
                    for (int r = 0; r < RC; ++r)
#pragma unroll
                        for (int q = 0; q < 4; ++q) v[(p * RC + r) * 4 + q] = acc[p][r][q];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const bool upper = (lane & o) != 0;
#pragma unroll
                    for (int i = 0; i < o; ++i) {
                        const double send = upper ? v[i] : v[i + o];
                        const double keep = upper ? v[i + o] : v[i];
                        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                    }
                }
                red[warp][lane] = v[0];
                __syncthreads();
                if (tid < PMAX * RC * 4) {
                    double v = 0.0;
                    for (int w = 0; w < kTaylorBlock / 32; ++w) v += red[w][tid];
                    red[0][tid] = v;  // safe: each tid reads column tid of all warps before writing row 0
                }
                __syncthreads();
                // epilogue: one thread per (particle, row)
                if (tid < PMAX * RC) {
                    const int p = tid / RC, r = tid % RC;
                    if (act[p] && r < nr) {
                        const Ctrl &c = ctrl[p];
                        const int i = c0 + r;
                        const double2 yk = make_double2(red[0][(p * RC + r) * 4 + 0], red[0][(p * RC + r) * 4 + 1]);
                        const double2 yb = make_double2(red[0][(p * RC + r) * 4 + 2], red[0][(p * RC + r) * 4 + 3]);
                        const double2 tk = cmul(rr[p], yk), tb = cmul(rr[p], yb);
                        const double2 ok = __ldcg(vec(p, c.old, 1) + i), ob = __ldcg(vec(p, c.old, 0) + i);
                        const double2 nk = make_double2(ok.x + tk.x, ok.y + tk.y);
                        const double2 nb = make_double2(ob.x + tb.x, ob.y + tb.y);
                        vec(p, c.out_term, 1)[i] = tk;
                        vec(p, c.out_term, 0)[i] = tb;
                        vec(p, c.out_acc, 1)[i] = nk;
                        vec(p, c.out_acc, 0)[i] = nb;
                        const double db = hypot(nb.x - ob.x, nb.y - ob.y);
                        const double dk = hypot(nk.x - ok.x, nk.y - ok.y);
                        part[p][r][0] = fmax(part[p][r][0], db);
                        part[p][r][1] = fmax(part[p][r][1], dk);
                        part[p][r][2] += nb.x * nk.x + nb.y * nk.y;
                        part[p][r][3] += nb.x * nk.y - nb.y * nk.x;
                    }
                }
                __syncthreads();
            }
            if (tid < P && act[tid]) {
                const int p = tid;
                double mb = 0.0, mk = 0.0, dre = 0.0, dim = 0.0;
                for (int r = 0; r < RC; ++r) {
                    mb = fmax(mb, part[p][r][0]);
                    mk = fmax(mk, part[p][r][1]);
                    dre += part[p][r][2];
                    dim += part[p][r][3];
                }
                cta_rec[p][0] = mb;
                cta_rec[p][1] = mk;
                cta_rec[p][2] = dre;
                cta_rec[p][3] = dim;
            }
        }
        __syncthreads();
        // publish this CTA's partial record
        if (tid < P * PW) {
            const int p = tid / PW, q = tid % PW;
            L.partials[(((size_t)parity * PMAX + p) * G + blockIdx.x) * PW + q] = cta_rec[p][q];
        }

        if (!grid_barrier(L.bar_count, G, L.error)) break;

        // ------------------------------------------------ phase B: reduce + advance
        // warp p reduces particle p's records in a fixed order (identical in every CTA)
        __shared__ double tot[PMAX][PW];
        if (warp < P) {
            // only the max |delta| and <bra|ket> fields matter after a GEMV round;
            // the population fields are read after a norm round only
            const int p = warp;
            const int nq = (ctrl[p].phase == PH_NORM) ? PW : 4;
            double v[PW];
#pragma unroll
            for (int q = 0; q < PW; ++q) v[q] = 0.0;
            for (int g = lane; g < G; g += 32) {
                const double *rec = L.partials + (((size_t)parity * PMAX + p) * G + g) * PW;
                v[0] = fmax(v[0], __ldcg(rec + 0));
                v[1] = fmax(v[1], __ldcg(rec + 1));
                v[2] += __ldcg(rec + 2);
                v[3] += __ldcg(rec + 3);
                for (int q = 4; q < nq; ++q) v[q] += __ldcg(rec + q);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                v[0] = fmax(v[0], __shfl_xor_sync(0xffffffffu, v[0], o));
                v[1] = fmax(v[1], __shfl_xor_sync(0xffffffffu, v[1], o));
                v[2] += __shfl_xor_sync(0xffffffffu, v[2], o);
                v[3] += __shfl_xor_sync(0xffffffffu, v[3], o);
            }
            if (nq > 4)
                for (int o = 16; o > 0; o >>= 1)
                    for (int q = 4; q < PW; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
            if (lane == 0)
                for (int q = 0; q < PW; ++q) tot[p][q] = v[q];
        }
        __syncthreads();
        parity ^= 1;

        if (tid == 0) {
            bool all_done = true;
            for (int p = 0; p < P; ++p) {
                Ctrl &c = ctrl[p];
                const double dotabs = hypot(tot[p][2], tot[p][3]);
                if (c.phase == PH_NORM) {
                    c.norm_ref = dotabs;  // Taylor.f:62
                    c.first = 1;
                    c.conv_step = 0;
                    start_conv(c, L.max_conv_calls);
                } else if (c.phase == PH_CONV) {
                    c.orders++;
                    const bool conv = !(tot[p][0] > L.tol) && !(tot[p][1] > L.tol) &&
                                      fabs(dotabs - c.norm_ref) < L.norm_tol;
                    if (conv) {
                        c.psi = c.out_acc;
                        after_accept(c, s_tinit, s_tmax);
                    } else {
                        c.old = c.out_acc;
                        c.src = c.out_term;
                        c.k++;
                        if (c.k > c.kmax) {
                            c.tau = c.tau * (c.first ? 0.9 : 0.975);  // Taylor.f:69, :110
                            start_conv(c, L.max_conv_calls);
                        } else {
                            pick_out_slots(c);
                        }
                    }
                } else if (c.phase == PH_MAIN) {
                    c.orders++;
                    if (c.k < c.kmax) {
                        c.old = c.out_acc;
                        c.src = c.out_term;
                        c.k++;
                        pick_out_slots(c);
                    } else if (fabs(dotabs - c.norm_ref) < L.norm_tol) {  // Taylor.f:103-106
                        c.psi = c.out_acc;
                        c.substeps++;
                        c.t = c.t + (c.tau * kHbar);
                        if (s_tmax - c.t < c.tau * kHbar) {
                            c.tau = (s_tmax - c.t) / kHbar;
                            set_coefficients(c);
                        }
                        if (c.t < s_tmax) start_main(c); else c.phase = PH_DONE;
                    } else {  // Taylor.f:107-114
                        c.tau = c.tau * 0.975;
                        start_conv(c, L.max_conv_calls);
                    }
                }
                if (c.phase != PH_DONE) all_done = false;
            }
            if (all_done) {
                // populations of the finished step come from a PH_NORM round on the
                // next step (or the final round below)
                s_step++;
            }
        }
        __syncthreads();

        bool all_done = true;
        for (int p = 0; p < P; ++p) all_done &= (ctrl[p].phase == PH_DONE);
        if (!all_done) continue;

        // ---- step finished for every particle: population round + step driver
        // population partials of the final Psi, one more barrier round
        if (tid < PMAX * PW) (&cta_rec[0][0])[tid] = 0.0;
        __syncthreads();
        if (tid < P) {
            const int p = tid;
            const double2 *b = vec(p, ctrl[p].psi, 0), *k = vec(p, ctrl[p].psi, 1);
            double pops[kMaxFrag + 1];
            for (int f = 0; f <= kMaxFrag; ++f) pops[f] = 0.0;
            for (int i = r0; i < r1; ++i) {
                const double2 bi = __ldcg(b + i), ki = __ldcg(k + i);
                const double v = ki.x * bi.x + ki.y * bi.y;
                if (L.ao_frag) {
                    const int f = L.ao_frag[i];
                    if (f >= 0 && f < nf) pops[f] += v;
                }
                pops[kMaxFrag] += v;
            }
            for (int f = 0; f <= kMaxFrag; ++f) cta_rec[p][4 + f] = pops[f];
        }
        __syncthreads();
        if (tid < P * PW) {
            const int p = tid / PW, q = tid % PW;
            L.partials[(((size_t)parity * PMAX + p) * G + blockIdx.x) * PW + q] = cta_rec[p][q];
        }
        if (!grid_barrier(L.bar_count, G, L.error)) break;
        if (warp < P) {
            const int p = warp;
            double v[kMaxFrag + 1];
            for (int f = 0; f <= kMaxFrag; ++f) v[f] = 0.0;
            for (int g = lane; g < G; g += 32) {
                const double *rec = L.partials + (((size_t)parity * PMAX + p) * G + g) * PW;
                for (int f = 0; f <= kMaxFrag; ++f) v[f] += __ldcg(rec + 4 + f);
            }
            for (int o = 16; o > 0; o >>= 1)
                for (int f = 0; f <= kMaxFrag; ++f) v[f] += __shfl_xor_sync(0xffffffffu, v[f], o);
            if (lane == 0) {
                for (int f = 0; f <= kMaxFrag; ++f) tot[p][4 + f] = v[f];
            }
        }
        __syncthreads();
        parity ^= 1;
        const int step_done = s_step - 1;
        if (blockIdx.x == 0 && tid < P && L.pops && step_done < L.nsteps) {
            const int p = tid;
            double *dst = L.pops + ((size_t)step_done * P + p) * (L.nfrag + 1);
            for (int f = 0; f < nf; ++f) dst[f] = tot[p][4 + f];
            dst[L.nfrag] = tot[p][4 + kMaxFrag];
        }
        bool failed = false;
        for (int p = 0; p < P; ++p) failed |= (ctrl[p].status != ELHL_OK);
        if (s_step >= L.nsteps || failed) break;
        __syncthreads();
        if (tid == 0) {
            // next nuclear step (ElHl_Chebyshev.f:174-187, :267): t_init = t, t_max = dt*fs*(it-1)
            s_it++;
            s_tinit = s_tinit + L.dt_frame;
            s_tmax = L.dt_frame * (double)(s_it - 1);
            // first_call_ is already false after the launch's first step
            for (int p = 0; p < P; ++p) {
                Ctrl &c = ctrl[p];
                const double tau = c.save_tau * 1.15;
                c.tau = tau > L.tau_max ? L.tau_max : tau;
                c.t = s_tinit;
                c.phase = PH_NORM;
            }
        }
        __syncthreads();
    }

    // ------------------------------------------------ write-out: final Psi into slot 0
    // (own rows only; no other CTA touches them after the last barrier)
    __syncthreads();
    for (int p = 0; p < P; ++p) {
        const Ctrl &c = ctrl[p];
        if (c.psi == 0) continue;
        const double2 *b = vec(p, c.psi, 0), *k = vec(p, c.psi, 1);
        double2 *b0 = vec(p, 0, 0), *k0 = vec(p, 0, 1);
        for (int i = r0 + tid; i < r1; i += kTaylorBlock) {
            b0[i] = __ldcg(b + i);
            k0[i] = __ldcg(k + i);
        }
    }
    if (blockIdx.x == 0 && tid < P) {
        const Ctrl &c = ctrl[tid];
        TaylorParticle &o = L.part[tid];
        o.save_tau = c.save_tau;
        o.tau_out = c.tau;
        o.orders = c.orders;
        o.conv_calls = c.conv_calls;
        o.substeps = c.substeps;
        o.status = c.status;
        o.psi_slot = c.psi;
        if (tid == 0 && L.t_final) {
            // time after the last completed step (the driver's t)
            *L.t_final = s_tinit + L.dt_frame;
        }
    }
}

}  // namespace

int taylor_grid_size(int block, int *grid_out) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, taylor_kernel, block, 0) != cudaSuccess) return -1;
    if (per_sm < 1) return -1;
    *grid_out = sms;  // one CTA per SM
    return 0;
}

cudaError_t launch_taylor(const TaylorLaunch &L, int grid, int block, cudaStream_t st) {
    TaylorLaunch copy = L;
    void *args[] = {&copy};
    const cudaError_t e = cudaLaunchCooperativeKernel((const void *)taylor_kernel, dim3(grid), dim3(block), args, 0, st);
    count_launch();
    return e;
}

}  // namespace elhl
