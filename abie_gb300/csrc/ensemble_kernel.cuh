// The batched Radau15 kernel (one system per group of W warps), shared by
// ensemble.cu (exact, fast FP64 and mixed forms) and ensemble_plain.cu (the
// plain FP64 form, compiled with FMA contraction).  The host side that
// schedules the launches lives in ensemble.cu.
#pragma once
#include "abi_state.cuh"
#include "ensemble.cuh"
#include "mlp.cuh"
#include "radau_comp.cuh"

namespace abie {

static constexpr int ENS_MAX_BODIES = 21;  // 3N <= 64: one component per thread of two warps
static constexpr int WARPS = 4;            // warps per block
static constexpr int STATE_PER_COMP = 18;  // y0 dy0 F1 b[7] g[7] b6p

struct EnsScalars {
    double t, h;
    int loop_count, phase;  // phase 0: fresh, 1: running, 2: done
    long long steps, attempts, iterations, force_calls;
    int status;
    int fallbacks;  // attempts redone from the plain guess after the network's guess failed
};

struct EnsArgs {
    const long long *offsets;
    const double *m;
    double *pos, *vel;  // packed 3*total, updated at the end
    double *state;      // STATE_PER_COMP * 3 * total
    EnsScalars *sc;     // per system
    const int *active;  // systems to run in this launch
    int n_active;
    int *queue;
    double G, t_end;
    unsigned long long budget_ns;    // a warp yields once this long after the launch began
    const LearnedPredictor *mlp;     // device view of the learned predictor; null: plain predictor
    float *samples;                  // training-sample store (null: no collection)
    long long sample_cap;
    unsigned long long *sample_count;
    float tau[7];                    // output scales of the learned predictor's targets
    int consistent_g;                // set g = C^-1 b after the guess (learned or plain)
};

// Per-warp shared buffers of the learned predictor (systems of at most 16 bodies).
constexpr int LP_ROWS = 16;
struct LearnSmem {
    float row[LP_ROWS][MLP_OUT_PAD];                     // staging; later the network output
    __nv_bfloat16 xh2[LP_ROWS][MLP_HID + 8];             // features (ld 40), then H2 (ld 136)
    __nv_bfloat16 h1[LP_ROWS][MLP_HID + 8];
    float pfeat[LP_ROWS][MLP_FEAT];                      // features of the pending sample
    float pE[LP_ROWS][MLP_OUT];                          // plain guess / scale of the pending sample
    float ps[LP_ROWS][7];                                // per-order scales of the pending sample
    float scale[LP_ROWS][7];                             // per-order scales of this step
    double plain[3 * LP_ROWS][8];                        // plain guess b and b6p, kept while the network's is tried
};

// Network outputs for LP_ROWS rows of features (bf16, ld 40, in xh2) into
// row[][] (fp32).  One warp; weights from global memory.
static __device__ __noinline__ void mlp_warp_forward(const LearnedPredictor *P, LearnSmem &L)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const __nv_bfloat16 *W1 = P->W1, *W2 = P->W2, *W3 = P->W3;
    const float *b1 = P->b1, *b2 = P->b2, *b3 = P->b3;
    const __nv_bfloat16 *X = &L.xh2[0][0];
    for (int n0 = 0; n0 < MLP_HID; n0 += 8) {
        float c[4];
        mma_tile(X, 40, W1, MLP_IN, 0, n0, MLP_IN, c);
        for (int e = 0; e < 4; e++) {
            int r = g + (e >> 1) * 8, n = n0 + 2 * t + (e & 1);
            L.h1[r][n] = __float2bfloat16_rn(fmaxf(c[e] + b1[n], 0.0f));
        }
    }
    __syncwarp();
    __nv_bfloat16 *H2 = &L.xh2[0][0];  // features are dead now
    for (int n0 = 0; n0 < MLP_HID; n0 += 8) {
        float c[4];
        mma_tile(&L.h1[0][0], MLP_HID + 8, W2, MLP_HID, 0, n0, MLP_HID, c);
        __syncwarp();  // every lane has read its A fragments of this tile before H2 overwrites
        for (int e = 0; e < 4; e++) {
            int r = g + (e >> 1) * 8, n = n0 + 2 * t + (e & 1);
            H2[r * (MLP_HID + 8) + n] = __float2bfloat16_rn(fmaxf(c[e] + b2[n], 0.0f));
        }
    }
    __syncwarp();
    for (int n0 = 0; n0 < MLP_OUT_PAD; n0 += 8) {
        float c[4];
        mma_tile(H2, MLP_HID + 8, W3, MLP_HID, 0, n0, MLP_HID, c);
        for (int e = 0; e < 4; e++) {
            int r = g + (e >> 1) * 8, n = n0 + 2 * t + (e & 1);
            L.row[r][n] = c[e] + b3[n];
        }
    }
    __syncwarp();
}

// At an accepted step (not the last): emit the pending training sample
// when this step was reached by a single attempt after the previous accept,
// then replace refine_bs's plain guess E_k by E_k + s_k tau_k out_k (network
// output) when a network is active, and remember this step's features and
// E.  Scales s_k are per coefficient order: the largest |b_k| of the body.
template <int W>
__device__ __forceinline__ void learned_refine(const EnsArgs &a, LearnSmem &L, Group<W> &grp,
                                               Comp &X, int n, bool has, double q, double h,
                                               double dtreq, const double *m, bool &pend_valid,
                                               bool first_attempt, bool &net_guess,
                                               bool make_consistent)
{
    constexpr int GS = 32 * W;
    const int gl = grp.gl;
    double h_next = (dtreq / h > 1.0 / FAC) ? h / FAC : ((dtreq < 1.e-12) ? h * FAC : dtreq);
    if (h_next < H_MIN) h_next = H_MIN;
    // converged b of this step, per body row (7 per component)
    if (has) {
        const int i = gl / 3, d = gl % 3;
#pragma unroll
        for (int k = 0; k < 7; k++) L.row[i][7 * d + k] = (float)X.b[k];
    }
    grp.sync();
    for (int e = gl; e < n * 7; e += GS) {
        int i = e / 7, k = e % 7;
        float sc = fmaxf(fmaxf(fabsf(L.row[i][k]), fabsf(L.row[i][7 + k])), fabsf(L.row[i][14 + k]));
        L.scale[i][k] = (sc > 0.0f && isfinite(sc)) ? sc : 1.0f;
    }
    grp.sync();
    // the pending sample: features of the previous accept, target from this b
    if (a.samples && pend_valid && first_attempt) {
        unsigned long long base = 0;
        if (gl == 0) base = atomicAdd(a.sample_count, (unsigned long long)n);
        base = (unsigned long long)grp.bcast0((long long)base);
        if (base + (unsigned long long)n <= (unsigned long long)a.sample_cap) {
            for (int e = gl; e < n * MLP_IN; e += GS) {
                int i = e / MLP_IN, k = e % MLP_IN;
                a.samples[(base + i) * MLP_SAMPLE + k] = k < MLP_FEAT ? L.pfeat[i][k] : 0.0f;
            }
            for (int e = gl; e < n * (MLP_OUT_PAD - MLP_OUT); e += GS) {
                int i = e / (MLP_OUT_PAD - MLP_OUT), k = MLP_OUT + e % (MLP_OUT_PAD - MLP_OUT);
                a.samples[(base + i) * MLP_SAMPLE + MLP_IN + k] = 0.0f;
            }
            if (has) {
                const int i = gl / 3, d = gl % 3;
#pragma unroll
                for (int k = 0; k < 7; k++) {
                    float tgt = ((float)(X.b[k] / (double)L.ps[i][k]) - L.pE[i][7 * d + k]) / a.tau[k];
                    a.samples[(base + i) * MLP_SAMPLE + MLP_IN + 7 * d + k] = tgt;
                }
            }
        }
    }
    // features of this step (into xh2 as bf16, ld 40) and the plain guess E
    grp.sync();
    float lq = fminf(fmaxf(log2f((float)q), -8.0f), 8.0f) * 0.25f;
    float lh = fminf(fmaxf(log2f((float)(h_next / h)), -8.0f), 8.0f) * 0.25f;
    if (has) {
        const int i = gl / 3, d = gl % 3;
#pragma unroll
        for (int k = 0; k < 7; k++) {
            float f = L.row[i][7 * d + k] / L.scale[i][k];
            L.xh2[i][7 * d + k] = __float2bfloat16_rn(f);
            L.pfeat[i][7 * d + k] = f;
        }
    }
    e_refine(X, q);
    if (has) {
        const int i = gl / 3, d = gl % 3;
#pragma unroll
        for (int k = 0; k < 7; k++) L.pE[i][7 * d + k] = (float)(X.b[k] / (double)L.scale[i][k]);
    }
    for (int e = gl; e < LP_ROWS * 40; e += GS) {
        int i = e / 40, k = e % 40;
        if (i < n && k < MLP_OUT) continue;
        float f = 0.0f;
        if (i < n) {
            if (k == 21) f = lq;
            else if (k == 22) f = lh;
            else if (k == 23) f = log10f(fmaxf((float)(m[i] / m[0]), 1e-20f)) * 0.1f;
            else if (k >= 24 && k < 30)
                f = fminf(fmaxf(log10f(L.scale[i][k - 23] / L.scale[i][0]), -30.0f), 30.0f) * 0.1f;
        }
        L.xh2[i][k] = __float2bfloat16_rn(f);
        if (i < n && k < MLP_FEAT) L.pfeat[i][k] = f;
    }
    for (int e = gl; e < n * 7; e += GS) L.ps[e / 7][e % 7] = L.scale[e / 7][e % 7];
    pend_valid = a.samples != nullptr;
    grp.sync();
    if (a.mlp) {
        if (grp.wig == 0) mlp_warp_forward(a.mlp, L);
        grp.sync();
        if (has) {
            const int i = gl / 3, d = gl % 3;
#pragma unroll
            for (int k = 0; k < 7; k++) L.plain[gl][k] = X.b[k];
            L.plain[gl][7] = X.b6p;
#pragma unroll
            for (int k = 0; k < 7; k++) {
                // outside the training range (|target| <= 20) or non-finite:
                // keep the plain guess for this coefficient
                float o = L.row[i][7 * d + k];
                o = (isfinite(o) && fabsf(o) <= 20.0f) ? o : 0.0f;
                X.b[k] += (double)L.scale[i][k] * (double)a.tau[k] * (double)o;
            }
        }
        grp.sync();
        net_guess = true;
    }
    if (make_consistent && has) consistent_g(X);
}

// Back to the plain guess (consistent g) that learned_refine kept.
__device__ __forceinline__ void restore_plain_guess(LearnSmem &L, Comp &X, int gl, bool has)
{
    if (!has) return;
#pragma unroll
    for (int k = 0; k < 7; k++) X.b[k] = L.plain[gl][k];
    X.b6p = L.plain[gl][7];
    consistent_g(X);
}

// Blocks per SM the register budget is sized for, per variant (the
// learned variants hold the network's fragments and take 3).
#ifndef ABIE_ENS_MINB
#define ABIE_ENS_MINB 4
#endif
template <int W, bool LEARN>
struct EnsOccupancy {
    static constexpr int value = LEARN ? 3 : ABIE_ENS_MINB;
};

template <int MODE, int W, bool LEARN>
__global__ void __launch_bounds__(32 * WARPS, (EnsOccupancy<W, LEARN>::value)) ensemble_kernel(EnsArgs a)
{
    constexpr int GROUPS = WARPS / W;
    __shared__ double s_pos[GROUPS][32][SPW];
    __shared__ double s_acc[GROUPS][32][3];
    constexpr int NB = W == 1 ? 10 : ENS_MAX_BODIES;  // bodies a group of W warps holds
    __shared__ CtrRow<NB> s_ctr[ref_ops<MODE>() ? 1 : GROUPS][NB];  // pair terms
    __shared__ double s_red[GROUPS][2 * W + 1];
    __shared__ int s_flg[GROUPS][2 * W];
    extern __shared__ __align__(16) unsigned char ens_dyn[];  // learned path only
    Group<W> grp;
    {
        const int w = threadIdx.x >> 5;
        grp.lane = threadIdx.x & 31;
        grp.wig = w % W;
        grp.gidx = w / W;
        grp.gl = grp.wig * 32 + grp.lane;
        grp.red = s_red[grp.gidx];
        grp.flg = s_flg[grp.gidx];
        grp.tog = 0;
    }
    const int gl = grp.gl;
    LearnSmem &LS = reinterpret_cast<LearnSmem *>(ens_dyn)[grp.gidx];
    double(*sp)[SPW] = s_pos[grp.gidx];
    double(*sa)[3] = s_acc[grp.gidx];
    const unsigned long long deadline = ens_timer() + a.budget_ns;

    for (;;) {
        int qi = 0;
        if (gl == 0) qi = atomicAdd(a.queue, 1);
        qi = (int)grp.bcast0(qi);
        if (qi >= a.n_active) break;
        const int sid = a.active[qi];
        const long long off = a.offsets[sid];
        const int n = (int)(a.offsets[sid + 1] - off);
        const int dim = 3 * n;
        const double *m = a.m + off;
        EnsScalars S = a.sc[sid];
        const bool has = gl < dim;  // this thread's component c = gl
        Comp X;
        double *st = a.state + (size_t)STATE_PER_COMP * 3 * off;
        auto slot = [&](int k) -> double & { return st[(size_t)k * dim + gl]; };
        if (!has || S.phase == 0) {
            X.y0 = has ? a.pos[3 * off + gl] : 0.0;
            X.dy0 = has ? a.vel[3 * off + gl] : 0.0;
            X.F1 = X.b6p = 0.0;
#pragma unroll
            for (int k = 0; k < 7; k++) X.b[k] = X.g[k] = 0.0;
        } else {
            X.y0 = slot(0);
            X.dy0 = slot(1);
            X.F1 = slot(2);
            // the fast forms carry g only: b is formed from g at the next
            // accept, so it is neither saved at a yield nor read back
#pragma unroll
            for (int k = 0; k < 7; k++) X.b[k] = ref_ops<MODE>() ? slot(3 + k) : 0.0;
#pragma unroll
            for (int k = 0; k < 7; k++) X.g[k] = slot(10 + k);
            X.b6p = slot(17);
        }
        const double G = a.G;
        // G m of every body once per system; alive: this component's body has m >= 0
        if (gl < n) sp[gl][3] = m[gl] > 0.0 ? G * m[gl] : 0.0;
        const bool alive = has && m[gl / 3] >= 0.0;
        unsigned hmask = 0u;  // mixed form: the heavy partners
        if constexpr (MODE == ABIE_FORCE_MIXED) {
            grp.sync();
            hmask = heavy_mask(n, sp);
        }
        // publish a predicted position for every body (components of a
        // body may sit on different lanes, so go through shared memory)
        auto publish = [&](double p) {
            if (has) sp[gl / 3][gl % 3] = p;
            grp.sync();
        };
        auto force_here = [&]() -> double { return alive ? sa[gl / 3][gl % 3] : 0.0; };
        // the forces of the published positions: the fast form takes each
        // pair once for both bodies
        auto forces = [&]() {
            if constexpr (MODE == ABIE_FORCE_MIXED) {
                group_force_sym_mixed<W, NB>(grp, n, sp, sa, s_ctr[grp.gidx], hmask);
            } else if constexpr (!ref_ops<MODE>()) {
                group_force_sym<W, NB>(grp, n, sp, sa, s_ctr[grp.gidx]);
            } else {
                group_force<MODE, W>(grp, n, sp, sa);
            }
        };

        if (S.phase == 0) {
            // F1 = f(y0), then initial_time_step (:9-54)
            publish(X.y0);
            forces();
            if (has) X.F1 = force_here();
            S.force_calls++;
            // d0, d1 over the first n of the 3n entries, as the reference does
            unsigned long long k0 = 0, k1 = 0;
            if (gl < n) {
                k0 = absmax_key(X.y0);
                k1 = absmax_key(X.F1);
            }
            const double d0 = grp.maxk(k0);
            const double d1 = grp.maxk(k1);
            double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
            grp.sync();
            publish(X.y0 + dt0 * X.dy0);
            forces();
            S.force_calls++;
            const double d2 = grp.maxk(has ? absmax_key(force_here() - X.F1) : 0ull) / dt0;
            double dt1;
            if (fmax(d1, d2) <= 1e-15) dt1 = fmax(1e-6, dt0 * 1e-3);
            else dt1 = pow(0.01 / fmax(d1, d2), (1.0 / (15 + 1)));
            S.h = fmin(100 * dt0, dt1);
            S.loop_count = 0;
            S.phase = 1;
            grp.sync();
        }

        double t = S.t, h = S.h;
        int loop_count = S.loop_count;
        bool done = false;
        // learned predictor: pending training sample, first attempt after an accept
        const bool learn = LEARN && (a.mlp != nullptr || a.samples != nullptr) && n <= LP_ROWS;
        bool pend_valid = false, first_attempt = false;
        bool net_guess = false;  // this attempt started from the network's guess
        while (!done) {
            if (grp.any(ens_timer() > deadline)) break;
            int iters = 0;
            for (int ipc = 0; ipc < 12; ipc++) {
                iters++;
                unsigned long long kf8 = 0, kdb6 = 0;
                for (int ih = 1; ih < 8; ih++) {
                    grp.sync();
                    const double sh = e_hs[ih], ds = h * sh, hh = 0.5 * ds * ds;
                    publish(e_pred_pos<MODE>(X, ih, sh, h, ds, hh));
                    forces();
                    if (has) {
                        const double F = force_here();
                        e_gb_update<MODE>(X, ih, F);
                        if (ih == 7) {
                            kf8 = absmax_key(F);
                            kdb6 = absmax_key(e_b6<MODE>(X) - X.b6p);
                        }
                    }
                }
                S.force_calls += 7;
                const double f8 = grp.maxk(kf8);
                const double db6 = grp.maxk(kdb6);
                if (corrector_converged<MODE>(db6, f8)) break;
                X.b6p = e_b6<MODE>(X);
            }
            S.iterations += iters;
            S.attempts++;
            // advance
            grp.sync();
            const double hh1 = 0.5 * h * h;
            const double ya = e_pred_pos<MODE>(X, 8, 1.0, h, h, hh1);
            const double va = e_pred_vel<MODE>(X, h);
            publish(ya);
            forces();
            S.force_calls++;
            const double dd = has ? force_here() : 0.0;
            const bool bad = has && !(finite_bits(ya) && finite_bits(dd) && finite_bits(va));
            if (grp.any(bad)) {
                if (net_guess) {
                    // the network's guess led the corrector astray: redo the
                    // attempt from the plain guess
                    restore_plain_guess(LS, X, gl, has);
                    net_guess = false;
                    S.fallbacks++;
                    continue;
                }
                S.status = ABIE_ERR_NUMERICS;  // non-finite state: report, stop this system
                done = true;
                break;
            }
            const double mb6 = grp.maxk(has ? absmax_key(e_b6<MODE>(X)) : 0ull);
            const double mdd = grp.maxk(has ? absmax_key(dd) : 0ull);
            const double estim_b6 = mb6 / mdd;
            double err, dtreq, rq;
            step_size<MODE>(estim_b6, h, err, dtreq, rq);
            if (!(err == err)) {  // NaN step control: the state is not finite
                if (net_guess) {
                    restore_plain_guess(LS, X, gl, has);
                    net_guess = false;
                    S.fallbacks++;
                    continue;
                }
                S.status = ABIE_ERR_NUMERICS;
                done = true;
                break;
            }
            net_guess = false;
            if (err <= 1 || loop_count > 100) {
                t += h;
                loop_count = 0;
                S.steps++;
                bool stop = false;
                if (t > a.t_end) {
                    h = a.t_end - t;
                    stop = true;
                }
                const double q = ref_ops<MODE>() ? dtreq / h : rq;
                if (!ref_ops<MODE>()) e_b_from_g(X);  // the fast form carries g only
                X.y0 = ya;
                X.dy0 = va;
                X.F1 = dd;
                X.b6p = X.b[6];
                // the fast form always continues from g consistent with the guess
                const bool make_consistent = a.consistent_g || !ref_ops<MODE>();
                if (!stop && learn) {
                    learned_refine<W>(a, LS, grp, X, n, has, q, h, dtreq, m, pend_valid,
                                      first_attempt, net_guess, make_consistent);
                } else if (!stop) {
                    e_refine(X, q);
                    if (make_consistent) consistent_g(X);
                }
                first_attempt = true;
                if (stop) {
                    done = true;
                    break;
                }
            } else {
                loop_count += 1;
                first_attempt = false;
            }
            if ((ref_ops<MODE>() ? dtreq / h : rq) > 1.0 / FAC) h /= FAC;
            else if (dtreq < 1.e-12) h *= FAC;
            else h = dtreq;
            if (h < H_MIN) h = H_MIN;
        }
        S.t = t;
        S.h = h;
        S.loop_count = loop_count;
        if (done) S.phase = 2;
        if (has) {
            if (done) {
                a.pos[3 * off + gl] = X.y0;
                a.vel[3 * off + gl] = X.dy0;
            } else {
                slot(0) = X.y0;
                slot(1) = X.dy0;
                slot(2) = X.F1;
                if (ref_ops<MODE>()) {
#pragma unroll
                    for (int k = 0; k < 7; k++) slot(3 + k) = X.b[k];
                }
#pragma unroll
                for (int k = 0; k < 7; k++) slot(10 + k) = X.g[k];
                slot(17) = X.b6p;
            }
        }
        if (gl == 0) a.sc[sid] = S;
        grp.sync();
    }
}


}  // namespace abie
