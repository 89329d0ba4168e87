// Batched Gauss-Radau 15 over many independent small systems.
//
// A group of threads integrates one system (at most 21 bodies) from a work
// queue -- one warp for up to 10 bodies, two warps (a named barrier each)
// for 11-21, four warps for the slowest quarter of the systems, each class a
// kernel on its own stream -- and a finished group takes the next system,
// so systems of uneven size and difficulty do not wait for each other.  Each thread owns
// one of the system's 3N components and keeps its Radau state (y0, dy0,
// F1, b[7], g[7], previous b6) in registers.  For the force, the predicted
// positions go to shared memory and the pairs spread over the lanes: each
// warp takes ceil(N / warps) sinks with L = 32 / that lanes per sink, each
// summing every L-th source, partial sums added as a fixed tree (L = 1 and
// the reference's operations in the exact form).  The
// sweep itself -- predictor, g/b updates, convergence test, step control,
// refine_bs -- is the reference's (src/integrator_gauss_radau15.c:221-380)
// component by component, as in the single-system engine.  The fast form
// runs the corrector on the Newton-form coefficients g alone: predicted
// positions come straight from g with tabulated weights, b = C g is formed
// once per accepted step for refine_bs, and the next step starts from g
// consistent with the refined guess.  Far fewer FP64 instructions per
// substep (on this GPU each FP64 warp instruction holds the SM
// sub-partition's FP64 pipe for ~64 cycles whatever the number of active
// lanes, so the instruction count sets the time per substep), the same
// converged solution, and fewer corrector iterations.  The maxima behind
// the convergence test and the step control are integer maxima of the
// values' bit patterns, and the fast form's step-size root is taken in
// single precision (radau_comp.cuh, step_size).
//
// Systems start longest first (shortest two-body time scale first), since
// a batch lasts at least as long as its slowest system.
//
// Launches are bounded in time: a warp that has run past the launch's time
// budget saves its system's state and leaves; the host launches again over
// the systems not yet done.
#include <algorithm>
#include <vector>

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
__device__ __noinline__ void mlp_warp_forward(const LearnedPredictor *P, LearnSmem &L)
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

// Blocks per SM the register budget is sized for, per variant.
template <int W, bool LEARN>
struct EnsOccupancy {
    static constexpr int value = LEARN ? 3 : 4;
};

template <int MODE, int W, bool LEARN>
__global__ void __launch_bounds__(32 * WARPS, (EnsOccupancy<W, LEARN>::value)) ensemble_kernel(EnsArgs a)
{
    constexpr int GROUPS = WARPS / W;
    __shared__ double s_pos[GROUPS][32][4];
    __shared__ double s_acc[GROUPS][32][3];
    constexpr int NB = W == 1 ? 10 : ENS_MAX_BODIES;  // bodies a group of W warps holds
    __shared__ double s_ctr[MODE == ABIE_FORCE_EXACT ? 1 : GROUPS][NB][NB - 1][4];  // pair terms
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
    double(*sp)[4] = s_pos[grp.gidx];
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
#pragma unroll
            for (int k = 0; k < 7; k++) X.b[k] = slot(3 + k);
#pragma unroll
            for (int k = 0; k < 7; k++) X.g[k] = slot(10 + k);
            X.b6p = slot(17);
        }
        const double G = a.G;
        // G m of every body once per system; alive: this component's body has m >= 0
        if (gl < n) sp[gl][3] = m[gl] > 0.0 ? G * m[gl] : 0.0;
        const bool alive = has && m[gl / 3] >= 0.0;
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
            if constexpr (MODE != ABIE_FORCE_EXACT) {
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
                const double q = MODE == ABIE_FORCE_EXACT ? dtreq / h : rq;
                if (MODE != ABIE_FORCE_EXACT) e_b_from_g(X);  // the fast form carries g only
                X.y0 = ya;
                X.dy0 = va;
                X.F1 = dd;
                X.b6p = X.b[6];
                // the fast form always continues from g consistent with the guess
                const bool make_consistent = a.consistent_g || MODE != ABIE_FORCE_EXACT;
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
            if ((MODE == ABIE_FORCE_EXACT ? dtreq / h : rq) > 1.0 / FAC) h /= FAC;
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
#pragma unroll
                for (int k = 0; k < 7; k++) slot(3 + k) = X.b[k];
#pragma unroll
                for (int k = 0; k < 7; k++) slot(10 + k) = X.g[k];
                slot(17) = X.b6p;
            }
        }
        if (gl == 0) a.sc[sid] = S;
        grp.sync();
    }
}

static double g_last_seconds = 0.0;
// The slowest 1 in heavy_div systems (longest first) run on four warps.  On
// 4,096 planetary systems over 1 yr in the fast form the batch took 81-84
// ms with 1 in 256, 79-80 with 1 in 16, 76 with 1 in 8, 70-72 with 1 in 4,
// 85 with 1 in 2 and 78 with all: a batch ends with its slow systems, and a
// four-warp group cuts their per-step latency at the cost of more warps per
// system.  The exact form, whose group force does not split a pair's work,
// keeps 1 in 256 (with 1 in 4 its batch ran 76k system-steps/s against
// 100k).  abie_debug_ensemble_heavy sets one share for both.
static int g_heavy_div = 0;
static int heavy_div(int mode) { return g_heavy_div > 0 ? g_heavy_div : (mode == ABIE_FORCE_EXACT ? 256 : 4); }

template <int MODE, bool LEARN>
static const void *ensemble_fn_l(int w)
{
    return w == 1 ? (const void *)ensemble_kernel<MODE, 1, LEARN>
                  : (w == 2 ? (const void *)ensemble_kernel<MODE, 2, LEARN>
                            : (const void *)ensemble_kernel<MODE, 4, LEARN>);
}

// The kernel for a force form, warps per system and whether the learned
// predictor (or sample collection) is in use: without it the variant leaves
// the predictor's code out.
static const void *ensemble_fn(int mode, int w, bool learn)
{
    if (mode == ABIE_FORCE_EXACT)
        return learn ? ensemble_fn_l<ABIE_FORCE_EXACT, true>(w) : ensemble_fn_l<ABIE_FORCE_EXACT, false>(w);
    return learn ? ensemble_fn_l<ABIE_FORCE_FP64, true>(w) : ensemble_fn_l<ABIE_FORCE_FP64, false>(w);
}

static size_t learn_smem(int w) { return (size_t)(WARPS / w) * sizeof(LearnSmem); }

static int launch_ensemble(int mode, int w, int blocks, const EnsArgs &a, cudaStream_t st)
{
    const bool learn = a.mlp || a.samples;
    size_t dyn = learn ? learn_smem(w) : 0;
    void *args[] = {const_cast<EnsArgs *>(&a)};
    ABIE_CUDA(cudaLaunchKernel(ensemble_fn(mode, w, learn), dim3(blocks), dim3(32 * WARPS), args, dyn, st));
    return 0;
}

static cudaStream_t g_ens_stream[2] = {nullptr, nullptr};  // besides the caller's stream

int ensemble_run(double *pos, double *vel, const double *m, const long long *offsets, int ns,
                 double G, double t0, double t_end, double *t_out, int *status, long long *steps,
                 int mode, const LearnedPredictor *mlp, cudaStream_t st, EnsembleStats *stats,
                 const EnsembleLearnIO *learn_io, bool consistent, const float *mlp_tau)
{
    if (ns <= 0) return 0;
    long long total = offsets[ns];
    for (int s = 0; s < ns; s++) {
        long long k = offsets[s + 1] - offsets[s];
        if (k < 1 || k > ENS_MAX_BODIES) {
            set_error(ABIE_ERR_ARGUMENT, "ensemble system %d has %lld bodies (1..%d supported)", s,
                      k, ENS_MAX_BODIES);
            return ABIE_ERR_ARGUMENT;
        }
    }
    if (mode == ABIE_FORCE_NAIVE || mode == ABIE_FORCE_MIXED) mode = ABIE_FORCE_FP64;
    double *d_pos, *d_vel, *d_m, *d_state;
    long long *d_off;
    EnsScalars *d_sc;
    int *d_active, *d_queue;
    ABIE_CUDA(cudaMalloc(&d_pos, 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_vel, 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_m, total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_state, (size_t)STATE_PER_COMP * 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_off, (ns + 1) * sizeof(long long)));
    ABIE_CUDA(cudaMalloc(&d_sc, ns * sizeof(EnsScalars)));
    ABIE_CUDA(cudaMalloc(&d_active, ns * sizeof(int)));
    ABIE_CUDA(cudaMalloc(&d_queue, 3 * sizeof(int)));
    std::vector<EnsScalars> sc(ns);
    for (int s = 0; s < ns; s++) {
        memset(&sc[s], 0, sizeof(EnsScalars));
        sc[s].t = t0;
    }
    // Longest-first order: a system's step count follows its shortest
    // two-body time scale sqrt(r_ij^3 / G(m_i + m_j)), and the batch takes
    // at least as long as its slowest system, so those start first.
    std::vector<double> rate(ns, 0.0);
    {
        std::vector<double> hp(3 * (size_t)total), hm(m, m + total);
        memcpy(hp.data(), pos, 3 * total * sizeof(double));
        for (int s = 0; s < ns; s++) {
            double best = 0.0;
            for (long long i = offsets[s]; i < offsets[s + 1]; i++)
                for (long long j = i + 1; j < offsets[s + 1]; j++) {
                    double mu = G * (std::max(hm[i], 0.0) + std::max(hm[j], 0.0));
                    double dx = hp[3 * i] - hp[3 * j], dy = hp[3 * i + 1] - hp[3 * j + 1],
                           dz = hp[3 * i + 2] - hp[3 * j + 2];
                    double r2 = dx * dx + dy * dy + dz * dz;
                    if (mu > 0.0 && r2 > 0.0) best = std::max(best, sqrt(mu / (r2 * sqrt(r2))));
                }
            rate[s] = best;
        }
    }
    std::vector<int> active(ns);
    for (int s = 0; s < ns; s++) active[s] = s;
    std::stable_sort(active.begin(), active.end(), [&](int x, int y) { return rate[x] > rate[y]; });
    ABIE_CUDA(cudaMemcpyAsync(d_pos, pos, 3 * total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_vel, vel, 3 * total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_m, m, total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_off, offsets, (ns + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_sc, sc.data(), ns * sizeof(EnsScalars), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaStreamSynchronize(st));

    const bool learning = mlp || (learn_io && learn_io->samples);
    // three classes of system: up to 10 bodies on one warp, 11-21 on two,
    // and the slowest few (longest-first order) on four warps, which cuts
    // their per-substep latency -- the batch ends with its slowest system
    const int WC[3] = {1, 2, 4};
    int bps[3] = {1, 1, 1};
    for (int k = 0; k < 3; k++) {
        const void *fn = ensemble_fn(mode, WC[k], learning);
        const size_t dyn = learning ? learn_smem(WC[k]) : 0;
        if (learning)
            ABIE_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[k], fn, 32 * WARPS, dyn));
        bps[k] = std::max(bps[k], 1);
    }
    std::vector<unsigned char> cls(ns);
    {
        const int heavy = std::min(ns, std::max(1, ns / heavy_div(mode)));
        for (int q = 0; q < ns; q++) {
            const int s2 = active[q];
            cls[s2] = q < heavy ? 2 : (3 * (offsets[s2 + 1] - offsets[s2]) <= 32 ? 0 : 1);
        }
    }
    for (int k = 0; k < 2; k++)
        if (!g_ens_stream[k]) ABIE_CUDA(cudaStreamCreateWithFlags(&g_ens_stream[k], cudaStreamNonBlocking));
    cudaEvent_t e0, e1, ej;
    ABIE_CUDA(cudaEventCreate(&e0));
    ABIE_CUDA(cudaEventCreate(&e1));
    ABIE_CUDA(cudaEventCreateWithFlags(&ej, cudaEventDisableTiming));
    double gpu_ms = 0.0;
    int launches = 0;
    int n_active = ns;
    std::vector<int> part(ns);
    while (n_active > 0) {
        // the classes' lists, each in longest-first order
        int first[4] = {0, 0, 0, 0};
        {
            int k2 = 0;
            for (int c = 0; c < 3; c++) {
                first[c] = k2;
                for (int q = 0; q < n_active; q++)
                    if (cls[active[q]] == c) part[k2++] = active[q];
            }
            first[3] = k2;
        }
        ABIE_CUDA(cudaMemcpyAsync(d_active, part.data(), n_active * sizeof(int),
                                  cudaMemcpyHostToDevice, st));
        ABIE_CUDA(cudaMemsetAsync(d_queue, 0, 3 * sizeof(int), st));
        EnsArgs a;
        a.offsets = d_off;
        a.m = d_m;
        a.pos = d_pos;
        a.vel = d_vel;
        a.state = d_state;
        a.sc = d_sc;
        a.G = G;
        a.t_end = t_end;
        a.mlp = mlp;
        a.samples = learn_io ? learn_io->samples : nullptr;
        a.sample_cap = learn_io ? learn_io->cap : 0;
        a.sample_count = learn_io ? learn_io->count : nullptr;
        for (int k = 0; k < 7; k++) a.tau[k] = learn_io ? learn_io->tau[k] : (mlp_tau ? mlp_tau[k] : 1.0f);
        a.consistent_g = consistent ? 1 : 0;
        a.budget_ns = 2000000000ull;  // each launch yields after about two seconds
        ABIE_CUDA(cudaEventRecord(e0, st));
        ABIE_CUDA(cudaEventRecord(ej, st));
        for (int k = 0; k < 2; k++) ABIE_CUDA(cudaStreamWaitEvent(g_ens_stream[k], ej, 0));
        for (int k = 0; k < 3; k++) {
            const int cnt = first[k + 1] - first[k];
            if (cnt == 0) continue;
            EnsArgs ak = a;
            ak.active = d_active + first[k];
            ak.n_active = cnt;
            ak.queue = d_queue + k;
            const int per_block = WARPS / WC[k];  // systems per block
            int blocks = (int)std::min<long long>((long long)bps[k] * g_sim.num_sms,
                                                  (cnt + per_block - 1) / per_block);
            blocks = std::max(blocks, 1);
            int lrc = launch_ensemble(mode, WC[k], blocks, ak, k == 0 ? st : g_ens_stream[k - 1]);
            if (lrc) return lrc;
        }
        for (int k = 0; k < 2; k++) {
            ABIE_CUDA(cudaEventRecord(ej, g_ens_stream[k]));
            ABIE_CUDA(cudaStreamWaitEvent(st, ej, 0));
        }
        ABIE_CUDA(cudaEventRecord(e1, st));
        ABIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        gpu_ms += ms;
        launches++;
        ABIE_CUDA(cudaMemcpy(sc.data(), d_sc, ns * sizeof(EnsScalars), cudaMemcpyDeviceToHost));
        int k = 0;
        for (int q = 0; q < n_active; q++) {  // keeps the longest-first order
            const int s2 = active[q];
            if (sc[s2].phase != 2 && sc[s2].status == 0) active[k++] = s2;
        }
        n_active = k;
    }
    cudaEventDestroy(ej);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ABIE_CUDA(cudaMemcpy(pos, d_pos, 3 * total * sizeof(double), cudaMemcpyDeviceToHost));
    ABIE_CUDA(cudaMemcpy(vel, d_vel, 3 * total * sizeof(double), cudaMemcpyDeviceToHost));
    for (int s = 0; s < ns; s++) {
        if (t_out) t_out[s] = sc[s].t;
        if (status) status[s] = sc[s].status;
        if (steps) steps[s] = sc[s].steps;
        if (stats) {
            stats->attempts += sc[s].attempts;
            stats->iterations += sc[s].iterations;
            stats->force_calls += sc[s].force_calls;
            stats->steps += sc[s].steps;
            stats->fallbacks += sc[s].fallbacks;
        }
    }
    if (stats) stats->launches += launches;
    g_last_seconds = gpu_ms * 1e-3;
    cudaFree(d_pos);
    cudaFree(d_vel);
    cudaFree(d_m);
    cudaFree(d_state);
    cudaFree(d_off);
    cudaFree(d_sc);
    cudaFree(d_active);
    cudaFree(d_queue);
    return 0;
}

double ensemble_last_seconds() { return g_last_seconds; }

}  // namespace abie

using namespace abie;

extern "C" {
// The share of systems (the slowest 1 in div, longest first) that run on
// four-warp groups; 0 restores the default.  For tests and tuning.
void abie_debug_ensemble_heavy(int div) { abie::g_heavy_div = div > 0 ? div : 0; }


int abie_gr_ensemble(double *pos, double *vel, const double *m, const long long *offsets,
                     int n_systems, double G, double t0, double t_end, double *t_out, int *status,
                     long long *steps, int flags)
{
    int rc = ensure_device(-1);
    if (rc) return rc;
    const LearnedPredictor *mlp = (flags & 1) ? learned_predictor_current() : nullptr;
    if ((flags & 1) && !mlp) {
        set_error(ABIE_ERR_ARGUMENT, "abie_gr_ensemble: learned predictor requested, none enabled");
        return ABIE_ERR_ARGUMENT;
    }
    EnsembleLearnIO io = {};
    if (flags & 2) {
        rc = mlp_collect_begin(&io);
        if (rc) return rc;
    }
    EnsembleStats st = {};
    rc = ensemble_run(pos, vel, m, offsets, n_systems, G, t0, t_end, t_out, status, steps,
                      g_sim.force_mode, mlp, g_sim.st, &st, (flags & 2) ? &io : nullptr,
                      (flags & 1) || (flags & 4), mlp ? learned_predictor_tau() : nullptr);
    if (flags & 2) mlp_collect_end(&io);
    if (rc == 0) {
        g_sim.ctr.attempts += st.attempts;
        g_sim.ctr.iterations += st.iterations;
        g_sim.ctr.force_calls += st.force_calls;
        g_sim.ctr.accepts += st.steps;
        g_sim.ctr.rejects += st.attempts - st.steps;
        g_sim.ctr.learned_fallbacks += st.fallbacks;
    }
    return rc;
}

double abie_last_ensemble_seconds(void) { return ensemble_last_seconds(); }

}  // extern "C"
