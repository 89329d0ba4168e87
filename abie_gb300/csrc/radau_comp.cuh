// Radau15 on one component per thread (src/integrator_gauss_radau15.c:56-218),
// shared by the batched ensemble (ensemble.cu) and the split engine for
// systems with few massive bodies (radau.cu).  Each thread keeps its
// component's state -- y0, dy0, F1, b[7], g[7], previous b6 -- in
// registers.  MODE ABIE_FORCE_EXACT repeats the reference's expressions in
// its order (built with --fmad=false); ABIE_FORCE_NAIVE, the plain FP64
// form, runs the same expressions in a unit built with FMA contraction; the
// fast and mixed forms run the corrector on the Newton-form coefficients g
// with tabulated weights.
#pragma once
#include "common.cuh"
#include "radau_constants.h"

namespace abie {

// Forms that run the reference's operations: its Horner predictor on b, b
// rebuilt from g after every force, the division in the convergence test
// and pow in the step control.
template <int MODE>
__host__ __device__ constexpr bool ref_ops()
{
    return MODE == ABIE_FORCE_EXACT || MODE == ABIE_FORCE_NAIVE;
}

static __constant__ double e_hs[8] = ABIE_RADAU_HS_INIT;
static __constant__ double e_rs[8][8] = ABIE_RADAU_RS_INIT;
static __constant__ double e_cs[8][8] = ABIE_RADAU_CS_INIT;
static __constant__ double e_rsp[8][8] = ABIE_RADAU_RSP_INIT;  // fast sweep: expanded g recurrence
static __constant__ double e_wg[9][7] = ABIE_RADAU_WG_INIT;    // fast sweep: position weights on g, row 8 = spacing 1
static __constant__ double e_vg[7] = ABIE_RADAU_VG_INIT;       // fast sweep: velocity weights on g at spacing 1
static __constant__ double e_vgs[9][7] = ABIE_RADAU_VGS_INIT;  // velocity weights on g at every spacing


// Doubles per row of the shared predicted-position tables {x, y, z, G m}:
// one pad entry, so consecutive bodies' rows start 10 banks apart and a
// warp reading sixteen different bodies' rows hits distinct bank pairs
// (with 4 doubles, every body's row starts in one of 4 banks).
static constexpr int SPW = 5;

// Row of the pair-term table of one body (group_force_sym*): 4 doubles per
// partner {w, dx, dy, dz} plus one pad double, so that the rows of
// different bodies start in different banks (without it every row of a
// 21-body table starts in the same bank and the lanes of one component
// conflict 12 ways).
template <int NB>
struct CtrRow {
    double e[NB - 1][4];
    double pad;
};

static constexpr double EPSB = 1.e-4;
static constexpr double FAC = 0.25;
static constexpr double TOLPC = 1.e-16;
static constexpr double H_MIN = 1.e-13;

__device__ __forceinline__ unsigned long long ens_timer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Component state of one lane.
struct Comp {
    double y0, dy0, F1, b[7], g[7], b6p;
};

// Predicted position at spacing s = e_hs[row] (row 8: s = 1) of a step dt.
// Exact form: the reference's Horner polynomial in b with its divisions.
// Fast form: the same polynomial written on the Newton-form coefficients
// g (b = C g), y0 + ds dy0 + hh (F1 + sum_j g_j W_j(s)) with the weights
// W_j(s) = sum_{k<=j} cs[j][k] s^(k+1) / ((k+2)(k+3)/2) tabulated, and
// ds = dt s, hh = ds^2 / 2 once per substep: 11 FP64 instructions, and b
// is never needed inside the corrector.
template <int MODE>
__device__ __forceinline__ double e_pred_pos(const Comp &c, int row, double s, double dt, double ds,
                                             double hh)
{
    const double *b = c.b;
    if (ref_ops<MODE>())
        return c.y0 + dt * s * (c.dy0 + dt * s * (c.F1 + s * (b[0] / 0.3e1 + s * (b[1] / 0.6e1 + s * (b[2] / 0.10e2 + s * (b[3] / 0.15e2 + s * (b[4] / 0.21e2 + s * (b[5] / 0.28e2 + s * b[6] / 0.36e2))))))) / 0.2e1);
    const double *w = e_wg[row];
    const double *g = c.g;
    double u = g[6] * w[6];
    u = fma(g[5], w[5], u);
    u = fma(g[4], w[4], u);
    u = fma(g[3], w[3], u);
    u = fma(g[2], w[2], u);
    u = fma(g[1], w[1], u);
    u = fma(g[0], w[0], u);
    // the step's displacement first, then one rounding at the position's
    // scale, as the reference's Horner form adds it: two FMAs into y0
    // round twice there, which over 10^4 yr doubled the fast form's median
    // energy error in a host emulation of its arithmetic (64 systems:
    // 9.9e-13 against the reference method's 3.1-4.4e-13; this order
    // 5.0e-13, 46 of 64 within 1e-12 against 43-45).  The part without g
    // is formed off the chain that waits for u.
    const double p = fma(ds, c.dy0, hh * c.F1);
    return c.y0 + fma(hh, u, p);
}

// Predicted velocity at spacing 1 (the advance).
template <int MODE>
__device__ __forceinline__ double e_pred_vel(const Comp &c, double dt)
{
    const double *b = c.b;
    if (ref_ops<MODE>()) {
        const double s = 1.0;
        return c.dy0 + dt * s * (c.F1 + s * (b[0] / 0.2e1 + s * (b[1] / 0.3e1 + s * (b[2] / 0.4e1 + s * (b[3] / 0.5e1 + s * (b[4] / 0.6e1 + s * (b[5] / 0.7e1 + s * b[6] / 0.8e1)))))));
    }
    const double *g = c.g;
    double u = g[6] * e_vg[6];
    u = fma(g[5], e_vg[5], u);
    u = fma(g[4], e_vg[4], u);
    u = fma(g[3], e_vg[3], u);
    u = fma(g[2], e_vg[2], u);
    u = fma(g[1], e_vg[1], u);
    u = fma(g[0], e_vg[0], u);
    return fma(dt, c.F1 + u, c.dy0);
}

// Predicted velocity at spacing s = e_hs[row] (row 8: s = 1), needed only
// by velocity-dependent forces (src/integrator_gauss_radau15.c:63-68).
template <int MODE>
__device__ __forceinline__ double e_pred_vel_at(const Comp &c, int row, double s, double dt)
{
    const double *b = c.b;
    if (ref_ops<MODE>())
        return c.dy0 + dt * s * (c.F1 + s * (b[0] / 0.2e1 + s * (b[1] / 0.3e1 + s * (b[2] / 0.4e1 + s * (b[3] / 0.5e1 + s * (b[4] / 0.6e1 + s * (b[5] / 0.7e1 + s * b[6] / 0.8e1)))))));
    const double *w = e_vgs[row];
    const double *g = c.g;
    double u = g[6] * w[6];
    u = fma(g[5], w[5], u);
    u = fma(g[4], w[4], u);
    u = fma(g[3], w[3], u);
    u = fma(g[2], w[2], u);
    u = fma(g[1], w[1], u);
    u = fma(g[0], w[0], u);
    return fma(dt * s, c.F1 + u, c.dy0);
}

// b6 of the corrector: b_6 = cs[6][6] g_6 = g_6, read from g in the fast form.
template <int MODE>
__device__ __forceinline__ double e_b6(const Comp &c)
{
    return ref_ops<MODE>() ? c.b[6] : c.g[6];
}

// g and b after the force F of substep IH (src/integrator_gauss_radau15.c:70-175);
// one fully static variant per substep keeps the coefficients in registers.
template <int MODE, int IH>
__device__ __forceinline__ void e_gb_update_ih(Comp &c, double F)
{
    double v = (F - c.F1) * e_rs[IH][0];
#pragma unroll
    for (int l = 1; l < IH; l++) v = (v - c.g[l - 1]) * e_rs[IH][l];
    c.g[IH - 1] = v;
#pragma unroll
    for (int k = 0; k < IH; k++) {
        double s = e_cs[k][k] * c.g[k];
#pragma unroll
        for (int jj = k + 1; jj < 7; jj++) {
            if (ref_ops<MODE>()) s = s + e_cs[jj][k] * c.g[jj];  // reference roundings
            else s = fma(e_cs[jj][k], c.g[jj], s);
        }
        c.b[k] = s;
    }
}

// Fast form: only the new Newton coefficient, g_{IH-1} from the expanded
// recurrence (F - F1) rsp[IH][0] - sum_{l<IH-1} g_l rsp[IH][l+1]; b is
// formed from g once per accepted step (e_b_from_g).
template <int IH>
__device__ __forceinline__ void e_g_update_ih(Comp &c, double F)
{
    double v = (F - c.F1) * e_rsp[IH][0];
#pragma unroll
    for (int l = 1; l < IH; l++) v = fma(-c.g[l - 1], e_rsp[IH][l], v);
    c.g[IH - 1] = v;
}

template <int MODE>
__device__ __forceinline__ void e_gb_update(Comp &c, int ih, double F)
{
    if (ref_ops<MODE>()) {
        switch (ih) {
        case 1: e_gb_update_ih<MODE, 1>(c, F); break;
        case 2: e_gb_update_ih<MODE, 2>(c, F); break;
        case 3: e_gb_update_ih<MODE, 3>(c, F); break;
        case 4: e_gb_update_ih<MODE, 4>(c, F); break;
        case 5: e_gb_update_ih<MODE, 5>(c, F); break;
        case 6: e_gb_update_ih<MODE, 6>(c, F); break;
        default: e_gb_update_ih<MODE, 7>(c, F); break;
        }
        return;
    }
    switch (ih) {
    case 1: e_g_update_ih<1>(c, F); break;
    case 2: e_g_update_ih<2>(c, F); break;
    case 3: e_g_update_ih<3>(c, F); break;
    case 4: e_g_update_ih<4>(c, F); break;
    case 5: e_g_update_ih<5>(c, F); break;
    case 6: e_g_update_ih<6>(c, F); break;
    default: e_g_update_ih<7>(c, F); break;
    }
}

// b_k = sum_{j>=k} cs[j][k] g_j for every k (fast form, at an accept).
__device__ __forceinline__ void e_b_from_g(Comp &c)
{
#pragma unroll
    for (int k = 0; k < 7; k++) {
        double s = c.g[k];  // cs[k][k] = 1
#pragma unroll
        for (int j = k + 1; j < 7; j++) s = fma(e_cs[j][k], c.g[j], s);
        c.b[k] = s;
    }
}

__device__ __forceinline__ void e_refine(Comp &c, double q)
{
    double *b = c.b;
    double q2 = q * q, q3 = q2 * q, q4 = q2 * q2, q5 = q2 * q3, q6 = q3 * q3, q7 = q2 * q5;
    double e0 = q * (b[6] * 7.0 + b[5] * 6.0 + b[4] * 5.0 + b[3] * 4.0 + b[2] * 3.0 + b[1] * 2.0 + b[0]);
    double e1 = q2 * (b[6] * 21.0 + b[5] * 15.0 + b[4] * 10.0 + b[3] * 6.0 + b[2] * 3.0 + b[1]);
    double e2 = q3 * (b[6] * 35.0 + b[5] * 20.0 + b[4] * 10.0 + b[3] * 4.0 + b[2]);
    double e3 = q4 * (b[6] * 35.0 + b[5] * 15.0 + b[4] * 5.0 + b[3]);
    double e4 = q5 * (b[6] * 21.0 + b[5] * 6.0 + b[4]);
    double e5 = q6 * (b[6] * 7.0 + b[5]);
    double e6 = q7 * b[6];
    b[0] = e0 + 0.0;
    b[1] = e1 + 0.0;
    b[2] = e2 + 0.0;
    b[3] = e3 + 0.0;
    b[4] = e4 + 0.0;
    b[5] = e5 + 0.0;
    b[6] = e6 + 0.0;
}

// Max over the warp of absmax_key values (integer instructions only).
__device__ __forceinline__ unsigned long long warp_maxk(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// The corrector's convergence test (src/integrator_gauss_radau15.c:300),
// db6 / f8 < tolpc.  The fast form multiplies instead of dividing.
template <int MODE>
__device__ __forceinline__ bool corrector_converged(double db6, double f8)
{
    return ref_ops<MODE>() ? db6 / f8 < TOLPC : db6 < TOLPC * f8;
}

// Step control (src/integrator_gauss_radau15.c:313-367): err =
// (estim_b6 / epsb)^(1/7) and dtreq = h / err.  The fast form returns
// rq = 1 / err as well (so dtreq = h rq, and the ratio dtreq / h the
// controller tests is rq) and takes the seventh root in single precision
// (log2 / exp2 of the ratio truncated to a float; NaN, infinite or negative
// ratios take the reference's path): the step size only steers the
// integrator.  The one visible difference: a retry after a rejection lands
// at err = 1 within rounding, and the single-precision err accepts it where
// the reference's last bits may reject it again (fewer attempts, about the
// same accepted steps).  Whenever the float err exceeds 1 its reciprocal is
// below 1, so a rejection always shrinks the step.
template <int MODE>
__device__ __forceinline__ void step_size(double estim_b6, double h, double &err, double &dtreq,
                                          double &rq)
{
    if (ref_ops<MODE>()) {  // the reference's operations
        err = pow(estim_b6 / EPSB, 1. / 7);
        dtreq = h / err;
        rq = dtreq / h;
        return;
    }
    const double x = estim_b6 * (1.0 / EPSB);
    if (!finite_bits(x) || !(__double2hiint(x) >= 0)) {  // NaN, infinite or negative
        err = pow(estim_b6 / EPSB, 1. / 7);
        dtreq = h / err;
        rq = dtreq / h;
        return;
    }
    const float xf = f64_to_f32_trunc23(x);  // exponent clamped to the float range; 0 stays tiny
    const float l7 = log2f(xf) * (1.0f / 7.0f);
    const float ef = exp2f(l7), rf = exp2f(-l7);
    err = f32_bits_to_f64(__float_as_int(ef));  // positive normal floats: exact
    rq = f32_bits_to_f64(__float_as_int(rf));
    dtreq = h * rq;
}

// g = C^-1 b for one component: back-substitution through the triangular
// change of basis b_k = sum_{j>=k} cs[j][k] g_j, so that the corrector's
// first sweep starts from the polynomial the guess describes.  (The
// reference keeps the previous step's g, which the first sweep mixes into
// every b it rebuilds, src/integrator_gauss_radau15.c:123-175.)
__device__ __forceinline__ void consistent_g(Comp &c)
{
#pragma unroll
    for (int k = 6; k >= 0; k--) {
        double v = c.b[k];
#pragma unroll
        for (int j = k + 1; j < 7; j++) v -= e_cs[j][k] * c.g[j];
        c.g[k] = v;
    }
}

// A system's thread group: W warps (32 W threads, one component each).
// W = 1 syncs with __syncwarp and reduces with shuffles; W = 2 syncs with a
// named barrier per group and meets the warps' partial reductions in shared
// memory (two alternating slots, so a slot is rewritten only after a barrier
// that every reader of its previous value has passed).
template <int W>
struct Group {
    int gl;    // lane in the group, 0 .. 32 W - 1
    int lane;  // lane in the warp
    int wig;   // warp in the group
    int gidx;  // group in the block
    double *red;
    int *flg;
    int tog;
    __device__ __forceinline__ void sync() const
    {
        if (W == 1) __syncwarp();
        else asm volatile("bar.sync %0, %1;" ::"r"(1 + gidx), "r"(32 * W) : "memory");
    }
    // max over the group of absmax_key values, as the double absmax_value
    // gives back (-DBL_MAX when every value was NaN or absent)
    __device__ __forceinline__ double maxk(unsigned long long v)
    {
        v = warp_maxk(v);
        if (W == 1) return absmax_value(v);
        unsigned long long *slot = reinterpret_cast<unsigned long long *>(red);
        if (lane == 0) slot[tog * W + wig] = v;
        sync();
        unsigned long long r = slot[tog * W];
#pragma unroll
        for (int k = 1; k < W; k++) r = slot[tog * W + k] > r ? slot[tog * W + k] : r;
        tog ^= 1;
        return absmax_value(r);
    }
    __device__ __forceinline__ bool any(bool b)
    {
        b = __any_sync(0xffffffffu, b);
        if (W == 1) return b;
        if (lane == 0) flg[tog * W + wig] = b ? 1 : 0;
        sync();
        int r = 0;
#pragma unroll
        for (int k = 0; k < W; k++) r |= flg[tog * W + k];
        tog ^= 1;
        return r != 0;
    }
    // the value group lane 0 holds, in every lane (one slot: the next write
    // comes many barriers later)
    __device__ __forceinline__ long long bcast0(long long v)
    {
        if (W == 1) return __shfl_sync(0xffffffffu, v, 0);
        long long *slot = reinterpret_cast<long long *>(red + 2 * W);
        if (gl == 0) *slot = v;
        sync();
        const long long r = *slot;
        sync();
        return r;
    }
};

// Accelerations of the n bodies whose predicted positions and G m are in
// sp[k] = {x, y, z, Gm}; the result of sink i goes to sa[i].  Warp w of the
// group takes sinks w spw .. (w + 1) spw - 1, spw = ceil(n / W), with
// L = 32 / spw lanes per sink (1 in the exact form), each summing every
// L-th source; the partial sums of the lanes holding work meet in a fixed
// tree of shuffles (a sink's lanes never straddle warps).
template <int MODE, int W>
__device__ __forceinline__ void group_force(const Group<W> &grp, int n, const double (*sp)[SPW],
                                            double (*sa)[3])
{
    const int spw = (n + W - 1) / W;
    const int L = MODE == ABIE_FORCE_EXACT ? 1 : max(1, 32 / max(spw, 1));
    static_assert(MODE != ABIE_FORCE_MIXED, "the mixed form uses group_force_sym_mixed");
    const int lane = grp.lane;
    const int gw = lane / L, hh = lane % L;
    const int g = grp.wig * spw + gw;
    const bool sink = gw < spw && g < n;
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (sink) {
        const double xi = sp[g][0], yi = sp[g][1], zi = sp[g][2];
        for (int k = hh; k < n; k += L) {
            double gm = sp[k][3];
            // gm > 0 on its bit pattern (an FP64 compare would hold the
            // FP64 pipe like a seventh instruction of the pair term)
            if (k == g || __double_as_longlong(gm) <= 0) continue;
            Src s{sp[k][0], sp[k][1], sp[k][2], gm};
            if (MODE == ABIE_FORCE_EXACT) pair_exact(xi, yi, zi, s, ax, ay, az);
            else if (MODE == ABIE_FORCE_NAIVE) pair_naive(xi, yi, zi, s, ax, ay, az);
            else pair_fast(xi, yi, zi, s, ax, ay, az);
        }
    }
    const int Wt = L < n ? L : n;
    for (int o = 1; o < Wt; o <<= 1) {
        int src = lane + o;
        src = src < 32 ? src : 31;
        double ox = __shfl_sync(0xffffffffu, ax, src);
        double oy = __shfl_sync(0xffffffffu, ay, src);
        double oz = __shfl_sync(0xffffffffu, az, src);
        if (hh + o < Wt) {
            ax += ox;
            ay += oy;
            az += oz;
        }
    }
    if (sink && hh == 0) {
        sa[g][0] = ax;
        sa[g][1] = ay;
        sa[g][2] = az;
    }
    grp.sync();
}


// A group's forces with each pair once for both bodies (fast form, n <= NB
// bodies): group lane p takes the p-th pair (i, k), i < k, shares the
// separation d = x_i - x_k, r^2 and r^-3, and stores for each body the
// factor and d -- {-G m_k r^-3, d} in ctr[i].e[k - 1], {G m_i r^-3, d} in
// ctr[k].e[i] (each body's partners in index order: partner j at slot j
// below the body, j - 1 above it; the first factor's sign flipped on its bit
// pattern, an integer operation).  The lane of component c of body b then
// sums its row with one FMA per partner, in that order, so each term is
// rounded once as in group_force.  3 FP64 instructions per pair round and
// n - 1 per component, against 6 per pair term and a shuffle tree.
template <int W, int NB>
__device__ __forceinline__ void group_force_sym(const Group<W> &grp, int n, const double (*sp)[SPW],
                                                double (*sa)[3], CtrRow<NB> *ctr)
{
    const int gl = grp.gl;
    const int P = n * (n - 1) / 2;
    for (int p0 = 0; p0 < P; p0 += 32 * W) {
        const int p = p0 + gl;
        if (p < P) {
            int i = 0, rem = p;
            while (rem >= n - 1 - i) {
                rem -= n - 1 - i;
                i++;
            }
            const int k = i + 1 + rem;
            const double dx = sp[i][0] - sp[k][0], dy = sp[i][1] - sp[k][1], dz = sp[i][2] - sp[k][2];
            unsigned long long Mr, Wn;
            int Er, eW;
            r2_int(dx, dy, dz, Mr, Er);
            inv_r3_core(Mr, Er, Wn, eW);
            const double gi = sp[i][3], gk = sp[k][3];
            const double wi = __double_as_longlong(gk) > 0 ? gm_times_inv_r3(Wn, eW, gk) : 0.0;
            const double wk = __double_as_longlong(gi) > 0 ? gm_times_inv_r3(Wn, eW, gi) : 0.0;
            ctr[i].e[k - 1][0] = __longlong_as_double(__double_as_longlong(wi) ^ (long long)0x8000000000000000ull);
            ctr[i].e[k - 1][1] = dx;
            ctr[i].e[k - 1][2] = dy;
            ctr[i].e[k - 1][3] = dz;
            ctr[k].e[i][0] = wk;
            ctr[k].e[i][1] = dx;
            ctr[k].e[i][2] = dy;
            ctr[k].e[i][3] = dz;
        }
    }
    grp.sync();
    if (gl < 3 * n) {
        const int b = gl / 3, c = gl % 3;
        double s = 0.0;
        for (int q = 0; q < n - 1; q++) s = fma(ctr[b].e[q][0], ctr[b].e[q][1 + c], s);
        sa[b][c] = s;
    }
    grp.sync();
}

// Mixed form of group_force_sym: the pair lanes work as there (FP64
// separations, the integer r^-3 core), and a partner counts as heavy when
// bit j of hmask is set (a G m of at least 1/128 of the system's largest:
// the star, or both stars of a binary).  A body's terms from heavy partners
// are stored and summed as in the fast form (one FP64 FMA each); a term from
// a light partner is stored as two-float pairs (w and the separation split
// exactly to 48 bits, split_ff) in the same 32-byte slot (four float2) and summed in FP32
// two-float arithmetic with compensated sums (ff_add_product), about 2^-46
// relative to the light terms.  Per component that leaves one FP64 FMA per
// heavy partner and two FP64 additions (the two-float sum, converted exactly)
// in place of n - 1 FMAs.
template <int W, int NB>
__device__ __forceinline__ void group_force_sym_mixed(const Group<W> &grp, int n,
                                                      const double (*sp)[SPW], double (*sa)[3],
                                                      CtrRow<NB> *ctr, unsigned hmask)
{
    const int gl = grp.gl;
    const int P = n * (n - 1) / 2;
    for (int p0 = 0; p0 < P; p0 += 32 * W) {
        const int p = p0 + gl;
        if (p < P) {
            int i = 0, rem = p;
            while (rem >= n - 1 - i) {
                rem -= n - 1 - i;
                i++;
            }
            const int k = i + 1 + rem;
            const double dx = sp[i][0] - sp[k][0], dy = sp[i][1] - sp[k][1], dz = sp[i][2] - sp[k][2];
            unsigned long long Mr, Wn;
            int Er, eW;
            r2_int(dx, dy, dz, Mr, Er);
            inv_r3_core(Mr, Er, Wn, eW);
            const double gi = sp[i][3], gk = sp[k][3];
            const double wi = __double_as_longlong(gk) > 0 ? gm_times_inv_r3(Wn, eW, gk) : 0.0;
            const double wk = __double_as_longlong(gi) > 0 ? gm_times_inv_r3(Wn, eW, gi) : 0.0;
            const double nwi = __longlong_as_double(__double_as_longlong(wi) ^ (long long)0x8000000000000000ull);
            const bool k_heavy = (hmask >> k) & 1u, i_heavy = (hmask >> i) & 1u;
            float2 fx = make_float2(0.f, 0.f), fy = fx, fz = fx;
            if (!(k_heavy && i_heavy)) {
                fx = split_ff(dx);
                fy = split_ff(dy);
                fz = split_ff(dz);
            }
            double *e1 = ctr[i].e[k - 1];  // body i, partner k
            if (k_heavy) {
                e1[0] = nwi;
                e1[1] = dx;
                e1[2] = dy;
                e1[3] = dz;
            } else {
                float2 *f = reinterpret_cast<float2 *>(e1);
                f[0] = split_ff(nwi);
                f[1] = fx;
                f[2] = fy;
                f[3] = fz;
            }
            double *e2 = ctr[k].e[i];  // body k, partner i
            if (i_heavy) {
                e2[0] = wk;
                e2[1] = dx;
                e2[2] = dy;
                e2[3] = dz;
            } else {
                float2 *f = reinterpret_cast<float2 *>(e2);
                f[0] = split_ff(wk);
                f[1] = fx;
                f[2] = fy;
                f[3] = fz;
            }
        }
    }
    grp.sync();
    if (gl < 3 * n) {
        const int b = gl / 3, c = gl % 3;
        float S = 0.0f, C = 0.0f;
        for (int q = 0; q < n - 1; q++) {
            const int j = q + (q >= b ? 1 : 0);
            if ((hmask >> j) & 1u) continue;
            const float2 *f = reinterpret_cast<const float2 *>(ctr[b].e[q]);
            ff_add_product(f[0], f[1 + c], S, C);
        }
        double s = f32_to_f64_exact(S) + f32_to_f64_exact(C);
        for (int q = 0; q < n - 1; q++) {
            const int j = q + (q >= b ? 1 : 0);
            if ((hmask >> j) & 1u) s = fma(ctr[b].e[q][0], ctr[b].e[q][1 + c], s);
        }
        sa[b][c] = s;
    }
    grp.sync();
}

// The heavy partners of a system for group_force_sym_mixed: bit j set when
// body j's G m (sp[j][3], zero for massless and deleted bodies) is at least
// 1/128 of the largest (the exponent lowered by 7); compared on bit patterns
// (positive doubles order as integers), so no FP64 instruction.
__device__ __forceinline__ unsigned heavy_mask(int n, const double (*sp)[SPW])
{
    long long top = 0;
    for (int j = 0; j < n; j++) top = max(top, __double_as_longlong(sp[j][3]));
    if (top <= 0) return 0u;
    const long long thr = top - (7ll << 52);
    unsigned m = 0u;
    for (int j = 0; j < n; j++)
        if (__double_as_longlong(sp[j][3]) >= thr && __double_as_longlong(sp[j][3]) > 0) m |= 1u << j;
    return m;
}

}  // namespace abie
