// Wisdom-Holman kick-drift-kick on the device.
//
// Reference: src/integrator_wisdom_holman.c:456-522.  Bodies split into
//   head: 0 .. the last body with nonzero mass (at least body 1), and
//   tail: the massless bodies after it.
// Massless bodies add exact zeros to every running sum of the reference
// (Jacobi centres of mass, interior masses, indirect and pairwise terms),
// so every tail body sees the same head quantities: the centre of mass
// and momentum that shift it into and out of Jacobi coordinates, the
// Kepler parameter G m0 eta/eta and the indirect and accel2 terms.  A
// one-block kernel computes the head (its sequential prefixes in the
// reference's order, its Kepler drifts in parallel) and publishes those
// quantities; a one-thread-per-body kernel then runs the whole step for
// each tail body.  Steps are replayed from a captured CUDA graph.
#include <algorithm>
#include <vector>

#include "abi_state.cuh"
#include "engine.cuh"

namespace abie {

static constexpr double KEPLER_TOL = 1e-12;  // src/integrator_wisdom_holman.h:7
static constexpr double TOL_ENERGY = 0.0;    // :11
static constexpr int KEPLER_MAX_IT = 500;    // :12
static constexpr int WH_HEAD_MAX = 4096;

// Quantities the head publishes for the tail.
struct WhShared {
    double R[3], V[3];    // helio -> Jacobi shift for tail bodies
    double Rp[3], Vp[3];  // Jacobi -> helio shift after the drift
    double ind[3];        // indirect term
    double a2[3];         // accel2 carried past the head
    double ind_a2[3];     // ind + a2 (the fast form adds them once)
    double gm_tail;       // Kepler parameter of a massless body
    double gm_tail_k[4];  // sqrt(gm_tail), 1/gm_tail, 1/sqrt(gm_tail), sqrt(gm_tail) dt
    unsigned long long kepler_failures;
};

struct WhArgs {
    int n, head;        // bodies, head size (head_end + 1)
    double G, dt;
    double dt2_6;       // dt * dt / 6 (the fast Kepler start)
    double *pos, *vel, *acc;  // heliocentric state and last acceleration (3n)
    const double *m;
    double *jpos, *jvel;      // head Jacobi state (3 * head)
    double *eta, *gm;         // head interior masses and Kepler parameters
    double *ir3h, *ir3j;      // head inverse cubes
    WhShared *sh;             // two sets, by step parity
    double *hsrc;             // two sets of the massive head bodies: x y z G m (4 per body)
};

// x^3 rounded once: x*x with its exact error (fma), times x (Dekker-style
// error-free products), so the value matches a correctly rounded pow(x, 3).
__device__ __forceinline__ double cube_cr(double x)
{
    double p = x * x;
    double e = fma(x, x, -p);
    double q = p * x;
    double f = fma(p, x, -q);
    return q + fma(e, x, f);
}

__device__ __forceinline__ double norm3(double a, double b, double c)
{
    double s = 0.0;
    s += a * a;
    s += b * b;
    s += c * c;
    return sqrt(s);
}

// src/integrator_wisdom_holman.c:15-32
__device__ __forceinline__ void stumpff(double psi, double &c2, double &c3)
{
    if (psi > 1.e-10) {
        double sp = sqrt(psi), s, c;
        sincos(sp, &s, &c);
        c2 = (1.0 - c) / psi;
        c3 = (sp - s) / sqrt(cube_cr(psi));
    } else if (psi < -1.e-6) {
        double sp = sqrt(-psi);
        c2 = (1 - cosh(sp)) / psi;
        c3 = (sinh(sp) - sp) / sqrt(-cube_cr(psi));
    } else {
        c2 = 0.5;
        c3 = 1.0 / 6.0;
    }
}

// src/integrator_wisdom_holman.c:51-132 on one body's Jacobi state.
// Returns 1 when Newton did not converge within the iteration cap.
__device__ int kepler_drift(double r0v[3], double v0v[3], double gm, double dt)
{
    double r0 = norm3(r0v[0], r0v[1], r0v[2]);
    double v0 = norm3(v0v[0], v0v[1], v0v[2]);
    double sqrtgm = sqrt(gm);
    double xi = 0.5 * v0 * v0 - gm / r0;
    double sma = -gm / (2 * xi);
    double alpha = 1.0 / sma;
    double rv = r0v[0] * v0v[0] + r0v[1] * v0v[1] + r0v[2] * v0v[2];
    double chi0;
    if (alpha > TOL_ENERGY) {
        chi0 = sqrtgm * dt * alpha;
    } else if (alpha < TOL_ENERGY) {
        double sg = (double)((dt > 0) - (dt < 0));
        chi0 = sg * (sqrt(-sma) * log(-2.0 * gm * alpha * dt / (rv + sqrt(-gm * sma) * (1.0 - r0 * alpha))));
    } else {
        double c0 = r0v[1] * v0v[2] - r0v[2] * v0v[1];
        double c1 = r0v[2] * v0v[0] - r0v[0] * v0v[2];
        double c2_ = r0v[0] * v0v[1] - r0v[1] * v0v[0];
        double cn = sqrt(c0 * c0 + c1 * c1 + c2_ * c2_);
        double p = cn * cn / gm;
        double s = 0.5 * atan(1.0 / (3.0 * sqrt(gm / cube_cr(p)) * dt));
        double w = atan(pow(tan(s), 1.0 / 3.0));
        chi0 = sqrt(p) * 2 / tan(2 * w);
    }
    double chi = 0.0, r = 0.0, c2 = 0.0, c3 = 0.0, psi = 0.0;
    const double rvs = rv / sqrtgm;
    for (int it = 0; it < KEPLER_MAX_IT; it++) {
        psi = chi0 * chi0 * alpha;
        stumpff(psi, c2, c3);
        r = chi0 * chi0 * c2 + rvs * chi0 * (1.0 - psi * c3) + r0 * (1 - psi * c2);
        chi = chi0 + (sqrtgm * dt - cube_cr(chi0) * c3 - rvs * (chi0 * chi0) * c2 - r0 * chi0 * (1.0 - psi * c3)) / r;
        if (fabs(chi - chi0) < KEPLER_TOL) break;
        chi0 = chi;
    }
    int failed = fabs(chi - chi0) > KEPLER_TOL;
    double f = 1.0 - chi * chi / r0 * c2;
    double g = dt - cube_cr(chi) / sqrtgm * c3;
    double dg = 1.0 - chi * chi / r * c2;
    double df = sqrtgm / (r * r0) * chi * (psi * c3 - 1.0);
    double nr[3], nv[3];
    for (int c = 0; c < 3; c++) {
        nr[c] = f * r0v[c] + g * v0v[c];
        nv[c] = df * r0v[c] + dg * v0v[c];
    }
    for (int c = 0; c < 3; c++) {
        r0v[c] = nr[c];
        v0v[c] = nv[c];
    }
    return failed;
}

// Stumpff functions by their series, c2 = sum_k (-psi)^k / (2k+2)!,
// c3 = sum_k (-psi)^k / (2k+3)!, for |psi| <= 0.5 (nine terms each; the
// first omitted term is below 1e-18).  More accurate there than the
// closed forms, whose 1 - cos(sqrt(psi)) cancels, and free of sqrt and
// sincos.
__device__ __forceinline__ void stumpff_series(double psi, double &c2, double &c3)
{
    const double x = -psi;
    double a = 1.0 / 6402373705728000.0;   // 1/18!
    a = fma(a, x, 1.0 / 20922789888000.0); // 1/16!
    a = fma(a, x, 1.0 / 87178291200.0);    // 1/14!
    a = fma(a, x, 1.0 / 479001600.0);      // 1/12!
    a = fma(a, x, 1.0 / 3628800.0);        // 1/10!
    a = fma(a, x, 1.0 / 40320.0);          // 1/8!
    a = fma(a, x, 1.0 / 720.0);            // 1/6!
    a = fma(a, x, 1.0 / 24.0);             // 1/4!
    c2 = fma(a, x, 0.5);                   // 1/2!
    double b = 1.0 / 121645100408832000.0; // 1/19!
    b = fma(b, x, 1.0 / 355687428096000.0);  // 1/17!
    b = fma(b, x, 1.0 / 1307674368000.0);    // 1/15!
    b = fma(b, x, 1.0 / 6227020800.0);       // 1/13!
    b = fma(b, x, 1.0 / 39916800.0);         // 1/11!
    b = fma(b, x, 1.0 / 362880.0);           // 1/9!
    b = fma(b, x, 1.0 / 5040.0);             // 1/7!
    b = fma(b, x, 1.0 / 120.0);              // 1/5!
    c3 = fma(b, x, 1.0 / 6.0);               // 1/3!
}

// The same series to five terms each, for |psi| <= 0.01: the first omitted
// terms, psi^5 / 12! and psi^5 / 13!, are below 3e-19 of c2 and c3.
__device__ __forceinline__ void stumpff_series_short(double psi, double &c2, double &c3)
{
    const double x = -psi;
    double a = 1.0 / 3628800.0;        // 1/10!
    a = fma(a, x, 1.0 / 40320.0);      // 1/8!
    a = fma(a, x, 1.0 / 720.0);        // 1/6!
    a = fma(a, x, 1.0 / 24.0);         // 1/4!
    c2 = fma(a, x, 0.5);               // 1/2!
    double b = 1.0 / 39916800.0;       // 1/11!
    b = fma(b, x, 1.0 / 362880.0);     // 1/9!
    b = fma(b, x, 1.0 / 5040.0);       // 1/7!
    b = fma(b, x, 1.0 / 120.0);        // 1/5!
    c3 = fma(b, x, 1.0 / 6.0);         // 1/3!
}

// Fast form of kepler_drift: the same universal-variable Newton iteration,
// convergence test (|dchi| < 1e-12) and f, g functions, with
//  * a starting value from the Taylor series of chi(t) (dchi/dt = sqrt(gm)/r)
//    to third order when the step covers a short arc (below), so one or
//    two Newton steps suffice instead of three or four on bound orbits;
//  * the series Stumpff functions for |psi| <= 0.5 where the reference uses
//    the closed forms (five terms each up to |psi| = 0.01, nine beyond; its
//    constants 1/2, 1/6 in -1e-6 <= psi <= 1e-10 and the closed forms
//    beyond |psi| = 0.5 are kept);
//  * 1/r and 1/sqrt from rcp_fast / inv_sqrt_fast instead of divisions and
//    sqrt, and sqrt(gm), 1/gm, 1/sqrt(gm) precomputed (k[0..2]).
// The converged chi is the same root; the state agrees with the reference
// form to rounding.  Distances must lie within the FP32 exponent range.
// A solve counts as failed as in the reference (its last two iterates
// still apart after the iteration cap).  The start: on a short arc
// (|w1^2 alpha| < 0.1, w1 = sqrt(gm) dt / r0) the Taylor series of chi(t)
// to third order for any conic -- the
// derivatives of chi come from r(t) and do not depend on the sign of
// alpha -- so an escaping test particle on a hyperbolic orbit needs one or
// two Newton steps where the reference's logarithmic start takes 27 on
// average and up to 200 (a C restatement of both iterations over 200,000
// hyperbolic states, r0 10 .. 3e4 au: the same roots to 1e-11, 1.04
// iterations on average).  rcp_fast takes either sign: the radius function
// r(chi) can turn negative far from the root, where a reciprocal for
// positive numbers only sent the iteration to NaN (escaping particles of
// the 1,048,582-body swarm did, some hundred over 2 x 10^5 steps).
// Comparisons on the bit patterns of doubles, with integer instructions
// (an FP64 compare holds the FP64 pipe like any FP64 instruction): |x| < t
// and x > t for a positive threshold t, x < t for a negative one.  NaN
// compares like a large magnitude; the callers' NaN states fail the
// convergence test either way.
__device__ __forceinline__ unsigned long long dmag(double x)
{
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ bool dneg(double x) { return __double_as_longlong(x) < 0; }
__device__ __forceinline__ bool abs_lt(double x, double t) { return dmag(x) < dmag(t); }
__device__ __forceinline__ bool abs_le(double x, double t) { return dmag(x) <= dmag(t); }
__device__ __forceinline__ bool gt_pos(double x, double t) { return !dneg(x) && dmag(x) > dmag(t); }
__device__ __forceinline__ bool lt_neg(double x, double t) { return dneg(x) && dmag(x) > dmag(t); }

__device__ int kepler_drift_fast(double r0v[3], double v0v[3], double gm, const double k[4],
                                 double dt, double dt2_6)
{
    const double sqrtgm = k[0], igm = k[1], isqrtgm = k[2], sgdt = k[3];
    const double r02 = fma(r0v[2], r0v[2], fma(r0v[1], r0v[1], r0v[0] * r0v[0]));
    const double v02 = fma(v0v[2], v0v[2], fma(v0v[1], v0v[1], v0v[0] * v0v[0]));
    const double ir0 = inv_sqrt_fast(r02);
    const double r0 = r02 * ir0;
    const double gmir0 = gm * ir0;
    const double alpha = fma(-v02, igm, ir0 + ir0);  // -2 xi / gm, xi = v0^2 / 2 - gm / r0
    const double rv = fma(r0v[2], v0v[2], fma(r0v[1], v0v[1], r0v[0] * v0v[0]));
    double chi0;
    const double w1 = sgdt * ir0;  // first-order arc
    if (abs_lt(w1 * w1 * alpha, 0.1)) {  // a short arc of any conic
        const double ir02 = ir0 * ir0;
        const double u = rv * ir02;                       // rdot / r
        const double w2 = -0.5 * u * dt;                  // second-order factor
        const double w3 = fma(v02 - gmir0, ir02, -3.0 * u * u);
        chi0 = w1 * fma(dt2_6, -w3, 1.0 + w2);
    } else if (alpha > TOL_ENERGY) {
        chi0 = sqrtgm * dt * alpha;
    } else if (alpha < TOL_ENERGY) {
        const double sma = 1.0 / alpha;
        double sg = (double)((dt > 0) - (dt < 0));
        chi0 = sg * (sqrt(-sma) * log(-2.0 * gm * alpha * dt / (rv + sqrt(-gm * sma) * (1.0 - r0 * alpha))));
    } else {
        double c0 = r0v[1] * v0v[2] - r0v[2] * v0v[1];
        double c1 = r0v[2] * v0v[0] - r0v[0] * v0v[2];
        double c2_ = r0v[0] * v0v[1] - r0v[1] * v0v[0];
        double cn = sqrt(c0 * c0 + c1 * c1 + c2_ * c2_);
        double p = cn * cn / gm;
        double s = 0.5 * atan(1.0 / (3.0 * sqrt(gm / cube_cr(p)) * dt));
        double w = atan(pow(tan(s), 1.0 / 3.0));
        chi0 = sqrt(p) * 2 / tan(2 * w);
    }
    double chi = 0.0, r = 0.0, c2 = 0.0, c3 = 0.0, psi = 0.0;
    const double rvs = rv * isqrtgm;
    for (int it = 0; it < KEPLER_MAX_IT; it++) {
        const double chi2 = chi0 * chi0;
        psi = chi2 * alpha;
        if (gt_pos(psi, 1.e-10) || lt_neg(psi, -1.e-6)) {
            if (abs_le(psi, 0.01)) stumpff_series_short(psi, c2, c3);
            else if (abs_le(psi, 0.5)) stumpff_series(psi, c2, c3);
            else stumpff(psi, c2, c3);
        } else {
            c2 = 0.5;
            c3 = 1.0 / 6.0;
        }
        const double s3 = fma(-psi, c3, 1.0), s2 = fma(-psi, c2, 1.0);
        r = fma(chi2, c2, fma(rvs * chi0, s3, r0 * s2));
        // sgdt - chi^3 c3 - rvs chi^2 c2 - r0 chi s3, nested
        const double num = fma(-chi0, fma(chi0, fma(chi0, c3, rvs * c2), r0 * s3), sgdt);
        chi = fma(num, rcp_fast(r), chi0);
        if (abs_lt(chi - chi0, KEPLER_TOL)) break;
        chi0 = chi;
    }
    const int failed = !abs_le(chi - chi0, KEPLER_TOL);
    const double chi2 = chi * chi;
    const double f = fma(-chi2 * ir0, c2, 1.0);
    const double g = fma(-chi2 * chi * isqrtgm, c3, dt);
    const double ir = rcp_fast(r);
    const double dg = fma(-chi2 * ir, c2, 1.0);
    const double df = sqrtgm * ir * ir0 * chi * fma(psi, c3, -1.0);
    double nr[3], nv[3];
    for (int c = 0; c < 3; c++) {
        nr[c] = fma(f, r0v[c], g * v0v[c]);
        nv[c] = fma(df, r0v[c], dg * v0v[c]);
    }
    for (int c = 0; c < 3; c++) {
        r0v[c] = nr[c];
        v0v[c] = nv[c];
    }
    return failed;
}

// One block.  init != 0: only Jacobi coordinates and accelerations (the
// set-up at the start of integrator_wh, :509-510); otherwise a full step.
// MODE as for the tail: the fast form divides by multiplying with
// rcp_fast, drifts with kepler_drift_fast and takes r^-3 from gm_inv_r3.
// The head is latency-bound (a few bodies, sequential prefixes), so its
// time is its FP64 instruction count on one warp.
template <int MODE>
__device__ __forceinline__ double wdiv(double x, double y)
{
    return MODE == ABIE_FORCE_EXACT ? x / y : x * rcp_fast(y);
}

// G m |(x, y, z)|^-3 in integer arithmetic (the fast form's pair term core).
__device__ __forceinline__ double wh_gm_ir3(double x, double y, double z, double gm)
{
    unsigned long long Mr;
    int Er;
    r2_int(x, y, z, Mr, Er);
    return gm_inv_r3_int(Mr, Er, gm);
}

template <int MODE>
__device__ __forceinline__ double wh_ir3(double x, double y, double z)
{
    if (MODE == ABIE_FORCE_EXACT) return 1.0 / cube_cr(norm3(x, y, z));
    unsigned long long Mr;
    int Er;
    r2_int(x, y, z, Mr, Er);
    return gm_inv_r3_int(Mr, Er, 1.0);
}

template <int MODE>
__global__ void __launch_bounds__(256) wh_head_kernel(WhArgs a, int init, int parity)
{
    const int H = a.head, n = a.n;
    const double dt = a.dt, half = dt / 2;
    const double *m = a.m;
    WhShared *sh = a.sh + parity;
    if (!init)
        for (int i = 1 + threadIdx.x; i < H; i += blockDim.x)
            for (int c = 0; c < 3; c++) a.vel[3 * i + c] += a.acc[3 * i + c] * half;
    __syncthreads();
    if (threadIdx.x == 0) {
        // interior masses and Kepler parameters (:174-191, :209-214)
        a.eta[0] = m[0];
        for (int i = 1; i < H; i++) a.eta[i] = m[i] + a.eta[i - 1];
        double eta0 = m[0];
        for (int i = 1; i < H; i++) {
            double eta = eta0 + m[i];
            a.gm[i] = a.G * m[0] * eta / eta0;
            eta0 = eta;
        }
        {
            double eta = eta0 + 0.0;
            const double gmt = a.G * m[0] * eta / eta0;
            sh->gm_tail = gmt;
            sh->gm_tail_k[0] = sqrt(gmt);
            sh->gm_tail_k[1] = 1.0 / gmt;
            sh->gm_tail_k[2] = 1.0 / sqrt(gmt);
            sh->gm_tail_k[3] = sqrt(gmt) * a.dt;
        }
        // helio -> Jacobi for the head (:206-265)
        double *jp = a.jpos, *jv = a.jvel;
        for (int c = 0; c < 3; c++) {
            jp[c] = 0.0;
            jv[c] = 0.0;
            jp[3 + c] = a.pos[3 + c];
            jv[3 + c] = a.vel[3 + c];
        }
        double aR[3], aV[3], R[3], V[3];
        for (int c = 0; c < 3; c++) {
            aR[c] = m[1] * a.pos[3 + c];
            aV[c] = m[1] * a.vel[3 + c];
            R[c] = wdiv<MODE>(aR[c], a.eta[1]);
            V[c] = wdiv<MODE>(aV[c], a.eta[1]);
        }
        for (int i = 2; i < H; i++) {
            for (int c = 0; c < 3; c++) {
                jp[3 * i + c] = a.pos[3 * i + c] - R[c];
                jv[3 * i + c] = a.vel[3 * i + c] - V[c];
            }
            if (i < n - 1) {
                for (int c = 0; c < 3; c++) {
                    aR[c] += (m[i] * a.pos[3 * i + c]);
                    aV[c] += (m[i] * a.vel[3 * i + c]);
                    R[c] = wdiv<MODE>(aR[c], a.eta[i]);
                    V[c] = wdiv<MODE>(aV[c], a.eta[i]);
                }
            }
        }
        for (int c = 0; c < 3; c++) {
            sh->R[c] = R[c];
            sh->V[c] = V[c];
        }
    }
    __syncthreads();
    if (!init) {
        // drift the head bodies (:174-191), independent given Jacobi states
        for (int i = 1 + threadIdx.x; i < H; i += blockDim.x) {
            double r[3] = {a.jpos[3 * i], a.jpos[3 * i + 1], a.jpos[3 * i + 2]};
            double v[3] = {a.jvel[3 * i], a.jvel[3 * i + 1], a.jvel[3 * i + 2]};
            int failed;
            if (MODE == ABIE_FORCE_EXACT) {
                failed = kepler_drift(r, v, a.gm[i], dt);
            } else {
                const double sg = sqrt(a.gm[i]);
                const double k[4] = {sg, 1.0 / a.gm[i], 1.0 / sg, sg * dt};
                failed = kepler_drift_fast(r, v, a.gm[i], k, dt, a.dt2_6);
            }
            if (failed) atomicAdd(&sh->kepler_failures, 1ull);
            for (int c = 0; c < 3; c++) {
                a.jpos[3 * i + c] = r[c];
                a.jvel[3 * i + c] = v[c];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // Jacobi -> helio for the head (:280-332)
            const double *jp = a.jpos, *jv = a.jvel;
            for (int c = 0; c < 3; c++) {
                a.pos[3 + c] = jp[3 + c];
                a.vel[3 + c] = jv[3 + c];
                a.pos[c] = 0.0;
                a.vel[c] = 0.0;
            }
            double R[3], V[3];
            for (int c = 0; c < 3; c++) {
                R[c] = wdiv<MODE>(m[1] * jp[3 + c], a.eta[1]);
                V[c] = wdiv<MODE>(m[1] * jv[3 + c], a.eta[1]);
            }
            for (int i = 2; i < H; i++) {
                for (int c = 0; c < 3; c++) {
                    a.pos[3 * i + c] = jp[3 * i + c] + R[c];
                    a.vel[3 * i + c] = jv[3 * i + c] + V[c];
                }
                if (i < n - 1) {
                    for (int c = 0; c < 3; c++) {
                        R[c] += wdiv<MODE>(m[i] * jp[3 * i + c], a.eta[i]);
                        V[c] += wdiv<MODE>(m[i] * jv[3 * i + c], a.eta[i]);
                    }
                }
            }
            for (int c = 0; c < 3; c++) {
                sh->Rp[c] = R[c];
                sh->Vp[c] = V[c];
            }
        }
        __syncthreads();
    }
    // the massive head bodies' positions of this step for the tail kernel
    // (its own copy, so the next step's head can run beside this tail)
    if (threadIdx.x == 0) {
        double *hs = a.hsrc + parity * 4 * WH_HEAD_MAX;
        int q = 0;
        for (int i = 1; i < H; i++) {
            if (m[i] == 0.0) continue;
            hs[4 * q] = a.pos[3 * i];
            hs[4 * q + 1] = a.pos[3 * i + 1];
            hs[4 * q + 2] = a.pos[3 * i + 2];
            hs[4 * q + 3] = a.G * m[i];
            q++;
        }
    }
    // accelerations of the head (:349-436)
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        double h = 0.0, j = 0.0;
        if (i >= 2) {
            if (MODE == ABIE_FORCE_EXACT) {
                h = cube_cr(1.0 / norm3(a.pos[3 * i], a.pos[3 * i + 1], a.pos[3 * i + 2]));
                j = cube_cr(1.0 / norm3(a.jpos[3 * i], a.jpos[3 * i + 1], a.jpos[3 * i + 2]));
            } else {
                h = wh_ir3<MODE>(a.pos[3 * i], a.pos[3 * i + 1], a.pos[3 * i + 2]);
                j = wh_ir3<MODE>(a.jpos[3 * i], a.jpos[3 * i + 1], a.jpos[3 * i + 2]);
            }
        }
        a.ir3h[i] = h;
        a.ir3j[i] = j;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ind[3] = {0.0, 0.0, 0.0};
        for (int i = 2; i < H; i++)
            for (int c = 0; c < 3; c++) ind[c] -= a.G * m[i] * a.pos[3 * i + c] * a.ir3h[i];
        double a2[3] = {0.0, 0.0, 0.0};
        double etai = m[0];
        for (int i = 2; i < H; i++) {
            etai += m[i - 1];
            for (int c = 0; c < 3; c++)
                a2[c] = a2[c] + wdiv<MODE>(a.G * m[i] * m[0] * a.ir3j[i], etai) * a.jpos[3 * i + c];
            for (int c = 0; c < 3; c++) a.acc[3 * i + c] = a2[c];  // temporarily: accel2[i]
        }
        for (int c = 0; c < 3; c++) {
            sh->ind[c] = ind[c];
            sh->a2[c] = a2[c];
            sh->ind_a2[c] = ind[c] + a2[c];
            a.acc[c] = 0.0;
            a.acc[3 + c] = 0.0;
        }
    }
    __syncthreads();
    // per head body: a3 in the reference's order (pairs with i < j first,
    // ascending, then pairs with k > j, ascending), then the sum
    for (int j = threadIdx.x; j < H; j += blockDim.x) {
        double a3[3] = {0.0, 0.0, 0.0};
        if (j >= 1) {
            for (int i = 1; i < j; i++) {
                if (m[i] == 0.0) continue;
                double d[3];
                for (int c = 0; c < 3; c++) d[c] = a.pos[3 * j + c] - a.pos[3 * i + c];
                double aux = wh_ir3<MODE>(d[0], d[1], d[2]);
                for (int c = 0; c < 3; c++) a3[c] -= a.G * m[i] * aux * d[c];
            }
            for (int k = j + 1; k < H; k++) {
                if (m[k] == 0.0) continue;
                double d[3];
                for (int c = 0; c < 3; c++) d[c] = a.pos[3 * k + c] - a.pos[3 * j + c];
                double aux = wh_ir3<MODE>(d[0], d[1], d[2]);
                for (int c = 0; c < 3; c++) a3[c] += a.G * m[k] * aux * d[c];
            }
        }
        for (int c = 0; c < 3; c++) {
            double ind = (j >= 1) ? sh->ind[c] : 0.0;
            double cent = 0.0;
            if (j >= 2)
                cent = a.G * m[0] * (a.jpos[3 * j + c] * a.ir3j[j] - a.pos[3 * j + c] * a.ir3h[j]);
            double acc2 = (j >= 2) ? a.acc[3 * j + c] : 0.0;
            double tot = ind + cent + acc2 + a3[c];
            a.acc[3 * j + c] = tot;
        }
    }
    __syncthreads();
    if (!init)
        for (int i = 1 + threadIdx.x; i < H; i += blockDim.x)
            for (int c = 0; c < 3; c++) a.vel[3 * i + c] += a.acc[3 * i + c] * half;
}

// One thread per tail body: the whole step (kick, Jacobi shift, drift, shift
// back, acceleration, kick) with the head's published quantities.
// MODE: ABIE_FORCE_EXACT keeps the reference's expressions (sqrt, divisions,
// correctly rounded cubes, closed-form Stumpff functions); the fast form
// uses kepler_drift_fast and the one-instruction r^-3 of the force kernels.
//
// ABIE_FORCE_MIXED is the fast form with the planets' pull on the particle
// in FP32 two-float arithmetic: heliocentric coordinates are relative to
// the star, which serves as the FP64 anchor; the particle's and each
// planet's coordinates and G m are split exactly into two floats (48
// bits), the separation, r^2, r^-1/2 (rsqrtf and one correction), r^-3 and
// the products are two-float operations, and each component's sum is a
// compensated two-float sum, added once to the FP64 indirect and accel2
// terms: about 2^-44 relative to the planet terms, no FP64 instruction per
// planet (the fast form spends six).
template <int MODE>
__global__ void __launch_bounds__(256) wh_tail_kernel(WhArgs a, int init, int parity, int n_src)
{
    extern __shared__ double hs[];  // 4 doubles per massive head body: x y z G*m
    // mixed form: the same values split into two floats, after the doubles
    float2 *hf = reinterpret_cast<float2 *>(hs + 4 * n_src);
    const int H = a.head;
    const double *hsrc = a.hsrc + parity * 4 * WH_HEAD_MAX;
    for (int e = threadIdx.x; e < 4 * n_src; e += blockDim.x) {
        hs[e] = hsrc[e];
        if (MODE == ABIE_FORCE_MIXED) hf[e] = split_ff(hsrc[e]);
    }
    __syncthreads();
    const long long i = (long long)H + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const WhShared *sh = a.sh + parity;
    const double half = a.dt / 2;
    double p[3], v[3], jp[3], jv[3];
    for (int c = 0; c < 3; c++) {
        p[c] = a.pos[3 * i + c];
        v[c] = a.vel[3 * i + c];
        if (!init) {
            if (MODE == ABIE_FORCE_EXACT) v[c] += a.acc[3 * i + c] * half;
            else v[c] = fma(a.acc[3 * i + c], half, v[c]);
        }
        jp[c] = p[c] - sh->R[c];
        jv[c] = v[c] - sh->V[c];
    }
    if (!init) {
        const int failed = MODE == ABIE_FORCE_EXACT ? kepler_drift(jp, jv, sh->gm_tail, a.dt)
                                                    : kepler_drift_fast(jp, jv, sh->gm_tail, sh->gm_tail_k, a.dt, a.dt2_6);
        if (failed) atomicAdd(&a.sh[parity].kepler_failures, 1ull);
        for (int c = 0; c < 3; c++) {
            p[c] = jp[c] + sh->Rp[c];
            v[c] = jv[c] + sh->Vp[c];
        }
    }
    double ir3h, ir3j;
    double a3[3] = {0.0, 0.0, 0.0};
    if (MODE == ABIE_FORCE_EXACT) {
        ir3h = cube_cr(1.0 / norm3(p[0], p[1], p[2]));
        ir3j = cube_cr(1.0 / norm3(jp[0], jp[1], jp[2]));
        for (int q = 0; q < n_src; q++) {
            double d[3];
            for (int c = 0; c < 3; c++) d[c] = p[c] - hs[4 * q + c];
            double aux = 1.0 / cube_cr(norm3(d[0], d[1], d[2]));
            for (int c = 0; c < 3; c++) a3[c] -= hs[4 * q + 3] * aux * d[c];
        }
    } else if (MODE == ABIE_FORCE_MIXED) {
        ir3h = wh_gm_ir3(p[0], p[1], p[2], a.G * a.m[0]);
        ir3j = wh_gm_ir3(jp[0], jp[1], jp[2], a.G * a.m[0]);
        const float2 px = split_ff(p[0]), py = split_ff(p[1]), pz = split_ff(p[2]);
        float S[3] = {0.0f, 0.0f, 0.0f}, C[3] = {0.0f, 0.0f, 0.0f};
        for (int q = 0; q < n_src; q++) {
            const float2 dx = ff_sub(px, hf[4 * q]), dy = ff_sub(py, hf[4 * q + 1]),
                         dz = ff_sub(pz, hf[4 * q + 2]);
            const float2 r2 = ff_add(ff_add(ff_sqr(dx), ff_sqr(dy)), ff_sqr(dz));
            const float2 y = ff_rsqrt(r2);
            const float2 w = ff_mul(hf[4 * q + 3], ff_mul(ff_sqr(y), y));  // G m r^-3
            const float2 nw = make_float2(-w.x, -w.y);
            ff_add_product(nw, dx, S[0], C[0]);
            ff_add_product(nw, dy, S[1], C[1]);
            ff_add_product(nw, dz, S[2], C[2]);
        }
        for (int c = 0; c < 3; c++)
            a3[c] = sh->ind_a2[c] + (f32_to_f64_exact(S[c]) + f32_to_f64_exact(C[c]));
    } else {
        // G m0 folded into the inverse cubes; the planets' sum starts from
        // the indirect and accel2 terms
        ir3h = wh_gm_ir3(p[0], p[1], p[2], a.G * a.m[0]);
        ir3j = wh_gm_ir3(jp[0], jp[1], jp[2], a.G * a.m[0]);
        for (int c = 0; c < 3; c++) a3[c] = sh->ind_a2[c];
        for (int q = 0; q < n_src; q++) {
            Src sq{hs[4 * q], hs[4 * q + 1], hs[4 * q + 2], hs[4 * q + 3]};
            pair_fast(p[0], p[1], p[2], sq, a3[0], a3[1], a3[2]);
        }
    }
    const double Gm0 = a.G * a.m[0];
    for (int c = 0; c < 3; c++) {
        double acc;
        if (MODE == ABIE_FORCE_EXACT) {
            const double cent = Gm0 * (jp[c] * ir3j - p[c] * ir3h);
            acc = sh->ind[c] + cent + sh->a2[c] + a3[c];
        } else {
            acc = a3[c] + fma(jp[c], ir3j, -p[c] * ir3h);
        }
        a.acc[3 * i + c] = acc;
        if (!init) {
            if (MODE == ABIE_FORCE_EXACT) v[c] += acc * half;
            else v[c] = fma(acc, half, v[c]);
        }
        a.pos[3 * i + c] = p[c];
        a.vel[3 * i + c] = v[c];
    }
}

struct WhBuffers {
    double *acc = nullptr, *scratch = nullptr;
    size_t acc_n = 0;
    WhShared *sh = nullptr;  // two sets
    cudaStream_t tail_stream = nullptr;
    cudaEvent_t ev_head = nullptr, ev_tail[2] = {nullptr, nullptr};
};
static WhBuffers g_wh;

void free_wh_buffers()
{
    if (g_wh.acc) cudaFree(g_wh.acc);
    if (g_wh.scratch) cudaFree(g_wh.scratch);
    if (g_wh.sh) cudaFree(g_wh.sh);
    if (g_wh.ev_head) cudaEventDestroy(g_wh.ev_head);
    for (int k = 0; k < 2; k++)
        if (g_wh.ev_tail[k]) cudaEventDestroy(g_wh.ev_tail[k]);
    if (g_wh.tail_stream) cudaStreamDestroy(g_wh.tail_stream);
    g_wh = WhBuffers();
}

static void wh_launch_head(const WhArgs &a, int init, int parity, int mode, cudaStream_t st)
{
    if (mode == ABIE_FORCE_EXACT) wh_head_kernel<ABIE_FORCE_EXACT><<<1, 256, 0, st>>>(a, init, parity);
    else wh_head_kernel<ABIE_FORCE_FP64><<<1, 256, 0, st>>>(a, init, parity);
}

// Dynamic shared memory of the tail kernel: the massive head bodies as
// doubles, and in the mixed form also as two-float pairs.
static size_t wh_tail_smem(int n_src, int mode)
{
    const size_t k = 4 * (size_t)std::max(n_src, 1);
    return k * sizeof(double) + (mode == ABIE_FORCE_MIXED ? k * sizeof(float2) : 0);
}

static void wh_launch_tail(const WhArgs &a, int init, int parity, int n_src, int mode, cudaStream_t st)
{
    long long tail = (long long)a.n - a.head;
    if (tail <= 0) return;
    unsigned blocks = (unsigned)((tail + 255) / 256);
    size_t smem = 4 * sizeof(double) * (size_t)std::max(n_src, 1);
    if (mode == ABIE_FORCE_EXACT)
        wh_tail_kernel<ABIE_FORCE_EXACT><<<blocks, 256, smem, st>>>(a, init, parity, n_src);
    else if (mode == ABIE_FORCE_MIXED)
        wh_tail_kernel<ABIE_FORCE_MIXED><<<blocks, 256, wh_tail_smem(n_src, mode), st>>>(a, init, parity,
                                                                                         n_src);
    else
        wh_tail_kernel<ABIE_FORCE_FP64><<<blocks, 256, smem, st>>>(a, init, parity, n_src);
}

// count steps: heads on st, tails on the tail stream.  The massive bodies
// never feel the test particles, so head k+1 runs beside tail k; step
// parity selects the published set, and head k waits for tail k-2, the
// last reader of its set.  Ends with st waiting for the last tail.
static int wh_launch_steps(const WhArgs &a, int count, int n_src, int mode, cudaStream_t st)
{
    cudaStream_t st2 = g_wh.tail_stream;
    for (int k = 0; k < count; k++) {
        const int par = k & 1;
        if (k >= 2) ABIE_CUDA(cudaStreamWaitEvent(st, g_wh.ev_tail[par], 0));
        wh_launch_head(a, 0, par, mode, st);
        ABIE_CUDA(cudaEventRecord(g_wh.ev_head, st));
        ABIE_CUDA(cudaStreamWaitEvent(st2, g_wh.ev_head, 0));
        wh_launch_tail(a, 0, par, n_src, mode, st2);
        ABIE_CUDA(cudaEventRecord(g_wh.ev_tail[par], st2));
    }
    if (count > 0) ABIE_CUDA(cudaStreamWaitEvent(st, g_wh.ev_tail[(count - 1) & 1], 0));
    return 0;
}

int wh_run(const SystemView &sys, double t, double t_end, double dt, double *t_out,
           abie_counters *ctr, cudaStream_t st)
{
    const int n = sys.n;
    if (n < 2) {
        set_error(ABIE_ERR_ARGUMENT, "integrator_wh needs at least two bodies (N=%d)", n);
        return ABIE_ERR_ARGUMENT;
    }
    int last = 1;
    for (int i = 0; i < n; i++)
        if (sys.h_m[i] != 0.0) last = std::max(last, i);
    int H = last + 1;
    if (H > WH_HEAD_MAX) {
        set_error(ABIE_ERR_CAPACITY, "integrator_wh: %d bodies before the last massive one (max %d)",
                  H, WH_HEAD_MAX);
        return ABIE_ERR_CAPACITY;
    }
    int n_src = 0;
    for (int i = 1; i < H; i++) n_src += (sys.h_m[i] != 0.0);
    int rc;
    if ((rc = reserve(&g_wh.acc, &g_wh.acc_n, 3 * (size_t)n))) return rc;
    if (!g_wh.scratch) ABIE_CUDA(cudaMalloc(&g_wh.scratch, (size_t)WH_HEAD_MAX * 18 * sizeof(double)));
    if (!g_wh.sh) ABIE_CUDA(cudaMalloc(&g_wh.sh, 2 * sizeof(WhShared)));
    if (!g_wh.tail_stream) {
        ABIE_CUDA(cudaStreamCreateWithFlags(&g_wh.tail_stream, cudaStreamNonBlocking));
        ABIE_CUDA(cudaEventCreateWithFlags(&g_wh.ev_head, cudaEventDisableTiming));
        for (int k = 0; k < 2; k++) ABIE_CUDA(cudaEventCreateWithFlags(&g_wh.ev_tail[k], cudaEventDisableTiming));
    }
    ABIE_CUDA(cudaMemsetAsync(g_wh.sh, 0, 2 * sizeof(WhShared), st));
    WhArgs a;
    a.n = n;
    a.head = H;
    a.G = sys.G;
    a.dt = dt;
    a.dt2_6 = dt * dt / 6.0;
    a.pos = sys.pos;
    a.vel = sys.vel;
    a.acc = g_wh.acc;
    a.m = sys.m;
    double *s = g_wh.scratch;
    a.jpos = s;
    a.jvel = s + 3 * WH_HEAD_MAX;
    a.eta = s + 6 * WH_HEAD_MAX;
    a.gm = s + 7 * WH_HEAD_MAX;
    a.ir3h = s + 8 * WH_HEAD_MAX;
    a.ir3j = s + 9 * WH_HEAD_MAX;
    a.sh = g_wh.sh;
    a.hsrc = s + 10 * WH_HEAD_MAX;  // 2 x 4 x WH_HEAD_MAX

    long long steps = 0;
    double tt = t;
    while (tt < t_end) {  // :513-520, the same accumulation of t
        tt += dt;
        steps++;
    }
    const int mode = g_sim.force_mode;
    if (mode == ABIE_FORCE_NAIVE) {
        set_error(ABIE_ERR_UNSUPPORTED,
                  "integrator_wh: the naive force form is the force comparator only; use the exact, "
                  "fp64 or mixed form");
        return ABIE_ERR_UNSUPPORTED;
    }
    size_t smem = wh_tail_smem(n_src, mode);
    if (smem > 48 * 1024) {  // up to WH_HEAD_MAX massive head bodies
        ABIE_CUDA(cudaFuncSetAttribute(wh_tail_kernel<ABIE_FORCE_EXACT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ABIE_CUDA(cudaFuncSetAttribute(wh_tail_kernel<ABIE_FORCE_FP64>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ABIE_CUDA(cudaFuncSetAttribute(wh_tail_kernel<ABIE_FORCE_MIXED>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    // set-up (:509-510): Jacobi coordinates and accelerations, in order
    wh_launch_head(a, 1, 0, mode, st);
    wh_launch_tail(a, 1, 0, n_src, mode, st);
    ABIE_CUDA(cudaGetLastError());
    if (steps > 0) {
        const int CH = 32;  // steps per captured graph (even: parities line up)
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        long long full = steps / CH;
        if (full > 0) {
            ABIE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            rc = wh_launch_steps(a, CH, n_src, mode, st);
            cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            ABIE_CUDA(ce);
            ABIE_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            for (long long k = 0; k < full; k++) ABIE_CUDA(cudaGraphLaunch(exec, st));
        }
        rc = wh_launch_steps(a, (int)(steps - full * CH), n_src, mode, st);
        if (rc) return rc;
        ABIE_CUDA(cudaGetLastError());
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
    WhShared h[2];
    ABIE_CUDA(cudaMemcpyAsync(h, g_wh.sh, sizeof h, cudaMemcpyDeviceToHost, st));
    ABIE_CUDA(cudaStreamSynchronize(st));
    if (ctr) {
        ctr->kepler_failures += (long long)(h[0].kepler_failures + h[1].kepler_failures);
        ctr->wh_steps += steps;
    }
    *t_out = tt;
    return 0;
}

}  // namespace abie

using namespace abie;

extern "C" {

int integrator_wh(double t, double t_end, double dt)
{
    Sim &s = g_sim;
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "integrator_wh before initialize_code");
        return ABIE_ERR_NOT_INITIALIZED;
    }
    SystemView v{s.pos, s.vel, s.m, s.r, nullptr, s.h_m.data(), s.h_r.data(), (int)s.n, s.G};
    double t_out = t;
    int rc = wh_run(v, t, t_end, dt, &t_out, &s.ctr, s.st);
    if (rc == 0 && t_out != t) s.t = t_out;
    return rc;
}

void integrator_wisdom_holman(double *pos, double *vel, double *m_vec, double *r_vec, size_t N,
                              double G, double t, double t_end, double dt)
{
    if (ensure_device(-1)) return;
    Sim &s = g_sim;
    N &= 0xffffffffull;
    double *dp = nullptr, *dv = nullptr, *dm = nullptr;
    size_t cp = 0, cv = 0, cm = 0;
    if (reserve(&dp, &cp, 3 * N) || reserve(&dv, &cv, 3 * N) || reserve(&dm, &cm, N)) return;
    cudaMemcpy(dp, pos, 3 * N * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dv, vel, 3 * N * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dm, m_vec, N * 8, cudaMemcpyHostToDevice);
    SystemView v{dp, dv, dm, nullptr, nullptr, m_vec, r_vec, (int)N, G};
    double t_out = t;
    if (wh_run(v, t, t_end, dt, &t_out, &s.ctr, s.st) == 0) {
        cudaMemcpy(pos, dp, 3 * N * 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(vel, dv, 3 * N * 8, cudaMemcpyDeviceToHost);
        if (t_out != t) s.t = t_out;
    }
    cudaFree(dp);
    cudaFree(dv);
    cudaFree(dm);
}

}  // extern "C"
