// Gauss-Radau 15 on the device for one system of any size.
//
// The reference (src/integrator_gauss_radau15.c:221-380) loops on the host
// and calls the force on every Radau substep, copying positions to the GPU
// and accelerations back each time (src/gpuforce.cu:142-156).  Here the
// whole predictor-corrector sweep runs inside one cooperative persistent
// kernel: per-body state (y0, dy0, F1, b[7], g[7], ...) stays in GPU memory,
// every thread group owns a fixed set of bodies, and the grid meets at a
// software barrier (bounded wait) once per Radau substep.  Scalars that
// steer the sweep (t, h, convergence, accept/reject) are computed by every
// thread from the same reduced values, so control flow stays uniform.
//
// The per-component arithmetic repeats the reference's expressions in the
// reference's order, and the translation unit is built with --fmad=false,
// so with the exact force form each substep reproduces the reference's
// doubles; the step-size exponentiation uses the device pow(), which may
// differ from the host libm in the last bit.
//
// A call runs as a series of launches, each bounded to a number of step
// attempts (sized from the measured time of the previous launch), so no
// launch holds the GPU for long and every wait has a limit.
//
// Three paths share the per-component device functions: the split engine
// (radau_split, at most 10 massive bodies: a replica of them per block, no
// grid barrier per substep), the persistent engine (radau_engine), and,
// from 2^20 interactions per force evaluation in the fast form without
// post-Newtonian terms, the stepped engine (st_* kernels driven from the
// host, the standalone force kernel for every substep), which below 8,192
// bodies gives the persistent engine's doubles.
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "abi_state.cuh"
#include "engine.cuh"
#include "pn.cuh"
#include "radau_comp.cuh"
#include "radau_constants.h"
#include "mixed.cuh"

namespace abie {

__constant__ double c_hs[8] = ABIE_RADAU_HS_INIT;
__constant__ double c_rs[8][8] = ABIE_RADAU_RS_INIT;
__constant__ double c_cs[8][8] = ABIE_RADAU_CS_INIT;
__constant__ double c_rsp[8][8] = ABIE_RADAU_RSP_INIT;  // fast form: expanded g recurrence
__constant__ double c_wg[9][7] = ABIE_RADAU_WG_INIT;    // fast form: position weights on g
__constant__ double c_vg[7] = ABIE_RADAU_VG_INIT;       // fast form: velocity weights on g at spacing 1

// EPSB, FAC, TOLPC, H_MIN (src/integrator_gauss_radau15.h:17-63): radau_comp.cuh

struct EventRec {
    int j, k, kind;  // kind 0: close encounter, 1: collision
    double sep;
};

struct EngineCtl {
    unsigned int bar;
    int err;
    int flag;
    int n_ev;
    unsigned long long red[4][4];
    // resumable scalars
    double t, h;
    int loop_count;
    int phase;  // 0: not started, 1: running, 2: done
    int pc;     // publish counter (which position buffer is current)
    int red_idx;
    long long attempts_done;
    // counters
    long long force_calls, iterations, attempts, accepts, rejects;
    unsigned long long n_ce, n_coll;
    int ev_overflow;
    int hmin_warned;
    // stepped engine (host-driven): source count, sink counter of the force
    // kernel, and the step control's decision for the host
    int n_src;
    unsigned int next_sink;
    int accepted, stop;
    double q, dt0, d1;
};

struct EngineArgs {
    int n, dim, n_src;
    const int *src_body;  // [n_src] body index of each massive body, ascending
    const int *src_slot;  // [n] slot in the source list or -1
    const int *tp_body;   // [n_tp] bodies without positive mass, ascending (split engine)
    int n_tp;
    double C;             // speed of light: post-Newtonian terms when > 0
    PnConst pn;
    const double *m, *r, *ext;
    double G;
    double *y0, *dy0, *F1, *b, *g, *b6p, *ddy, *dyp;
    double *yp[2], *ypa;
    double *vp[2];  // predicted velocities of the published substeps (post-Newtonian terms only)
    float2 *ypf;  // [3n] accepted positions as {float, bound on its error} for the event prefilter
    Src *src[2], *srca;
    double t_end;
    double ce_dist, thr2;
    long long max_ce, max_coll;
    double *buf_ce, *buf_coll;
    EventRec *ev;
    int ev_cap;
    EngineCtl *ctl;
    long long timeout_ns;
    long long attempt_budget;
};

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier: block 0 adds 2^31 - (nblocks - 1), every other block adds 1,
// so the top bit of the counter flips exactly when all blocks have arrived.
// The wait is bounded; on timeout the error word is set and every block
// leaves at its next barrier.  Thread 0 alone reads the error word and hands
// its verdict to the block through shared memory, so all threads of a block
// leave (or go on) together.  The clock is read every 256 spins, or every
// spin for limits below a millisecond (set only by the debug setter).
__device__ __forceinline__ bool grid_sync(EngineCtl *ctl, long long timeout_ns)
{
    __shared__ int s_grid_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int nb = gridDim.x;
        unsigned int inc = (blockIdx.x == 0) ? (0x80000000u - (nb - 1u)) : 1u;
        const unsigned int every = timeout_ns < 1000000ll ? 0u : 255u;
        __threadfence();
        unsigned int old = atomicAdd(&ctl->bar, inc);
        unsigned long long t0 = gtimer();
        unsigned int spins = 0;
        while (((*(volatile unsigned int *)&ctl->bar ^ old) & 0x80000000u) == 0u) {
            if ((++spins & every) == 0u) {
                if (*(volatile int *)&ctl->err) break;
                if (gtimer() - t0 > (unsigned long long)timeout_ns) {
                    atomicCAS(&ctl->err, 0, ABIE_ERR_TIMEOUT);
                    break;
                }
            }
        }
        __threadfence();
        s_grid_ok = *(volatile int *)&ctl->err == 0;
    }
    __syncthreads();
    return s_grid_ok != 0;
}

__device__ __forceinline__ Src load_src(const Src *p)
{
    double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
    double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
    Src s;
    s.x = a.x;
    s.y = a.y;
    s.z = b.x;
    s.gm = b.y;
    return s;
}

// Acceleration of sink j from the published sources, returned to every
// lane of the sink's group.  EXACT: lane 0 alone, in the reference's order
// and operations, then broadcast.  Otherwise the JS lanes split the sources
// and meet in a shuffle butterfly.  All 32 lanes of the warp call this
// together (the sink loops are warp-uniform).
template <int MODE, int JS>
__device__ __forceinline__ void sink_accel(const EngineArgs &a, int j, const Src *src, double xj,
                                           double yj, double zj, int lane, double &ax, double &ay,
                                           double &az)
{
    ax = 0.0;
    ay = 0.0;
    az = 0.0;
    if (MODE == ABIE_FORCE_EXACT) {
        if (lane == 0) {
            for (int q = 0; q < a.n_src; q++) {
                if (a.src_body[q] == j) continue;
                pair_exact(xj, yj, zj, load_src(src + q), ax, ay, az);
            }
        }
        if (JS > 1) {
            ax = __shfl_sync(0xffffffffu, ax, 0, JS);
            ay = __shfl_sync(0xffffffffu, ay, 0, JS);
            az = __shfl_sync(0xffffffffu, az, 0, JS);
        }
    } else {
        int q = lane;
        for (; q + JS < a.n_src; q += 2 * JS) {
            Src s0 = load_src(src + q), s1 = load_src(src + q + JS);
            pair_fast(xj, yj, zj, s0, ax, ay, az);
            pair_fast(xj, yj, zj, s1, ax, ay, az);
        }
        if (q < a.n_src) pair_fast(xj, yj, zj, load_src(src + q), ax, ay, az);
        if (JS > 1) {
#pragma unroll
            for (int o = JS / 2; o > 0; o >>= 1) {
                ax += __shfl_xor_sync(0xffffffffu, ax, o, JS);
                ay += __shfl_xor_sync(0xffffffffu, ay, o, JS);
                az += __shfl_xor_sync(0xffffffffu, az, o, JS);
            }
        }
    }
}

// Post-Newtonian sum of the massive sources on sink j (src/additional_forces.c:14-121):
// source positions from the list src, velocities from vel (3n, the same
// evaluation's), masses from m.  The exact form sums in source order on lane
// 0, as the reference's loop over k; the fast form spreads the sources over
// the JS lanes.
template <int MODE, int JS>
__device__ __noinline__ void sink_pn(const EngineArgs &a, int j, const Src *src, const double *vel,
                                     double xj, double yj, double zj, int lane, double &ax,
                                     double &ay, double &az)
{
    ax = 0.0;
    ay = 0.0;
    az = 0.0;
    const double vxj = vel[3 * j], vyj = vel[3 * j + 1], vzj = vel[3 * j + 2], mj = a.m[j];
    const int q0 = MODE == ABIE_FORCE_EXACT ? 0 : lane;
    const int qs = MODE == ABIE_FORCE_EXACT ? 1 : JS;
    if (MODE != ABIE_FORCE_EXACT || lane == 0) {
        for (int q = q0; q < a.n_src; q += qs) {
            const int k = a.src_body[q];
            if (k == j) continue;
            const Src sk = load_src(src + q);
            pn_term<MODE>(a.pn, xj, yj, zj, vxj, vyj, vzj, mj, sk.x, sk.y, sk.z, vel[3 * k],
                    vel[3 * k + 1], vel[3 * k + 2], a.m[k], ax, ay, az);
        }
    }
    if (JS > 1) {
        if (MODE == ABIE_FORCE_EXACT) {
            ax = __shfl_sync(0xffffffffu, ax, 0, JS);
            ay = __shfl_sync(0xffffffffu, ay, 0, JS);
            az = __shfl_sync(0xffffffffu, az, 0, JS);
        } else {
#pragma unroll
            for (int o = JS / 2; o > 0; o >>= 1) {
                ax += __shfl_xor_sync(0xffffffffu, ax, o, JS);
                ay += __shfl_xor_sync(0xffffffffu, ay, o, JS);
                az += __shfl_xor_sync(0xffffffffu, az, o, JS);
            }
        }
    }
}

// Newton, plus the post-Newtonian sum when C > 0 (velocities vel), as
// src/common.c:82-114 adds them; the caller adds the external acceleration.
template <int MODE, int JS, bool PN>
__device__ __forceinline__ void sink_force(const EngineArgs &a, int j, const Src *src,
                                           const double *vel, double xj, double yj, double zj,
                                           int lane, double f[3])
{
    sink_accel<MODE, JS>(a, j, src, xj, yj, zj, lane, f[0], f[1], f[2]);
    if (PN) {
        double px, py, pz;
        sink_pn<MODE, JS>(a, j, src, vel, xj, yj, zj, lane, px, py, pz);
        f[0] += px;
        f[1] += py;
        f[2] += pz;
    }
}

// f[c] without a dynamically indexed local array.
__device__ __forceinline__ double pick3(const double f[3], int c)
{
    return c == 0 ? f[0] : (c == 1 ? f[1] : f[2]);
}

// Components of a body handled by a lane of its group: with JS >= 4 lanes
// 0, 1, 2 take x, y, z; with JS == 1 the single lane takes all three.
template <int JS>
__device__ __forceinline__ int comp_lo(int lane) { return JS >= 4 ? lane : 0; }
template <int JS>
__device__ __forceinline__ int comp_hi(int lane) { return JS >= 4 ? (lane < 3 ? lane + 1 : 0) : 3; }

// Predicted position of component i at spacing s = c_hs[row] (row 8:
// s = 1) of a step dt (src/integrator_gauss_radau15.c:56-68).  Exact
// form: the reference's Horner polynomial in b with its divisions by
// constants.  Fast form: the same polynomial on the Newton-form
// coefficients g (b = C g), y0 + ds dy0 + hh (F1 + sum_j g_j W_j(s)), the
// weights tabulated and ds = dt s, hh = ds^2 / 2 computed once per substep
// (10 FP64 instructions instead of 19, and b is not needed in the corrector).
template <int MODE>
__device__ __forceinline__ double pred_pos(const EngineArgs &a, int i, int row, double s, double dt,
                                           double ds, double hh)
{
    const int d = a.dim;
    if (MODE == ABIE_FORCE_EXACT) {
        const double *b = a.b;
        return a.y0[i] + dt * s * (a.dy0[i] + dt * s * (a.F1[i] + s * (b[i] / 0.3e1 + s * (b[d + i] / 0.6e1 + s * (b[2 * d + i] / 0.10e2 + s * (b[3 * d + i] / 0.15e2 + s * (b[4 * d + i] / 0.21e2 + s * (b[5 * d + i] / 0.28e2 + s * b[6 * d + i] / 0.36e2))))))) / 0.2e1);
    }
    const double *g = a.g;
    const double *w = c_wg[row];
    double u = g[6 * d + i] * w[6];
    u = fma(g[5 * d + i], w[5], u);
    u = fma(g[4 * d + i], w[4], u);
    u = fma(g[3 * d + i], w[3], u);
    u = fma(g[2 * d + i], w[2], u);
    u = fma(g[d + i], w[1], u);
    u = fma(g[i], w[0], u);
    return fma(hh, a.F1[i] + u, fma(ds, a.dy0[i], a.y0[i]));
}

// Predicted velocity at spacing 1 (the advance).
template <int MODE>
__device__ __forceinline__ double pred_vel(const EngineArgs &a, int i, double dt)
{
    const int d = a.dim;
    if (MODE == ABIE_FORCE_EXACT) {
        const double *b = a.b;
        const double s = 1.0;
        return a.dy0[i] + dt * s * (a.F1[i] + s * (b[i] / 0.2e1 + s * (b[d + i] / 0.3e1 + s * (b[2 * d + i] / 0.4e1 + s * (b[3 * d + i] / 0.5e1 + s * (b[4 * d + i] / 0.6e1 + s * (b[5 * d + i] / 0.7e1 + s * b[6 * d + i] / 0.8e1)))))));
    }
    const double *g = a.g;
    double u = g[6 * d + i] * c_vg[6];
    u = fma(g[5 * d + i], c_vg[5], u);
    u = fma(g[4 * d + i], c_vg[4], u);
    u = fma(g[3 * d + i], c_vg[3], u);
    u = fma(g[2 * d + i], c_vg[2], u);
    u = fma(g[d + i], c_vg[1], u);
    u = fma(g[i], c_vg[0], u);
    return fma(dt, a.F1[i] + u, a.dy0[i]);
}

// Predicted velocity at spacing s = c_hs[row] (src/integrator_gauss_radau15.c:63-68),
// needed only by the post-Newtonian terms.  Fast form: from g with the
// tabulated weights of that spacing.
template <int MODE>
__device__ __forceinline__ double pred_vel_at(const EngineArgs &a, int i, int row, double s, double dt)
{
    const int d = a.dim;
    if (MODE == ABIE_FORCE_EXACT) {
        const double *b = a.b;
        return a.dy0[i] + dt * s * (a.F1[i] + s * (b[i] / 0.2e1 + s * (b[d + i] / 0.3e1 + s * (b[2 * d + i] / 0.4e1 + s * (b[3 * d + i] / 0.5e1 + s * (b[4 * d + i] / 0.6e1 + s * (b[5 * d + i] / 0.7e1 + s * b[6 * d + i] / 0.8e1)))))));
    }
    const double *g = a.g;
    const double *w = e_vgs[row];
    double u = g[6 * d + i] * w[6];
    u = fma(g[5 * d + i], w[5], u);
    u = fma(g[4 * d + i], w[4], u);
    u = fma(g[3 * d + i], w[3], u);
    u = fma(g[2 * d + i], w[2], u);
    u = fma(g[d + i], w[1], u);
    u = fma(g[i], w[0], u);
    return fma(dt * s, a.F1[i] + u, a.dy0[i]);
}

// The corrector's b6 (b_6 = cs[6][6] g_6 = g_6: read from g in the fast form).
template <int MODE>
__device__ __forceinline__ double b6_at(const EngineArgs &a, int i)
{
    return MODE == ABIE_FORCE_EXACT ? a.b[6 * a.dim + i] : a.g[6 * a.dim + i];
}

// The accepted coordinate p as the nearest float and an upper bound on the
// rounding error, for the event scan's single-precision prefilter.
__device__ __forceinline__ void put_prefilter(const EngineArgs &a, int i, double p)
{
    const float f = __double2float_rn(p);
    a.ypf[i] = make_float2(f, __double2float_ru(fabs(p - (double)f)));
}

// Predicted component c of body j into yp, and into the source list when j
// is massive (lane of component 0 also writes G m).
template <int MODE>
__device__ __forceinline__ void publish_comp(const EngineArgs &a, int j, int c, int row, double s,
                                             double dt, double ds, double hh, double *yp, Src *src,
                                             double *vp = nullptr)
{
    const int i = 3 * j + c;
    const double p = pred_pos<MODE>(a, i, row, s, dt, ds, hh);
    yp[i] = p;
    if (vp) vp[i] = pred_vel_at<MODE>(a, i, row, s, dt);
    if (row == 8) put_prefilter(a, i, p);
    const int slot = a.src_slot[j];
    if (slot >= 0) {
        double *rec = reinterpret_cast<double *>(src + slot);
        rec[c] = p;
        if (c == 0) rec[3] = a.G * a.m[j];
    }
}

// Exact form: g and b after the force F at substep IH (1..7) for component
// i (src/integrator_gauss_radau15.c:70-175; only g[IH-1] is new, the lower
// g the reference recomputes are bitwise the stored ones), in the
// reference's order and roundings.  Fast form: only g[IH-1], from the
// expanded recurrence (F - F1) rsp[IH][0] - sum_{l<IH-1} g_l rsp[IH][l+1];
// b is formed from g once per accepted step.  One static variant per
// substep keeps every index a constant.
template <int MODE, int IH>
__device__ __forceinline__ void gb_update_ih(const EngineArgs &a, int i, double F)
{
    const int d = a.dim;
    double *g = a.g;
    if (MODE == ABIE_FORCE_EXACT) {
        double gl[7];
#pragma unroll
        for (int k = 0; k < 7; k++) gl[k] = g[k * d + i];
        double v = (F - a.F1[i]) * c_rs[IH][0];
#pragma unroll
        for (int l = 1; l < IH; l++) v = (v - gl[l - 1]) * c_rs[IH][l];
        g[(IH - 1) * d + i] = v;
        gl[IH - 1] = v;
#pragma unroll
        for (int k = 0; k < IH; k++) {
            double s = c_cs[k][k] * gl[k];
#pragma unroll
            for (int jj = k + 1; jj < 7; jj++) s = s + c_cs[jj][k] * gl[jj];  // reference roundings
            a.b[k * d + i] = s;
        }
        return;
    }
    double v = (F - a.F1[i]) * c_rsp[IH][0];
#pragma unroll
    for (int l = 1; l < IH; l++) v = fma(-g[(l - 1) * d + i], c_rsp[IH][l], v);
    g[(IH - 1) * d + i] = v;
}

template <int MODE>
__device__ __forceinline__ void gb_update(const EngineArgs &a, int i, int ih, double F)
{
    switch (ih) {
    case 1: gb_update_ih<MODE, 1>(a, i, F); break;
    case 2: gb_update_ih<MODE, 2>(a, i, F); break;
    case 3: gb_update_ih<MODE, 3>(a, i, F); break;
    case 4: gb_update_ih<MODE, 4>(a, i, F); break;
    case 5: gb_update_ih<MODE, 5>(a, i, F); break;
    case 6: gb_update_ih<MODE, 6>(a, i, F); break;
    default: gb_update_ih<MODE, 7>(a, i, F); break;
    }
}

// Fast form at an accepted step: b = C g, the previous-b6 record, the
// reference's refine_bs guess E(q), and g = C^-1 E so that the next step's
// corrector starts from the polynomial the guess describes.
__device__ __forceinline__ void refine_g(const EngineArgs &a, int i, double q, bool last)
{
    const int d = a.dim;
    double gl[7], b[7];
#pragma unroll
    for (int k = 0; k < 7; k++) gl[k] = a.g[k * d + i];
#pragma unroll
    for (int k = 0; k < 7; k++) {
        double s = gl[k];  // cs[k][k] = 1
#pragma unroll
        for (int j = k + 1; j < 7; j++) s = fma(c_cs[j][k], gl[j], s);
        b[k] = s;
    }
    a.b6p[i] = b[6];
    if (last) return;
    double q2 = q * q, q3 = q2 * q, q4 = q2 * q2, q5 = q2 * q3, q6 = q3 * q3, q7 = q2 * q5;
    double e[7];
    e[0] = q * (b[6] * 7.0 + b[5] * 6.0 + b[4] * 5.0 + b[3] * 4.0 + b[2] * 3.0 + b[1] * 2.0 + b[0]);
    e[1] = q2 * (b[6] * 21.0 + b[5] * 15.0 + b[4] * 10.0 + b[3] * 6.0 + b[2] * 3.0 + b[1]);
    e[2] = q3 * (b[6] * 35.0 + b[5] * 20.0 + b[4] * 10.0 + b[3] * 4.0 + b[2]);
    e[3] = q4 * (b[6] * 35.0 + b[5] * 15.0 + b[4] * 5.0 + b[3]);
    e[4] = q5 * (b[6] * 21.0 + b[5] * 6.0 + b[4]);
    e[5] = q6 * (b[6] * 7.0 + b[5]);
    e[6] = q7 * b[6];
#pragma unroll
    for (int k = 6; k >= 0; k--) {
        double v = e[k];
#pragma unroll
        for (int j = k + 1; j < 7; j++) v -= c_cs[j][k] * gl[j];
        gl[k] = v;
        a.g[k * d + i] = v;
    }
}

// src/integrator_gauss_radau15.c:178-218 (bd is always zero there).
__device__ __forceinline__ void refine_b(const EngineArgs &a, int i, double q)
{
    const int d = a.dim;
    double *b = a.b;
    double b0 = b[i], b1 = b[d + i], b2 = b[2 * d + i], b3 = b[3 * d + i], b4 = b[4 * d + i],
           b5 = b[5 * d + i], b6 = b[6 * d + i];
    double q2 = q * q, q3 = q2 * q, q4 = q2 * q2, q5 = q2 * q3, q6 = q3 * q3, q7 = q2 * q5;
    double e0 = q * (b6 * 7.0 + b5 * 6.0 + b4 * 5.0 + b3 * 4.0 + b2 * 3.0 + b1 * 2.0 + b0);
    double e1 = q2 * (b6 * 21.0 + b5 * 15.0 + b4 * 10.0 + b3 * 6.0 + b2 * 3.0 + b1);
    double e2 = q3 * (b6 * 35.0 + b5 * 20.0 + b4 * 10.0 + b3 * 4.0 + b2);
    double e3 = q4 * (b6 * 35.0 + b5 * 15.0 + b4 * 5.0 + b3);
    double e4 = q5 * (b6 * 21.0 + b5 * 6.0 + b4);
    double e5 = q6 * (b6 * 7.0 + b5);
    double e6 = q7 * b6;
    b[i] = e0 + 0.0;
    b[d + i] = e1 + 0.0;
    b[2 * d + i] = e2 + 0.0;
    b[3 * d + i] = e3 + 0.0;
    b[4 * d + i] = e4 + 0.0;
    b[5 * d + i] = e5 + 0.0;
    b[6 * d + i] = e6 + 0.0;
}

__device__ __forceinline__ void reduce2(EngineCtl *ctl, int idx, unsigned long long k0,
                                        unsigned long long k1)
{
    k0 = warp_max_u64(k0);
    k1 = warp_max_u64(k1);
    if ((threadIdx.x & 31) == 0) {
        if (k0) atomicMax(&ctl->red[idx & 3][0], k0);
        if (k1) atomicMax(&ctl->red[idx & 3][1], k1);
    }
}

// After the barrier that completes reduction idx: read it, and clear the
// slot two reductions ahead (its last readers finished two barriers ago).
__device__ __forceinline__ void read2(EngineCtl *ctl, int idx, double &v0, double &v1)
{
    v0 = absmax_value(*(volatile unsigned long long *)&ctl->red[idx & 3][0]);
    v1 = absmax_value(*(volatile unsigned long long *)&ctl->red[idx & 3][1]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->red[(idx + 2) & 3][0] = 0ull;
        ctl->red[(idx + 2) & 3][1] = 0ull;
    }
}

__device__ __forceinline__ void ring_put(double *buf, unsigned long long count, long long cap,
                                         double t, int i, int j, double d)
{
    if (!buf || cap <= 0) return;
    unsigned long long w = 4ull * (unsigned long long)cap;
    buf[(4ull * count) % w] = t;
    buf[(4ull * count + 1) % w] = (double)i;
    buf[(4ull * count + 2) % w] = (double)j;
    buf[(4ull * count + 3) % w] = d;
}

// Pairs j < k closer than the event thresholds (src/common.c:116-158).
// One warp per body j (grid-stride over warps), its lanes over k > j, so a
// check costs about N / 32 pair tests per warp instead of N per thread
// (the order of the records does not matter: commit_events sorts them).
//
// Single-precision prefilter: with each coordinate held as a float f and a
// bound e >= |x - f| (put_prefilter), a pair whose floats differ in some
// coordinate by more than (T + e_j + e_k)(1 + 2^-21) is farther apart than
// T >= sqrt(thr2) (1 + 2^-20) in exact arithmetic -- the factor covers the
// float roundings of the test -- so its FP64 r2 exceeds thr2 and the
// reference's test cannot fire.  Every other pair (NaN or infinite
// coordinates included: their comparisons are false) takes the FP64 test
// r2 <= thr2, then the reference's comparisons.  The FP64 pipe sees only
// pairs within about the threshold of each other.
__device__ void scan_events(const EngineArgs &a, double t, int tid, int nthreads)
{
    (void)t;
    EngineCtl *ctl = a.ctl;
    const int lane = tid & 31;
    const int warp = tid >> 5, nwarps = nthreads >> 5;
    const float T = __double2float_ru(sqrt(a.thr2) * (1.0 + 0x1p-20));
    const float widen = 1.0f + 0x1p-21f;
    for (int j = warp; j < a.n; j += nwarps) {
        const float2 fx = __ldcg(a.ypf + 3 * j), fy = __ldcg(a.ypf + 3 * j + 1),
                     fz = __ldcg(a.ypf + 3 * j + 2);
        const float tx = T + fx.y, ty = T + fy.y, tz = T + fz.y;
        const double rj = a.r[j];
        for (int k = j + 1 + lane; k < a.n; k += 32) {
            const float2 gx = __ldcg(a.ypf + 3 * k), gy = __ldcg(a.ypf + 3 * k + 1),
                         gz = __ldcg(a.ypf + 3 * k + 2);
            if (fabsf(fx.x - gx.x) > (tx + gx.y) * widen || fabsf(fy.x - gy.x) > (ty + gy.y) * widen ||
                fabsf(fz.x - gz.x) > (tz + gz.y) * widen)
                continue;
            const double xj = __ldcg(a.ypa + 3 * j), yj = __ldcg(a.ypa + 3 * j + 1),
                         zj = __ldcg(a.ypa + 3 * j + 2);
            double dx = xj - __ldcg(a.ypa + 3 * k);
            double dy = yj - __ldcg(a.ypa + 3 * k + 1);
            double dz = zj - __ldcg(a.ypa + 3 * k + 2);
            double r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 <= a.thr2)) continue;
            double sep = sqrt(r2);
            double rr = rj + a.r[k];
            if (sep <= a.ce_dist) {
                int e = atomicAdd(&ctl->n_ev, 1);
                if (e < a.ev_cap) a.ev[e] = EventRec{j, k, 0, sep};
            }
            if (rr > 0 && sep <= rr) {
                int e = atomicAdd(&ctl->n_ev, 1);
                if (e < a.ev_cap) a.ev[e] = EventRec{j, k, 1, sep};
            }
        }
    }
}

// The event test of one pair on the accepted positions, in the
// reference's arithmetic (src/common.c:125-152): the separation of the
// lower index j minus the higher k, r2 = dx^2 + dy^2 + dz^2, sep = sqrt(r2);
// a close encounter when sep <= the close-encounter distance, a collision
// when the radii sum is positive and sep <= it.  (pj, pk) are the two
// bodies' positions in either order; the squares do not depend on it.
__device__ __forceinline__ void event_pair(const EngineArgs &a, int j, int k, double xj, double yj,
                                           double zj, double xk, double yk, double zk)
{
    const double dx = xj - xk, dy = yj - yk, dz = zj - zk;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 <= a.thr2)) return;
    const int lo = j < k ? j : k, hi = j < k ? k : j;
    const double sep = sqrt(r2);
    const double rr = a.r[lo] + a.r[hi];
    EngineCtl *ctl = a.ctl;
    if (sep <= a.ce_dist) {
        int e = atomicAdd(&ctl->n_ev, 1);
        if (e < a.ev_cap) a.ev[e] = EventRec{lo, hi, 0, sep};
    }
    if (rr > 0 && sep <= rr) {
        int e = atomicAdd(&ctl->n_ev, 1);
        if (e < a.ev_cap) a.ev[e] = EventRec{lo, hi, 1, sep};
    }
}

// The event check fused into the advance force evaluation (spacing 1,
// whose positions become the accepted ones): while the force loop walks a
// sink's sources, each (sink, source) pair is tested as well -- a pair of
// two sources once, from the lower index; a massless or deleted sink with
// every source.  Records of an attempt that is rejected are dropped; the
// pairs the force never visits (two bodies without positive mass) are
// tested by scan_events_nonsources after an accepted step.
template <int JS>
__device__ __forceinline__ void sink_events(const EngineArgs &a, int j, const Src *src, double xj,
                                            double yj, double zj, int lane)
{
    const bool j_src = a.src_slot[j] >= 0;
    for (int q = lane; q < a.n_src; q += JS) {
        const int k = a.src_body[q];
        if (k == j || (j_src && k < j)) continue;
        const Src s = load_src(src + q);
        event_pair(a, j, k, xj, yj, zj, s.x, s.y, s.z);
    }
}

// Pairs of two bodies without positive mass (the split and persistent
// engines' remaining check after an accepted step): scan_events' warp
// layout and prefilter over the bodies listed in tp_body.
__device__ void scan_events_nonsources(const EngineArgs &a, int tid, int nthreads)
{
    const int lane = tid & 31;
    const int warp = tid >> 5, nwarps = nthreads >> 5;
    const float T = __double2float_ru(sqrt(a.thr2) * (1.0 + 0x1p-20));
    const float widen = 1.0f + 0x1p-21f;
    for (int u = warp; u < a.n_tp; u += nwarps) {
        const int j = a.tp_body[u];
        const float2 fx = __ldcg(a.ypf + 3 * j), fy = __ldcg(a.ypf + 3 * j + 1),
                     fz = __ldcg(a.ypf + 3 * j + 2);
        const float tx = T + fx.y, ty = T + fy.y, tz = T + fz.y;
        for (int v = u + 1 + lane; v < a.n_tp; v += 32) {
            const int k = a.tp_body[v];
            const float2 gx = __ldcg(a.ypf + 3 * k), gy = __ldcg(a.ypf + 3 * k + 1),
                         gz = __ldcg(a.ypf + 3 * k + 2);
            if (fabsf(fx.x - gx.x) > (tx + gx.y) * widen || fabsf(fy.x - gy.x) > (ty + gy.y) * widen ||
                fabsf(fz.x - gz.x) > (tz + gz.y) * widen)
                continue;
            event_pair(a, j, k, __ldcg(a.ypa + 3 * j), __ldcg(a.ypa + 3 * j + 1),
                       __ldcg(a.ypa + 3 * j + 2), __ldcg(a.ypa + 3 * k), __ldcg(a.ypa + 3 * k + 1),
                       __ldcg(a.ypa + 3 * k + 2));
        }
    }
}

// One thread: order the events of this check as the reference's loops
// would meet them, append them to the ring buffers, compute the flag.
__device__ void commit_events(const EngineArgs &a, double t)
{
    EngineCtl *ctl = a.ctl;
    int n = *(volatile int *)&ctl->n_ev;
    if (n > a.ev_cap) {
        ctl->ev_overflow = 1;
        n = a.ev_cap;
    }
    for (int x = 1; x < n; x++) {  // insertion sort by (j, k, kind)
        EventRec v = a.ev[x];
        int y = x - 1;
        while (y >= 0) {
            EventRec u = a.ev[y];
            bool greater = (u.j > v.j) || (u.j == v.j && (u.k > v.k || (u.k == v.k && u.kind > v.kind)));
            if (!greater) break;
            a.ev[y + 1] = u;
            y--;
        }
        a.ev[y + 1] = v;
    }
    for (int x = 0; x < n; x++) {
        EventRec v = a.ev[x];
        if (v.kind == 0) {
            ring_put(a.buf_ce, ctl->n_ce, a.max_ce, t, v.j, v.k, v.sep);
            ctl->n_ce++;
        } else {
            ring_put(a.buf_coll, ctl->n_coll, a.max_coll, t, v.j, v.k, v.sep);
            ctl->n_coll++;
        }
    }
    int flag = 0;
    if (a.max_ce > 0 && ctl->n_ce >= (unsigned long long)a.max_ce) flag = 1;
    else if (a.max_coll > 0 && ctl->n_coll >= (unsigned long long)a.max_coll) flag = 2;
    ctl->flag = flag;
    ctl->n_ev = 0;
    __threadfence();
}

template <int MODE, int JS, bool PN>
__global__ void __launch_bounds__(256) radau_engine(EngineArgs a)
{
    EngineCtl *ctl = a.ctl;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthreads = gridDim.x * blockDim.x;
    const int lane = tid % JS;
    const int gid = tid / JS;
    const int ngroups = nthreads / JS;
    const bool leader = (blockIdx.x == 0 && threadIdx.x == 0);
    const long long T = a.timeout_ns;
    const int n = a.n;
    // sink loops run to a multiple of the groups in a warp, so every lane of
    // a warp takes part in each iteration's shuffles; jj >= n is a dummy
    const int gpw = 32 / JS;
    const int n_loop = (n + gpw - 1) / gpw * gpw;
    const int c0 = comp_lo<JS>(lane), c1 = comp_hi<JS>(lane);

    double t, h;
    int loop_count, pc, red_idx;
    long long my_attempts = 0;

    if (ctl->phase == 0) {
        // --- F1 = f(y0): publish y0 (spacing 0 gives y0 exactly), then force
        for (int j = gid; j < n; j += ngroups)
            for (int c = c0; c < c1; c++)
                publish_comp<MODE>(a, j, c, 0, 0.0, 0.0, 0.0, 0.0, a.yp[0], a.src[0]);
        if (!grid_sync(ctl, T)) return;
        for (int jj = gid; jj < n_loop; jj += ngroups) {
            const bool live = jj < n;
            const int j = live ? jj : n - 1;
            double f[3];
            sink_force<MODE, JS, PN>(a, j, a.src[0], a.dy0, a.y0[3 * j], a.y0[3 * j + 1],
                                 a.y0[3 * j + 2], lane, f);
            if (!live) continue;
            const bool alive = a.m[j] >= 0.0;
            for (int c = c0; c < c1; c++)
                a.F1[3 * j + c] = (alive ? pick3(f, c) : 0.0) + (a.ext ? a.ext[3 * j + c] : 0.0);
        }
        if (leader) ctl->force_calls++;
        if (!grid_sync(ctl, T)) return;
        // --- initial_time_step (src/integrator_gauss_radau15.c:9-54): the
        // reference scans only the first n of the 3n entries for d0 and d1
        unsigned long long k0 = 0, k1 = 0;
        for (int i = tid; i < n; i += nthreads) {
            unsigned long long u = absmax_key(a.y0[i]), w = absmax_key(__ldcg(a.F1 + i));
            k0 = u > k0 ? u : k0;
            k1 = w > k1 ? w : k1;
        }
        red_idx = 0;
        reduce2(ctl, red_idx, k0, k1);
        if (!grid_sync(ctl, T)) return;
        double d0, d1;
        read2(ctl, red_idx++, d0, d1);
        double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
        // Euler probe y1 = y0 + dt0 dy0 into yp[1] / src[1] (and, for the
        // post-Newtonian terms, dy1 = dy0 + dt0 f0 into vp[1])
        for (int j = gid; j < n; j += ngroups) {
            const int slot = a.src_slot[j];
            for (int c = c0; c < c1; c++) {
                const double p = a.y0[3 * j + c] + dt0 * a.dy0[3 * j + c];
                a.yp[1][3 * j + c] = p;
                if (PN) a.vp[1][3 * j + c] = a.dy0[3 * j + c] + dt0 * __ldcg(a.F1 + 3 * j + c);
                if (slot >= 0) {
                    double *rec = reinterpret_cast<double *>(a.src[1] + slot);
                    rec[c] = p;
                    if (c == 0) rec[3] = a.G * a.m[j];
                }
            }
        }
        if (!grid_sync(ctl, T)) return;
        unsigned long long k2 = 0;
        for (int jj = gid; jj < n_loop; jj += ngroups) {
            const bool live = jj < n;
            const int j = live ? jj : n - 1;
            double f[3];
            sink_force<MODE, JS, PN>(a, j, a.src[1], a.vp[1], a.yp[1][3 * j], a.yp[1][3 * j + 1],
                                 a.yp[1][3 * j + 2], lane, f);
            if (!live) continue;
            const bool alive = a.m[j] >= 0.0;
            for (int c = c0; c < c1; c++) {
                double fi = (alive ? pick3(f, c) : 0.0) + (a.ext ? a.ext[3 * j + c] : 0.0);
                unsigned long long u = absmax_key(fi - a.F1[3 * j + c]);
                k2 = u > k2 ? u : k2;
            }
        }
        if (leader) ctl->force_calls++;
        reduce2(ctl, red_idx, k2, 0ull);
        if (!grid_sync(ctl, T)) return;
        double d2, unused;
        read2(ctl, red_idx++, d2, unused);
        d2 = d2 / dt0;
        double dt1;
        if (fmax(d1, d2) <= 1e-15) dt1 = fmax(1e-6, dt0 * 1e-3);
        else dt1 = pow(0.01 / fmax(d1, d2), (1.0 / (15 + 1)));
        h = fmin(100 * dt0, dt1);
        t = ctl->t;
        loop_count = 0;
        pc = 0;
        // first attempt's substep-1 prediction
        {
            const double ds = h * c_hs[1], hh = 0.5 * ds * ds;
            for (int j = gid; j < n; j += ngroups)
                for (int c = c0; c < c1; c++)
                    publish_comp<MODE>(a, j, c, 1, c_hs[1], h, ds, hh, a.yp[pc & 1], a.src[pc & 1],
                                       PN ? a.vp[pc & 1] : nullptr);
        }
        if (!grid_sync(ctl, T)) return;
    } else {
        t = ctl->t;
        h = ctl->h;
        loop_count = ctl->loop_count;
        pc = ctl->pc;
        red_idx = ctl->red_idx;
    }

    bool done = false;
    while (!done && my_attempts < a.attempt_budget) {
        // ---------------- corrector iterations ----------------
        int iters = 0;
        for (int ipc = 0; ipc < 12; ipc++) {
            iters++;
            unsigned long long kdb = 0, kf8 = 0;
            for (int ih = 1; ih < 8; ih++) {
                const double *yp = a.yp[pc & 1];
                const Src *src = a.src[pc & 1];
                // spacing of the next publication: substep ih + 1, or at
                // ih = 7 the next iteration's substep 1 (speculative)
                const int nrow = ih < 7 ? ih + 1 : 1;
                const double ns = c_hs[nrow], nds = h * ns, nhh = 0.5 * nds * nds;
                const double hh1 = 0.5 * h * h;
                for (int jj = gid; jj < n_loop; jj += ngroups) {
                    const bool live = jj < n;
                    const int j = live ? jj : n - 1;
                    double f[3];
                    sink_force<MODE, JS, PN>(a, j, src, a.vp[pc & 1], yp[3 * j], yp[3 * j + 1],
                                         yp[3 * j + 2], lane, f);
                    if (!live) continue;
                    const bool alive = a.m[j] >= 0.0;
                    for (int c = c0; c < c1; c++) {
                        const int i = 3 * j + c;
                        const double fi = (alive ? pick3(f, c) : 0.0) + (a.ext ? a.ext[i] : 0.0);
                        gb_update<MODE>(a, i, ih, fi);
                        if (ih == 7) {
                            unsigned long long u = absmax_key(b6_at<MODE>(a, i) - a.b6p[i]);
                            unsigned long long w = absmax_key(fi);
                            kdb = u > kdb ? u : kdb;
                            kf8 = w > kf8 ? w : kf8;
                        }
                        publish_comp<MODE>(a, j, c, nrow, ns, h, nds, nhh, a.yp[(pc + 1) & 1],
                                           a.src[(pc + 1) & 1],
                                           PN ? a.vp[(pc + 1) & 1] : nullptr);
                        if (ih == 7) {
                            // speculative advance (spacing 1)
                            publish_comp<MODE>(a, j, c, 8, 1.0, h, h, hh1, a.ypa, a.srca);
                            a.dyp[i] = pred_vel<MODE>(a, i, h);
                        }
                    }
                }
                pc++;
                if (ih == 7) reduce2(ctl, red_idx, kdb, kf8);
                if (!grid_sync(ctl, T)) return;
            }
            if (leader) ctl->force_calls += 7;
            double db6, f8;
            read2(ctl, red_idx++, db6, f8);
            if (corrector_converged<MODE>(db6, f8)) break;  // src/integrator_gauss_radau15.c:300
            for (int j = gid; j < n; j += ngroups)
                for (int c = c0; c < c1; c++) a.b6p[3 * j + c] = b6_at<MODE>(a, 3 * j + c);
        }
        // ---------------- advance (spacing 1) ----------------
        unsigned long long kb6 = 0, kdd = 0;
        for (int jj = gid; jj < n_loop; jj += ngroups) {
            const bool live = jj < n;
            const int j = live ? jj : n - 1;
            double f[3];
            sink_force<MODE, JS, PN>(a, j, a.srca, a.dyp, a.ypa[3 * j], a.ypa[3 * j + 1],
                                 a.ypa[3 * j + 2], lane, f);
            if (!live) continue;
            if (a.thr2 > 0.0)  // the event check, fused into this force loop
                sink_events<JS>(a, j, a.srca, a.ypa[3 * j], a.ypa[3 * j + 1], a.ypa[3 * j + 2], lane);
            const bool alive = a.m[j] >= 0.0;
            for (int c = c0; c < c1; c++) {
                const int i = 3 * j + c;
                const double fi = (alive ? pick3(f, c) : 0.0) + (a.ext ? a.ext[i] : 0.0);
                a.ddy[i] = fi;
                if (!(finite_bits(fi) && finite_bits(a.ypa[i]) && finite_bits(a.dyp[i])))
                    atomicCAS(&ctl->err, 0, ABIE_ERR_NUMERICS);
                unsigned long long u = absmax_key(b6_at<MODE>(a, i));
                unsigned long long w = absmax_key(fi);
                kb6 = u > kb6 ? u : kb6;
                kdd = w > kdd ? w : kdd;
            }
        }
        reduce2(ctl, red_idx, kb6, kdd);
        if (!grid_sync(ctl, T)) return;
        if (leader) {
            ctl->force_calls += 1;
            ctl->iterations += iters;
            ctl->attempts += 1;
        }
        double mb6, mdd;
        read2(ctl, red_idx++, mb6, mdd);
        // ---------------- step control (src/integrator_gauss_radau15.c:313-367) ----------------
        double estim_b6 = mb6 / mdd;
        double err, dtreq, rq;
        step_size<MODE>(estim_b6, h, err, dtreq, rq);
        bool accepted = (err <= 1 || loop_count > 100);
        bool stop = false;
        if (accepted) {
            t += h;
            loop_count = 0;
            if (t > a.t_end) {
                h = a.t_end - t;
                stop = true;
            }
            double q = MODE == ABIE_FORCE_EXACT ? dtreq / h : rq;
            for (int j = gid; j < n; j += ngroups) {
                for (int c = c0; c < c1; c++) {
                    int i = 3 * j + c;
                    a.y0[i] = a.ypa[i];
                    a.dy0[i] = a.dyp[i];
                    a.F1[i] = a.ddy[i];
                    if (MODE == ABIE_FORCE_EXACT) {
                        a.b6p[i] = a.b[6 * a.dim + i];
                        refine_b(a, i, q);
                    } else {
                        refine_g(a, i, q, stop);
                    }
                }
            }
            if (a.thr2 > 0.0) scan_events_nonsources(a, tid, nthreads);
            if (leader) ctl->accepts++;
        } else {
            loop_count += 1;
            if (leader) {
                ctl->rejects++;
                ctl->n_ev = 0;  // the fused check's records of a rejected attempt
            }
        }
        if (!stop) {
            if ((MODE == ABIE_FORCE_EXACT ? dtreq / h : rq) > 1.0 / FAC) h /= FAC;
            else if (dtreq < 1.e-12) h *= FAC;
            else h = dtreq;
            if (h < H_MIN) h = H_MIN;
            // next attempt's substep-1 prediction
            const double ds = h * c_hs[1], hh = 0.5 * ds * ds;
            for (int j = gid; j < n; j += ngroups)
                for (int c = c0; c < c1; c++)
                    publish_comp<MODE>(a, j, c, 1, c_hs[1], h, ds, hh, a.yp[pc & 1], a.src[pc & 1],
                                       PN ? a.vp[pc & 1] : nullptr);
        }
        if (!grid_sync(ctl, T)) return;
        if (accepted && *(volatile int *)&ctl->n_ev > 0) {
            if (leader) commit_events(a, t);
            if (!grid_sync(ctl, T)) return;
            if (*(volatile int *)&ctl->flag > 0) stop = true;
        }
        my_attempts++;
        if (accepted && leader) ctl->t = t;
        done = stop;
    }
    if (leader) {
        ctl->t = t;
        ctl->h = h;
        ctl->loop_count = loop_count;
        ctl->pc = pc;
        ctl->red_idx = red_idx;
        ctl->phase = done ? 2 : 1;
        ctl->attempts_done += my_attempts;
        __threadfence();
    }
}

// ---------------------------------------------------------------------------
// Split engine: systems whose massive bodies fit one warp (3 n_src <= 32),
// such as a star, planets and many test particles.  Massless bodies never
// act on the massive ones, so every block integrates a private replica of
// the massive subsystem (warp 0, one component per lane, bitwise the same in
// every block) next to its own test particles (warp 1, SPLIT_TPW particles
// of 4 lanes: lanes 0..2 own x, y, z and the 4 lanes split the sources).
// All state stays in registers; a substep needs only a block barrier, and
// the grid meets once per corrector iteration (the convergence test) and
// per step attempt (the step control, the event check), instead of once per
// substep.  The per-component arithmetic is radau_comp.cuh's, so the exact
// form repeats the reference's expressions and the results equal the
// single-system engine's.
constexpr int SPLIT_TPW = 8;  // test particles per block

template <int MODE>
__device__ __forceinline__ void split_tp_force(const EngineArgs &a, const double (*sp)[SPW], int n_m,
                                               double p, int lane, double &fx, double &fy,
                                               double &fz)
{
    // the particle's position from its component lanes
    const double x = __shfl_sync(0xffffffffu, p, 0, 4);
    const double y = __shfl_sync(0xffffffffu, p, 1, 4);
    const double z = __shfl_sync(0xffffffffu, p, 2, 4);
    const int q0 = lane & 3;
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (MODE == ABIE_FORCE_EXACT) {
        if (q0 == 0)
            for (int k = 0; k < n_m; k++) {
                Src s{sp[k][0], sp[k][1], sp[k][2], sp[k][3]};
                pair_exact(x, y, z, s, ax, ay, az);
            }
        fx = __shfl_sync(0xffffffffu, ax, 0, 4);
        fy = __shfl_sync(0xffffffffu, ay, 0, 4);
        fz = __shfl_sync(0xffffffffu, az, 0, 4);
    } else {
        for (int k = q0; k < n_m; k += 4) {
            Src s{sp[k][0], sp[k][1], sp[k][2], sp[k][3]};
            pair_fast(x, y, z, s, ax, ay, az);
        }
#pragma unroll
        for (int o = 2; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o, 4);
            ay += __shfl_xor_sync(0xffffffffu, ay, o, 4);
            az += __shfl_xor_sync(0xffffffffu, az, o, 4);
        }
        fx = ax;
        fy = ay;
        fz = az;
    }
}

template <int MODE, bool PN>
__global__ void __launch_bounds__(64) radau_split(EngineArgs a)
{
    __shared__ double s_sp[2][32][SPW];  // massive predicted positions, G m (two buffers)
    __shared__ double s_sv[2][32][4];  // massive predicted velocities, m (post-Newtonian only)
    __shared__ double s_sa[32][3];     // massive accelerations
    EngineCtl *ctl = a.ctl;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    const bool leader = (blockIdx.x == 0 && threadIdx.x == 0);
    const long long T = a.timeout_ns;
    const int n_m = a.n_src;
    // this thread's component
    int gi = -1;        // global component index
    bool alive = true;  // m >= 0
    bool writer = true; // owns the component's copy in global memory
    if (warp == 0) {
        if (lane < 3 * n_m) gi = 3 * a.src_body[lane / 3] + lane % 3;
        writer = blockIdx.x == 0;
    } else {
        const int tpi = blockIdx.x * SPLIT_TPW + lane / 4;
        if ((lane & 3) < 3 && tpi < a.n_tp) {
            const int body = a.tp_body[tpi];
            gi = 3 * body + (lane & 3);
            alive = a.m[body] >= 0.0;
        }
    }
    const bool has = gi >= 0;
    const double ext = (has && a.ext) ? a.ext[gi] : 0.0;
    Group<1> mg;  // the massive warp as a group
    mg.gl = lane;
    mg.lane = lane;
    mg.wig = 0;
    mg.gidx = 0;
    mg.red = nullptr;
    mg.flg = nullptr;
    mg.tog = 0;
    constexpr bool pn = PN;  // post-Newtonian terms (src/common.c:101-107), a.C > 0
    const double my_m = has ? a.m[gi / 3] : 0.0;
    if (threadIdx.x < n_m) {
        const double mm = a.m[a.src_body[threadIdx.x]];
        const double gm = a.G * mm;
        s_sp[0][threadIdx.x][3] = gm;
        s_sp[1][threadIdx.x][3] = gm;
        s_sv[0][threadIdx.x][3] = mm;
        s_sv[1][threadIdx.x][3] = mm;
    }
    Comp X;
    X.y0 = has ? a.y0[gi] : 0.0;
    X.dy0 = has ? a.dy0[gi] : 0.0;
    if (ctl->phase == 0 || !has) {
        X.F1 = X.b6p = 0.0;
#pragma unroll
        for (int k = 0; k < 7; k++) X.b[k] = X.g[k] = 0.0;
    } else {
        X.F1 = a.F1[gi];
        X.b6p = a.b6p[gi];
#pragma unroll
        for (int k = 0; k < 7; k++) X.b[k] = a.b[k * a.dim + gi];
#pragma unroll
        for (int k = 0; k < 7; k++) X.g[k] = a.g[k * a.dim + gi];
    }
    int ib = 0;
    // forces at this thread's position p and velocity v (one component
    // each): publish the massive positions (and velocities for the
    // post-Newtonian terms), one block barrier, then the massive warp's
    // group force or the particle's sum over the massive sources.  Newton,
    // then the post-Newtonian sum, then the external acceleration, as
    // src/common.c:82-114 adds them.
    // With events on, the advance evaluation (whose positions become the
    // accepted ones) also runs the event test on the pairs it visits: the
    // massive pairs once, in block 0, and each particle with every massive
    // body (sink_events' rule; scan_events_nonsources covers the rest).
    auto forces = [&](double p, double v, bool advance = false) -> double {
        if (warp == 0 && has) {
            s_sp[ib][lane / 3][lane % 3] = p;
            if (pn) s_sv[ib][lane / 3][lane % 3] = v;
        }
        __syncthreads();
        double F = 0.0;
        if (advance && a.thr2 > 0.0) {
            const double(*P)[SPW] = s_sp[ib];
            if (warp == 0) {
                if (blockIdx.x == 0)
                    for (int pr = lane; pr < n_m * (n_m - 1) / 2; pr += 32) {
                        int i = 0, rem = pr;
                        while (rem >= n_m - 1 - i) {
                            rem -= n_m - 1 - i;
                            i++;
                        }
                        const int k = i + 1 + rem;
                        event_pair(a, a.src_body[i], a.src_body[k], P[i][0], P[i][1], P[i][2], P[k][0],
                                   P[k][1], P[k][2]);
                    }
            } else {
                const double x = __shfl_sync(0xffffffffu, p, 0, 4);
                const double y = __shfl_sync(0xffffffffu, p, 1, 4);
                const double z = __shfl_sync(0xffffffffu, p, 2, 4);
                const int tpi = blockIdx.x * SPLIT_TPW + lane / 4;
                if ((lane & 3) == 0 && tpi < a.n_tp) {
                    const int body = a.tp_body[tpi];
                    for (int k = 0; k < n_m; k++)
                        event_pair(a, body, a.src_body[k], x, y, z, P[k][0], P[k][1], P[k][2]);
                }
            }
        }
        if (warp == 0) {
            group_force<MODE, 1>(mg, n_m, s_sp[ib], s_sa);
            if (pn) {
                if (lane < n_m) {
                    const double(*P)[SPW] = s_sp[ib];
                    const double(*V)[4] = s_sv[ib];
                    double ax = 0.0, ay = 0.0, az = 0.0;
                    for (int k = 0; k < n_m; k++) {
                        if (k == lane) continue;
                        pn_term<MODE>(a.pn, P[lane][0], P[lane][1], P[lane][2], V[lane][0], V[lane][1],
                                V[lane][2], V[lane][3], P[k][0], P[k][1], P[k][2], V[k][0], V[k][1],
                                V[k][2], V[k][3], ax, ay, az);
                    }
                    s_sa[lane][0] += ax;
                    s_sa[lane][1] += ay;
                    s_sa[lane][2] += az;
                }
                __syncwarp();
            }
            if (has) F = s_sa[lane / 3][lane % 3];
        } else {
            double fx, fy, fz;
            split_tp_force<MODE>(a, s_sp[ib], n_m, p, lane, fx, fy, fz);
            if (pn) {
                const double x = __shfl_sync(0xffffffffu, p, 0, 4);
                const double y = __shfl_sync(0xffffffffu, p, 1, 4);
                const double z = __shfl_sync(0xffffffffu, p, 2, 4);
                const double vx = __shfl_sync(0xffffffffu, v, 0, 4);
                const double vy = __shfl_sync(0xffffffffu, v, 1, 4);
                const double vz = __shfl_sync(0xffffffffu, v, 2, 4);
                double ax = 0.0, ay = 0.0, az = 0.0;
                if ((lane & 3) == 0) {
                    const double(*P)[SPW] = s_sp[ib];
                    const double(*V)[4] = s_sv[ib];
                    for (int k = 0; k < n_m; k++)
                        pn_term<MODE>(a.pn, x, y, z, vx, vy, vz, my_m, P[k][0], P[k][1], P[k][2],
                                V[k][0], V[k][1], V[k][2], V[k][3], ax, ay, az);
                }
                fx += __shfl_sync(0xffffffffu, ax, 0, 4);
                fy += __shfl_sync(0xffffffffu, ay, 0, 4);
                fz += __shfl_sync(0xffffffffu, az, 0, 4);
            }
            const int c = lane & 3;
            F = c == 0 ? fx : (c == 1 ? fy : fz);
        }
        ib ^= 1;
        return has ? ((alive ? F : 0.0) + ext) : 0.0;
    };

    double t, h;
    int loop_count, red_idx;
    long long my_attempts = 0;
    if (ctl->phase == 0) {
        // F1 = f(y0), then initial_time_step (src/integrator_gauss_radau15.c:9-54)
        X.F1 = forces(X.y0, X.dy0);
        if (leader) ctl->force_calls++;
        unsigned long long k0 = 0, k1 = 0;
        if (has && gi < a.n && writer) {  // the reference scans the first n of 3n entries
            k0 = absmax_key(X.y0);
            k1 = absmax_key(X.F1);
        }
        red_idx = 0;
        reduce2(ctl, red_idx, k0, k1);
        if (!grid_sync(ctl, T)) return;
        double d0, d1;
        read2(ctl, red_idx++, d0, d1);
        const double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
        const double f1 = forces(X.y0 + dt0 * X.dy0, X.dy0 + dt0 * X.F1);
        if (leader) ctl->force_calls++;
        const unsigned long long k2 = (has && writer) ? absmax_key(f1 - X.F1) : 0ull;
        reduce2(ctl, red_idx, k2, 0ull);
        if (!grid_sync(ctl, T)) return;
        double d2, unused;
        read2(ctl, red_idx++, d2, unused);
        d2 = d2 / dt0;
        double dt1;
        if (fmax(d1, d2) <= 1e-15) dt1 = fmax(1e-6, dt0 * 1e-3);
        else dt1 = pow(0.01 / fmax(d1, d2), (1.0 / (15 + 1)));
        h = fmin(100 * dt0, dt1);
        t = ctl->t;
        loop_count = 0;
    } else {
        t = ctl->t;
        h = ctl->h;
        loop_count = ctl->loop_count;
        red_idx = ctl->red_idx;
    }

    bool done = false;
    while (!done && my_attempts < a.attempt_budget) {
        int iters = 0;
        for (int ipc = 0; ipc < 12; ipc++) {
            iters++;
            unsigned long long kdb = 0, kf8 = 0;
            for (int ih = 1; ih < 8; ih++) {
                const double sh = e_hs[ih], ds = h * sh, hh = 0.5 * ds * ds;
                const double F = forces(has ? e_pred_pos<MODE>(X, ih, sh, h, ds, hh) : 0.0,
                                        (has && pn) ? e_pred_vel_at<MODE>(X, ih, sh, h) : 0.0);
                if (has) {
                    e_gb_update<MODE>(X, ih, F);
                    if (ih == 7 && writer) {
                        kdb = absmax_key(e_b6<MODE>(X) - X.b6p);
                        kf8 = absmax_key(F);
                    }
                }
            }
            if (leader) ctl->force_calls += 7;
            reduce2(ctl, red_idx, kdb, kf8);
            if (!grid_sync(ctl, T)) return;
            double db6, f8;
            read2(ctl, red_idx++, db6, f8);
            if (corrector_converged<MODE>(db6, f8)) break;  // src/integrator_gauss_radau15.c:300
            X.b6p = e_b6<MODE>(X);
        }
        // advance (spacing 1)
        const double hh1 = 0.5 * h * h;
        const double ya = has ? e_pred_pos<MODE>(X, 8, 1.0, h, h, hh1) : 0.0;
        const double va = has ? e_pred_vel<MODE>(X, h) : 0.0;
        const double dd = forces(ya, va, true);
        unsigned long long kb6 = 0, kdd = 0;
        if (has && writer) {
            a.ypa[gi] = ya;
            put_prefilter(a, gi, ya);
            if (!(finite_bits(dd) && finite_bits(ya) && finite_bits(va)))
                atomicCAS(&ctl->err, 0, ABIE_ERR_NUMERICS);
            kb6 = absmax_key(e_b6<MODE>(X));
            kdd = absmax_key(dd);
        }
        reduce2(ctl, red_idx, kb6, kdd);
        if (!grid_sync(ctl, T)) return;
        if (leader) {
            ctl->force_calls += 1;
            ctl->iterations += iters;
            ctl->attempts += 1;
        }
        double mb6, mdd;
        read2(ctl, red_idx++, mb6, mdd);
        // step control (src/integrator_gauss_radau15.c:313-367)
        const double estim_b6 = mb6 / mdd;
        double err, dtreq, rq;
        step_size<MODE>(estim_b6, h, err, dtreq, rq);
        const bool accepted = (err <= 1 || loop_count > 100);
        bool stop = false;
        if (accepted) {
            t += h;
            loop_count = 0;
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
            e_refine(X, q);
            if (MODE != ABIE_FORCE_EXACT) consistent_g(X);
            if (a.thr2 > 0.0) scan_events_nonsources(a, tid, nthreads);
            if (leader) ctl->accepts++;
        } else {
            loop_count += 1;
            if (leader) {
                ctl->rejects++;
                ctl->n_ev = 0;  // the fused check's records of a rejected attempt
            }
        }
        if (!stop) {
            if ((MODE == ABIE_FORCE_EXACT ? dtreq / h : rq) > 1.0 / FAC) h /= FAC;
            else if (dtreq < 1.e-12) h *= FAC;
            else h = dtreq;
            if (h < H_MIN) h = H_MIN;
        }
        if (!grid_sync(ctl, T)) return;
        if (accepted && *(volatile int *)&ctl->n_ev > 0) {
            if (leader) commit_events(a, t);
            if (!grid_sync(ctl, T)) return;
            if (*(volatile int *)&ctl->flag > 0) stop = true;
        }
        my_attempts++;
        if (accepted && leader) ctl->t = t;
        done = stop;
    }
    // state back to global memory (one writer per component)
    if (has && writer) {
        a.y0[gi] = X.y0;
        a.dy0[gi] = X.dy0;
        a.F1[gi] = X.F1;
        a.b6p[gi] = X.b6p;
#pragma unroll
        for (int k = 0; k < 7; k++) a.b[k * a.dim + gi] = X.b[k];
#pragma unroll
        for (int k = 0; k < 7; k++) a.g[k * a.dim + gi] = X.g[k];
    }
    if (leader) {
        ctl->t = t;
        ctl->h = h;
        ctl->loop_count = loop_count;
        ctl->red_idx = red_idx;
        ctl->phase = done ? 2 : 1;
        ctl->attempts_done += my_attempts;
        __threadfence();
    }
}

}  // namespace abie

namespace abie {

struct EngineBuffers {
    double *slab = nullptr;
    size_t slab_n = 0;  // bodies the slab holds
    Src *srcs = nullptr;
    int *src_body = nullptr, *src_slot = nullptr, *tp_body = nullptr;
    size_t src_n = 0;
    EngineCtl *ctl = nullptr;
    EventRec *ev = nullptr;
    double *partial = nullptr;  // stepped engine: two source chunks' partial sums (6 per body)
    size_t partial_n = 0;
    double *d_ce = nullptr, *d_coll = nullptr;
    size_t d_ce_n = 0, d_coll_n = 0;
};
static EngineBuffers g_eb;
static const int EV_CAP = 4096;
// y0 dy0 F1 b g b6p ddy dyp yp[2] ypa vp[2], and ypf (a float2 per component)
static const int SLAB_PER_BODY = 3 * (3 + 7 + 7 + 1 + 1 + 1 + 2 + 1 + 2 + 1);

void free_engine_buffers()
{
    EngineBuffers &e = g_eb;
    if (e.slab) cudaFree(e.slab);
    if (e.srcs) cudaFree(e.srcs);
    if (e.src_body) cudaFree(e.src_body);
    if (e.src_slot) cudaFree(e.src_slot);
    if (e.tp_body) cudaFree(e.tp_body);
    if (e.ctl) cudaFree(e.ctl);
    if (e.ev) cudaFree(e.ev);
    if (e.d_ce) cudaFree(e.d_ce);
    if (e.d_coll) cudaFree(e.d_coll);
    if (e.partial) cudaFree(e.partial);
    e = EngineBuffers();
}

static int engine_reserve(size_t n, size_t max_ce, size_t max_coll)
{
    EngineBuffers &e = g_eb;
    if (n > e.slab_n || !e.slab) {
        if (e.slab) cudaFree(e.slab);
        if (e.srcs) cudaFree(e.srcs);
        if (e.src_body) cudaFree(e.src_body);
        if (e.src_slot) cudaFree(e.src_slot);
        if (e.tp_body) cudaFree(e.tp_body);
        e.slab = nullptr;
        size_t c = n < 64 ? 64 : n;
        ABIE_CUDA(cudaMalloc(&e.slab, c * SLAB_PER_BODY * sizeof(double)));
        ABIE_CUDA(cudaMalloc(&e.srcs, 3 * c * sizeof(Src)));
        ABIE_CUDA(cudaMalloc(&e.src_body, c * sizeof(int)));
        ABIE_CUDA(cudaMalloc(&e.src_slot, c * sizeof(int)));
        ABIE_CUDA(cudaMalloc(&e.tp_body, c * sizeof(int)));
        e.slab_n = c;
    }
    if (!e.ctl) ABIE_CUDA(cudaMalloc(&e.ctl, sizeof(EngineCtl)));
    if (!e.ev) ABIE_CUDA(cudaMalloc(&e.ev, EV_CAP * sizeof(EventRec)));
    if (4 * max_ce > e.d_ce_n || !e.d_ce) {
        if (e.d_ce) cudaFree(e.d_ce);
        e.d_ce_n = 4 * (max_ce ? max_ce : 1);
        ABIE_CUDA(cudaMalloc(&e.d_ce, e.d_ce_n * sizeof(double)));
    }
    if (4 * max_coll > e.d_coll_n || !e.d_coll) {
        if (e.d_coll) cudaFree(e.d_coll);
        e.d_coll_n = 4 * (max_coll ? max_coll : 1);
        ABIE_CUDA(cudaMalloc(&e.d_coll, e.d_coll_n * sizeof(double)));
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Stepped engine for large systems (fast form, no post-Newtonian terms; from
// 2^20 interactions per force evaluation, where it overtakes the persistent
// engine: 45 against 50 us per force call at 1,025 bodies, 80 against 170
// at 2,049, 795 against 988 at 8,193): the host drives radau_engine's sweep
// one phase per kernel, and every force evaluation is the standalone force
// kernel on the published substep (launch_force_published), which keeps 40
// warps per SM busy on the FP64 pipe where the persistent engine, holding
// the whole sweep in registers, keeps 16.  The per-component device
// functions, the force sums (the engine's order for the same lanes per
// body, below 8,192 bodies; two source chunks from there, as the
// standalone force) and the scalar step control (one thread, the engine's
// expressions) are the persistent engine's, so below 8,192 bodies both
// give the same trajectory.  The host
// reads two maxima per corrector iteration and the controller's decision
// per attempt.

template <int MODE>
__global__ void __launch_bounds__(256) st_publish_kernel(EngineArgs a, int row, double h, int buf)
{
    const double s = row == 8 ? 1.0 : c_hs[row], ds = h * s, hh = 0.5 * ds * ds;
    double *yp = buf < 2 ? a.yp[buf] : a.ypa;
    Src *src = buf < 2 ? a.src[buf] : a.srca;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x)
        publish_comp<MODE>(a, i / 3, i % 3, row, row == 0 ? 0.0 : s, row == 0 ? 0.0 : h,
                           row == 0 ? 0.0 : ds, row == 0 ? 0.0 : hh, yp, src);
}

__device__ __forceinline__ void st_keys(unsigned long long *keys, unsigned long long k0,
                                        unsigned long long k1)
{
    k0 = warp_max_u64(k0);
    k1 = warp_max_u64(k1);
    if ((threadIdx.x & 31) == 0) {
        if (k0) atomicMax(&keys[0], k0);
        if (k1) atomicMax(&keys[1], k1);
    }
}

__device__ __forceinline__ double st_force_at(const EngineArgs &a, const double *acc, int i)
{
    return (a.m[i / 3] >= 0.0 ? acc[i] : 0.0) + (a.ext ? a.ext[i] : 0.0);
}

// F1 = f(y0); maxima of |y0| and |F1| over the first n entries (as the
// reference's initial_time_step scans them)
__global__ void __launch_bounds__(256) st_f1_kernel(EngineArgs a, const double *acc)
{
    unsigned long long k0 = 0, k1 = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x) {
        const double fi = st_force_at(a, acc, i);
        a.F1[i] = fi;
        if (i < a.n) {
            const unsigned long long u = absmax_key(a.y0[i]), w = absmax_key(fi);
            k0 = u > k0 ? u : k0;
            k1 = w > k1 ? w : k1;
        }
    }
    st_keys(&a.ctl->red[0][0], k0, k1);
}

// initial_time_step's dt0 (src/integrator_gauss_radau15.c:9-54), one thread
__global__ void st_dt0_kernel(EngineArgs a)
{
    EngineCtl *ctl = a.ctl;
    const double d0 = absmax_value(ctl->red[0][0]), d1 = absmax_value(ctl->red[0][1]);
    ctl->dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
    ctl->d1 = d1;
    ctl->red[0][0] = ctl->red[0][1] = 0ull;
}

// the Euler probe y1 = y0 + dt0 dy0 into yp[1] / src[1]
__global__ void __launch_bounds__(256) st_probe_kernel(EngineArgs a)
{
    const double dt0 = a.ctl->dt0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x) {
        const int j = i / 3, c = i % 3;
        const double p = a.y0[i] + dt0 * a.dy0[i];
        a.yp[1][i] = p;
        const int slot = a.src_slot[j];
        if (slot >= 0) {
            double *rec = reinterpret_cast<double *>(a.src[1] + slot);
            rec[c] = p;
            if (c == 0) rec[3] = a.G * a.m[j];
        }
    }
}

__global__ void __launch_bounds__(256) st_d2_kernel(EngineArgs a, const double *acc)
{
    unsigned long long k2 = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x) {
        const unsigned long long u = absmax_key(st_force_at(a, acc, i) - a.F1[i]);
        k2 = u > k2 ? u : k2;
    }
    st_keys(&a.ctl->red[0][0], k2, 0ull);
}

// the first step size, one thread
__global__ void st_h0_kernel(EngineArgs a)
{
    EngineCtl *ctl = a.ctl;
    const double dt0 = ctl->dt0, d1 = ctl->d1;
    const double d2 = absmax_value(ctl->red[0][0]) / dt0;
    double dt1;
    if (fmax(d1, d2) <= 1e-15) dt1 = fmax(1e-6, dt0 * 1e-3);
    else dt1 = pow(0.01 / fmax(d1, d2), (1.0 / (15 + 1)));
    ctl->h = fmin(100 * dt0, dt1);
    ctl->loop_count = 0;
    ctl->red[0][0] = ctl->red[0][1] = 0ull;
}

// one substep after its forces: new g (b), the next publication, and at
// the last substep the convergence maxima and the speculative advance
template <int MODE>
__global__ void __launch_bounds__(256) st_sweep_kernel(EngineArgs a, const double *acc, int ih,
                                                       double h, int pc)
{
    const int nrow = ih < 7 ? ih + 1 : 1;
    const double ns = c_hs[nrow], nds = h * ns, nhh = 0.5 * nds * nds;
    const double hh1 = 0.5 * h * h;
    unsigned long long kdb = 0, kf8 = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x) {
        const int j = i / 3, c = i % 3;
        const double fi = st_force_at(a, acc, i);
        gb_update<MODE>(a, i, ih, fi);
        if (ih == 7) {
            const unsigned long long u = absmax_key(b6_at<MODE>(a, i) - a.b6p[i]);
            const unsigned long long w = absmax_key(fi);
            kdb = u > kdb ? u : kdb;
            kf8 = w > kf8 ? w : kf8;
        }
        publish_comp<MODE>(a, j, c, nrow, ns, h, nds, nhh, a.yp[(pc + 1) & 1], a.src[(pc + 1) & 1]);
        if (ih == 7) {
            publish_comp<MODE>(a, j, c, 8, 1.0, h, h, hh1, a.ypa, a.srca);
            a.dyp[i] = pred_vel<MODE>(a, i, h);
        }
    }
    if (ih == 7) st_keys(&a.ctl->red[0][0], kdb, kf8);
}

template <int MODE>
__global__ void __launch_bounds__(256) st_b6p_kernel(EngineArgs a)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x)
        a.b6p[i] = b6_at<MODE>(a, i);
}

template <int MODE>
__global__ void __launch_bounds__(256) st_advance_kernel(EngineArgs a, const double *acc)
{
    unsigned long long kb6 = 0, kdd = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x) {
        const double fi = st_force_at(a, acc, i);
        a.ddy[i] = fi;
        if (!(finite_bits(fi) && finite_bits(a.ypa[i]) && finite_bits(a.dyp[i])))
            atomicCAS(&a.ctl->err, 0, ABIE_ERR_NUMERICS);
        const unsigned long long u = absmax_key(b6_at<MODE>(a, i)), w = absmax_key(fi);
        kb6 = u > kb6 ? u : kb6;
        kdd = w > kdd ? w : kdd;
    }
    st_keys(&a.ctl->red[0][0], kb6, kdd);
}

// step control (src/integrator_gauss_radau15.c:313-367) as radau_engine
// runs it, one thread; the decision goes to the host through ctl
template <int MODE>
__global__ void st_control_kernel(EngineArgs a)
{
    EngineCtl *ctl = a.ctl;
    const double mb6 = absmax_value(ctl->red[0][0]), mdd = absmax_value(ctl->red[0][1]);
    ctl->red[0][0] = ctl->red[0][1] = 0ull;
    double h = ctl->h, t = ctl->t;
    int loop_count = ctl->loop_count;
    const double estim_b6 = mb6 / mdd;
    double err, dtreq, rq;
    step_size<MODE>(estim_b6, h, err, dtreq, rq);
    const bool accepted = (err <= 1 || loop_count > 100);
    bool stop = false;
    double q = 0.0;
    if (accepted) {
        t += h;
        loop_count = 0;
        if (t > a.t_end) {
            h = a.t_end - t;
            stop = true;
        }
        q = MODE == ABIE_FORCE_EXACT ? dtreq / h : rq;
        ctl->accepts++;
    } else {
        loop_count += 1;
        ctl->rejects++;
    }
    if (!stop) {
        if ((MODE == ABIE_FORCE_EXACT ? dtreq / h : rq) > 1.0 / FAC) h /= FAC;
        else if (dtreq < 1.e-12) h *= FAC;
        else h = dtreq;
        if (h < H_MIN) h = H_MIN;
    }
    ctl->t = t;
    ctl->h = h;
    ctl->loop_count = loop_count;
    ctl->accepted = accepted ? 1 : 0;
    ctl->stop = stop ? 1 : 0;
    ctl->q = q;
}

template <int MODE>
__global__ void __launch_bounds__(256) st_accept_kernel(EngineArgs a)
{
    const double q = a.ctl->q;
    const bool stop = a.ctl->stop != 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.dim; i += gridDim.x * blockDim.x) {
        a.y0[i] = a.ypa[i];
        a.dy0[i] = a.dyp[i];
        a.F1[i] = a.ddy[i];
        if (MODE == ABIE_FORCE_EXACT) {
            a.b6p[i] = a.b[6 * a.dim + i];
            refine_b(a, i, q);
        } else {
            refine_g(a, i, q, stop);
        }
    }
}

__global__ void __launch_bounds__(256) st_scan_kernel(EngineArgs a)
{
    scan_events(a, a.ctl->t, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

__global__ void st_commit_kernel(EngineArgs a)
{
    if (a.ctl->n_ev > 0) commit_events(a, a.ctl->t);
}

// The host loop; the state sits in the engine's buffers (phase 0 start).
template <int MODE>
static int stepped_run(const EngineArgs &a, int num_sms, cudaStream_t st, EngineCtl *out,
                       bool mixed = false)
{
    EngineCtl *ctl = a.ctl;
    double *acc = a.vp[0];  // force output (the velocity buffers serve post-Newtonian runs only)
    const int threads = 256;
    const int blocks = (int)std::max<long long>(1, std::min<long long>(((long long)a.dim + threads - 1) / threads,
                                                                       (long long)num_sms * 8));
    long long force_calls = 0, iterations = 0, attempts = 0;
    // lanes per sink and source chunks as the standalone force picks them
    // (force_shape_default): from 8,192 sinks two chunks, or the symmetric
    // form when every body is massive, whose orders of sums differ from the
    // persistent engine's
    const int lanes = a.n_src <= 64 ? 1 : (a.n_src <= 1024 ? 8 : 32);
    double *partial = nullptr;
    if (lanes == 32 && a.n >= 8192) {
        EngineBuffers &e = g_eb;
        if ((size_t)a.n > e.partial_n) {
            if (e.partial) cudaFree(e.partial);
            e.partial = nullptr;
            e.partial_n = 0;
            ABIE_CUDA(cudaMalloc(&e.partial, 6 * (size_t)a.n * sizeof(double)));
            e.partial_n = (size_t)a.n;
        }
        partial = e.partial;
    }
    // every body massive: the symmetric form on the published list
    const bool sym = force_sym_applies(a.n, a.n_src);
    auto force = [&](int buf) {
        const double *pos = buf < 2 ? a.yp[buf] : a.ypa;
        const Src *src = buf < 2 ? a.src[buf] : a.srca;
        force_calls++;
        if (mixed) return launch_force_mixed_src(pos, a.m, a.n, src, &ctl->n_src, g_sim.fs, acc, st);
        if (sym) return launch_force_published_sym(src, a.n, &ctl->n_src, acc, g_sim.fs, st);
        return launch_force_published(pos, a.m, a.n, src, &ctl->n_src, lanes, acc, &ctl->next_sink, st,
                                      partial);
    };
    unsigned long long hk[2];
    auto read_keys = [&](double &v0, double &v1) -> int {
        ABIE_CUDA(cudaMemcpyAsync(hk, &ctl->red[0][0], sizeof hk, cudaMemcpyDeviceToHost, st));
        ABIE_CUDA(cudaMemsetAsync(&ctl->red[0][0], 0, sizeof hk, st));
        ABIE_CUDA(cudaStreamSynchronize(st));
        v0 = absmax_value(hk[0]);
        v1 = absmax_value(hk[1]);
        return 0;
    };
    EngineCtl c;
    auto read_ctl = [&]() -> int {
        ABIE_CUDA(cudaMemcpyAsync(&c, ctl, sizeof c, cudaMemcpyDeviceToHost, st));
        ABIE_CUDA(cudaStreamSynchronize(st));
        return 0;
    };
    int rc;
    // F1 = f(y0), then initial_time_step
    st_publish_kernel<MODE><<<blocks, threads, 0, st>>>(a, 0, 0.0, 0);
    if ((rc = force(0))) return rc;
    st_f1_kernel<<<blocks, threads, 0, st>>>(a, acc);
    st_dt0_kernel<<<1, 1, 0, st>>>(a);
    st_probe_kernel<<<blocks, threads, 0, st>>>(a);
    if ((rc = force(1))) return rc;
    st_d2_kernel<<<blocks, threads, 0, st>>>(a, acc);
    st_h0_kernel<<<1, 1, 0, st>>>(a);
    ABIE_CUDA(cudaGetLastError());
    if ((rc = read_ctl())) return rc;
    int pc = 0;
    double h = c.h;
    st_publish_kernel<MODE><<<blocks, threads, 0, st>>>(a, 1, h, pc & 1);
    for (;;) {
        int iters = 0;
        for (int ipc = 0; ipc < 12; ipc++) {
            iters++;
            for (int ih = 1; ih < 8; ih++) {
                if ((rc = force(pc & 1))) return rc;
                st_sweep_kernel<MODE><<<blocks, threads, 0, st>>>(a, acc, ih, h, pc);
                pc++;
            }
            double db6, f8;
            if ((rc = read_keys(db6, f8))) return rc;
            const bool conv = MODE == ABIE_FORCE_EXACT ? db6 / f8 < TOLPC : db6 < TOLPC * f8;
            if (conv) break;
            st_b6p_kernel<MODE><<<blocks, threads, 0, st>>>(a);
        }
        iterations += iters;
        attempts++;
        if ((rc = force(2))) return rc;
        st_advance_kernel<MODE><<<blocks, threads, 0, st>>>(a, acc);
        st_control_kernel<MODE><<<1, 1, 0, st>>>(a);
        ABIE_CUDA(cudaGetLastError());
        if ((rc = read_ctl())) return rc;
        if (c.err) break;
        bool stop = c.stop != 0;
        if (c.accepted) {
            st_accept_kernel<MODE><<<blocks, threads, 0, st>>>(a);
            st_scan_kernel<<<blocks, threads, 0, st>>>(a);
            st_commit_kernel<<<1, 1, 0, st>>>(a);
            ABIE_CUDA(cudaGetLastError());
        }
        if (!stop) {
            h = c.h;
            st_publish_kernel<MODE><<<blocks, threads, 0, st>>>(a, 1, h, pc & 1);
        }
        if (c.accepted) {
            if ((rc = read_ctl())) return rc;
            if (c.flag > 0) stop = true;
        }
        if (stop) break;
    }
    if ((rc = read_ctl())) return rc;
    c.force_calls = force_calls;
    c.iterations = iterations;
    c.attempts = attempts;
    c.phase = 2;
    *out = c;
    return 0;
}

static int g_radau_path = 0;  // debug override: 0 automatic, 1 persistent engine, 2 stepped
static long long g_engine_timeout_ns = -1;  // debug override of the barrier wait limit (-1: automatic)

template <int MODE, int JS, bool PN = false>
static int launch_engine(const EngineArgs &a, int num_sms, int block, cudaStream_t st, int *grid_out)
{
    int bps = 0;
    ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, radau_engine<MODE, JS, PN>, block, 0));
    if (bps < 1) {
        set_error(ABIE_ERR_CUDA, "radau engine does not fit on an SM");
        return ABIE_ERR_CUDA;
    }
    const int gpw = 32 / JS;
    long long want = ((long long)(a.n + gpw - 1) / gpw * 32 + block - 1) / block;
    long long grid = std::min<long long>((long long)bps * num_sms, std::max<long long>(want, 1));
    EngineArgs args = a;
    void *params[] = {&args};
    ABIE_CUDA(cudaLaunchCooperativeKernel((const void *)radau_engine<MODE, JS, PN>, dim3((unsigned)grid),
                                          dim3(block), params, 0, st));
    *grid_out = (int)grid;
    return 0;
}

static int dispatch_engine(int mode, int js, int block, const EngineArgs &a, int num_sms,
                           cudaStream_t st, int *grid)
{
    if (a.C > 0.0) {  // post-Newtonian variants: one, four or (fast form) 32 lanes per body
        if (mode == ABIE_FORCE_EXACT)
            return js >= 4 ? launch_engine<ABIE_FORCE_EXACT, 4, true>(a, num_sms, block, st, grid)
                           : launch_engine<ABIE_FORCE_EXACT, 1, true>(a, num_sms, block, st, grid);
        if (js >= 32) return launch_engine<ABIE_FORCE_FP64, 32, true>(a, num_sms, block, st, grid);
        return js >= 4 ? launch_engine<ABIE_FORCE_FP64, 4, true>(a, num_sms, block, st, grid)
                       : launch_engine<ABIE_FORCE_FP64, 1, true>(a, num_sms, block, st, grid);
    }
    if (mode == ABIE_FORCE_EXACT) {
        if (js == 4) return launch_engine<ABIE_FORCE_EXACT, 4>(a, num_sms, block, st, grid);
        return launch_engine<ABIE_FORCE_EXACT, 1>(a, num_sms, block, st, grid);
    }
    switch (js) {
    case 1: return launch_engine<ABIE_FORCE_FP64, 1>(a, num_sms, block, st, grid);
    case 4: return launch_engine<ABIE_FORCE_FP64, 4>(a, num_sms, block, st, grid);
    case 8: return launch_engine<ABIE_FORCE_FP64, 8>(a, num_sms, block, st, grid);
    case 16: return launch_engine<ABIE_FORCE_FP64, 16>(a, num_sms, block, st, grid);
    default: return launch_engine<ABIE_FORCE_FP64, 32>(a, num_sms, block, st, grid);
    }
}

static int g_engine_js = 0, g_engine_block = 0;  // debug override (0: automatic)

static const void *split_fn(int mode, bool pn)
{
    if (mode == ABIE_FORCE_EXACT)
        return pn ? (const void *)radau_split<ABIE_FORCE_EXACT, true>
                  : (const void *)radau_split<ABIE_FORCE_EXACT, false>;
    return pn ? (const void *)radau_split<ABIE_FORCE_FP64, true>
              : (const void *)radau_split<ABIE_FORCE_FP64, false>;
}

// Launch shape.  Each FP64 warp instruction occupies an SM sub-partition's
// FP64 pipe for about 64 cycles however many lanes are active, so the time
// of a substep is about (warps per sub-partition) x (FP64 instructions per
// warp).  With JS lanes per body, lanes 0..2 own x, y, z (JS >= 4) and the
// sources split JS ways; with one lane per body that lane does everything.
// The shape minimising that estimate is taken (small systems spread thin,
// large ones keep every lane busy), with blocks small enough that every SM
// gets work.  A post-Newtonian pair term (a square root, two divisions and
// ~80 other operations) costs about 110 FP64 instructions more; its fast
// form has variants of 1, 4 and 32 lanes per body.
static void engine_shape(int mode, int n, int n_src, int num_sms, bool pn, int *js, int *block)
{
    const long long subparts = 4LL * num_sms;
    const int cand_fast[5] = {1, 4, 8, 16, 32}, cand_exact[2] = {1, 4}, cand_pn[3] = {1, 4, 32};
    const int *cand = mode == ABIE_FORCE_EXACT ? cand_exact : (pn ? cand_pn : cand_fast);
    const int nc = mode == ABIE_FORCE_EXACT ? 2 : (pn ? 3 : 5);
    const double pair = (mode == ABIE_FORCE_EXACT ? 20.0 : 13.0) + (pn ? 110.0 : 0.0);  // FP64 instructions
    const double sweep = mode == ABIE_FORCE_EXACT ? 50.0 : 30.0; // per component and substep
    double best = 0.0;
    for (int k = 0; k < nc; k++) {
        const int w = cand[k];
        const long long warps = ((long long)n * w + 31) / 32;
        const long long per_sub = (warps + subparts - 1) / subparts;
        double force = mode == ABIE_FORCE_EXACT ? pair * n_src : pair * ((n_src + w - 1) / w);
        int lg = 0;
        while ((1 << lg) < w) lg++;
        const double instr = force + 3.0 * lg + (w >= 4 ? sweep : 3.0 * sweep);
        const double cost = (double)per_sub * instr;
        if (k == 0 || cost < best) {
            best = cost;
            *js = w;
        }
    }
    const long long threads = ((long long)n * *js + 31) / 32 * 32;
    long long b = (threads + num_sms - 1) / num_sms;  // one block per SM when that is enough
    b = (b + 31) / 32 * 32;
    *block = (int)std::max<long long>(32, std::min<long long>(256, b));
    if (g_engine_js > 0) *js = g_engine_js;
    if (g_engine_block > 0) *block = g_engine_block;
}

int radau_run(const SystemView &sys, double t, double t_end, int mode, EventState *evs,
              double *t_out, abie_counters *ctr, cudaStream_t st)
{
    const int n = sys.n;
    if (n <= 0) {
        *t_out = t;
        return 0;
    }
    if (mode == ABIE_FORCE_NAIVE) {
        set_error(ABIE_ERR_UNSUPPORTED,
                  "Radau15: the naive force form is the force comparator only; integrate in the "
                  "exact, fp64 or mixed form");
        return ABIE_ERR_UNSUPPORTED;
    }
    // The mixed form: the fast sweep with the mixed all-pairs force (FP32
    // pair terms for light sources) on every substep, through the stepped
    // engine, whatever the size.
    const bool mixed = mode == ABIE_FORCE_MIXED;
    if (mixed && g_sim.C > 0.0) {
        set_error(ABIE_ERR_UNSUPPORTED,
                  "Radau15: the post-Newtonian terms have no mixed form; use the exact or fp64 form");
        return ABIE_ERR_UNSUPPORTED;
    }
    if (mixed) mode = ABIE_FORCE_FP64;
    size_t max_ce = evs ? evs->max_ce : 0, max_coll = evs ? evs->max_coll : 0;
    int rc = engine_reserve((size_t)n, max_ce, max_coll);
    if (rc) return rc;
    EngineBuffers &e = g_eb;
    const size_t d = 3 * (size_t)n;

    // source list: massive bodies in body order
    std::vector<int> body, slot(n, -1);
    double rmax = 0.0;
    for (int j = 0; j < n; j++) {
        if (sys.h_m[j] > 0.0) {
            slot[j] = (int)body.size();
            body.push_back(j);
        }
        if (sys.h_r && sys.h_r[j] > rmax) rmax = sys.h_r[j];
    }
    int n_src = (int)body.size();
    if (n_src) ABIE_CUDA(cudaMemcpyAsync(e.src_body, body.data(), n_src * sizeof(int), cudaMemcpyHostToDevice, st));
    std::vector<int> tps;
    for (int j = 0; j < n; j++)
        if (!(sys.h_m[j] > 0.0)) tps.push_back(j);
    const int n_tp = (int)tps.size();
    if (n_tp) ABIE_CUDA(cudaMemcpyAsync(e.tp_body, tps.data(), n_tp * sizeof(int), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(e.src_slot, slot.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));

    ABIE_CUDA(cudaMemsetAsync(e.slab, 0, (size_t)n * SLAB_PER_BODY * sizeof(double), st));
    EngineArgs a = {};
    a.n = n;
    a.dim = (int)d;
    a.n_src = n_src;
    a.src_body = e.src_body;
    a.tp_body = e.tp_body;
    a.n_tp = n_tp;
    a.src_slot = e.src_slot;
    a.m = sys.m;
    a.r = sys.r;
    a.ext = sys.ext;
    a.G = sys.G;
    double *p = e.slab;
    a.y0 = p; p += d;
    a.dy0 = p; p += d;
    a.F1 = p; p += d;
    a.b = p; p += 7 * d;
    a.g = p; p += 7 * d;
    a.b6p = p; p += d;
    a.ddy = p; p += d;
    a.dyp = p; p += d;
    a.yp[0] = p; p += d;
    a.yp[1] = p; p += d;
    a.ypa = p; p += d;
    a.vp[0] = p; p += d;
    a.vp[1] = p; p += d;
    a.ypf = reinterpret_cast<float2 *>(p); p += d;
    a.src[0] = e.srcs;
    a.src[1] = e.srcs + n;
    a.srca = e.srcs + 2 * n;
    a.t_end = t_end;
    a.C = g_sim.C;  // the stored speed of light, as src/common.c:101-107 reads it
    a.pn = pn_const(sys.G, a.C > 0.0 ? a.C : 1.0);
    double ce = evs ? evs->ce_dist : 0.0;
    a.ce_dist = ce;
    double thr = std::max(ce, 2.0 * rmax);
    a.thr2 = thr * thr * (1.0 + 1e-12);
    a.max_ce = (long long)max_ce;
    a.max_coll = (long long)max_coll;
    a.buf_ce = max_ce ? e.d_ce : nullptr;
    a.buf_coll = max_coll ? e.d_coll : nullptr;
    a.ev = e.ev;
    a.ev_cap = EV_CAP;
    a.ctl = e.ctl;
    // a phase's work bounds its barrier wait (post-Newtonian pairs cost ~20x more)
    a.timeout_ns = 2000000000ll + (a.C > 0.0 ? 240ll : 12ll) * (long long)n * (long long)std::max(n_src, 1);
    if (g_engine_timeout_ns >= 0) a.timeout_ns = g_engine_timeout_ns;

    ABIE_CUDA(cudaMemcpyAsync(a.y0, sys.pos, d * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(a.dy0, sys.vel, d * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (evs && max_ce)
        ABIE_CUDA(cudaMemcpyAsync(e.d_ce, evs->buf_ce->data(), 4 * max_ce * sizeof(double),
                                  cudaMemcpyHostToDevice, st));
    if (evs && max_coll)
        ABIE_CUDA(cudaMemcpyAsync(e.d_coll, evs->buf_coll->data(), 4 * max_coll * sizeof(double),
                                  cudaMemcpyHostToDevice, st));
    EngineCtl c0;
    memset(&c0, 0, sizeof c0);
    c0.t = t;
    c0.n_ce = evs ? *evs->n_ce : 0;
    c0.n_coll = evs ? *evs->n_coll : 0;
    c0.n_src = n_src;
    ABIE_CUDA(cudaMemcpyAsync(e.ctl, &c0, sizeof c0, cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaStreamSynchronize(st));

    int js = 1, block = 256;
    engine_shape(mode, n, n_src, g_sim.num_sms, a.C > 0.0, &js, &block);
    // few massive bodies: the split engine (a replica of them per block),
    // unless a launch shape is forced or the particles exceed one
    // resident wave
    bool split = false;
    if (n_src <= 10 && g_engine_js == 0 && !mixed) {
        int bps = 0;
        ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, split_fn(mode, a.C > 0.0), 64, 0));
        split = (long long)std::max(1, (n_tp + SPLIT_TPW - 1) / SPLIT_TPW) <=
                (long long)bps * g_sim.num_sms;
    }
    EngineCtl c;
    // large systems in the fast form without post-Newtonian terms: the
    // stepped engine (the standalone force kernel for every substep)
    const bool stepped =
        mixed || (!split && a.C <= 0.0 && mode == ABIE_FORCE_FP64 &&
                  (g_radau_path == 2 ||
                   (g_radau_path == 0 && g_engine_js == 0 && (long long)n * (long long)n_src >= (1ll << 20))));
    if (stepped) {
        rc = stepped_run<ABIE_FORCE_FP64>(a, g_sim.num_sms, st, &c, mixed);
        if (rc) return rc;
        if (c.err) {
            set_error(c.err, "radau engine stopped (code %d, t=%g)", c.err, c.t);
            return c.err;
        }
    }
    long long budget = 4;
    for (; !stepped;) {
        a.attempt_budget = budget;
        cudaEvent_t e0, e1;
        ABIE_CUDA(cudaEventCreate(&e0));
        ABIE_CUDA(cudaEventCreate(&e1));
        ABIE_CUDA(cudaEventRecord(e0, st));
        int grid = 0;
        if (split) {
            EngineArgs args = a;
            void *params[] = {&args};
            grid = std::max(1, (n_tp + SPLIT_TPW - 1) / SPLIT_TPW);
            ABIE_CUDA(cudaLaunchCooperativeKernel(split_fn(mode, a.C > 0.0), dim3((unsigned)grid), dim3(64),
                                                  params, 0, st));
            rc = 0;
        } else {
            rc = dispatch_engine(mode, js, block, a, g_sim.num_sms, st, &grid);
        }
        if (rc) return rc;
        ABIE_CUDA(cudaEventRecord(e1, st));
        ABIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ABIE_CUDA(cudaMemcpy(&c, e.ctl, sizeof c, cudaMemcpyDeviceToHost));
        if (c.err) {
            set_error(c.err, "radau engine stopped (code %d, t=%g)", c.err, c.t);
            return c.err;
        }
        if (c.phase == 2) break;
        // aim each launch at about 100 ms of GPU time
        double per = ms / (double)std::max<long long>(budget, 1);
        long long next = per > 0 ? (long long)(100.0 / per) : budget * 4;
        budget = std::max<long long>(1, std::min<long long>(next, budget * 8));
        budget = std::min<long long>(budget, 1 << 20);
    }
    if (c.ev_overflow) {
        set_error(ABIE_ERR_CAPACITY, "more than %d events in one check; ring buffers incomplete",
                  EV_CAP);
    }
    ABIE_CUDA(cudaMemcpyAsync(sys.pos, a.y0, d * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(sys.vel, a.dy0, d * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (evs && max_ce)
        ABIE_CUDA(cudaMemcpyAsync(evs->buf_ce->data(), e.d_ce, 4 * max_ce * sizeof(double),
                                  cudaMemcpyDeviceToHost, st));
    if (evs && max_coll)
        ABIE_CUDA(cudaMemcpyAsync(evs->buf_coll->data(), e.d_coll, 4 * max_coll * sizeof(double),
                                  cudaMemcpyDeviceToHost, st));
    ABIE_CUDA(cudaStreamSynchronize(st));
    if (evs) {
        *evs->n_ce = (size_t)c.n_ce;
        *evs->n_coll = (size_t)c.n_coll;
    }
    *t_out = c.t;
    if (ctr) {
        ctr->force_calls += c.force_calls;
        ctr->iterations += c.iterations;
        ctr->attempts += c.attempts;
        ctr->accepts += c.accepts;
        ctr->rejects += c.rejects;
        ctr->last_h = c.h;
    }
    return c.flag;
}

}  // namespace abie

using namespace abie;

extern "C" {

void abie_debug_radau_path(int path) { g_radau_path = (path == 1 || path == 2) ? path : 0; }

void abie_debug_engine_timeout(long long ns) { g_engine_timeout_ns = ns >= 0 ? ns : -1; }

void abie_debug_engine_shape(int lanes_per_body, int block)
{
    const bool ok_js = lanes_per_body == 0 || lanes_per_body == 1 || lanes_per_body == 4 ||
                       lanes_per_body == 8 || lanes_per_body == 16 || lanes_per_body == 32;
    const bool ok_block = block == 0 || (block >= 32 && block <= 256 && block % 32 == 0);
    g_engine_js = ok_js ? lanes_per_body : 0;
    g_engine_block = ok_block ? block : 0;
}

int integrator_gr(double t, double t_end, double dt)
{
    (void)dt;  // ignored, as in the reference (h comes from initial_time_step)
    Sim &s = g_sim;
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "integrator_gr before initialize_code");
        return ABIE_ERR_NOT_INITIALIZED;
    }
    SystemView v{s.pos, s.vel, s.m, s.r, s.ext_enabled ? s.ext_acc : nullptr,
                 s.h_m.data(), s.h_r.data(), (int)s.n, s.G};
    EventState ev{s.ce_dist, s.max_ce, s.max_coll, &s.n_ce, &s.n_coll, &s.buf_ce, &s.buf_coll};
    double t_out = t;
    int rc = radau_run(v, t, t_end, s.force_mode, &ev, &t_out, &s.ctr, s.st);
    if (rc >= 0) s.t = t_out;
    return rc;
}

size_t integrator_gauss_radau15(double *pos, double *vel, double *m_vec, double *r_vec, size_t N,
                                double G, double t, double t_end, double dt)
{
    (void)dt;
    int rc = ensure_device(-1);
    if (rc) return (size_t)(long long)rc;
    Sim &s = g_sim;
    N &= 0xffffffffull;
    double *dp = nullptr, *dv = nullptr, *dm = nullptr, *dr = nullptr;
    size_t cp = 0, cv = 0, cm = 0, cr = 0;
    if ((rc = reserve(&dp, &cp, 3 * N)) || (rc = reserve(&dv, &cv, 3 * N)) ||
        (rc = reserve(&dm, &cm, N)) || (rc = reserve(&dr, &cr, N)))
        return (size_t)(long long)rc;
    cudaMemcpy(dp, pos, 3 * N * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dv, vel, 3 * N * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dm, m_vec, N * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dr, r_vec, N * 8, cudaMemcpyHostToDevice);
    // the external accelerations of set_additional_forces apply here too,
    // as the reference's calculate_accelerations adds them to every call
    const double *ext = (s.inited && s.ext_enabled && N <= s.n_max) ? s.ext_acc : nullptr;
    SystemView v{dp, dv, dm, dr, ext, m_vec, r_vec, (int)N, G};
    EventState ev{s.ce_dist, s.max_ce, s.max_coll, &s.n_ce, &s.n_coll, &s.buf_ce, &s.buf_coll};
    double t_out = t;
    rc = radau_run(v, t, t_end, s.force_mode, s.inited ? &ev : nullptr, &t_out, &s.ctr, s.st);
    if (rc >= 0) {
        cudaMemcpy(pos, dp, 3 * N * 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(vel, dv, 3 * N * 8, cudaMemcpyDeviceToHost);
        s.t = t_out;
    }
    cudaFree(dp);
    cudaFree(dv);
    cudaFree(dm);
    cudaFree(dr);
    return (size_t)(long long)rc;
}

}
