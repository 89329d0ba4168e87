// Post-Newtonian pair terms (src/additional_forces.c:14-121), on the device:
// 1PN, 2PN and 2.5PN of source k acting on sink j, summed over k by the
// caller and added to the Newtonian acceleration.  pn_pair keeps the
// reference's expressions and order (built with --fmad=false; the exact
// force form); pn_pair_fast regroups them without square root or division
// (the fast form).
//
// Sources of zero mass contribute exact zeros to a sink of nonzero mass
// (every term carries G m_k or nu = m_j m_k / (m_j + m_k)^2), so callers may
// skip them; for a massless sink and a massless source the reference
// evaluates 0/0 and its acceleration becomes NaN, while skipping gives the
// physical zero.
#pragma once
#include "common.cuh"

namespace abie {

struct PnConst {
    double G, CM2, CM5;  // G, C^-2, C^-5 (as src/additional_forces.c:27-30 forms them)
};

__host__ __device__ inline PnConst pn_const(double G, double C)
{
    PnConst k;
    const double CM1 = 1.0 / C;
    k.G = G;
    k.CM2 = CM1 * CM1;
    const double CM4 = k.CM2 * k.CM2;
    k.CM5 = CM1 * CM4;
    return k;
}

// Terms of source (xk, vk, Mk) on sink (x, v, Mj), added to (ax, ay, az).
static __device__ __noinline__ void pn_pair(const PnConst &K, double x, double y, double z, double vx,
                                        double vy, double vz, double Mj, double xk, double yk,
                                        double zk, double vxk, double vyk, double vzk, double Mk,
                                        double &ax, double &ay, double &az)
{
    const double c8div5 = (8.0 / 5.0), c17div3 = (17.0 / 3.0);
    const double GM = K.G * Mk;
    const double GM_C_PM2 = GM * K.CM2;
    const double GM_P2_C_PM2 = GM * GM_C_PM2;
    const double dx = x - xk, dy = y - yk, dz = z - zk;
    const double dvx = vx - vxk, dvy = vy - vyk, dvz = vz - vzk;
    const double r_dot_v = dx * dvx + dy * dvy + dz * dvz;
    const double v_dot_v = dvx * dvx + dvy * dvy + dvz * dvz;
    const double rel_sep2 = dx * dx + dy * dy + dz * dz;
    const double rel_sep1 = sqrt(rel_sep2);
    const double d1 = 1.0 / rel_sep1;
    const double d2 = d1 * d1;
    const double d3 = d1 * d2;
    const double d4 = d1 * d3;
    // 1PN
    const double F0 = 4.0 * GM_C_PM2 * r_dot_v * d3;
    const double F1 = 4.0 * GM_P2_C_PM2 * d4;
    const double F2 = -GM_C_PM2 * v_dot_v * d3;
    ax += F0 * dvx + F1 * dx + F2 * dx;
    ay += F0 * dvy + F1 * dy + F2 * dy;
    az += F0 * dvz + F1 * dz + F2 * dz;
    // 2PN
    const double GM_P2_RC_PM4 = GM_P2_C_PM2 * K.CM2 * d4;
    const double G0 = 2.0 * r_dot_v * r_dot_v * d2;
    const double G1 = -9.0 * GM * d1;
    const double G2 = -2.0 * r_dot_v;
    ax += GM_P2_RC_PM4 * (G0 * dx + G1 * dx + G2 * dvx);
    ay += GM_P2_RC_PM4 * (G0 * dy + G1 * dy + G2 * dvy);
    az += GM_P2_RC_PM4 * (G0 * dz + G1 * dz + G2 * dvz);
    // 2.5PN
    const double M_tot = Mj + Mk;
    const double nu = Mj * Mk / (M_tot * M_tot);
    const double GM_tot = K.G * M_tot;
    const double H0 = -c8div5 * GM_tot * GM_tot * nu * K.CM5 * d3;
    const double H1 = v_dot_v + 3.0 * GM_tot * d1;
    const double H2 = -(3.0 * v_dot_v + c17div3 * GM_tot * d1) * r_dot_v * d2;
    ax += H0 * (H1 * dvx + H2 * dx);
    ay += H0 * (H1 * dvy + H2 * dy);
    az += H0 * (H1 * dvz + H2 * dz);
}

// Fast form of pn_pair: the same three terms, regrouped so that each sums
// to A d + B dv,
//   A = (F1 + F2) + P (G0 + G1) + H0 H2,   B = F0 + P G2 + H0 H1,
// with F1 + F2 = (G m_k / c^2) r^-3 (4 G m_k / r - v^2) and, since
// (G M)^2 nu = G^2 m_j m_k, H0 = -8/5 G^2 m_j m_k c^-5 r^-3: no square root
// and no division (r^-3 from the integer core of the Newtonian term, r^-1 =
// r^2 r^-3), two FMAs per component, ~60 FP64 instructions against ~136.
// Coincident bodies (r = 0) add nothing.  The terms round differently from
// the reference's expressions; they are ~(v/c)^2 of the Newtonian
// acceleration, so the difference stays far below FP64 rounding of the total.
static __device__ __noinline__ void pn_pair_fast(const PnConst &K, double x, double y, double z,
                                                 double vx, double vy, double vz, double Mj,
                                                 double xk, double yk, double zk, double vxk,
                                                 double vyk, double vzk, double Mk, double &ax,
                                                 double &ay, double &az)
{
    const double dx = x - xk, dy = y - yk, dz = z - zk;
    unsigned long long Mr, Wn;
    int Er, eW;
    r2_int(dx, dy, dz, Mr, Er);
    if (Mr == 0ull) return;
    inv_r3_core(Mr, Er, Wn, eW);
    const double d3 = gm_times_inv_r3(Wn, eW, 1.0);
    const double dvx = vx - vxk, dvy = vy - vyk, dvz = vz - vzk;
    const double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
    const double rv = fma(dz, dvz, fma(dy, dvy, dx * dvx));
    const double vv = fma(dvz, dvz, fma(dvy, dvy, dvx * dvx));
    const double d1 = r2 * d3, d2 = d1 * d1;
    const double GM = K.G * Mk, gc = GM * K.CM2;
    // 1PN
    const double F0 = 4.0 * gc * rv * d3;
    const double F12 = gc * d3 * fma(4.0 * GM, d1, -vv);
    // 2PN
    const double P = GM * gc * K.CM2 * (d2 * d2);
    const double G01 = fma(2.0 * rv * rv, d2, -9.0 * GM * d1);
    const double G2 = -2.0 * rv;
    // 2.5PN
    const double GMt = K.G * (Mj + Mk);
    const double H0 = -(8.0 / 5.0) * (K.G * Mj) * GM * K.CM5 * d3;
    const double H1 = fma(3.0 * GMt, d1, vv);
    const double H2 = -fma(3.0, vv, (17.0 / 3.0) * GMt * d1) * rv * d2;
    const double A = F12 + fma(P, G01, H0 * H2);
    const double B = F0 + fma(P, G2, H0 * H1);
    ax = fma(A, dx, fma(B, dvx, ax));
    ay = fma(A, dy, fma(B, dvy, ay));
    az = fma(A, dz, fma(B, dvz, az));
}

// The pair term of the force form: the reference's expressions (exact) or
// the regrouped fast form.
template <int MODE>
__device__ __forceinline__ void pn_term(const PnConst &K, double x, double y, double z, double vx,
                                        double vy, double vz, double Mj, double xk, double yk,
                                        double zk, double vxk, double vyk, double vzk, double Mk,
                                        double &ax, double &ay, double &az)
{
    if (MODE == ABIE_FORCE_EXACT)
        pn_pair(K, x, y, z, vx, vy, vz, Mj, xk, yk, zk, vxk, vyk, vzk, Mk, ax, ay, az);
    else
        pn_pair_fast(K, x, y, z, vx, vy, vz, Mj, xk, yk, zk, vxk, vyk, vzk, Mk, ax, ay, az);
}

// acc[j] += sum over k != j with m_k != 0 of the pair terms, for all n sinks.
// fast: the regrouped pair term (pn_pair_fast) instead of the reference's.
int launch_post_newtonian(const double *pos, const double *vel, const double *m, int n, double G,
                          double C, double *acc, cudaStream_t st, bool fast = false);

}  // namespace abie
