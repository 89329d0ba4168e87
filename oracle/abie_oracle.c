/*
 * CPU oracle for ABIE's gravity hot path -- TEST INFRASTRUCTURE ONLY.
 * See abie_oracle.h.  Built with -std=c99 -ffp-contract=off so that every
 * product and sum is rounded on its own, exactly like the reference build
 * (gcc -O3 -std=c99, which implies no FMA contraction).
 *
 * Every expression below keeps the reference's operand order; that order is
 * what makes the results bit-identical, so where a line looks unusual (for
 * example (G*m)*aux*diff instead of G*(m*aux*diff)) it is deliberate.
 */
#define _POSIX_C_SOURCE 200809L
#include "abie_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "radau_constants.h"

/* ------------------------------------------------------------------ */
/* Force: src/common.c:39-77                                          */
/* ------------------------------------------------------------------ */
void orc_force(const double *pos, size_t n, double G, const double *m,
               double *acc, size_t j0, size_t j1)
{
    for (size_t j = j0; j < j1 && j < n; j++) {
        if (m[j] < 0.0) continue; /* deleted particle: acc left as is (:49) */
        const double xj = pos[3 * j], yj = pos[3 * j + 1], zj = pos[3 * j + 2];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (size_t k = 0; k < n; k++) {
            if (k == j || m[k] <= 0.0) continue; /* :60 */
            const double gm = G * m[k];
            const double dx = xj - pos[3 * k];
            const double dy = yj - pos[3 * k + 1];
            const double dz = zj - pos[3 * k + 2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double r1 = sqrt(r2);
            const double r3 = r1 * r2;
            ax -= gm * dx / r3;
            ay -= gm * dy / r3;
            az -= gm * dz / r3;
        }
        acc[3 * j] = ax;
        acc[3 * j + 1] = ay;
        acc[3 * j + 2] = az;
    }
}

typedef struct {
    const double *pos, *m;
    double *acc;
    size_t n, j0, j1;
    double G;
} force_job;

static void *force_worker(void *arg)
{
    force_job *w = (force_job *)arg;
    orc_force(w->pos, w->n, w->G, w->m, w->acc, w->j0, w->j1);
    return NULL;
}

int orc_force_threads(const double *pos, size_t n, double G, const double *m,
                      double *acc, size_t j0, size_t j1, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (j1 > n) j1 = n;
    if (j0 >= j1) return 0;
    size_t span = j1 - j0;
    if ((size_t)nthreads > span) nthreads = (int)span;
    pthread_t *tid = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    force_job *jobs = (force_job *)calloc((size_t)nthreads, sizeof(force_job));
    if (!tid || !jobs) { free(tid); free(jobs); return -1; }
    int started = 0, rc = 0;
    for (int t = 0; t < nthreads; t++) {
        jobs[t].pos = pos; jobs[t].m = m; jobs[t].acc = acc; jobs[t].n = n; jobs[t].G = G;
        jobs[t].j0 = j0 + span * (size_t)t / (size_t)nthreads;
        jobs[t].j1 = j0 + span * (size_t)(t + 1) / (size_t)nthreads;
        if (pthread_create(&tid[t], NULL, force_worker, &jobs[t]) != 0) {
            force_worker(&jobs[t]); /* run inline if a thread cannot start */
            tid[t] = 0;
            rc = 1;
        } else {
            started++;
        }
    }
    for (int t = 0; t < nthreads; t++)
        if (tid[t]) pthread_join(tid[t], NULL);
    free(tid);
    free(jobs);
    (void)started;
    return rc;
}

/* ------------------------------------------------------------------ */
/* Small vector helpers: src/common.c:192-223                           */
/* ------------------------------------------------------------------ */
static double max_abs(const double *v, size_t n)
{
    double best = -DBL_MAX; /* :317; NaN never replaces it */
    for (size_t i = 0; i < n; i++) {
        double a = fabs(v[i]);
        if (best < a) best = a;
    }
    return best;
}

static double norm3(const double *v)
{
    double s = 0.0;
    s += v[0] * v[0];
    s += v[1] * v[1];
    s += v[2] * v[2];
    return sqrt(s);
}

static double dot3(const double *a, const double *b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

static double cross_norm3(const double *a, const double *b)
{
    double c0 = a[1] * b[2] - a[2] * b[1];
    double c1 = a[2] * b[0] - a[0] * b[2];
    double c2 = a[0] * b[1] - a[1] * b[0];
    return sqrt(c0 * c0 + c1 * c1 + c2 * c2);
}

static double sgn(double x) { return (double)((x > 0) - (x < 0)); }

/* ------------------------------------------------------------------ */
/* Energy: src/common.c:340-357                                         */
/* ------------------------------------------------------------------ */
double orc_energy(const double *pos, const double *vel, const double *m,
                  size_t n, double G)
{
    double e = 0.0;
    double d[3];
    for (size_t i = 0; i < n; i++) {
        if (m[i] == 0) continue;
        e += 0.5 * m[i] * pow(norm3(&vel[3 * i]), 2.0);
        for (size_t j = 0; j < n; j++) {
            if (i == j || m[j] == 0) continue;
            d[0] = pos[3 * i] - pos[3 * j];
            d[1] = pos[3 * i + 1] - pos[3 * j + 1];
            d[2] = pos[3 * i + 2] - pos[3 * j + 2];
            e -= 0.5 * G * m[i] * m[j] / norm3(d);
        }
    }
    return e;
}

/* ------------------------------------------------------------------ */
/* Close encounters and collisions: src/common.c:116-158                */
/* ------------------------------------------------------------------ */
static void ring_put(double *buf, size_t count, size_t cap, double t, size_t i,
                     size_t j, double d)
{
    if (!buf || cap == 0) return;
    size_t w = 4 * cap;
    buf[(4 * count) % w] = t;
    buf[(4 * count + 1) % w] = (double)i;
    buf[(4 * count + 2) % w] = (double)j;
    buf[(4 * count + 3) % w] = d;
}

int orc_check_events(const double *pos, const double *r, size_t n, double t,
                     orc_events *ev)
{
    for (size_t j = 0; j < n; j++) {
        for (size_t k = j + 1; k < n; k++) { /* the reference tests j<k (:133,:144) */
            double dx = pos[3 * j] - pos[3 * k];
            double dy = pos[3 * j + 1] - pos[3 * k + 1];
            double dz = pos[3 * j + 2] - pos[3 * k + 2];
            double sep = sqrt(dx * dx + dy * dy + dz * dz);
            double rr = r[j] + r[k];
            if (sep <= ev->ce_dist) {
                ring_put(ev->buf_ce, ev->n_ce, ev->max_ce, t, j, k, sep);
                ev->n_ce += 1;
            }
            if (rr > 0 && sep <= rr) {
                ring_put(ev->buf_coll, ev->n_coll, ev->max_coll, t, j, k, sep);
                ev->n_coll += 1;
            }
        }
    }
    if (ev->max_ce > 0 && ev->n_ce >= ev->max_ce) return 1;
    if (ev->max_coll > 0 && ev->n_coll >= ev->max_coll) return 2;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Gauss-Radau 15: src/integrator_gauss_radau15.c                       */
/* ------------------------------------------------------------------ */
static const double HS[8] = ABIE_RADAU_HS_INIT;
static const double RS[8][8] = ABIE_RADAU_RS_INIT;
static const double CS[8][8] = ABIE_RADAU_CS_INIT;
static const double EPSB = 1.e-4;        /* .h:58 */
static const double FAC = 0.25;          /* .h:59 */
static const double TOLPC = 1.e-16;      /* .h:63 */
static const double H_MIN = 1.e-13;      /* .h:17 */
#define EXPONENT (1. / 7)                /* .h:61 */

/* src/additional_forces.c:14-121: adds the 1PN, 2PN and 2.5PN terms of
 * every pair to acc (the pair loop runs over all k != j, massless bodies
 * included). */
void orc_post_newtonian(const double *pos, const double *vel, size_t n, double G, double C,
                        const double *m, double *acc)
{
    double CM1 = 1.0 / C;
    double CM2 = CM1 * CM1;
    double CM4 = CM2 * CM2;
    double CM5 = CM1 * CM4;
    double c8div5 = (8.0 / 5.0);
    double c17div3 = (17.0 / 3.0);
    for (size_t j = 0; j < n; j++) {
        double x = pos[j * 3], y = pos[j * 3 + 1], z = pos[j * 3 + 2];
        double vx = vel[j * 3], vy = vel[j * 3 + 1], vz = vel[j * 3 + 2];
        double M_j = m[j];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (size_t k = 0; k < n; k++) {
            if (j == k) continue;
            double M_k = m[k];
            double GM = G * M_k;
            double GM_C_PM2 = GM * CM2;
            double GM_P2_C_PM2 = GM * GM_C_PM2;
            double dx = x - pos[k * 3], dy = y - pos[k * 3 + 1], dz = z - pos[k * 3 + 2];
            double dvx = vx - vel[k * 3], dvy = vy - vel[k * 3 + 1], dvz = vz - vel[k * 3 + 2];
            double r_dot_v = dx * dvx + dy * dvy + dz * dvz;
            double v_dot_v = dvx * dvx + dvy * dvy + dvz * dvz;
            double rel_sep2 = dx * dx + dy * dy + dz * dz;
            double rel_sep1 = sqrt(rel_sep2);
            double d1 = 1.0 / rel_sep1;
            double d2 = d1 * d1;
            double d3 = d1 * d2;
            double d4 = d1 * d3;
            /* 1PN */
            double F0 = 4.0 * GM_C_PM2 * r_dot_v * d3;
            double F1 = 4.0 * GM_P2_C_PM2 * d4;
            double F2 = -GM_C_PM2 * v_dot_v * d3;
            ax += F0 * dvx + F1 * dx + F2 * dx;
            ay += F0 * dvy + F1 * dy + F2 * dy;
            az += F0 * dvz + F1 * dz + F2 * dz;
            /* 2PN */
            double GM_P2_RC_PM4 = GM_P2_C_PM2 * CM2 * d4;
            double G0 = 2.0 * r_dot_v * r_dot_v * d2;
            double G1 = -9.0 * GM * d1;
            double G2 = -2.0 * r_dot_v;
            ax += GM_P2_RC_PM4 * (G0 * dx + G1 * dx + G2 * dvx);
            ay += GM_P2_RC_PM4 * (G0 * dy + G1 * dy + G2 * dvy);
            az += GM_P2_RC_PM4 * (G0 * dz + G1 * dz + G2 * dvz);
            /* 2.5PN */
            double M_tot = M_j + M_k;
            double nu = M_j * M_k / (M_tot * M_tot);
            double GM_tot = G * M_tot;
            double H0 = -c8div5 * GM_tot * GM_tot * nu * CM5 * d3;
            double H1 = v_dot_v + 3.0 * GM_tot * d1;
            double H2 = -(3.0 * v_dot_v + c17div3 * GM_tot * d1) * r_dot_v * d2;
            ax += H0 * (H1 * dvx + H2 * dx);
            ay += H0 * (H1 * dvy + H2 * dy);
            az += H0 * (H1 * dvz + H2 * dz);
        }
        acc[j * 3] += ax;
        acc[j * 3 + 1] += ay;
        acc[j * 3 + 2] += az;
    }
}

/* The GPU fast form's arithmetic in orc_radau15, for the long-horizon
 * accuracy study only (not bit-identical to the device: the device takes
 * G m r^-3 by integer arithmetic within 0.53 ulp and its own single-
 * precision log2 / exp2).  Five changes from the reference's operations:
 * each pair term's G m r^-3 formed once and the sums by FMA; the
 * corrector's new g coefficient from the expanded recurrence (one FMA per
 * term); positions predicted from g with the tabulated weights, the
 * displacement formed first and added to y0 once; the step-size seventh
 * root in single precision; each step started from g consistent with the
 * refined guess.  Newtonian forces only. */
static int g_orc_fast = 0;
void orc_set_fastform(int on) { g_orc_fast = on; }

static void orc_force_fastform(const double *pos, size_t n, double G, const double *m, double *acc)
{
    for (size_t j = 0; j < n; j++) {
        if (m[j] < 0.0) continue;
        const double xj = pos[3 * j], yj = pos[3 * j + 1], zj = pos[3 * j + 2];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (size_t k = 0; k < n; k++) {
            if (k == j || m[k] <= 0.0) continue;
            const double gm = G * m[k];
            const double dx = xj - pos[3 * k], dy = yj - pos[3 * k + 1], dz = zj - pos[3 * k + 2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double w = gm / (sqrt(r2) * r2);
            ax = fma(-w, dx, ax);
            ay = fma(-w, dy, ay);
            az = fma(-w, dz, az);
        }
        acc[3 * j] = ax;
        acc[3 * j + 1] = ay;
        acc[3 * j + 2] = az;
    }
}

/* src/common.c:82-114: Newton, then the post-Newtonian terms when C > 0,
 * then the external accelerations when set (:107-112, added component by
 * component after the other terms). */
static double g_orc_C = 0.0;
static const double *g_orc_ext = NULL;
static void force_counted_v(const double *y, const double *dy, size_t n, double G, const double *m,
                            double *acc, orc_radau_stats *st)
{
    /* sinks with negative mass keep a zero acceleration (the reference leaves
     * their entries of freshly malloc'd buffers untouched) */
    memset(acc, 0, 3 * n * sizeof(double));
    if (g_orc_fast) orc_force_fastform(y, n, G, m, acc);
    else orc_force(y, n, G, m, acc, 0, n);
    if (g_orc_C > 0.0) orc_post_newtonian(y, dy, n, G, g_orc_C, m, acc);
    if (g_orc_ext)
        for (size_t i = 0; i < 3 * n; i++) acc[i] += g_orc_ext[i];
    if (st) st->force_calls++;
}

/* Speed of light for the oracle's Radau15 (0: no post-Newtonian terms). */
void orc_set_pn(double C) { g_orc_C = C; }


/* External accelerations (3N, kept by pointer) added to every force call of
 * the oracle's Radau15, like src/common.c:364-380 with :107-112; NULL: none. */
void orc_set_ext(const double *ext) { g_orc_ext = ext; }

/* :9-54 */
static double initial_step(const double *y0, const double *dy0, double G,
                           const double *m, size_t n, orc_radau_stats *st)
{
    const int p = 15;
    size_t dim = 3 * n;
    double *f0 = (double *)malloc(dim * sizeof(double));
    double *f1 = (double *)malloc(dim * sizeof(double));
    double *y1 = (double *)malloc(dim * sizeof(double));
    double *dy1 = (double *)malloc(dim * sizeof(double));
    double dt0, dt1;
    force_counted_v(y0, dy0, n, G, m, f0, st);
    double d0 = max_abs(y0, n); /* the reference scans n (not 3n) entries (:23-24) */
    double d1 = max_abs(f0, n);
    if (d0 < 1e-5 || d1 < 1e-5) dt0 = 1e-6;
    else dt0 = 0.01 * (d0 / d1);
    for (size_t i = 0; i < dim; i++) {
        y1[i] = y0[i] + dt0 * dy0[i];
        dy1[i] = dy0[i] + dt0 * f0[i];
    }
    force_counted_v(y1, dy1, n, G, m, f1, st);
    double d2 = -DBL_MAX;
    for (size_t i = 0; i < dim; i++) {
        double a = fabs(f1[i] - f0[i]);
        if (d2 < a) d2 = a;
    }
    d2 = d2 / dt0;
    if (fmax(d1, d2) <= 1e-15) dt1 = fmax(1e-6, dt0 * 1e-3);
    else dt1 = pow(0.01 / fmax(d1, d2), (1.0 / (p + 1)));
    double dt = fmin(100 * dt0, dt1);
    free(f0); free(f1); free(y1); free(dy1);
    return dt;
}

/* :56-61 and :63-68.  The reference's parameter named h receives the
 * Radau spacing s (hs[ih], or 1 for the advance) and the one named T receives
 * the step dt: y = y1 + dt s (dy1 + dt s (F1 + s (b0/3 + s (b1/6 + ...))) / 2). */
static void predict_pos(const double *y1, const double *dy1, const double *F1,
                        double s, double *const b[7], size_t dim, double dt,
                        double *y)
{
    for (size_t i = 0; i < dim; i++) {
        y[i] = y1[i] + dt * s * (dy1[i] + dt * s * (F1[i] + s * (b[0][i] / 0.3e1 + s * (b[1][i] / 0.6e1 + s * (b[2][i] / 0.10e2 + s * (b[3][i] / 0.15e2 + s * (b[4][i] / 0.21e2 + s * (b[5][i] / 0.28e2 + s * b[6][i] / 0.36e2))))))) / 0.2e1);
    }
}

static void predict_vel(const double *dy1, const double *F1, double s,
                        double *const b[7], size_t dim, double dt, double *dy)
{
    for (size_t i = 0; i < dim; i++) {
        dy[i] = dy1[i] + dt * s * (F1[i] + s * (b[0][i] / 0.2e1 + s * (b[1][i] / 0.3e1 + s * (b[2][i] / 0.4e1 + s * (b[3][i] / 0.5e1 + s * (b[4][i] / 0.6e1 + s * (b[5][i] / 0.7e1 + s * b[6][i] / 0.8e1)))))));
    }
}

/* :70-121.  At substep ih the reference recomputes g[0..ih-1] from the
 * sampled forces; the nested form below is the same recurrence, evaluated
 * in the same order: g_k = ((..((F_{k+1}-F_0)*r_{k+1,0} - g_0)*r_{k+1,1} ..)
 *                          - g_{k-1}) * r_{k+1,k}. */
static void update_g(double *const F[8], int ih, size_t dim, double *g[7])
{
    for (size_t i = 0; i < dim; i++) {
        for (int k = 0; k < ih; k++) {
            double v = (F[k + 1][i] - F[0][i]) * RS[k + 1][0];
            for (int l = 1; l <= k; l++) v = (v - g[l - 1][i]) * RS[k + 1][l];
            g[k][i] = v;
        }
    }
}

/* The fast form's pieces (orc_set_fastform): the new g from the expanded
 * recurrence, (F - F1) rsp[ih][0] - sum_l g_l rsp[ih][l+1]; positions from
 * g with the tabulated weights W_j(s) (row ih of a substep, row 8 for the
 * step's end); the velocity at the step's end likewise; g = C^-1 b. */
static const double RSP[8][8] = ABIE_RADAU_RSP_INIT;
static const double WG[9][7] = ABIE_RADAU_WG_INIT;
static const double VG[7] = ABIE_RADAU_VG_INIT;

static void update_g_fast(double *const F[8], int ih, size_t dim, double *g[7])
{
    if (ih == 0) return;
    for (size_t i = 0; i < dim; i++) {
        double v = (F[ih][i] - F[0][i]) * RSP[ih][0];
        for (int l = 1; l < ih; l++) v = fma(-g[l - 1][i], RSP[ih][l], v);
        g[ih - 1][i] = v;
    }
}

static void predict_pos_fast(const double *y1, const double *dy1, const double *F1, int row,
                             double s, double *const g[7], size_t dim, double dt, double *y)
{
    const double ds = dt * s, hh = 0.5 * ds * ds;
    for (size_t i = 0; i < dim; i++) {
        if (row == 0) {
            y[i] = y1[i];
            continue;
        }
        double u = g[6][i] * WG[row][6];
        for (int j = 5; j >= 0; j--) u = fma(g[j][i], WG[row][j], u);
        y[i] = y1[i] + fma(hh, u, fma(ds, dy1[i], hh * F1[i]));
    }
}

static void predict_vel_end_fast(const double *dy1, const double *F1, double *const g[7],
                                 size_t dim, double dt, double *dy)
{
    for (size_t i = 0; i < dim; i++) {
        double u = g[6][i] * VG[6];
        for (int j = 5; j >= 0; j--) u = fma(g[j][i], VG[j], u);
        dy[i] = fma(dt, F1[i] + u, dy1[i]);
    }
}

static void consistent_g(double *const b[7], size_t dim, double *g[7])
{
    for (size_t i = 0; i < dim; i++)
        for (int k = 6; k >= 0; k--) {
            double v = b[k][i];
            for (int j = k + 1; j < 7; j++) v -= CS[j][k] * g[j][i];
            g[k][i] = v;
        }
}

/* :123-175.  b_k = sum_{j>=k} cs[j][k] g_j for k < ih, added left to right
 * starting from j = k (the reference writes b[0] starting with cs[0][0]*g0). */
static void update_b(double *const g[7], int ih, size_t dim, double *b[7])
{
    for (size_t i = 0; i < dim; i++) {
        for (int k = 0; k < ih; k++) {
            double s = CS[k][k] * g[k][i];
            for (int j = k + 1; j < 7; j++) s = s + CS[j][k] * g[j][i];
            b[k][i] = s;
        }
    }
}

/* :178-218.  The reference's 'inited' flag is never set, so bd is always 0
 * and b <- E(q) + 0. */
static void refine_b(double *b[7], double q, double *E[7], size_t dim)
{
    double q2 = q * q, q3 = q2 * q, q4 = q2 * q2, q5 = q2 * q3, q6 = q3 * q3, q7 = q2 * q5;
    for (size_t i = 0; i < dim; i++) {
        E[0][i] = q * (b[6][i] * 7.0 + b[5][i] * 6.0 + b[4][i] * 5.0 + b[3][i] * 4.0 + b[2][i] * 3.0 + b[1][i] * 2.0 + b[0][i]);
        E[1][i] = q2 * (b[6][i] * 21.0 + b[5][i] * 15.0 + b[4][i] * 10.0 + b[3][i] * 6.0 + b[2][i] * 3.0 + b[1][i]);
        E[2][i] = q3 * (b[6][i] * 35.0 + b[5][i] * 20.0 + b[4][i] * 10.0 + b[3][i] * 4.0 + b[2][i]);
        E[3][i] = q4 * (b[6][i] * 35.0 + b[5][i] * 15.0 + b[4][i] * 5.0 + b[3][i]);
        E[4][i] = q5 * (b[6][i] * 21.0 + b[5][i] * 6.0 + b[4][i]);
        E[5][i] = q6 * (b[6][i] * 7.0 + b[5][i]);
        E[6][i] = q7 * b[6][i];
    }
    for (size_t i = 0; i < dim; i++)
        for (int k = 0; k < 7; k++) b[k][i] = E[k][i] + 0.0;
}

int orc_radau15(double *pos, double *vel, const double *m, const double *r,
                size_t n, double G, double t, double t_end, orc_events *ev,
                double *t_out, orc_radau_stats *st)
{
    size_t dim = 3 * n;
    /* one slab: y0 dy0 ddy0 y dy db6 ddy | b[7] b0[7] g[7] E[7] | F[8] */
    double *slab = (double *)calloc(dim * (7 + 28 + 8) + 1, sizeof(double));
    if (!slab) return -1;
    double *y0 = slab, *dy0 = y0 + dim, *ddy0 = dy0 + dim, *y = ddy0 + dim;
    double *dy = y + dim, *db6 = dy + dim, *ddy = db6 + dim;
    double *b[7], *b0[7], *g[7], *E[7], *F[8];
    double *cur = ddy + dim;
    for (int k = 0; k < 7; k++) { b[k] = cur; cur += dim; }
    for (int k = 0; k < 7; k++) { b0[k] = cur; cur += dim; }
    for (int k = 0; k < 7; k++) { g[k] = cur; cur += dim; }
    for (int k = 0; k < 7; k++) { E[k] = cur; cur += dim; }
    for (int k = 0; k < 8; k++) { F[k] = cur; cur += dim; }

    memcpy(y0, pos, dim * sizeof(double));
    memcpy(dy0, vel, dim * sizeof(double));
    int flag = 0;
    force_counted_v(y0, dy0, n, G, m, ddy0, st);         /* :270 */
    double h = initial_step(y0, dy0, G, m, n, st);        /* :273 */

    int running = 1, rejects_in_row = 0;
    while (running) {
        int iters = 0;
        for (int ipc = 0; ipc < 12; ipc++) {               /* :281 */
            iters++;
            for (int k = 0; k < 8; k++) memset(F[k], 0, dim * sizeof(double));
            for (int ih = 0; ih < 8; ih++) {
                if (g_orc_fast) predict_pos_fast(y0, dy0, ddy0, ih, HS[ih], g, dim, h, y);
                else predict_pos(y0, dy0, ddy0, HS[ih], b, dim, h, y);
                predict_vel(dy0, ddy0, HS[ih], b, dim, h, dy);
                force_counted_v(y, dy, n, G, m, F[ih], st);
                if (g_orc_fast) update_g_fast(F, ih, dim, g);
                else update_g(F, ih, dim, g);
                update_b(g, ih, dim, b);
            }
            for (size_t i = 0; i < dim; i++) db6[i] = b[6][i] - b0[6][i];
            if (max_abs(db6, dim) / max_abs(F[7], dim) < TOLPC) break; /* :300 */
            for (int k = 0; k < 7; k++) memcpy(b0[k], b[k], dim * sizeof(double));
        }
        if (st) {
            st->iterations += iters;
            st->attempts++;
            st->iter_hist[iters]++;
        }
        if (g_orc_fast) {
            predict_pos_fast(y0, dy0, ddy0, 8, 1., g, dim, h, y);
            predict_vel_end_fast(dy0, ddy0, g, dim, h, dy);
        } else {
            predict_pos(y0, dy0, ddy0, 1., b, dim, h, y);    /* :309 */
            predict_vel(dy0, ddy0, 1., b, dim, h, dy);
        }
        force_counted_v(y, dy, n, G, m, ddy, st);
        double estim_b6 = max_abs(b[6], dim) / max_abs(ddy, dim);
        double err = pow(estim_b6 / EPSB, EXPONENT);
        double dtreq = h / err;
        double rq = dtreq / h;
        if (g_orc_fast) {  /* the seventh root in single precision */
            const double x = estim_b6 * (1.0 / EPSB);
            if (isfinite(x) && x >= 0) {
                const float l7 = log2f((float)x) * (1.0f / 7.0f);
                err = (double)exp2f(l7);
                rq = (double)exp2f(-l7);
                dtreq = h * rq;
            }
        }
        if (err <= 1 || rejects_in_row > 100) {             /* :320 */
            t += h;
            if (t_out) *t_out = t;
            rejects_in_row = 0;
            if (st) st->accepts++;
            if (t > t_end) {
                h = t_end - t;
                running = 0;
            }
            memcpy(y0, y, dim * sizeof(double));
            memcpy(dy0, dy, dim * sizeof(double));
            memcpy(ddy0, ddy, dim * sizeof(double));
            for (int k = 0; k < 7; k++) memcpy(b0[k], b[k], dim * sizeof(double));
            refine_b(b, g_orc_fast ? rq : dtreq / h, E, dim);
            if (g_orc_fast) consistent_g(b, dim, g);
            if (ev) flag = orc_check_events(y, r, n, t, ev);
            if (flag > 0) break;
        } else {
            rejects_in_row += 1;
            if (st) st->rejects++;
        }
        if ((g_orc_fast ? rq : dtreq / h) > 1.0 / FAC) h /= FAC;  /* :349 */
        else if (dtreq < 1.e-12) h *= FAC;
        else h = dtreq;
        if (h < H_MIN) h = H_MIN;
        if (st) st->h_last = h;
    }
    memcpy(pos, y0, dim * sizeof(double));                  /* :371-374 */
    memcpy(vel, dy, dim * sizeof(double));
    free(slab);
    return flag;
}

/* ------------------------------------------------------------------ */
/* Wisdom-Holman: src/integrator_wisdom_holman.c                        */
/* ------------------------------------------------------------------ */
static const double KEPLER_TOL = 1e-12;   /* .h:7 */
static const double TOL_ENERGY = 0.0;     /* .h:11 */
static const size_t KEPLER_MAX_IT = 500;  /* .h:12 */

/* :15-32 */
static void stumpff(double psi, double *c2, double *c3)
{
    if (psi > 1.e-10) {
        *c2 = (1.0 - cos(sqrt(psi))) / psi;
        *c3 = (sqrt(psi) - sin(sqrt(psi))) / sqrt(pow(psi, 3.0));
    } else if (psi < -1.e-6) {
        *c2 = (1 - cosh(sqrt(-psi))) / psi;
        *c3 = (sinh(sqrt(-psi)) - sqrt(-psi)) / sqrt(-pow(psi, 3.0));
    } else {
        *c2 = 0.5;
        *c3 = 1.0 / 6.0;
    }
}

/* :51-132 */
int orc_kepler(double *jpos, double *jvel, double gm, double dt, size_t id)
{
    double r0v[3], v0v[3];
    for (int c = 0; c < 3; c++) { r0v[c] = jpos[3 * id + c]; v0v[c] = jvel[3 * id + c]; }
    double r0 = norm3(r0v);
    double v0 = norm3(v0v);
    double sqrtgm = sqrt(gm);
    double xi = 0.5 * v0 * v0 - gm / r0;
    double sma = -gm / (2 * xi);
    double alpha = 1.0 / sma;
    double chi0;
    if (alpha > TOL_ENERGY) {
        chi0 = sqrtgm * dt * alpha;
    } else if (alpha < TOL_ENERGY) {
        chi0 = sgn(dt) * (sqrt(-sma) * log(-2.0 * gm * alpha * dt / (dot3(r0v, v0v) + sqrt(-gm * sma) * (1.0 - r0 * alpha))));
    } else {
        double cn = cross_norm3(r0v, v0v);
        double p = cn * cn / gm;
        double s = 0.5 * atan(1.0 / (3.0 * sqrt(gm / pow(p, 3.0)) * dt));
        double w = atan(pow(tan(s), 1.0 / 3.0));
        chi0 = sqrt(p) * 2 / tan(2 * w);
    }
    double chi = 0.0, r = 0.0, c2 = 0.0, c3 = 0.0, psi = 0.0;
    for (size_t it = 0; it < KEPLER_MAX_IT; it++) {
        psi = chi0 * chi0 * alpha;
        stumpff(psi, &c2, &c3);
        r = chi0 * chi0 * c2 + dot3(r0v, v0v) / sqrtgm * chi0 * (1.0 - psi * c3) + r0 * (1 - psi * c2);
        chi = chi0 + (sqrtgm * dt - pow(chi0, 3.0) * c3 - dot3(r0v, v0v) / sqrtgm * pow(chi0, 2.0) * c2 - r0 * chi0 * (1.0 - psi * c3)) / r;
        if (fabs(chi - chi0) < KEPLER_TOL) break;
        chi0 = chi;
    }
    int failed = fabs(chi - chi0) > KEPLER_TOL;
    double f = 1.0 - chi * chi / r0 * c2;
    double g = dt - pow(chi, 3.0) / sqrtgm * c3;
    double dg = 1.0 - chi * chi / r * c2;
    double df = sqrtgm / (r * r0) * chi * (psi * c3 - 1.0);
    for (int c = 0; c < 3; c++) {
        jpos[3 * id + c] = f * r0v[c] + g * v0v[c];
        jvel[3 * id + c] = df * r0v[c] + dg * v0v[c];
    }
    return failed;
}

/* :206-265.  auxR/auxV are running mass-weighted sums over bodies 1..i,
 * R/V = aux/eta_i. */
void orc_helio2jacobi(const double *pos, const double *vel, const double *m,
                      size_t n, double *jpos, double *jvel)
{
    double *eta = (double *)malloc(n * sizeof(double));
    eta[0] = m[0];
    for (size_t i = 1; i < n; i++) eta[i] = m[i] + eta[i - 1];
    for (int c = 0; c < 3; c++) { jpos[c] = 0.0; jvel[c] = 0.0; }
    if (n > 1) {
        for (int c = 0; c < 3; c++) { jpos[3 + c] = pos[3 + c]; jvel[3 + c] = vel[3 + c]; }
        double aR[3], aV[3], R[3], V[3];
        for (int c = 0; c < 3; c++) {
            aR[c] = m[1] * pos[3 + c];
            aV[c] = m[1] * vel[3 + c];
        }
        for (int c = 0; c < 3; c++) { R[c] = aR[c] / eta[1]; V[c] = aV[c] / eta[1]; }
        for (size_t i = 2; i < n; i++) {
            for (int c = 0; c < 3; c++) {
                jpos[3 * i + c] = pos[3 * i + c] - R[c];
                jvel[3 * i + c] = vel[3 * i + c] - V[c];
            }
            if (i < n - 1) {
                for (int c = 0; c < 3; c++) {
                    aR[c] += (m[i] * pos[3 * i + c]);
                    aV[c] += (m[i] * vel[3 * i + c]);
                }
                for (int c = 0; c < 3; c++) { R[c] = aR[c] / eta[i]; V[c] = aV[c] / eta[i]; }
            }
        }
    }
    free(eta);
}

/* :280-332.  Here R/V accumulate m_i * x_i / eta_i term by term. */
void orc_jacobi2helio(const double *jpos, const double *jvel, const double *m,
                      size_t n, double *pos, double *vel)
{
    if (n > 1)
        for (int c = 0; c < 3; c++) { pos[3 + c] = jpos[3 + c]; vel[3 + c] = jvel[3 + c]; }
    double *eta = (double *)malloc(n * sizeof(double));
    eta[0] = m[0];
    for (size_t i = 1; i < n; i++) eta[i] = m[i] + eta[i - 1];
    for (int c = 0; c < 3; c++) { pos[c] = 0.0; vel[c] = 0.0; }
    if (n > 1) {
        double R[3], V[3];
        for (int c = 0; c < 3; c++) {
            R[c] = m[1] * jpos[3 + c] / eta[1];
            V[c] = m[1] * jvel[3 + c] / eta[1];
        }
        for (size_t i = 2; i < n; i++) {
            for (int c = 0; c < 3; c++) {
                pos[3 * i + c] = jpos[3 * i + c] + R[c];
                vel[3 * i + c] = jvel[3 * i + c] + V[c];
            }
            if (i < n - 1) {
                for (int c = 0; c < 3; c++) {
                    R[c] += m[i] * jpos[3 * i + c] / eta[i];
                    V[c] += m[i] * jvel[3 * i + c] / eta[i];
                }
            }
        }
    }
    free(eta);
}

/* :349-436.  With sparse != 0 the pairwise loop (:415-428) visits only pairs
 * whose other member has nonzero mass; a zero-mass partner adds an exact
 * zero to the reference's sums, so the massive-partner terms and their order
 * are unchanged. */
void orc_wh_accel(const double *pos, const double *jpos, const double *m,
                  size_t n, double G, double *accel, int sparse)
{
    double *ir3h = (double *)calloc(n, sizeof(double));
    double *ir3j = (double *)calloc(n, sizeof(double));
    double *a3 = (double *)calloc(3 * n, sizeof(double));
    double *a2 = (double *)calloc(3 * n, sizeof(double));
    for (size_t i = 2; i < n; i++) {
        double ih = 1.0 / norm3(&pos[3 * i]);
        ir3h[i] = pow(ih, 3.0);
        double ij = 1.0 / norm3(&jpos[3 * i]);
        ir3j[i] = pow(ij, 3.0);
    }
    double ind[3] = {0.0, 0.0, 0.0};
    for (size_t i = 2; i < n; i++)
        for (int c = 0; c < 3; c++) ind[c] -= G * m[i] * pos[3 * i + c] * ir3h[i];
    double etai = m[0];
    for (size_t i = 2; i < n; i++) {
        etai += m[i - 1];
        for (int c = 0; c < 3; c++)
            a2[3 * i + c] = a2[3 * (i - 1) + c] + G * m[i] * m[0] * ir3j[i] / etai * jpos[3 * i + c];
    }
    if (!sparse) {
        for (size_t i = 1; i + 1 < n; i++) {
            for (size_t j = i + 1; j < n; j++) {
                double d[3];
                for (int c = 0; c < 3; c++) d[c] = pos[3 * j + c] - pos[3 * i + c];
                double aux = 1.0 / pow(norm3(d), 3.0);
                for (int c = 0; c < 3; c++) a3[3 * j + c] -= G * m[i] * aux * d[c];
                for (int c = 0; c < 3; c++) a3[3 * i + c] += G * m[j] * aux * d[c];
            }
        }
    } else {
        /* body j collects: first the i<j terms (ascending i), then the
         * j'>j terms (ascending j'), which is the order the full double loop
         * adds them in. */
        size_t nm = 0;
        size_t *mi = (size_t *)malloc(n * sizeof(size_t));
        for (size_t i = 1; i < n; i++) if (m[i] != 0.0) mi[nm++] = i;
        for (size_t j = 1; j < n; j++) {
            for (size_t q = 0; q < nm; q++) {
                size_t i = mi[q];
                if (i >= j) break;
                double d[3];
                for (int c = 0; c < 3; c++) d[c] = pos[3 * j + c] - pos[3 * i + c];
                double aux = 1.0 / pow(norm3(d), 3.0);
                for (int c = 0; c < 3; c++) a3[3 * j + c] -= G * m[i] * aux * d[c];
            }
            /* as the outer index: += G m_k aux d for massive k > j (the
             * partner's mass, so massless bodies collect these too) */
            for (size_t q = 0; q < nm; q++) {
                size_t k = mi[q];
                if (k <= j) continue;
                double d[3];
                for (int c = 0; c < 3; c++) d[c] = pos[3 * k + c] - pos[3 * j + c];
                double aux = 1.0 / pow(norm3(d), 3.0);
                for (int c = 0; c < 3; c++) a3[3 * j + c] += G * m[k] * aux * d[c];
            }
        }
        free(mi);
    }
    for (size_t i = 0; i < 3 * n; i++) {
        double ai = (i >= 3) ? ind[i % 3] : 0.0;
        size_t b = i / 3;
        double ac = 0.0;
        if (b >= 2)
            ac = G * m[0] * (jpos[i] * ir3j[b] - pos[i] * ir3h[b]);
        accel[i] = ai + ac + a2[i] + a3[i];
    }
    free(ir3h); free(ir3j); free(a3); free(a2);
}

/* :456-477 */
long orc_wh_step(double *pos, double *vel, double *jpos, double *jvel,
                 const double *m, size_t n, double G, double dt, double *accel,
                 int sparse)
{
    long failed = 0;
    for (size_t i = 3; i < 3 * n; i++) vel[i] += accel[i] * (dt / 2);
    orc_helio2jacobi(pos, vel, m, n, jpos, jvel);
    double eta0 = m[0];
    for (size_t i = 1; i < n; i++) {                     /* :174-191 */
        double eta = eta0 + m[i];
        double gm = G * m[0] * eta / eta0;
        failed += orc_kepler(jpos, jvel, gm, dt, i);
        eta0 = eta;
    }
    orc_jacobi2helio(jpos, jvel, m, n, pos, vel);
    orc_wh_accel(pos, jpos, m, n, G, accel, sparse);
    for (size_t i = 3; i < 3 * n; i++) vel[i] += accel[i] * (dt / 2);
    return failed;
}

/* :498-522 */
long orc_wh(double *pos, double *vel, const double *m, size_t n, double G,
            double t, double t_end, double dt, double *t_out, int sparse)
{
    double *jpos = (double *)calloc(3 * n, sizeof(double));
    double *jvel = (double *)calloc(3 * n, sizeof(double));
    double *acc = (double *)calloc(3 * n, sizeof(double));
    long failed = 0;
    orc_helio2jacobi(pos, vel, m, n, jpos, jvel);
    orc_wh_accel(pos, jpos, m, n, G, acc, sparse);
    while (t < t_end) {
        failed += orc_wh_step(pos, vel, jpos, jvel, m, n, G, dt, acc, sparse);
        t += dt;
        if (t_out) *t_out = t;
    }
    free(jpos); free(jvel); free(acc);
    return failed;
}

/* ------------------------------------------------------------------ */
/* Runge-Kutta 4: src/integrator_runge_kutta.c                          */

/* src/common.c:3-36.  Sources are the bodies with nonzero mass (negative
 * masses included, unlike ode_n_body_second_order); every body is a sink. */
void orc_first_order(const double *vec, size_t n, double G, const double *m, double *dxdt)
{
    for (size_t i = 0; i < 3 * n; i++) dxdt[i] = vec[3 * n + i];
    for (size_t j = 0; j < n; j++) {
        double x = vec[j * 3], y = vec[j * 3 + 1], z = vec[j * 3 + 2];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (size_t k = 0; k < n; k++) {
            if ((j == k) || (m[k] == 0)) continue;
            double GM = G * m[k];
            double dx = x - vec[k * 3];
            double dy = y - vec[k * 3 + 1];
            double dz = z - vec[k * 3 + 2];
            double r2 = dx * dx + dy * dy + dz * dz;
            double r3 = sqrt(r2) * r2;
            ax -= (GM * dx / r3);
            ay -= (GM * dy / r3);
            az -= (GM * dz / r3);
        }
        dxdt[(n + j) * 3] = ax;
        dxdt[(n + j) * 3 + 1] = ay;
        dxdt[(n + j) * 3 + 2] = az;
    }
}

/* src/integrator_runge_kutta.c:6-50 */
void orc_rk(double *pos, double *vel, const double *m, size_t n, double G, double t,
            double t_end, double dt, double *t_out)
{
    size_t d = 6 * n;
    double *k1 = (double *)malloc(d * sizeof(double));
    double *k2 = (double *)malloc(d * sizeof(double));
    double *k3 = (double *)malloc(d * sizeof(double));
    double *k4 = (double *)malloc(d * sizeof(double));
    double *tmp = (double *)malloc(d * sizeof(double));
    double *vec = (double *)malloc(d * sizeof(double));
    for (size_t i = 0; i < 3 * n; i++) vec[i] = pos[i];
    for (size_t i = 3 * n; i < d; i++) vec[i] = vel[i - 3 * n];
    while (t < t_end) {
        orc_first_order(vec, n, G, m, k1);
        for (size_t i = 0; i < d; i++) tmp[i] = vec[i] + 0.5 * dt * k1[i];
        orc_first_order(tmp, n, G, m, k2);
        for (size_t i = 0; i < d; i++) tmp[i] = vec[i] + 0.5 * dt * k2[i];
        orc_first_order(tmp, n, G, m, k3);
        for (size_t i = 0; i < d; i++) tmp[i] = vec[i] + dt * k3[i];
        orc_first_order(tmp, n, G, m, k4);
        for (size_t i = 0; i < d; i++) vec[i] += (dt * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]) / 6.0);
        t += dt;
    }
    if (t_out) *t_out = t;
    for (size_t i = 0; i < 3 * n; i++) pos[i] = vec[i];
    for (size_t i = 3 * n; i < d; i++) vel[i - 3 * n] = vec[i];
    free(k1); free(k2); free(k3); free(k4); free(tmp); free(vec);
}
