/*
 * CPU oracle for ABIE's gravity hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C99 restatement of the reference algorithms, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * Nothing in the product library links or calls it.  Each function cites the
 * reference file:line it follows.  Parity of this restatement with the
 * reference is pinned bit for bit by tests/test_oracle.py (against the
 * reference library built by oracle/build_ref.sh, and against the committed
 * vectors in tests/golden/).
 */
#ifndef ABIE_ORACLE_H
#define ABIE_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Event ring buffers: src/common.h:49-64, src/common.c:116-158. */
typedef struct {
    double ce_dist;
    size_t max_ce, max_coll;
    size_t n_ce, n_coll;
    double *buf_ce;   /* 4*max_ce doubles or NULL */
    double *buf_coll; /* 4*max_coll doubles or NULL */
} orc_events;

typedef struct {
    long force_calls;
    long iterations;   /* corrector iterations, summed over attempts */
    long attempts;     /* step attempts (accepted + rejected) */
    long accepts;
    long rejects;
    long iter_hist[13];
    double h_last;
} orc_radau_stats;

/* src/common.c:39-77: a_j for sinks j in [j0, j1). */
void orc_force(const double *pos, size_t n, double G, const double *m,
               double *acc, size_t j0, size_t j1);
/* The same arithmetic per sink, sinks split over nthreads POSIX threads. */
int orc_force_threads(const double *pos, size_t n, double G, const double *m,
                      double *acc, size_t j0, size_t j1, int nthreads);
/* src/common.c:340-357 */
double orc_energy(const double *pos, const double *vel, const double *m,
                  size_t n, double G);
/* src/common.c:116-158 */
int orc_check_events(const double *pos, const double *r, size_t n, double t,
                     orc_events *ev);
/* src/integrator_gauss_radau15.c:221-380 (with :9-218). Returns 0/1/2. */
int orc_radau15(double *pos, double *vel, const double *m, const double *r,
                size_t n, double G, double t, double t_end, orc_events *ev,
                double *t_out, orc_radau_stats *st);
/* src/integrator_wisdom_holman.c:498-522.  sparse=0 follows the reference's
 * O(N^2) compute_accel; sparse=1 skips zero-mass partners (same sums, same
 * order, for the massive terms).  Returns the number of failed Kepler solves. */
long orc_wh(double *pos, double *vel, const double *m, size_t n, double G,
            double t, double t_end, double dt, double *t_out, int sparse);
/* One WH step on an already heliocentric state, accel in/out (3n). */
long orc_wh_step(double *pos, double *vel, double *jpos, double *jvel,
                 const double *m, size_t n, double G, double dt, double *accel,
                 int sparse);
/* src/integrator_wisdom_holman.c:349-436 */
void orc_wh_accel(const double *pos, const double *jpos, const double *m,
                  size_t n, double G, double *accel, int sparse);
/* src/integrator_wisdom_holman.c:206-265 and :280-332 */
void orc_helio2jacobi(const double *pos, const double *vel, const double *m,
                      size_t n, double *jpos, double *jvel);
void orc_jacobi2helio(const double *jpos, const double *jvel, const double *m,
                      size_t n, double *pos, double *vel);
/* src/integrator_wisdom_holman.c:51-132; returns 1 when not converged. */
int orc_kepler(double *jpos, double *jvel, double gm, double dt, size_t id);
/* src/additional_forces.c:14-121: adds the post-Newtonian pair terms to acc. */
void orc_post_newtonian(const double *pos, const double *vel, size_t n, double G, double C,
                        const double *m, double *acc);
/* Speed of light used by orc_radau15's accelerations (0: Newtonian only). */
void orc_set_pn(double C);
/* 1: orc_radau15 with the GPU fast form's arithmetic (FMA pair sums, the
 * expanded g recurrence, positions predicted from g, a single-precision
 * step-size root, g consistent with each step's guess), for the
 * long-horizon accuracy study; 0 (default): the reference's operations. */
void orc_set_fastform(int on);
/* External accelerations (3N doubles, kept by pointer; NULL: none) added to
 * every force call of orc_radau15 (src/common.c:107-112). */
void orc_set_ext(const double *ext);
/* src/common.c:3-36: derivative of the first-order state vec = (pos, vel). */
void orc_first_order(const double *vec, size_t n, double G, const double *m, double *dxdt);
/* src/integrator_runge_kutta.c:6-50: classical RK4 from t while t < t_end
 * in steps of dt; pos/vel updated in place, *t_out the accumulated time. */
void orc_rk(double *pos, double *vel, const double *m, size_t n, double G, double t,
            double t_end, double dt, double *t_out);

#ifdef __cplusplus
}
#endif
#endif
