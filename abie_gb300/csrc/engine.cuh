// Device-resident integrators: Gauss-Radau 15 (radau.cu) and Wisdom-Holman
// (wh.cu) on one system, and the batched Radau15 ensemble (ensemble.cu).
#pragma once
#include "abi_state.cuh"

namespace abie {

// One system in device memory.  pos/vel are read at the start and
// overwritten with the final state.  h_m / h_r are host copies of the
// masses and radii (used to build the source list and event thresholds).
struct SystemView {
    double *pos, *vel;
    const double *m, *r, *ext;  // device; ext may be null
    const double *h_m, *h_r;    // host
    int n;
    double G;
};

// Event configuration and ring buffers (host side, updated in place).
struct EventState {
    double ce_dist;
    size_t max_ce, max_coll;
    size_t *n_ce, *n_coll;
    std::vector<double> *buf_ce, *buf_coll;
};

// Radau15 from t to the first accepted time past t_end.  Returns 0/1/2 (the
// reference's event codes) or a negative ABIE_ERR_*; *t_out gets the final
// time.
int radau_run(const SystemView &sys, double t, double t_end, int mode, EventState *ev,
              double *t_out, abie_counters *ctr, cudaStream_t st);

// Wisdom-Holman (wh.cu) from t while t < t_end in steps of dt on a
// heliocentric state; *t_out gets the accumulated time.
int wh_run(const SystemView &sys, double t, double t_end, double dt, double *t_out,
           abie_counters *ctr, cudaStream_t st);
void free_wh_buffers();

// Runge-Kutta 4 (rk.cu) on device arrays, in the current force form.
int rk_run(double *pos, double *vel, const double *m, int n, double G, double t, double t_end,
           double dt, double *t_out, cudaStream_t st);
void free_rk_buffers();

}  // namespace abie
