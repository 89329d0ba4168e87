// Batched Radau15 ensemble (ensemble.cu) and the learned predictor hook.
#pragma once
#include "abi_state.cuh"

namespace abie {

// Learned b-coefficient predictor (mlp.cu); null when none is loaded.
struct LearnedPredictor;
const LearnedPredictor *learned_predictor_current();

// Device store that the ensemble appends training samples to.
struct EnsembleLearnIO {
    float *samples;
    long long cap;
    unsigned long long *count;  // device counter
    float tau[7];
};
int mlp_collect_begin(EnsembleLearnIO *io);
void mlp_collect_end(EnsembleLearnIO *io);

struct EnsembleStats {
    long long attempts, iterations, force_calls, steps, launches, fallbacks;
};

int ensemble_run(double *pos, double *vel, const double *m, const long long *offsets, int ns,
                 double G, double t0, double t_end, double *t_out, int *status, long long *steps,
                 int mode, const LearnedPredictor *mlp, cudaStream_t st, EnsembleStats *stats,
                 const EnsembleLearnIO *learn_io, bool consistent_g, const float *mlp_tau);
// The plain FP64 form's kernel for groups of w warps (ensemble_plain.cu).
const void *ensemble_plain_fn(int w);
// Host copy of the output scales of the enabled learned predictor.
const float *learned_predictor_tau();
double ensemble_last_seconds();

}  // namespace abie
