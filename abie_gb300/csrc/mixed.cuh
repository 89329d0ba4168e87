// Mixed-precision all-pairs force (FP32 pair terms on anchored coordinates,
// compensated accumulation; heavy sources in FP64).
#pragma once
#include "force.cuh"

namespace abie {

int launch_force_mixed(const double *pos, const double *m, int n, double G, ForceScratch &s,
                       double *acc, cudaStream_t st);
// The same on a compacted source list already on the device (src, its
// count *n_src), as the stepped Radau15 engine publishes it.
int launch_force_mixed_src(const double *pos, const double *m, int n, const Src *src,
                           const int *n_src, ForceScratch &s, double *acc, cudaStream_t st);

// Sources whose G m is at least this fraction of the largest G m are summed
// in FP64; the rest in FP32.
void mixed_set_heavy_fraction(double f);
double mixed_heavy_fraction();

}  // namespace abie
