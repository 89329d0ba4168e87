// Mixed-precision all-pairs force -- see mixed.cuh.
#include "mixed.cuh"

namespace abie {

static double g_heavy_fraction = 1e-6;

void mixed_set_heavy_fraction(double f) { g_heavy_fraction = f; }
double mixed_heavy_fraction() { return g_heavy_fraction; }

int launch_force_mixed(const double *pos, const double *m, int n, double G, ForceScratch &s,
                       double *acc, cudaStream_t st)
{
    (void)pos; (void)m; (void)n; (void)G; (void)s; (void)acc; (void)st;
    set_error(ABIE_ERR_UNSUPPORTED, "mixed-precision force not built yet");
    return ABIE_ERR_UNSUPPORTED;
}

}  // namespace abie
