// Gauss-Radau 15 on the device (placeholder until the engine lands).
#include "abi_state.cuh"

namespace abie {
void free_engine_buffers() {}
}  // namespace abie

extern "C" {
int integrator_gr(double t, double t_end, double dt)
{
    (void)t; (void)t_end; (void)dt;
    abie::set_error(ABIE_ERR_UNSUPPORTED, "integrator_gr: engine not built yet");
    return ABIE_ERR_UNSUPPORTED;
}
size_t integrator_gauss_radau15(double *pos, double *vel, double *m_vec, double *r_vec, size_t N,
                                double G, double t, double t_end, double dt)
{
    (void)pos; (void)vel; (void)m_vec; (void)r_vec; (void)N; (void)G; (void)t; (void)t_end; (void)dt;
    return (size_t)(long long)ABIE_ERR_UNSUPPORTED;
}
int integrator_wh(double t, double t_end, double dt)
{
    (void)t; (void)t_end; (void)dt;
    return ABIE_ERR_UNSUPPORTED;
}
void integrator_wisdom_holman(double *pos, double *vel, double *m_vec, double *r_vec, size_t N,
                              double G, double t, double t_end, double dt)
{
    (void)pos; (void)vel; (void)m_vec; (void)r_vec; (void)N; (void)G; (void)t; (void)t_end; (void)dt;
}
int abie_gr_ensemble(double *pos, double *vel, const double *m, const long long *offsets,
                     int n_systems, double G, double t0, double t_end, double *t_out, int *status,
                     long long *steps, int flags)
{
    (void)pos; (void)vel; (void)m; (void)offsets; (void)n_systems; (void)G; (void)t0; (void)t_end;
    (void)t_out; (void)status; (void)steps; (void)flags;
    return ABIE_ERR_UNSUPPORTED;
}
double abie_last_ensemble_seconds(void) { return 0.0; }
}
