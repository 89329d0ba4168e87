// Classical Runge-Kutta 4 on the device (src/integrator_runge_kutta.c:6-50).
//
// The reference integrates the first-order state vec = (pos, vel) with
// four evaluations of ode_n_body_first_order per step (src/common.c:3-36),
// while t < t_end in fixed steps of dt.  Here the state and the four slopes
// stay in GPU memory; each slope is the velocity half of its stage state
// (a copy) and the library's force kernel on its position half, in the
// current force form.  The stage and update arithmetic repeats the
// reference's expressions in its order (this file is built with
// --fmad=false), so with the exact force form a step reproduces the
// reference's doubles for bodies of non-negative mass.  (The reference's
// first-order force also lets negative masses act as sources and computes
// their sinks; the library's force skips both, as ode_n_body_second_order
// does: such "deleted" bodies keep a zero acceleration here.)
//
// One step is captured once as a CUDA graph and replayed.
#include <algorithm>

#include "abi_state.cuh"
#include "engine.cuh"
#include "force.cuh"

namespace abie {

// tmp = vec + c * k over the 6N entries (c = 0.5 * dt or dt, as the
// reference writes it).
__global__ void rk_stage_kernel(const double *vec, const double *k, double c, double *tmp,
                                long long d6)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d6;
         i += (long long)gridDim.x * blockDim.x)
        tmp[i] = vec[i] + c * k[i];
}

// vec += (dt * (k1 + 2 k2 + 2 k3 + k4) / 6.0), in the reference's order.
__global__ void rk_update_kernel(double *vec, const double *k1, const double *k2, const double *k3,
                                 const double *k4, double dt, long long d6)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d6;
         i += (long long)gridDim.x * blockDim.x)
        vec[i] += (dt * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]) / 6.0);
}

struct RkBuffers {
    double *slab = nullptr;  // vec, tmp, k1..k4: 6 x 6N
    size_t cap = 0;          // bodies
};
static RkBuffers g_rk;

void free_rk_buffers()
{
    if (g_rk.slab) cudaFree(g_rk.slab);
    g_rk = RkBuffers();
}

// Slope of a stage state s (6N): velocities, then accelerations.
static int rk_slope(int mode, const double *s, const double *m, int n, double G, double *k,
                    cudaStream_t st)
{
    const size_t d3 = 3 * (size_t)n;
    ABIE_CUDA(cudaMemcpyAsync(k, s + d3, d3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaMemsetAsync(k + d3, 0, d3 * sizeof(double), st));
    return launch_force(mode, s, m, n, G, g_sim.fs, k + d3, st);
}

static int rk_step(int mode, const double *m, int n, double G, double dt, cudaStream_t st)
{
    const size_t d6 = 6 * (size_t)n;
    double *vec = g_rk.slab, *tmp = vec + d6, *k1 = tmp + d6, *k2 = k1 + d6, *k3 = k2 + d6,
           *k4 = k3 + d6;
    const int threads = 256;
    const int blocks = (int)std::min<long long>(((long long)d6 + threads - 1) / threads,
                                                (long long)g_sim.num_sms * 8);
    int rc;
    if ((rc = rk_slope(mode, vec, m, n, G, k1, st))) return rc;
    rk_stage_kernel<<<blocks, threads, 0, st>>>(vec, k1, 0.5 * dt, tmp, (long long)d6);
    if ((rc = rk_slope(mode, tmp, m, n, G, k2, st))) return rc;
    rk_stage_kernel<<<blocks, threads, 0, st>>>(vec, k2, 0.5 * dt, tmp, (long long)d6);
    if ((rc = rk_slope(mode, tmp, m, n, G, k3, st))) return rc;
    rk_stage_kernel<<<blocks, threads, 0, st>>>(vec, k3, dt, tmp, (long long)d6);
    if ((rc = rk_slope(mode, tmp, m, n, G, k4, st))) return rc;
    rk_update_kernel<<<blocks, threads, 0, st>>>(vec, k1, k2, k3, k4, dt, (long long)d6);
    ABIE_CUDA(cudaGetLastError());
    return 0;
}

// RK4 on device arrays pos/vel (3N each), updated in place.  Returns the
// accumulated time in *t_out.
int rk_run(double *pos, double *vel, const double *m, int n, double G, double t, double t_end,
           double dt, double *t_out, cudaStream_t st)
{
    *t_out = t;
    if (n <= 0) return 0;
    int mode = g_sim.force_mode;
    const size_t d3 = 3 * (size_t)n, d6 = 2 * d3;
    if ((size_t)n > g_rk.cap) {
        if (g_rk.slab) cudaFree(g_rk.slab);
        g_rk.slab = nullptr;
        ABIE_CUDA(cudaMalloc(&g_rk.slab, 6 * d6 * sizeof(double)));
        g_rk.cap = (size_t)n;
    }
    double *vec = g_rk.slab;
    ABIE_CUDA(cudaMemcpyAsync(vec, pos, d3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(vec + d3, vel, d3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    long long steps = 0;
    double tt = t;
    while (tt < t_end) {  // the reference's accumulation of t
        tt += dt;
        steps++;
    }
    int rc = 0;
    if (steps > 0) {
        // the first step runs directly (it sizes the force scratch); the
        // rest replay a captured step
        rc = rk_step(mode, m, n, G, dt, st);
        if (rc) return rc;
        if (steps > 1) {
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            ABIE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            rc = rk_step(mode, m, n, G, dt, st);
            cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            ABIE_CUDA(ce);
            ABIE_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            for (long long k = 1; k < steps; k++) ABIE_CUDA(cudaGraphLaunch(exec, st));
            cudaGraphExecDestroy(exec);
            cudaGraphDestroy(graph);
        }
        g_sim.ctr.force_calls += 4 * steps;
    }
    ABIE_CUDA(cudaMemcpyAsync(pos, vec, d3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(vel, vec + d3, d3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaStreamSynchronize(st));
    *t_out = tt;
    return 0;
}

}  // namespace abie

using namespace abie;

extern "C" {

// src/common.c:405-408.  Like the reference, leaves the model time alone.
int integrator_rk(double t, double t_end, double dt)
{
    Sim &s = g_sim;
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "integrator_rk before initialize_code");
        return ABIE_ERR_NOT_INITIALIZED;
    }
    double t_out = t;
    return rk_run(s.pos, s.vel, s.m, (int)s.n, s.G, t, t_end, dt, &t_out, s.st);
}

// src/integrator_runge_kutta.c:52-60 on caller arrays.
void integrator_runge_kutta(double *pos, double *vel, double *m_vec, double *r_vec, size_t N,
                            double G, double t, double t_end, double dt)
{
    (void)r_vec;
    if (ensure_device(-1)) return;
    N &= 0xffffffffull;
    double *dp = nullptr, *dv = nullptr, *dm = nullptr;
    size_t cp = 0, cv = 0, cm = 0;
    if (reserve(&dp, &cp, 3 * N) || reserve(&dv, &cv, 3 * N) || reserve(&dm, &cm, N)) return;
    cudaMemcpy(dp, pos, 3 * N * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dv, vel, 3 * N * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dm, m_vec, N * 8, cudaMemcpyHostToDevice);
    double t_out = t;
    if (rk_run(dp, dv, dm, (int)N, G, t, t_end, dt, &t_out, g_sim.st) == 0) {
        cudaMemcpy(pos, dp, 3 * N * 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(vel, dv, 3 * N * 8, cudaMemcpyDeviceToHost);
    }
    cudaFree(dp);
    cudaFree(dv);
    cudaFree(dm);
}

}  // extern "C"
