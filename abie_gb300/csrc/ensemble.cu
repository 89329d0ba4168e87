// Batched Gauss-Radau 15 over many independent small systems.
//
// A group of threads integrates one system (at most 21 bodies) from a work
// queue -- one warp for up to 10 bodies, two warps (a named barrier each)
// for 11-21, four warps for the slowest quarter of the systems, each class a
// kernel on its own stream -- and a finished group takes the next system,
// so systems of uneven size and difficulty do not wait for each other.  Each thread owns
// one of the system's 3N components and keeps its Radau state (y0, dy0,
// F1, b[7], g[7], previous b6) in registers.  For the force, the predicted
// positions go to shared memory and the pairs spread over the lanes: each
// warp takes ceil(N / warps) sinks with L = 32 / that lanes per sink, each
// summing every L-th source, partial sums added as a fixed tree (L = 1 and
// the reference's operations in the exact form).  The
// sweep itself -- predictor, g/b updates, convergence test, step control,
// refine_bs -- is the reference's (src/integrator_gauss_radau15.c:221-380)
// component by component, as in the single-system engine.  The fast form
// runs the corrector on the Newton-form coefficients g alone: predicted
// positions come straight from g with tabulated weights, b = C g is formed
// once per accepted step for refine_bs, and the next step starts from g
// consistent with the refined guess.  Far fewer FP64 instructions per
// substep (on this GPU each FP64 warp instruction holds the SM
// sub-partition's FP64 pipe for ~64 cycles whatever the number of active
// lanes, so the instruction count sets the time per substep), the same
// converged solution, and fewer corrector iterations.  The maxima behind
// the convergence test and the step control are integer maxima of the
// values' bit patterns, and the fast form's step-size root is taken in
// single precision (radau_comp.cuh, step_size).
//
// Systems start longest first (shortest two-body time scale first), since
// a batch lasts at least as long as its slowest system.
//
// Launches are bounded in time: a warp that has run past the launch's time
// budget saves its system's state and leaves; the host launches again over
// the systems not yet done.
#include <algorithm>
#include <vector>

#include "ensemble_kernel.cuh"

namespace abie {

static double g_last_seconds = 0.0;
// The slowest 1 in heavy_div systems (longest first) run on four warps.  On
// 4,096 planetary systems over 1 yr in the fast form the batch took 81-84
// ms with 1 in 256, 79-80 with 1 in 16, 76 with 1 in 8, 70-72 with 1 in 4,
// 85 with 1 in 2 and 78 with all: a batch ends with its slow systems, and a
// four-warp group cuts their per-step latency at the cost of more warps per
// system.  The exact form, whose group force does not split a pair's work,
// keeps 1 in 256 (with 1 in 4 its batch ran 76k system-steps/s against
// 100k).  abie_debug_ensemble_heavy sets one share for both.
static int g_heavy_div = 0;
static int heavy_div(int mode) { return g_heavy_div > 0 ? g_heavy_div : (mode == ABIE_FORCE_EXACT ? 256 : 4); }
// (The plain FP64 form splits each sink's sources over the lanes, like the
// fast form's groups, so it takes the fast forms' share.)

template <int MODE, bool LEARN>
static const void *ensemble_fn_l(int w)
{
    return w == 1 ? (const void *)ensemble_kernel<MODE, 1, LEARN>
                  : (w == 2 ? (const void *)ensemble_kernel<MODE, 2, LEARN>
                            : (const void *)ensemble_kernel<MODE, 4, LEARN>);
}

// The kernel for a force form, warps per system and whether the learned
// predictor (or sample collection) is in use: without it the variant leaves
// the predictor's code out.
static const void *ensemble_fn(int mode, int w, bool learn)
{
    switch (mode) {
    case ABIE_FORCE_EXACT:
        return learn ? ensemble_fn_l<ABIE_FORCE_EXACT, true>(w) : ensemble_fn_l<ABIE_FORCE_EXACT, false>(w);
    case ABIE_FORCE_MIXED:
        return learn ? ensemble_fn_l<ABIE_FORCE_MIXED, true>(w) : ensemble_fn_l<ABIE_FORCE_MIXED, false>(w);
    case ABIE_FORCE_NAIVE:
        return learn ? nullptr : ensemble_plain_fn(w);
    default:
        return learn ? ensemble_fn_l<ABIE_FORCE_FP64, true>(w) : ensemble_fn_l<ABIE_FORCE_FP64, false>(w);
    }
}

static size_t learn_smem(int w) { return (size_t)(WARPS / w) * sizeof(LearnSmem); }

static int launch_ensemble(int mode, int w, int blocks, const EnsArgs &a, cudaStream_t st)
{
    const bool learn = a.mlp || a.samples;
    size_t dyn = learn ? learn_smem(w) : 0;
    void *args[] = {const_cast<EnsArgs *>(&a)};
    ABIE_CUDA(cudaLaunchKernel(ensemble_fn(mode, w, learn), dim3(blocks), dim3(32 * WARPS), args, dyn, st));
    return 0;
}

static cudaStream_t g_ens_stream[2] = {nullptr, nullptr};  // besides the caller's stream

int ensemble_run(double *pos, double *vel, const double *m, const long long *offsets, int ns,
                 double G, double t0, double t_end, double *t_out, int *status, long long *steps,
                 int mode, const LearnedPredictor *mlp, cudaStream_t st, EnsembleStats *stats,
                 const EnsembleLearnIO *learn_io, bool consistent, const float *mlp_tau)
{
    if (ns <= 0) return 0;
    long long total = offsets[ns];
    for (int s = 0; s < ns; s++) {
        long long k = offsets[s + 1] - offsets[s];
        if (k < 1 || k > ENS_MAX_BODIES) {
            set_error(ABIE_ERR_ARGUMENT, "ensemble system %d has %lld bodies (1..%d supported)", s,
                      k, ENS_MAX_BODIES);
            return ABIE_ERR_ARGUMENT;
        }
    }
    const bool learning_req = mlp || (learn_io && learn_io->samples);
    if (mode == ABIE_FORCE_NAIVE && learning_req) {
        set_error(ABIE_ERR_UNSUPPORTED,
                  "abie_gr_ensemble: the plain FP64 form runs the reference's predictor only "
                  "(no learned predictor, no sample collection)");
        return ABIE_ERR_UNSUPPORTED;
    }
    double *d_pos, *d_vel, *d_m, *d_state;
    long long *d_off;
    EnsScalars *d_sc;
    int *d_active, *d_queue;
    ABIE_CUDA(cudaMalloc(&d_pos, 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_vel, 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_m, total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_state, (size_t)STATE_PER_COMP * 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&d_off, (ns + 1) * sizeof(long long)));
    ABIE_CUDA(cudaMalloc(&d_sc, ns * sizeof(EnsScalars)));
    ABIE_CUDA(cudaMalloc(&d_active, ns * sizeof(int)));
    ABIE_CUDA(cudaMalloc(&d_queue, 3 * sizeof(int)));
    std::vector<EnsScalars> sc(ns);
    for (int s = 0; s < ns; s++) {
        memset(&sc[s], 0, sizeof(EnsScalars));
        sc[s].t = t0;
    }
    // Longest-first order: a system's step count follows its shortest
    // two-body time scale sqrt(r_ij^3 / G(m_i + m_j)), and the batch takes
    // at least as long as its slowest system, so those start first.
    std::vector<double> rate(ns, 0.0);
    {
        std::vector<double> hp(3 * (size_t)total), hm(m, m + total);
        memcpy(hp.data(), pos, 3 * total * sizeof(double));
        for (int s = 0; s < ns; s++) {
            double best = 0.0;
            for (long long i = offsets[s]; i < offsets[s + 1]; i++)
                for (long long j = i + 1; j < offsets[s + 1]; j++) {
                    double mu = G * (std::max(hm[i], 0.0) + std::max(hm[j], 0.0));
                    double dx = hp[3 * i] - hp[3 * j], dy = hp[3 * i + 1] - hp[3 * j + 1],
                           dz = hp[3 * i + 2] - hp[3 * j + 2];
                    double r2 = dx * dx + dy * dy + dz * dz;
                    if (mu > 0.0 && r2 > 0.0) best = std::max(best, sqrt(mu / (r2 * sqrt(r2))));
                }
            rate[s] = best;
        }
    }
    std::vector<int> active(ns);
    for (int s = 0; s < ns; s++) active[s] = s;
    std::stable_sort(active.begin(), active.end(), [&](int x, int y) { return rate[x] > rate[y]; });
    ABIE_CUDA(cudaMemcpyAsync(d_pos, pos, 3 * total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_vel, vel, 3 * total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_m, m, total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_off, offsets, (ns + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(d_sc, sc.data(), ns * sizeof(EnsScalars), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaStreamSynchronize(st));

    const bool learning = mlp || (learn_io && learn_io->samples);
    // three classes of system: up to 10 bodies on one warp, 11-21 on two,
    // and the slowest few (longest-first order) on four warps, which cuts
    // their per-substep latency -- the batch ends with its slowest system
    const int WC[3] = {1, 2, 4};
    int bps[3] = {1, 1, 1};
    for (int k = 0; k < 3; k++) {
        const void *fn = ensemble_fn(mode, WC[k], learning);
        const size_t dyn = learning ? learn_smem(WC[k]) : 0;
        if (learning)
            ABIE_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[k], fn, 32 * WARPS, dyn));
        bps[k] = std::max(bps[k], 1);
    }
    std::vector<unsigned char> cls(ns);
    {
        const int heavy = std::min(ns, std::max(1, ns / heavy_div(mode)));
        for (int q = 0; q < ns; q++) {
            const int s2 = active[q];
            cls[s2] = q < heavy ? 2 : (3 * (offsets[s2 + 1] - offsets[s2]) <= 32 ? 0 : 1);
        }
    }
    for (int k = 0; k < 2; k++)
        if (!g_ens_stream[k]) ABIE_CUDA(cudaStreamCreateWithFlags(&g_ens_stream[k], cudaStreamNonBlocking));
    cudaEvent_t e0, e1, ej;
    ABIE_CUDA(cudaEventCreate(&e0));
    ABIE_CUDA(cudaEventCreate(&e1));
    ABIE_CUDA(cudaEventCreateWithFlags(&ej, cudaEventDisableTiming));
    double gpu_ms = 0.0;
    int launches = 0;
    int n_active = ns;
    std::vector<int> part(ns);
    while (n_active > 0) {
        // the classes' lists, each in longest-first order
        int first[4] = {0, 0, 0, 0};
        {
            int k2 = 0;
            for (int c = 0; c < 3; c++) {
                first[c] = k2;
                for (int q = 0; q < n_active; q++)
                    if (cls[active[q]] == c) part[k2++] = active[q];
            }
            first[3] = k2;
        }
        ABIE_CUDA(cudaMemcpyAsync(d_active, part.data(), n_active * sizeof(int),
                                  cudaMemcpyHostToDevice, st));
        ABIE_CUDA(cudaMemsetAsync(d_queue, 0, 3 * sizeof(int), st));
        EnsArgs a;
        a.offsets = d_off;
        a.m = d_m;
        a.pos = d_pos;
        a.vel = d_vel;
        a.state = d_state;
        a.sc = d_sc;
        a.G = G;
        a.t_end = t_end;
        a.mlp = mlp;
        a.samples = learn_io ? learn_io->samples : nullptr;
        a.sample_cap = learn_io ? learn_io->cap : 0;
        a.sample_count = learn_io ? learn_io->count : nullptr;
        for (int k = 0; k < 7; k++) a.tau[k] = learn_io ? learn_io->tau[k] : (mlp_tau ? mlp_tau[k] : 1.0f);
        a.consistent_g = consistent ? 1 : 0;
        a.budget_ns = 2000000000ull;  // each launch yields after about two seconds
        ABIE_CUDA(cudaEventRecord(e0, st));
        ABIE_CUDA(cudaEventRecord(ej, st));
        for (int k = 0; k < 2; k++) ABIE_CUDA(cudaStreamWaitEvent(g_ens_stream[k], ej, 0));
        for (int k = 0; k < 3; k++) {
            const int cnt = first[k + 1] - first[k];
            if (cnt == 0) continue;
            EnsArgs ak = a;
            ak.active = d_active + first[k];
            ak.n_active = cnt;
            ak.queue = d_queue + k;
            const int per_block = WARPS / WC[k];  // systems per block
            int blocks = (int)std::min<long long>((long long)bps[k] * g_sim.num_sms,
                                                  (cnt + per_block - 1) / per_block);
            blocks = std::max(blocks, 1);
            int lrc = launch_ensemble(mode, WC[k], blocks, ak, k == 0 ? st : g_ens_stream[k - 1]);
            if (lrc) return lrc;
        }
        for (int k = 0; k < 2; k++) {
            ABIE_CUDA(cudaEventRecord(ej, g_ens_stream[k]));
            ABIE_CUDA(cudaStreamWaitEvent(st, ej, 0));
        }
        ABIE_CUDA(cudaEventRecord(e1, st));
        ABIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        gpu_ms += ms;
        launches++;
        ABIE_CUDA(cudaMemcpy(sc.data(), d_sc, ns * sizeof(EnsScalars), cudaMemcpyDeviceToHost));
        int k = 0;
        for (int q = 0; q < n_active; q++) {  // keeps the longest-first order
            const int s2 = active[q];
            if (sc[s2].phase != 2 && sc[s2].status == 0) active[k++] = s2;
        }
        n_active = k;
    }
    cudaEventDestroy(ej);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ABIE_CUDA(cudaMemcpy(pos, d_pos, 3 * total * sizeof(double), cudaMemcpyDeviceToHost));
    ABIE_CUDA(cudaMemcpy(vel, d_vel, 3 * total * sizeof(double), cudaMemcpyDeviceToHost));
    for (int s = 0; s < ns; s++) {
        if (t_out) t_out[s] = sc[s].t;
        if (status) status[s] = sc[s].status;
        if (steps) steps[s] = sc[s].steps;
        if (stats) {
            stats->attempts += sc[s].attempts;
            stats->iterations += sc[s].iterations;
            stats->force_calls += sc[s].force_calls;
            stats->steps += sc[s].steps;
            stats->fallbacks += sc[s].fallbacks;
        }
    }
    if (stats) stats->launches += launches;
    g_last_seconds = gpu_ms * 1e-3;
    cudaFree(d_pos);
    cudaFree(d_vel);
    cudaFree(d_m);
    cudaFree(d_state);
    cudaFree(d_off);
    cudaFree(d_sc);
    cudaFree(d_active);
    cudaFree(d_queue);
    return 0;
}

double ensemble_last_seconds() { return g_last_seconds; }

}  // namespace abie

using namespace abie;

extern "C" {
// The share of systems (the slowest 1 in div, longest first) that run on
// four-warp groups; 0 restores the default.  For tests and tuning.
void abie_debug_ensemble_heavy(int div) { abie::g_heavy_div = div > 0 ? div : 0; }


int abie_gr_ensemble(double *pos, double *vel, const double *m, const long long *offsets,
                     int n_systems, double G, double t0, double t_end, double *t_out, int *status,
                     long long *steps, int flags)
{
    int rc = ensure_device(-1);
    if (rc) return rc;
    const LearnedPredictor *mlp = (flags & 1) ? learned_predictor_current() : nullptr;
    if ((flags & 1) && !mlp) {
        set_error(ABIE_ERR_ARGUMENT, "abie_gr_ensemble: learned predictor requested, none enabled");
        return ABIE_ERR_ARGUMENT;
    }
    EnsembleLearnIO io = {};
    if (flags & 2) {
        rc = mlp_collect_begin(&io);
        if (rc) return rc;
    }
    EnsembleStats st = {};
    rc = ensemble_run(pos, vel, m, offsets, n_systems, G, t0, t_end, t_out, status, steps,
                      g_sim.force_mode, mlp, g_sim.st, &st, (flags & 2) ? &io : nullptr,
                      (flags & 1) || (flags & 4), mlp ? learned_predictor_tau() : nullptr);
    if (flags & 2) mlp_collect_end(&io);
    if (rc == 0) {
        g_sim.ctr.attempts += st.attempts;
        g_sim.ctr.iterations += st.iterations;
        g_sim.ctr.force_calls += st.force_calls;
        g_sim.ctr.accepts += st.steps;
        g_sim.ctr.rejects += st.attempts - st.steps;
        g_sim.ctr.learned_fallbacks += st.fallbacks;
    }
    return rc;
}

double abie_last_ensemble_seconds(void) { return ensemble_last_seconds(); }

}  // extern "C"
