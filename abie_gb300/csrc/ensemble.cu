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
#include <sys/stat.h>

#include <algorithm>
#include <string>
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

// ---------------------------------------------------------------------------
// Host side.  A batch keeps its device buffers and pinned staging for the
// whole call.  Every launch over the systems not yet done is one replay of
// a CUDA graph built once per batch: the active lists' upload from pinned
// memory, the work counters' reset, one kernel node per class of system
// (independent nodes, so the classes run side by side) and the per-system
// scalars' download.  Between replays only the kernel nodes' arguments and
// grids change (cudaGraphExecKernelNodeSetParams); each launch yields after
// about two seconds of GPU time, so a long run is a few hundred replays.

struct EnsBatch {
    int ns = 0;
    long long total = 0;
    double *d_pos = nullptr, *d_vel = nullptr, *d_m = nullptr, *d_state = nullptr;
    double *d_pos0 = nullptr, *d_vel0 = nullptr;  // the inputs, for the tuner's trials
    long long *d_off = nullptr;
    EnsScalars *d_sc = nullptr;
    int *d_active = nullptr, *d_queue = nullptr;
    int *h_active = nullptr;     // pinned
    EnsScalars *h_sc = nullptr;  // pinned
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t kern[3] = {nullptr, nullptr, nullptr};
    const void *fn[3] = {nullptr, nullptr, nullptr};
    size_t dyn[3] = {0, 0, 0};
    int bps[3] = {1, 1, 1};
    ~EnsBatch()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (double *p : {d_pos, d_vel, d_m, d_state, d_pos0, d_vel0})
            if (p) cudaFree(p);
        if (d_off) cudaFree(d_off);
        if (d_sc) cudaFree(d_sc);
        if (d_active) cudaFree(d_active);
        if (d_queue) cudaFree(d_queue);
        if (h_active) cudaFreeHost(h_active);
        if (h_sc) cudaFreeHost(h_sc);
    }
};

static const int WC[3] = {1, 2, 4};  // warps per system in each class

// The graph of one launch over the batch (see above); kernel nodes start
// with empty work and get their arguments before each replay.
static int build_graph(EnsBatch &B, const EnsArgs &base)
{
    ABIE_CUDA(cudaGraphCreate(&B.graph, 0));
    cudaGraphNode_t up, reset, down;
    ABIE_CUDA(cudaGraphAddMemcpyNode1D(&up, B.graph, nullptr, 0, B.d_active, B.h_active,
                                       (size_t)B.ns * sizeof(int), cudaMemcpyHostToDevice));
    cudaMemsetParams ms = {};
    ms.dst = B.d_queue;
    ms.value = 0;
    ms.elementSize = sizeof(int);
    ms.width = 3;
    ms.height = 1;
    ABIE_CUDA(cudaGraphAddMemsetNode(&reset, B.graph, nullptr, 0, &ms));
    cudaGraphNode_t deps[2] = {up, reset};
    for (int k = 0; k < 3; k++) {
        EnsArgs a = base;
        a.active = B.d_active;
        a.n_active = 0;
        a.queue = B.d_queue + k;
        void *args[] = {&a};
        cudaKernelNodeParams p = {};
        p.func = const_cast<void *>(B.fn[k]);
        p.gridDim = dim3(1);
        p.blockDim = dim3(32 * WARPS);
        p.sharedMemBytes = (unsigned)B.dyn[k];
        p.kernelParams = args;
        ABIE_CUDA(cudaGraphAddKernelNode(&B.kern[k], B.graph, deps, 2, &p));
    }
    ABIE_CUDA(cudaGraphAddMemcpyNode1D(&down, B.graph, B.kern, 3, B.h_sc, B.d_sc,
                                       (size_t)B.ns * sizeof(EnsScalars), cudaMemcpyDeviceToHost));
    ABIE_CUDA(cudaGraphInstantiate(&B.exec, B.graph, 0));
    return 0;
}

// Runs the batch from its current device state until every system is done
// (or has stopped with an error); t_stop replaces the systems' end time
// (the tuner's trials stop early).  Adds the GPU time of the launches to
// *gpu_s and their number to *launches; leaves the scalars in B.h_sc.
static int run_launches(EnsBatch &B, const EnsArgs &base, const std::vector<int> &order,
                        const std::vector<unsigned char> &cls, double t_stop, cudaStream_t st,
                        double *gpu_s, int *launches)
{
    cudaEvent_t e0, e1;
    ABIE_CUDA(cudaEventCreate(&e0));
    ABIE_CUDA(cudaEventCreate(&e1));
    std::vector<int> active(order);
    int n_active = (int)active.size();
    int rc = 0;
    while (n_active > 0) {
        // the classes' lists, each in longest-first order, one after another
        int first[4] = {0, 0, 0, 0};
        int k2 = 0;
        for (int c = 0; c < 3; c++) {
            first[c] = k2;
            for (int q = 0; q < n_active; q++)
                if (cls[active[q]] == c) B.h_active[k2++] = active[q];
        }
        first[3] = k2;
        for (int k = 0; k < 3; k++) {
            const int cnt = first[k + 1] - first[k];
            EnsArgs a = base;
            a.t_end = t_stop;
            a.active = B.d_active + first[k];
            a.n_active = cnt;
            a.queue = B.d_queue + k;
            const int per_block = WARPS / WC[k];
            const int blocks = cnt == 0 ? 1
                                        : (int)std::max<long long>(1, std::min<long long>(
                                              (long long)B.bps[k] * g_sim.num_sms,
                                              (cnt + per_block - 1) / per_block));
            void *args[] = {&a};
            cudaKernelNodeParams p = {};
            p.func = const_cast<void *>(B.fn[k]);
            p.gridDim = dim3((unsigned)blocks);
            p.blockDim = dim3(32 * WARPS);
            p.sharedMemBytes = (unsigned)B.dyn[k];
            p.kernelParams = args;
            cudaError_t e = cudaGraphExecKernelNodeSetParams(B.exec, B.kern[k], &p);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "ensemble graph: kernel node parameters");
                break;
            }
        }
        if (rc) break;
        cudaError_t e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) e = cudaGraphLaunch(B.exec, st);
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "ensemble graph launch");
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        *gpu_s += ms * 1e-3;
        ++*launches;
        int k = 0;
        for (int q = 0; q < n_active; q++) {  // keeps the longest-first order
            const int s2 = active[q];
            if (B.h_sc[s2].phase != 2 && B.h_sc[s2].status == 0) active[k++] = s2;
        }
        n_active = k;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// Class of each system for a share of four-warp groups: the slowest 1 in
// div (longest first) on four warps, the rest by size.
static void classes(const std::vector<int> &order, const long long *offsets, int div,
                    std::vector<unsigned char> &cls)
{
    const int ns = (int)order.size();
    cls.assign(ns, 0);
    const int heavy = std::min(ns, std::max(1, ns / div));
    for (int q = 0; q < ns; q++) {
        const int s2 = order[q];
        cls[s2] = q < heavy ? 2 : (3 * (offsets[s2 + 1] - offsets[s2]) <= 32 ? 0 : 1);
    }
}

// --- autotuner ---------------------------------------------------------------
// The share of systems on four-warp groups is picked per workload by timing
// candidate shares on the batch itself: each trial restarts the systems
// from their inputs (device copies) and runs them over a slice of the
// requested span, sized from a short probe so that a trial takes about
// 0.2 s of GPU time (or the whole span when that is shorter); each share is
// timed twice and the faster time counts; the fastest share wins, unless
// the default share (1 in 4 for the fast forms, 1 in 256 for the reference's
// operations) is within 2 % of it.  The choice is cached in a text file keyed by the device, the
// build of this library, the force form, the number of systems, a hash of
// their body counts and masses, and the span, so a workload is tuned once.
// ABIE_ENSEMBLE_TUNE=0 switches the tuner off (the defaults below then
// apply); ABIE_TUNE_CACHE names the cache file (default
// $XDG_CACHE_HOME/abie_gb300/ensemble_tune.tsv or
// $HOME/.cache/abie_gb300/ensemble_tune.tsv).
struct EnsTuneInfo {
    int heavy_div = 0;
    int from_cache = 0;   // 1: read from the cache file, 2: debug override, 0: measured or default
    double tune_seconds = 0.0;
    int candidates = 0;
};
static EnsTuneInfo g_last_tune;
static const char *ENS_BUILD = __DATE__ " " __TIME__;

static std::string tune_cache_path()
{
    if (const char *p = getenv("ABIE_TUNE_CACHE")) return p;
    std::string base;
    if (const char *x = getenv("XDG_CACHE_HOME")) base = x;
    else if (const char *h = getenv("HOME")) base = std::string(h) + "/.cache";
    else return "";
    return base + "/abie_gb300/ensemble_tune.tsv";
}

static void mkdirs_for(const std::string &file)
{
    for (size_t i = 1; i < file.size(); i++)
        if (file[i] == '/') mkdir(file.substr(0, i).c_str(), 0755);
}

static std::string tune_key(int mode, bool net, int ns, const long long *offsets, const double *m,
                            double span)
{
    unsigned long long h = 1469598103934665603ull;  // FNV-1a over body counts and masses
    auto mix = [&](unsigned long long v) {
        for (int b = 0; b < 8; b++) {
            h ^= (v >> (8 * b)) & 0xff;
            h *= 1099511628211ull;
        }
    };
    for (int s = 0; s <= ns; s++) mix((unsigned long long)offsets[s]);
    for (long long i = 0; i < offsets[ns]; i++) {
        unsigned long long b;
        memcpy(&b, &m[i], sizeof b);
        mix(b);
    }
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, g_sim.dev);
    char key[512];
    snprintf(key, sizeof key, "%s|%s|mode%d%s|ns%d|h%016llx|span%.3g", p.name, ENS_BUILD, mode,
             net ? "+net" : "", ns, h, span);
    for (char *c = key; *c; c++)
        if (*c == '\t' || *c == '\n') *c = ' ';
    return key;
}

static int tune_lookup(const std::string &key)
{
    const std::string path = tune_cache_path();
    if (path.empty()) return 0;
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return 0;
    char line[1024];
    int found = 0;
    while (fgets(line, sizeof line, f)) {
        char *tab = strchr(line, '\t');
        if (!tab) continue;
        *tab = 0;
        if (key == line) found = atoi(tab + 1);  // the last entry wins
    }
    fclose(f);
    return found;
}

static void tune_store(const std::string &key, int div, double secs, const std::vector<double> &times,
                       const std::vector<int> &cands)
{
    const std::string path = tune_cache_path();
    if (path.empty()) return;
    mkdirs_for(path);
    FILE *f = fopen(path.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s\t%d\t%.6f\t", key.c_str(), div, secs);
    for (size_t i = 0; i < cands.size(); i++)
        fprintf(f, "%s%d:%.6f", i ? "," : "", cands[i], times[i]);
    fprintf(f, "\n");
    fclose(f);
}

static bool tuner_on()
{
    const char *v = getenv("ABIE_ENSEMBLE_TUNE");  // read on every call
    return !(v && v[0] == '0');
}

// Restart every system of the batch from its inputs.
static int batch_restart(EnsBatch &B, const std::vector<EnsScalars> &sc0, cudaStream_t st)
{
    ABIE_CUDA(cudaMemcpyAsync(B.d_pos, B.d_pos0, 3 * B.total * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(B.d_vel, B.d_vel0, 3 * B.total * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(B.d_sc, sc0.data(), B.ns * sizeof(EnsScalars), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaStreamSynchronize(st));
    return 0;
}

int ensemble_run(double *pos, double *vel, const double *m, const long long *offsets, int ns,
                 double G, double t0, double t_end, double *t_out, int *status, long long *steps,
                 int mode, const LearnedPredictor *mlp, cudaStream_t st, EnsembleStats *stats,
                 const EnsembleLearnIO *learn_io, bool consistent, const float *mlp_tau)
{
    if (ns <= 0) return 0;
    const long long total = offsets[ns];
    for (int s = 0; s < ns; s++) {
        long long k = offsets[s + 1] - offsets[s];
        if (k < 1 || k > ENS_MAX_BODIES) {
            set_error(ABIE_ERR_ARGUMENT, "ensemble system %d has %lld bodies (1..%d supported)", s,
                      k, ENS_MAX_BODIES);
            return ABIE_ERR_ARGUMENT;
        }
    }
    const bool learning = mlp || (learn_io && learn_io->samples);
    if (mode == ABIE_FORCE_NAIVE && learning) {
        set_error(ABIE_ERR_UNSUPPORTED,
                  "abie_gr_ensemble: the plain FP64 form runs the reference's predictor only "
                  "(no learned predictor, no sample collection)");
        return ABIE_ERR_UNSUPPORTED;
    }
    EnsBatch B;
    B.ns = ns;
    B.total = total;
    ABIE_CUDA(cudaMalloc(&B.d_pos, 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&B.d_vel, 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&B.d_m, total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&B.d_state, (size_t)STATE_PER_COMP * 3 * total * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&B.d_off, (ns + 1) * sizeof(long long)));
    ABIE_CUDA(cudaMalloc(&B.d_sc, ns * sizeof(EnsScalars)));
    ABIE_CUDA(cudaMalloc(&B.d_active, ns * sizeof(int)));
    ABIE_CUDA(cudaMalloc(&B.d_queue, 3 * sizeof(int)));
    ABIE_CUDA(cudaMallocHost(&B.h_active, ns * sizeof(int)));
    ABIE_CUDA(cudaMallocHost(&B.h_sc, ns * sizeof(EnsScalars)));
    std::vector<EnsScalars> sc0(ns);
    for (int s = 0; s < ns; s++) {
        memset(&sc0[s], 0, sizeof(EnsScalars));
        sc0[s].t = t0;
    }
    // Longest-first order: a system's step count follows its shortest
    // two-body time scale sqrt(r_ij^3 / G(m_i + m_j)), and the batch takes
    // at least as long as its slowest system, so those start first.
    std::vector<double> rate(ns, 0.0);
    for (int s = 0; s < ns; s++) {
        double best = 0.0;
        for (long long i = offsets[s]; i < offsets[s + 1]; i++)
            for (long long j = i + 1; j < offsets[s + 1]; j++) {
                double mu = G * (std::max(m[i], 0.0) + std::max(m[j], 0.0));
                double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
                       dz = pos[3 * i + 2] - pos[3 * j + 2];
                double r2 = dx * dx + dy * dy + dz * dz;
                if (mu > 0.0 && r2 > 0.0) best = std::max(best, sqrt(mu / (r2 * sqrt(r2))));
            }
        rate[s] = best;
    }
    std::vector<int> order(ns);
    for (int s = 0; s < ns; s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return rate[x] > rate[y]; });
    ABIE_CUDA(cudaMemcpyAsync(B.d_pos, pos, 3 * total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(B.d_vel, vel, 3 * total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(B.d_m, m, total * sizeof(double), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(B.d_off, offsets, (ns + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaMemcpyAsync(B.d_sc, sc0.data(), ns * sizeof(EnsScalars), cudaMemcpyHostToDevice, st));
    ABIE_CUDA(cudaStreamSynchronize(st));

    // three classes of system: up to 10 bodies on one warp, 11-21 on two,
    // and the slowest few (longest-first order) on four warps, which cuts
    // their per-substep latency -- the batch ends with its slowest system
    for (int k = 0; k < 3; k++) {
        B.fn[k] = ensemble_fn(mode, WC[k], learning);
        B.dyn[k] = learning ? learn_smem(WC[k]) : 0;
        if (learning)
            ABIE_CUDA(cudaFuncSetAttribute(B.fn[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B.dyn[k]));
        ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&B.bps[k], B.fn[k], 32 * WARPS, B.dyn[k]));
        B.bps[k] = std::max(B.bps[k], 1);
    }
    EnsArgs base = {};
    base.offsets = B.d_off;
    base.m = B.d_m;
    base.pos = B.d_pos;
    base.vel = B.d_vel;
    base.state = B.d_state;
    base.sc = B.d_sc;
    base.G = G;
    base.t_end = t_end;
    base.mlp = mlp;
    base.samples = learn_io ? learn_io->samples : nullptr;
    base.sample_cap = learn_io ? learn_io->cap : 0;
    base.sample_count = learn_io ? learn_io->count : nullptr;
    for (int k = 0; k < 7; k++) base.tau[k] = learn_io ? learn_io->tau[k] : (mlp_tau ? mlp_tau[k] : 1.0f);
    base.consistent_g = consistent ? 1 : 0;
    base.budget_ns = 2000000000ull;  // each launch yields after about two seconds
    int rc = build_graph(B, base);
    if (rc) return rc;

    // the share of four-warp groups: the debug override, the tuner (not
    // while collecting training samples: trials would append some; the
    // network's inference only reads its weights), or the default
    EnsTuneInfo info;
    std::vector<unsigned char> cls;
    const double span = t_end - t0;
    const bool collecting = learn_io && learn_io->samples;
    if (g_heavy_div > 0) {
        info.heavy_div = g_heavy_div;
        info.from_cache = 2;
    } else if (!collecting && tuner_on() && span > 0.0) {
        const std::string key = tune_key(mode, mlp != nullptr, ns, offsets, m, span);
        info.heavy_div = tune_lookup(key);
        if (info.heavy_div > 0) {
            info.from_cache = 1;
        } else {
            ABIE_CUDA(cudaMalloc(&B.d_pos0, 3 * total * sizeof(double)));
            ABIE_CUDA(cudaMalloc(&B.d_vel0, 3 * total * sizeof(double)));
            ABIE_CUDA(cudaMemcpyAsync(B.d_pos0, B.d_pos, 3 * total * sizeof(double), cudaMemcpyDeviceToDevice, st));
            ABIE_CUDA(cudaMemcpyAsync(B.d_vel0, B.d_vel, 3 * total * sizeof(double), cudaMemcpyDeviceToDevice, st));
            // probe: the default share over 0.2 % of the span
            double probe_s = 0.0;
            int probe_l = 0;
            classes(order, offsets, heavy_div(mode), cls);
            if ((rc = run_launches(B, base, order, cls, t0 + 0.002 * span, st, &probe_s, &probe_l))) return rc;
            const double est_full = probe_s / 0.002;
            const double frac = std::min(1.0, std::max(0.002, 0.2 / std::max(est_full, 1e-9)));
            const std::vector<int> cands = mode == ABIE_FORCE_EXACT ? std::vector<int>{4, 16, 64, 256}
                                                                    : std::vector<int>{2, 4, 8, 16, 64, 256};
            // each candidate timed twice (the faster counts); the default
            // share stays unless a candidate beats it by more than 2 %
            std::vector<double> times;
            double best = 1e300, spent = probe_s;
            const int dflt = heavy_div(mode);
            double t_dflt = 1e300;
            for (int div : cands) {
                double tmin = 1e300;
                for (int rep = 0; rep < 2; rep++) {
                    if ((rc = batch_restart(B, sc0, st))) return rc;
                    classes(order, offsets, div, cls);
                    double s = 0.0;
                    int l = 0;
                    if ((rc = run_launches(B, base, order, cls, t0 + frac * span, st, &s, &l))) return rc;
                    tmin = std::min(tmin, s);
                    spent += s;
                }
                times.push_back(tmin);
                if (div == dflt) t_dflt = tmin;
                if (tmin < best) {
                    best = tmin;
                    info.heavy_div = div;
                }
            }
            if (t_dflt <= 1.02 * best) info.heavy_div = dflt;
            info.tune_seconds = spent;
            info.candidates = (int)cands.size();
            tune_store(key, info.heavy_div, info.tune_seconds, times, cands);
            if ((rc = batch_restart(B, sc0, st))) return rc;
        }
    } else {
        info.heavy_div = heavy_div(mode);
    }
    classes(order, offsets, info.heavy_div, cls);
    double gpu_s = 0.0;
    int launches = 0;
    if ((rc = run_launches(B, base, order, cls, t_end, st, &gpu_s, &launches))) return rc;
    ABIE_CUDA(cudaMemcpy(pos, B.d_pos, 3 * total * sizeof(double), cudaMemcpyDeviceToHost));
    ABIE_CUDA(cudaMemcpy(vel, B.d_vel, 3 * total * sizeof(double), cudaMemcpyDeviceToHost));
    for (int s = 0; s < ns; s++) {
        const EnsScalars &S = B.h_sc[s];
        if (t_out) t_out[s] = S.t;
        if (status) status[s] = S.status;
        if (steps) steps[s] = S.steps;
        if (stats) {
            stats->attempts += S.attempts;
            stats->iterations += S.iterations;
            stats->force_calls += S.force_calls;
            stats->steps += S.steps;
            stats->fallbacks += S.fallbacks;
        }
    }
    if (stats) stats->launches += launches;
    g_last_seconds = gpu_s;
    g_last_tune = info;
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

int abie_ensemble_last_tuning(int *heavy_div, int *source, double *tune_seconds)
{
    if (heavy_div) *heavy_div = abie::g_last_tune.heavy_div;
    if (source) *source = abie::g_last_tune.from_cache;
    if (tune_seconds) *tune_seconds = abie::g_last_tune.tune_seconds;
    return abie::g_last_tune.candidates;
}

}  // extern "C"
