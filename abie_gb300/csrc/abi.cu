// C ABI shell: the reference's libabie entry points (src/common.c:200-413)
// over a device-resident simulation state.
//
// The reference keeps one global Simulation (src/common.h:26-70) on the
// host and offloads only the force loop (src/gpuforce.cu); here the state
// lives in GPU memory from set_state to get_state, and the integrators run
// on the device without host round trips.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "abi_state.cuh"
#include "engine.cuh"
#include "pn.cuh"
#include "force.cuh"

namespace abie {

Sim g_sim;
static char g_err[512] = "";

void set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int k = snprintf(g_err, sizeof g_err, "[%d] ", code);
    if (k < 0) k = 0;
    vsnprintf(g_err + k, sizeof g_err - (size_t)k, fmt, ap);
    va_end(ap);
    fprintf(stderr, "abie_gb300: %s\n", g_err);
}

int cuda_fail(cudaError_t e, const char *what)
{
    set_error(ABIE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return ABIE_ERR_CUDA;
}

static size_t lo32(size_t v) { return v & 0xffffffffull; }

// A CUDA context on one sm_103 device plus the library stream.  Used by the
// stateless entry points before (or without) initialize_code.
int ensure_device(int want)
{
    Sim &s = g_sim;
    if (s.dev >= 0) {
        if (want >= 0 && want != s.dev) {
            set_error(ABIE_ERR_ARGUMENT, "device %d requested, library bound to device %d", want,
                      s.dev);
            return ABIE_ERR_ARGUMENT;
        }
        return 0;
    }
    if (want < 0) want = 0;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        set_error(ABIE_ERR_NO_DEVICE, "no CUDA device available (%s)",
                  e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
        return ABIE_ERR_NO_DEVICE;
    }
    if (want >= count) {
        set_error(ABIE_ERR_NO_DEVICE, "device %d requested, %d present", want, count);
        return ABIE_ERR_NO_DEVICE;
    }
    cudaDeviceProp p;
    ABIE_CUDA(cudaGetDeviceProperties(&p, want));
    if (p.major != 10 || p.minor != 3) {
        set_error(ABIE_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a",
                  want, p.major, p.minor);
        return ABIE_ERR_NO_DEVICE;
    }
    ABIE_CUDA(cudaSetDevice(want));
    ABIE_CUDA(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    s.dev = want;
    s.num_sms = p.multiProcessorCount;
    return 0;
}

int reserve(double **p, size_t *cap, size_t n)
{
    if (n <= *cap && *p) return 0;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    size_t c = n < 64 ? 64 : n;
    ABIE_CUDA(cudaMalloc(p, c * sizeof(double)));
    *cap = c;
    return 0;
}

static void free_dev(double *&p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

// Host-array force into host acc (used by ode_n_body_second_order and
// abie_force_host).  For sinks with m < 0 the caller's acc entries are kept,
// as the reference leaves them untouched.
static int host_force(const double *pos, const double *m, size_t n, double G, double *acc,
                      int mode, const double *vel = nullptr, double C = 0.0)
{
    int rc = ensure_device(-1);
    if (rc) return rc;
    if (n == 0) return 0;
    Sim &s = g_sim;
    if ((rc = reserve(&s.tmp_pos, &s.tmp_pos_cap, 3 * n))) return rc;
    if ((rc = reserve(&s.tmp_m, &s.tmp_m_cap, n))) return rc;
    if ((rc = reserve(&s.tmp_acc, &s.tmp_acc_cap, 3 * n))) return rc;
    bool any_deleted = false;
    for (size_t i = 0; i < n; i++) any_deleted |= (m[i] < 0.0);
    ABIE_CUDA(cudaMemcpyAsync(s.tmp_pos, pos, 3 * n * sizeof(double), cudaMemcpyHostToDevice, s.st));
    ABIE_CUDA(cudaMemcpyAsync(s.tmp_m, m, n * sizeof(double), cudaMemcpyHostToDevice, s.st));
    if (any_deleted)
        ABIE_CUDA(cudaMemcpyAsync(s.tmp_acc, acc, 3 * n * sizeof(double), cudaMemcpyHostToDevice,
                                  s.st));
    rc = launch_force(mode, s.tmp_pos, s.tmp_m, (int)n, G, s.fs, s.tmp_acc, s.st);
    if (rc) return rc;
    if (vel && C > 0.0) {  // src/common.c:101-107 -> src/additional_forces.c:14-121
        if ((rc = reserve(&s.tmp_vel, &s.tmp_vel_cap, 3 * n))) return rc;
        ABIE_CUDA(cudaMemcpyAsync(s.tmp_vel, vel, 3 * n * sizeof(double), cudaMemcpyHostToDevice, s.st));
        rc = launch_post_newtonian(s.tmp_pos, s.tmp_vel, s.tmp_m, (int)n, G, C, s.tmp_acc, s.st,
                                   mode == ABIE_FORCE_FP64 || mode == ABIE_FORCE_MIXED);
        if (rc) return rc;
    }
    ABIE_CUDA(cudaMemcpyAsync(acc, s.tmp_acc, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, s.st));
    ABIE_CUDA(cudaStreamSynchronize(s.st));
    s.ctr.force_calls++;
    return 0;
}

}  // namespace abie

using namespace abie;

extern "C" {

int abie_last_error(char *buf, size_t len)
{
    size_t k = strlen(g_err);
    if (buf && len) {
        size_t c = k < len - 1 ? k : len - 1;
        memcpy(buf, g_err, c);
        buf[c] = 0;
    }
    return (int)k;
}

int abie_set_force_mode(int mode)
{
    if (mode < ABIE_FORCE_EXACT || mode > ABIE_FORCE_NAIVE) {
        set_error(ABIE_ERR_ARGUMENT, "unknown force mode %d", mode);
        return ABIE_ERR_ARGUMENT;
    }
    int old = g_sim.force_mode;
    g_sim.force_mode = mode;
    return old;
}

int abie_get_force_mode(void) { return g_sim.force_mode; }

int abie_get_counters(abie_counters *out)
{
    if (!out) return ABIE_ERR_ARGUMENT;
    *out = g_sim.ctr;
    return 0;
}

void abie_reset_counters(void) { memset(&g_sim.ctr, 0, sizeof g_sim.ctr); }

int initialize_code(double G, double C, size_t N_MAX, size_t MAX_N_CE, size_t MAX_N_COLLISIONS,
                    int deviceID)
{
    Sim &s = g_sim;
    if (s.inited) return 0;  // once per process, src/common.c:227
    if (deviceID < 0) {
        // The reference's default (abie/__init__.py:31) selects its CPU code;
        // this library has only the GPU path, so it runs on GPU 0 and says so
        // (the reference's binding ignores initialize_code's return value).
        fprintf(stderr,
                "abie_gb300: deviceID=%d selects the reference's CPU code; this library has "
                "only the GPU path and runs on GPU 0\n",
                deviceID);
        deviceID = 0;
    }
    int rc = ensure_device(deviceID);
    if (rc) return rc;
    N_MAX = lo32(N_MAX);
    s.G = G;
    s.C = C;
    s.max_ce = lo32(MAX_N_CE);
    s.max_coll = lo32(MAX_N_COLLISIONS);
    s.n_ce = 0;
    s.n_coll = 0;
    s.buf_ce.assign(4 * s.max_ce, 0.0);
    s.buf_coll.assign(4 * s.max_coll, 0.0);
    s.n_max = N_MAX;
    size_t nm = N_MAX ? N_MAX : 1;
    if ((rc = reserve(&s.pos, &s.pos_cap, 3 * nm))) return rc;
    if ((rc = reserve(&s.vel, &s.vel_cap, 3 * nm))) return rc;
    if ((rc = reserve(&s.m, &s.m_cap, nm))) return rc;
    if ((rc = reserve(&s.r, &s.r_cap, nm))) return rc;
    if ((rc = reserve(&s.ext_acc, &s.ext_cap, 3 * nm))) return rc;
    ABIE_CUDA(cudaMemsetAsync(s.ext_acc, 0, 3 * nm * sizeof(double), s.st));
    ABIE_CUDA(cudaStreamSynchronize(s.st));
    s.ext_enabled = false;
    s.n = 0;
    s.t = 0.0;
    s.inited = true;
    return 0;
}

int finalize_code(void)
{
    Sim &s = g_sim;
    free_dev(s.pos);
    free_dev(s.vel);
    free_dev(s.m);
    free_dev(s.r);
    free_dev(s.ext_acc);
    free_dev(s.tmp_pos);
    free_dev(s.tmp_m);
    free_dev(s.tmp_acc);
    free_dev(s.tmp_vel);
    free_dev(s.energy_partials);
    s.pos_cap = s.vel_cap = s.m_cap = s.r_cap = s.ext_cap = 0;
    s.tmp_pos_cap = s.tmp_m_cap = s.tmp_acc_cap = s.tmp_vel_cap = s.energy_cap = 0;
    force_scratch_free(s.fs);
    free_engine_buffers();
    free_wh_buffers();
    free_rk_buffers();
    // like the reference, a finalized library is not re-initialized in the
    // same process (src/common.c:382-398 leaves code_inited set)
    return 0;
}

void set_state(double *pos, double *vel, double *m, double *r, size_t N, double G, double C)
{
    Sim &s = g_sim;
    N = lo32(N);
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "set_state before initialize_code");
        return;
    }
    if (N > s.n_max) {
        set_error(ABIE_ERR_CAPACITY, "set_state: N=%zu above N_MAX=%zu", N, s.n_max);
        return;
    }
    s.n = N;
    s.G = G;
    s.C = C;
    s.h_m.assign(m, m + N);
    s.h_r.assign(r, r + N);
    if (N == 0) return;
    cudaError_t e = cudaMemcpyAsync(s.pos, pos, 3 * N * sizeof(double), cudaMemcpyHostToDevice, s.st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.vel, vel, 3 * N * sizeof(double), cudaMemcpyHostToDevice, s.st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.m, m, N * sizeof(double), cudaMemcpyHostToDevice, s.st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.r, r, N * sizeof(double), cudaMemcpyHostToDevice, s.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s.st);
    if (e != cudaSuccess) cuda_fail(e, "set_state");
}

int get_state(double *pos, double *vel, double *m, double *r)
{
    Sim &s = g_sim;
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "get_state before initialize_code");
        return ABIE_ERR_NOT_INITIALIZED;
    }
    size_t N = s.n;
    if (N == 0) return 0;
    ABIE_CUDA(cudaMemcpyAsync(pos, s.pos, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, s.st));
    ABIE_CUDA(cudaMemcpyAsync(vel, s.vel, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, s.st));
    ABIE_CUDA(cudaStreamSynchronize(s.st));
    if (m) memcpy(m, s.h_m.data(), N * sizeof(double));
    if (r) memcpy(r, s.h_r.data(), N * sizeof(double));
    return (int)N;
}

double get_model_time(void) { return g_sim.t; }

void set_close_encounter_distance(double d) { g_sim.ce_dist = d; }

double get_close_encounter_distance(void) { return g_sim.ce_dist; }

void get_close_encounter_buffer(double *buf_ce)
{
    if (buf_ce && !g_sim.buf_ce.empty())
        memcpy(buf_ce, g_sim.buf_ce.data(), g_sim.buf_ce.size() * sizeof(double));
}

void get_collision_buffer(double *buf_collision)
{
    if (buf_collision && !g_sim.buf_coll.empty())
        memcpy(buf_collision, g_sim.buf_coll.data(), g_sim.buf_coll.size() * sizeof(double));
}

void reset_close_encounter_buffer(void)
{
    g_sim.n_ce = 0;
    std::fill(g_sim.buf_ce.begin(), g_sim.buf_ce.end(), 0.0);
}

void reset_collision_buffer(void)
{
    g_sim.n_coll = 0;
    std::fill(g_sim.buf_coll.begin(), g_sim.buf_coll.end(), 0.0);
}

size_t set_additional_forces(size_t N, double *ext_acc)
{
    Sim &s = g_sim;
    N = lo32(N);
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "set_additional_forces before initialize_code");
        return 0;
    }
    if (N > s.n_max) {
        set_error(ABIE_ERR_CAPACITY, "set_additional_forces: N=%zu above N_MAX=%zu", N, s.n_max);
        return 0;
    }
    // a NULL vector switches the external accelerations off again (the
    // reference has no way to do so)
    s.ext_enabled = ext_acc != nullptr;
    if (N && ext_acc) {
        cudaError_t e = cudaMemcpyAsync(s.ext_acc, ext_acc, 3 * N * sizeof(double),
                                        cudaMemcpyHostToDevice, s.st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s.st);
        if (e != cudaSuccess) cuda_fail(e, "set_additional_forces");
    }
    return 0;
}

double calculate_energy(void)
{
    Sim &s = g_sim;
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "calculate_energy before initialize_code");
        return 0.0;
    }
    if (reserve(&s.energy_partials, &s.energy_cap, 2 * (s.n / 8 + 2))) return 0.0;
    double e = 0.0;
    if (launch_energy(s.pos, s.vel, s.m, (int)s.n, s.G, s.energy_partials, &e, s.st)) return 0.0;
    return e;
}

double abie_energy_host(const double *pos, const double *vel, const double *m, size_t N, double G)
{
    Sim &s = g_sim;
    N = lo32(N);
    if (ensure_device(-1)) return 0.0;
    if (reserve(&s.tmp_pos, &s.tmp_pos_cap, 3 * N) || reserve(&s.tmp_acc, &s.tmp_acc_cap, 3 * N) ||
        reserve(&s.tmp_m, &s.tmp_m_cap, N) ||
        reserve(&s.energy_partials, &s.energy_cap, 2 * (N / 8 + 2)))
        return 0.0;
    if (cudaMemcpyAsync(s.tmp_pos, pos, 3 * N * 8, cudaMemcpyHostToDevice, s.st) ||
        cudaMemcpyAsync(s.tmp_acc, vel, 3 * N * 8, cudaMemcpyHostToDevice, s.st) ||
        cudaMemcpyAsync(s.tmp_m, m, N * 8, cudaMemcpyHostToDevice, s.st)) {
        cuda_fail(cudaGetLastError(), "abie_energy_host copy");
        return 0.0;
    }
    double e = 0.0;
    launch_energy(s.tmp_pos, s.tmp_acc, s.tmp_m, (int)N, G, s.energy_partials, &e, s.st);
    return e;
}

size_t ode_n_body_second_order(const double *pos, size_t N, double G, const double *masses,
                               const double *radii, double *acc)
{
    (void)radii;
    int rc = host_force(pos, masses, lo32(N), G, acc, g_sim.force_mode);
    return rc ? (size_t)(long long)rc : 0;
}

size_t calculate_accelerations(const double *pos, const double *vel, size_t N, double G,
                               const double *masses, const double *radii, double *acc)
{
    (void)radii;
    Sim &s = g_sim;
    N = lo32(N);
    // Newton, then the post-Newtonian terms when the stored C is positive
    // (src/common.c:82-114), then the external accelerations
    int rc = host_force(pos, masses, N, G, acc, s.force_mode, vel, s.C);
    if (rc) return (size_t)(long long)rc;
    if (s.ext_enabled && s.inited && N <= s.n_max) {
        std::vector<double> ext(3 * N);
        if (cudaMemcpy(ext.data(), s.ext_acc, 3 * N * sizeof(double), cudaMemcpyDeviceToHost) !=
            cudaSuccess)
            return (size_t)(long long)cuda_fail(cudaGetLastError(), "ext_acc readback");
        for (size_t i = 0; i < 3 * N; i++) acc[i] += ext[i];
    }
    return 0;
}

int abie_force_host(const double *pos, const double *m, size_t N, double G, double *acc, int mode)
{
    if (mode < ABIE_FORCE_EXACT || mode > ABIE_FORCE_NAIVE) {
        set_error(ABIE_ERR_ARGUMENT, "unknown force mode %d", mode);
        return ABIE_ERR_ARGUMENT;
    }
    return host_force(pos, m, lo32(N), G, acc, mode);
}

int abie_force_device(const double *d_pos, const double *d_m, size_t N, double G, double *d_acc,
                      int mode, void *stream)
{
    int rc = ensure_device(-1);
    if (rc) return rc;
    if (mode < ABIE_FORCE_EXACT || mode > ABIE_FORCE_NAIVE) {
        set_error(ABIE_ERR_ARGUMENT, "unknown force mode %d", mode);
        return ABIE_ERR_ARGUMENT;
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : g_sim.st;
    rc = launch_force(mode, d_pos, d_m, (int)lo32(N), G, g_sim.fs, d_acc, st);
    if (!rc) g_sim.ctr.force_calls++;
    return rc;
}

}  // extern "C"

extern "C" {
// Fixes the fast FP64 kernel's launch shape (lanes per sink, source chunks)
// for tests and the autotuner; (0, 0) restores the automatic choice.
void abie_debug_force_shape(int lanes_per_sink, int chunks)
{
    abie::force_shape_override(lanes_per_sink, chunks);
}
}
