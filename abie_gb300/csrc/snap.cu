// Device snapshots: what the reference's Python layer stores after every
// chunk of store_dt (abie/integrator.py:158-204 with store_state, :233-252),
// kept in GPU memory instead of a get_state round trip and a Python loop
// over the bodies per chunk.
//
// Per chunk: the integrator on the device-resident state (integrator_gr or
// integrator_wh, as integrate_ctypes calls them), then on the device the
// model time, a copy of positions and velocities, a, e, i of every body
// about the primary (Particles.calculate_aei, abie/particles.py:352-376,
// over Tools.from_cartesian_to_aei's single-body branch,
// abie/tools.py:256-285) and the energy (calculate_energy).  The snapshots
// leave the GPU once, at the end.
//
// The chunk schedule is integrate()'s: dt = min(store_dt, t_end - t) once,
// then next_t = t + dt - ((t + dt) % dt) with Python's float modulo while
// t < t_end, t being the model time each chunk reaches.
#include <math.h>

#include <algorithm>

#include "abi_state.cuh"
#include "engine.cuh"

extern "C" int integrator_gr(double t, double t_end, double dt);
extern "C" int integrator_wh(double t, double t_end, double dt);
extern "C" double get_model_time(void);
extern "C" double calculate_energy(void);

namespace abie {

namespace {

struct PrimaryRec {
    double m, x, y, z, vx, vy, vz;
};

// Knuth's TwoSum: s + e = a + b exactly.
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e)
{
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (sh, sl) += (bh, bl), a double-double sum.
__device__ __forceinline__ void dd_add(double &sh, double &sl, double bh, double bl)
{
    double s, e;
    two_sum(sh, bh, s, e);
    e += sl + bl;
    two_sum(s, e, sh, sl);
}

constexpr int PT = 256;  // threads of the primary kernel (one block)

// The primary body (abie/particles.py:378-397).  mode -1: centre of mass of
// all bodies with their total mass (particles.py:301-315); the sums are
// double-double in a fixed order, so the result is the exact sum rounded
// once (the reference's sequential sum can differ in its last bits).
// mode -2 / -3: the body of largest / smallest mass, first index on ties
// (np.argmax / np.argmin); mode >= 0: that body.
__global__ void __launch_bounds__(PT) primary_kernel(const double *__restrict__ pos,
                                                     const double *__restrict__ vel,
                                                     const double *__restrict__ m, int n, int mode,
                                                     PrimaryRec *__restrict__ out)
{
    __shared__ double sh[7][PT], sl[7][PT];
    __shared__ double bv[PT];
    __shared__ int bi[PT];
    const int tid = threadIdx.x;
    if (mode >= 0) {
        if (tid == 0) {
            const int k = mode;
            *out = PrimaryRec{m[k], pos[3 * k], pos[3 * k + 1], pos[3 * k + 2],
                              vel[3 * k], vel[3 * k + 1], vel[3 * k + 2]};
        }
        return;
    }
    if (mode == -1) {
        double h[7] = {0, 0, 0, 0, 0, 0, 0}, l[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int k = tid; k < n; k += PT) {
            const double mk = m[k];
            const double v[7] = {mk, pos[3 * k] * mk, pos[3 * k + 1] * mk, pos[3 * k + 2] * mk,
                                 vel[3 * k] * mk, vel[3 * k + 1] * mk, vel[3 * k + 2] * mk};
#pragma unroll
            for (int q = 0; q < 7; q++) dd_add(h[q], l[q], v[q], 0.0);
        }
#pragma unroll
        for (int q = 0; q < 7; q++) {
            sh[q][tid] = h[q];
            sl[q][tid] = l[q];
        }
        __syncthreads();
        for (int o = PT / 2; o > 0; o >>= 1) {
            if (tid < o) {
#pragma unroll
                for (int q = 0; q < 7; q++) {
                    double a = sh[q][tid], b = sl[q][tid];
                    dd_add(a, b, sh[q][tid + o], sl[q][tid + o]);
                    sh[q][tid] = a;
                    sl[q][tid] = b;
                }
            }
            __syncthreads();
        }
        if (tid == 0) {
            double r[7];
#pragma unroll
            for (int q = 0; q < 7; q++) r[q] = sh[q][0] + sl[q][0];
            *out = PrimaryRec{r[0], r[1] / r[0], r[2] / r[0], r[3] / r[0],
                              r[4] / r[0], r[5] / r[0], r[6] / r[0]};
        }
        return;
    }
    // argmax (-2) / argmin (-3), the first index among equals
    const bool want_max = mode == -2;
    double best = want_max ? -INFINITY : INFINITY;
    int bidx = n;
    for (int k = tid; k < n; k += PT) {
        const double v = m[k];
        if (want_max ? (v > best) : (v < best)) {
            best = v;
            bidx = k;
        }
    }
    bv[tid] = best;
    bi[tid] = bidx;
    __syncthreads();
    for (int o = PT / 2; o > 0; o >>= 1) {
        if (tid < o) {
            const double v = bv[tid + o];
            const int i = bi[tid + o];
            const bool better = want_max ? (v > bv[tid]) : (v < bv[tid]);
            if (better || (v == bv[tid] && i < bi[tid])) {
                bv[tid] = v;
                bi[tid] = i;
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        const int k = bi[0] < n ? bi[0] : 0;
        *out = PrimaryRec{m[k], pos[3 * k], pos[3 * k + 1], pos[3 * k + 2],
                          vel[3 * k], vel[3 * k + 1], vel[3 * k + 2]};
    }
}

// a, e, i of every body about the primary (abie/tools.py:256-285, in its
// operation order): one thread per body.  A body at the primary's position
// gets NaN, as the reference returns for r == 0.
__global__ void __launch_bounds__(256) aei_kernel(const double *__restrict__ pos,
                                                  const double *__restrict__ vel,
                                                  const double *__restrict__ m, int n, double G,
                                                  const PrimaryRec *__restrict__ pr,
                                                  double *__restrict__ aei)
{
    const PrimaryRec P = *pr;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double x = pos[3 * k] - P.x, y = pos[3 * k + 1] - P.y, z = pos[3 * k + 2] - P.z;
        const double vx = vel[3 * k] - P.vx, vy = vel[3 * k + 1] - P.vy, vz = vel[3 * k + 2] - P.vz;
        const double total_mass = m[k] + P.m;
        const double mu = G * total_mass;
        const double v_sq = vx * vx + vy * vy + vz * vz;
        const double r_sq = x * x + y * y + z * z;
        const double r = sqrt(r_sq);
        if (r == 0.0) {
            aei[3 * k] = aei[3 * k + 1] = aei[3 * k + 2] = nan("");
            continue;
        }
        const double specific_energy = (1.0 / 2.0) * v_sq - G * total_mass / r;
        const double a = -G * total_mass / (2.0 * specific_energy);
        const double hx = y * vz - z * vy, hy = z * vx - x * vz, hz = x * vy - y * vx;
        const double hn = sqrt(hx * hx + hy * hy + hz * hz);
        const double c = v_sq - mu / r, rv = x * vx + y * vy + z * vz;
        const double ex = (c * x - rv * vx) / mu, ey = (c * y - rv * vy) / mu,
                     ez = (c * z - rv * vz) / mu;
        // z . h_unit = 0 hx/|h| + 0 hy/|h| + 1 hz/|h|
        const double cz = 0.0 * (hx / hn) + 0.0 * (hy / hn) + 1.0 * (hz / hn);
        aei[3 * k] = a;
        aei[3 * k + 1] = sqrt(ex * ex + ey * ey + ez * ez);
        aei[3 * k + 2] = acos(cz);
    }
}

// Python's float x % y (the result takes the sign of y).
double py_mod(double x, double y)
{
    double r = fmod(x, y);
    if (r != 0.0) {
        if ((y < 0) != (r < 0)) r += y;
    } else {
        r = copysign(0.0, y);
    }
    return r;
}

}  // namespace

// The chunk loop into the device slab (max_snaps x [positions, velocities,
// a/e/i]); times and energies into ht / he.
static int snapshots_run(int integrator, double t, double t_end, double store_dt, double h,
                         int primary, int max_snaps, double *slab, PrimaryRec *d_pr,
                         std::vector<double> &ht, std::vector<double> &he)
{
    Sim &s = g_sim;
    const int n = (int)s.n;
    const size_t d = 3 * (size_t)n, per = 3 * d;
    const double dt = std::min(store_dt, t_end - t);
    int k = 0;
    while (t < t_end) {
        if (k >= max_snaps) {
            set_error(ABIE_ERR_CAPACITY, "abie_integrate_snapshots: more than %d chunks", max_snaps);
            return ABIE_ERR_CAPACITY;
        }
        const double next_t = t + dt - py_mod(t + dt, dt);
        const int flag = integrator == 0 ? integrator_gr(t, next_t, 1.0) : integrator_wh(t, next_t, h);
        if (flag < 0) return flag;
        t = get_model_time();
        double *sp = slab + (size_t)k * per;
        ABIE_CUDA(cudaMemcpyAsync(sp, s.pos, d * sizeof(double), cudaMemcpyDeviceToDevice, s.st));
        ABIE_CUDA(cudaMemcpyAsync(sp + d, s.vel, d * sizeof(double), cudaMemcpyDeviceToDevice, s.st));
        if (n >= 2) {
            primary_kernel<<<1, PT, 0, s.st>>>(s.pos, s.vel, s.m, n, primary, d_pr);
            const int blocks = std::max(1, std::min((n + 255) / 256, s.num_sms * 8));
            aei_kernel<<<blocks, 256, 0, s.st>>>(s.pos, s.vel, s.m, n, s.G, d_pr, sp + 2 * d);
            ABIE_CUDA(cudaGetLastError());
        } else if (n == 1) {
            const double nan3[3] = {nan(""), nan(""), nan("")};
            ABIE_CUDA(cudaMemcpyAsync(sp + 2 * d, nan3, 3 * sizeof(double), cudaMemcpyHostToDevice, s.st));
            ABIE_CUDA(cudaStreamSynchronize(s.st));
        }
        ht.push_back(t);
        he.push_back(calculate_energy());
        k++;
        if (flag > 0) return flag;  // an event ends the run after its snapshot
    }
    return 0;
}

}  // namespace abie

using namespace abie;

extern "C" {

int abie_integrate_snapshots(int integrator, double t, double t_end, double store_dt, double h,
                             int primary, int max_snaps, double *snap_t, double *snap_pos,
                             double *snap_vel, double *snap_aei, double *snap_energy, int *n_snaps)
{
    Sim &s = g_sim;
    if (n_snaps) *n_snaps = 0;
    if (!s.inited) {
        set_error(ABIE_ERR_NOT_INITIALIZED, "abie_integrate_snapshots before initialize_code");
        return ABIE_ERR_NOT_INITIALIZED;
    }
    const int n = (int)s.n;
    if ((integrator != 0 && integrator != 1) || max_snaps < 0 || !(store_dt > 0.0) ||
        primary < -3 || primary >= n || (integrator == 1 && !(h > 0.0))) {
        set_error(ABIE_ERR_ARGUMENT, "abie_integrate_snapshots: integrator (0 = GR, 1 = WH), "
                  "store_dt, h (WH), primary or max_snaps out of range");
        return ABIE_ERR_ARGUMENT;
    }
    const size_t d = 3 * (size_t)n, per = 3 * d;
    double *slab = nullptr;
    PrimaryRec *d_pr = nullptr;
    if (max_snaps > 0 && d > 0 &&
        cudaMalloc(&slab, (size_t)max_snaps * per * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        set_error(ABIE_ERR_CAPACITY, "abie_integrate_snapshots: %d snapshots of %d bodies do not "
                  "fit in GPU memory", max_snaps, n);
        return ABIE_ERR_CAPACITY;
    }
    if (cudaMalloc(&d_pr, sizeof(PrimaryRec)) != cudaSuccess) {
        if (slab) cudaFree(slab);
        return cuda_fail(cudaGetLastError(), "abie_integrate_snapshots");
    }
    std::vector<double> ht, he;
    int rc = snapshots_run(integrator, t, t_end, store_dt, h, primary, max_snaps, slab, d_pr, ht, he);
    const int k = (int)ht.size();
    cudaError_t ce = cudaStreamSynchronize(s.st);
    // one strided copy per array: [k][positions | velocities | a/e/i] -> [k][3N]
    const size_t row = d * sizeof(double), pitch = per * sizeof(double);
    if (ce == cudaSuccess && k > 0 && d > 0) {
        if (snap_pos && ce == cudaSuccess)
            ce = cudaMemcpy2D(snap_pos, row, slab, pitch, row, k, cudaMemcpyDeviceToHost);
        if (snap_vel && ce == cudaSuccess)
            ce = cudaMemcpy2D(snap_vel, row, slab + d, pitch, row, k, cudaMemcpyDeviceToHost);
        if (snap_aei && ce == cudaSuccess)
            ce = cudaMemcpy2D(snap_aei, row, slab + 2 * d, pitch, row, k, cudaMemcpyDeviceToHost);
    }
    for (int q = 0; q < k; q++) {
        if (snap_t) snap_t[q] = ht[q];
        if (snap_energy) snap_energy[q] = he[q];
    }
    if (slab) cudaFree(slab);
    cudaFree(d_pr);
    if (ce != cudaSuccess) return cuda_fail(ce, "abie_integrate_snapshots copy-out");
    if (n_snaps) *n_snaps = k;
    return rc;
}

}  // extern "C"
