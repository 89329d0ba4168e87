// Mixed-precision all-pairs force.
//
// Sources (the massive bodies, compacted in body order) are split by G m:
//   heavy: G m >= theta * max G m (the star of a planetary system) -> the
//          fast FP64 pair term (gm_inv_r3), added straight into FP64 sums;
//   light: everything else -> FP32 pair terms.
// Light pairs use coordinates relative to an FP64 anchor (the first source)
// held as two floats, hi + lo (48 significant bits), so the difference
// (hi_i - hi_j) + (lo_i - lo_j) keeps the separation of close pairs accurate
// to FP32 rounding however far the pair sits from the anchor.  r^-1/2 is
// rsqrtf with one Newton step.  Each thread accumulates a tile of light
// terms in FP32 and folds the tile sum into FP64, so the FP32 sums never run
// over more than one tile (compensated two-level accumulation).
//
// The kernel works in blocks of SINKS x TILE: every thread owns 4 sinks and
// reads each source once from shared memory, so shared-memory traffic is 8
// bytes per interaction.  Sources split into chunks across blocks; chunk
// partial sums are added in chunk order by a second pass (deterministic).
#include <algorithm>

#include "mixed.cuh"

namespace abie {

static double g_heavy_fraction = 1e-6;

void mixed_set_heavy_fraction(double f) { g_heavy_fraction = f; }
double mixed_heavy_fraction() { return g_heavy_fraction; }

namespace {

constexpr int MT = 128;       // threads per block
constexpr int MS = 4;         // sinks per thread
constexpr int MTILE = 128;    // sources per shared-memory tile
constexpr int SINKS_PER_BLOCK = MT * MS;

struct __align__(16) LightSrc {
    float xh, yh, zh, gm;  // gm = 0 for heavy sources (they go through FP64)
    float xl, yl, zl, pad;
};

__device__ __forceinline__ void split_df(double v, float &hi, float &lo)
{
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
}

// max G m over the sources -> *gm_max (as ordered integer bits)
__global__ void max_gm_kernel(const Src *__restrict__ src, const int *__restrict__ n_src_p,
                              unsigned long long *__restrict__ gm_max)
{
    const int n_src = *n_src_p;
    unsigned long long best = 0ull;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n_src; q += gridDim.x * blockDim.x) {
        unsigned long long k = (unsigned long long)__double_as_longlong(src[q].gm);
        best = k > best ? k : best;
    }
    best = warp_max_u64(best);
    if ((threadIdx.x & 31) == 0 && best) atomicMax(gm_max, best);
}

__global__ void __launch_bounds__(MT) force_mixed_kernel(
    const double *__restrict__ pos, const double *__restrict__ m, int n,
    const Src *__restrict__ src, const int *__restrict__ n_src_p,
    const unsigned long long *__restrict__ gm_max_bits, double heavy_fraction, int chunks,
    double *__restrict__ acc, double *__restrict__ partial)
{
    __shared__ LightSrc tile[MTILE];
    __shared__ Src heavy[MTILE];
    __shared__ int n_heavy;
    const int n_src = *n_src_p;
    const int sink_block = blockIdx.x / chunks;
    const int chunk = blockIdx.x % chunks;
    const double thr = heavy_fraction * __longlong_as_double((long long)*gm_max_bits);
    // anchor: the first source (FP64)
    double ax0 = 0.0, ay0 = 0.0, az0 = 0.0;
    if (n_src > 0) {
        ax0 = src[0].x;
        ay0 = src[0].y;
        az0 = src[0].z;
    }
    // sinks of this thread
    int sj[MS];
    double px[MS], py[MS], pz[MS];
    float hx[MS], hy[MS], hz[MS], lx[MS], ly[MS], lz[MS];
    double sx[MS], sy[MS], sz[MS];
#pragma unroll
    for (int k = 0; k < MS; k++) {
        int j = sink_block * SINKS_PER_BLOCK + k * MT + threadIdx.x;
        sj[k] = j;
        int jj = j < n ? j : (n > 0 ? n - 1 : 0);
        px[k] = pos[3 * jj];
        py[k] = pos[3 * jj + 1];
        pz[k] = pos[3 * jj + 2];
        split_df(px[k] - ax0, hx[k], lx[k]);
        split_df(py[k] - ay0, hy[k], ly[k]);
        split_df(pz[k] - az0, hz[k], lz[k]);
        sx[k] = sy[k] = sz[k] = 0.0;
    }
    const int tiles = (n_src + MTILE - 1) / MTILE;
    const int per = (tiles + chunks - 1) / chunks;
    const int t0 = chunk * per, t1 = min(tiles, t0 + per);
    for (int t = t0; t < t1; t++) {
        const int base = t * MTILE;
        __syncthreads();
        if (threadIdx.x == 0) n_heavy = 0;
        __syncthreads();
        {
            const int q = base + threadIdx.x;
            LightSrc L;
            bool is_heavy = false;
            Src s = {0.0, 0.0, 0.0, 0.0};
            if (q < n_src) {
                s = src[q];
                is_heavy = s.gm >= thr;
                split_df(s.x - ax0, L.xh, L.xl);
                split_df(s.y - ay0, L.yh, L.yl);
                split_df(s.z - az0, L.zh, L.zl);
                L.gm = is_heavy ? 0.0f : __double2float_rn(s.gm);
            } else {
                L.xh = L.yh = L.zh = 0.0f;
                L.xl = L.yl = L.zl = 0.0f;
                L.gm = 0.0f;
            }
            L.pad = 0.0f;
            tile[threadIdx.x] = L;
            // heavy sources in source order: warp ballots, then a running base
            unsigned bal = __ballot_sync(0xffffffffu, is_heavy);
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            for (int w = 0; w < MT / 32; w++) {
                __syncthreads();
                if (warp == w && is_heavy)
                    heavy[n_heavy + __popc(bal & ((1u << lane) - 1u))] = s;
                __syncthreads();
                if (warp == w && lane == 0) n_heavy += __popc(bal);
            }
        }
        __syncthreads();
        float fx[MS], fy[MS], fz[MS];
#pragma unroll
        for (int k = 0; k < MS; k++) fx[k] = fy[k] = fz[k] = 0.0f;
        const int cnt = min(MTILE, n_src - base);
#pragma unroll 2
        for (int q = 0; q < cnt; q++) {
            const LightSrc L = tile[q];
#pragma unroll
            for (int k = 0; k < MS; k++) {
                float dx = (hx[k] - L.xh) + (lx[k] - L.xl);
                float dy = (hy[k] - L.yh) + (ly[k] - L.yl);
                float dz = (hz[k] - L.zh) + (lz[k] - L.zl);
                float r2 = fmaxf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)), 1e-20f);
                float y = rsqrtf(r2);
                y = y * fmaf(-0.5f * r2, y * y, 1.5f);  // one Newton step
                float w = L.gm * (y * y) * y;
                fx[k] = fmaf(-w, dx, fx[k]);
                fy[k] = fmaf(-w, dy, fy[k]);
                fz[k] = fmaf(-w, dz, fz[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < MS; k++) {
            sx[k] += (double)fx[k];
            sy[k] += (double)fy[k];
            sz[k] += (double)fz[k];
        }
        for (int q = 0; q < n_heavy; q++) {
            const Src s = heavy[q];
#pragma unroll
            for (int k = 0; k < MS; k++) pair_fast(px[k], py[k], pz[k], s, sx[k], sy[k], sz[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < MS; k++) {
        const int j = sj[k];
        if (j >= n) continue;
        if (chunks == 1) {
            if (m[j] < 0.0) continue;
            acc[3 * j] = sx[k];
            acc[3 * j + 1] = sy[k];
            acc[3 * j + 2] = sz[k];
        } else {
            double *p = partial + 3 * ((long long)j * chunks + chunk);
            p[0] = sx[k];
            p[1] = sy[k];
            p[2] = sz[k];
        }
    }
}

__global__ void mixed_sum_chunks_kernel(const double *__restrict__ partial,
                                        const double *__restrict__ m, int n, int chunks,
                                        double *__restrict__ acc)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n || m[j] < 0.0) return;
    const double *p = partial + 3ll * j * chunks;
    double ax = p[0], ay = p[1], az = p[2];
    for (int c = 1; c < chunks; c++) {
        ax += p[3 * c];
        ay += p[3 * c + 1];
        az += p[3 * c + 2];
    }
    acc[3 * j] = ax;
    acc[3 * j + 1] = ay;
    acc[3 * j + 2] = az;
}

}  // namespace

int launch_force_mixed(const double *pos, const double *m, int n, double G, ForceScratch &s,
                       double *acc, cudaStream_t st)
{
    (void)G;
    // s.src / s.n_src were filled by launch_force's compaction
    return launch_force_mixed_src(pos, m, n, s.src, s.n_src, s, acc, st);
}

int launch_force_mixed_src(const double *pos, const double *m, int n, const Src *src,
                           const int *n_src, ForceScratch &s, double *acc, cudaStream_t st)
{
    if (!s.gm_max) ABIE_CUDA(cudaMalloc(&s.gm_max, sizeof(unsigned long long)));
    ABIE_CUDA(cudaMemsetAsync(s.gm_max, 0, sizeof(unsigned long long), st));
    max_gm_kernel<<<std::max(1, std::min(152, (n + 255) / 256)), 256, 0, st>>>(src, n_src, s.gm_max);
    ABIE_CUDA(cudaGetLastError());
    const int sink_blocks = (n + SINKS_PER_BLOCK - 1) / SINKS_PER_BLOCK;
    int num_sms = 152;
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, 0);
    // enough blocks to fill the GPU several times; each chunk at least a tile
    const int tiles = (n + MTILE - 1) / MTILE;
    int chunks = std::max(1, std::min(tiles, (8 * num_sms + sink_blocks - 1) / sink_blocks));
    if (chunks > 1) {
        size_t need = 3ull * (size_t)n * (size_t)chunks;
        if (need > s.partial_cap) {
            if (s.partial) cudaFree(s.partial);
            s.partial = nullptr;
            ABIE_CUDA(cudaMalloc(&s.partial, need * sizeof(double)));
            s.partial_cap = need;
        }
    }
    force_mixed_kernel<<<sink_blocks * chunks, MT, 0, st>>>(pos, m, n, src, n_src, s.gm_max,
                                                             g_heavy_fraction, chunks, acc, s.partial);
    ABIE_CUDA(cudaGetLastError());
    if (chunks > 1) {
        mixed_sum_chunks_kernel<<<(n + 255) / 256, 256, 0, st>>>(s.partial, m, n, chunks, acc);
        ABIE_CUDA(cudaGetLastError());
    }
    return 0;
}

}  // namespace abie
