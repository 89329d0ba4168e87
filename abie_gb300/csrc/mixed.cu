// Mixed-precision all-pairs force.
//
// Sources (the massive bodies, compacted in body order) are split by G m:
//   heavy: G m >= theta * max G m (the star of a planetary system) -> the
//          fast FP64 pair term (pair_fast), added straight into FP64 sums;
//   light: everything else -> FP32 pair terms.
// Light pairs use coordinates relative to an FP64 anchor (the first source)
// held as two floats, hi + lo (48 significant bits), so the difference
// (hi_i - hi_j) + (lo_i - lo_j) keeps the separation of close pairs accurate
// to FP32 rounding however far the pair sits from the anchor.  r^-1/2 is
// rsqrtf with one Newton step.  Each thread accumulates a tile of light
// terms in FP32 and folds the tile sum into FP64, so the FP32 sums never run
// over more than one tile (compensated two-level accumulation).
//
// The light pair term runs on Blackwell's packed FP32 instructions
// (add/sub/mul/fma .f32x2: two single-precision operations per lane and
// instruction): one instruction serves a sink against two sources, so a
// pair term costs 12 issued instructions instead of 24.  Each packed
// operation rounds exactly as its scalar counterpart.  The FMA pipe still
// does one lane operation per cycle per lane, so the kernel is bound by
// that pipe (73 % busy on the 16,385-body disk) rather than by issue.
//
// A first pass writes the sources once as anchored two-float coordinates
// and -G m (struct of arrays, +0 marking a heavy source, -0 the padding
// after the last source); the force kernel works in blocks of SINKS x TILE:
// every thread owns MS sinks and reads each source once from shared memory.
// Sources split into chunks across blocks; chunk partial sums are added in
// chunk order by a second pass (deterministic).  Block shape: a sweep on
// the disk (per force call) gave 984 Gint/s for 256 threads x 2 sinks at
// 2 blocks per SM, 966 for 128 x 2 at 5, 961 for 128 x 2 at 4 and 922 for
// 128 x 4 at 3.
#include <algorithm>

#include "mixed.cuh"

namespace abie {

static double g_heavy_fraction = 1e-6;

void mixed_set_heavy_fraction(double f) { g_heavy_fraction = f; }
double mixed_heavy_fraction() { return g_heavy_fraction; }

namespace {

#ifndef ABIE_MIXED_MT
#define ABIE_MIXED_MT 256
#endif
#ifndef ABIE_MIXED_MS
#define ABIE_MIXED_MS 2
#endif
#ifndef ABIE_MIXED_MINB
#define ABIE_MIXED_MINB 2
#endif
constexpr int MT = ABIE_MIXED_MT;  // threads per block
constexpr int MS = ABIE_MIXED_MS;  // sinks per thread
constexpr int MTILE = 128;    // sources per shared-memory tile
constexpr int SINKS_PER_BLOCK = MT * MS;
constexpr int NSOA = 7;       // xh yh zh xl yl zl -Gm
static_assert(MT >= MTILE && MT % 32 == 0, "a tile is loaded by the block's first MTILE threads");

// Two floats in one 64-bit register, the first in the low half.
typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 pk2(float lo, float hi)
{
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(f32x2 v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c)
{
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

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

// The sources as anchored two-float coordinates and -G m, struct of arrays
// of stride entries each: a light source's -G m is negative (-0 if it
// underflows single precision), a heavy source's +0 (its term runs in FP64),
// and the entries after the last source hold zeros with -G m = -0.
__global__ void mixed_sources_kernel(const Src *__restrict__ src, const int *__restrict__ n_src_p,
                                     const unsigned long long *__restrict__ gm_max_bits,
                                     double heavy_fraction, float *__restrict__ soa, int stride)
{
    const int n_src = *n_src_p;
    const double thr = heavy_fraction * __longlong_as_double((long long)*gm_max_bits);
    double ax0 = 0.0, ay0 = 0.0, az0 = 0.0;
    if (n_src > 0) {
        ax0 = src[0].x;
        ay0 = src[0].y;
        az0 = src[0].z;
    }
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < stride; q += gridDim.x * blockDim.x) {
        float xh = 0.0f, yh = 0.0f, zh = 0.0f, xl = 0.0f, yl = 0.0f, zl = 0.0f, ngm = -0.0f;
        if (q < n_src) {
            const Src s = src[q];
            split_df(s.x - ax0, xh, xl);
            split_df(s.y - ay0, yh, yl);
            split_df(s.z - az0, zh, zl);
            ngm = s.gm >= thr ? 0.0f : -__double2float_rn(s.gm);
        }
        soa[q] = xh;
        soa[stride + q] = yh;
        soa[2 * stride + q] = zh;
        soa[3 * stride + q] = xl;
        soa[4 * stride + q] = yl;
        soa[5 * stride + q] = zl;
        soa[6 * stride + q] = ngm;
    }
}

__global__ void __launch_bounds__(MT, ABIE_MIXED_MINB) force_mixed_kernel(
    const double *__restrict__ pos, const double *__restrict__ m, int n,
    const Src *__restrict__ src, const int *__restrict__ n_src_p, const float *__restrict__ soa,
    int stride, int chunks, int per, double *__restrict__ acc, double *__restrict__ partial)
{
    __shared__ __align__(16) float tile[NSOA][MTILE];
    __shared__ unsigned heavy_bits[MTILE / 32];
    const int n_src = *n_src_p;
    const int sink_block = blockIdx.x / chunks;
    const int chunk = blockIdx.x % chunks;
    // anchor: the first source (FP64)
    double ax0 = 0.0, ay0 = 0.0, az0 = 0.0;
    if (n_src > 0) {
        ax0 = src[0].x;
        ay0 = src[0].y;
        az0 = src[0].z;
    }
    // sinks of this thread: anchored two-float coordinates in both halves
    f32x2 HX[MS], HY[MS], HZ[MS], LX[MS], LY[MS], LZ[MS];
    double sx[MS], sy[MS], sz[MS];
#pragma unroll
    for (int k = 0; k < MS; k++) {
        const int j = sink_block * SINKS_PER_BLOCK + k * MT + threadIdx.x;
        const int jj = j < n ? j : (n > 0 ? n - 1 : 0);
        float hx, hy, hz, lx, ly, lz;
        split_df(pos[3 * jj] - ax0, hx, lx);
        split_df(pos[3 * jj + 1] - ay0, hy, ly);
        split_df(pos[3 * jj + 2] - az0, hz, lz);
        HX[k] = pk2(hx, hx);
        HY[k] = pk2(hy, hy);
        HZ[k] = pk2(hz, hz);
        LX[k] = pk2(lx, lx);
        LY[k] = pk2(ly, ly);
        LZ[k] = pk2(lz, lz);
        sx[k] = sy[k] = sz[k] = 0.0;
    }
    // r^2 starts at 1e-20 (a self pair gets a finite r^-3 and a zero term)
    const f32x2 R2MIN = pk2(1e-20f, 1e-20f), MHALF = pk2(-0.5f, -0.5f), THREEHALF = pk2(1.5f, 1.5f);
    const int tiles = (n_src + MTILE - 1) / MTILE;
    const int t0 = chunk * per, t1 = min(tiles, t0 + per);
    for (int t = t0; t < t1; t++) {
        const int base = t * MTILE;
        __syncthreads();  // the previous tile is consumed
        if (threadIdx.x < MTILE) {  // one source per thread of the first MTILE
#pragma unroll
            for (int a = 0; a < NSOA; a++) tile[a][threadIdx.x] = soa[a * stride + base + threadIdx.x];
            const bool heavy = base + (int)threadIdx.x < n_src &&
                               __float_as_uint(tile[6][threadIdx.x]) == 0u;
            const unsigned bal = __ballot_sync(0xffffffffu, heavy);
            if ((threadIdx.x & 31) == 0) heavy_bits[threadIdx.x >> 5] = bal;
        }
        __syncthreads();
        f32x2 FX[MS], FY[MS], FZ[MS];
#pragma unroll
        for (int k = 0; k < MS; k++) FX[k] = FY[k] = FZ[k] = 0ull;  // +0, +0
        // four sources per step (the padding after the last source adds zeros)
        const int cnt = (min(MTILE, n_src - base) + 3) & ~3;
#pragma unroll 1
        for (int q = 0; q < cnt; q += 4) {
            const ulonglong2 XH = *reinterpret_cast<const ulonglong2 *>(&tile[0][q]);
            const ulonglong2 YH = *reinterpret_cast<const ulonglong2 *>(&tile[1][q]);
            const ulonglong2 ZH = *reinterpret_cast<const ulonglong2 *>(&tile[2][q]);
            const ulonglong2 XL = *reinterpret_cast<const ulonglong2 *>(&tile[3][q]);
            const ulonglong2 YL = *reinterpret_cast<const ulonglong2 *>(&tile[4][q]);
            const ulonglong2 ZL = *reinterpret_cast<const ulonglong2 *>(&tile[5][q]);
            const ulonglong2 NG = *reinterpret_cast<const ulonglong2 *>(&tile[6][q]);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const f32x2 xh = h ? XH.y : XH.x, yh = h ? YH.y : YH.x, zh = h ? ZH.y : ZH.x;
                const f32x2 xl = h ? XL.y : XL.x, yl = h ? YL.y : YL.x, zl = h ? ZL.y : ZL.x;
                const f32x2 ng = h ? NG.y : NG.x;
#pragma unroll
                for (int k = 0; k < MS; k++) {
                    const f32x2 dx = add2(sub2(HX[k], xh), sub2(LX[k], xl));
                    const f32x2 dy = add2(sub2(HY[k], yh), sub2(LY[k], yl));
                    const f32x2 dz = add2(sub2(HZ[k], zh), sub2(LZ[k], zl));
                    const f32x2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, R2MIN)));
                    float r2a, r2b;
                    upk2(r2, r2a, r2b);
                    f32x2 y = pk2(rsqrtf(r2a), rsqrtf(r2b));
                    y = mul2(y, fma2(mul2(MHALF, r2), mul2(y, y), THREEHALF));  // one Newton step
                    const f32x2 w = mul2(mul2(ng, mul2(y, y)), y);               // -G m r^-3
                    FX[k] = fma2(w, dx, FX[k]);
                    FY[k] = fma2(w, dy, FY[k]);
                    FZ[k] = fma2(w, dz, FZ[k]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < MS; k++) {
            float a, b;
            upk2(FX[k], a, b);
            sx[k] += (double)(a + b);
            upk2(FY[k], a, b);
            sy[k] += (double)(a + b);
            upk2(FZ[k], a, b);
            sz[k] += (double)(a + b);
        }
        // heavy sources of the tile, in source order, in FP64
#pragma unroll 1
        for (int wq = 0; wq < MTILE / 32; wq++) {
            unsigned bits = heavy_bits[wq];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1u;
                const Src s = src[base + 32 * wq + b];
#pragma unroll
                for (int k = 0; k < MS; k++) {
                    const int j = sink_block * SINKS_PER_BLOCK + k * MT + threadIdx.x;
                    const int jj = j < n ? j : (n > 0 ? n - 1 : 0);
                    pair_fast(pos[3 * jj], pos[3 * jj + 1], pos[3 * jj + 2], s, sx[k], sy[k], sz[k]);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < MS; k++) {
        const int j = sink_block * SINKS_PER_BLOCK + k * MT + threadIdx.x;
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
    if (n <= 0) return 0;
    if (!s.gm_max) ABIE_CUDA(cudaMalloc(&s.gm_max, sizeof(unsigned long long)));
    // n_src <= n stays on the device; the source arrays are sized for n
    const int stride = (n + MTILE - 1) / MTILE * MTILE;
    if ((size_t)NSOA * stride > s.mixed_cap) {
        if (s.mixed_soa) cudaFree(s.mixed_soa);
        s.mixed_soa = nullptr;
        ABIE_CUDA(cudaMalloc(&s.mixed_soa, (size_t)NSOA * stride * sizeof(float)));
        s.mixed_cap = (size_t)NSOA * stride;
    }
    ABIE_CUDA(cudaMemsetAsync(s.gm_max, 0, sizeof(unsigned long long), st));
    max_gm_kernel<<<std::max(1, std::min(152, (n + 255) / 256)), 256, 0, st>>>(src, n_src, s.gm_max);
    ABIE_CUDA(cudaGetLastError());
    mixed_sources_kernel<<<std::max(1, std::min(4 * 152, stride / 256 + 1)), 256, 0, st>>>(
        src, n_src, s.gm_max, g_heavy_fraction, s.mixed_soa, stride);
    ABIE_CUDA(cudaGetLastError());
    const int sink_blocks = (n + SINKS_PER_BLOCK - 1) / SINKS_PER_BLOCK;
    // blocks the current GPU holds at once (host-side queries, no sync)
    int dev = 0, num_sms = 152, bps = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, force_mixed_kernel, MT, 0);
    const int resident = std::max(1, bps) * num_sms;
    // source chunks per sink block: the fewest that reach the least
    // (waves of resident blocks) x (tiles per block), i.e. the shortest
    // launch by whole waves, with no chunk left without tiles and at most
    // about four waves of blocks (the partial sums take 24 bytes per sink
    // and chunk)
    const int tiles = stride / MTILE;
    const int max_chunks = std::min(tiles, std::max(1, (4 * resident + sink_blocks - 1) / sink_blocks));
    int chunks = 1, per = tiles;
    long long best = -1;
    for (int c = 1; c <= max_chunks; c++) {
        const int pc = (tiles + c - 1) / c;
        if ((tiles + pc - 1) / pc != c) continue;
        const long long waves = ((long long)sink_blocks * c + resident - 1) / resident;
        if (best < 0 || waves * pc < best) {
            best = waves * pc;
            chunks = c;
            per = pc;
        }
    }
    if (chunks > 1) {
        size_t need = 3ull * (size_t)n * (size_t)chunks;
        if (need > s.partial_cap) {
            if (s.partial) cudaFree(s.partial);
            s.partial = nullptr;
            ABIE_CUDA(cudaMalloc(&s.partial, need * sizeof(double)));
            s.partial_cap = need;
        }
    }
    force_mixed_kernel<<<sink_blocks * chunks, MT, 0, st>>>(pos, m, n, src, n_src, s.mixed_soa, stride,
                                                             chunks, per, acc, s.partial);
    ABIE_CUDA(cudaGetLastError());
    if (chunks > 1) {
        mixed_sum_chunks_kernel<<<(n + 255) / 256, 256, 0, st>>>(s.partial, m, n, chunks, acc);
        ABIE_CUDA(cudaGetLastError());
    }
    return 0;
}

}  // namespace abie
