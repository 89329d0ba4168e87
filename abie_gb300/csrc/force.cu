// All-pairs Newtonian acceleration kernels (sm_103a).
//
//   exact : one thread per sink, sources visited in body order with the
//           reference's operations (sqrt, r*r2, (gm*d)/r3), so every
//           acceleration is bit-identical to src/common.c:39-77.
//   fp64  : the production FP64 form.  A group of 1, 8 or 32 lanes shares a
//           sink and splits its sources; partial sums meet in a fixed
//           butterfly of warp shuffles, so results are deterministic.  The
//           pair term is pair_fast() (6 FP64 operations per interaction).
//           Below 8,192 sinks, sinks are handed out to lane groups from an
//           atomic counter (force_fp64_dyn_kernel); from 8,192 sinks each
//           sink's sources split into two chunks, one lane group per (sink,
//           chunk) on a static grid (force_fp64_kernel), and a second pass
//           adds the chunks' partial sums in chunk order.  When every body
//           is massive (8,192 .. 131,072 bodies) the symmetric form
//           (force_sym_kernel) evaluates each pair once for both bodies.
//   naive : one thread per sink over global memory with rsqrt, the
//           semantics of the reference's GPU offload (src/gpuforce.cu:61-84):
//           sources with m == 0 and coincident pairs are skipped, sinks and
//           sources with m < 0 are not.
//   mixed : in mixed.cu.
#include <algorithm>
#include <vector>

#include "force.cuh"
#include "pn.cuh"
#include "mixed.cuh"

namespace abie {

static ForceShape g_shape_override = {0, 0};

void force_shape_override(int lanes_per_sink, int chunks)
{
    g_shape_override.lanes_per_sink = lanes_per_sink;
    g_shape_override.chunks = chunks;
}

int force_scratch_reserve(ForceScratch &s, size_t n)
{
    if (n <= s.cap && s.src) return 0;
    force_scratch_free(s);
    size_t cap = n < 1024 ? 1024 : n;
    ABIE_CUDA(cudaMalloc(&s.src, cap * sizeof(Src)));
    ABIE_CUDA(cudaMalloc(&s.src_body, cap * sizeof(int)));
    ABIE_CUDA(cudaMalloc(&s.n_src, sizeof(int)));
    ABIE_CUDA(cudaMalloc(&s.next, sizeof(unsigned int)));
    ABIE_CUDA(cudaMalloc(&s.counts, ((cap + 2047) / 2048) * sizeof(int)));
    s.cap = cap;
    return 0;
}

void force_scratch_free(ForceScratch &s)
{
    if (s.src) cudaFree(s.src);
    if (s.src_body) cudaFree(s.src_body);
    if (s.n_src) cudaFree(s.n_src);
    if (s.partial) cudaFree(s.partial);
    if (s.gm_max) cudaFree(s.gm_max);
    if (s.mixed_soa) cudaFree(s.mixed_soa);
    if (s.next) cudaFree(s.next);
    if (s.counts) cudaFree(s.counts);
    if (s.sym_items) cudaFree(s.sym_items);
    if (s.sym_row) cudaFree(s.sym_row);
    if (s.sym_apart) cudaFree(s.sym_apart);
    if (s.sym_bpart) cudaFree(s.sym_bpart);
    s = ForceScratch();
}

// ---------------------------------------------------------------------------
// Order-preserving compaction of the massive bodies, one block.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) compact_sources_kernel(const double *__restrict__ pos,
                                                               const double *__restrict__ m, int n,
                                                               double G, Src *__restrict__ src,
                                                               int *__restrict__ src_body,
                                                               int *__restrict__ n_src)
{
    __shared__ int warp_count[32];
    __shared__ int base_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) base_s = 0;
    __syncthreads();
    for (int off = 0; off < n; off += blockDim.x) {
        int i = off + threadIdx.x;
        bool keep = (i < n) && (m[i] > 0.0);
        unsigned ballot = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) warp_count[warp] = __popc(ballot);
        __syncthreads();
        int before = 0;
        for (int w = 0; w < warp; w++) before += warp_count[w];
        int base = base_s;
        if (keep) {
            int slot = base + before + __popc(ballot & ((1u << lane) - 1u));
            Src s;
            s.x = pos[3 * i];
            s.y = pos[3 * i + 1];
            s.z = pos[3 * i + 2];
            s.gm = G * m[i];
            src[slot] = s;
            src_body[slot] = i;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += warp_count[w];
            base_s = base + tot;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *n_src = base_s;
}

int launch_compact_sources(const double *pos, const double *m, int n, double G, Src *src,
                           int *src_body, int *n_src, cudaStream_t st)
{
    compact_sources_kernel<<<1, 1024, 0, st>>>(pos, m, n, G, src, src_body, n_src);
    ABIE_CUDA(cudaGetLastError());
    return 0;
}

// Parallel form: chunks of CCH bodies, one block each.  Pass 1 counts the
// massive bodies of every chunk; pass 2 gives each block its offset (the
// sum of the earlier chunks' counts) and compacts its chunk in order, so
// the list equals compact_sources_kernel's.
constexpr int CCH = 2048;

__device__ __forceinline__ int block_sum_256(int v, int *ws)
{
    v = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) t += ws[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(256) count_sources_kernel(const double *__restrict__ m, int n,
                                                            int *__restrict__ counts)
{
    __shared__ int ws[8];
    const int base = blockIdx.x * CCH, end = min(n, base + CCH);
    int c = 0;
    for (int i = base + threadIdx.x; i < end; i += 256) c += m[i] > 0.0 ? 1 : 0;
    c = block_sum_256(c, ws);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

__global__ void __launch_bounds__(256) scatter_sources_kernel(const double *__restrict__ pos,
                                                              const double *__restrict__ m, int n,
                                                              double G, const int *__restrict__ counts,
                                                              Src *__restrict__ src,
                                                              int *__restrict__ src_body,
                                                              int *__restrict__ n_src)
{
    __shared__ int ws[8];
    __shared__ int wc[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int part = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += 256) part += counts[b];
    int base = block_sum_256(part, ws);
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *n_src = base + counts[blockIdx.x];
    const int start = blockIdx.x * CCH, end = min(n, start + CCH);
    for (int off = start; off < end; off += 256) {
        const int i = off + threadIdx.x;
        const bool keep = i < end && m[i] > 0.0;
        const unsigned ballot = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) wc[warp] = __popc(ballot);
        __syncthreads();
        int before = 0, tot = 0;
#pragma unroll
        for (int w = 0; w < 8; w++) {
            before += w < warp ? wc[w] : 0;
            tot += wc[w];
        }
        if (keep) {
            const int slot = base + before + __popc(ballot & ((1u << lane) - 1u));
            Src s;
            s.x = pos[3 * i];
            s.y = pos[3 * i + 1];
            s.z = pos[3 * i + 2];
            s.gm = G * m[i];
            src[slot] = s;
            src_body[slot] = i;
        }
        base += tot;
        __syncthreads();
    }
}

int launch_compact_sources_parallel(const double *pos, const double *m, int n, double G, Src *src,
                                    int *src_body, int *n_src, int *counts, cudaStream_t st)
{
    if (n <= 4096 || !counts) return launch_compact_sources(pos, m, n, G, src, src_body, n_src, st);
    const int nb = (n + CCH - 1) / CCH;
    count_sources_kernel<<<nb, 256, 0, st>>>(m, n, counts);
    scatter_sources_kernel<<<nb, 256, 0, st>>>(pos, m, n, G, counts, src, src_body, n_src);
    ABIE_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// exact
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) force_exact_kernel(const double *__restrict__ pos,
                                                          const double *__restrict__ m, int n,
                                                          const Src *__restrict__ src,
                                                          const int *__restrict__ src_body,
                                                          const int *__restrict__ n_src_p,
                                                          double *__restrict__ acc)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    if (m[j] < 0.0) return;
    const int n_src = *n_src_p;
    double xj = pos[3 * j], yj = pos[3 * j + 1], zj = pos[3 * j + 2];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int q = 0; q < n_src; q++) {
        if (src_body[q] == j) continue;
        pair_exact(xj, yj, zj, src[q], ax, ay, az);
    }
    acc[3 * j] = ax;
    acc[3 * j + 1] = ay;
    acc[3 * j + 2] = az;
}

// ---------------------------------------------------------------------------
// fp64
// ---------------------------------------------------------------------------
// Tuning knobs of the chunked form: blocks per SM the registers are sized
// for, sources per loop iteration.  Measured on the 16,385- and 32,769-body
// disks with 32 lanes per sink and 2 source chunks (Gint/s): (1, 4) 85.3 /
// 86.7, (3, 2) 87.7 / 89.2, (4, 2) 90.5 / 92.1, (5, 2) 91.6 / 93.2, (4, 4)
// 91.9 / 93.4 (kept: 64 registers, 32 warps per SM).
#ifndef ABIE_FORCE_S_MINB
#define ABIE_FORCE_S_MINB 4
#endif
#ifndef ABIE_FORCE_S_UNROLL
#define ABIE_FORCE_S_UNROLL 4
#endif
template <int JS>
__global__ void __launch_bounds__(256, ABIE_FORCE_S_MINB) force_fp64_kernel(const double *__restrict__ pos,
                                                         const double *__restrict__ m, int n,
                                                         const Src *__restrict__ src,
                                                         const int *__restrict__ n_src_p,
                                                         int chunks, double *__restrict__ acc,
                                                         double *__restrict__ partial,
                                                         bool sym_launched = false)
{
    // the symmetric form took this call (every body massive)
    if (sym_launched && *n_src_p == n) return;
    const int groups_per_block = 256 / JS;
    const long long group = (long long)blockIdx.x * groups_per_block + threadIdx.x / JS;
    const int lane = threadIdx.x % JS;
    const int n_src = *n_src_p;
    const long long n_groups = (long long)n * chunks;
    const bool live = group < n_groups;
    const int j = live ? (int)(group / chunks) : 0;
    const int c = live ? (int)(group % chunks) : 0;
    const int per = (n_src + chunks - 1) / chunks;
    const int q0 = c * per;
    const int q1 = min(n_src, q0 + per);
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (live) {
        const double xj = pos[3 * j], yj = pos[3 * j + 1], zj = pos[3 * j + 2];
        int q = q0 + lane;
        constexpr int U = ABIE_FORCE_S_UNROLL;
#pragma unroll 1
        for (; q + (U - 1) * JS < q1; q += U * JS) {
            Src sv[U];
#pragma unroll
            for (int u = 0; u < U; u++) sv[u] = src[q + u * JS];
#pragma unroll
            for (int u = 0; u < U; u++) pair_fast(xj, yj, zj, sv[u], ax, ay, az);
        }
        for (; q < q1; q += JS) pair_fast(xj, yj, zj, src[q], ax, ay, az);
    }
    if (JS > 1) {
#pragma unroll
        for (int o = JS / 2; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o, JS);
            ay += __shfl_xor_sync(0xffffffffu, ay, o, JS);
            az += __shfl_xor_sync(0xffffffffu, az, o, JS);
        }
    }
    if (!live || lane != 0) return;
    if (chunks == 1) {
        if (m[j] < 0.0) return;
        acc[3 * j] = ax;
        acc[3 * j + 1] = ay;
        acc[3 * j + 2] = az;
    } else {
        double *p = partial + 3 * group;
        p[0] = ax;
        p[1] = ay;
        p[2] = az;
    }
}

// Persistent form: a grid that fills the GPU once, lane groups take sinks
// from an atomic counter (*next must be zero at launch).  Tuning knobs:
// blocks per SM the registers are sized for, sources per loop iteration.
// Measured on the 16,385-body disk (ms per launch): (1, 4) 3.233, (3, 4)
// 3.052, (4, 4) 3.039, (1, 2) 3.155, (4, 2) 3.076, (5, 2) 3.021, (1, 8)
// 3.150; (5, 2) keeps 48 registers for 40 warps per SM.
#ifndef ABIE_FORCE_MINB
#define ABIE_FORCE_MINB 5
#endif
#ifndef ABIE_FORCE_UNROLL
#define ABIE_FORCE_UNROLL 2
#endif
template <int JS>
__global__ void __launch_bounds__(256, ABIE_FORCE_MINB) force_fp64_dyn_kernel(const double *__restrict__ pos,
                                                             const double *__restrict__ m, int n,
                                                             const Src *__restrict__ src,
                                                             const int *__restrict__ n_src_p,
                                                             double *__restrict__ acc,
                                                             unsigned int *__restrict__ next)
{
    const int lane = threadIdx.x % JS;
    const int gl = threadIdx.x / JS;  // group within the block
    const int n_src = *n_src_p;
    const unsigned mask = JS == 32 ? 0xffffffffu : (((1u << JS) - 1u) << ((threadIdx.x & 31) / JS * JS));
    for (;;) {
        int j = 0;
        if (lane == 0) j = (int)atomicAdd(next, 1u);
        j = __shfl_sync(mask, j, (threadIdx.x & 31) / JS * JS);
        if (j >= n) break;
        const double xj = pos[3 * j], yj = pos[3 * j + 1], zj = pos[3 * j + 2];
        double ax = 0.0, ay = 0.0, az = 0.0;
        int q = lane;
        constexpr int U = ABIE_FORCE_UNROLL;
#pragma unroll 1
        for (; q + (U - 1) * JS < n_src; q += U * JS) {
            Src sv[U];
#pragma unroll
            for (int u = 0; u < U; u++) sv[u] = src[q + u * JS];
#pragma unroll
            for (int u = 0; u < U; u++) pair_fast(xj, yj, zj, sv[u], ax, ay, az);
        }
        for (; q < n_src; q += JS) pair_fast(xj, yj, zj, src[q], ax, ay, az);
        if (JS > 1) {
#pragma unroll
            for (int o = JS / 2; o > 0; o >>= 1) {
                ax += __shfl_xor_sync(mask, ax, o, JS);
                ay += __shfl_xor_sync(mask, ay, o, JS);
                az += __shfl_xor_sync(mask, az, o, JS);
            }
        }
        if (lane == 0 && m[j] >= 0.0) {
            acc[3 * j] = ax;
            acc[3 * j + 1] = ay;
            acc[3 * j + 2] = az;
        }
    }
    (void)gl;
}

// ---------------------------------------------------------------------------
// Symmetric form, for systems whose bodies are all massive (from 8,192
// bodies): every unordered pair is evaluated once, for both of its bodies.
// The separation, r^2 and r^-3 are shared; the two G m r^-3 factors differ
// only in the mass (inv_r3_core once, gm_times_inv_r3 twice), so a pair
// costs 3 separations and 6 accumulating FMAs: 4.5 FP64 instructions per
// interaction against 6, and half the integer work.
//
// Bodies are tiled by 32.  A warp takes a work item -- tile I (its lanes'
// sinks) and SYM_K source tiles J >= I -- from an atomic counter, stages
// each source tile in shared memory and walks it as a ring: at step s lane
// t pairs sink 32 I + t with body 32 J + (t + s) % 32, adds the sink's term
// to its own sum and the body's to a ring sum that moves one lane down per
// step, so after 32 steps lane t holds the sum for body 32 J + t.  The
// diagonal tile (J = I) is summed one way only.  Each item writes its
// sinks' partial sums and one partial sum per source tile; a second pass
// adds, for every body, the partials of its own row's items and of the
// items of the rows above that hold its tile, in a fixed order.
#ifndef ABIE_SYM_K
#define ABIE_SYM_K 2
#endif
#ifndef ABIE_SYM_MINB
#define ABIE_SYM_MINB 4
#endif
#ifndef ABIE_SYM_UNROLL
#define ABIE_SYM_UNROLL 2
#endif
constexpr int SYM_K = ABIE_SYM_K;  // source tiles per work item
constexpr int SYM_UNROLL = ABIE_SYM_UNROLL;  // ring steps per loop iteration
// Partial sums take n^2 / 32 x 12 bytes (6.4 GB at 131,072 bodies); above
// that the chunked form runs.
constexpr int SYM_MAX_BODIES = 131072;

__global__ void __launch_bounds__(256, ABIE_SYM_MINB) force_sym_kernel(const Src *__restrict__ src, int n,
                                                           const int2 *__restrict__ items, int n_items,
                                                           int nt, double *__restrict__ apart,
                                                           double *__restrict__ bpart,
                                                           unsigned int *__restrict__ next,
                                                           const int *__restrict__ n_src_p)
{
    __shared__ double tile[8][32][4];  // one staged source tile per warp
    if (*n_src_p != n) return;  // some body is not massive: the chunked form runs instead
    const int lane = threadIdx.x & 31;
    double(*T)[4] = tile[threadIdx.x >> 5];
    for (;;) {
        int it = 0;
        if (lane == 0) it = (int)atomicAdd(next, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= n_items) break;
        const int2 item = items[it];
        const int I = item.x, J0 = item.y, J1 = min(nt, J0 + SYM_K);
        const int i = 32 * I + lane;
        const bool vi = i < n;
        const Src si = vi ? src[i] : Src{0.0, 0.0, 0.0, 1.0};
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (int J = J0; J < J1; J++) {
            const int j = 32 * J + lane;
            const bool vj = j < n;
            const Src sj = vj ? src[j] : Src{0.0, 0.0, 0.0, 0.0};
            __syncwarp();
            T[lane][0] = sj.x;
            T[lane][1] = sj.y;
            T[lane][2] = sj.z;
            T[lane][3] = sj.gm;  // 0 for a missing body: no term
            __syncwarp();
            if (J == I) {
#pragma unroll 1
                for (int s = 1; s < 32; s++) {
                    const int k = (lane + s) & 31;
                    const double gmk = T[k][3];
                    const double dx = si.x - T[k][0], dy = si.y - T[k][1], dz = si.z - T[k][2];
                    unsigned long long Mr, Wn;
                    int Er, eW;
                    r2_int(dx, dy, dz, Mr, Er);
                    inv_r3_core(Mr, Er, Wn, eW);
                    const double wi = __double_as_longlong(gmk) > 0 ? gm_times_inv_r3(Wn, eW, gmk) : 0.0;
                    ax = fma(-wi, dx, ax);
                    ay = fma(-wi, dy, ay);
                    az = fma(-wi, dz, az);
                }
            } else {
                double bx = 0.0, by = 0.0, bz = 0.0;
#pragma unroll SYM_UNROLL
                for (int s = 0; s < 32; s++) {
                    const int k = (lane + s) & 31;
                    const double gmk = T[k][3];
                    const double dx = si.x - T[k][0], dy = si.y - T[k][1], dz = si.z - T[k][2];
                    unsigned long long Mr, Wn;
                    int Er, eW;
                    r2_int(dx, dy, dz, Mr, Er);
                    inv_r3_core(Mr, Er, Wn, eW);
                    const double wi = __double_as_longlong(gmk) > 0 ? gm_times_inv_r3(Wn, eW, gmk) : 0.0;
                    const double wj = vi ? gm_times_inv_r3(Wn, eW, si.gm) : 0.0;
                    ax = fma(-wi, dx, ax);
                    ay = fma(-wi, dy, ay);
                    az = fma(-wi, dz, az);
                    bx = fma(wj, dx, bx);
                    by = fma(wj, dy, by);
                    bz = fma(wj, dz, bz);
                    bx = __shfl_sync(0xffffffffu, bx, (lane + 1) & 31);
                    by = __shfl_sync(0xffffffffu, by, (lane + 1) & 31);
                    bz = __shfl_sync(0xffffffffu, bz, (lane + 1) & 31);
                }
                double *bp = bpart + (((long long)it * SYM_K + (J - J0)) * 32 + lane) * 3;
                bp[0] = bx;
                bp[1] = by;
                bp[2] = bz;
            }
        }
        double *ap = apart + ((long long)it * 32 + lane) * 3;
        ap[0] = ax;
        ap[1] = ay;
        ap[2] = az;
    }
}

// acc of the bodies of tile J (one block): their row's item partials and
// the partials the rows above left for tile J, spread over the block's
// SYM_RW warps (warp w takes every SYM_RW-th term) and the warps' sums
// added in warp order, so the order is fixed.
constexpr int SYM_RW = 32;
__global__ void __launch_bounds__(32 * SYM_RW) sym_reduce_kernel(const double *__restrict__ apart,
                                                         const double *__restrict__ bpart,
                                                         const int *__restrict__ row_item, int n,
                                                         double *__restrict__ acc,
                                                         const int *__restrict__ n_src_p)
{
    __shared__ double part[SYM_RW][32][3];
    if (*n_src_p != n) return;
    const int J = blockIdx.x, t = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int a0 = row_item[J], na = row_item[J + 1] - a0;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int k = w; k < na + J; k += SYM_RW) {
        const double *p;
        if (k < na) {
            p = apart + ((long long)(a0 + k) * 32 + t) * 3;
        } else {
            const int I = k - na;
            const int it = row_item[I] + (J - I) / SYM_K, jj = (J - I) % SYM_K;
            p = bpart + (((long long)it * SYM_K + jj) * 32 + t) * 3;
        }
        ax += p[0];
        ay += p[1];
        az += p[2];
    }
    part[w][t][0] = ax;
    part[w][t][1] = ay;
    part[w][t][2] = az;
    __syncthreads();
    const int j = 32 * J + t;
    if (w == 0 && j < n) {
        double sx = part[0][t][0], sy = part[0][t][1], sz = part[0][t][2];
#pragma unroll 8
        for (int q = 1; q < SYM_RW; q++) {
            sx += part[q][t][0];
            sy += part[q][t][1];
            sz += part[q][t][2];
        }
        acc[3 * j] = sx;
        acc[3 * j + 1] = sy;
        acc[3 * j + 2] = sz;
    }
}

__global__ void sum_chunks_kernel(const double *__restrict__ partial, const double *__restrict__ m,
                                  int n, int chunks, double *__restrict__ acc,
                                  const int *__restrict__ n_src_p = nullptr)
{
    if (n_src_p && *n_src_p == n) return;  // the symmetric form took this call
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

// ---------------------------------------------------------------------------
// naive (src/gpuforce.cu:61-84 semantics)
// ---------------------------------------------------------------------------
__global__ void force_naive_kernel(const double *__restrict__ pos, const double *__restrict__ m,
                                   double G, int n, double *__restrict__ acc)
{
    int i = blockDim.x * blockIdx.x + threadIdx.x;
    if (i >= n) return;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int j = 0; j < n; j++) {
        double mj = m[j];
        if (i == j || mj == 0) continue;
        double dx = pos[3 * i] - pos[3 * j];
        double dy = pos[3 * i + 1] - pos[3 * j + 1];
        double dz = pos[3 * i + 2] - pos[3 * j + 2];
        double d2 = dx * dx + dy * dy + dz * dz;
        if (d2 == 0.0) continue;
        double inv = rsqrt(d2);
        double inv3 = inv * inv * inv;
        fx -= G * mj * dx * inv3;
        fy -= G * mj * dy * inv3;
        fz -= G * mj * dz * inv3;
    }
    acc[3 * i] = fx;
    acc[3 * i + 1] = fy;
    acc[3 * i + 2] = fz;
}

ForceShape force_shape_default(int n_sink, int n_src)
{
    if (g_shape_override.lanes_per_sink > 0) {
        ForceShape s;
        s.lanes_per_sink = g_shape_override.lanes_per_sink;
        s.chunks = g_shape_override.chunks > 0 ? g_shape_override.chunks : 1;
        return s;
    }
    return force_shape_auto(n_sink, n_src);
}

ForceShape force_shape_auto(int n_sink, int n_src)
{
    ForceShape s;
    s.lanes_per_sink = n_src <= 64 ? 1 : (n_src <= 1024 ? 8 : 32);
    // from 8,192 sinks two source chunks per sink (partial sums added in
    // chunk order): finer work items than the sink queue's and fewer idle
    // SMs at the end; on the disks of 8,193 / 16,385 / 32,769 / 65,537
    // bodies 85.3 / 91.7 / 93.2 / 94.0 Gint/s against 84.5 / 89.5 / 87.6 /
    // 92.2 for one chunk from the sink queue
    s.chunks = (s.lanes_per_sink == 32 && n_sink >= 8192) ? 2 : 1;
    return s;
}

int launch_force_published(const double *pos, const double *m, int n, const Src *src,
                           const int *n_src_dev, int lanes, double *acc, unsigned int *next,
                           cudaStream_t st, double *partial)
{
    if (n <= 0) return 0;
    if (partial && lanes == 32) {
        // two source chunks per sink on a static grid, then the chunk sum
        const long long groups = 2ll * n;
        const int blocks = (int)((groups + 7) / 8);
        force_fp64_kernel<32><<<blocks, 256, 0, st>>>(pos, m, n, src, n_src_dev, 2, acc, partial);
        sum_chunks_kernel<<<(n + 255) / 256, 256, 0, st>>>(partial, m, n, 2, acc);
        ABIE_CUDA(cudaGetLastError());
        return 0;
    }
    int dev = 0, sms = 152, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const void *fn = lanes == 1 ? (const void *)force_fp64_dyn_kernel<1>
                     : lanes == 8 ? (const void *)force_fp64_dyn_kernel<8>
                                  : (const void *)force_fp64_dyn_kernel<32>;
    ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, 256, 0));
    const long long want = ((long long)n * lanes + 255) / 256;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((long long)sms * std::max(bps, 1), want));
    ABIE_CUDA(cudaMemsetAsync(next, 0, sizeof(unsigned int), st));
    if (lanes == 1) force_fp64_dyn_kernel<1><<<blocks, 256, 0, st>>>(pos, m, n, src, n_src_dev, acc, next);
    else if (lanes == 8) force_fp64_dyn_kernel<8><<<blocks, 256, 0, st>>>(pos, m, n, src, n_src_dev, acc, next);
    else force_fp64_dyn_kernel<32><<<blocks, 256, 0, st>>>(pos, m, n, src, n_src_dev, acc, next);
    ABIE_CUDA(cudaGetLastError());
    return 0;
}

bool force_shape_overridden() { return g_shape_override.lanes_per_sink > 0; }

// Work items of the symmetric form for n bodies: row I, first source tile
// J0, row by row; row_item[I] = the first item of row I.  Partial sums:
// 32 x 3 per item (its sinks), 32 x 3 x SYM_K per item (its source tiles).
int sym_reserve(ForceScratch &s, int n)
{
    if (s.sym_n == n && s.sym_items) return 0;
    const int nt = (n + 31) / 32;
    std::vector<int2> items;
    std::vector<int> row(nt + 1);
    for (int I = 0; I < nt; I++) {
        row[I] = (int)items.size();
        for (int J0 = I; J0 < nt; J0 += SYM_K) items.push_back(make_int2(I, J0));
    }
    row[nt] = (int)items.size();
    if (s.sym_items) cudaFree(s.sym_items);
    if (s.sym_row) cudaFree(s.sym_row);
    if (s.sym_apart) cudaFree(s.sym_apart);
    if (s.sym_bpart) cudaFree(s.sym_bpart);
    s.sym_items = nullptr;
    s.sym_row = nullptr;
    s.sym_apart = s.sym_bpart = nullptr;
    s.sym_n = 0;
    const size_t ni = items.size();
    ABIE_CUDA(cudaMalloc(&s.sym_items, ni * sizeof(int2)));
    ABIE_CUDA(cudaMalloc(&s.sym_row, (nt + 1) * sizeof(int)));
    ABIE_CUDA(cudaMalloc(&s.sym_apart, ni * 32 * 3 * sizeof(double)));
    ABIE_CUDA(cudaMalloc(&s.sym_bpart, ni * SYM_K * 32 * 3 * sizeof(double)));
    ABIE_CUDA(cudaMemcpy(s.sym_items, items.data(), ni * sizeof(int2), cudaMemcpyHostToDevice));
    ABIE_CUDA(cudaMemcpy(s.sym_row, row.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice));
    s.sym_n = n;
    s.sym_nt = nt;
    s.sym_items_n = (int)ni;
    return 0;
}

int launch_force_published_sym(const Src *src, int n, const int *n_src_dev, double *acc,
                               ForceScratch &s, cudaStream_t st)
{
    int rc = force_scratch_reserve(s, (size_t)n);
    if (rc) return rc;
    rc = sym_reserve(s, n);
    if (rc) return rc;
    int dev = 0, sms = 152, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, force_sym_kernel, 256, 0));
    const int blocks = (int)std::max<long long>(
        1, std::min<long long>((long long)sms * std::max(bps, 1), ((long long)s.sym_items_n + 7) / 8));
    ABIE_CUDA(cudaMemsetAsync(s.next, 0, sizeof(unsigned int), st));
    force_sym_kernel<<<blocks, 256, 0, st>>>(src, n, s.sym_items, s.sym_items_n, s.sym_nt,
                                             s.sym_apart, s.sym_bpart, s.next, n_src_dev);
    sym_reduce_kernel<<<s.sym_nt, 32 * SYM_RW, 0, st>>>(s.sym_apart, s.sym_bpart, s.sym_row, n, acc,
                                                         n_src_dev);
    ABIE_CUDA(cudaGetLastError());
    return 0;
}

bool force_sym_applies(int n, int n_src)
{
    return n_src == n && n >= 8192 && n <= SYM_MAX_BODIES && !force_shape_overridden();
}

int launch_force(int mode, const double *pos, const double *m, int n, double G, ForceScratch &s,
                 double *acc, cudaStream_t st)
{
    if (n <= 0) return 0;
    if (mode == ABIE_FORCE_NAIVE) {
        force_naive_kernel<<<(n + 255) / 256, 256, 0, st>>>(pos, m, G, n, acc);
        ABIE_CUDA(cudaGetLastError());
        return 0;
    }
    int rc = force_scratch_reserve(s, (size_t)n);
    if (rc) return rc;
    rc = launch_compact_sources_parallel(pos, m, n, G, s.src, s.src_body, s.n_src, s.counts, st);
    if (rc) return rc;
    if (mode == ABIE_FORCE_EXACT) {
        force_exact_kernel<<<(n + 255) / 256, 256, 0, st>>>(pos, m, n, s.src, s.src_body, s.n_src,
                                                            acc);
        ABIE_CUDA(cudaGetLastError());
        return 0;
    }
    if (mode == ABIE_FORCE_MIXED) return launch_force_mixed(pos, m, n, G, s, acc, st);
    // fp64: the number of sources is on the device; the shape uses n as its
    // upper bound.
    ForceShape sh = force_shape_default(n, n);
    bool sym = false;
    if (sh.lanes_per_sink == 32 && sh.chunks == 2 && !force_shape_overridden() &&
        n <= SYM_MAX_BODIES) {
        // the symmetric form; its kernels (and the chunked ones below) see
        // on the device whether every body is massive and only one of them
        // does the work
        int rc2 = sym_reserve(s, n);
        if (rc2) return rc2;
        int dev = 0, sms = 152, bps = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, force_sym_kernel, 256, 0));
        const int blocks = (int)std::max<long long>(
            1, std::min<long long>((long long)sms * std::max(bps, 1), ((long long)s.sym_items_n + 7) / 8));
        ABIE_CUDA(cudaMemsetAsync(s.next, 0, sizeof(unsigned int), st));
        force_sym_kernel<<<blocks, 256, 0, st>>>(s.src, n, s.sym_items, s.sym_items_n, s.sym_nt,
                                                 s.sym_apart, s.sym_bpart, s.next, s.n_src);
        sym_reduce_kernel<<<s.sym_nt, 32 * SYM_RW, 0, st>>>(s.sym_apart, s.sym_bpart, s.sym_row, n,
                                                             acc, s.n_src);
        ABIE_CUDA(cudaGetLastError());
        sym = true;
    }
    if (sh.chunks > 1) {
        size_t need = 3ull * (size_t)n * (size_t)sh.chunks;
        if (need > s.partial_cap) {
            if (s.partial) cudaFree(s.partial);
            s.partial = nullptr;
            ABIE_CUDA(cudaMalloc(&s.partial, need * sizeof(double)));
            s.partial_cap = need;
        }
    }
    if (sh.chunks == 1 && s.next) {
        // persistent grid, sinks from an atomic counter
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int bps = 0;
        const void *fn = sh.lanes_per_sink == 1 ? (const void *)force_fp64_dyn_kernel<1>
                         : sh.lanes_per_sink == 8 ? (const void *)force_fp64_dyn_kernel<8>
                                                  : (const void *)force_fp64_dyn_kernel<32>;
        ABIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, 256, 0));
        long long want = ((long long)n * sh.lanes_per_sink + 255) / 256;
        int blocks = (int)std::max<long long>(1, std::min<long long>((long long)sms * std::max(bps, 1), want));
        ABIE_CUDA(cudaMemsetAsync(s.next, 0, sizeof(unsigned int), st));
        switch (sh.lanes_per_sink) {
        case 1:
            force_fp64_dyn_kernel<1><<<blocks, 256, 0, st>>>(pos, m, n, s.src, s.n_src, acc, s.next);
            break;
        case 8:
            force_fp64_dyn_kernel<8><<<blocks, 256, 0, st>>>(pos, m, n, s.src, s.n_src, acc, s.next);
            break;
        default:
            force_fp64_dyn_kernel<32><<<blocks, 256, 0, st>>>(pos, m, n, s.src, s.n_src, acc, s.next);
            break;
        }
        ABIE_CUDA(cudaGetLastError());
        return 0;
    }
    long long groups = (long long)n * sh.chunks;
    int gpb = 256 / sh.lanes_per_sink;
    int blocks = (int)((groups + gpb - 1) / gpb);
    switch (sh.lanes_per_sink) {
    case 1:
        force_fp64_kernel<1><<<blocks, 256, 0, st>>>(pos, m, n, s.src, s.n_src, sh.chunks, acc,
                                                     s.partial);
        break;
    case 8:
        force_fp64_kernel<8><<<blocks, 256, 0, st>>>(pos, m, n, s.src, s.n_src, sh.chunks, acc,
                                                     s.partial);
        break;
    case 32:
        force_fp64_kernel<32><<<blocks, 256, 0, st>>>(pos, m, n, s.src, s.n_src, sh.chunks, acc,
                                                      s.partial, sym);
        break;
    default:
        set_error(ABIE_ERR_ARGUMENT, "lanes_per_sink must be 1, 8 or 32");
        return ABIE_ERR_ARGUMENT;
    }
    ABIE_CUDA(cudaGetLastError());
    if (sh.chunks > 1) {
        sum_chunks_kernel<<<(n + 255) / 256, 256, 0, st>>>(s.partial, m, n, sh.chunks, acc,
                                                           sym ? s.n_src : nullptr);
        ABIE_CUDA(cudaGetLastError());
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Energy: src/common.c:340-357, the reference's kinetic and pair terms summed
// as double-double values in a fixed order (energy_kernel below).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e)
{
    s = a + b;
    double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void dd_add(double &hi, double &lo, double v)
{
    double s, e;
    two_sum(hi, v, s, e);
    e += lo;
    two_sum(s, e, hi, lo);
}

// calculate_energy (src/common.c:340-357): one warp per body i with m_i != 0.
// Lane 0 starts from the kinetic term 0.5 m |v|^2 (|v| from sqrt, squared,
// as the reference does); the lanes take the partners j = lane, lane + 32,
// ... (m_j != 0, j != i), each adding the reference's term -(G m_i / 2) m_j
// / sqrt(r^2) to a double-double sum; the lanes, then the block's 8 warps,
// meet in a fixed order, and the host adds the blocks' sums in block order.
// (One thread per body left the FP64 pipe idle: 512 warps for 16,385
// bodies.)
constexpr int ENERGY_WARPS = 8;
__global__ void __launch_bounds__(32 * ENERGY_WARPS) energy_kernel(const double *__restrict__ pos,
                                                                   const double *__restrict__ vel,
                                                                   const double *__restrict__ m, int n,
                                                                   double G,
                                                                   double *__restrict__ partials)
{
    __shared__ double sh[ENERGY_WARPS][2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * ENERGY_WARPS + w;
    double hi = 0.0, lo = 0.0;
    if (i < n && m[i] != 0.0) {
        if (lane == 0) {
            double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
            double s = 0.0;
            s += vx * vx;
            s += vy * vy;
            s += vz * vz;
            double nv = sqrt(s);
            dd_add(hi, lo, 0.5 * m[i] * (nv * nv));
        }
        double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
        double c = 0.5 * G * m[i];
        for (int j = lane; j < n; j += 32) {
            double mj = m[j];
            if (j == i || mj == 0.0) continue;
            double dx = xi - pos[3 * j], dy = yi - pos[3 * j + 1], dz = zi - pos[3 * j + 2];
            double r2 = 0.0;
            r2 += dx * dx;
            r2 += dy * dy;
            r2 += dz * dz;
            dd_add(hi, lo, -(c * mj / sqrt(r2)));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double h2 = __shfl_down_sync(0xffffffffu, hi, o);
        const double l2 = __shfl_down_sync(0xffffffffu, lo, o);
        if (lane < o) {
            dd_add(hi, lo, h2);
            dd_add(hi, lo, l2);
        }
    }
    if (lane == 0) {
        sh[w][0] = hi;
        sh[w][1] = lo;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double h = sh[0][0], l = sh[0][1];
        for (int q = 1; q < ENERGY_WARPS; q++) {
            dd_add(h, l, sh[q][0]);
            dd_add(h, l, sh[q][1]);
        }
        partials[2 * blockIdx.x] = h;
        partials[2 * blockIdx.x + 1] = l;
    }
}

int launch_energy(const double *pos, const double *vel, const double *m, int n, double G,
                  double *d_partials, double *h_out, cudaStream_t st)
{
    if (n <= 0) {
        *h_out = 0.0;
        return 0;
    }
    const int blocks = (n + ENERGY_WARPS - 1) / ENERGY_WARPS;
    energy_kernel<<<blocks, 32 * ENERGY_WARPS, 0, st>>>(pos, vel, m, n, G, d_partials);
    ABIE_CUDA(cudaGetLastError());
    double *host = (double *)malloc(2 * (size_t)blocks * sizeof(double));
    if (!host) {
        set_error(ABIE_ERR_ARGUMENT, "out of host memory");
        return ABIE_ERR_ARGUMENT;
    }
    cudaError_t e = cudaMemcpyAsync(host, d_partials, 2 * (size_t)blocks * sizeof(double),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        free(host);
        return cuda_fail(e, "energy readback");
    }
    // host double-double sum of the block results, in block order
    double hi = 0.0, lo = 0.0;
    for (int b = 0; b < 2 * blocks; b++) {
        double v = host[b];
        double s = hi + v, bb = s - hi;
        double err = (hi - (s - bb)) + (v - bb);
        err += lo;
        hi = s + err;
        lo = err - (hi - s);
    }
    free(host);
    *h_out = hi + lo;
    return 0;
}

}  // namespace abie

namespace abie {

// Fast FP64 force with scratch the caller provides (compact source list,
// its body indices and count); launches the compaction and one force kernel
// and allocates nothing.  Always the one-chunk kernel (no partial sums) with
// the automatic lanes per sink (1, 8 or 32); the debug shape override does
// not apply here.
int launch_force_fp64_scratch(const double *pos, const double *m, int n, double G, Src *src,
                              int *src_body, int *n_src, double *acc, cudaStream_t st)
{
    if (n <= 0) return 0;
    compact_sources_kernel<<<1, 1024, 0, st>>>(pos, m, n, G, src, src_body, n_src);
    ABIE_CUDA(cudaGetLastError());
    const ForceShape sh = force_shape_auto(n, n);
    const int gpb = 256 / sh.lanes_per_sink;
    int blocks = (n + gpb - 1) / gpb;
    switch (sh.lanes_per_sink) {
    case 1:
        force_fp64_kernel<1><<<blocks, 256, 0, st>>>(pos, m, n, src, n_src, 1, acc, nullptr);
        break;
    case 8:
        force_fp64_kernel<8><<<blocks, 256, 0, st>>>(pos, m, n, src, n_src, 1, acc, nullptr);
        break;
    default:
        force_fp64_kernel<32><<<blocks, 256, 0, st>>>(pos, m, n, src, n_src, 1, acc, nullptr);
        break;
    }
    ABIE_CUDA(cudaGetLastError());
    return 0;
}

// Exact form: one thread per sink, sources in index order
// (src/additional_forces.c:46-117), the reference's pair term.  Fast form:
// one warp per sink, the lanes over the sources, the regrouped pair term,
// the lanes' sums added in a fixed shuffle tree.
template <int MODE>
__global__ void __launch_bounds__(256) post_newtonian_kernel(const double *__restrict__ pos,
                                                             const double *__restrict__ vel,
                                                             const double *__restrict__ m, int n,
                                                             PnConst K, double *__restrict__ acc)
{
    if constexpr (MODE != ABIE_FORCE_EXACT) {
        const int lane = threadIdx.x & 31;
        const int j = blockIdx.x * 8 + (threadIdx.x >> 5);
        if (j >= n) return;  // whole warps leave together
        const double x = pos[3 * j], y = pos[3 * j + 1], z = pos[3 * j + 2];
        const double vx = vel[3 * j], vy = vel[3 * j + 1], vz = vel[3 * j + 2];
        const double Mj = m[j];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (int k = lane; k < n; k += 32) {
            const double Mk = m[k];
            if (k == j || Mk == 0.0) continue;
            pn_term<MODE>(K, x, y, z, vx, vy, vz, Mj, pos[3 * k], pos[3 * k + 1], pos[3 * k + 2],
                          vel[3 * k], vel[3 * k + 1], vel[3 * k + 2], Mk, ax, ay, az);
        }
        for (int o = 16; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o);
            ay += __shfl_xor_sync(0xffffffffu, ay, o);
            az += __shfl_xor_sync(0xffffffffu, az, o);
        }
        if (lane == 0) {
            acc[3 * j] += ax;
            acc[3 * j + 1] += ay;
            acc[3 * j + 2] += az;
        }
        return;
    }
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double x = pos[3 * j], y = pos[3 * j + 1], z = pos[3 * j + 2];
    const double vx = vel[3 * j], vy = vel[3 * j + 1], vz = vel[3 * j + 2];
    const double Mj = m[j];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int k = 0; k < n; k++) {
        const double Mk = m[k];
        if (k == j || Mk == 0.0) continue;
        pn_term<MODE>(K, x, y, z, vx, vy, vz, Mj, pos[3 * k], pos[3 * k + 1], pos[3 * k + 2], vel[3 * k],
                vel[3 * k + 1], vel[3 * k + 2], Mk, ax, ay, az);
    }
    acc[3 * j] += ax;
    acc[3 * j + 1] += ay;
    acc[3 * j + 2] += az;
}

int launch_post_newtonian(const double *pos, const double *vel, const double *m, int n, double G,
                          double C, double *acc, cudaStream_t st, bool fast)
{
    if (n <= 0) return 0;
    if (fast)
        post_newtonian_kernel<ABIE_FORCE_FP64>
            <<<(n + 7) / 8, 256, 0, st>>>(pos, vel, m, n, pn_const(G, C), acc);
    else
        post_newtonian_kernel<ABIE_FORCE_EXACT>
            <<<(n + 255) / 256, 256, 0, st>>>(pos, vel, m, n, pn_const(G, C), acc);
    ABIE_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace abie
