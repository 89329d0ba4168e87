// abie_force_device_noalloc: the fast FP64 all-pairs force for callers that
// cannot allocate GPU memory.
//
// Who needs it: code that may not call cudaMalloc -- a real-time or
// host-callback loop that must not block on the allocator (cudaMalloc can
// synchronise the device), a process whose memory budget hands the library
// only the caller's own input and output buffers, or a host framework that
// owns every allocation on the device.  abie_force_device allocates its
// scratch (the compact list of massive sources) on first use and whenever N
// grows; this variant uses a fixed scratch area compiled into the library
// instead, and always runs the one-chunk force kernel (never the symmetric
// or two-chunk forms), so from 8,192 bodies its results agree with
// abie_force_device's to rounding, not bit for bit.
//
// The scratch is a file-scope __device__ array sized for at most
// ABIE_NOALLOC_MAX_BODIES bodies (2.25 MiB); every GPU that loads the library
// holds it until the process exits.  Every call shares it and it keeps the
// previous call's contents: the source count is rewritten by each call
// before it is read, so nothing needs clearing, but two calls whose kernels
// overlap on the GPU (different streams, no ordering between them) race on
// the same scratch and give wrong results.  Order such calls on one stream.
//
// In host code the array names below are host-side stand-ins, not device
// addresses.  The first call on each device, with that device current, asks
// the runtime for their device addresses with cudaGetSymbolAddress and keeps
// them (under a lock, so concurrent first calls from several host threads
// are safe); make that first call before any stream capture begins.
#include <atomic>
#include <mutex>

#include "abi_state.cuh"
#include "force.cuh"

namespace abie {

static __device__ __align__(256) Src g_noalloc_src[ABIE_NOALLOC_MAX_BODIES];
static __device__ __align__(256) int g_noalloc_body[ABIE_NOALLOC_MAX_BODIES];
static __device__ __align__(256) int g_noalloc_count;

struct NoallocPtrs {
    Src *src;
    int *body;
    int *count;
};
static const int NOALLOC_MAX_DEVICES = 64;
static NoallocPtrs g_noalloc_ptrs[NOALLOC_MAX_DEVICES];
static std::atomic<bool> g_noalloc_ready[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_lock;

// Device addresses of the scratch on the current device (set-up on first use).
static int noalloc_setup(int dev, NoallocPtrs *out)
{
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_error(ABIE_ERR_ARGUMENT, "abie_force_device_noalloc: device %d out of range", dev);
        return ABIE_ERR_ARGUMENT;
    }
    if (!g_noalloc_ready[dev].load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> guard(g_noalloc_lock);
        if (g_noalloc_ready[dev].load(std::memory_order_relaxed)) {
            *out = g_noalloc_ptrs[dev];
            return 0;
        }
        int major = 0, minor = 0;
        ABIE_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
        ABIE_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
        if (major != 10 || minor != 3) {
            set_error(ABIE_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a",
                      dev, major, minor);
            return ABIE_ERR_NO_DEVICE;
        }
        NoallocPtrs p = {};
        ABIE_CUDA(cudaGetSymbolAddress((void **)&p.src, g_noalloc_src));
        ABIE_CUDA(cudaGetSymbolAddress((void **)&p.body, g_noalloc_body));
        ABIE_CUDA(cudaGetSymbolAddress((void **)&p.count, g_noalloc_count));
        g_noalloc_ptrs[dev] = p;
        g_noalloc_ready[dev].store(true, std::memory_order_release);
    }
    *out = g_noalloc_ptrs[dev];
    return 0;
}

}  // namespace abie

extern "C" int abie_force_device_noalloc(const double *d_pos, const double *d_m, size_t N,
                                         double G, double *d_acc, void *stream)
{
    using namespace abie;
    // the full size_t is checked (no 32-bit convention here: this entry point
    // has no reference caller passing c_int)
    if (N > (size_t)ABIE_NOALLOC_MAX_BODIES) {
        set_error(ABIE_ERR_CAPACITY,
                  "abie_force_device_noalloc: N=%zu exceeds its fixed scratch of %d bodies; use "
                  "abie_force_device",
                  N, ABIE_NOALLOC_MAX_BODIES);
        return ABIE_ERR_CAPACITY;
    }
    if (N == 0) return 0;
    int dev = -1;
    ABIE_CUDA(cudaGetDevice(&dev));
    NoallocPtrs p;
    int rc = noalloc_setup(dev, &p);
    if (rc) return rc;
    return launch_force_fp64_scratch(d_pos, d_m, (int)N, G, p.src, p.body, p.count, d_acc,
                                     (cudaStream_t)stream);
}
