// orbc_gpu_morton_order_noalloc: the Morton-order sort of
// orbc_gpu_morton_order for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc / cudaFree: applications whose device
// memory is owned entirely by another allocator (a framework's caching pool
// that is the only permitted allocator), and latency-bound loops where the
// implicit device synchronisation of cudaMalloc / cudaFree is unacceptable.
// This entry point takes device pointers for its input and output and keeps
// its scratch (sort keys, the second value buffer, the per-tile digit counts)
// in one file-scope __device__ array of fixed size.  Every GPU that loads the
// library holds that array (about 3.1 MB) until the process exits.
#include <cuda.h>

#include <mutex>

#include "orbc_device.cuh"
#include "orbc_gpu.h"

namespace orbc {
namespace {

constexpr int64_t NA_MAX = ORBC_NOALLOC_MAX_POINTS;
constexpr int NA_TILES = int((NA_MAX + SORT_TILE - 1) / SORT_TILE);
// layout of the scratch array (all offsets 256-byte aligned)
constexpr size_t NA_KEYS0 = 0;
constexpr size_t NA_KEYS1 = NA_KEYS0 + size_t(NA_MAX) * 4;
constexpr size_t NA_VALS1 = NA_KEYS1 + size_t(NA_MAX) * 4;
constexpr size_t NA_COUNTS = NA_VALS1 + size_t(NA_MAX) * 4;
constexpr size_t NA_TOTAL = NA_COUNTS + size_t(256) * NA_TILES * 4;
constexpr size_t NA_BYTES = NA_TOTAL + 256 * 4;
static_assert(NA_KEYS1 % 256 == 0 && NA_VALS1 % 256 == 0 && NA_COUNTS % 256 == 0 && NA_TOTAL % 256 == 0,
              "scratch sub-buffers must stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_lock;
unsigned char *g_na_ptr[NA_MAX_DEVICES] = {};
unsigned long long g_na_ctx[NA_MAX_DEVICES] = {};  // context the cached address belongs to

/* Identity of the calling thread's current context.  Context ids are unique
 * for the life of the process, so after a cudaDeviceReset (which replaces the
 * device's context and may reload the module elsewhere) the cached address no
 * longer matches and is looked up again.  The driver calls are reached through
 * the runtime's entry-point query, so the library needs no link to libcuda. */
cudaError_t current_context_id(unsigned long long *id) {
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess)
            e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return e;
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return cudaErrorSymbolNotFound;
        get_current = reinterpret_cast<GetCurrent>(f1);
        get_id = reinterpret_cast<GetId>(f2);
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
    if (get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorContextIsDestroyed;
    return cudaSuccess;
}

__global__ void k_na_iota(int *v, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        v[i] = int(i);
}

int na_fail(const char *what, cudaError_t e) {
    set_standalone_error(what, cudaGetErrorString(e));
    return ORBC_ERR_CUDA;
}

/* Device address of the scratch array on the current device.  In host code
 * the symbol g_noalloc_scratch is only a host-side stand-in, so the address is
 * looked up once per device and context (with that device current) and
 * cached. */
int scratch_of_current_device(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail("morton_order_noalloc: cudaGetDevice", e);
    if (dev < 0 || dev >= NA_MAX_DEVICES) {
        set_standalone_error("morton_order_noalloc", "device ordinal beyond the library's table of 64 devices");
        return ORBC_ERR_ARG;
    }
    std::lock_guard<std::mutex> g(g_na_lock);
    unsigned long long ctx = 0;
    e = current_context_id(&ctx);
    if (e != cudaSuccess) return na_fail("morton_order_noalloc: current context", e);
    if (!g_na_ptr[dev] || g_na_ctx[dev] != ctx) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return na_fail("morton_order_noalloc: cudaGetSymbolAddress", e != cudaSuccess ? e : cudaErrorInvalidSymbol);
        g_na_ptr[dev] = static_cast<unsigned char *>(p);
        g_na_ctx[dev] = ctx;
    }
    *out = g_na_ptr[dev];
    return ORBC_OK;
}

}  // namespace
}  // namespace orbc

extern "C" int orbc_gpu_morton_order_noalloc(const double *d_p3, int64_t n, const double *bsize3, int32_t *d_order,
                                             void *stream) {
    using namespace orbc;
    if (n < 0 || n > NA_MAX) {
        set_standalone_error("morton_order_noalloc", "n must lie in 0 .. ORBC_NOALLOC_MAX_POINTS (262,144)");
        return ORBC_ERR_ARG;
    }
    if (n == 0) return ORBC_OK;
    if (!d_p3 || !bsize3 || !d_order) {
        set_standalone_error("morton_order_noalloc", "null pointer argument");
        return ORBC_ERR_ARG;
    }
    // an error left pending by the caller's earlier work would otherwise be
    // read back below as this call's failure; report it without clearing it
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) return na_fail("morton_order_noalloc: CUDA error pending before the call", pending);
    unsigned char *base = nullptr;
    const int rc = scratch_of_current_device(&base);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t *keys[2] = {reinterpret_cast<uint32_t *>(base + NA_KEYS0), reinterpret_cast<uint32_t *>(base + NA_KEYS1)};
    // the caller's output buffer is value buffer 0: four passes end in it
    int *vals[2] = {reinterpret_cast<int *>(d_order), reinterpret_cast<int *>(base + NA_VALS1)};
    int *counts = reinterpret_cast<int *>(base + NA_COUNTS);
    int *total = reinterpret_cast<int *>(base + NA_TOTAL);
    // nothing in the scratch needs clearing: the keys are written by the
    // encoder, and every pass rewrites all digit counts and totals it reads
    launch_morton(d_p3, n, bsize3, keys[0], st);
    k_na_iota<<<int(std::min<int64_t>((n + 255) / 256, 1024)), 256, 0, st>>>(vals[0], n);
    const int fin = radix_sort_pairs(keys, vals, counts, total, nullptr, n, 4, sort_tiles(n), nullptr, st);
    // the launches' own errors (nothing was pending at entry)
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail("morton_order_noalloc: launch", e);
    if (fin != 0) {  // four passes always end in buffer 0
        set_standalone_error("morton_order_noalloc", "radix sort ended in the scratch buffer");
        return ORBC_ERR_CUDA;
    }
    return ORBC_OK;
}
