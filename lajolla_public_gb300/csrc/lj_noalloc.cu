// lj_gpu_morton_sort_noalloc: the Morton-code + radix-sort stage of the BVH
// build for callers that cannot allocate device memory.
//
// Who needs it: code that must not call cudaMalloc at the moment it sorts --
// for example a host application whose device memory is handed out by its
// own arena sized once at start-up, or a latency-sensitive loop in which the
// device-wide synchronisation that an allocation can cause is not acceptable.
// Such callers still own the input and output buffers; everything else the
// sort needs lives in one fixed array compiled into this library.
//
// The scratch is a file-scope __device__ array of kNoallocScratchBytes
// (2 MiB) that every GPU which loads the library keeps until the process
// exits.  It limits n to LJ_NOALLOC_MORTON_MAX_TRIANGLES (65536); larger
// requests are rejected with LJ_ERR_SIZE_LIMIT before any work is queued.
//
// Host code cannot use the array's name as a device address (on the host it
// names a shadow variable), so the first call in each CUDA context (the
// runtime's primary context of a device, or a driver-API context the caller
// made current) asks the runtime for the address with cudaGetSymbolAddress
// and caches it under that context's unique id (cuCtxGetId); later calls in
// the same context reuse it.  A context that is destroyed and created again
// -- cudaDeviceReset, or cuCtxDestroy + cuCtxCreate -- has a new id, so the
// first call after it looks the address up again.  Make the first call in
// a context before any stream capture begins.
//
// All calls share the one array and it keeps whatever the previous call left
// in it; each call initialises what it reads (the centroid bounds are reset,
// histograms are rewritten each pass).  Calls whose work overlaps on the GPU
// (different streams, or different host threads, without ordering between
// them) race on the array: callers must order them.
#include <cuda_runtime.h>

#include <mutex>
#include <utility>
#include <vector>

#include "lj_host.h"

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)2 << 20;
constexpr int64_t kNoallocMaxTris = LJ_NOALLOC_MORTON_MAX_TRIANGLES;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr size_t round256(size_t b) { return (b + 255) / 256 * 256; }

// bytes used for n triangles: bounds | centroids | keys | tmp keys | tmp values | histogram
constexpr size_t noalloc_bytes(int64_t n) {
    return 256 + round256(sizeof(float4) * n) + 3 * round256(sizeof(uint32_t) * n) +
           round256(sizeof(uint32_t) * lj::radix_hist_entries(n));
}
static_assert(noalloc_bytes(kNoallocMaxTris) <= kNoallocScratchBytes,
              "scratch array too small for LJ_NOALLOC_MORTON_MAX_TRIANGLES");

__global__ void k_noalloc_iota(uint32_t *p, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (uint32_t)i;
}

// Driver entry points, fetched through the runtime so that the library does
// not link libcuda itself (it must load, for its exports to be checked, on
// machines without a GPU driver).
typedef int (*CtxGetCurrentFn)(void **ctx);                       // cuCtxGetCurrent
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);     // cuCtxGetId
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
std::once_flag g_entry_once;

void load_entry_points() {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_get_id = (CtxGetIdFn)f;
    cudaGetLastError();
}

// Unique id of the CUDA context current on this thread; false if there is
// none yet or the driver cannot say.
bool current_context_id(unsigned long long *id) {
    std::call_once(g_entry_once, load_entry_points);
    if (!g_ctx_get_current || !g_ctx_get_id) return false;
    void *ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0 || !ctx) return false;
    return g_ctx_get_id(ctx, id) == 0;
}

std::mutex g_noalloc_mutex;
std::vector<std::pair<unsigned long long, void *>> g_noalloc_ptr;   // context id -> address

// Device address of the scratch array in the current context (looked up
// with cudaGetSymbolAddress on the first call in each context).
int scratch_address(unsigned char **out) {
    unsigned long long id = 0;
    bool known = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (known) {
        for (auto &e : g_noalloc_ptr) {
            if (e.first == id) {
                *out = (unsigned char *)e.second;
                return LJ_OK;
            }
        }
    }
    // The lookup makes the runtime bind a context to this thread if none is
    // current yet (the device's primary context), so the id is read again
    // after it.
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? LJ_ERR_NO_DEVICE : LJ_ERR_CUDA;
    }
    if (current_context_id(&id)) g_noalloc_ptr.emplace_back(id, p);
    *out = (unsigned char *)p;
    return LJ_OK;
}

}  // namespace

extern "C" int lj_gpu_morton_sort_noalloc(const float *d_tri_vertices, int64_t n, uint32_t *d_codes,
                                          uint32_t *d_order, void *stream) {
    if (n < 0 || (n > 0 && (!d_tri_vertices || !d_codes || !d_order))) return LJ_ERR_INVALID_ARG;
    if (n > kNoallocMaxTris) return LJ_ERR_SIZE_LIMIT;
    if (n == 0) return LJ_OK;
    if (noalloc_bytes(n) > kNoallocScratchBytes) return LJ_ERR_SIZE_LIMIT;
    unsigned char *base = nullptr;
    int rc = scratch_address(&base);
    if (rc != LJ_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    unsigned char *p = base;
    uint32_t *bounds = (uint32_t *)p;
    p += 256;
    float4 *cent = (float4 *)p;
    p += round256(sizeof(float4) * n);
    uint32_t *keys = (uint32_t *)p;
    p += round256(sizeof(uint32_t) * n);
    uint32_t *tk = (uint32_t *)p;
    p += round256(sizeof(uint32_t) * n);
    uint32_t *tv = (uint32_t *)p;
    p += round256(sizeof(uint32_t) * n);
    uint32_t *hist = (uint32_t *)p;
    std::string err;
    if (lj::morton_codes_tris_into(d_tri_vertices, n, d_codes, bounds, cent, s)) return LJ_ERR_CUDA;
    if (cudaMemcpyAsync(keys, d_codes, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return LJ_ERR_CUDA;
    k_noalloc_iota<<<(int)((n + 255) / 256), 256, 0, s>>>(d_order, n);
    if (cudaGetLastError() != cudaSuccess) return LJ_ERR_CUDA;
    if (lj::radix_sort_pairs(keys, d_order, tk, tv, hist, n, s, &err)) return LJ_ERR_CUDA;
    return LJ_OK;
}
