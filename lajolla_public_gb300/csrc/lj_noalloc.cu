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
// names a shadow variable), so the first call on each device, with that
// device current, asks the runtime for the address with cudaGetSymbolAddress
// and caches it; later calls on that device reuse it.  Make that first call
// before any stream capture begins.
//
// All calls share the one array and it keeps whatever the previous call left
// in it; each call initialises what it reads (the centroid bounds are reset,
// histograms are rewritten each pass).  Calls whose work overlaps on the GPU
// (different streams, or different host threads, without ordering between
// them) race on the array: callers must order them.
#include <cuda_runtime.h>

#include <mutex>

#include "lj_host.h"

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)2 << 20;
constexpr int64_t kNoallocMaxTris = LJ_NOALLOC_MORTON_MAX_TRIANGLES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kMaxDevices] = {};

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

// bytes used for n triangles: bounds | centroids | keys | tmp keys | tmp values | histogram
size_t noalloc_bytes(int64_t n) {
    return 256 + round256(sizeof(float4) * n) + 3 * round256(sizeof(uint32_t) * n) +
           round256(sizeof(uint32_t) * lj::radix_hist_entries(n));
}

__global__ void k_noalloc_iota(uint32_t *p, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (uint32_t)i;
}

// Device address of the scratch array on the current device (set-up on the
// first call per device).
int scratch_address(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return LJ_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return LJ_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_ptr[dev];
    return LJ_OK;
}

}  // namespace

extern "C" int lj_gpu_morton_sort_noalloc(const float *d_tri_vertices, int64_t n, uint32_t *d_codes,
                                          uint32_t *d_order, void *stream) {
    static_assert(256 + (size_t)16 * kNoallocMaxTris + 3 * (size_t)4 * kNoallocMaxTris +
                          (size_t)4 * 256 * ((kNoallocMaxTris + 2047) / 2048) <= kNoallocScratchBytes,
                  "scratch array too small for LJ_NOALLOC_MORTON_MAX_TRIANGLES");
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
