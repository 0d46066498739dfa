// sd_sort_noalloc.cu -- the onesweep radix sort with library-owned scratch.
//
// sd_sort_pairs needs a device scratch buffer from its caller.  Some callers
// cannot provide one: code that runs where cudaMalloc is not allowed or not
// wanted -- a real-time stepping loop that must never block on the device
// allocator (cudaMalloc may synchronise the whole device), or a host
// application that hands this library only the key and value buffers it
// already owns and keeps a fixed device-memory budget.  For them this file
// keeps the sort's scratch in a fixed array in device memory that the module
// itself defines, and sd_sort_pairs_noalloc allocates nothing.
//
// Limits and sharing:
//   * the array holds kNoAllocScratchBytes (8 MiB); a sort whose scratch
//     need (sd_sort_scratch_bytes) is larger is rejected with
//     SD_ERR_CAPACITY -- e.g. up to 2,093,056 keys of 32 bits or 4,188,160
//     keys of at most 18 bits;
//   * every GPU that loads the library keeps the 8 MiB until process exit;
//   * all calls share the one array: two calls whose work overlaps on the GPU
//     (different streams, no ordering between them) race and corrupt each
//     other's results; order them on one stream or with events;
//   * each call clears the parts of the array that must start at zero
//     (status word, tile tickets, histograms, look-back flags), so nothing
//     carries over from the previous call.
#include <cuda_runtime.h>

#include <string>

#include "../../include/stardust.h"
#include "sd_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;
constexpr size_t kNoAllocScratchWords = kNoAllocScratchBytes / sizeof(uint32_t);
// The scratch.  Host code must not use this name as an address (on the host
// it is only a stand-in for the device symbol); its device address comes from
// cudaGetSymbolAddress with the device current.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

// failures are reported through sd_last_error(NULL, ...)
sd_status noalloc_fail(sd_status code, const std::string& msg) {
    sd::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" sd_status sd_sort_pairs_noalloc(uint32_t* d_keys, uint32_t* d_vals, uint32_t* d_keys_tmp,
                                           uint32_t* d_vals_tmp, uint64_t n, int32_t key_bits,
                                           uint32_t* d_status, void* stream) {
    if (key_bits < 1 || key_bits > 32) return noalloc_fail(SD_ERR_INVALID_ARG, "key_bits must be 1..32");
    if (n >= (1ull << 30)) return noalloc_fail(SD_ERR_CAPACITY, "n must be < 2^30");
    const uint64_t need = sd::sort_scratch_words(n, key_bits) * sizeof(uint32_t);
    if (need > kNoAllocScratchBytes)
        return noalloc_fail(SD_ERR_CAPACITY, "sort of " + std::to_string(n) + " keys of " + std::to_string(key_bits) +
                                                 " bits needs " + std::to_string(need) +
                                                 " bytes of scratch; the built-in array holds " +
                                                 std::to_string(kNoAllocScratchBytes));
    if (n == 0) return SD_OK;
    if (!d_keys || !d_vals || !d_keys_tmp || !d_vals_tmp)
        return noalloc_fail(SD_ERR_INVALID_ARG, "NULL key/value buffer");

    // the array's device address on the current device, looked up on every
    // call: once the module is loaded this is a table lookup, and it stays
    // right across a cudaDeviceReset (which unloads the module and may place
    // the array elsewhere when it is loaded again)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
        return noalloc_fail(SD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    uint32_t* scratch = static_cast<uint32_t*>(p);

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the status word (error bits) starts at zero on every call; the sort
    // clears its tickets, histograms and look-back flags itself
    e = cudaMemsetAsync(scratch, 0, 16, st);
    bool in_tmp = false;
    if (e == cudaSuccess)
        e = sd::sort_pairs_async(d_keys, d_vals, d_keys_tmp, d_vals_tmp, (uint32_t)n, key_bits, scratch, st, &in_tmp);
    if (e == cudaSuccess && in_tmp) {
        e = cudaMemcpyAsync(d_keys, d_keys_tmp, 4 * n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_vals, d_vals_tmp, 4 * n, cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess && d_status) e = cudaMemcpyAsync(d_status, scratch, 4, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return noalloc_fail(SD_ERR_CUDA, std::string("sort: ") + cudaGetErrorString(e));
    return SD_OK;
}
