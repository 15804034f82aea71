// tess_noalloc.cu -- CSR offsets for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc: code running with a fixed device
// memory budget that must not grow, code under an allocator that owns all
// device memory, or code on a path where an allocation's implicit
// synchronisation is not allowed.  They hold per-cell face counts on the
// device (for example computed from tess_results_device) and need the CSR
// offsets.  tess_csr_offsets_noalloc runs the same exclusive scan as the
// library's own CSR compaction.  Its block-sum scratch lives in a file-scope
// device array instead of a buffer allocated per call.
//
// That array (kScratchWords 64-bit words, 128 KiB) is part of the module:
// every GPU that loads the library holds it until the process exits.  All
// calls share it and it keeps the last call's contents; the scan overwrites
// every word it reads, so nothing needs clearing between calls.  Calls whose
// work overlaps on the GPU (different streams, or other host threads) race on
// it.
#include <cstdio>
#include <mutex>

#include "tess_internal.cuh"
#include "tessellator.h"

namespace {

// Largest input: 2^26 counts, i.e. ceil(2^26 / 4096) block sums + 2 words.
constexpr size_t kMaxCounts = (size_t)1 << 26;
constexpr size_t kScratchWords = (kMaxCounts + 4095) / 4096 + 2;

static __device__ __align__(256) uint64_t g_scan_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (with that device current) and cached.
tess_status scratch_address(int dev, uint64_t** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
        if (e != cudaSuccess) {
            tess::set_error("tess_csr_offsets_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return TESS_E_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = static_cast<uint64_t*>(g_scratch_ptr[dev]);
    return TESS_OK;
}

}  // namespace

extern "C" tess_status tess_csr_offsets_noalloc(const uint32_t* d_counts, size_t n, uint64_t* d_offs,
                                                void* stream) {
    if (!d_offs || (n > 0 && !d_counts)) {
        tess::set_error("tess_csr_offsets_noalloc: NULL device pointer");
        return TESS_E_INVALID;
    }
    if (n > kMaxCounts || tess::csr_tmp_words((uint32_t)n) > kScratchWords) {
        tess::set_error("tess_csr_offsets_noalloc: %zu counts exceed the maximum of %zu", n, kMaxCounts);
        return TESS_E_CAPACITY;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        tess::set_error("tess_csr_offsets_noalloc: no usable CUDA device (%s)", cudaGetErrorString(e));
        return TESS_E_CUDA;
    }
    uint64_t* scratch = nullptr;
    const tess_status st = scratch_address(dev, &scratch);
    if (st != TESS_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        e = cudaMemsetAsync(d_offs, 0, sizeof(uint64_t), s);
    } else {
        e = tess::launch_csr_offsets(d_counts, (uint32_t)n, d_offs, scratch, s);
    }
    if (e != cudaSuccess) {
        tess::set_error("tess_csr_offsets_noalloc: %s", cudaGetErrorString(e));
        return TESS_E_CUDA;
    }
    return TESS_OK;
}
