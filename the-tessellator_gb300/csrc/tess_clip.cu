// tess_clip.cu -- dispatch to the clipping kernel instantiations
// (tess_clip_f32.cu, tess_clip_f64.cu; kernel source tess_clip_impl.cuh) and
// the CSR compaction of the per-cell face lists: offsets = exclusive scan of
// the face counts, then a gather from the face pool into original cell order
// (the bulk form of Cell::compute_faces, interface.rs:373-384).
#include "tess_internal.cuh"

namespace tess {
namespace {

constexpr unsigned FULL = 0xffffffffu;

// ---- CSR compaction: offsets = exclusive scan of face counts, then gather ----
constexpr int kCsrThreads = 1024;
constexpr int kCsrItems = 4;

__device__ unsigned long long block_excl_scan64(unsigned long long v, unsigned long long* sh) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    unsigned long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(FULL, inc, o);
        if (l >= o) inc += t;
    }
    if (l == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        unsigned long long s = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0ull;
        unsigned long long si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long t = __shfl_up_sync(FULL, si, o);
            if (l >= o) si += t;
        }
        sh[l] = si - s;
        if (l == 31) sh[32] = si;
    }
    __syncthreads();
    const unsigned long long r = inc - v + sh[w];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kCsrThreads) k_csr_partial(const uint32_t* cnt, uint32_t n,
                                                             unsigned long long* sums) {
    __shared__ unsigned long long sh[33];
    const uint64_t base = ((uint64_t)blockIdx.x * kCsrThreads + threadIdx.x) * kCsrItems;
    unsigned long long s = 0;
    for (int k = 0; k < kCsrItems; ++k) s += (base + k < n) ? cnt[base + k] : 0u;
    unsigned long long ex = block_excl_scan64(s, sh);
    if (threadIdx.x == kCsrThreads - 1) sums[blockIdx.x] = ex + s;
}

__global__ void __launch_bounds__(kCsrThreads) k_csr_sums(unsigned long long* sums, uint32_t nb) {
    __shared__ unsigned long long sh[33];
    unsigned long long carry = 0;
    for (uint32_t b0 = 0; b0 < nb; b0 += kCsrThreads) {
        const uint32_t b = b0 + threadIdx.x;
        const unsigned long long v = b < nb ? sums[b] : 0ull;
        const unsigned long long ex = block_excl_scan64(v, sh);
        if (b < nb) sums[b] = carry + ex;
        __shared__ unsigned long long tot;
        if (threadIdx.x == kCsrThreads - 1) tot = ex + v;
        __syncthreads();
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void __launch_bounds__(kCsrThreads) k_csr_final(const uint32_t* cnt, uint32_t n,
                                                           const unsigned long long* sums, uint64_t* offs) {
    __shared__ unsigned long long sh[33];
    const uint64_t base = ((uint64_t)blockIdx.x * kCsrThreads + threadIdx.x) * kCsrItems;
    uint32_t v[kCsrItems];
    unsigned long long s = 0;
    for (int k = 0; k < kCsrItems; ++k) {
        v[k] = (base + k < n) ? cnt[base + k] : 0u;
        s += v[k];
    }
    unsigned long long run = sums[blockIdx.x] + block_excl_scan64(s, sh);
    for (int k = 0; k < kCsrItems; ++k) {
        if (base + k < n) offs[base + k] = run;
        run += v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) offs[n] = sums[gridDim.x];
}

// One warp per 32 consecutive cells: their CSR range is contiguous, so the
// warp writes it as one coalesced stream; each output element finds its cell
// (lane) by a binary search over the warp's prefix sums of the face counts
// and reads from that cell's contiguous run in the face pool.
__global__ void __launch_bounds__(256) k_csr_gather(const uint32_t* cnt, const uint64_t* fstart,
                                                    const int32_t* fnbr, const double* farea, uint32_t n,
                                                    const uint64_t* offs, int32_t* nbr, double* area) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint64_t c0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ull;
    if (c0 >= n) return;                          // whole warps leave together
    const uint64_t i = c0 + lane;
    uint32_t c = 0;
    uint64_t src = 0;
    if (i < n) {
        c = cnt[i];
        src = fstart[i];
    }
    const uint64_t dst0 = offs[c0];
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    const uint32_t tot = __shfl_sync(kFull, incl, 31);
    const uint32_t excl = incl - c;
    for (uint32_t o = 0; o < tot; o += 32) {
        const uint32_t t = o + lane;
        int L = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const uint32_t v = __shfl_sync(kFull, incl, L + step - 1);
            if (v <= t) L += step;
        }
        const uint32_t ex = __shfl_sync(kFull, excl, L);
        const uint64_t sb = __shfl_sync(kFull, src, L);
        if (t < tot) {
            const uint64_t k = sb + (t - ex);
            if (nbr) nbr[dst0 + t] = fnbr[k];
            if (area) area[dst0 + t] = farea[k];
        }
    }
}

}  // namespace

cudaError_t launch_clip(const ClipParams& p, int precision, int slots, int form, int wpb, int blocks,
                        cudaStream_t s) {
    return precision == 1 ? launch_clip_f32(p, slots, form, wpb, blocks, s)
                          : launch_clip_f64(p, slots, form, wpb, blocks, s);
}

int clip_blocks_for(int precision, int slots, int form, int wpb, int device) {
    return precision == 1 ? clip_blocks_f32(slots, form, wpb, device) : clip_blocks_f64(slots, form, wpb, device);
}

size_t csr_tmp_words(uint32_t n) {
    const uint64_t per = (uint64_t)kCsrThreads * kCsrItems;
    return (size_t)((n + per - 1) / per) + 2;
}

cudaError_t launch_csr_offsets(const uint32_t* nface, uint32_t n, uint64_t* offs, uint64_t* scan_tmp,
                               cudaStream_t s) {
    const uint64_t per = (uint64_t)kCsrThreads * kCsrItems;
    const uint32_t nb = (uint32_t)((n + per - 1) / per);
    unsigned long long* sums = reinterpret_cast<unsigned long long*>(scan_tmp);
    k_csr_partial<<<nb, kCsrThreads, 0, s>>>(nface, n, sums);
    k_csr_sums<<<1, kCsrThreads, 0, s>>>(sums, nb);
    k_csr_final<<<nb, kCsrThreads, 0, s>>>(nface, n, sums, offs);
    return cudaGetLastError();
}

cudaError_t launch_csr_gather(const uint32_t* nface, const uint64_t* fstart, const int32_t* face_nbr,
                              const double* face_area, uint32_t n, const uint64_t* offs, int32_t* nbr_out,
                              double* area_out, cudaStream_t s) {
    k_csr_gather<<<(n + 255) / 256, 256, 0, s>>>(nface, fstart, face_nbr, face_area, n, offs, nbr_out, area_out);
    return cudaGetLastError();
}

}  // namespace tess
