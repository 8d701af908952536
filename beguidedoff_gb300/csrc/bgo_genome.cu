// Strand upload: reference 2-bit packing -> device H/L/N bit planes.
//
// Replaces the device caches of beguidedoff/cuda_search.py:321-381 (which kept
// the packed uint32 array and the byte mask as uploaded).  The scan kernels
// read 32 positions of one plane per 32-bit word, so the two bits of each base
// are split into separate planes once here and never again per scan.
#include <cuda_runtime.h>

#include <new>
#include <string>

#include "bgo_internal.cuh"

namespace bgo {

// Gathers the 16 even-indexed bits of x into bits 0..15.
__device__ __forceinline__ uint32_t even_bits16(uint32_t x) {
    x &= 0x55555555u;
    x = (x | (x >> 1)) & 0x33333333u;
    x = (x | (x >> 2)) & 0x0F0F0F0Fu;
    x = (x | (x >> 4)) & 0x00FF00FFu;
    x = (x | (x >> 8)) & 0x0000FFFFu;
    return x;
}

__global__ void planes_from_packed_kernel(const uint32_t *__restrict__ packed, int64_t n_words,
                                          const uint8_t *__restrict__ nmask, int64_t n_mask_bytes,
                                          int64_t total_bp, int64_t plane_words,
                                          uint32_t *__restrict__ planes) {
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= plane_words) return;
    int64_t first = w * 32;
    uint32_t keep = 0;
    if (first < total_bp) {
        int64_t left = total_bp - first;
        keep = left >= 32 ? 0xFFFFFFFFu : ((1u << left) - 1u);
    }
    uint32_t p0 = (2 * w < n_words) ? packed[2 * w] : 0u;
    uint32_t p1 = (2 * w + 1 < n_words) ? packed[2 * w + 1] : 0u;
    uint32_t L = even_bits16(p0) | (even_bits16(p1) << 16);
    uint32_t H = even_bits16(p0 >> 1) | (even_bits16(p1 >> 1) << 16);
    uint32_t N = 0;
    if (nmask) {
        for (int b = 0; b < 4; ++b) {
            int64_t i = 4 * w + b;
            uint32_t v = (i < n_mask_bytes) ? nmask[i] : 0u;
            N |= v << (8 * b);
        }
    }
    planes[w] = H & keep;
    planes[plane_words + w] = L & keep;
    planes[2 * plane_words + w] = N & keep;
}

// N summary of a strand: warp v builds summary word v, whose bit k covers
// N-plane words [32 (32 v + k), + 32): in step k lane i reads word
// 32 (32 v + k) + i (the warp's 32 loads coalesced) and the warp votes.
__global__ void nsum_kernel(const uint32_t *__restrict__ nplane, int64_t plane_words,
                            uint32_t *__restrict__ nsum, int64_t nsum_words) {
    const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    uint32_t bits = 0;
    for (int k = 0; k < 32; ++k) {
        const int64_t w = (v * 32 + k) * kNSumGroup + lane;
        const uint32_t x = (v < nsum_words && w < plane_words) ? nplane[w] : 0u;
        if (__any_sync(0xFFFFFFFFu, x != 0u)) bits |= 1u << k;
    }
    if (lane == 0 && v < nsum_words) nsum[v] = bits;
}

static cudaError_t build_nsum(bgo_genome *g, cudaStream_t s) {
    if (!g->d_nsum) return cudaSuccess;
    const int64_t threads = 32 * g->nsum_words;
    nsum_kernel<<<(unsigned)ceil_div(threads, 256), 256, 0, s>>>(
        g->d_planes + 2 * g->plane_words, g->plane_words, g->d_nsum, g->nsum_words);
    return cudaGetLastError();
}

}  // namespace bgo

extern "C" int bgo_genome_create(const uint32_t *packed, int64_t n_words, int64_t total_bp,
                                 const uint8_t *n_mask_le, int64_t n_mask_bytes, int device,
                                 void *stream, bgo_genome **out) {
    using namespace bgo;
    if (!out || !packed || n_words <= 0 || total_bp <= 0 || n_mask_bytes < 0) {
        set_error("bgo_genome_create: invalid argument");
        return BGO_ERR_ARG;
    }
    if (total_bp > 0xFFFFFFFFll || n_words * 16 < total_bp) {
        set_error("bgo_genome_create: total_bp must be < 2^32 and covered by n_words*16");
        return BGO_ERR_ARG;
    }
    *out = nullptr;
    BGO_CUDA(cudaSetDevice(device));
    cudaStream_t s = (cudaStream_t)stream;
    bgo_genome *g = new (std::nothrow) bgo_genome();
    if (!g) {
        set_error("bgo_genome_create: host allocation failed");
        return BGO_ERR_OOM;
    }
    g->device = device;
    g->total_bp = total_bp;
    g->has_n = (n_mask_le && n_mask_bytes > 0) ? 1 : 0;
    g->plane_words = plane_words_for(total_bp);
    g->bytes = 3 * g->plane_words * (int64_t)sizeof(uint32_t);
    uint32_t *d_packed = nullptr;
    uint8_t *d_mask = nullptr;
    int rc = BGO_OK;
    g->d_nsum = nullptr;
    g->nsum_words = g->has_n ? nsum_words_for(g->plane_words) : 0;
    cudaError_t e = cudaMalloc(&g->d_planes, (size_t)g->bytes);
    if (e == cudaSuccess && g->has_n)
        e = cudaMalloc(&g->d_nsum, sizeof(uint32_t) * (size_t)g->nsum_words);
    if (e == cudaSuccess) e = cudaMalloc(&d_packed, (size_t)n_words * sizeof(uint32_t));
    if (e == cudaSuccess && g->has_n) e = cudaMalloc(&d_mask, (size_t)n_mask_bytes);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_packed, packed, (size_t)n_words * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && g->has_n)
        e = cudaMemcpyAsync(d_mask, n_mask_le, (size_t)n_mask_bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        int threads = 256;
        int64_t blocks = ceil_div(g->plane_words, threads);
        planes_from_packed_kernel<<<(unsigned)blocks, threads, 0, s>>>(
            d_packed, n_words, d_mask, g->has_n ? n_mask_bytes : 0, total_bp, g->plane_words,
            g->d_planes);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = build_nsum(g, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_fail(e, "bgo_genome_create");
    if (d_packed) cudaFree(d_packed);
    if (d_mask) cudaFree(d_mask);
    if (rc != BGO_OK) {
        if (g->d_planes) cudaFree(g->d_planes);
        if (g->d_nsum) cudaFree(g->d_nsum);
        delete g;
        return rc;
    }
    *out = g;
    return BGO_OK;
}

extern "C" int bgo_genome_upload(bgo_genome *g, const uint32_t *packed, int64_t n_words,
                                 const uint8_t *n_mask_le, int64_t n_mask_bytes, void *stream) {
    using namespace bgo;
    if (!g || !packed || n_words * 16 < g->total_bp || n_mask_bytes < 0 ||
        ((n_mask_le && n_mask_bytes > 0) ? 1 : 0) != g->has_n) {
        set_error("bgo_genome_upload: the arrays must cover the genome's total_bp and keep "
                  "its N-mask presence");
        return BGO_ERR_ARG;
    }
    BGO_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t need = (size_t)n_words * sizeof(uint32_t) + (size_t)n_mask_bytes + 256;
    if (need > g->stage_bytes) {
        BGO_CUDA(cudaStreamSynchronize(s));
        if (g->d_stage) cudaFree(g->d_stage);
        g->d_stage = nullptr;
        g->stage_bytes = 0;
        BGO_CUDA(cudaMalloc(&g->d_stage, need));
        g->stage_bytes = need;
    }
    uint32_t *d_packed = reinterpret_cast<uint32_t *>(g->d_stage);
    uint8_t *d_mask = g->has_n ? g->d_stage + ((size_t)n_words * sizeof(uint32_t) + 255) / 256 * 256
                               : nullptr;
    BGO_CUDA(cudaMemcpyAsync(d_packed, packed, (size_t)n_words * sizeof(uint32_t),
                             cudaMemcpyHostToDevice, s));
    if (g->has_n)
        BGO_CUDA(cudaMemcpyAsync(d_mask, n_mask_le, (size_t)n_mask_bytes, cudaMemcpyHostToDevice, s));
    const int threads = 256;
    const int64_t blocks = ceil_div(g->plane_words, threads);
    planes_from_packed_kernel<<<(unsigned)blocks, threads, 0, s>>>(
        d_packed, n_words, d_mask, g->has_n ? n_mask_bytes : 0, g->total_bp, g->plane_words,
        g->d_planes);
    BGO_CUDA(cudaGetLastError());
    BGO_CUDA(build_nsum(g, s));
    return BGO_OK;
}

extern "C" int bgo_genome_destroy(bgo_genome *genome) {
    if (!genome) return BGO_OK;
    cudaSetDevice(genome->device);
    if (genome->d_stage) cudaFree(genome->d_stage);
    if (genome->d_nsum) cudaFree(genome->d_nsum);
    cudaError_t e = genome->d_planes ? cudaFree(genome->d_planes) : cudaSuccess;
    delete genome;
    if (e != cudaSuccess) return bgo::cuda_fail(e, "bgo_genome_destroy");
    return BGO_OK;
}

extern "C" int bgo_genome_info(const bgo_genome *genome, int64_t *total_bp, int *has_n_mask,
                               int64_t *device_bytes) {
    if (!genome) return BGO_ERR_ARG;
    if (total_bp) *total_bp = genome->total_bp;
    if (has_n_mask) *has_n_mask = genome->has_n;
    if (device_bytes) *device_bytes = genome->bytes;
    return BGO_OK;
}
