// FASTA sequence bytes -> the reference's 2-bit .npz arrays on the device
// (beguidedoff/genome_converter.py:15-108, which walks every base in Python).
//
// Format (the reference's, kept exactly):
//   * base code A/a 0, C/c 1, G/g 2, T/t 3, every other byte 0;
//   * genome_forward: chromosomes concatenated, 16 bases per uint32 word, base
//     i at bits 2 * (i % 16), the last word zero-padded;
//   * genome_rc: each chromosome reverse-complemented (3 - code, reversed
//     within the chromosome), concatenated in the same chromosome order;
//   * n_mask: one bit per forward position set for N or n only, packed most
//     significant bit first (np.packbits), the last byte zero-padded.
// One thread per 16 positions writes one forward word, one reverse-complement
// word and two mask bytes; the reads of 16 consecutive bytes (ascending for
// the forward strand, descending within a chromosome for the other) coalesce.
#include <cuda_runtime.h>

#include <vector>

#include "bgo_internal.cuh"

namespace bgo {

__device__ __forceinline__ uint32_t base_code(uint8_t b) {
    switch (b | 0x20) {  // lower case
        case 'c': return 1u;
        case 'g': return 2u;
        case 't': return 3u;
        default: return 0u;
    }
}

struct EncodeParams {
    const uint8_t *seq;
    int64_t total;
    const int64_t *offsets;  // [n_chroms]
    const int64_t *lengths;
    int32_t n_chroms;
    uint32_t *fwd;
    uint32_t *rc;       // nullptr: not wanted
    uint8_t *nmask;     // nullptr: not wanted
};

__global__ void encode_kernel(EncodeParams e, int64_t n_words) {
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n_words) return;
    const int64_t q0 = 16 * w;
    uint32_t f = 0, r = 0, nm = 0;
    // chromosome of the word's first position (last offset <= q0)
    int c = 0;
    if (e.rc) {
        int lo = 0, hi = e.n_chroms;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (e.offsets[mid] <= q0) lo = mid + 1;
            else hi = mid;
        }
        c = lo > 0 ? lo - 1 : 0;
    }
    for (int j = 0; j < 16; ++j) {
        const int64_t q = q0 + j;
        if (q >= e.total) break;
        const uint8_t b = e.seq[q];
        f |= base_code(b) << (2 * j);
        if ((b | 0x20) == 'n') nm |= 1u << j;
        if (e.rc) {
            while (c + 1 < e.n_chroms && e.offsets[c + 1] <= q) ++c;
            const int64_t src = e.offsets[c] + e.lengths[c] - 1 - (q - e.offsets[c]);
            r |= (3u - base_code(e.seq[src])) << (2 * j);
        }
    }
    e.fwd[w] = f;
    if (e.rc) e.rc[w] = r;
    if (e.nmask) {
        // positions q0..q0+7 -> byte 2w (bit 7 - k), q0+8..q0+15 -> byte 2w+1
        uint32_t b0 = 0, b1 = 0;
        for (int k = 0; k < 8; ++k) {
            b0 |= ((nm >> k) & 1u) << (7 - k);
            b1 |= ((nm >> (8 + k)) & 1u) << (7 - k);
        }
        const int64_t n_bytes = (e.total + 7) / 8;
        if (2 * w < n_bytes) e.nmask[2 * w] = (uint8_t)b0;
        if (2 * w + 1 < n_bytes) e.nmask[2 * w + 1] = (uint8_t)b1;
    }
}

}  // namespace bgo

using namespace bgo;

extern "C" int bgo_encode_genome(const uint8_t *seq, const int64_t *chrom_lengths,
                                 int32_t n_chroms, int device, uint32_t *fwd_out,
                                 uint32_t *rc_out, uint8_t *n_mask_big_out) {
    if (!chrom_lengths || n_chroms <= 0 || !fwd_out) {
        set_error("bgo_encode_genome: invalid argument");
        return BGO_ERR_ARG;
    }
    std::vector<int64_t> offs((size_t)n_chroms);
    int64_t total = 0;
    for (int i = 0; i < n_chroms; ++i) {
        if (chrom_lengths[i] < 0) {
            set_error("bgo_encode_genome: negative chromosome length");
            return BGO_ERR_ARG;
        }
        offs[(size_t)i] = total;
        total += chrom_lengths[i];
    }
    if (total > 0 && !seq) {
        set_error("bgo_encode_genome: no sequence bytes");
        return BGO_ERR_ARG;
    }
    const int64_t n_words = (total + 15) / 16;
    const int64_t n_bytes = (total + 7) / 8;
    if (n_words == 0) return BGO_OK;
    BGO_CUDA(cudaSetDevice(device));
    // one block: sequence | offsets | lengths | forward | rc | mask
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t b_seq = al((size_t)total), b_tab = al(sizeof(int64_t) * (size_t)n_chroms);
    const size_t b_w = al(sizeof(uint32_t) * (size_t)n_words), b_m = al((size_t)n_bytes);
    unsigned char *d = nullptr;
    BGO_CUDA(cudaMalloc(&d, b_seq + 2 * b_tab + 2 * b_w + b_m));
    EncodeParams e{};
    e.seq = d;
    e.total = total;
    int64_t *d_off = (int64_t *)(d + b_seq);
    int64_t *d_len = (int64_t *)(d + b_seq + b_tab);
    e.offsets = d_off;
    e.lengths = d_len;
    e.n_chroms = n_chroms;
    e.fwd = (uint32_t *)(d + b_seq + 2 * b_tab);
    e.rc = rc_out ? (uint32_t *)(d + b_seq + 2 * b_tab + b_w) : nullptr;
    e.nmask = n_mask_big_out ? (uint8_t *)(d + b_seq + 2 * b_tab + 2 * b_w) : nullptr;
    cudaError_t ce = cudaMemcpy(d, seq, (size_t)total, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
        ce = cudaMemcpy(d_off, offs.data(), sizeof(int64_t) * (size_t)n_chroms,
                        cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
        ce = cudaMemcpy(d_len, chrom_lengths, sizeof(int64_t) * (size_t)n_chroms,
                        cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) {
        encode_kernel<<<(unsigned)((n_words + 255) / 256), 256>>>(e, n_words);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess)
        ce = cudaMemcpy(fwd_out, e.fwd, sizeof(uint32_t) * (size_t)n_words, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && rc_out)
        ce = cudaMemcpy(rc_out, e.rc, sizeof(uint32_t) * (size_t)n_words, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && n_mask_big_out)
        ce = cudaMemcpy(n_mask_big_out, e.nmask, (size_t)n_bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (ce != cudaSuccess) return cuda_fail(ce, "bgo_encode_genome");
    return BGO_OK;
}
