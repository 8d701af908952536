// Tools library (libbgo_tools.so, include/bgo_tools.h), not the product:
// seeded synthetic genomes in the reference .npz layout, generated on the
// device for the benchmarks and tests, and a probe of the integer pipes'
// throughput for the benchmark's roofline figures.
//
// Genome generator: every base is a pure function of (seed, forward position):
// byte (p & 7) of splitmix64(seed * 0x9E3779B97F4A7C15 + (p >> 3)) (the
// SplitMix64 finaliser of Steele, Lea and Flood, 2014) compared with three
// cumulative thresholds out of 256 gives A, C, G or T.  Positions inside the
// caller's N blocks are N (encoded A on the forward array and marked in the N
// mask).  The reverse-complement array is built per chromosome in the same
// chromosome order as the reference converter (beguidedoff/genome_converter.py
// :66-71), so the output is exactly what convert() writes for the same FASTA.
//
// Repeat families (optional): the genome is cut into n_copies equal regions and
// region r holds one copy of family f_r at a seeded offset, in a seeded
// orientation, with each base substituted (to one of the three other bases)
// with the given probability.  Copies never overlap, and a copy base is again
// a pure function of its position, so both strands stay consistent.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "../bgo_internal.cuh"
#include "bgo_tools.h"

namespace bgo {

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct SynthParams {
    uint64_t seed;
    int64_t total_bp;
    int32_t n_chroms;
    int64_t n_blocks;
    const int64_t *offsets;   // [n_chroms]
    const int64_t *lengths;   // [n_chroms]
    const int64_t *nb_start;  // [n_blocks] sorted, disjoint
    const int64_t *nb_end;
    uint32_t t0, t1, t2;
    // repeat families (rep_copies == 0: none)
    int64_t rep_copies, rep_region;
    int32_t rep_len, rep_families;
    uint32_t rep_div16;              // substitution probability x 65536
    uint64_t rep_seed;
    const uint8_t *rep_seq;          // [rep_families * rep_len] base codes
};

__device__ __forceinline__ uint32_t gen_base(const SynthParams &p, int64_t pos) {
    if (p.rep_copies) {
        const int64_t r = pos / p.rep_region;
        if (r < p.rep_copies) {
            const uint64_t h = splitmix64(p.rep_seed * 0xD6E8FEB86659FD93ull + (uint64_t)r);
            const int64_t start = r * p.rep_region +
                                  (int64_t)(h % (uint64_t)(p.rep_region - p.rep_len + 1));
            const int64_t i = pos - start;
            if (i >= 0 && i < p.rep_len) {
                const int f = (int)(((h >> 32) & 0xFFFFFFull) % (uint64_t)p.rep_families);
                const uint8_t *seq = p.rep_seq + (size_t)f * p.rep_len;
                uint32_t b = (h >> 63) ? 3u - seq[p.rep_len - 1 - i] : seq[i];
                const uint64_t h2 = splitmix64((p.rep_seed ^ 0xA0761D6478BD642Full) + (uint64_t)pos);
                if ((uint32_t)(h2 & 0xFFFFu) < p.rep_div16)
                    b = (b + 1u + (uint32_t)((h2 >> 16) % 3u)) & 3u;
                return b;
            }
        }
    }
    const uint64_t h = splitmix64(p.seed * 0x9E3779B97F4A7C15ull + (uint64_t)(pos >> 3));
    const uint32_t b = (uint32_t)(h >> (8 * (pos & 7))) & 0xFFu;
    return b < p.t0 ? 0u : b < p.t1 ? 1u : b < p.t2 ? 2u : 3u;
}

// Big-endian N mask byte b (np.packbits order): bit 7-k = position 8b+k.
__global__ void synth_nmask_kernel(SynthParams p, uint8_t *__restrict__ mask, int64_t n_bytes) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_bytes) return;
    int64_t lo = 0, hi = p.n_blocks;  // first block with end > 8b
    const int64_t first = 8 * b;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (p.nb_end[mid] <= first) lo = mid + 1;
        else hi = mid;
    }
    uint32_t v = 0;
    for (int k = 0; k < 8; ++k) {
        const int64_t pos = first + k;
        if (pos >= p.total_bp) break;
        int64_t i = lo;
        while (i < p.n_blocks && p.nb_end[i] <= pos) ++i;
        if (i < p.n_blocks && p.nb_start[i] <= pos) v |= 1u << (7 - k);
    }
    mask[b] = (uint8_t)v;
}

__device__ __forceinline__ bool is_n(const uint8_t *mask, int64_t pos) {
    return (mask[pos >> 3] >> (7 - (pos & 7))) & 1u;
}

__global__ void synth_packed_kernel(SynthParams p, const uint8_t *__restrict__ mask,
                                    uint32_t *__restrict__ fwd, uint32_t *__restrict__ rc,
                                    int64_t n_words) {
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n_words) return;
    uint32_t f = 0, r = 0;
    int c = 0;
    for (int j = 0; j < 16; ++j) {
        const int64_t q = 16 * w + j;
        if (q >= p.total_bp) break;
        const uint32_t bf = is_n(mask, q) ? 0u : gen_base(p, q);
        f |= bf << (2 * j);
        while (c + 1 < p.n_chroms && p.offsets[c + 1] <= q) ++c;
        const int64_t src = p.offsets[c] + p.lengths[c] - 1 - (q - p.offsets[c]);
        const uint32_t bs = is_n(mask, src) ? 0u : gen_base(p, src);
        r |= (3u - bs) << (2 * j);
    }
    fwd[w] = f;
    rc[w] = r;
}

template <int OP>
__global__ void int_probe_kernel(uint32_t *out, uint32_t seed, int iters) {
    uint32_t a0 = seed ^ threadIdx.x, a1 = a0 * 3u, a2 = a0 * 5u, a3 = a0 * 7u;
    uint32_t a4 = a0 + 11u, a5 = a0 + 13u, a6 = a0 + 17u, a7 = a0 + 19u;
    const uint32_t b = seed * 0x9E3779B9u;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (OP == 0) {
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a0) : "r"(a1), "r"(b));
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a1) : "r"(a2), "r"(b));
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a2) : "r"(a3), "r"(b));
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a3) : "r"(a4), "r"(b));
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a4) : "r"(a5), "r"(b));
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a5) : "r"(a6), "r"(b));
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a6) : "r"(a7), "r"(b));
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a7) : "r"(a0), "r"(b));
            } else if (OP == 1) {
                asm volatile("popc.b32 %0, %0;" : "+r"(a0));
                asm volatile("popc.b32 %0, %0;" : "+r"(a1));
                asm volatile("popc.b32 %0, %0;" : "+r"(a2));
                asm volatile("popc.b32 %0, %0;" : "+r"(a3));
                asm volatile("popc.b32 %0, %0;" : "+r"(a4));
                asm volatile("popc.b32 %0, %0;" : "+r"(a5));
                asm volatile("popc.b32 %0, %0;" : "+r"(a6));
                asm volatile("popc.b32 %0, %0;" : "+r"(a7));
            } else {
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a0) : "r"(a1));
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a1) : "r"(a2));
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a2) : "r"(a3));
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a3) : "r"(a4));
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a4) : "r"(a5));
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a5) : "r"(a6));
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a6) : "r"(a7));
                asm volatile("add.u32 %0, %0, %1;" : "+r"(a7) : "r"(a0));
            }
        }
    }
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
}

}  // namespace bgo

using namespace bgo;

static int synth(uint64_t seed, const int64_t *chrom_lengths, int32_t n_chroms,
                 const int64_t *n_starts, const int64_t *n_ends, int64_t n_blocks,
                 const uint8_t *thresholds, const bgo_repeat_spec *rep, uint8_t *families_out,
                 int device, uint32_t *fwd_out, uint32_t *rc_out, uint8_t *n_mask_big_out) {
    if (!chrom_lengths || n_chroms <= 0 || n_blocks < 0 || (n_blocks > 0 && (!n_starts || !n_ends)) ||
        !thresholds || !fwd_out || !rc_out || !n_mask_big_out) {
        set_error("bgo_synth_genome: invalid argument");
        return BGO_ERR_ARG;
    }
    if (!(thresholds[0] <= thresholds[1] && thresholds[1] <= thresholds[2])) {
        set_error("bgo_synth_genome: thresholds must be non-decreasing");
        return BGO_ERR_ARG;
    }
    std::vector<int64_t> offs((size_t)n_chroms);
    int64_t total = 0;
    for (int i = 0; i < n_chroms; ++i) {
        if (chrom_lengths[i] <= 0) {
            set_error("bgo_synth_genome: chromosome lengths must be positive");
            return BGO_ERR_ARG;
        }
        offs[(size_t)i] = total;
        total += chrom_lengths[i];
    }
    for (int64_t i = 0; i < n_blocks; ++i) {
        if (n_starts[i] < 0 || n_ends[i] < n_starts[i] || n_ends[i] > total ||
            (i > 0 && n_starts[i] < n_ends[i - 1])) {
            set_error("bgo_synth_genome: N blocks must be sorted, disjoint and inside the genome");
            return BGO_ERR_ARG;
        }
    }
    if (total > 0xFFFFFFFFll) {
        set_error("bgo_synth_genome: total length must be < 2^32");
        return BGO_ERR_ARG;
    }
    std::vector<uint8_t> fam;
    if (rep && rep->n_copies > 0) {
        if (rep->n_families <= 0 || rep->family_len <= 0 || rep->divergence_65536 > 65536u ||
            total / rep->n_copies < rep->family_len || !families_out) {
            set_error("bgo_synth_genome: repeat families must fit one per region");
            return BGO_ERR_ARG;
        }
        fam.resize((size_t)rep->n_families * rep->family_len);
        for (size_t i = 0; i < fam.size(); ++i)
            fam[i] = (uint8_t)(splitmix64(rep->seed * 0x9E3779B97F4A7C15ull + 0x5851F42D4C957F2Dull +
                                          (uint64_t)i) >> 62);
        memcpy(families_out, fam.data(), fam.size());
    }
    BGO_CUDA(cudaSetDevice(device));
    const int64_t n_words = ceil_div(total, 16);
    const int64_t n_bytes = ceil_div(total, 8);
    int64_t *d_tab = nullptr;
    uint8_t *d_mask = nullptr;
    uint32_t *d_fwd = nullptr, *d_rc = nullptr;
    const size_t tab = (size_t)(2 * n_chroms + 2 * n_blocks + 2);
    const size_t tab_bytes = tab * sizeof(int64_t);
    cudaError_t e = cudaMalloc(&d_tab, tab_bytes + fam.size());
    if (e == cudaSuccess) e = cudaMalloc(&d_mask, (size_t)n_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&d_fwd, (size_t)n_words * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_rc, (size_t)n_words * 4);
    SynthParams p{};
    p.seed = seed;
    p.total_bp = total;
    p.n_chroms = n_chroms;
    p.n_blocks = n_blocks;
    p.t0 = thresholds[0];
    p.t1 = thresholds[1];
    p.t2 = thresholds[2];
    if (!fam.empty()) {
        p.rep_copies = rep->n_copies;
        p.rep_region = total / rep->n_copies;
        p.rep_len = rep->family_len;
        p.rep_families = rep->n_families;
        p.rep_div16 = rep->divergence_65536;
        p.rep_seed = rep->seed;
    }
    if (e == cudaSuccess && !fam.empty()) {
        p.rep_seq = (const uint8_t *)d_tab + tab_bytes;
        e = cudaMemcpy((uint8_t *)d_tab + tab_bytes, fam.data(), fam.size(), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        p.offsets = d_tab;
        p.lengths = d_tab + n_chroms;
        p.nb_start = d_tab + 2 * n_chroms;
        p.nb_end = d_tab + 2 * n_chroms + n_blocks;
        e = cudaMemcpy(d_tab, offs.data(), sizeof(int64_t) * n_chroms, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(d_tab + n_chroms, chrom_lengths, sizeof(int64_t) * n_chroms,
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess && n_blocks)
            e = cudaMemcpy(d_tab + 2 * n_chroms, n_starts, sizeof(int64_t) * n_blocks,
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess && n_blocks)
            e = cudaMemcpy(d_tab + 2 * n_chroms + n_blocks, n_ends, sizeof(int64_t) * n_blocks,
                           cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        synth_nmask_kernel<<<(unsigned)ceil_div(n_bytes, 256), 256>>>(p, d_mask, n_bytes);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        synth_packed_kernel<<<(unsigned)ceil_div(n_words, 256), 256>>>(p, d_mask, d_fwd, d_rc,
                                                                       n_words);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(fwd_out, d_fwd, (size_t)n_words * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rc_out, d_rc, (size_t)n_words * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(n_mask_big_out, d_mask, (size_t)n_bytes, cudaMemcpyDeviceToHost);
    if (d_tab) cudaFree(d_tab);
    if (d_mask) cudaFree(d_mask);
    if (d_fwd) cudaFree(d_fwd);
    if (d_rc) cudaFree(d_rc);
    if (e != cudaSuccess) return cuda_fail(e, "bgo_synth_genome");
    return BGO_OK;
}

extern "C" int bgo_synth_genome(uint64_t seed, const int64_t *chrom_lengths, int32_t n_chroms,
                                const int64_t *n_starts, const int64_t *n_ends, int64_t n_blocks,
                                const uint8_t *thresholds, int device, uint32_t *fwd_out,
                                uint32_t *rc_out, uint8_t *n_mask_big_out) {
    return synth(seed, chrom_lengths, n_chroms, n_starts, n_ends, n_blocks, thresholds, nullptr,
                 nullptr, device, fwd_out, rc_out, n_mask_big_out);
}

extern "C" int bgo_synth_genome_repeats(uint64_t seed, const int64_t *chrom_lengths,
                                        int32_t n_chroms, const int64_t *n_starts,
                                        const int64_t *n_ends, int64_t n_blocks,
                                        const uint8_t *thresholds, const bgo_repeat_spec *repeats,
                                        uint8_t *families_out, int device, uint32_t *fwd_out,
                                        uint32_t *rc_out, uint8_t *n_mask_big_out) {
    if (!repeats) {
        set_error("bgo_synth_genome_repeats: repeats is NULL");
        return BGO_ERR_ARG;
    }
    return synth(seed, chrom_lengths, n_chroms, n_starts, n_ends, n_blocks, thresholds, repeats,
                 families_out, device, fwd_out, rc_out, n_mask_big_out);
}

extern "C" int bgo_probe_int_throughput(int device, int op, double *gops_per_s) {
    if (!gops_per_s || op < 0 || op > 2) return BGO_ERR_ARG;
    BGO_CUDA(cudaSetDevice(device));
    int sms = 0;
    BGO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int threads = 256, blocks = sms * 8, iters = 2048;
    uint32_t *out = nullptr;
    BGO_CUDA(cudaMalloc(&out, sizeof(uint32_t) * threads * blocks));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    cudaError_t err = cudaSuccess;
    for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {
        cudaEventRecord(e0);
        if (op == 0) int_probe_kernel<0><<<blocks, threads>>>(out, 1234u + rep, iters);
        if (op == 1) int_probe_kernel<1><<<blocks, threads>>>(out, 1234u + rep, iters);
        if (op == 2) int_probe_kernel<2><<<blocks, threads>>>(out, 1234u + rep, iters);
        cudaEventRecord(e1);
        err = cudaEventSynchronize(e1);
        if (err == cudaSuccess) err = cudaGetLastError();
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return cuda_fail(err, "bgo_probe_int_throughput");
    *gops_per_s = (double)blocks * threads * iters * 64.0 / (best * 1e-3) / 1e9;
    return BGO_OK;
}
