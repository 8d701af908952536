// Prefiltered segment-index scan kernel (scan mode 2 with tuning.prefilter),
// included by the translation units that instantiate its forms (chunk length
// 2,048 or 4,096 positions, survivor index in shared or global memory:
// bgo_filter.cu, bgo_filter_2k_g.cu, bgo_filter_4k.cu, bgo_filter_4k_s.cu) so
// that they compile in parallel.  The algorithm and its exactness argument are
// at the top of bgo_filter.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bgo_device.cuh"
#include "bgo_internal.cuh"
#include "bgo_seed_kernel.cuh"

namespace bgo {

#ifndef BGO_FILTER_THREADS
#define BGO_FILTER_THREADS 896
#endif
constexpr int kFilterThreads = BGO_FILTER_THREADS;  // one CTA per SM
constexpr int kFilterWarps = kFilterThreads / 32;
constexpr int kClaimChunks = 2;      // chunks per work claim
#ifndef BGO_FILTER_STATIC_QUARTERS
#define BGO_FILTER_STATIC_QUARTERS 3
#endif
// quarters of a family's chunks handed out in a static grid stride
constexpr int kStaticQuarters = BGO_FILTER_STATIC_QUARTERS;
#ifndef BGO_FILTER_PER
#define BGO_FILTER_PER 3
#endif
// list positions per lane in one filter round
constexpr int kFilterPer = BGO_FILTER_PER;
// per-warp survivor queue: up to 31 left from earlier rounds plus one
// round's 32 * kFilterPer
constexpr int kSurvCap = 32 * (kFilterPer + 1);
// a bounded wait on a chunk copy gives up after this many nanoseconds
constexpr unsigned long long kCopyWaitNs = 2000000000ull;
// static shared memory of the kernel (counters, the chunk-order start and
// the warps' index views) stays below this; the dynamic block takes the rest
// of the 227 KB a CTA may hold
constexpr int kFilterStaticSmem = 2048;
// dynamic shared memory a prefiltered form may take
constexpr int kFilterSmemLimit = 227 * 1024 - kFilterStaticSmem;

// Filter regions: the tolerance-1 regions SegT<K, 1> of the segment index,
// keyed by their first <= kFilterKeyLen bases; region j's table of one byte
// per key starts at filt_off<K>(j).
template <int K>
__host__ __device__ constexpr int filt_klen(int j) {
    return SegT<K, 1>::len(j) < kFilterKeyLen ? SegT<K, 1>::len(j) : kFilterKeyLen;
}
template <int K>
__host__ __device__ constexpr uint32_t filt_off(int j) {
    return j == 0 ? 0u : filt_off<K>(j - 1) + (1u << (2 * filt_klen<K>(j - 1)));
}
template <int K>
struct FiltT {
    using G = SegT<K, 1>;
    static constexpr int S = G::S;
    // with no exact region, at least M regions are within one mismatch
    static constexpr int M = 2 * S - K;
    static constexpr uint32_t kBytes = filt_off<K>(S);
    static constexpr uint32_t kBytesAl = (kBytes + 127u) / 128u * 128u;
};

// Per-warp shared-memory slice for chunks of CH positions: two chunk buffers
// (H and L planes, each CH/32 + 4 words; the N plane stays in global memory,
// read only for survivors of chunks whose N summary is set), the compacted
// list of the PAM-passing positions' window starts (position + the family's
// window offset), the survivor queue (plus one slot that absorbs the stores
// of lanes without a survivor) and the two chunk buffers' mbarriers.
template <int CH>
struct FiltChunk {
    static constexpr int kRows = CH / 1024;     // 32-position words per lane
    static constexpr int kWords = CH / 32 + 4;  // + halo, a multiple of 4 words
    static constexpr uint32_t kPlaneBytes = kWords * 4u;
    static constexpr size_t kBuf = 2 * (size_t)kPlaneBytes;
    static constexpr int kListCap = CH >= 4096 ? 512 : 1024;
    static constexpr int kPasses = CH / kListCap;
    static constexpr size_t kListOff = 2 * kBuf;
    // the list array holds whole rounds, so that a round reads entries
    // without a bound check (entries past the list are valid positions)
    static constexpr int kListAlloc =
        (kListCap + 32 * kFilterPer - 1) / (32 * kFilterPer) * (32 * kFilterPer);
    static constexpr size_t kQueueOff = (kListOff + kListAlloc * sizeof(uint16_t) + 15) / 16 * 16;
    static constexpr size_t kBarOff = kQueueOff + (kSurvCap + 1) * sizeof(uint4);
    static constexpr size_t kSlice = kBarOff + 16;
    static_assert(kPlaneBytes % 16 == 0, "bulk copies are whole 16-byte units");
    static_assert(kBuf % 16 == 0 && kQueueOff % 16 == 0 && kSlice % 16 == 0,
                  "slice parts stay 16-byte aligned");
};

// Dynamic shared memory of a form besides the survivor index: filter tables,
// the family's SeedFam and the warps' slices.
template <int K, int CH>
constexpr size_t filter_smem_fixed() {
    return FiltT<K>::kBytesAl + (sizeof(SeedFam) + 15) / 16 * 16 +
           (size_t)kFilterWarps * FiltChunk<CH>::kSlice;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// 1-D bulk copy global -> this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
            "r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Waits for phase `parity` of `bar`; false if it has not completed within
// kCopyWaitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 0u && global_ns() - t0 > kCopyWaitNs) return false;
    }
}

// Bits set in at least two of the S words.
template <int S>
__device__ __forceinline__ uint32_t at_least_two(const uint32_t (&x)[S]) {
    if constexpr (S == 1) {
        return 0u;
    } else if constexpr (S == 2) {
        return x[0] & x[1];
    } else if constexpr (S == 3) {
        return (x[0] & x[1]) | (x[2] & (x[0] | x[1]));
    } else {
        return (x[0] & x[1]) | (x[2] & x[3]) | ((x[0] | x[1]) & (x[2] | x[3]));
    }
}

// The survivor rounds' view of a family's index, held in registers and kept
// small (the filter rounds around it are register-bound).  Shared form: per
// region seg[j] = descriptor start | entry start << 16 (both < 2^16), and
// sizes = descriptors | guide-plane byte offset << 15 of the family's block
// at sidx.  Global form: descriptor starts seg[j] and entry starts ent[j].
template <int K, int ISM>
struct FiltView {
    uint32_t seg[SegT<K, 1>::S];
    uint32_t ent[ISM ? 1 : SegT<K, 1>::S];
    uint32_t sizes;
    uint32_t gbeg;  // first row of the family in the family-sorted guide table
};

// Survivor record: x = h20 | strand index << 31, y = l20, z = N bits of the
// guide window (0 without an N in the 26-position span), w = position.
// The full segment-index check of one survivor per lane (`valid` lanes): per
// region the bucket of the key's single-substitution neighbourhood, then
// every entry's full compare and the N correction (finish_candidate, as in
// scan_seed_kernel).  The index is read from shared memory (ISM: at sidx the
// family's 16-bit descriptors, entry start | count << 12, then the
// family-local guide index of each entry, then the family's guide planes) or
// from global memory (32-bit descriptors, entry start | count << 16, entries
// with their guide planes, entry guide indices).  Returns the entries
// compared.
template <int K, int ISM>
__device__ __forceinline__ uint32_t filter_heavy(const ScanParams &p, const FilterArgs &fa,
                                                 const unsigned char *sidx,
                                                 const FiltView<K, ISM> &fv, uint4 r,
                                                 bool valid) {
    using G = SegT<K, 1>;
    constexpr int S = G::S;
    const uint32_t h20 = r.x & 0xFFFFFu, l20 = r.y;
    const int si = (int)(r.x >> 31);
    const uint32_t ne = (uint32_t)(si ? p.strand[1].n_encoded : p.strand[0].n_encoded);
    const uint64_t slot = (uint64_t)(si ? p.strand[1].slot : p.strand[0].slot);
    const uint64_t pos = (uint64_t)r.w;
    const uint16_t *off16 = reinterpret_cast<const uint16_t *>(sidx);
    const uint16_t *idx16 = off16 + (fv.sizes & 0x7FFFu);
    const uint2 *gpl = reinterpret_cast<const uint2 *>(sidx + (fv.sizes >> 15));
    uint32_t cand = 0;
#pragma unroll
    for (int j = 0; j < S; ++j) {
        const int st = G::start(j), kl = G::klen(j);
        const uint32_t km = (1u << kl) - 1u;
        const uint32_t code = (((h20 >> st) & km) << kl) | ((l20 >> st) & km);
        uint32_t nn, e0;
        if (ISM) {
            const uint32_t d = valid ? off16[(fv.seg[j] & 0xFFFFu) + code] : 0u;
            nn = d >> 12;
            e0 = (fv.seg[j] >> 16) + (d & 0xFFFu);
        } else {
            const uint32_t d = valid ? __ldg(fa.offsets + fv.seg[j] + code) : 0u;
            nn = d >> 16;
            e0 = fv.ent[ISM ? 0 : j] + (d & 0xFFFFu);
        }
        cand += nn;
        for (uint32_t i = 0; i < nn; ++i) {
            uint2 e;
            uint32_t gi = 0;
            if (ISM) {
                gi = idx16[e0 + i];
                e = gpl[gi];
            } else {
                e = __ldg(fa.entries + e0 + i);
            }
            const uint32_t m = (h20 ^ e.x) | (l20 ^ e.y);
            const int cm = __popc(m);
            if (cm <= K) {
                if (!ISM) gi = __ldg(fa.entry_idx + e0 + i);
                if (finish_candidate<K, 1>(p, m, cm, e, gi, j, r.z, ne, slot, pos, fv.gbeg))
                    mark_dropped(pos, slot, p.drop_bits, p.drop_base1);
            }
        }
    }
    return cand;
}

template <int K, int CH, int ISM>
__global__ void __launch_bounds__(kFilterThreads, 1)
    scan_filter_kernel(ScanParams p, FilterArgs fa) {
    using FT = FiltT<K>;
    using G = SegT<K, 1>;
    constexpr int S = G::S;
    using C = FiltChunk<CH>;
    // (its own name: the segment-index kernels in the same translation unit
    // declare the dynamic block with 16-byte alignment)
    extern __shared__ __align__(128) unsigned char filt_smem[];
    uint8_t *sTab = filt_smem;
    SeedFam *sSF = reinterpret_cast<SeedFam *>(filt_smem + FT::kBytesAl);
    unsigned char *sIdxBlk = filt_smem + FT::kBytesAl + (sizeof(SeedFam) + 15) / 16 * 16;
    unsigned char *slices = sIdxBlk + (ISM ? fa.idx_smem_bytes : 0);
    __shared__ unsigned long long sCand;
    __shared__ FiltView<K, ISM> sFV[kFilterWarps];
    static_assert(sizeof(sFV) + 64 <= kFilterStaticSmem, "static shared memory within its reserve");

    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    unsigned char *slice = slices + warp * C::kSlice;
    uint16_t *wList = reinterpret_cast<uint16_t *>(slice + C::kListOff);
    uint4 *wQ = reinterpret_cast<uint4 *>(slice + C::kQueueOff);
    const uint32_t bar0 = smem_u32(slice + C::kBarOff);
    const uint32_t buf0 = smem_u32(slice);

    if (t == 0) sCand = 0;
    // every list entry holds a window start inside the chunk buffer, so that
    // a round may read entries past the list (its lanes keep nothing)
    for (int i = lane; i < C::kListAlloc; i += 32) wList[i] = 0;
    if (lane == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar0 + 8, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();

    // chunk indices fit 32 bits (the host checks tiles_total < 2^31); a
    // rescan scans only the chunks of its list (items index the list)
    const int chunks0 = (int)p.strand[0].n_tiles;
    const int n_chunks = p.chunk_list ? (int)p.n_list : (int)p.tiles_total;
    // the list pointer is read from shared memory where it is used (once per
    // chunk), so that the rounds keep no register for it
    __shared__ const uint32_t *sChunkList;
    if (t == 0) sChunkList = p.chunk_list;
    auto chunk_at = [&](int i) -> int {
        const uint32_t *cl = *(const uint32_t *volatile *)&sChunkList;
        return cl ? (int)cl[i] : i;
    };
    // Copies chunk c's words [c*CH/32, c*CH/32 + kWords) of the H and L planes
    // into buffer b (the planes are padded so that the copy never leaves them,
    // and zero beyond total_bp).  One lane issues the two bulk copies.
    auto issue = [&](int c, int b) {
        if (lane == 0) {
            const bool second = c >= chunks0;
            const int64_t w0 = (int64_t)(second ? c - chunks0 : c) * (CH / 32);
            const StrandDesc &sd = second ? p.strand[1] : p.strand[0];
            const uint32_t dst = buf0 + (uint32_t)(b * C::kBuf);
            const uint32_t bar = bar0 + 8u * (uint32_t)b;
            // the warp's reads of this buffer (generic proxy) come before the
            // copy's writes (async proxy)
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(bar, 2u * C::kPlaneBytes);
            bulk_g2s(dst, sd.H + w0, C::kPlaneBytes, bar);
            bulk_g2s(dst + C::kPlaneBytes, sd.L + w0, C::kPlaneBytes, bar);
        }
    };
    // Chunk order of a warp: the first kStaticQuarters/4 of the chunks in a
    // static grid stride over all warps (no atomics), the rest claimed in runs
    // of kClaimChunks from the family's counter, so that warps that finish
    // early take the tail.  A warp's place in it is three registers: the next
    // chunk, the end of the current stretch and the stride (all warps in the
    // static part, 1 in a claimed run); where the claimed chunks start is in
    // shared memory.
    __shared__ int sDyn0;
    if (t == 0) {
        const int n_warps = (int)gridDim.x * kFilterWarps;
        sDyn0 = (int)((int64_t)n_chunks * kStaticQuarters / 4 / n_warps) * n_warps;
    }
    int run = 0, run_end = 0, step = 0;
    auto start_order = [&]() {
        run = (int)blockIdx.x * kFilterWarps + warp;
        run_end = *(volatile int *)&sDyn0;
        step = (int)gridDim.x * kFilterWarps;
    };
    auto next_chunk = [&](int fi) -> int {
        if (run < run_end) {
            const int c = run;
            run += step;
            return c;
        }
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(fa.work + fi, (uint32_t)kClaimChunks);
        run = *(volatile int *)&sDyn0 + (int)__shfl_sync(0xFFFFFFFFu, c, 0);
        run_end = run + kClaimChunks < n_chunks ? run + kClaimChunks : n_chunks;
        step = 1;
        return run < n_chunks ? run++ : n_chunks;
    };

    uint32_t cand = 0;
    uint32_t phase = 0;  // bit b: parity of buffer b's next completion
    bool dead = false;   // a copy wait gave up: no further work
    const int n_fams = p.fam_end - p.fam_begin;
    for (int fi = 0; fi < n_fams; ++fi) {
        const int f = p.fam_begin + fi;
        const FamilyDesc F = p.fams[f];
        if (fi > 0) __syncthreads();  // every warp is done with the previous tables
        {
            const uint4 *src = reinterpret_cast<const uint4 *>(fa.tables + (size_t)fi * fa.tab_bytes);
            uint4 *dst = reinterpret_cast<uint4 *>(sTab);
            for (int i = t; i < (int)(FT::kBytesAl / 16); i += kFilterThreads) dst[i] = __ldg(src + i);
            for (int i = t; i < (int)(sizeof(SeedFam) / 16); i += kFilterThreads)
                reinterpret_cast<uint4 *>(sSF)[i] =
                    __ldg(reinterpret_cast<const uint4 *>(fa.fams + fi) + i);
            if (ISM) {
                const uint2 sz = fa.fam_sizes[fi];
                // the family's descriptors (16 bits: the host checked that
                // every entry start fits 12 bits and every count 4), the
                // entries' guide indices and the family's guide planes
                const SeedFam &gf = fa.fams[fi];
                const uint32_t off0 = gf.seg[0].off, list0 = gf.list_off;
                uint16_t *dOff = reinterpret_cast<uint16_t *>(sIdxBlk);
                uint16_t *dIdx = dOff + sz.x;
                uint2 *dG =
                    reinterpret_cast<uint2 *>(sIdxBlk + ((sz.x * 2u + sz.y * 2u + 15u) & ~15u));
                for (uint32_t i = t; i < sz.x; i += kFilterThreads) {
                    const uint32_t d = __ldg(fa.offsets + off0 + i);
                    dOff[i] = (uint16_t)((d & 0xFFFu) | ((d >> 16) << 12));
                }
                for (uint32_t i = t; i < sz.y; i += kFilterThreads)
                    dIdx[i] = __ldg(fa.entry_idx + list0 + i);
                for (int i = t; i < F.gend - F.gbeg; i += kFilterThreads) {
                    const GuideRec g = p.guides[F.gbeg + i];
                    dG[i] = make_uint2(g.h & 0xFFFFFu, g.l & 0xFFFFFu);
                }
            }
        }
        __syncthreads();
        if (dead) continue;

        const uint32_t win_off = F.three_prime ? 0u : (uint32_t)F.plen;
        const int n_tests = sSF->n_tests;
        const bool all_fixed = sSF->pam_generic == 0;
        // the warp's view of the family's survivor index: written by lane 0,
        // read by the survivor checks (kept out of the rounds' registers)
        FiltView<K, ISM> &fv = sFV[warp];
        if (lane == 0) {
            fv.gbeg = (uint32_t)F.gbeg;
            fv.sizes = 0;
            if (ISM) {
                // descriptors < 2^15 (<= 4 regions of 4,096 keys), guide
                // planes at a byte offset < 2^17 (the block stays in 227 KB)
                const uint2 sz = fa.fam_sizes[fi];
                fv.sizes = sz.x | (((sz.x * 2u + sz.y * 2u + 15u) & ~15u) << 15);
            }
#pragma unroll
            for (int j = 0; j < S; ++j) {
                if (ISM) {
                    fv.seg[j] = (sSF->seg[j].off - sSF->seg[0].off) | (sSF->seg[j].ent << 16);
                } else {
                    fv.seg[j] = sSF->seg[j].off;
                    fv.ent[ISM ? 0 : j] = sSF->list_off + sSF->seg[j].ent;
                }
            }
        }
        __syncwarp();
        int qn = 0;  // survivors queued (warp-uniform)

        start_order();
        int cur = next_chunk(fi);
        int buf = 0;
        if (cur < n_chunks) issue(chunk_at(cur), buf);
        while (cur < n_chunks) {
            const int nxt = next_chunk(fi);
            const bool has_next = nxt < n_chunks;
            if (has_next) issue(chunk_at(nxt), buf ^ 1);
            const bool ok = mbar_wait_bounded(bar0 + 8u * (uint32_t)buf, (phase >> buf) & 1u);
            phase ^= 1u << buf;
            if (!__all_sync(0xFFFFFFFFu, ok)) {
                if (lane == 0) atomicOr(fa.err, 1);
                if (has_next) {
                    // let the copy in flight land before the warp leaves
                    mbar_wait_bounded(bar0 + 8u * (uint32_t)(buf ^ 1), (phase >> (buf ^ 1)) & 1u);
                }
                dead = true;
                break;
            }
            const uint32_t *wH = reinterpret_cast<const uint32_t *>(slice + buf * C::kBuf);
            const uint32_t *wL = wH + C::kWords;
            const int chunk = chunk_at(cur);
            const bool second = chunk >= chunks0;
            const uint32_t lc = (uint32_t)(second ? chunk - chunks0 : chunk);
            const uint32_t total_bp =
                (uint32_t)(second ? p.strand[1].total_bp : p.strand[0].total_bp);
            // an N in the chunk's words [lc * CH/32, + kWords): summary bits
            // [g0, g0 + CH/1024 + 1) of groups of 32 words
            bool has_n = false;
            {
                const uint32_t *ns = second ? p.strand[1].nsum : p.strand[0].nsum;
                if (ns) {
                    const uint32_t g0 = lc * (uint32_t)(CH / 1024);
                    const uint32_t lo = __ldg(ns + (g0 >> 5)), hi = __ldg(ns + (g0 >> 5) + 1);
                    has_n = (sfshr(lo, hi, g0 & 31u) & ((2u << (CH / 1024)) - 1u)) != 0u;
                }
            }
            const uint32_t strand_bit = second ? 0x80000000u : 0u;
            // positions [0, lim) of this chunk are scanned (total_bp - 26
            // overall); total_bp < 2^32, and a chunk starts below total_bp - 26
            const uint32_t base32 = lc * (uint32_t)CH;
            const uint32_t left = total_bp - (uint32_t)kSiteSpan - base32;
            const int lim = left > (uint32_t)CH ? CH : (int)left;

            // PAM tests of the lane's words (funnel shifts + LOP3).  The
            // families in use (NGG, NG, NNGRRT, NNNRRT, NRN) test only fixed
            // bits; the allowed-set form runs only for S, W and the three-base
            // codes.  A chunk with more passing positions than the list holds
            // runs the tests again for each further pass, so that no pass word
            // stays live through the rounds.
            auto pam_pass = [&](uint32_t (&pass)[C::kRows]) {
                uint32_t hw[C::kRows][2], lw[C::kRows][2];
#pragma unroll
                for (int u = 0; u < C::kRows; ++u) {
                    const int wi = u * 32 + lane;
                    const int rem = lim - 32 * wi;
                    pass[u] = rem >= 32 ? 0xFFFFFFFFu : (rem <= 0 ? 0u : (1u << rem) - 1u);
                    hw[u][0] = wH[wi];
                    hw[u][1] = wH[wi + 1];
                    lw[u][0] = wL[wi];
                    lw[u][1] = wL[wi + 1];
                }
#pragma unroll 1
                for (int k = 0; k < n_tests; ++k) {
                    const uint32_t sh = sSF->pam_shift[k];
                    const uint4 m = sSF->pam_mask[k];
                    if (all_fixed || !((sSF->pam_generic >> k) & 1u)) {
#pragma unroll
                        for (int u = 0; u < C::kRows; ++u) {
                            const uint32_t h = sfshr(hw[u][0], hw[u][1], sh);
                            const uint32_t l = sfshr(lw[u][0], lw[u][1], sh);
                            pass[u] &= ~(((h ^ m.x) & m.y) | ((l ^ m.z) & m.w));
                        }
                    } else {
#pragma unroll
                        for (int u = 0; u < C::kRows; ++u) {
                            const uint32_t h = sfshr(hw[u][0], hw[u][1], sh);
                            const uint32_t l = sfshr(lw[u][0], lw[u][1], sh);
                            pass[u] &= (~h & ~l & m.x) | (~h & l & m.y) | (h & ~l & m.z) |
                                       (h & l & m.w);
                        }
                    }
                }
            };
            int total = 0;
#pragma unroll 1
            for (int pass_i = 0; pass_i < C::kPasses; ++pass_i) {
                // a further pass only while listed positions remain (the
                // tests are not run again to find that the chunk is done)
                if (pass_i > 0 && pass_i * C::kListCap >= total) break;
                uint32_t pass[C::kRows];
                pam_pass(pass);
                // The list is row-major: row u's positions of lanes 0..31, then
                // row u + 1's.  A round's lanes then read window words of
                // neighbouring lanes' words, which lie in different banks (a
                // lane-major list put a round's positions in one lane's words,
                // all in the same bank).  Row offsets: one warp scan per two
                // rows, the two counts in 16-bit halves (sums <= 1,024).
                int rowoff[C::kRows];
                {
                    int base = 0;
#pragma unroll
                    for (int h = 0; h < C::kRows / 2; ++h) {
                        const uint32_t pk = (uint32_t)__popc(pass[2 * h]) |
                                            ((uint32_t)__popc(pass[2 * h + 1]) << 16);
                        uint32_t incl = pk;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                            if (lane >= o) incl += v;
                        }
                        const uint32_t tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
                        const uint32_t ex = incl - pk;
                        rowoff[2 * h] = base + (int)(ex & 0xFFFFu);
                        base += (int)(tot & 0xFFFFu);
                        rowoff[2 * h + 1] = base + (int)(ex >> 16);
                        base += (int)(tot >> 16);
                    }
                    if (pass_i == 0) total = base;
                }
                const int lo = pass_i * C::kListCap;
                if (lo >= total) break;
                const int n_list = min(total - lo, C::kListCap);
                // list positions [lo, lo + n_list) of the chunk's passing
                // positions (the order within a lane's word is irrelevant: each
                // word is walked from its highest passing bit)
                if (total <= C::kListCap) {
#pragma unroll
                    for (int u = 0; u < C::kRows; ++u) {
                        uint16_t *out = wList + rowoff[u];
                        uint32_t m = pass[u];
                        const uint32_t wb = 32u * (uint32_t)(u * 32 + lane) + 31u + win_off;
                        // three steps without a loop branch (most words hold at
                        // most three passing positions; the loop after them runs
                        // as long as the warp's fullest word needs), then the
                        // rest
#pragma unroll
                        for (int it = 0; it < 3; ++it) {
                            const uint32_t z = __clz(m);
                            if (m) *out = (uint16_t)(wb - z);
                            out += m ? 1 : 0;
                            m &= ~(uint32_t)(0x80000000ull >> z);  // z = 32 when m = 0
                        }
                        while (m) {
                            const uint32_t z = __clz(m);
                            m ^= 0x80000000u >> z;
                            *out++ = (uint16_t)(wb - z);
                        }
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < C::kRows; ++u) {
                        int off = rowoff[u] - lo;
                        uint32_t m = pass[u];
                        const uint32_t wb = 32u * (uint32_t)(u * 32 + lane) + 31u + win_off;
                        while (m) {
                            const uint32_t z = __clz(m);
                            m ^= 0x80000000u >> z;
                            if ((unsigned)off < (unsigned)n_list) wList[off] = (uint16_t)(wb - z);
                            ++off;
                        }
                    }
                }
                __syncwarp();
                for (int k0 = 0; k0 < n_list; k0 += 32 * kFilterPer) {
                    // filter: one byte per region key (bit 0: a guide's key
                    // equals it; bits 1-7: colours of the guides within one
                    // mismatch of it).  Lanes past the list read a stale or
                    // initial entry (a window start inside the buffer) and
                    // keep nothing.
                    uint32_t sv[kFilterPer], hv[kFilterPer], lv[kFilterPer];
                    bool keep[kFilterPer];
#pragma unroll
                    for (int v = 0; v < kFilterPer; ++v) {
                        const int k = k0 + v * 32 + lane;
                        const bool has = k < n_list;
                        const uint32_t wo = wList[k];  // the window's start (position + win_off)
                        const uint32_t s = wo - win_off;
                        const uint32_t wi = wo >> 5, b = wo & 31u;
                        const uint32_t h20 = sfshr(wH[wi], wH[wi + 1], b);
                        const uint32_t l20 = sfshr(wL[wi], wL[wi + 1], b);
                        uint32_t x[S];
#pragma unroll
                        for (int j = 0; j < S; ++j) {
                            const int st = G::start(j), kl = filt_klen<K>(j);
                            const uint32_t km = (1u << kl) - 1u;
                            const uint32_t code = (((h20 >> st) & km) << kl) | ((l20 >> st) & km);
                            x[j] = sTab[filt_off<K>(j) + code];
                        }
                        uint32_t any = 0;
#pragma unroll
                        for (int j = 0; j < S; ++j) any |= x[j];
                        bool kp;
                        if constexpr (FT::M <= 1) {
                            kp = (any & 0xFEu) != 0u;
                        } else if constexpr (FT::M > S) {
                            kp = (any & 1u) != 0u;
                        } else {
                            kp = ((any & 1u) | (at_least_two<S>(x) & 0xFEu)) != 0u;
                        }
                        sv[v] = s;
                        hv[v] = h20;
                        lv[v] = l20;
                        keep[v] = has && kp;
                    }
                    // the round's survivors into the queue at once, then a
                    // warp of them through the index while the queue holds one
                    uint32_t bal[kFilterPer], any_bal = 0;
#pragma unroll
                    for (int v = 0; v < kFilterPer; ++v) {
                        bal[v] = __ballot_sync(0xFFFFFFFFu, keep[v]);
                        any_bal |= bal[v];
                    }
                    if (any_bal) {
#pragma unroll
                        for (int v = 0; v < kFilterPer; ++v) {
                            const uint32_t s = sv[v];
                            uint32_t n20g = 0;
                            if (has_n && keep[v]) {  // a survivor's s is a listed position
                                // the chunk's N words, from global memory
                                const uint32_t *gN =
                                    (strand_bit ? p.strand[1].N : p.strand[0].N) + (base32 >> 5);
                                const uint32_t wo = s + win_off;
                                const uint32_t n26 = sfshr(__ldg(gN + (s >> 5)),
                                                           __ldg(gN + (s >> 5) + 1), s & 31u) &
                                                     0x3FFFFFFu;
                                const uint32_t n20 = sfshr(__ldg(gN + (wo >> 5)),
                                                           __ldg(gN + (wo >> 5) + 1), wo & 31u) &
                                                     0xFFFFFu;
                                n20g = n26 ? n20 : 0u;
                            }
                            // a lane without a survivor stores into the spare slot
                            const int at = keep[v] ? qn + __popc(bal[v] & lt_mask) : kSurvCap;
                            wQ[at] = make_uint4((hv[v] & 0xFFFFFu) | strand_bit, lv[v] & 0xFFFFFu,
                                                n20g, base32 + s);
                            qn += __popc(bal[v]);
                        }
                        while (qn >= 32) {
                            __syncwarp();
                            cand += filter_heavy<K, ISM>(p, fa, sIdxBlk, fv, wQ[qn - 32 + lane],
                                                         true);
                            qn -= 32;
                            __syncwarp();
                        }
                    }
                }
                __syncwarp();  // the next pass overwrites the list
            }
            if (!has_next) break;
            cur = nxt;
            buf ^= 1;
        }
        // the family's remaining survivors
        if (qn > 0) {
            __syncwarp();
            const bool v = lane < qn;
            cand += filter_heavy<K, ISM>(p, fa, sIdxBlk, fv, wQ[v ? lane : 0], v);
            __syncwarp();
        }
    }
    for (int o = 16; o > 0; o >>= 1) cand += __shfl_down_sync(0xFFFFFFFFu, cand, o);
    if (lane == 0 && cand) atomicAdd(&sCand, (unsigned long long)cand);
    __syncthreads();
    if (t == 0 && sCand) atomicAdd(p.counter + 1, sCand);
}

template <int K, int CH, int ISM>
static int launch_filter_k(const ScanParams &p, const FilterArgs &fa, int sm_count,
                           cudaStream_t s) {
    const size_t smem = filter_smem_fixed<K, CH>() + (ISM ? (size_t)fa.idx_smem_bytes : 0);
    static_assert(filter_smem_fixed<K, CH>() <= kFilterSmemLimit, "filter form fits in shared memory");
    static size_t configured = 0;
    if (smem > configured) {
        BGO_CUDA(cudaFuncSetAttribute(scan_filter_kernel<K, CH, ISM>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = smem;
    }
    // one persistent CTA per SM; warps take chunks in a grid stride, then
    // claim the rest from per-family counters
    scan_filter_kernel<K, CH, ISM><<<(unsigned)sm_count, kFilterThreads, smem, s>>>(p, fa);
    BGO_CUDA(cudaGetLastError());
    return BGO_OK;
}

template <int CH, int ISM>
static int launch_filter_ch(const ScanParams &p, const FilterArgs &fa, int sm_count,
                            cudaStream_t s) {
    switch (p.max_mm) {
        case 0: return launch_filter_k<0, CH, ISM>(p, fa, sm_count, s);
        case 1: return launch_filter_k<1, CH, ISM>(p, fa, sm_count, s);
        case 2: return launch_filter_k<2, CH, ISM>(p, fa, sm_count, s);
        case 3: return launch_filter_k<3, CH, ISM>(p, fa, sm_count, s);
        case 4: return launch_filter_k<4, CH, ISM>(p, fa, sm_count, s);
        case 5: return launch_filter_k<5, CH, ISM>(p, fa, sm_count, s);
        case 6: return launch_filter_k<6, CH, ISM>(p, fa, sm_count, s);
        case 7: return launch_filter_k<7, CH, ISM>(p, fa, sm_count, s);
        default:
            set_error("prefiltered segment index: max_mismatches outside 0..7");
            return BGO_ERR_ARG;
    }
}

}  // namespace bgo
