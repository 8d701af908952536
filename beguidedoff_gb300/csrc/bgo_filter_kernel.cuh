// Prefiltered segment-index scan kernel (scan mode 2 with tuning.prefilter),
// included by the translation units that instantiate its chunk lengths
// (bgo_filter.cu: 2,048 positions, bgo_filter_4k.cu: 4,096) so that they
// compile in parallel.  The algorithm and its exactness argument are at the
// top of bgo_filter.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bgo_device.cuh"
#include "bgo_internal.cuh"
#include "bgo_seed_kernel.cuh"

namespace bgo {

constexpr int kFilterThreads = 768;  // one CTA per SM, 24 warps
constexpr int kFilterWarps = kFilterThreads / 32;
constexpr int kSurvCap = 64;         // per-warp survivor queue (two rounds)
constexpr int kClaimChunks = 4;      // chunks per work claim
// a bounded wait on a chunk copy gives up after this many nanoseconds
constexpr unsigned long long kCopyWaitNs = 2000000000ull;

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
// (H, L, N planes, each CH/32 + 4 words), the compacted list of PAM-passing
// positions, the survivor queue and the two chunk buffers' mbarriers.
template <int CH>
struct FiltChunk {
    static constexpr int kRows = CH / 1024;     // 32-position words per lane
    static constexpr int kWords = CH / 32 + 4;  // + halo, a multiple of 4 words
    static constexpr uint32_t kPlaneBytes = kWords * 4u;
    static constexpr size_t kBuf = 3 * (size_t)kPlaneBytes;
    static constexpr int kListCap = 1024;
    static constexpr int kPasses = CH / kListCap;
    static constexpr size_t kListOff = 2 * kBuf;
    static constexpr size_t kQueueOff = kListOff + kListCap * sizeof(uint16_t);
    static constexpr size_t kBarOff = kQueueOff + kSurvCap * sizeof(uint4);
    static constexpr size_t kSlice = kBarOff + 16;
    static_assert(kPlaneBytes % 16 == 0, "bulk copies are whole 16-byte units");
    static_assert(kBuf % 16 == 0 && kQueueOff % 16 == 0 && kSlice % 16 == 0,
                  "slice parts stay 16-byte aligned");
};

template <int K, int CH>
constexpr size_t filter_smem_bytes() {
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

// Survivor record: x = h20 | strand index << 31, y = l20, z = N bits of the
// guide window (0 without an N in the 26-position span), w = position.
// The full segment-index check of one survivor per lane (`valid` lanes).
template <int K>
__device__ __forceinline__ void filter_heavy(const ScanParams &p, const FilterArgs &fa, uint4 r,
                                             bool valid, const uint32_t (&seg_off)[SegT<K, 1>::S],
                                             const uint32_t (&seg_ent)[SegT<K, 1>::S],
                                             uint32_t gbeg, uint32_t &cand) {
    using G = SegT<K, 1>;
    constexpr int S = G::S;
    const uint32_t h20 = r.x & 0xFFFFFu, l20 = r.y;
    const int si = (int)(r.x >> 31);
    const uint32_t ne = (uint32_t)(si ? p.strand[1].n_encoded : p.strand[0].n_encoded);
    const uint64_t slot = (uint64_t)(si ? p.strand[1].slot : p.strand[0].slot);
    const uint64_t pos = (uint64_t)r.w;
#pragma unroll
    for (int j = 0; j < S; ++j) {
        const int st = G::start(j), kl = G::klen(j);
        const uint32_t km = (1u << kl) - 1u;
        const uint32_t code = (((h20 >> st) & km) << kl) | ((l20 >> st) & km);
        const uint32_t d = valid ? __ldg(fa.offsets + seg_off[j] + code) : 0u;
        const uint32_t nn = d >> 16, e0 = seg_ent[j] + (d & 0xFFFFu);
        cand += nn;
        for (uint32_t i = 0; i < nn; ++i) {
            const uint2 e = __ldg(fa.entries + e0 + i);
            const uint32_t m = (h20 ^ e.x) | (l20 ^ e.y);
            const int cm = __popc(m);
            if (cm <= K)
                finish_candidate<K, 1>(p, m, cm, e, __ldg(fa.entry_idx + e0 + i), j, r.z, ne,
                                       slot, pos, gbeg);
        }
    }
}

template <int K, int CH>
__global__ void __launch_bounds__(kFilterThreads, 1)
    scan_filter_kernel(ScanParams p, FilterArgs fa) {
    using FT = FiltT<K>;
    using G = SegT<K, 1>;
    constexpr int S = G::S;
    using C = FiltChunk<CH>;
    extern __shared__ __align__(128) unsigned char smem[];
    uint8_t *sTab = smem;
    SeedFam *sSF = reinterpret_cast<SeedFam *>(smem + FT::kBytesAl);
    unsigned char *slices = smem + FT::kBytesAl + (sizeof(SeedFam) + 15) / 16 * 16;
    __shared__ unsigned long long sCand;

    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
    unsigned char *slice = slices + warp * C::kSlice;
    uint16_t *wList = reinterpret_cast<uint16_t *>(slice + C::kListOff);
    uint4 *wQ = reinterpret_cast<uint4 *>(slice + C::kQueueOff);
    const uint32_t bar0 = smem_u32(slice + C::kBarOff);
    const uint32_t buf0 = smem_u32(slice);

    if (t == 0) sCand = 0;
    if (lane == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar0 + 8, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();

    const int64_t chunks0 = p.strand[0].n_tiles;
    const int64_t n_chunks = p.tiles_total;
    // Copies chunk c's words [c*CH/32, c*CH/32 + kWords) of the three planes
    // into buffer b (the planes are padded so that the copy never leaves them,
    // and zero beyond total_bp).  One lane issues the three bulk copies.
    auto issue = [&](int64_t c, int b) {
        if (lane == 0) {
            const bool second = c >= chunks0;
            const int64_t w0 = (second ? c - chunks0 : c) * (CH / 32);
            const StrandDesc &sd = second ? p.strand[1] : p.strand[0];
            const uint32_t dst = buf0 + (uint32_t)(b * C::kBuf);
            const uint32_t bar = bar0 + 8u * (uint32_t)b;
            // the warp's reads of this buffer (generic proxy) come before the
            // copy's writes (async proxy)
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(bar, 3u * C::kPlaneBytes);
            bulk_g2s(dst, sd.H + w0, C::kPlaneBytes, bar);
            bulk_g2s(dst + C::kPlaneBytes, sd.L + w0, C::kPlaneBytes, bar);
            bulk_g2s(dst + 2u * C::kPlaneBytes, sd.N + w0, C::kPlaneBytes, bar);
        }
    };
    auto claim = [&](int fi) -> int64_t {
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(fa.work + fi, (uint32_t)kClaimChunks);
        return (int64_t)__shfl_sync(0xFFFFFFFFu, c, 0);
    };

    uint32_t cand = 0;
    uint32_t phase = 0;  // bit b: parity of buffer b's next completion
    bool dead = false;   // a copy wait gave up: no further work
    const int n_fams = p.fam_end - p.fam_begin;
    for (int fi = 0; fi < n_fams; ++fi) {
        const int f = p.fam_begin + fi;
        if (fi > 0) __syncthreads();  // every warp is done with the previous tables
        {
            const uint4 *src = reinterpret_cast<const uint4 *>(fa.tables + (size_t)fi * fa.tab_bytes);
            uint4 *dst = reinterpret_cast<uint4 *>(sTab);
            for (int i = t; i < (int)(FT::kBytesAl / 16); i += kFilterThreads) dst[i] = __ldg(src + i);
            for (int i = t; i < (int)(sizeof(SeedFam) / 16); i += kFilterThreads)
                reinterpret_cast<uint4 *>(sSF)[i] =
                    __ldg(reinterpret_cast<const uint4 *>(fa.fams + fi) + i);
        }
        __syncthreads();
        if (dead) continue;

        const FamilyDesc F = p.fams[f];
        const uint32_t win_off = F.three_prime ? 0u : (uint32_t)F.plen;
        const uint32_t gbeg = (uint32_t)F.gbeg;
        const int n_tests = sSF->n_tests;
        uint32_t seg_off[S], seg_ent[S];
#pragma unroll
        for (int j = 0; j < S; ++j) {
            seg_off[j] = sSF->seg[j].off;
            seg_ent[j] = sSF->list_off + sSF->seg[j].ent;
        }
        int qn = 0;  // survivors queued (warp-uniform)

        int64_t cur = claim(fi);
        int64_t cend = cur + kClaimChunks < n_chunks ? cur + kClaimChunks : n_chunks;
        int buf = 0;
        if (cur < n_chunks) issue(cur, buf);
        while (cur < n_chunks) {
            int64_t nxt = cur + 1;
            if (nxt >= cend) {
                nxt = claim(fi);
                cend = nxt + kClaimChunks < n_chunks ? nxt + kClaimChunks : n_chunks;
            }
            const bool has_next = nxt < n_chunks;
            if (has_next) issue(nxt, buf ^ 1);
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
            const uint32_t *wN = wL + C::kWords;
            const bool second = cur >= chunks0;
            const int64_t lc = second ? cur - chunks0 : cur;
            const int64_t total_bp = second ? p.strand[1].total_bp : p.strand[0].total_bp;
            int has_n = second ? p.strand[1].has_n : p.strand[0].has_n;
            if (has_n) {
                uint32_t nw = 0;
                for (int i = lane; i < C::kWords; i += 32) nw |= wN[i];
                has_n = __any_sync(0xFFFFFFFFu, nw != 0u);
            }
            const uint32_t strand_bit = second ? 0x80000000u : 0u;
            const int64_t base = lc * CH;
            const int64_t lim64 = total_bp - kSiteSpan - base;
            const int lim = lim64 > CH ? CH : (int)lim64;

            // PAM tests of the lane's words (funnel shifts + LOP3)
            uint32_t pass[C::kRows], hw[C::kRows][2], lw[C::kRows][2];
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
                const bool generic = (sSF->pam_generic >> k) & 1u;
#pragma unroll
                for (int u = 0; u < C::kRows; ++u) {
                    const uint32_t h = sfshr(hw[u][0], hw[u][1], sh);
                    const uint32_t l = sfshr(lw[u][0], lw[u][1], sh);
                    pass[u] &= generic ? (~h & ~l & m.x) | (~h & l & m.y) | (h & ~l & m.z) |
                                             (h & l & m.w)
                                       : ~(((h ^ m.x) & m.y) | ((l ^ m.z) & m.w));
                }
            }
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < C::kRows; ++u) cnt += __popc(pass[u]);
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            const int off0 = incl - cnt;
#pragma unroll 1
            for (int pass_i = 0; pass_i < C::kPasses; ++pass_i) {
                const int lo = pass_i * C::kListCap;
                if (lo >= total) break;
                const int n_list = min(total - lo, C::kListCap);
                // list positions [lo, lo + n_list) of the chunk's passing positions
                if (total <= C::kListCap) {
                    int off = off0;
#pragma unroll
                    for (int u = 0; u < C::kRows; ++u) {
                        uint32_t m = pass[u];
                        while (m) {
                            const int j = __ffs(m) - 1;
                            m &= m - 1u;
                            wList[off++] = (uint16_t)(32 * (u * 32 + lane) + j);
                        }
                    }
                } else if (off0 + cnt > lo && off0 < lo + n_list) {
                    int off = off0 - lo;
#pragma unroll
                    for (int u = 0; u < C::kRows; ++u) {
                        uint32_t m = pass[u];
                        while (m) {
                            const int j = __ffs(m) - 1;
                            m &= m - 1u;
                            if ((unsigned)off < (unsigned)n_list)
                                wList[off] = (uint16_t)(32 * (u * 32 + lane) + j);
                            ++off;
                        }
                    }
                }
                __syncwarp();
                for (int k0 = 0; k0 < n_list; k0 += 32) {
                    const int k = k0 + lane;
                    const bool has = k < n_list;
                    uint32_t s = 0, h20 = 0, l20 = 0;
                    bool keep = false;
                    if (has) {
                        s = wList[k];
                        const uint32_t wo = s + win_off;
                        const uint32_t wi = wo >> 5, b = wo & 31u;
                        h20 = sfshr(wH[wi], wH[wi + 1], b);
                        l20 = sfshr(wL[wi], wL[wi + 1], b);
                        // filter: one byte per region key (bit 0: a guide's key
                        // equals it; bits 1-7: colours of the guides within one
                        // mismatch of it)
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
                        if constexpr (FT::M <= 1) {
                            keep = (any & 0xFEu) != 0u;
                        } else if constexpr (FT::M > S) {
                            keep = (any & 1u) != 0u;
                        } else {
                            keep = ((any & 1u) | (at_least_two<S>(x) & 0xFEu)) != 0u;
                        }
                    }
                    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
                    if (bal) {
                        if (keep) {
                            uint32_t n20g = 0;
                            if (has_n) {
                                const uint32_t n26 =
                                    sfshr(wN[s >> 5], wN[(s >> 5) + 1], s & 31u) & 0x3FFFFFFu;
                                if (n26) {
                                    const uint32_t wo = s + win_off;
                                    n20g = sfshr(wN[wo >> 5], wN[(wo >> 5) + 1], wo & 31u) &
                                           0xFFFFFu;
                                }
                            }
                            const int at = qn + __popc(bal & ((1u << lane) - 1u));
                            wQ[at] = make_uint4((h20 & 0xFFFFFu) | strand_bit, l20 & 0xFFFFFu, n20g,
                                                (uint32_t)(base + s));
                        }
                        qn += __popc(bal);
                        if (qn >= 32) {
                            __syncwarp();
                            filter_heavy<K>(p, fa, wQ[qn - 32 + lane], true, seg_off, seg_ent,
                                            gbeg, cand);
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
            filter_heavy<K>(p, fa, wQ[v ? lane : 0], v, seg_off, seg_ent, gbeg, cand);
            __syncwarp();
        }
    }
    for (int o = 16; o > 0; o >>= 1) cand += __shfl_down_sync(0xFFFFFFFFu, cand, o);
    if (lane == 0 && cand) atomicAdd(&sCand, (unsigned long long)cand);
    __syncthreads();
    if (t == 0 && sCand) atomicAdd(p.counter + 1, sCand);
}

template <int K, int CH>
static int launch_filter_k(const ScanParams &p, const FilterArgs &fa, int sm_count,
                           cudaStream_t s) {
    constexpr size_t smem = filter_smem_bytes<K, CH>();
    static_assert(smem <= 227 * 1024, "filter form fits in shared memory");
    static bool configured = false;
    if (!configured) {
        BGO_CUDA(cudaFuncSetAttribute(scan_filter_kernel<K, CH>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
    }
    // one persistent CTA per SM; warps claim chunks from per-family counters
    scan_filter_kernel<K, CH><<<(unsigned)sm_count, kFilterThreads, smem, s>>>(p, fa);
    BGO_CUDA(cudaGetLastError());
    return BGO_OK;
}

template <int CH>
static int launch_filter_ch(const ScanParams &p, const FilterArgs &fa, int sm_count,
                            cudaStream_t s) {
    switch (p.max_mm) {
        case 0: return launch_filter_k<0, CH>(p, fa, sm_count, s);
        case 1: return launch_filter_k<1, CH>(p, fa, sm_count, s);
        case 2: return launch_filter_k<2, CH>(p, fa, sm_count, s);
        case 3: return launch_filter_k<3, CH>(p, fa, sm_count, s);
        case 4: return launch_filter_k<4, CH>(p, fa, sm_count, s);
        case 5: return launch_filter_k<5, CH>(p, fa, sm_count, s);
        case 6: return launch_filter_k<6, CH>(p, fa, sm_count, s);
        case 7: return launch_filter_k<7, CH>(p, fa, sm_count, s);
        default:
            set_error("prefiltered segment index: max_mismatches outside 0..7");
            return BGO_ERR_ARG;
    }
}

}  // namespace bgo
