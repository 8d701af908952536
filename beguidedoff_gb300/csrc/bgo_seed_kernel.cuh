// Segment-indexed scan kernel (scan mode 2), included by the translation
// units that instantiate its forms - tolerance 0 with one inline guide per
// bucket and the warp range queue (bgo_seed.cu) or the per-lane walk
// (bgo_seed_walk.cu), tolerance 0 with two inline guides (bgo_seed_i2.cu),
// tolerance 1 with two and the walk (bgo_seed_t1.cu) - so that they compile in
// parallel.  The algorithm is described at the top of bgo_seed.cu.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "bgo_device.cuh"
#include "bgo_internal.cuh"

namespace bgo {

constexpr int kQueueCap = 32 * (kSeedMaxK + 1);  // bucket ranges per round

// Per-warp shared-memory slice for chunks of CH positions: two chunk buffers
// (H, L, N planes), the compacted list of passing positions, and, unless the
// lanes walk their own
// leftover guides (WALK), the round's position records and the bucket-range
// queue (word + count).
template <int CH, int WALK>
struct SeedChunk {
    static constexpr int kRows = CH / 1024;      // 32-position words per lane
    static constexpr int kWords = CH / 32 + 4;   // + halo, a multiple of 4 words
    static constexpr int kVecs = kWords / 4;     // 16-byte copies per plane
    static constexpr size_t kBuf = 3 * kWords * sizeof(uint32_t);
    static constexpr size_t kListOff = 2 * kBuf;
    // the list holds up to 1,024 positions; a 2,048-position chunk with more
    // passing positions is worked through in two passes
    static constexpr int kListCap = CH < 1024 ? CH : 1024;
    static constexpr int kPasses = CH / kListCap;
    static constexpr size_t kRecOff = (kListOff + kListCap * sizeof(uint16_t) + 15) / 16 * 16;
    static constexpr size_t kQueueOff = kRecOff + 32 * sizeof(uint4);
    static constexpr size_t kCountOff = kQueueOff + kQueueCap * sizeof(uint32_t);
    static constexpr size_t kSlice =
        WALK ? kRecOff : (kCountOff + kQueueCap * sizeof(uint16_t) + 15) / 16 * 16;
    static_assert(kWords % 4 == 0, "chunk copies are whole 16-byte vectors");
    static_assert(kBuf % 16 == 0, "chunk buffers stay 16-byte aligned");
};

// The key regions for K mismatches and tolerance TOL: S = K / (TOL + 1) + 1
// disjoint segments over the 20 guide positions, keyed by their first <= 6
// bases.  S * (TOL + 1) > K, so every hit has a region with <= TOL mismatches.
template <int K, int TOL>
struct SegT {
    static constexpr int S = K / (TOL + 1) + 1;
    static constexpr int q = kGuideLen / S, r = kGuideLen % S;
    __host__ __device__ static constexpr int start(int j) { return j * q + (j < r ? j : r); }
    __host__ __device__ static constexpr int len(int j) { return q + (j < r ? 1 : 0); }
    __host__ __device__ static constexpr int klen(int j) {
        return len(j) < kMaxKeyLen ? len(j) : kMaxKeyLen;
    }
};

// The full check of a candidate whose raw count cm <= K, found through
// region j: emits the hit if j is its first region with <= TOL mismatches
// and it stays within K after the N correction.  Returns true when the hit
// did not fit the hit buffer (the caller marks its granule).  Inlined: as a
// call, its calling convention spilled registers of every kernel that uses it
// (the prefiltered kernel at 72 registers spilled 56 bytes; inlined, none).
template <int K, int TOL>
__device__ __forceinline__ bool finish_candidate(const ScanParams &p, uint32_t m, int cm, uint2 e,
                                              uint32_t idx, int j, uint32_t n20g, uint32_t ne,
                                              uint64_t slot, uint64_t pos, uint32_t gbeg) {
    using G = SegT<K, TOL>;
    bool first = true;
#pragma unroll
    for (int jj = 0; jj < G::S - 1; ++jj)
        if (jj < j)
            first = first && __popc((m >> G::start(jj)) & ((1u << G::klen(jj)) - 1u)) > TOL;
    if (!first) return false;
    int mmf = cm;
    if (n20g) {
        const uint32_t eh = (ne & 2u) ? e.x : ~e.x;
        const uint32_t el = (ne & 1u) ? e.y : ~e.y;
        mmf = cm + __popc(n20g & eh & el);
    }
    if (mmf > K) return false;
    const uint32_t row = __ldg(&p.guides[gbeg + idx].row);
    return semit(((uint64_t)row << 39) | (slot << 38) | (pos << 6) | (uint64_t)mmf, p.keys, p.cap,
                 p.counter);
}

// CTA shapes by MINB: 3 or 4 CTAs of 256 threads per SM; or one CTA per SM
// whose warps share a large index, of 768 threads (MINB = 1, 24 warps) or 512
// (MINB = 2, 16 warps, for an index too large to leave room for 24 warps'
// chunk slices).
template <int MINB>
struct SeedCta {
    static constexpr int kThreads = MINB == 1 ? 768 : MINB == 2 ? 512 : kSeedThreads;
    static constexpr int kWarps = kThreads / 32;
    static constexpr int kPerSm = MINB <= 2 ? 1 : MINB;
};

template <int K, int TOL, int INLINE, int WALK, int CH, int MINB>
__global__ void __launch_bounds__(SeedCta<MINB>::kThreads, SeedCta<MINB>::kPerSm)
    scan_seed_kernel(ScanParams p, SeedArgs sa) {
    constexpr int THREADS = SeedCta<MINB>::kThreads;
    constexpr int WARPS = SeedCta<MINB>::kWarps;
    using G = SegT<K, TOL>;
    constexpr int S = G::S;
    using C = SeedChunk<CH, WALK>;
    extern __shared__ __align__(16) unsigned char smem[];
    SeedFam *sFam = reinterpret_cast<SeedFam *>(smem);
    uint2 *sEnt = reinterpret_cast<uint2 *>(sFam + sa.n_fams);
    uint32_t *sOff = reinterpret_cast<uint32_t *>(sEnt + sa.n_lists);
    uint16_t *sIdx = reinterpret_cast<uint16_t *>(sOff + sa.n_offsets);
    unsigned char *slices =
        smem + ((sizeof(SeedFam) * sa.n_fams + sizeof(uint2) * sa.n_lists +
                 sizeof(uint32_t) * sa.n_offsets + sizeof(uint16_t) * sa.n_lists + 15) / 16 * 16);
    __shared__ unsigned long long sCand;

    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
    unsigned char *slice = slices + warp * C::kSlice;
    uint16_t *wList = reinterpret_cast<uint16_t *>(slice + C::kListOff);
    uint4 *wRec = reinterpret_cast<uint4 *>(slice + C::kRecOff);
    uint32_t *wQ = reinterpret_cast<uint32_t *>(slice + C::kQueueOff);
    uint16_t *wCnt = reinterpret_cast<uint16_t *>(slice + C::kCountOff);

    for (int i = t; i < sa.n_fams; i += THREADS) sFam[i] = sa.fams[i];
    for (int i = t; i < sa.n_lists; i += THREADS) {
        sEnt[i] = sa.entries[i];
        sIdx[i] = sa.entry_idx[i];
    }
    for (int i = t; i < sa.n_offsets; i += THREADS) sOff[i] = sa.offsets[i];
    if (t == 0) sCand = 0;
    __syncthreads();

    const int64_t chunks0 = p.strand[0].n_tiles;
    const int64_t n_chunks = p.tiles_total;
    const int64_t stride = (int64_t)gridDim.x * WARPS;
    // Chunk c's words [c*CH/32, c*CH/32 + kWords) of the three planes, copied
    // into buffer b as 16-byte vectors (the planes are padded so that the copy
    // never leaves them, and zero beyond total_bp).
    auto issue = [&](int64_t c, int b) {
        const bool second = c >= chunks0;
        const int64_t w0 = (second ? c - chunks0 : c) * (CH / 32);
        const StrandDesc &sd = second ? p.strand[1] : p.strand[0];
        uint32_t *dst = reinterpret_cast<uint32_t *>(slice + b * C::kBuf);
        for (int i = lane; i < 3 * C::kVecs; i += 32) {
            const int plane = i / C::kVecs, v = i - plane * C::kVecs;
            const uint32_t *src = plane == 0 ? sd.H : plane == 1 ? sd.L : sd.N;
            cp_async16(dst + plane * C::kWords + 4 * v, src + w0 + 4 * v);
        }
    };
    uint32_t cand = 0;
    // the chunks to scan: all of them, or a rescan's list
    const int64_t n_items = p.chunk_list ? p.n_list : n_chunks;
    auto chunk_at = [&](int64_t i) -> int64_t {
        return p.chunk_list ? (int64_t)p.chunk_list[i] : i;
    };
    const int64_t i_first = (int64_t)blockIdx.x * WARPS + warp;
    if (i_first < n_items) issue(chunk_at(i_first), 0);
    cp_async_commit();
    int buf = 0;
    for (int64_t it = i_first; it < n_items; it += stride, buf ^= 1) {
        const int64_t c = chunk_at(it);
        if (it + stride < n_items) issue(chunk_at(it + stride), buf ^ 1);
        cp_async_commit();
        cp_async_wait<1>();  // this chunk's copies are done; the next one is in flight
        __syncwarp();
        const uint32_t *wH = reinterpret_cast<const uint32_t *>(slice + buf * C::kBuf);
        const uint32_t *wL = wH + C::kWords;
        const uint32_t *wN = wL + C::kWords;
        const bool second = c >= chunks0;
        const int64_t lc = second ? c - chunks0 : c;
        const int64_t total_bp = second ? p.strand[1].total_bp : p.strand[0].total_bp;
        // the N correction applies only in chunks whose words hold an N
        int has_n = second ? p.strand[1].has_n : p.strand[0].has_n;
        if (has_n) {
            uint32_t nw = 0;
            for (int i = lane; i < C::kWords; i += 32) nw |= wN[i];
            has_n = __any_sync(0xFFFFFFFFu, nw != 0u);
        }
        const uint32_t ne = (uint32_t)(second ? p.strand[1].n_encoded : p.strand[0].n_encoded);
        const uint64_t slot = (uint64_t)(second ? p.strand[1].slot : p.strand[0].slot);
        const int64_t base = lc * CH;
        // positions [0, lim) of this chunk are scanned (total_bp - 26 overall)
        const int64_t lim64 = total_bp - kSiteSpan - base;
        const int lim = lim64 > CH ? CH : (int)lim64;

        for (int f = p.fam_begin; f < p.fam_end; ++f) {
            const FamilyDesc F = p.fams[f];
            const uint32_t win_off = F.three_prime ? 0u : (uint32_t)F.plen;
            const SeedFam &SF = sFam[f - p.fam_begin];
            const int n_tests = SF.n_tests;
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
            // only the family's own tests run (a loop, not predicated slots),
            // each test's parameters loaded once for all rows
#pragma unroll 1
            for (int k = 0; k < n_tests; ++k) {
                const uint32_t sh = SF.pam_shift[k];
                const uint4 m = SF.pam_mask[k];
                const bool generic = (SF.pam_generic >> k) & 1u;
#pragma unroll
                for (int u = 0; u < C::kRows; ++u) {
                    const uint32_t h = sfshr(hw[u][0], hw[u][1], sh);
                    const uint32_t l = sfshr(lw[u][0], lw[u][1], sh);
                    pass[u] &= generic ? (~h & ~l & m.x) | (~h & l & m.y) | (h & ~l & m.z) |
                                             (h & l & m.w)
                                       : ~(((h ^ m.x) & m.y) | ((l ^ m.z) & m.w));
                }
            }
            // The list is row-major (row u's positions of lanes 0..31, then row
            // u + 1's), so that a round's lanes read window words of
            // neighbouring lanes' words, in different banks.  Row offsets: one
            // warp scan per two rows, the counts in 16-bit halves.
            int rowoff[C::kRows];
            int total = 0;
#pragma unroll
            for (int h = 0; h < (C::kRows + 1) / 2; ++h) {
                // (the second row's index is clamped so that the one-row form
                // has no out-of-range access even in its dead branch)
                const bool two = 2 * h + 1 < C::kRows;
                const uint32_t pk = (uint32_t)__popc(pass[2 * h]) |
                                    (two ? (uint32_t)__popc(pass[two ? 2 * h + 1 : 0]) << 16 : 0u);
                uint32_t incl = pk;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                    if (lane >= o) incl += v;
                }
                const uint32_t tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
                const uint32_t ex = incl - pk;
                rowoff[2 * h] = total + (int)(ex & 0xFFFFu);
                total += (int)(tot & 0xFFFFu);
                if (two) {
                    rowoff[two ? 2 * h + 1 : 0] = total + (int)(ex >> 16);
                    total += (int)(tot >> 16);
                }
            }
            // the family's bucket tables and entry bases, held in registers
            uint32_t seg_off[S], seg_ent[S];
            {
                const uint32_t list_off = sFam[f - p.fam_begin].list_off;
#pragma unroll
                for (int j = 0; j < S; ++j) {
                    seg_off[j] = sFam[f - p.fam_begin].seg[j].off;
                    seg_ent[j] = list_off + sFam[f - p.fam_begin].seg[j].ent;
                }
            }
            const uint32_t gbeg = (uint32_t)F.gbeg;
#pragma unroll 1
            for (int pass_i = 0; pass_i < C::kPasses; ++pass_i) {
                const int lo = pass_i * C::kListCap;
                if (lo >= total) break;
                const int n_list = min(total - lo, C::kListCap);
                // list positions [lo, lo + n_list) of the chunk's passing positions
                // (one pass, the common case: every lane lists all of its own)
                if (C::kPasses == 1 || total <= C::kListCap) {
#pragma unroll
                    for (int u = 0; u < C::kRows; ++u) {
                        int off = rowoff[u];
                        uint32_t m = pass[u];
                        while (m) {
                            const int j = __ffs(m) - 1;
                            m &= m - 1u;
                            wList[off++] = (uint16_t)(32 * (u * 32 + lane) + j);
                        }
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < C::kRows; ++u) {
                        int off = rowoff[u] - lo;
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
                    uint32_t s = 0, h20 = 0, l20 = 0, n20g = 0;
                    if (has) {
                        s = wList[k];
                        const uint32_t wo = s + win_off;
                        const uint32_t wi = wo >> 5, b = wo & 31u;
                        h20 = sfshr(wH[wi], wH[wi + 1], b) & 0xFFFFFu;
                        l20 = sfshr(wL[wi], wL[wi + 1], b) & 0xFFFFFu;
                        if (has_n) {
                            const uint32_t n26 =
                                sfshr(wN[s >> 5], wN[(s >> 5) + 1], s & 31u) & 0x3FFFFFFu;
                            if (n26) n20g = sfshr(wN[wi], wN[wi + 1], b) & 0xFFFFFu;
                        }
                    }
                    const uint64_t pos = (uint64_t)(base + s);
                    // Branch-free in three phases so that the regions' load
                    // chains overlap: (1) every region's bucket descriptor, (2) an
                    // inline compare of each bucket's first INLINE (1 or 2) entry
                    // slots, (3) the rare candidates within K.  A slot past the
                    // bucket's end is compared too and its result ignored: it is
                    // a later entry or, past the last list, the bucket table that
                    // follows the lists in shared memory, so the load stays in
                    // bounds.  Guides beyond the inline slots are walked by their
                    // lane (WALK) or queued as ranges for the warp.
                    constexpr uint32_t INL = (uint32_t)INLINE;
                    uint32_t nn[S], e0v[S];
                    uint32_t T = 0, maxn = 0;
#pragma unroll
                    for (int j = 0; j < S; ++j) {
                        const int st = G::start(j), kl = G::klen(j);
                        const uint32_t km = (1u << kl) - 1u;
                        const uint32_t code = (((h20 >> st) & km) << kl) | ((l20 >> st) & km);
                        const uint32_t d = has ? sOff[seg_off[j] + code] : 0u;
                        nn[j] = d >> 16;
                        e0v[j] = seg_ent[j] + (d & 0xFFFFu);
                        T += nn[j];
                        maxn = max(maxn, nn[j]);
                    }
                    uint32_t hit = 0;  // bit j * INL + a: slot a of bucket j is within K
#pragma unroll
                    for (int j = 0; j < S; ++j) {
#pragma unroll
                        for (uint32_t a = 0; a < INL; ++a) {
                            const uint2 e = sEnt[e0v[j] + a];
                            const bool in = nn[j] > a && __popc((h20 ^ e.x) | (l20 ^ e.y)) <= K;
                            hit |= (in ? 1u : 0u) << (j * INL + a);
                        }
                    }
                    if (hit) {
#pragma unroll
                        for (int j = 0; j < S; ++j) {
#pragma unroll
                            for (uint32_t a = 0; a < INL; ++a) {
                                if ((hit >> (j * INL + a)) & 1u) {
                                    const uint32_t ei = e0v[j] + a;
                                    const uint2 e = sEnt[ei];
                                    const uint32_t m = (h20 ^ e.x) | (l20 ^ e.y);
                                    if (finish_candidate<K, TOL>(p, m, __popc(m), e, sIdx[ei], j, n20g,
                                                             ne, slot, pos, gbeg))
                                    mark_dropped(pos, slot, p.drop_bits, p.drop_base1);
                                }
                            }
                        }
                    }
                    cand += T;
                    if (!__any_sync(0xFFFFFFFFu, maxn > INL)) continue;
                    if constexpr (WALK == 1) {
                        // buckets that rarely hold more than the inline guides:
                        // each lane walks its own few remaining entries
#pragma unroll
                        for (int j = 0; j < S; ++j) {
                            for (uint32_t i = INL; i < nn[j]; ++i) {
                                const uint32_t ei = e0v[j] + i;
                                const uint2 e = sEnt[ei];
                                const uint32_t m = (h20 ^ e.x) | (l20 ^ e.y);
                                const int cm = __popc(m);
                                if (cm <= K)
                                    if (finish_candidate<K, TOL>(p, m, cm, e, sIdx[ei], j, n20g,
                                                             ne, slot, pos, gbeg))
                                    mark_dropped(pos, slot, p.drop_bits, p.drop_base1);
                            }
                        }
                        continue;
                    }
                    // buckets with more guides: ranges spread over the warp's lanes
                    uint32_t R = 0;
#pragma unroll
                    for (int j = 0; j < S; ++j) R += nn[j] > INL ? 1u : 0u;
                    uint32_t rin = R;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, rin, o);
                        if (lane >= o) rin += v;
                    }
                    const uint32_t RT = __shfl_sync(0xFFFFFFFFu, rin, 31);
                    wRec[lane] = make_uint4(h20, l20, n20g, s);
                    uint32_t qp = rin - R;
#pragma unroll
                    for (int j = 0; j < S; ++j) {
                        if (nn[j] > INL) {
                            wQ[qp] = (e0v[j] + INL) | ((uint32_t)j << 22) | ((uint32_t)lane << 27);
                            wCnt[qp] = (uint16_t)(nn[j] - INL);
                            ++qp;
                        }
                    }
                    __syncwarp();
                    for (uint32_t q = lane; q < RT; q += 32) {
                        const uint32_t v = wQ[q];
                        const uint32_t n = wCnt[q];
                        const uint4 r = wRec[v >> 27];
                        const uint32_t e0 = v & 0x3FFFFFu;
                        const int j = (int)((v >> 22) & 31u);
                        for (uint32_t i = 0; i < n; ++i) {
                            const uint2 e = sEnt[e0 + i];
                            const uint32_t m = (r.x ^ e.x) | (r.y ^ e.y);
                            const int cm = __popc(m);
                            if (cm <= K)
                                if (finish_candidate<K, TOL>(p, m, cm, e, sIdx[e0 + i], j, r.z,
                                                         ne, slot, (uint64_t)(base + r.w),
                                                         gbeg))
                                    mark_dropped((uint64_t)(base + r.w), slot, p.drop_bits, p.drop_base1);
                        }
                    }
                    __syncwarp();
                }
                __syncwarp();  // the next pass overwrites the list
            }
        }
    }
    cp_async_wait<0>();
    for (int o = 16; o > 0; o >>= 1) cand += __shfl_down_sync(0xFFFFFFFFu, cand, o);
    if (lane == 0 && cand) atomicAdd(&sCand, (unsigned long long)cand);
    __syncthreads();
    if (t == 0 && sCand) atomicAdd(p.counter + 1, sCand);
}

template <int K, int TOL, int INLINE, int WALK, int CH, int MINB>
static int launch_k(const ScanParams &p, const SeedArgs &sa, int sm_count, int ctas_per_sm,
                    cudaStream_t s) {
    const size_t smem = seed_smem_bytes(sa, CH, SeedCta<MINB>::kWarps, WALK == 1);
    static size_t configured = 0;
    if (smem > configured) {
        BGO_CUDA(cudaFuncSetAttribute(scan_seed_kernel<K, TOL, INLINE, WALK, CH, MINB>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = smem;
    }
    int per_sm = 0;
    BGO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, scan_seed_kernel<K, TOL, INLINE, WALK, CH, MINB>, SeedCta<MINB>::kThreads,
        smem));
    if (per_sm < 1) per_sm = 1;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
    constexpr int WARPS = SeedCta<MINB>::kWarps;
    const int64_t items = p.chunk_list ? p.n_list : p.tiles_total;
    const int64_t blocks_needed = (items + WARPS - 1) / WARPS;
    const int64_t grid = std::min<int64_t>(blocks_needed, (int64_t)sm_count * per_sm);
    scan_seed_kernel<K, TOL, INLINE, WALK, CH, MINB>
        <<<(unsigned)grid, SeedCta<MINB>::kThreads, smem, s>>>(p, sa);
    BGO_CUDA(cudaGetLastError());
    return BGO_OK;
}

template <int TOL, int INLINE, int WALK, int CH, int MINB>
static int launch_cm(const ScanParams &p, const SeedArgs &sa, int sm_count, int ctas_per_sm,
                     cudaStream_t s) {
    switch (p.max_mm) {
        case 0: return launch_k<0, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        case 1: return launch_k<1, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        case 2: return launch_k<2, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        case 3: return launch_k<3, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        case 4: return launch_k<4, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        case 5: return launch_k<5, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        case 6: return launch_k<6, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        case 7: return launch_k<7, TOL, INLINE, WALK, CH, MINB>(p, sa, sm_count, ctas_per_sm, s);
        default:
            set_error("segment index: max_mismatches outside 0..7");
            return BGO_ERR_ARG;
    }
}

// All chunk lengths and occupancy targets for one (tolerance, inline guides,
// leftover walk) form.
template <int TOL, int INLINE, int WALK>
static int launch_form(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                       int min_blocks, int ctas_per_sm, cudaStream_t s) {
    const bool c1k = chunk_sites == 1024;
    if (min_blocks == 4)
        return c1k ? launch_cm<TOL, INLINE, WALK, 1024, 4>(p, sa, sm_count, ctas_per_sm, s)
                   : launch_cm<TOL, INLINE, WALK, 2048, 4>(p, sa, sm_count, ctas_per_sm, s);
    if (min_blocks == 1)
        return c1k ? launch_cm<TOL, INLINE, WALK, 1024, 1>(p, sa, sm_count, ctas_per_sm, s)
                   : launch_cm<TOL, INLINE, WALK, 2048, 1>(p, sa, sm_count, ctas_per_sm, s);
    if (min_blocks == 2)
        return c1k ? launch_cm<TOL, INLINE, WALK, 1024, 2>(p, sa, sm_count, ctas_per_sm, s)
                   : launch_cm<TOL, INLINE, WALK, 2048, 2>(p, sa, sm_count, ctas_per_sm, s);
    return c1k ? launch_cm<TOL, INLINE, WALK, 1024, 3>(p, sa, sm_count, ctas_per_sm, s)
               : launch_cm<TOL, INLINE, WALK, 2048, 3>(p, sa, sm_count, ctas_per_sm, s);
}

}  // namespace bgo
