// Segment-indexed scan (scan mode 2): the same hits as scan_kernel with far
// fewer guide comparisons.
//
// Exactness.  A hit has at most K = max_mismatches raw mismatches over the 20
// guide positions (the N correction only adds to the raw count,
// beguidedoff/cuda_search.py:272-308).  Split the 20 positions into K + 1
// disjoint segments: by the pigeonhole principle at least one segment of every
// hit matches the genome exactly.  So for each PAM-passing position the kernel
// looks up, per segment, the guides whose bases in that segment equal the
// genome's (a per-family index built on the host: 4^k buckets per segment over
// the segment's first k <= 6 bases) and runs the reference's full compare
// (XOR / pair-OR / popcount, then the N correction) on those candidates only.
// A candidate reached through segment j is reported only if no earlier segment
// also matches exactly, so each (position, guide) hit is emitted once.
//
// Layout.  Warps work independently (no CTA barrier after the start): each
// warp takes chunks of kSeedChunkSites positions of one strand and copies the
// next chunk's H/L/N words with cp.async while it works on the current one
// (double buffering).  Per PAM family it runs the family's compiled PAM test
// on 32 positions per lane and word (funnel shifts + LOP3), compacts the
// passing positions with one warp scan, then processes them 32 per round (one
// per lane): the lane computes the K + 1 segment codes of its window, loads
// each bucket descriptor and compares the bucket's first guide inline (all
// lanes in step, predicated); buckets holding more guides leave the rest as a
// range in the warp's queue, which the warp then works through.  The segment
// layout is a compile-time function of K.  Hits are appended with one
// atomicAdd per warp.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "bgo_device.cuh"
#include "bgo_internal.cuh"

namespace bgo {

constexpr int kSeedWarps = kSeedThreads / 32;
constexpr int kChunkRows = kSeedChunkSites / 1024;     // 32-position words per lane
constexpr int kChunkWords = kSeedChunkSites / 32 + 4;  // 64 + halo, a multiple of 4 words
constexpr int kChunkVecs = kChunkWords / 4;            // 16-byte copies per plane
constexpr int kQueueCap = 32 * (kSeedMaxK + 1);        // bucket ranges per round
// per warp: two chunk buffers (H, L, N planes), the compacted list, the round's
// position records and the bucket-range queue (word + count)
constexpr size_t kBufBytes = 3 * kChunkWords * sizeof(uint32_t);
constexpr size_t kListOff = 2 * kBufBytes;
constexpr size_t kRecOff = (kListOff + kSeedChunkSites * sizeof(uint16_t) + 15) / 16 * 16;
constexpr size_t kQueueOff = kRecOff + 32 * sizeof(uint4);
constexpr size_t kCountOff = kQueueOff + kQueueCap * sizeof(uint32_t);
constexpr size_t kWarpSliceBytes = (kCountOff + kQueueCap * sizeof(uint16_t) + 15) / 16 * 16;
static_assert(kChunkWords % 4 == 0, "chunk copies are whole 16-byte vectors");
static_assert(kBufBytes % 16 == 0, "chunk buffers stay 16-byte aligned");

// The K + 1 segments: start and key length (the segment's first <= 6 bases).
template <int K>
struct Seg {
    static constexpr int S = K + 1;
    static constexpr int q = kGuideLen / S, r = kGuideLen % S;
    __host__ __device__ static constexpr int start(int j) { return j * q + (j < r ? j : r); }
    __host__ __device__ static constexpr int len(int j) { return q + (j < r ? 1 : 0); }
    __host__ __device__ static constexpr int klen(int j) {
        return len(j) < kMaxKeyLen ? len(j) : kMaxKeyLen;
    }
};

// The full check of a candidate whose raw count cm <= K, found through
// segment j: emits the hit if j is its first exact segment and it stays
// within K after the N correction.
template <int K>
__device__ __noinline__ void finish_candidate(const ScanParams &p, uint32_t m, int cm, uint2 e,
                                              uint32_t idx, int j, uint32_t n20g, uint32_t ne,
                                              uint64_t slot, uint64_t pos, uint32_t gbeg) {
    bool first = true;
#pragma unroll
    for (int jj = 0; jj < K; ++jj)
        if (jj < j)
            first = first &&
                    (((m >> Seg<K>::start(jj)) & ((1u << Seg<K>::klen(jj)) - 1u)) != 0u);
    if (!first) return;
    int mmf = cm;
    if (n20g) {
        const uint32_t eh = (ne & 2u) ? e.x : ~e.x;
        const uint32_t el = (ne & 1u) ? e.y : ~e.y;
        mmf = cm + __popc(n20g & eh & el);
    }
    if (mmf > K) return;
    const uint32_t row = __ldg(&p.guides[gbeg + idx].row);
    semit(((uint64_t)row << 39) | (slot << 38) | (pos << 6) | (uint64_t)mmf, p.keys, p.cap,
          p.counter);
}

template <int K>
__global__ void __launch_bounds__(kSeedThreads, 3) scan_seed_kernel(ScanParams p, SeedArgs sa) {
    constexpr int S = K + 1;
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
    unsigned char *slice = slices + warp * kWarpSliceBytes;
    uint16_t *wList = reinterpret_cast<uint16_t *>(slice + kListOff);
    uint4 *wRec = reinterpret_cast<uint4 *>(slice + kRecOff);
    uint32_t *wQ = reinterpret_cast<uint32_t *>(slice + kQueueOff);
    uint16_t *wCnt = reinterpret_cast<uint16_t *>(slice + kCountOff);

    for (int i = t; i < sa.n_fams; i += kSeedThreads) sFam[i] = sa.fams[i];
    for (int i = t; i < sa.n_lists; i += kSeedThreads) {
        sEnt[i] = sa.entries[i];
        sIdx[i] = sa.entry_idx[i];
    }
    for (int i = t; i < sa.n_offsets; i += kSeedThreads) sOff[i] = sa.offsets[i];
    if (t == 0) sCand = 0;
    __syncthreads();

    const int64_t chunks0 = p.strand[0].n_tiles;
    const int64_t n_chunks = p.tiles_total;
    const int64_t stride = (int64_t)gridDim.x * kSeedWarps;
    // Chunk c's words [c*64, c*64 + kChunkWords) of the three planes, copied
    // into buffer b as 16-byte vectors (the planes are padded so that the copy
    // never leaves them, and zero beyond total_bp).
    auto issue = [&](int64_t c, int b) {
        const bool second = c >= chunks0;
        const int64_t w0 = (second ? c - chunks0 : c) * (kSeedChunkSites / 32);
        const StrandDesc &sd = second ? p.strand[1] : p.strand[0];
        uint32_t *dst = reinterpret_cast<uint32_t *>(slice + b * kBufBytes);
        for (int i = lane; i < 3 * kChunkVecs; i += 32) {
            const int plane = i / kChunkVecs, v = i - plane * kChunkVecs;
            const uint32_t *src = plane == 0 ? sd.H : plane == 1 ? sd.L : sd.N;
            cp_async16(dst + plane * kChunkWords + 4 * v, src + w0 + 4 * v);
        }
    };
    uint32_t cand = 0;
    const int64_t c_first = (int64_t)blockIdx.x * kSeedWarps + warp;
    if (c_first < n_chunks) issue(c_first, 0);
    cp_async_commit();
    int buf = 0;
    for (int64_t c = c_first; c < n_chunks; c += stride, buf ^= 1) {
        if (c + stride < n_chunks) issue(c + stride, buf ^ 1);
        cp_async_commit();
        cp_async_wait<1>();  // this chunk's copies are done; the next one is in flight
        __syncwarp();
        const uint32_t *wH = reinterpret_cast<const uint32_t *>(slice + buf * kBufBytes);
        const uint32_t *wL = wH + kChunkWords;
        const uint32_t *wN = wL + kChunkWords;
        const bool second = c >= chunks0;
        const int64_t lc = second ? c - chunks0 : c;
        const int64_t total_bp = second ? p.strand[1].total_bp : p.strand[0].total_bp;
        const int has_n = second ? p.strand[1].has_n : p.strand[0].has_n;
        const uint32_t ne = (uint32_t)(second ? p.strand[1].n_encoded : p.strand[0].n_encoded);
        const uint64_t slot = (uint64_t)(second ? p.strand[1].slot : p.strand[0].slot);
        const int64_t base = lc * kSeedChunkSites;
        // positions [0, lim) of this chunk are scanned (total_bp - 26 overall)
        const int64_t lim64 = total_bp - kSiteSpan - base;
        const int lim = lim64 > kSeedChunkSites ? kSeedChunkSites : (int)lim64;

        for (int f = p.fam_begin; f < p.fam_end; ++f) {
            const FamilyDesc F = p.fams[f];
            const uint32_t win_off = F.three_prime ? 0u : (uint32_t)F.plen;
            const int n_tests = sFam[f - p.fam_begin].n_tests;
            uint32_t tsh[kMaxPam], tcd[kMaxPam];
#pragma unroll
            for (int k = 0; k < kMaxPam; ++k) {
                tsh[k] = sFam[f - p.fam_begin].pam_shift[k];
                tcd[k] = sFam[f - p.fam_begin].pam_code[k];
            }
            uint32_t pass[kChunkRows];
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < kChunkRows; ++u) {
                const int wi = u * 32 + lane;
                const int rem = lim - 32 * wi;
                uint32_t ps = rem >= 32 ? 0xFFFFFFFFu : (rem <= 0 ? 0u : (1u << rem) - 1u);
                const uint32_t h0 = wH[wi], h1 = wH[wi + 1], l0 = wL[wi], l1 = wL[wi + 1];
#pragma unroll
                for (int k = 0; k < kMaxPam; ++k) {
                    if (k < n_tests)
                        ps &= pam_test(sfshr(h0, h1, tsh[k]), sfshr(l0, l1, tsh[k]), tcd[k]);
                }
                pass[u] = ps;
                cnt += __popc(ps);
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            int off = incl - cnt;
#pragma unroll
            for (int u = 0; u < kChunkRows; ++u) {
                uint32_t m = pass[u];
                while (m) {
                    const int j = __ffs(m) - 1;
                    m &= m - 1u;
                    wList[off++] = (uint16_t)(32 * (u * 32 + lane) + j);
                }
            }
            __syncwarp();
            // the family's bucket tables and entry bases, held in registers
            uint32_t seg_off[S], seg_ent[S];
            {
                const uint32_t list_off = sFam[f - p.fam_begin].list_off;
                const uint32_t gf = (uint32_t)(F.gend - F.gbeg);
#pragma unroll
                for (int j = 0; j < S; ++j) {
                    seg_off[j] = sFam[f - p.fam_begin].seg[j].off;
                    seg_ent[j] = list_off + (uint32_t)j * gf;
                }
            }
            const uint32_t gbeg = (uint32_t)F.gbeg;
            for (int k0 = 0; k0 < total; k0 += 32) {
                const int k = k0 + lane;
                const bool has = k < total;
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
                // per segment: bucket descriptor and an inline compare of the
                // bucket's first guide; further guides stay as a range
                uint32_t ra[S], rn[S];
                uint32_t T = 0, R = 0;
#pragma unroll
                for (int j = 0; j < S; ++j) {
                    const int st = Seg<K>::start(j), kl = Seg<K>::klen(j);
                    const uint32_t km = (1u << kl) - 1u;
                    const uint32_t code = (((h20 >> st) & km) << kl) | ((l20 >> st) & km);
                    const uint32_t d = has ? sOff[seg_off[j] + code] : 0u;
                    const uint32_t n = d >> 16;
                    const uint32_t e0 = seg_ent[j] + (d & 0xFFFFu);
                    T += n;
                    if (n) {
                        const uint2 e = sEnt[e0];
                        const uint32_t m = (h20 ^ e.x) | (l20 ^ e.y);
                        const int cm = __popc(m);
                        if (cm <= K)
                            finish_candidate<K>(p, m, cm, e, sIdx[e0], j, n20g, ne, slot, pos,
                                                gbeg);
                    }
                    ra[j] = e0 + 1;
                    rn[j] = n > 1u ? n - 1u : 0u;
                    R += rn[j] != 0u;
                }
                cand += T;
                // buckets with more than one guide: ranges through the queue
                if (!__any_sync(0xFFFFFFFFu, R != 0u)) continue;
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
                    if (rn[j]) {
                        wQ[qp] = ra[j] | ((uint32_t)j << 22) | ((uint32_t)lane << 27);
                        wCnt[qp] = (uint16_t)rn[j];
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
                            finish_candidate<K>(p, m, cm, e, sIdx[e0 + i], j, r.z, ne, slot,
                                                (uint64_t)(base + r.w), gbeg);
                    }
                }
                __syncwarp();
            }
            __syncwarp();
        }
    }
    cp_async_wait<0>();
    for (int o = 16; o > 0; o >>= 1) cand += __shfl_down_sync(0xFFFFFFFFu, cand, o);
    if (lane == 0 && cand) atomicAdd(&sCand, (unsigned long long)cand);
    __syncthreads();
    if (t == 0 && sCand) atomicAdd(p.counter + 1, sCand);
}

size_t seed_smem_bytes(const SeedArgs &sa) {
    size_t b = sizeof(SeedFam) * sa.n_fams + sizeof(uint2) * sa.n_lists +
               sizeof(uint32_t) * sa.n_offsets + sizeof(uint16_t) * sa.n_lists;
    b = (b + 15) / 16 * 16;
    return b + kSeedWarps * kWarpSliceBytes;
}

template <int K>
static int launch_k(const ScanParams &p, const SeedArgs &sa, int sm_count, cudaStream_t s) {
    const size_t smem = seed_smem_bytes(sa);
    static size_t configured = 0;
    if (smem > configured) {
        BGO_CUDA(cudaFuncSetAttribute(scan_seed_kernel<K>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = smem;
    }
    int per_sm = 0;
    BGO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, scan_seed_kernel<K>,
                                                           kSeedThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t blocks_needed = (p.tiles_total + kSeedWarps - 1) / kSeedWarps;
    const int64_t grid = std::min<int64_t>(blocks_needed, (int64_t)sm_count * per_sm);
    scan_seed_kernel<K><<<(unsigned)grid, kSeedThreads, smem, s>>>(p, sa);
    BGO_CUDA(cudaGetLastError());
    return BGO_OK;
}

int launch_seed_kernel(const ScanParams &p, const SeedArgs &sa, int sm_count, cudaStream_t s) {
    switch (p.max_mm) {
        case 0: return launch_k<0>(p, sa, sm_count, s);
        case 1: return launch_k<1>(p, sa, sm_count, s);
        case 2: return launch_k<2>(p, sa, sm_count, s);
        case 3: return launch_k<3>(p, sa, sm_count, s);
        case 4: return launch_k<4>(p, sa, sm_count, s);
        case 5: return launch_k<5>(p, sa, sm_count, s);
        case 6: return launch_k<6>(p, sa, sm_count, s);
        case 7: return launch_k<7>(p, sa, sm_count, s);
        default:
            set_error("segment index: max_mismatches outside 0..7");
            return BGO_ERR_ARG;
    }
}

// PAM test program of a family: one test per constrained position (an N is
// skipped).  Sets whose members share a fixed bit pattern of the 2-bit code
// (single bases, R, Y, M, K) compare bits; S, W and the three-base codes use
// the generic allowed-set select.
void pam_program(const FamilyDesc &F, SeedFam &sf) {
    const uint32_t pam_off = F.three_prime ? 20u : 0u;
    sf.n_tests = 0;
    for (int k = 0; k < F.plen; ++k) {
        const uint32_t a = F.allowed[k] & 15u;
        if (a == 15u) continue;
        int nb = 0, b0 = -1, b1 = -1;
        for (int b = 0; b < 4; ++b)
            if (a & (1u << b)) {
                if (nb == 0) b0 = b;
                else b1 = b;
                ++nb;
            }
        uint16_t code;
        if (nb == 1) {
            code = (uint16_t)(((b0 >> 1) & 1) | 2 | ((b0 & 1) << 2) | 8);
        } else if (nb == 2 && ((b0 & 1) == (b1 & 1)) && ((b0 >> 1) != (b1 >> 1))) {
            code = (uint16_t)(((b0 & 1) << 2) | 8);  // low bit fixed (R, Y)
        } else if (nb == 2 && ((b0 >> 1) == (b1 >> 1)) && ((b0 & 1) != (b1 & 1))) {
            code = (uint16_t)(((b0 >> 1) & 1) | 2);  // high bit fixed (M, K)
        } else {
            code = (uint16_t)(0x100u | a);
        }
        sf.pam_shift[sf.n_tests] = (uint8_t)(pam_off + (uint32_t)k);
        sf.pam_code[sf.n_tests] = code;
        sf.n_tests++;
    }
}

// The host index for K mismatches; false when the filter does not apply (K
// outside 0..7, where K + 1 segments of 2-3 bases would not halve the
// comparisons) or a family is too large for 16-bit bucket fields.  Bucket
// descriptor = entry start within the segment's list | count << 16.
bool build_seed_index(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                      std::vector<SeedFam> &out_fams, std::vector<uint32_t> &offsets,
                      std::vector<uint2> &entries, std::vector<uint16_t> &entry_idx) {
    if (K < 0 || K > kSeedMaxK) return false;
    const int S = K + 1;
    const int q = kGuideLen / S, r = kGuideLen % S;
    out_fams.assign((size_t)n_fams, SeedFam{});
    offsets.clear();
    entries.clear();
    entry_idx.clear();
    for (int f = 0; f < n_fams; ++f) {
        const int G = fams[f].gend - fams[f].gbeg;
        if (G > 65535) return false;
        SeedFam &sf = out_fams[(size_t)f];
        sf.nseg = S;
        pam_program(fams[f], sf);
        sf.list_off = (uint32_t)entries.size();
        entries.resize(entries.size() + (size_t)S * (size_t)G);
        entry_idx.resize(entries.size());
        if (entries.size() >= (1u << 22)) return false;
        for (int j = 0; j < S; ++j) {
            SeedSeg sg{};
            sg.start = (uint8_t)(j * q + std::min(j, r));
            sg.len = (uint8_t)(q + (j < r ? 1 : 0));
            sg.klen = (uint8_t)std::min<int>(sg.len, kMaxKeyLen);
            sg.off = (uint32_t)offsets.size();
            const uint32_t nb = 1u << (2 * sg.klen);
            const uint32_t km = (1u << sg.klen) - 1u;
            std::vector<uint32_t> cnt(nb + 1, 0);
            std::vector<uint32_t> code((size_t)G);
            for (int i = 0; i < G; ++i) {
                const GuideRec &rr = recs[fams[f].gbeg + i];
                code[(size_t)i] = (((rr.h >> sg.start) & km) << sg.klen) | ((rr.l >> sg.start) & km);
                cnt[code[(size_t)i] + 1]++;
            }
            for (uint32_t c = 0; c < nb; ++c) cnt[c + 1] += cnt[c];
            for (uint32_t c = 0; c < nb; ++c) offsets.push_back(cnt[c] | ((cnt[c + 1] - cnt[c]) << 16));
            std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
            const size_t e_base = sf.list_off + (size_t)j * (size_t)G;
            for (int i = 0; i < G; ++i) {
                const GuideRec &rr = recs[fams[f].gbeg + i];
                const size_t at = e_base + fill[code[(size_t)i]]++;
                entries[at] = make_uint2(rr.h & 0xFFFFFu, rr.l & 0xFFFFFu);
                entry_idx[at] = (uint16_t)i;
            }
            sf.seg[j] = sg;
        }
    }
    return true;
}

}  // namespace bgo
