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
// Layout.  One persistent CTA of 512 threads per half SM; each tile is 32,768
// positions of one strand (two plane words per thread).  The PAM families'
// segment indexes and guide planes are copied to shared memory once per CTA.
// Per tile and family: bit-parallel PAM test of 64 positions per thread, CTA
// compaction of the passing positions, then one thread per compacted position
// walks its K + 1 buckets.  Hits are appended with one atomicAdd per warp.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "bgo_internal.cuh"

namespace bgo {

__device__ __forceinline__ uint32_t sfshr(uint32_t lo, uint32_t hi, uint32_t s) {
    return __funnelshift_r(lo, hi, s);
}

__device__ __forceinline__ uint32_t sallowed(uint32_t h, uint32_t l, uint32_t a) {
    uint32_t r = 0;
    if (a & 1u) r |= ~h & ~l;
    if (a & 2u) r |= ~h & l;
    if (a & 4u) r |= h & ~l;
    if (a & 8u) r |= h & l;
    return r;
}

__device__ __forceinline__ void semit(uint64_t key, uint64_t *keys, int64_t cap,
                                      unsigned long long *counter) {
    unsigned act = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(act) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(act));
    base = __shfl_sync(act, base, leader);
    unsigned long long slot = base + (unsigned long long)__popc(act & ((1u << lane) - 1u));
    if (slot < (unsigned long long)cap) keys[slot] = key;
}

// 20-bit H, L and gated N windows of compacted position s (tile-relative).
struct SiteWin {
    uint32_t h, l, n;
};

__global__ void __launch_bounds__(kSeedThreads) scan_seed_kernel(ScanParams p, SeedArgs sa) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *sH = reinterpret_cast<uint32_t *>(smem);
    uint32_t *sL = sH + kSeedTileWords;
    uint32_t *sN = sL + kSeedTileWords;
    uint16_t *sList = reinterpret_cast<uint16_t *>(sN + kSeedTileWords);
    SeedFam *sFam = reinterpret_cast<SeedFam *>(sList + kSeedTileSites);
    uint4 *sG = reinterpret_cast<uint4 *>(sFam + sa.n_fams);
    uint32_t *sOff = reinterpret_cast<uint32_t *>(sG + sa.n_guides);
    uint16_t *sLst = reinterpret_cast<uint16_t *>(sOff + sa.n_offsets);
    __shared__ int sWarp[kSeedThreads / 32];
    __shared__ int sTotal;
    __shared__ unsigned long long sCand;

    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
    const int K = p.max_mm;

    // stage the segment indexes and guide planes of every family once
    for (int i = t; i < sa.n_fams; i += kSeedThreads) sFam[i] = sa.fams[i];
    for (int i = t; i < sa.n_guides; i += kSeedThreads) {
        const GuideRec r = p.guides[i];
        sG[i] = make_uint4(r.h, r.l, r.row, 0u);
    }
    for (int i = t; i < sa.n_offsets; i += kSeedThreads) sOff[i] = sa.offsets[i];
    for (int i = t; i < sa.n_lists; i += kSeedThreads) sLst[i] = sa.lists[i];

    for (int64_t tile = blockIdx.x; tile < p.tiles_total; tile += gridDim.x) {
        const bool second = p.n_strands > 1 && tile >= p.strand[0].n_tiles;
        const int64_t lt = second ? tile - p.strand[0].n_tiles : tile;
        const uint32_t *H = second ? p.strand[1].H : p.strand[0].H;
        const uint32_t *L = second ? p.strand[1].L : p.strand[0].L;
        const uint32_t *N = second ? p.strand[1].N : p.strand[0].N;
        const int64_t total_bp = second ? p.strand[1].total_bp : p.strand[0].total_bp;
        const int has_n = second ? p.strand[1].has_n : p.strand[0].has_n;
        const uint32_t ne = (uint32_t)(second ? p.strand[1].n_encoded : p.strand[0].n_encoded);
        const uint64_t slot = (uint64_t)(second ? p.strand[1].slot : p.strand[0].slot);
        const int64_t base = lt * kSeedTileSites;
        const int64_t w0 = lt * (kSeedTileSites / 32);
        const int64_t valid_end = total_bp - kSiteSpan;
        const int64_t words_ok = (total_bp + 31) / 32 + 4;  // inside every plane allocation

        __syncthreads();
        for (int i = t; i < kSeedTileWords; i += kSeedThreads) {
            const int64_t w = w0 + i;
            const bool in = w < words_ok;
            sH[i] = in ? H[w] : 0u;
            sL[i] = in ? L[w] : 0u;
            sN[i] = in ? N[w] : 0u;
        }
        uint32_t valid[kSeedWpt];
#pragma unroll
        for (int u = 0; u < kSeedWpt; ++u) {
            const int64_t s0 = base + 32 * (kSeedWpt * t + u);
            valid[u] = 0xFFFFFFFFu;
            if (s0 >= valid_end) valid[u] = 0;
            else if (valid_end - s0 < 32) valid[u] = (1u << (uint32_t)(valid_end - s0)) - 1u;
        }
        __syncthreads();

        for (int f = p.fam_begin; f < p.fam_end; ++f) {
            const FamilyDesc F = p.fams[f];
            const uint32_t pam_off = F.three_prime ? 20u : 0u;
            const uint32_t win_off = F.three_prime ? 0u : (uint32_t)F.plen;
            if (t == 0) sCand = 0;

            uint32_t pass[kSeedWpt];
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < kSeedWpt; ++u) {
                const int wi = kSeedWpt * t + u;
                uint32_t ps = valid[u];
                for (int k = 0; k < F.plen; ++k) {
                    const uint32_t a = F.allowed[k] & 15u;
                    if (a == 15u) continue;
                    const uint32_t s = pam_off + (uint32_t)k;
                    ps &= sallowed(sfshr(sH[wi], sH[wi + 1], s), sfshr(sL[wi], sL[wi + 1], s), a);
                }
                pass[u] = ps;
                cnt += __popc(ps);
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) sWarp[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                int v = lane < kSeedThreads / 32 ? sWarp[lane] : 0;
                int inc = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                    if (lane >= o) inc += u;
                }
                if (lane < kSeedThreads / 32) sWarp[lane] = inc - v;
                if (lane == kSeedThreads / 32 - 1) sTotal = inc;
            }
            __syncthreads();
            {
                int off = sWarp[warp] + incl - cnt;
#pragma unroll
                for (int u = 0; u < kSeedWpt; ++u) {
                    uint32_t m = pass[u];
                    while (m) {
                        const int j = __ffs(m) - 1;
                        m &= m - 1u;
                        sList[off++] = (uint16_t)(32 * (kSeedWpt * t + u) + j);
                    }
                }
            }
            __syncthreads();
            const int n_sites = sTotal;
            const SeedFam &SF = sFam[f];
            const int nseg = SF.nseg;
            const uint32_t gfam = (uint32_t)(F.gend - F.gbeg);
            uint32_t cand = 0;
            for (int idx = t; idx < n_sites; idx += kSeedThreads) {
                const uint32_t s = sList[idx];
                const uint32_t wo = s + win_off;
                const uint32_t wi = wo >> 5, b = wo & 31u;
                const uint32_t h20 = sfshr(sH[wi], sH[wi + 1], b) & 0xFFFFFu;
                const uint32_t l20 = sfshr(sL[wi], sL[wi + 1], b) & 0xFFFFFu;
                for (int j = 0; j < nseg; ++j) {
                    const SeedSeg sg = SF.seg[j];
                    const uint32_t km = (1u << sg.klen) - 1u;
                    const uint32_t code =
                        (((h20 >> sg.start) & km) << sg.klen) | ((l20 >> sg.start) & km);
                    const uint32_t qb = sOff[sg.off + code];
                    const uint32_t qe = sOff[sg.off + code + 1];
                    const uint16_t *Lj = sLst + SF.list_off + (uint32_t)j * gfam;
                    cand += qe - qb;
                    for (uint32_t q = qb; q < qe; ++q) {
                        const uint4 G = sG[F.gbeg + Lj[q]];
                        const uint32_t m = (h20 ^ G.x) | (l20 ^ G.y);
                        const int cm = __popc(m);
                        if (cm > K) continue;
                        bool first = true;
                        for (int jj = 0; jj < j; ++jj) {
                            const SeedSeg s2 = SF.seg[jj];
                            if (((m >> s2.start) & ((1u << s2.klen) - 1u)) == 0u) {
                                first = false;
                                break;
                            }
                        }
                        if (!first) continue;
                        int mmf = cm;
                        if (has_n) {
                            const uint32_t n26 =
                                sfshr(sN[s >> 5], sN[(s >> 5) + 1], s & 31u) & 0x3FFFFFFu;
                            if (n26) {
                                const uint32_t n20 = sfshr(sN[wi], sN[wi + 1], b) & 0xFFFFFu;
                                const uint32_t eh = (ne & 2u) ? G.x : ~G.x;
                                const uint32_t el = (ne & 1u) ? G.y : ~G.y;
                                mmf = cm + __popc(n20 & eh & el);
                            }
                        }
                        if (mmf <= K) {
                            const uint64_t pos = (uint64_t)(base + s);
                            const uint64_t key = ((uint64_t)G.z << 39) | (slot << 38) |
                                                 (pos << 6) | (uint64_t)mmf;
                            semit(key, p.keys, p.cap, p.counter);
                        }
                    }
                }
            }
            for (int o = 16; o > 0; o >>= 1) cand += __shfl_down_sync(0xFFFFFFFFu, cand, o);
            if (lane == 0 && cand) atomicAdd(&sCand, (unsigned long long)cand);
            __syncthreads();
            if (t == 0 && sCand) atomicAdd(p.counter + 1, sCand);
        }
    }
}

size_t seed_static_smem_bytes() {
    return sizeof(uint32_t) * 3 * kSeedTileWords + sizeof(uint16_t) * kSeedTileSites;
}

size_t seed_smem_bytes(const SeedArgs &sa) {
    size_t b = seed_static_smem_bytes();
    b += sizeof(SeedFam) * sa.n_fams;
    b = (b + 15) / 16 * 16;
    b += sizeof(uint4) * sa.n_guides + sizeof(uint32_t) * sa.n_offsets +
         sizeof(uint16_t) * sa.n_lists;
    return (b + 15) / 16 * 16;
}

int launch_seed_kernel(const ScanParams &p, const SeedArgs &sa, int sm_count, cudaStream_t s) {
    const size_t smem = seed_smem_bytes(sa);
    static size_t configured = 0;
    if (smem > configured) {
        BGO_CUDA(cudaFuncSetAttribute(scan_seed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        configured = smem;
    }
    int per_sm = 0;
    BGO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, scan_seed_kernel, kSeedThreads,
                                                           smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t grid = std::min<int64_t>(p.tiles_total, (int64_t)sm_count * per_sm);
    scan_seed_kernel<<<(unsigned)grid, kSeedThreads, smem, s>>>(p, sa);
    BGO_CUDA(cudaGetLastError());
    return BGO_OK;
}

// K + 1 segments as equal as possible, longer ones first; each bucket key is
// the segment's first min(len, 6) bases.  False when the filter cannot apply.
static bool seed_layout(int K, int *nseg, SeedSeg *segs) {
    if (K < 0 || K + 1 > kGuideLen) return false;
    const int S = K + 1;
    const int q = kGuideLen / S, r = kGuideLen % S;
    int start = 0;
    for (int j = 0; j < S; ++j) {
        const int len = q + (j < r ? 1 : 0);
        segs[j].start = (uint8_t)start;
        segs[j].len = (uint8_t)len;
        segs[j].klen = (uint8_t)std::min(len, kMaxKeyLen);
        segs[j].pad = 0;
        segs[j].off = 0;
        start += len;
    }
    *nseg = S;
    return true;
}

bool build_seed_index(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                      std::vector<SeedFam> &out_fams, std::vector<uint32_t> &offsets,
                      std::vector<uint16_t> &lists) {
    SeedSeg layout[kMaxSeg];
    int S = 0;
    if (!seed_layout(K, &S, layout)) return false;
    double frac = 0;
    for (int j = 0; j < S; ++j) frac += 1.0 / (double)(1u << (2 * layout[j].klen));
    if (frac > 0.5) return false;  // the index would not halve the comparisons
    out_fams.assign((size_t)n_fams, SeedFam{});
    offsets.clear();
    lists.clear();
    for (int f = 0; f < n_fams; ++f) {
        const int G = fams[f].gend - fams[f].gbeg;
        if (G > 65535) return false;
        SeedFam &sf = out_fams[(size_t)f];
        sf.nseg = S;
        sf.list_off = (uint32_t)lists.size();
        lists.resize(lists.size() + (size_t)S * (size_t)G);
        for (int j = 0; j < S; ++j) {
            SeedSeg sg = layout[j];
            sg.off = (uint32_t)offsets.size();
            const uint32_t nb = 1u << (2 * sg.klen);
            const uint32_t km = (1u << sg.klen) - 1u;
            std::vector<uint32_t> cnt(nb + 1, 0);
            std::vector<uint32_t> code((size_t)G);
            for (int i = 0; i < G; ++i) {
                const GuideRec &r = recs[fams[f].gbeg + i];
                code[(size_t)i] = (((r.h >> sg.start) & km) << sg.klen) | ((r.l >> sg.start) & km);
                cnt[code[(size_t)i] + 1]++;
            }
            for (uint32_t c = 0; c < nb; ++c) cnt[c + 1] += cnt[c];
            offsets.insert(offsets.end(), cnt.begin(), cnt.end());
            std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
            uint16_t *Lp = lists.data() + sf.list_off + (size_t)j * (size_t)G;
            for (int i = 0; i < G; ++i) Lp[fill[code[(size_t)i]]++] = (uint16_t)i;
            sf.seg[j] = sg;
        }
    }
    return true;
}

}  // namespace bgo
