// Segment-mask scan (scan mode 3): the pigeonhole filter of scan mode 2 with
// the index stored as guide bitmasks.
//
// Exactness is the argument of bgo_seed.cu: a hit has at most K raw
// mismatches over the 20 guide positions, so with K + 1 disjoint segments at
// least one segment of every hit matches the genome exactly.  Here the key of
// segment j is its first <= 4 bases (code c < 256), and for every group of at
// most 128 guides of a PAM family the table holds, per (j, c), the bitmask of
// the group's guides whose segment-j key is c.  The candidates of a position
// are the OR of the K + 1 looked-up masks: every guide that could be a hit,
// each exactly once, so no de-duplication is needed.  Each candidate gets the
// reference's full compare (XOR / pair-OR / popcount, then the N correction,
// beguidedoff/cuda_search.py:272-308).
//
// Layout.  As in mode 2, warps work independently on chunks of positions whose
// H/L/N words are double-buffered in shared memory with cp.async; per family
// the compiled PAM test runs on 32 positions per lane and word, passing
// positions are compacted with one warp scan and processed one per lane.  A
// lane computes its K + 1 segment codes once per position and reuses them for
// every group of the family; a group costs K + 1 shared-memory loads of 4, 8
// or 16 bytes, then one compare per candidate.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "bgo_device.cuh"
#include "bgo_internal.cuh"

namespace bgo {

template <int K>
struct SegM {
    static constexpr int S = K + 1;
    static constexpr int q = kGuideLen / S, r = kGuideLen % S;
    __host__ __device__ static constexpr int start(int j) { return j * q + (j < r ? j : r); }
    __host__ __device__ static constexpr int len(int j) { return q + (j < r ? 1 : 0); }
    __host__ __device__ static constexpr int klen(int j) {
        return len(j) < kMaskKeyLen ? len(j) : kMaskKeyLen;
    }
    // first code of segment j in a group's table (codes of earlier segments)
    __host__ __device__ static constexpr int base(int j) {
        return j == 0 ? 0 : base(j - 1) + (1 << (2 * klen(j - 1)));
    }
    __host__ __device__ static constexpr int codes() { return base(S); }
};

// Codes per group table for K mismatches (host side of SegM<K>::codes()).
static int mask_codes(int K) {
    const int S = K + 1, q = kGuideLen / S, r = kGuideLen % S;
    int c = 0;
    for (int j = 0; j < S; ++j) c += 1 << (2 * std::min(q + (j < r ? 1 : 0), kMaskKeyLen));
    return c;
}

template <int K>
__device__ __forceinline__ void mask_finish(const ScanParams &p, int cm, uint2 e, uint32_t row_at,
                                            uint32_t n20g, uint32_t ne, uint64_t slot,
                                            uint64_t pos) {
    int mmf = cm;
    if (n20g) {
        const uint32_t eh = (ne & 2u) ? e.x : ~e.x;
        const uint32_t el = (ne & 1u) ? e.y : ~e.y;
        mmf = cm + __popc(n20g & eh & el);
    }
    if (mmf > K) return;
    const uint32_t row = __ldg(&p.guides[row_at].row);
    if (semit(((uint64_t)row << 39) | (slot << 38) | (pos << 6) | (uint64_t)mmf, p.keys, p.cap,
          p.counter))
        mark_dropped(pos, slot, p.drop_bits, p.drop_base1);
}

template <int CH>
struct MaskChunk {
    static constexpr int kRows = CH / 1024;      // 32-position words per lane
    static constexpr int kWords = CH / 32 + 4;   // + halo, a multiple of 4 words
    static constexpr int kVecs = kWords / 4;     // 16-byte copies per plane
    static constexpr size_t kBuf = 3 * kWords * sizeof(uint32_t);
    static constexpr size_t kSlice = (2 * kBuf + CH * sizeof(uint16_t) + 15) / 16 * 16;
    static_assert(kWords % 4 == 0, "chunk copies are whole 16-byte vectors");
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) / 16 * 16; }

// Bytes of the shared copies of the index (everything before the warp slices).
__host__ __device__ inline size_t mask_index_bytes(const MaskArgs &ma) {
    return align16(sizeof(uint32_t) * (size_t)ma.table_words) +
           align16(sizeof(uint2) * (size_t)ma.n_guides) + sizeof(MaskGroup) * (size_t)ma.n_groups +
           sizeof(MaskFam) * (size_t)ma.n_fams;
}

template <int K, int CH>
__global__ void __launch_bounds__(kMaskThreads, 3) scan_mask_kernel(ScanParams p, MaskArgs ma) {
    constexpr int S = K + 1;
    using C = MaskChunk<CH>;
    constexpr int kWarps = kMaskThreads / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *sTab = reinterpret_cast<uint32_t *>(smem);
    uint2 *sGd = reinterpret_cast<uint2 *>(smem + align16(sizeof(uint32_t) * (size_t)ma.table_words));
    MaskGroup *sGrp = reinterpret_cast<MaskGroup *>(
        reinterpret_cast<unsigned char *>(sGd) + align16(sizeof(uint2) * (size_t)ma.n_guides));
    MaskFam *sFam = reinterpret_cast<MaskFam *>(sGrp + ma.n_groups);
    unsigned char *slices = smem + mask_index_bytes(ma);
    __shared__ unsigned long long sCand;

    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
    unsigned char *slice = slices + warp * C::kSlice;
    uint16_t *wList = reinterpret_cast<uint16_t *>(slice + 2 * C::kBuf);

    {
        const uint4 *src = reinterpret_cast<const uint4 *>(ma.table);
        uint4 *dst = reinterpret_cast<uint4 *>(sTab);
        for (int i = t; i < ma.table_words / 4; i += kMaskThreads) dst[i] = src[i];
    }
    for (int i = t; i < ma.n_guides; i += kMaskThreads) sGd[i] = ma.guides[i];
    for (int i = t; i < ma.n_groups; i += kMaskThreads) sGrp[i] = ma.groups[i];
    for (int i = t; i < ma.n_fams; i += kMaskThreads) sFam[i] = ma.fams[i];
    if (t == 0) sCand = 0;
    __syncthreads();

    const int64_t chunks0 = p.strand[0].n_tiles;
    const int64_t n_chunks = p.tiles_total;
    const int64_t stride = (int64_t)gridDim.x * kWarps;
    // chunk c's words [c*CH/32, c*CH/32 + kWords) of the three planes (the
    // planes are padded so that the copy never leaves them)
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
    const int64_t c_first = (int64_t)blockIdx.x * kWarps + warp;
    if (c_first < n_chunks) issue(c_first, 0);
    cp_async_commit();
    int buf = 0;
    for (int64_t c = c_first; c < n_chunks; c += stride, buf ^= 1) {
        if (c + stride < n_chunks) issue(c + stride, buf ^ 1);
        cp_async_commit();
        cp_async_wait<1>();  // this chunk's copies are done; the next one is in flight
        __syncwarp();
        const uint32_t *wH = reinterpret_cast<const uint32_t *>(slice + buf * C::kBuf);
        const uint32_t *wL = wH + C::kWords;
        const uint32_t *wN = wL + C::kWords;
        const bool second = c >= chunks0;
        const int64_t lc = second ? c - chunks0 : c;
        const int64_t total_bp = second ? p.strand[1].total_bp : p.strand[0].total_bp;
        const int has_n = second ? p.strand[1].has_n : p.strand[0].has_n;
        const uint32_t ne = (uint32_t)(second ? p.strand[1].n_encoded : p.strand[0].n_encoded);
        const uint64_t slot = (uint64_t)(second ? p.strand[1].slot : p.strand[0].slot);
        const int64_t base = lc * CH;
        const int64_t lim64 = total_bp - kSiteSpan - base;
        const int lim = lim64 > CH ? CH : (int)lim64;

        for (int f = p.fam_begin; f < p.fam_end; ++f) {
            const uint32_t win_off = p.fams[f].three_prime ? 0u : (uint32_t)p.fams[f].plen;
            const int n_tests = sFam[f].n_tests;
            uint32_t tsh[kMaxPam], tcd[kMaxPam];
#pragma unroll
            for (int k = 0; k < kMaxPam; ++k) {
                tsh[k] = sFam[f].pam_shift[k];
                tcd[k] = sFam[f].pam_code[k];
            }
            uint32_t pass[C::kRows];
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < C::kRows; ++u) {
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
            for (int u = 0; u < C::kRows; ++u) {
                uint32_t m = pass[u];
                while (m) {
                    const int j = __ffs(m) - 1;
                    m &= m - 1u;
                    wList[off++] = (uint16_t)(32 * (u * 32 + lane) + j);
                }
            }
            __syncwarp();
            const int g0 = sFam[f].g0, g1 = sFam[f].g1;
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
                // the position's K + 1 segment codes, shared by all groups
                uint32_t code[S];
#pragma unroll
                for (int j = 0; j < S; ++j) {
                    const int st = SegM<K>::start(j), kl = SegM<K>::klen(j);
                    const uint32_t km = (1u << kl) - 1u;
                    code[j] = (uint32_t)SegM<K>::base(j) +
                              ((((h20 >> st) & km) << kl) | ((l20 >> st) & km));
                }
                for (int g = g0; g < g1; ++g) {
                    const MaskGroup G = sGrp[g];
                    uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
                    if (G.words == 4) {
                        const uint4 *tb = reinterpret_cast<const uint4 *>(sTab + G.table_off);
#pragma unroll
                        for (int j = 0; j < S; ++j) {
                            const uint4 v = tb[code[j]];
                            a0 |= v.x;
                            a1 |= v.y;
                            a2 |= v.z;
                            a3 |= v.w;
                        }
                    } else if (G.words == 2) {
                        const uint2 *tb = reinterpret_cast<const uint2 *>(sTab + G.table_off);
#pragma unroll
                        for (int j = 0; j < S; ++j) {
                            const uint2 v = tb[code[j]];
                            a0 |= v.x;
                            a1 |= v.y;
                        }
                    } else {
                        const uint32_t *tb = sTab + G.table_off;
#pragma unroll
                        for (int j = 0; j < S; ++j) a0 |= tb[code[j]];
                    }
                    if (!has) a0 = a1 = a2 = a3 = 0u;
                    cand += __popc(a0) + __popc(a1) + __popc(a2) + __popc(a3);
                    uint64_t lo = ((uint64_t)a1 << 32) | a0, hi = ((uint64_t)a3 << 32) | a2;
                    const uint2 *gd = sGd + G.guide_off;
                    while (lo | hi) {
                        const bool use_lo = lo != 0ull;
                        const uint64_t x = use_lo ? lo : hi;
                        const int idx = (__ffsll((long long)x) - 1) + (use_lo ? 0 : 64);
                        if (use_lo) lo &= lo - 1ull;
                        else hi &= hi - 1ull;
                        const uint2 e = gd[idx];
                        const int cm = __popc((h20 ^ e.x) | (l20 ^ e.y));
                        if (cm <= K)
                            mask_finish<K>(p, cm, e, G.gbeg + (uint32_t)idx, n20g, ne, slot, pos);
                    }
                }
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

size_t mask_smem_bytes(const MaskArgs &ma) {
    const size_t slice = ma.chunk_sites == 1024 ? MaskChunk<1024>::kSlice : MaskChunk<2048>::kSlice;
    return mask_index_bytes(ma) + (size_t)(kMaskThreads / 32) * slice;
}

template <int K, int CH>
static int launch_kc(const ScanParams &p, const MaskArgs &ma, int sm_count, int ctas_per_sm,
                     cudaStream_t s) {
    const size_t smem = mask_smem_bytes(ma);
    static size_t configured = 0;
    if (smem > configured) {
        BGO_CUDA(cudaFuncSetAttribute(scan_mask_kernel<K, CH>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = smem;
    }
    int per_sm = 0;
    BGO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, scan_mask_kernel<K, CH>,
                                                           kMaskThreads, smem));
    if (per_sm < 1) per_sm = 1;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
    const int warps = kMaskThreads / 32;
    const int64_t blocks_needed = (p.tiles_total + warps - 1) / warps;
    const int64_t grid = std::min<int64_t>(blocks_needed, (int64_t)sm_count * per_sm);
    scan_mask_kernel<K, CH><<<(unsigned)grid, kMaskThreads, smem, s>>>(p, ma);
    BGO_CUDA(cudaGetLastError());
    return BGO_OK;
}

template <int CH>
static int launch_c(const ScanParams &p, const MaskArgs &ma, int sm_count, int ctas_per_sm,
                    cudaStream_t s) {
    switch (p.max_mm) {
        case 0: return launch_kc<0, CH>(p, ma, sm_count, ctas_per_sm, s);
        case 1: return launch_kc<1, CH>(p, ma, sm_count, ctas_per_sm, s);
        case 2: return launch_kc<2, CH>(p, ma, sm_count, ctas_per_sm, s);
        case 3: return launch_kc<3, CH>(p, ma, sm_count, ctas_per_sm, s);
        case 4: return launch_kc<4, CH>(p, ma, sm_count, ctas_per_sm, s);
        case 5: return launch_kc<5, CH>(p, ma, sm_count, ctas_per_sm, s);
        case 6: return launch_kc<6, CH>(p, ma, sm_count, ctas_per_sm, s);
        case 7: return launch_kc<7, CH>(p, ma, sm_count, ctas_per_sm, s);
        default:
            set_error("segment masks: max_mismatches outside 0..7");
            return BGO_ERR_ARG;
    }
}

int launch_mask_kernel(const ScanParams &p, const MaskArgs &ma, int sm_count, int ctas_per_sm,
                       cudaStream_t s) {
    if (ma.chunk_sites == 1024) return launch_c<1024>(p, ma, sm_count, ctas_per_sm, s);
    if (ma.chunk_sites == 2048) return launch_c<2048>(p, ma, sm_count, ctas_per_sm, s);
    set_error("segment masks: chunk_sites must be 1024 or 2048");
    return BGO_ERR_ARG;
}

// The host index for K mismatches and groups of at most group_max guides;
// false when K is outside 0..7.
bool build_mask_index(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                      int group_max, std::vector<MaskFam> &out_fams,
                      std::vector<MaskGroup> &groups, std::vector<uint32_t> &table,
                      std::vector<uint2> &guides) {
    if (K < 0 || K > kMaskMaxK || group_max < 1 || group_max > kMaskGroupMax) return false;
    const int S = K + 1, q = kGuideLen / S, r = kGuideLen % S;
    const int n_codes = mask_codes(K);
    out_fams.assign((size_t)n_fams, MaskFam{});
    groups.clear();
    table.clear();
    guides.clear();
    for (int f = 0; f < n_fams; ++f) {
        SeedFam prog{};
        pam_program(fams[f], prog);
        MaskFam &mf = out_fams[(size_t)f];
        mf.n_tests = prog.n_tests;
        for (int k = 0; k < kMaxPam; ++k) {
            mf.pam_shift[k] = prog.pam_shift[k];
            mf.pam_code[k] = prog.pam_code[k];
        }
        mf.g0 = (uint16_t)groups.size();
        const int G = fams[f].gend - fams[f].gbeg;
        for (int c0 = 0; c0 < G; c0 += group_max) {
            const int n = std::min(group_max, G - c0);
            MaskGroup g{};
            g.n = (uint16_t)n;
            g.words = (uint8_t)(n <= 32 ? 1 : n <= 64 ? 2 : 4);
            // width-aligned start (16-byte vectors for 4-word masks)
            size_t at = (table.size() + g.words - 1) / g.words * g.words;
            g.table_off = (uint32_t)at;
            table.resize(at + (size_t)n_codes * g.words, 0u);
            g.guide_off = (uint32_t)guides.size();
            g.gbeg = (uint32_t)(fams[f].gbeg + c0);
            int code_base = 0;
            for (int j = 0; j < S; ++j) {
                const int st = j * q + std::min(j, r);
                const int kl = std::min(q + (j < r ? 1 : 0), kMaskKeyLen);
                const uint32_t km = (1u << kl) - 1u;
                for (int i = 0; i < n; ++i) {
                    const GuideRec &rr = recs[fams[f].gbeg + c0 + i];
                    const uint32_t code = (((rr.h >> st) & km) << kl) | ((rr.l >> st) & km);
                    table[at + ((size_t)code_base + code) * g.words + (size_t)(i >> 5)] |=
                        1u << (i & 31);
                }
                code_base += 1 << (2 * kl);
            }
            for (int i = 0; i < n; ++i) {
                const GuideRec &rr = recs[fams[f].gbeg + c0 + i];
                guides.push_back(make_uint2(rr.h & 0xFFFFFu, rr.l & 0xFFFFFu));
            }
            groups.push_back(g);
            if (groups.size() > 65535) return false;
        }
        mf.g1 = (uint16_t)groups.size();
    }
    table.resize((table.size() + 3) / 4 * 4, 0u);  // whole 16-byte vectors
    return true;
}

}  // namespace bgo
