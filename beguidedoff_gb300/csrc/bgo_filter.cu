// Prefiltered segment-index scan (scan mode 2 with tuning.prefilter): the same
// hits as the segment index, with a cheap lossless test in front of it.
//
// Regions.  The tolerance-1 segment index splits the 20 guide positions into
// S = K / 2 + 1 disjoint regions (SegT<K, 1>).  For a hit the raw mismatch
// counts d_1..d_S of the regions sum to at most K (the N correction only adds
// to the raw count, beguidedoff/cuda_search.py:272-308).  If no region is
// exact, every d_j >= 1 and sum (d_j - 1) <= K - S, so at least M = 2S - K
// regions have d_j = 1.  Hence every hit with guide g has
//     some region j with d_j(g) = 0, or
//     at least M regions with d_j(g) <= 1.
// A region's key (its first <= 7 bases) differs from the guide's in at most
// d_j bases, so the same holds with keys in place of regions.
//
// Filter tables.  Per PAM family and region, one byte per key (4^7 keys for a
// region of >= 7 bases): bit 0 is set if some guide's key equals it; bit
// 1 + (i mod 7) is set if guide i's key is within one substitution of it
// (its own key included).  For each PAM-passing position the kernel reads the
// S bytes of its keys and keeps the position iff
//     (OR of the bytes) has bit 0, or some colour bit is set in >= M bytes
// (M = 1: any colour bit; M > S: bit 0 only).  Guide g with an exact region
// sets bit 0; with M regions within one it sets its colour in M bytes: the
// test never drops a hit.  For 100 NGG guides at K = 4 about 6% of PAM-passing
// positions survive (bit 0 of the 6-base region alone passes 2.4%).
//
// Survivors.  Each kept position (its 20-base window planes, the N bits of
// the window when its 26-position span holds an N, strand and position) goes
// into a per-warp queue in shared memory.  Whenever the queue holds a full
// warp, every lane runs the segment index on one survivor: per region the
// bucket of the key's single-substitution neighbourhood, then the reference's
// full compare and N correction (finish_candidate, as in scan_seed_kernel).
// Each lane tests three list positions per round; the round's survivors go
// into the queue together (a lane without a survivor stores into a spare
// slot, so the round has no per-lane branch), and the queue is drained a warp
// at a time.
//
// Survivor index.  When the largest launch family's index fits beside the
// tables and slices, and its descriptors fit 16 bits (entry starts < 4,096,
// bucket counts < 16), the CTA copies each family's descriptors, the
// family-local guide index of every entry (2 bytes) and the family's guide
// planes (8 bytes per guide) into shared memory at the family's start; else
// survivors read the index (with full guide planes per entry) from global
// memory (L1/L2).
//
// Work.  One persistent 896-thread CTA (28 warps) per SM.  Per launch family the warps
// take the first three quarters of the chunks in a static grid stride and
// claim the rest in runs of two from a per-family counter (atomicAdd), so the
// families of a mixed plan share one launch without a tail per family; the
// CTA loads the next family's filter tables after all its warps are done with
// the previous one (a CTA barrier per family).  Chunks of 2,048 or 4,096
// positions are copied into the warp's double buffer by one lane with two
// 1-D bulk copies (cp.async.bulk, the H and L planes) completing on an
// mbarrier; the wait is bounded and reports BGO_ERR_TIMEOUT through the
// engine.  The N plane is not staged: the strand's N summary (one bit per
// 1,024 positions, built when the strand is uploaded) tells whether a chunk
// or its halo holds an N, and only then do the chunk's survivors read their
// N words from global memory.  That leaves room for 28 warps' slices beside
// the tables and the survivor index.
//
// This translation unit instantiates the 2,048-position form with the index
// in shared memory; bgo_filter_2k_g.cu, bgo_filter_4k.cu and bgo_filter_4k_s.cu
// the other forms.
#include <cuda_runtime.h>

#include <vector>

#include "bgo_filter_kernel.cuh"

namespace bgo {

size_t filter_smem_limit() { return (size_t)kFilterSmemLimit; }

uint32_t filter_tab_bytes(int K) {
    switch (K) {
        case 0: return FiltT<0>::kBytesAl;
        case 1: return FiltT<1>::kBytesAl;
        case 2: return FiltT<2>::kBytesAl;
        case 3: return FiltT<3>::kBytesAl;
        case 4: return FiltT<4>::kBytesAl;
        case 5: return FiltT<5>::kBytesAl;
        case 6: return FiltT<6>::kBytesAl;
        case 7: return FiltT<7>::kBytesAl;
        default: return 0;
    }
}

bool build_filter_tables(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                         std::vector<uint8_t> &tables, uint32_t &tab_bytes) {
    if (K < 0 || K > kSeedMaxK) return false;
    tab_bytes = filter_tab_bytes(K);
    tables.assign((size_t)n_fams * tab_bytes, 0);
    const int S = K / 2 + 1;
    const int q = kGuideLen / S, r = kGuideLen % S;
    for (int f = 0; f < n_fams; ++f) {
        uint8_t *T = tables.data() + (size_t)f * tab_bytes;
        uint32_t off = 0;
        for (int j = 0; j < S; ++j) {
            const int start = j * q + std::min(j, r);
            const int len = q + (j < r ? 1 : 0);
            const int kl = std::min(len, kFilterKeyLen);
            const uint32_t km = (1u << kl) - 1u;
            for (int i = 0; i < fams[f].gend - fams[f].gbeg; ++i) {
                const GuideRec &g = recs[fams[f].gbeg + i];
                const uint8_t colour = (uint8_t)(2u << (i % kFilterColors));
                const uint32_t hk = (g.h >> start) & km, lk = (g.l >> start) & km;
                T[off + ((hk << kl) | lk)] |= (uint8_t)(1u | colour);
                for (int b = 0; b < kl; ++b) {
                    const uint32_t cur = (((hk >> b) & 1u) << 1) | ((lk >> b) & 1u);
                    for (uint32_t v = 0; v < 4; ++v) {
                        if (v == cur) continue;
                        const uint32_t h2 = (hk & ~(1u << b)) | ((v >> 1) << b);
                        const uint32_t l2 = (lk & ~(1u << b)) | ((v & 1u) << b);
                        T[off + ((h2 << kl) | l2)] |= colour;
                    }
                }
            }
            off += 1u << (2 * kl);
        }
        if (off > tab_bytes) return false;
    }
    return true;
}

size_t filter_smem_fixed_bytes(int K, int chunk_sites) {
    const size_t per = (sizeof(SeedFam) + 15) / 16 * 16 +
                       (size_t)kFilterWarps * (chunk_sites == 4096 ? FiltChunk<4096>::kSlice
                                                                   : FiltChunk<2048>::kSlice);
    return filter_tab_bytes(K) + per;
}

int launch_filter_2k_g(const ScanParams &p, const FilterArgs &fa, int sm_count, cudaStream_t s);
int launch_filter_4k_g(const ScanParams &p, const FilterArgs &fa, int sm_count, cudaStream_t s);
int launch_filter_4k_s(const ScanParams &p, const FilterArgs &fa, int sm_count, cudaStream_t s);

int launch_filter_kernel(const ScanParams &p, const FilterArgs &fa, int sm_count, int chunk_sites,
                         cudaStream_t s) {
    if (fa.tab_bytes != (int32_t)filter_tab_bytes(p.max_mm)) {
        set_error("prefiltered segment index: tables built for another max_mismatches");
        return BGO_ERR_ARG;
    }
    if (chunk_sites != 2048 && chunk_sites != 4096) {
        set_error("prefiltered segment index: chunk_sites must be 2048 or 4096");
        return BGO_ERR_ARG;
    }
    if (fa.idx_smem_bytes < 0 || fa.idx_smem_bytes % 16 ||
        filter_smem_fixed_bytes(p.max_mm, chunk_sites) + (size_t)fa.idx_smem_bytes >
            (size_t)kFilterSmemLimit) {
        set_error("prefiltered segment index: the index does not fit in shared memory");
        return BGO_ERR_ARG;
    }
    const bool ism = fa.idx_smem_bytes > 0;
    if (chunk_sites == 4096)
        return ism ? launch_filter_4k_s(p, fa, sm_count, s) : launch_filter_4k_g(p, fa, sm_count, s);
    return ism ? launch_filter_ch<2048, 1>(p, fa, sm_count, s)
               : launch_filter_2k_g(p, fa, sm_count, s);
}

}  // namespace bgo
