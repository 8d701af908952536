// Segment-indexed scan (scan mode 2): the same hits as scan_kernel with far
// fewer guide comparisons.
//
// Exactness.  A hit has at most K = max_mismatches raw mismatches over the 20
// guide positions (the N correction only adds to the raw count,
// beguidedoff/cuda_search.py:272-308).  Split the 20 positions into
// S = K / (TOL + 1) + 1 disjoint segments and key each by its first <= 6
// bases.  The key regions are disjoint and S * (TOL + 1) > K, so by the
// pigeonhole principle one key region of every hit differs from the guide in
// at most TOL bases.  The host builds, per PAM family and region, buckets of
// guides under each key they can match: the guide's own key for TOL = 0, and
// also every single-base substitution of it for TOL = 1 (fewer, longer
// regions: 3 lookups instead of 6 at K = 5).  For each PAM-passing position
// the kernel looks up the bucket of each region's key and runs the reference's
// full compare (XOR / pair-OR / popcount, then the N correction) on those
// candidates only.  A candidate reached through region j is reported only if
// no earlier region differs in at most TOL bases, so each (position, guide)
// hit is emitted once.
//
// Layout.  The index (family PAM programs, bucket tables, entry lists) is
// copied into shared memory once per CTA: CTAs of 256 threads (3 or 4 per SM)
// or one CTA of 768 threads per SM, so that 24 warps share one copy of a large
// index.  Warps then work independently (no CTA barrier after the start): each
// warp takes chunks of 1,024 or 2,048 positions of one strand and copies the
// next chunk's H/L/N words with cp.async while it works on the current one
// (double buffering).  Per PAM family it runs the family's PAM tests on 32
// positions per lane and word (funnel shifts + LOP3 against host-decoded
// masks), compacts the passing positions with one warp scan, then processes
// them 32 per round (one per lane): the lane computes its region keys, loads
// each bucket descriptor and compares the bucket's first one or two entries
// inline (all lanes in step, predicated).  Guides beyond those are walked by
// their lane or spread over the warp as ranges in a queue.  The region layout
// is a compile-time function of (K, TOL).  Hits are appended with one
// atomicAdd per warp.
#include <cuda_runtime.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "bgo_seed_kernel.cuh"

namespace bgo {

size_t seed_smem_bytes(const SeedArgs &sa, int chunk_sites, int warps, bool walk) {
    size_t b = sizeof(SeedFam) * sa.n_fams + sizeof(uint2) * sa.n_lists +
               sizeof(uint32_t) * sa.n_offsets + sizeof(uint16_t) * sa.n_lists;
    b = (b + 15) / 16 * 16;
    const size_t slice = chunk_sites == 1024
                             ? (walk ? SeedChunk<1024, 1>::kSlice : SeedChunk<1024, 0>::kSlice)
                             : (walk ? SeedChunk<2048, 1>::kSlice : SeedChunk<2048, 0>::kSlice);
    return b + (size_t)warps * slice;
}

// The kernel form a tuning selects walks its leftover guides per lane for
// tolerance 1 (always), and for tolerance 0 with range_walk unless two guides
// per bucket are compared inline; launch_seed_kernel dispatches the same way.
size_t seed_tuning_smem(const SeedArgs &sa, const bgo_tuning &t) {
    const int chunk = t.chunk_sites ? t.chunk_sites : 2048;
    const int warps = t.min_blocks == 1   ? SeedCta<1>::kWarps
                      : t.min_blocks == 2 ? SeedCta<2>::kWarps
                                          : SeedCta<3>::kWarps;
    const bool walk = t.tolerance == 1 || (t.inline_entries != 2 && t.range_walk == 1);
    return seed_smem_bytes(sa, chunk, warps, walk);
}

int launch_seed_t1(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                   int min_blocks, int ctas_per_sm, cudaStream_t s);
int launch_seed_t1i1(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                     int min_blocks, int ctas_per_sm, cudaStream_t s);
int launch_seed_t0i2(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                     int min_blocks, int ctas_per_sm, cudaStream_t s);
int launch_seed_t0walk(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                       int min_blocks, int ctas_per_sm, cudaStream_t s);

int launch_seed_kernel(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                       int min_blocks, int tolerance, int inline_entries, int range_walk,
                       int ctas_per_sm, cudaStream_t s) {
    if (chunk_sites != 1024 && chunk_sites != 2048) {
        set_error("segment index: chunk_sites must be 1024 or 2048");
        return BGO_ERR_ARG;
    }
    if (tolerance == 1)
        return inline_entries == 1
                   ? launch_seed_t1i1(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s)
                   : launch_seed_t1(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
    if (inline_entries == 2)
        return launch_seed_t0i2(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
    if (range_walk == 1)
        return launch_seed_t0walk(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
    return launch_form<0, 1, 0>(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
}

// PAM test program of a family: one test per constrained position (an N is
// skipped).  Sets whose members share a fixed bit pattern of the 2-bit code
// (single bases, R, Y, M, K) compare bits; S, W and the three-base codes use
// the generic allowed-set select.
void pam_program(const FamilyDesc &F, SeedFam &sf) {
    const uint32_t pam_off = F.three_prime ? 20u : 0u;
    sf.n_tests = 0;
    sf.pam_generic = 0;
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
        const int t = sf.n_tests;
        sf.pam_shift[t] = (uint8_t)(pam_off + (uint32_t)k);
        sf.pam_code[t] = code;
        auto all = [](uint32_t bit) { return bit ? 0xFFFFFFFFu : 0u; };
        sf.pam_mask[t] = make_uint4(all(code & 1u), all(code & 2u), all(code & 4u), all(code & 8u));
        if (code & 0x100u) sf.pam_generic |= (uint8_t)(1u << t);
        sf.n_tests++;
    }
}

// The host index for K mismatches and tolerance tols[f] (0 or 1) per family;
// false when it does not apply (K outside 0..7, or a bucket list too long for
// the 16-bit descriptor fields).  Bucket descriptor = entry start within the
// region's list | count << 16; region j's list starts at the family's
// list_off + seg[j].ent.
bool build_seed_index(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                      const std::vector<int> &tols, std::vector<SeedFam> &out_fams,
                      std::vector<uint32_t> &offsets, std::vector<uint2> &entries,
                      std::vector<uint16_t> &entry_idx) {
    if (K < 0 || K > kSeedMaxK || (int)tols.size() < n_fams) return false;
    out_fams.assign((size_t)n_fams, SeedFam{});
    offsets.clear();
    entries.clear();
    entry_idx.clear();
    for (int f = 0; f < n_fams; ++f) {
        const int tol = tols[(size_t)f];
        if (tol < 0 || tol > 1) return false;
        const int S = K / (tol + 1) + 1;
        const int q = kGuideLen / S, r = kGuideLen % S;
        const int G = fams[f].gend - fams[f].gbeg;
        SeedFam &sf = out_fams[(size_t)f];
        sf.nseg = S;
        pam_program(fams[f], sf);
        sf.list_off = (uint32_t)entries.size();
        uint32_t ent = 0;
        for (int j = 0; j < S; ++j) {
            SeedSeg sg{};
            sg.start = (uint8_t)(j * q + std::min(j, r));
            sg.len = (uint8_t)(q + (j < r ? 1 : 0));
            sg.klen = (uint8_t)std::min<int>(sg.len, kMaxKeyLen);
            sg.off = (uint32_t)offsets.size();
            sg.ent = ent;
            const int kl = sg.klen;
            const uint32_t nb = 1u << (2 * kl);
            const uint32_t km = (1u << kl) - 1u;
            // (variant key, family-local guide index) pairs of this region
            std::vector<std::pair<uint32_t, uint16_t>> keys;
            keys.reserve((size_t)G * (1 + (size_t)tol * 3 * kl));
            for (int i = 0; i < G; ++i) {
                const GuideRec &rr = recs[fams[f].gbeg + i];
                const uint32_t hk = (rr.h >> sg.start) & km, lk = (rr.l >> sg.start) & km;
                keys.emplace_back((hk << kl) | lk, (uint16_t)i);
                if (tol == 1) {
                    for (int b = 0; b < kl; ++b) {
                        const uint32_t cur = (((hk >> b) & 1u) << 1) | ((lk >> b) & 1u);
                        for (uint32_t v = 0; v < 4; ++v) {
                            if (v == cur) continue;
                            const uint32_t h2 = (hk & ~(1u << b)) | ((v >> 1) << b);
                            const uint32_t l2 = (lk & ~(1u << b)) | ((v & 1u) << b);
                            keys.emplace_back((h2 << kl) | l2, (uint16_t)i);
                        }
                    }
                }
            }
            if (keys.size() > 65535) return false;
            std::vector<uint32_t> cnt(nb + 1, 0);
            for (const auto &kv : keys) cnt[kv.first + 1]++;
            for (uint32_t c = 0; c < nb; ++c) cnt[c + 1] += cnt[c];
            for (uint32_t c = 0; c < nb; ++c)
                offsets.push_back(cnt[c] | ((cnt[c + 1] - cnt[c]) << 16));
            std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
            const size_t e_base = entries.size();
            entries.resize(e_base + keys.size());
            entry_idx.resize(entries.size());
            for (const auto &kv : keys) {
                const GuideRec &rr = recs[fams[f].gbeg + kv.second];
                const size_t at = e_base + fill[kv.first]++;
                entries[at] = make_uint2(rr.h & 0xFFFFFu, rr.l & 0xFFFFFu);
                entry_idx[at] = kv.second;
            }
            ent += (uint32_t)keys.size();
            sf.seg[j] = sg;
        }
        if (entries.size() >= (1u << 22)) return false;
    }
    return true;
}

}  // namespace bgo
