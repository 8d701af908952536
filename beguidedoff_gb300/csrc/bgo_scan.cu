// Extensive off-target scan on sm_103a: plans, engine, scan kernel, collect,
// and the search_genome_cuda drop-in.
//
// Semantics follow beguidedoff/cuda_search.py:163-314 (search_chunk_kernel):
//   * positions [0, total_bp - 26) of one strand array, for every PAM length;
//   * PAM test on the raw 2-bit bases (N encodes as A / T there), per IUPAC
//     allowed-set nibble (equivalent to the reference's packed XOR/AND test and
//     its per-base fallback for S/W/B/D/H/V);
//   * raw mismatches = popcount over the 20 guide positions of
//     (genome_high ^ guide_high) | (genome_low ^ guide_low), i.e. the
//     reference's (x | x >> 1) & 0x5555555555 on 2-bit pairs, rejected above
//     max_mismatches;
//   * if any N lies in [pos, pos + 26), add the guide-window N positions whose
//     guide base equals n_encoded, and reject again;
//   * every surviving (row, position) is a hit with the corrected count.
//
// Kernel structure (one CTA = 256 threads = 8192 positions per tile):
//   1. stage the tile's H/L/N words (+ halo) in shared memory;
//   2. per PAM family: each thread tests its 32 positions bit-parallel
//      (funnel shifts + LOP3), the CTA compacts the PAM-passing positions
//      into a shared list (warp scans);
//   3. each thread takes compacted positions and runs the family's guides
//      (staged in shared memory, broadcast reads): 2 LOP3 + POPC per pair;
//   4. hits are appended with one atomicAdd per warp (coalesced groups).
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "bgo_device.cuh"
#include "bgo_internal.cuh"

namespace bgo {

constexpr int kGuideChunk = 512;

__device__ __forceinline__ uint32_t fshr(uint32_t lo, uint32_t hi, uint32_t s) {
    return __funnelshift_r(lo, hi, s);
}

// Bit j set iff the base given by (h_j, l_j) is in IUPAC allowed-set `a`.
__device__ __forceinline__ uint32_t allowed_bits(uint32_t h, uint32_t l, uint32_t a) {
    uint32_t r = 0;
    if (a & 1u) r |= ~h & ~l;
    if (a & 2u) r |= ~h & l;
    if (a & 4u) r |= h & ~l;
    if (a & 8u) r |= h & l;
    return r;
}

// Appends `key`; the lanes executing this call together share one atomicAdd.
__device__ __forceinline__ void emit_key(uint64_t key, uint64_t *keys, int64_t cap,
                                         unsigned long long *counter, uint32_t *drop_bits,
                                         int64_t drop_base1) {
    unsigned act = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(act) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(act));
    base = __shfl_sync(act, base, leader);
    unsigned long long slot = base + (unsigned long long)__popc(act & ((1u << lane) - 1u));
    if (slot < (unsigned long long)cap) keys[slot] = key;
    else mark_dropped((key >> 6) & 0xFFFFFFFFull, (key >> 38) & 1ull, drop_bits, drop_base1);
}

__global__ void __launch_bounds__(kTileThreads) scan_kernel(ScanParams p) {
    __shared__ uint32_t sH[kTileWords], sL[kTileWords], sN[kTileWords];
    __shared__ uint16_t sList[kTileSites];
    __shared__ uint4 sG[kGuideChunk];
    __shared__ int sWarp[kTileThreads / 32];
    __shared__ int sTotal;

    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
    const int K = p.max_mm;

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
        const int64_t base = lt * kTileSites;
        const int64_t w0 = lt * (kTileSites / 32);
        const int64_t valid_end = total_bp - kSiteSpan;

        __syncthreads();  // the previous tile is done with shared memory
        for (int i = t; i < kTileWords; i += kTileThreads) {
            sH[i] = H[w0 + i];
            sL[i] = L[w0 + i];
            sN[i] = N[w0 + i];
        }
        __syncthreads();

        uint32_t valid = 0xFFFFFFFFu;
        {
            int64_t s0 = base + 32 * t;
            if (s0 >= valid_end) valid = 0;
            else if (valid_end - s0 < 32) valid = (1u << (uint32_t)(valid_end - s0)) - 1u;
        }

        for (int f = p.fam_begin; f < p.fam_end; ++f) {
            const FamilyDesc F = p.fams[f];
            const uint32_t pam_off = F.three_prime ? 20u : 0u;
            const uint32_t win_off = F.three_prime ? 0u : (uint32_t)F.plen;

            // (2) PAM test of this thread's 32 positions, then compaction.
            uint32_t pass = valid;
            for (int k = 0; k < F.plen; ++k) {
                const uint32_t a = F.allowed[k] & 15u;
                if (a == 15u) continue;
                const uint32_t s = pam_off + (uint32_t)k;
                pass &= allowed_bits(fshr(sH[t], sH[t + 1], s), fshr(sL[t], sL[t + 1], s), a);
            }
            const int cnt = __popc(pass);
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) sWarp[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                int v = lane < kTileThreads / 32 ? sWarp[lane] : 0;
                int inc = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                    if (lane >= o) inc += u;
                }
                if (lane < kTileThreads / 32) sWarp[lane] = inc - v;
                if (lane == kTileThreads / 32 - 1) sTotal = inc;
            }
            __syncthreads();
            {
                int off = sWarp[warp] + incl - cnt;
                uint32_t m = pass;
                while (m) {
                    int j = __ffs(m) - 1;
                    m &= m - 1u;
                    sList[off++] = (uint16_t)(32 * t + j);
                }
            }
            __syncthreads();
            const int n_sites = sTotal;
            if (t == 0 && n_sites)
                atomicAdd(p.counter + 1, (unsigned long long)n_sites * (unsigned)(F.gend - F.gbeg));

            // (3) compare every compacted position with the family's guides.
            for (int gc = F.gbeg; gc < F.gend; gc += kGuideChunk) {
                const int gn = min(kGuideChunk, F.gend - gc);
                for (int i = t; i < gn; i += kTileThreads) {
                    const GuideRec r = p.guides[gc + i];
                    sG[i] = make_uint4(r.h, r.l, r.row, 0u);
                }
                __syncthreads();
                for (int idx = t; idx < n_sites; idx += kTileThreads) {
                    const uint32_t s = sList[idx];
                    const uint32_t wo = s + win_off;
                    const uint32_t wi = wo >> 5, b = wo & 31u;
                    const uint32_t h20 = fshr(sH[wi], sH[wi + 1], b) & 0xFFFFFu;
                    const uint32_t l20 = fshr(sL[wi], sL[wi + 1], b) & 0xFFFFFu;
#pragma unroll 4
                    for (int g = 0; g < gn; ++g) {
                        const uint4 G = sG[g];
                        const int c = __popc((h20 ^ G.x) | (l20 ^ G.y));
                        if (c <= K) {
                            int mmf = c;
                            if (has_n) {
                                const uint32_t n26 =
                                    fshr(sN[s >> 5], sN[(s >> 5) + 1], s & 31u) & 0x3FFFFFFu;
                                if (n26) {
                                    const uint32_t n20 = fshr(sN[wi], sN[wi + 1], b) & 0xFFFFFu;
                                    const uint32_t eh = (ne & 2u) ? G.x : ~G.x;
                                    const uint32_t el = (ne & 1u) ? G.y : ~G.y;
                                    mmf = c + __popc(n20 & eh & el);
                                }
                            }
                            if (mmf <= K) {
                                const uint64_t pos = (uint64_t)(base + s);
                                const uint64_t key = ((uint64_t)G.z << 39) | (slot << 38) |
                                                     (pos << 6) | (uint64_t)mmf;
                                emit_key(key, p.keys, p.cap, p.counter, p.drop_bits, p.drop_base1);
                            }
                        }
                    }
                }
                __syncthreads();
            }
        }
    }
}

static int blocks_per_sm() {
    static int cached = 0;
    if (!cached) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, scan_kernel, kTileThreads, 0) !=
                cudaSuccess ||
            n <= 0)
            n = 1;
        cached = n;
    }
    return cached;
}

}  // namespace bgo

using namespace bgo;

// ----------------------------------------------------------------------------
// engine
// ----------------------------------------------------------------------------
extern "C" int bgo_engine_create(int device, bgo_engine **out) {
    if (!out) return BGO_ERR_ARG;
    *out = nullptr;
    BGO_CUDA(cudaSetDevice(device));
    bgo_engine *e = new (std::nothrow) bgo_engine();
    if (!e) return BGO_ERR_OOM;
    e->device = device;
    e->cap = 0;
    cudaError_t ce = cudaMalloc(&e->d_counter, kEngineCounters * sizeof(unsigned long long));
    if (ce == cudaSuccess)
        ce = cudaMemset(e->d_counter, 0, kEngineCounters * sizeof(unsigned long long));
    if (ce == cudaSuccess) ce = cudaMalloc(&e->d_work, kWorkCap * sizeof(uint32_t));
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->keys_done, cudaEventDisableTiming);
    int sms = 0;
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (ce != cudaSuccess) {
        if (e->d_counter) cudaFree(e->d_counter);
        if (e->d_work) cudaFree(e->d_work);
        if (e->keys_done) cudaEventDestroy(e->keys_done);
        delete e;
        return cuda_fail(ce, "bgo_engine_create");
    }
    e->sm_count = sms;
    *out = e;
    return bgo_engine_reserve(e, 1 << 20);
}

extern "C" int bgo_engine_destroy(bgo_engine *e) {
    if (!e) return BGO_OK;
    cudaSetDevice(e->device);
    // the engine's queued work is done before its memory goes back
    if (e->keys_done) cudaEventSynchronize(e->keys_done);
    if (e->d_keys) pool_free(e->device, e->d_keys);
    if (e->d_drop) pool_free(e->device, e->d_drop);
    if (e->d_counter) cudaFree(e->d_counter);
    if (e->d_work) cudaFree(e->d_work);
    if (e->keys_done) cudaEventDestroy(e->keys_done);
    if (e->d_epi) cudaFree(e->d_epi);
    if (e->d_epi_rec) cudaFree(e->d_epi_rec);
    if (e->d_epi_out) cudaFree(e->d_epi_out);
    if (e->d_rank) cudaFree(e->d_rank);
    delete e;
    return BGO_OK;
}

extern "C" int bgo_engine_reserve(bgo_engine *e, int64_t n_hits) {
    if (!e || n_hits < 0) return BGO_ERR_ARG;
    if (n_hits <= e->cap) return BGO_OK;
    BGO_CUDA(cudaSetDevice(e->device));
    int64_t cap = std::max<int64_t>(n_hits, e->cap * 2);
    uint64_t *p = nullptr;
    BGO_CUDA(pool_alloc(e->device, (void **)&p, (size_t)cap * sizeof(uint64_t)));
    // the old buffer may still be read or written by the engine's last scan
    // or epilogue: wait for that work only (not for the device, where other
    // engines' scans may run), then return the buffer to the pool
    BGO_CUDA(cudaEventSynchronize(e->keys_done));
    if (e->d_keys) BGO_CUDA(pool_free(e->device, e->d_keys));
    e->d_keys = p;
    e->cap = cap;
    e->keys_gen++;
    return BGO_OK;
}

extern "C" int bgo_engine_transfer(const bgo_engine *e, int64_t *h2d_bytes, int64_t *d2h_bytes) {
    if (!e || !h2d_bytes || !d2h_bytes) return BGO_ERR_ARG;
    *h2d_bytes = e->h2d_bytes;
    *d2h_bytes = e->d2h_bytes;
    return BGO_OK;
}

extern "C" int bgo_engine_info(const bgo_engine *e, int64_t *hit_capacity, int64_t *n_launches) {
    if (!e) return BGO_ERR_ARG;
    if (hit_capacity) *hit_capacity = e->cap;
    if (n_launches) *n_launches = e->launches;
    return BGO_OK;
}

// ----------------------------------------------------------------------------
// plan
// ----------------------------------------------------------------------------
extern "C" int bgo_plan_create(bgo_engine *engine, const uint64_t *guide_encoded,
                               const uint8_t *pam_masks, const uint8_t *pam_lens,
                               const uint8_t *pam_3prime, int32_t n_guides, void *stream,
                               bgo_plan **out) {
    if (!engine || !out || n_guides < 0 ||
        (n_guides > 0 && (!guide_encoded || !pam_masks || !pam_lens || !pam_3prime))) {
        set_error("bgo_plan_create: invalid argument");
        return BGO_ERR_ARG;
    }
    if (n_guides >= (1 << 25)) {
        set_error("bgo_plan_create: at most 2^25 - 1 guide rows");
        return BGO_ERR_ARG;
    }
    *out = nullptr;
    BGO_CUDA(cudaSetDevice(engine->device));
    // Group rows by (allowed nibbles, length, orientation), first-seen order.
    std::map<std::vector<uint8_t>, int> fam_index;
    std::vector<std::vector<int32_t>> members;
    std::vector<FamilyDesc> fams;
    for (int32_t i = 0; i < n_guides; ++i) {
        const int plen = pam_lens[i];
        if (plen <= 0 || plen > kMaxPam) continue;  // never matches (cuda_search.py:139-140)
        std::vector<uint8_t> key(kMaxPam + 2, 0);
        for (int k = 0; k < plen; ++k) key[k] = pam_masks[i * kMaxPam + k] & 15u;
        key[kMaxPam] = (uint8_t)plen;
        key[kMaxPam + 1] = pam_3prime[i] ? 1 : 0;
        auto it = fam_index.find(key);
        int f;
        if (it == fam_index.end()) {
            f = (int)fams.size();
            fam_index.emplace(key, f);
            FamilyDesc d{};
            for (int k = 0; k < kMaxPam; ++k) d.allowed[k] = key[k];
            d.plen = (uint8_t)plen;
            d.three_prime = key[kMaxPam + 1];
            fams.push_back(d);
            members.emplace_back();
        } else {
            f = it->second;
        }
        members[f].push_back(i);
    }
    std::vector<GuideRec> recs;
    recs.reserve(n_guides);
    for (size_t f = 0; f < fams.size(); ++f) {
        fams[f].gbeg = (int32_t)recs.size();
        for (int32_t i : members[f]) {
            GuideRec r{};
            const uint64_t v = guide_encoded[i];
            for (int k = 0; k < kGuideLen; ++k) {
                const uint32_t b = (uint32_t)((v >> (2 * k)) & 3u);
                r.h |= ((b >> 1) & 1u) << k;
                r.l |= (b & 1u) << k;
            }
            r.row = (uint32_t)i;
            recs.push_back(r);
        }
        fams[f].gend = (int32_t)recs.size();
    }
    bgo_plan *pl = new (std::nothrow) bgo_plan();
    if (!pl) return BGO_ERR_OOM;
    pl->device = engine->device;
    pl->n_guides = n_guides;
    pl->n_active = (int32_t)recs.size();
    pl->n_families = (int32_t)fams.size();
    pl->h_fams = new (std::nothrow) FamilyDesc[fams.size() + 1];
    pl->h_guides = new (std::nothrow) GuideRec[recs.size() + 1];
    pl->seed_k = -1000;
    pl->d_seed_fam = nullptr;
    pl->mask_k = -1000;
    pl->mask_group = 0;
    pl->mask_ok = 0;
    pl->d_mask = nullptr;
    pl->tuning = bgo_tuning{};
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = (pl->h_fams && pl->h_guides) ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = cudaSetDevice(engine->device);
    if (e == cudaSuccess) e = event_take(pl->device, &pl->done);
    if (e == cudaSuccess) {
        std::copy(fams.begin(), fams.end(), pl->h_fams);
        std::copy(recs.begin(), recs.end(), pl->h_guides);
        e = pool_alloc(pl->device, (void **)&pl->d_fams, sizeof(FamilyDesc) * (fams.size() + 1));
    }
    if (e == cudaSuccess)
        e = pool_alloc(pl->device, (void **)&pl->d_guides, sizeof(GuideRec) * (recs.size() + 1));
    if (e == cudaSuccess && !fams.empty())
        e = cudaMemcpyAsync(pl->d_fams, fams.data(), sizeof(FamilyDesc) * fams.size(),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !recs.empty())
        e = cudaMemcpyAsync(pl->d_guides, recs.data(), sizeof(GuideRec) * recs.size(),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(pl->done, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        bgo_plan_destroy(pl);
        return cuda_fail(e, "bgo_plan_create");
    }
    engine->h2d_bytes += (int64_t)(sizeof(FamilyDesc) * fams.size() + sizeof(GuideRec) * recs.size());
    *out = pl;
    return BGO_OK;
}

extern "C" int bgo_plan_destroy(bgo_plan *pl) {
    if (!pl) return BGO_OK;
    cudaSetDevice(pl->device);
    // waits for the plan's last use only, not for the device
    if (pl->done) cudaEventSynchronize(pl->done);
    pool_free(pl->device, pl->d_fams);
    pool_free(pl->device, pl->d_guides);
    pool_free(pl->device, pl->d_seed);
    pool_free(pl->device, pl->d_seed_fam);
    pool_free(pl->device, pl->d_seed_sizes);
    pool_free(pl->device, pl->d_mask);
    pool_free(pl->device, pl->d_filter);
    event_give(pl->device, pl->done);
    delete[] pl->h_fams;
    delete[] pl->h_guides;
    delete pl;
    return BGO_OK;
}

static int check_tuning(const bgo_plan *pl, const bgo_tuning *t) {
    if (!pl || !t) return BGO_ERR_ARG;
    if ((t->chunk_sites != 0 && t->chunk_sites != 1024 && t->chunk_sites != 2048 &&
         !(t->chunk_sites == 4096 && t->prefilter == 1)) ||
        (t->prefilter == 1 && t->chunk_sites == 1024) || t->prefilter < 0 || t->prefilter > 1 ||
        (t->group_guides != 0 && t->group_guides != 32 && t->group_guides != 64 &&
         t->group_guides != 128) ||
        t->ctas_per_sm < 0 || t->split_families < 0 || t->split_families > 1 ||
        (t->min_blocks != 0 && (t->min_blocks < 1 || t->min_blocks > 4)) ||
        t->tolerance < 0 ||
        t->tolerance > 1 || t->family_form < 0 || t->family_form > 1 ||
        (t->inline_entries != 0 && t->inline_entries != 1 && t->inline_entries != 2) ||
        t->range_walk < 0 || t->range_walk > 1) {
        set_error("bgo_plan_set_tuning: chunk_sites 1024|2048 (2048|4096 with prefilter), "
                  "group_guides 32|64|128, ctas_per_sm >= 0, split_families 0|1, min_blocks 1-4, "
                  "tolerance 0|1, family_form 0|1, inline_entries 1|2, range_walk 0|1, "
                  "prefilter 0|1");
        return BGO_ERR_ARG;
    }
    return BGO_OK;
}

extern "C" int bgo_plan_set_tuning(bgo_plan *pl, const bgo_tuning *t) {
    const int rc = check_tuning(pl, t);
    if (rc != BGO_OK) return rc;
    pl->tuning = *t;
    pl->fam_tuning.clear();
    return BGO_OK;
}

extern "C" int bgo_plan_set_family_tuning(bgo_plan *pl, int32_t family, const bgo_tuning *t) {
    const int rc = check_tuning(pl, t);
    if (rc != BGO_OK) return rc;
    if (family < 0 || family >= pl->n_families) {
        set_error("bgo_plan_set_family_tuning: no such family");
        return BGO_ERR_ARG;
    }
    if (pl->fam_tuning.empty()) pl->fam_tuning.assign((size_t)pl->n_families, pl->tuning);
    pl->fam_tuning[(size_t)family] = *t;
    return BGO_OK;
}

extern "C" int bgo_plan_families(const bgo_plan *pl, int32_t *row_family) {
    if (!pl || (pl->n_guides > 0 && !row_family)) return BGO_ERR_ARG;
    for (int32_t i = 0; i < pl->n_guides; ++i) row_family[i] = -1;
    for (int f = 0; f < pl->n_families; ++f)
        for (int g = pl->h_fams[f].gbeg; g < pl->h_fams[f].gend; ++g)
            row_family[pl->h_guides[g].row] = f;
    return BGO_OK;
}

extern "C" int bgo_plan_info(const bgo_plan *pl, int32_t *n_families, int32_t *n_guides) {
    if (!pl) return BGO_ERR_ARG;
    if (n_families) *n_families = pl->n_families;
    if (n_guides) *n_guides = pl->n_guides;
    return BGO_OK;
}

// ----------------------------------------------------------------------------
// scan
// ----------------------------------------------------------------------------
static void fill_strand(StrandDesc &d, const bgo_genome *g, int32_t n_encoded, int32_t slot) {
    d.H = g->d_planes;
    d.L = g->d_planes + g->plane_words;
    d.N = g->d_planes + 2 * g->plane_words;
    d.nsum = g->d_nsum;
    d.total_bp = g->total_bp;
    d.n_tiles = tiles_for(g->total_bp);
    d.has_n = g->has_n;
    d.n_encoded = n_encoded;
    d.slot = slot;
    d.pad = 0;
}

// Builds (once per (max_mismatches, tolerance)) and uploads the plan's segment
// index and its per-family views.  Returns 1 when the index applies to the
// plan's launch form (all families in one launch, or one launch per family),
// 0 when the scan must compare every guide (mode 1), or a negative BGO_ERR_*.
static const bgo_tuning &family_tuning(const bgo_plan *pl, int f) {
    return pl->fam_tuning.empty() ? pl->tuning : pl->fam_tuning[(size_t)f];
}

// The tuning a segment-index launch over index `sa` runs with: the requested
// one when the index and the warps' chunk slices fit in shared memory, else
// the same tolerance and form with 1,024-position chunks, then with fewer
// warps per CTA (a 768-thread CTA steps down to 512, then to 256 threads; a
// 512-thread CTA to 256), each with the requested chunk and then 1,024.  False
// when none fits (the family, or the single launch, compares every guide
// instead).
static bool fitted_seed_tuning(const SeedArgs &sa, const bgo_tuning &t, bgo_tuning &out) {
    const size_t limit = 220 * 1024;
    const int shapes_768[] = {1, 2, 3}, shapes_512[] = {2, 3}, shapes_256[] = {t.min_blocks};
    const int *shapes =
        t.min_blocks == 1 ? shapes_768 : t.min_blocks == 2 ? shapes_512 : shapes_256;
    const int n_shapes = t.min_blocks == 1 ? 3 : t.min_blocks == 2 ? 2 : 1;
    bgo_tuning c = t;
    for (int i = 0; i < n_shapes; ++i) {
        for (int half = 0; half < 2; ++half) {
            c.min_blocks = shapes[i];
            c.chunk_sites = half ? 1024 : t.chunk_sites;
            if (seed_tuning_smem(sa, c) <= limit) {
                out = c;
                return true;
            }
        }
    }
    return false;
}

// The tolerance a family's index is built with: the prefiltered form always
// uses tolerance-1 regions.
static int index_tolerance(const bgo_tuning &t) { return t.prefilter ? 1 : t.tolerance; }

static int seed_prepare(bgo_engine *engine, bgo_plan *pl, int K, cudaStream_t s) {
    const bool split = pl->tuning.split_families && pl->n_families > 1;
    std::vector<int> tols((size_t)pl->n_families, index_tolerance(pl->tuning));
    if (split)
        for (int f = 0; f < pl->n_families; ++f)
            tols[(size_t)f] = index_tolerance(family_tuning(pl, f));
    // split launches: a family whose index does not fit in any form compares
    // every guide on its own
    auto applies = [&]() -> int {
        if (!pl->seed_ok) return 0;
        if (split) return 1;
        if (pl->tuning.prefilter) return 1;  // the index stays in global memory
        for (int v : tols)
            if (v != tols[0]) return 0;  // one launch needs one tolerance
        bgo_tuning fit;
        return fitted_seed_tuning(pl->seed, pl->tuning, fit) ? 1 : 0;
    };
    if (pl->seed_k == K && pl->seed_tols == tols) return applies();
    if (pl->d_seed || pl->d_seed_fam) {
        BGO_CUDA(cudaEventSynchronize(pl->done));  // launches that read the old index
        BGO_CUDA(pool_free(pl->device, pl->d_seed));
        BGO_CUDA(pool_free(pl->device, pl->d_seed_fam));
        BGO_CUDA(pool_free(pl->device, pl->d_seed_sizes));
        pl->d_seed = nullptr;
        pl->d_seed_fam = nullptr;
        pl->d_seed_sizes = nullptr;
        pl->index_gen++;
    }
    pl->seed_fam.clear();
    pl->seed_k = K;
    pl->seed_tols = tols;
    pl->seed_ok = 0;
    std::vector<SeedFam> sf;
    std::vector<uint32_t> offs;
    std::vector<uint2> ents;
    std::vector<uint16_t> eidx;
    if (!build_seed_index(pl->h_fams, pl->n_families, pl->h_guides, K, tols, sf, offs, ents, eidx))
        return 0;
    const size_t b_f = sizeof(SeedFam) * sf.size();
    const size_t b_e = sizeof(uint2) * ents.size();
    const size_t b_o = sizeof(uint32_t) * offs.size();
    const size_t b_i = sizeof(uint16_t) * eidx.size();
    const size_t o_e = (b_f + 255) / 256 * 256, o_o = o_e + (b_e + 255) / 256 * 256;
    const size_t o_i = o_o + (b_o + 255) / 256 * 256;
    SeedArgs sa{};
    sa.n_fams = (int32_t)sf.size();
    sa.n_guides = pl->n_active;
    sa.n_offsets = (int32_t)offs.size();
    sa.n_lists = (int32_t)ents.size();
    BGO_CUDA(pool_alloc(pl->device, (void **)&pl->d_seed, o_i + b_i + 16));
    BGO_CUDA(cudaMemcpyAsync(pl->d_seed, sf.data(), b_f, cudaMemcpyHostToDevice, s));
    if (b_e) {
        BGO_CUDA(cudaMemcpyAsync(pl->d_seed + o_e, ents.data(), b_e, cudaMemcpyHostToDevice, s));
        BGO_CUDA(cudaMemcpyAsync(pl->d_seed + o_i, eidx.data(), b_i, cudaMemcpyHostToDevice, s));
    }
    BGO_CUDA(cudaMemcpyAsync(pl->d_seed + o_o, offs.data(), b_o, cudaMemcpyHostToDevice, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->h2d_bytes += (int64_t)(b_f + b_e + b_i + b_o);
    sa.fams = reinterpret_cast<const SeedFam *>(pl->d_seed);
    sa.entries = reinterpret_cast<const uint2 *>(pl->d_seed + o_e);
    sa.offsets = reinterpret_cast<const uint32_t *>(pl->d_seed + o_o);
    sa.entry_idx = reinterpret_cast<const uint16_t *>(pl->d_seed + o_i);
    pl->seed = sa;
    // per-family views of the same index: family f's SeedFam rebased to its
    // own lists and bucket tables
    std::vector<SeedFam> rebased(sf);
    std::vector<SeedArgs> views(sf.size());
    pl->seed_sizes.assign(sf.size(), make_uint2(0, 0));
    pl->seed_maxcnt.assign(sf.size(), 0);
    pl->seed_maxreg.assign(sf.size(), 0);
    for (size_t f = 0; f < sf.size(); ++f) {
        const uint32_t off0 = sf[f].seg[0].off;
        const uint32_t off_end = f + 1 < sf.size() ? sf[f + 1].seg[0].off : (uint32_t)offs.size();
        const uint32_t list_end = f + 1 < sf.size() ? sf[f + 1].list_off : (uint32_t)ents.size();
        pl->seed_sizes[f] = make_uint2(off_end - off0, list_end - sf[f].list_off);
        for (uint32_t i = off0; i < off_end; ++i)
            pl->seed_maxcnt[f] = std::max(pl->seed_maxcnt[f], offs[i] >> 16);
        // the longest region list of the family (descriptor starts index into it)
        for (int j = 0; j < sf[f].nseg; ++j) {
            const uint32_t end = j + 1 < sf[f].nseg ? sf[f].seg[j + 1].ent
                                                    : list_end - sf[f].list_off;
            pl->seed_maxreg[f] = std::max(pl->seed_maxreg[f], end - sf[f].seg[j].ent);
        }
        rebased[f].list_off = 0;
        for (int j = 0; j < sf[f].nseg; ++j) rebased[f].seg[j].off = sf[f].seg[j].off - off0;
        SeedArgs v{};
        v.n_fams = 1;
        v.n_guides = pl->h_fams[f].gend - pl->h_fams[f].gbeg;
        v.n_offsets = (int32_t)(off_end - off0);
        v.n_lists = (int32_t)(list_end - sf[f].list_off);
        v.entries = sa.entries + sf[f].list_off;
        v.entry_idx = sa.entry_idx + sf[f].list_off;
        v.offsets = sa.offsets + off0;
        views[f] = v;
    }
    BGO_CUDA(pool_alloc(pl->device, (void **)&pl->d_seed_fam,
                        sizeof(SeedFam) * (rebased.size() + 1)));
    BGO_CUDA(cudaMemcpyAsync(pl->d_seed_fam, rebased.data(), sizeof(SeedFam) * rebased.size(),
                             cudaMemcpyHostToDevice, s));
    BGO_CUDA(pool_alloc(pl->device, (void **)&pl->d_seed_sizes,
                        sizeof(uint2) * (pl->seed_sizes.size() + 1)));
    BGO_CUDA(cudaMemcpyAsync(pl->d_seed_sizes, pl->seed_sizes.data(),
                             sizeof(uint2) * pl->seed_sizes.size(), cudaMemcpyHostToDevice, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->h2d_bytes += (int64_t)((sizeof(SeedFam) + sizeof(uint2)) * rebased.size());
    for (size_t f = 0; f < views.size(); ++f)
        views[f].fams = reinterpret_cast<const SeedFam *>(pl->d_seed_fam) + f;
    pl->seed_fam = views;
    pl->seed_ok = 1;
    return applies();
}

// Builds (once per max_mismatches) and uploads the plan's prefilter tables.
static int filter_prepare(bgo_engine *engine, bgo_plan *pl, int K, cudaStream_t s) {
    if (pl->filter_k == K && pl->d_filter) return BGO_OK;
    if (pl->d_filter) {
        BGO_CUDA(cudaEventSynchronize(pl->done));  // launches that read the old tables
        BGO_CUDA(pool_free(pl->device, pl->d_filter));
        pl->d_filter = nullptr;
        pl->index_gen++;
    }
    std::vector<uint8_t> tabs;
    uint32_t tab = 0;
    if (!build_filter_tables(pl->h_fams, pl->n_families, pl->h_guides, K, tabs, tab)) {
        set_error("prefiltered segment index: max_mismatches outside 0..7");
        return BGO_ERR_ARG;
    }
    BGO_CUDA(pool_alloc(pl->device, (void **)&pl->d_filter, tabs.size() + 16));
    BGO_CUDA(cudaMemcpyAsync(pl->d_filter, tabs.data(), tabs.size(), cudaMemcpyHostToDevice, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->h2d_bytes += (int64_t)tabs.size();
    pl->filter_k = K;
    pl->filter_tab = tab;
    return BGO_OK;
}

// Builds (once per (max_mismatches, group size)) and uploads the plan's
// segment-mask index.  Returns 1 when it applies, 0 when the scan must compare
// every guide (mode 1), or a negative BGO_ERR_*.
static int mask_prepare(bgo_engine *engine, bgo_plan *pl, int K, cudaStream_t s) {
    const int group = pl->tuning.group_guides ? pl->tuning.group_guides : kMaskGroupMax;
    const int chunk = pl->tuning.chunk_sites ? pl->tuning.chunk_sites : 2048;
    if (pl->mask_k == K && pl->mask_group == group) {
        pl->mask.chunk_sites = chunk;
        if (pl->mask_ok && mask_smem_bytes(pl->mask) > 220 * 1024) return 0;
        return pl->mask_ok;
    }
    if (pl->d_mask) {
        BGO_CUDA(cudaEventSynchronize(pl->done));  // launches that read the old index
        BGO_CUDA(pool_free(pl->device, pl->d_mask));
        pl->d_mask = nullptr;
        pl->index_gen++;
    }
    pl->mask_k = K;
    pl->mask_group = group;
    pl->mask_ok = 0;
    std::vector<MaskFam> mf;
    std::vector<MaskGroup> groups;
    std::vector<uint32_t> table;
    std::vector<uint2> gd;
    if (!build_mask_index(pl->h_fams, pl->n_families, pl->h_guides, K, group, mf, groups, table,
                          gd))
        return 0;
    const size_t b_f = sizeof(MaskFam) * mf.size(), b_g = sizeof(MaskGroup) * groups.size();
    const size_t b_t = sizeof(uint32_t) * table.size(), b_d = sizeof(uint2) * gd.size();
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t o_g = al(b_f), o_t = o_g + al(b_g), o_d = o_t + al(b_t);
    MaskArgs ma{};
    ma.n_fams = (int32_t)mf.size();
    ma.n_groups = (int32_t)groups.size();
    ma.table_words = (int32_t)table.size();
    ma.n_guides = (int32_t)gd.size();
    ma.chunk_sites = chunk;
    // the whole index must fit in shared memory beside the warps' chunk slices
    if (mask_smem_bytes(ma) > 220 * 1024) return 0;
    BGO_CUDA(pool_alloc(pl->device, (void **)&pl->d_mask, o_d + b_d + 16));
    BGO_CUDA(cudaMemcpyAsync(pl->d_mask, mf.data(), b_f, cudaMemcpyHostToDevice, s));
    if (b_g) BGO_CUDA(cudaMemcpyAsync(pl->d_mask + o_g, groups.data(), b_g, cudaMemcpyHostToDevice, s));
    if (b_t) BGO_CUDA(cudaMemcpyAsync(pl->d_mask + o_t, table.data(), b_t, cudaMemcpyHostToDevice, s));
    if (b_d) BGO_CUDA(cudaMemcpyAsync(pl->d_mask + o_d, gd.data(), b_d, cudaMemcpyHostToDevice, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->h2d_bytes += (int64_t)(b_f + b_g + b_t + b_d);
    ma.fams = reinterpret_cast<const MaskFam *>(pl->d_mask);
    ma.groups = reinterpret_cast<const MaskGroup *>(pl->d_mask + o_g);
    ma.table = reinterpret_cast<const uint32_t *>(pl->d_mask + o_t);
    ma.guides = reinterpret_cast<const uint2 *>(pl->d_mask + o_d);
    pl->mask = ma;
    pl->mask_ok = 1;
    return 1;
}

static int scan_launch(bgo_engine *engine, const bgo_plan *plan, const bgo_genome *const *strands,
                       const int32_t *n_encoded, int32_t n_strands, int32_t max_mismatches,
                       int32_t mode, void *stream) {
    if (!engine || !plan || !strands || !n_encoded || n_strands < 1 || n_strands > 2 ||
        mode < 0 || mode > 3) {
        set_error("bgo_scan_launch: invalid argument");
        return BGO_ERR_ARG;
    }
    for (int i = 0; i < n_strands; ++i) {
        if (!strands[i] || strands[i]->device != engine->device ||
            (n_encoded[i] < 0 || n_encoded[i] > 3)) {
            set_error("bgo_scan_launch: bad strand or n_encoded");
            return BGO_ERR_ARG;
        }
    }
    if (plan->device != engine->device) {
        set_error("bgo_scan_launch: plan and engine on different devices");
        return BGO_ERR_ARG;
    }
    BGO_CUDA(cudaSetDevice(engine->device));
    cudaStream_t s = (cudaStream_t)stream;
    // granules of each strand (kDropGranule positions), for the bitmap of
    // dropped keys
    int64_t gran[2] = {0, 0};
    for (int i = 0; i < n_strands; ++i)
        gran[i] = std::max<int64_t>(0, ceil_div(strands[i]->total_bp - kSiteSpan, kDropGranule));
    const int64_t drop_words = (gran[0] + gran[1]) / 32 + 1;
    if (!engine->rescan) {
        BGO_CUDA(cudaMemsetAsync(engine->d_counter, 0, kEngineCounters * sizeof(unsigned long long), s));
        if (engine->drop_words < drop_words) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            BGO_CUDA(cudaStreamIsCapturing(s, &cs));
            if (cs != cudaStreamCaptureStatusNone) {
                set_error("bgo_scan_launch: the dropped-key bitmap must grow outside a capture");
                return BGO_ERR_STATE;
            }
            if (engine->d_drop) {
                BGO_CUDA(cudaEventSynchronize(engine->keys_done));
                BGO_CUDA(pool_free(engine->device, engine->d_drop));
                engine->d_drop = nullptr;
            }
            BGO_CUDA(pool_alloc(engine->device, (void **)&engine->d_drop,
                                sizeof(uint32_t) * (size_t)drop_words));
            engine->drop_words = drop_words;
        }
        BGO_CUDA(cudaMemsetAsync(engine->d_drop, 0, sizeof(uint32_t) * (size_t)drop_words, s));
        engine->last_listable = 1;
    } else {
        // a rescan continues the counts; only the error word starts at zero
        BGO_CUDA(cudaMemsetAsync(engine->d_counter + 2, 0, sizeof(unsigned long long), s));
    }
    engine->launched = 1;
    if (plan->n_families == 0) return BGO_OK;
    ScanParams p{};
    p.drop_bits = engine->d_drop;
    p.drop_base1 = gran[0];
    p.max_mm = max_mismatches;
    p.fams = plan->d_fams;
    p.guides = plan->d_guides;
    p.keys = engine->d_keys;
    p.cap = engine->cap;
    p.counter = engine->d_counter;
    const int64_t max_grid = (int64_t)engine->sm_count * blocks_per_sm();
    if (mode == 0 || mode == 1 || mode == 3) engine->last_listable = 0;
    if (mode == 0) {
        for (int i = 0; i < n_strands; ++i) {
            fill_strand(p.strand[0], strands[i], n_encoded[i], i);
            p.n_strands = 1;
            p.tiles_total = p.strand[0].n_tiles;
            if (p.tiles_total == 0) continue;
            const int64_t grid = std::min<int64_t>(p.tiles_total, max_grid);
            for (int f = 0; f < plan->n_families; ++f) {
                p.fam_begin = f;
                p.fam_end = f + 1;
                scan_kernel<<<(unsigned)grid, kTileThreads, 0, s>>>(p);
                BGO_CUDA(cudaGetLastError());
                engine->launches++;
            }
        }
    }
    bgo_plan *mpl = const_cast<bgo_plan *>(plan);
    const int seeded = mode == 2 ? seed_prepare(engine, mpl, max_mismatches, s) : 0;
    if (seeded < 0) return seeded;
    const int masked = mode == 3 ? mask_prepare(engine, mpl, max_mismatches, s) : 0;
    if (masked < 0) return masked;
    if (mode == 0) {
        // launched above
    } else if (masked == 1) {
        const int chunk = plan->mask.chunk_sites;
        for (int i = 0; i < n_strands; ++i) {
            fill_strand(p.strand[i], strands[i], n_encoded[i], i);
            p.strand[i].n_tiles = seed_tiles_for(strands[i]->total_bp, chunk);
        }
        p.n_strands = n_strands;
        p.tiles_total = p.strand[0].n_tiles + (n_strands > 1 ? p.strand[1].n_tiles : 0);
        if (p.tiles_total == 0) return BGO_OK;
        p.fam_begin = 0;
        p.fam_end = plan->n_families;
        const int rc = launch_mask_kernel(p, plan->mask, engine->sm_count, plan->tuning.ctas_per_sm, s);
        if (rc != BGO_OK) return rc;
        engine->launches++;
    } else if (seeded == 1) {
        // one launch over all families, or one per family with its own form
        auto seed_launch = [&](int fb, int fe, const SeedArgs &sa, const bgo_tuning &t) -> int {
            const int chunk = t.chunk_sites ? t.chunk_sites : 2048;
            const int minb = t.min_blocks ? t.min_blocks : 3;
            ScanParams q = p;
            for (int i = 0; i < n_strands; ++i) {
                fill_strand(q.strand[i], strands[i], n_encoded[i], i);
                q.strand[i].n_tiles = seed_tiles_for(strands[i]->total_bp, chunk);
            }
            q.n_strands = n_strands;
            q.tiles_total = q.strand[0].n_tiles + (n_strands > 1 ? q.strand[1].n_tiles : 0);
            if (q.tiles_total == 0) return BGO_OK;
            if (engine->rescan) {
                const int li = chunk == 1024 ? 0 : 1;
                q.chunk_list = engine->rescan_list[li];
                q.n_list = engine->rescan_n[li];
                if (q.n_list == 0) return BGO_OK;
            }
            q.fam_begin = fb;
            q.fam_end = fe;
            const int rc = launch_seed_kernel(q, sa, engine->sm_count, chunk, minb, t.tolerance,
                                              t.inline_entries, t.range_walk, t.ctas_per_sm, s);
            if (rc == BGO_OK) engine->launches++;
            return rc;
        };
        // prefiltered form over families [fb, fe): one persistent launch whose
        // warps claim chunks family by family
        auto filter_launch = [&](int fb, int fe, const SeedArgs &sa, const bgo_tuning &t) -> int {
            const int chunk = t.chunk_sites ? t.chunk_sites : 2048;
            int rc = filter_prepare(engine, mpl, max_mismatches, s);
            if (rc != BGO_OK) return rc;
            for (int g0 = fb; g0 < fe; g0 += kWorkCap) {
                const int g1 = std::min(fe, g0 + kWorkCap);
                ScanParams q = p;
                for (int i = 0; i < n_strands; ++i) {
                    fill_strand(q.strand[i], strands[i], n_encoded[i], i);
                    q.strand[i].n_tiles = seed_tiles_for(strands[i]->total_bp, chunk);
                }
                q.n_strands = n_strands;
                q.tiles_total = q.strand[0].n_tiles + (n_strands > 1 ? q.strand[1].n_tiles : 0);
                if (q.tiles_total == 0) return BGO_OK;
                if (q.tiles_total >= (1ll << 31)) {
                    set_error("prefiltered segment index: more than 2^31 chunks");
                    return BGO_ERR_ARG;
                }
                if (engine->rescan) {
                    const int li = chunk == 4096 ? 2 : 1;
                    q.chunk_list = engine->rescan_list[li];
                    q.n_list = engine->rescan_n[li];
                    if (q.n_list == 0) return BGO_OK;
                }
                q.fam_begin = g0;
                q.fam_end = g1;
                FilterArgs fa{};
                fa.fams = sa.fams + (g0 - fb);
                fa.offsets = sa.offsets;
                fa.entries = sa.entries;
                fa.entry_idx = sa.entry_idx;
                fa.tables = plan->d_filter + (size_t)g0 * plan->filter_tab;
                fa.work = engine->d_work;
                fa.err = reinterpret_cast<int *>(engine->d_counter + 2);
                fa.fam_sizes = plan->d_seed_sizes + g0;
                fa.tab_bytes = (int32_t)plan->filter_tab;
                fa.n_fams = g1 - g0;
                // the survivor index goes to shared memory when the largest
                // family's index fits beside the tables and slices and its
                // descriptors fit 16 bits (entry starts < 4096, counts < 16)
                size_t need = 0;
                bool fits16 = true;
                for (int g = g0; g < g1; ++g) {
                    const uint2 sz = plan->seed_sizes[(size_t)g];
                    const size_t G = (size_t)(plan->h_fams[g].gend - plan->h_fams[g].gbeg);
                    fits16 = fits16 && plan->seed_maxreg[(size_t)g] <= 4096 &&
                             plan->seed_maxcnt[(size_t)g] <= 15;
                    need = std::max(need, ((size_t)sz.x * 2 + (size_t)sz.y * 2 + 15) / 16 * 16 +
                                              (G * 8 + 15) / 16 * 16);
                }
                fa.idx_smem_bytes =
                    fits16 && filter_smem_fixed_bytes(max_mismatches, chunk) + need <=
                                  filter_smem_limit()
                        ? (int32_t)need
                        : 0;
                BGO_CUDA(cudaMemsetAsync(engine->d_work, 0, sizeof(uint32_t) * (size_t)(g1 - g0), s));
                rc = launch_filter_kernel(q, fa, engine->sm_count, chunk, s);
                if (rc != BGO_OK) return rc;
                engine->launches++;
            }
            return BGO_OK;
        };
        auto every_guide_launch = [&](int fb, int fe) -> int {
            engine->last_listable = 0;
            ScanParams q = p;
            for (int i = 0; i < n_strands; ++i) fill_strand(q.strand[i], strands[i], n_encoded[i], i);
            q.n_strands = n_strands;
            q.tiles_total = q.strand[0].n_tiles + (n_strands > 1 ? q.strand[1].n_tiles : 0);
            if (q.tiles_total == 0) return BGO_OK;
            q.fam_begin = fb;
            q.fam_end = fe;
            const int64_t grid = std::min<int64_t>(q.tiles_total, max_grid);
            scan_kernel<<<(unsigned)grid, kTileThreads, 0, s>>>(q);
            BGO_CUDA(cudaGetLastError());
            engine->launches++;
            return BGO_OK;
        };
        if (plan->tuning.split_families && plan->n_families > 1) {
            for (int f = 0; f < plan->n_families; ++f) {
                const SeedArgs &sa = plan->seed_fam[(size_t)f];
                const bgo_tuning &ft = family_tuning(plan, f);
                bgo_tuning fit;
                const int rc = ft.family_form == 0 && ft.prefilter
                                   ? filter_launch(f, f + 1, sa, ft)
                               : ft.family_form == 0 && fitted_seed_tuning(sa, ft, fit)
                                   ? seed_launch(f, f + 1, sa, fit)
                                   : every_guide_launch(f, f + 1);
                if (rc != BGO_OK) return rc;
            }
        } else if (plan->tuning.prefilter) {
            const int rc = filter_launch(0, plan->n_families, plan->seed, plan->tuning);
            if (rc != BGO_OK) return rc;
        } else {
            bgo_tuning fit;
            fitted_seed_tuning(plan->seed, plan->tuning, fit);  // applies() checked it fits
            const int rc = seed_launch(0, plan->n_families, plan->seed, fit);
            if (rc != BGO_OK) return rc;
        }
    } else {
        engine->last_listable = 0;
        for (int i = 0; i < n_strands; ++i) fill_strand(p.strand[i], strands[i], n_encoded[i], i);
        p.n_strands = n_strands;
        p.tiles_total = p.strand[0].n_tiles + (n_strands > 1 ? p.strand[1].n_tiles : 0);
        if (p.tiles_total == 0) return BGO_OK;
        p.fam_begin = 0;
        p.fam_end = plan->n_families;
        const int64_t grid = std::min<int64_t>(p.tiles_total, max_grid);
        scan_kernel<<<(unsigned)grid, kTileThreads, 0, s>>>(p);
        BGO_CUDA(cudaGetLastError());
        engine->launches++;
    }
    return BGO_OK;
}

extern "C" int bgo_scan_launch(bgo_engine *engine, const bgo_plan *plan,
                               const bgo_genome *const *strands, const int32_t *n_encoded,
                               int32_t n_strands, int32_t max_mismatches, int32_t mode,
                               void *stream) {
    const int rc = scan_launch(engine, plan, strands, n_encoded, n_strands, max_mismatches, mode,
                               stream);
    if (rc != BGO_OK) return rc;
    // mark the plan's last use (not while a graph is being captured: the
    // replay records it instead)
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    BGO_CUDA(cudaStreamIsCapturing(s, &cap));
    if (cap == cudaStreamCaptureStatusNone) {
        BGO_CUDA(cudaEventRecord(plan->done, s));
        BGO_CUDA(cudaEventRecord(engine->keys_done, s));
    }
    return BGO_OK;
}

// Keys of granules whose keys were partly dropped are removed (their
// granules are scanned again); the others are appended to dst.
__global__ void drop_compact_kernel(const uint64_t *__restrict__ src, int64_t n,
                                    const uint32_t *__restrict__ bits, int64_t base1,
                                    uint64_t *__restrict__ dst, unsigned long long *counter) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        const int64_t i = i0 + threadIdx.x;
        bool keep = false;
        uint64_t k = 0;
        if (i < n) {
            k = src[i];
            const int64_t pos = (int64_t)((k >> 6) & 0xFFFFFFFFull);
            const int64_t g = (((k >> 38) & 1ull) ? base1 : 0) + pos / kDropGranule;
            keep = !((bits[g >> 5] >> (g & 31)) & 1u);
        }
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, keep);
        unsigned long long at = 0;
        if (lane == 0 && bal) at = atomicAdd(counter, (unsigned long long)__popc(bal));
        at = __shfl_sync(0xFFFFFFFFu, at, 0);
        if (keep) dst[at + __popc(bal & ((1u << lane) - 1u))] = k;
    }
}

extern "C" int bgo_scan_complete(bgo_engine *engine, const bgo_plan *plan,
                                 const bgo_genome *const *strands, const int32_t *n_encoded,
                                 int32_t n_strands, int32_t max_mismatches, int32_t mode,
                                 void *stream, int64_t *n_hits) {
    if (!engine || !plan || !strands || !n_encoded || !n_hits || n_strands < 1 || n_strands > 2) {
        set_error("bgo_scan_complete: invalid argument");
        return BGO_ERR_ARG;
    }
    if (!engine->launched) {
        set_error("bgo_scan_complete: no launch to complete");
        return BGO_ERR_STATE;
    }
    BGO_CUDA(cudaSetDevice(engine->device));
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long cnt[3] = {0, 0, 0};
    BGO_CUDA(cudaMemcpyAsync(cnt, engine->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->d2h_bytes += (int64_t)sizeof(cnt);
    if (cnt[2] & 1u) {
        set_error("bgo_scan_complete: a chunk copy of the last scan did not complete in time");
        return BGO_ERR_TIMEOUT;
    }
    const int64_t n = (int64_t)cnt[0];
    *n_hits = n;
    if (n <= engine->cap) return BGO_OK;
    if (!engine->last_listable) {
        // a form that scans tiles without a chunk list: grow and scan again
        int rc = bgo_engine_reserve(engine, n);
        if (rc == BGO_OK)
            rc = bgo_scan_launch(engine, plan, strands, n_encoded, n_strands, max_mismatches, mode,
                                 stream);
        if (rc != BGO_OK) return rc;
        BGO_CUDA(cudaMemcpyAsync(cnt, engine->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, s));
        BGO_CUDA(cudaStreamSynchronize(s));
        *n_hits = (int64_t)cnt[0];
        return BGO_OK;
    }
    // granules with dropped keys, and the chunks of each chunk length that
    // cover them
    int64_t gran[2] = {0, 0};
    for (int i = 0; i < n_strands; ++i)
        gran[i] = std::max<int64_t>(0, ceil_div(strands[i]->total_bp - kSiteSpan, kDropGranule));
    const int64_t words = (gran[0] + gran[1]) / 32 + 1;
    std::vector<uint32_t> bits((size_t)words);
    BGO_CUDA(cudaMemcpyAsync(bits.data(), engine->d_drop, sizeof(uint32_t) * (size_t)words,
                             cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->d2h_bytes += (int64_t)(sizeof(uint32_t) * (size_t)words);
    const int lens[3] = {1024, 2048, 4096};
    std::vector<uint32_t> lists[3];
    for (int64_t g = 0; g < gran[0] + gran[1]; ++g) {
        if (!((bits[(size_t)(g >> 5)] >> (g & 31)) & 1u)) continue;
        const int st = g >= gran[0] ? 1 : 0;
        const int64_t lg = g - (st ? gran[0] : 0);
        for (int li = 0; li < 3; ++li) {
            const int per = (int)(kDropGranule / lens[li]);
            const int64_t tiles = seed_tiles_for(strands[st]->total_bp, lens[li]);
            const int64_t base = st ? seed_tiles_for(strands[0]->total_bp, lens[li]) : 0;
            for (int k = 0; k < per; ++k) {
                const int64_t c = lg * per + k;
                if (c < tiles) lists[li].push_back((uint32_t)(base + c));
            }
        }
    }
    size_t list_words = 0;
    for (auto &l : lists) list_words += l.size();
    uint32_t *d_lists = nullptr;
    BGO_CUDA(pool_alloc(engine->device, (void **)&d_lists, sizeof(uint32_t) * (list_words + 1)));
    size_t at = 0;
    for (int li = 0; li < 3; ++li) {
        if (!lists[li].empty())
            BGO_CUDA(cudaMemcpyAsync(d_lists + at, lists[li].data(),
                                     sizeof(uint32_t) * lists[li].size(), cudaMemcpyHostToDevice, s));
        engine->rescan_list[li] = d_lists + at;
        engine->rescan_n[li] = (int64_t)lists[li].size();
        at += lists[li].size();
    }
    engine->h2d_bytes += (int64_t)(sizeof(uint32_t) * list_words);
    // a buffer for every hit; the kept keys of the old one move into it
    uint64_t *keys = nullptr;
    BGO_CUDA(pool_alloc(engine->device, (void **)&keys, sizeof(uint64_t) * (size_t)n));
    BGO_CUDA(cudaMemsetAsync(engine->d_counter, 0, sizeof(unsigned long long), s));
    const int64_t old_n = engine->cap;
    drop_compact_kernel<<<(unsigned)std::min<int64_t>(ceil_div(old_n, 256), 8L * engine->sm_count),
                          256, 0, s>>>(engine->d_keys, old_n, engine->d_drop, gran[0], keys,
                                       engine->d_counter);
    BGO_CUDA(cudaGetLastError());
    BGO_CUDA(pool_free_after(engine->device, engine->d_keys, s));
    engine->d_keys = keys;
    engine->cap = n;
    engine->keys_gen++;
    // scan the listed chunks again, appending to the compacted keys
    engine->rescan = 1;
    int rc = bgo_scan_launch(engine, plan, strands, n_encoded, n_strands, max_mismatches, mode,
                             stream);
    engine->rescan = 0;
    for (int li = 0; li < 3; ++li) {
        engine->rescan_list[li] = nullptr;
        engine->rescan_n[li] = 0;
    }
    cudaError_t fe = pool_free_after(engine->device, d_lists, s);
    if (rc != BGO_OK) return rc;
    BGO_CUDA(fe);
    BGO_CUDA(cudaMemcpyAsync(cnt, engine->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    if (cnt[2] & 1u) {
        set_error("bgo_scan_complete: a chunk copy of the rescan did not complete in time");
        return BGO_ERR_TIMEOUT;
    }
    if ((int64_t)cnt[0] != n) {
        set_error("bgo_scan_complete: the rescan of the dropped granules found " +
                  std::to_string(cnt[0]) + " keys in all, not " + std::to_string(n));
        return BGO_ERR_STATE;
    }
    *n_hits = n;
    return BGO_OK;
}

extern "C" int bgo_scan_time(bgo_engine *engine, const bgo_plan *plan,
                             const bgo_genome *const *strands, const int32_t *n_encoded,
                             int32_t n_strands, int32_t max_mismatches, int32_t mode, int32_t reps,
                             void *stream, double *ms_best) {
    if (!engine || !ms_best || reps < 1) return BGO_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = bgo_scan_launch(engine, plan, strands, n_encoded, n_strands, max_mismatches, mode, s);
    if (rc != BGO_OK) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BGO_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    float best = 1e30f;
    for (int r = 0; r < reps && ce == cudaSuccess && rc == BGO_OK; ++r) {
        ce = cudaEventRecord(e0, s);
        if (ce == cudaSuccess)
            rc = bgo_scan_launch(engine, plan, strands, n_encoded, n_strands, max_mismatches, mode, s);
        if (ce == cudaSuccess && rc == BGO_OK) ce = cudaEventRecord(e1, s);
        if (ce == cudaSuccess && rc == BGO_OK) ce = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (ce == cudaSuccess && rc == BGO_OK) ce = cudaEventElapsedTime(&ms, e0, e1);
        if (ce == cudaSuccess && rc == BGO_OK && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc != BGO_OK) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "bgo_scan_time");
    *ms_best = best;
    return BGO_OK;
}

struct bgo_graph {
    int device;
    bgo_engine *engine;
    cudaGraphExec_t exec;
    int64_t launches_per_replay;
    // what the graph scans, for a re-capture after the hit buffer moved
    const bgo_plan *plan;
    std::vector<const bgo_genome *> strands;
    std::vector<int32_t> n_encoded;
    int32_t max_mismatches, mode;
    uint64_t keys_gen;
    uint64_t plan_gen;  // the plan's index generation the capture used
};

// Captures one bgo_scan_launch on a private stream (nothing runs).
static int capture_scan(bgo_graph *g, cudaGraphExec_t *out) {
    bgo_engine *engine = g->engine;
    cudaStream_t cs = nullptr;
    BGO_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int64_t before = engine->launches;
    int rc = BGO_OK;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        rc = bgo_scan_launch(engine, g->plan, g->strands.data(), g->n_encoded.data(),
                             (int32_t)g->strands.size(), g->max_mismatches, g->mode, cs);
        cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (e2 != cudaSuccess && rc == BGO_OK) e = e2;
    }
    if (rc == BGO_OK && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    g->launches_per_replay = engine->launches - before;
    engine->launches = before;  // the capture itself ran nothing
    if (rc != BGO_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "bgo_graph capture");
    *out = exec;
    return BGO_OK;
}

// One ordinary launch (builds the index the graph scans with, sets kernel
// attributes and validates the arguments outside the capture), then the
// capture.
static int prepare_and_capture(bgo_graph *g, cudaGraphExec_t *out) {
    cudaStream_t cs = nullptr;
    BGO_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = bgo_scan_launch(g->engine, g->plan, g->strands.data(), g->n_encoded.data(),
                             (int32_t)g->strands.size(), g->max_mismatches, g->mode, cs);
    cudaError_t e = rc == BGO_OK ? cudaStreamSynchronize(cs) : cudaSuccess;
    cudaStreamDestroy(cs);
    if (rc != BGO_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "bgo_graph capture");
    g->keys_gen = g->engine->keys_gen;
    g->plan_gen = g->plan->index_gen;
    return capture_scan(g, out);
}

extern "C" int bgo_graph_create(bgo_engine *engine, const bgo_plan *plan,
                                const bgo_genome *const *strands, const int32_t *n_encoded,
                                int32_t n_strands, int32_t max_mismatches, int32_t mode,
                                bgo_graph **out) {
    if (!out) return BGO_ERR_ARG;
    *out = nullptr;
    if (!engine || !plan || !strands || !n_encoded || n_strands < 1 || n_strands > 2)
        return BGO_ERR_ARG;
    BGO_CUDA(cudaSetDevice(engine->device));
    bgo_graph *g = new (std::nothrow) bgo_graph();
    if (!g) return BGO_ERR_OOM;
    g->device = engine->device;
    g->engine = engine;
    g->plan = plan;
    g->strands.assign(strands, strands + n_strands);
    g->n_encoded.assign(n_encoded, n_encoded + n_strands);
    g->max_mismatches = max_mismatches;
    g->mode = mode;
    g->exec = nullptr;
    const int rc = prepare_and_capture(g, &g->exec);
    if (rc != BGO_OK) {
        delete g;
        return rc;
    }
    *out = g;
    return BGO_OK;
}

extern "C" int bgo_graph_launch(bgo_graph *g, void *stream) {
    if (!g) return BGO_ERR_ARG;
    BGO_CUDA(cudaSetDevice(g->device));
    if (g->keys_gen != g->engine->keys_gen || g->plan_gen != g->plan->index_gen) {
        // the hit buffer moved (bgo_engine_reserve) or the plan's index was
        // rebuilt by a launch with another max_mismatches or tolerance: the
        // captured kernels would use freed memory, so capture again
        cudaGraphExec_t exec = nullptr;
        const int rc = prepare_and_capture(g, &exec);
        if (rc != BGO_OK) return rc;
        cudaGraphExecDestroy(g->exec);
        g->exec = exec;
    }
    BGO_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    BGO_CUDA(cudaEventRecord(g->plan->done, (cudaStream_t)stream));
    BGO_CUDA(cudaEventRecord(g->engine->keys_done, (cudaStream_t)stream));
    g->engine->launched = 1;
    g->engine->launches += g->launches_per_replay;
    return BGO_OK;
}

extern "C" int bgo_graph_destroy(bgo_graph *g) {
    if (!g) return BGO_OK;
    cudaSetDevice(g->device);
    cudaGraphExecDestroy(g->exec);
    delete g;
    return BGO_OK;
}

extern "C" int bgo_scan_collect(bgo_engine *engine, uint64_t *keys, int64_t capacity,
                                int64_t *n_hits, void *stream) {
    if (!engine || !n_hits || capacity < 0) return BGO_ERR_ARG;
    if (!engine->launched) {
        set_error("bgo_scan_collect: no launch to collect");
        return BGO_ERR_STATE;
    }
    BGO_CUDA(cudaSetDevice(engine->device));
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long cnt[3] = {0, 0, 0};
    BGO_CUDA(cudaMemcpyAsync(cnt, engine->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->d2h_bytes += (int64_t)sizeof(cnt);
    if (cnt[2] & 1u) {
        set_error("bgo_scan_collect: a chunk copy of the last scan did not complete in time");
        return BGO_ERR_TIMEOUT;
    }
    const unsigned long long n = cnt[0];
    *n_hits = (int64_t)n;
    if (keys && (int64_t)n <= capacity && (int64_t)n <= engine->cap && n > 0) {
        BGO_CUDA(cudaMemcpyAsync(keys, engine->d_keys, (size_t)n * sizeof(uint64_t),
                                 cudaMemcpyDeviceToHost, s));
        BGO_CUDA(cudaStreamSynchronize(s));
        engine->d2h_bytes += (int64_t)(n * sizeof(uint64_t));
        std::sort(keys, keys + n);
    }
    return BGO_OK;
}

extern "C" int bgo_scan_stats(bgo_engine *engine, int64_t *pairs_evaluated, void *stream) {
    if (!engine || !pairs_evaluated) return BGO_ERR_ARG;
    if (!engine->launched) {
        set_error("bgo_scan_stats: no launch");
        return BGO_ERR_STATE;
    }
    BGO_CUDA(cudaSetDevice(engine->device));
    unsigned long long v = 0;
    cudaStream_t s = (cudaStream_t)stream;
    BGO_CUDA(cudaMemcpyAsync(&v, engine->d_counter + 1, sizeof(v), cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    *pairs_evaluated = (int64_t)v;
    return BGO_OK;
}

// ----------------------------------------------------------------------------
// search_genome_cuda drop-in
// ----------------------------------------------------------------------------
extern "C" int bgo_search_genome(bgo_engine *engine, const bgo_genome *strand,
                                 const uint64_t *guide_encoded, const uint8_t *pam_masks,
                                 const uint8_t *pam_lens, const uint8_t *pam_3prime,
                                 int32_t n_guides, int32_t max_mismatches, int32_t n_encoded,
                                 int64_t results_per_guide, int64_t *hit_counts,
                                 int64_t *hit_positions, int8_t *hit_mismatches, void *stream) {
    if (!engine || !strand || n_guides < 0 || results_per_guide < 0 ||
        (n_guides > 0 && !hit_counts) ||
        (results_per_guide > 0 && n_guides > 0 && (!hit_positions || !hit_mismatches))) {
        set_error("bgo_search_genome: invalid argument");
        return BGO_ERR_ARG;
    }
    bgo_plan *plan = nullptr;
    int rc = bgo_plan_create(engine, guide_encoded, pam_masks, pam_lens, pam_3prime, n_guides,
                             stream, &plan);
    if (rc != BGO_OK) return rc;
    std::vector<uint64_t> keys;
    int64_t n = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
        rc = bgo_scan_launch(engine, plan, &strand, &n_encoded, 1, max_mismatches, 0, stream);
        if (rc == BGO_OK) rc = bgo_scan_collect(engine, nullptr, 0, &n, stream);
        if (rc != BGO_OK) break;
        if (n <= engine->cap) break;
        rc = bgo_engine_reserve(engine, n);
        if (rc != BGO_OK) break;
    }
    if (rc == BGO_OK) {
        try {
            keys.resize((size_t)n);
        } catch (...) {
            rc = BGO_ERR_OOM;
        }
    }
    if (rc == BGO_OK && n > 0) rc = bgo_scan_collect(engine, keys.data(), n, &n, stream);
    bgo_plan_destroy(plan);
    if (rc != BGO_OK) return rc;
    for (int32_t g = 0; g < n_guides; ++g) hit_counts[g] = 0;
    for (int64_t i = 0; i < n; ++i) {
        const uint64_t k = keys[(size_t)i];
        const int64_t g = (int64_t)(k >> 39);
        const int64_t c = hit_counts[g]++;
        if (c < results_per_guide) {
            hit_positions[g * results_per_guide + c] = (int64_t)((k >> 6) & 0xFFFFFFFFull);
            hit_mismatches[g * results_per_guide + c] = (int8_t)(k & 63u);
        }
    }
    return BGO_OK;
}
