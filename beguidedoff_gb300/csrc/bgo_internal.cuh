// Internal declarations shared by the bgo translation units.
//
// Device genome layout (one strand array): three bit planes, 32 positions per
// uint32 word, bit j of word w = position 32*w + j:
//   H  - high bit of the 2-bit base (A0 C1 G2 T3 -> 0 0 1 1)
//   L  - low bit of the 2-bit base  (            -> 0 1 0 1)
//   N  - 1 where the N mask marks the position
// Each plane holds `plane_words` words, zero beyond total_bp, padded so that a
// tile load of kTileWords words starting at any tile never leaves the buffer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/bgo.h"

namespace bgo {

constexpr int kMaxPam = BGO_MAX_PAM_LEN;
constexpr int kGuideLen = BGO_GUIDE_LEN;
// The reference scans positions [0, total_bp - 26) for every PAM length
// (beguidedoff/cuda_search.py:211).
constexpr int kSiteSpan = 26;

// Tile geometry of the scan kernels: one thread per 32-position word.
constexpr int kTileThreads = 256;
constexpr int kTileSites = kTileThreads * 32;     // 8192 positions
constexpr int kTileWords = kTileSites / 32 + 4;   // + halo for window and PAM

struct FamilyDesc {
    uint8_t allowed[kMaxPam];  // IUPAC allowed-set nibble per PAM position
    uint8_t plen;              // 1..6
    uint8_t three_prime;       // 1: PAM after the guide
    int32_t gbeg, gend;        // rows [gbeg, gend) of the family-sorted guide table
};

struct GuideRec {
    uint32_t h;    // bit i = high bit of guide base i (20 bits)
    uint32_t l;    // bit i = low bit of guide base i
    uint32_t row;  // row index in the caller's guide table
    uint32_t pad;
};

struct StrandDesc {
    const uint32_t *H, *L, *N;
    // N summary: bit g set iff N-plane words [32g, 32g + 32) hold an N;
    // nullptr for a strand without an N mask
    const uint32_t *nsum;
    int64_t total_bp;
    int64_t n_tiles;
    int32_t has_n;
    int32_t n_encoded;
    int32_t slot;
    int32_t pad;
};

// Keys that do not fit the hit buffer mark their granule (kDropGranule
// positions of one strand) in a bitmap, so that an overflowing scan rescans
// only the granules whose keys were dropped.
constexpr int64_t kDropGranule = 4096;

struct ScanParams {
    StrandDesc strand[2];
    int32_t n_strands;
    int32_t fam_begin, fam_end;
    int32_t max_mm;
    const FamilyDesc *fams;
    const GuideRec *guides;
    uint64_t *keys;
    int64_t cap;
    unsigned long long *counter;
    int64_t tiles_total;
    // granule bitmap of dropped keys (NULL: none); granules of strand slot 1
    // start at drop_base1
    uint32_t *drop_bits;
    int64_t drop_base1;
    // chunks to scan (NULL: all tiles_total); the chunk-indexed kernels
    // (segment index, prefiltered) take this list on a rescan
    const uint32_t *chunk_list;
    int64_t n_list;
};

// Segment-indexed scan (scan mode 2): independent warps, each streaming chunks
// of kSeedChunkSites positions; max_mismatches up to kSeedMaxK.
constexpr int kSeedThreads = 256;
constexpr int kSeedChunkSites = 2048;
constexpr int kSeedMaxK = 7;
constexpr int kMaxSeg = 20;
constexpr int kMaxKeyLen = 6;

struct SeedSeg {
    uint8_t start, len, klen, pad;
    uint32_t off;  // first bucket offset of this segment in the offsets table
    uint32_t ent;  // first entry of this segment's list, from the family's list_off
};

struct SeedFam {
    int32_t nseg;
    uint32_t list_off;  // this family's lists: segment j at list_off + j * family size
    // PAM test program: n_tests constrained positions; test t checks the base
    // at shift pam_shift[t] from the site.  pam_code[t]: bit 8 set = generic
    // allowed-set test with nibble bits 0-3; else fixed bits: bit0 high-bit
    // value, bit1 high-bit compared, bit2 low-bit value, bit3 low-bit compared
    uint8_t n_tests;
    uint8_t pam_shift[kMaxPam];
    uint8_t pam_generic;  // bit t: test t is a generic allowed-set test
    uint16_t pam_code[kMaxPam];
    uint32_t pad1;
    // pam_code[t] decoded into whole-word masks (0 or all ones): generic
    // tests the allowed flag of A, C, G, T; fixed tests high-bit value,
    // high-bit compared, low-bit value, low-bit compared
    uint4 pam_mask[kMaxPam];
    SeedSeg seg[kMaxSeg];
};
static_assert(sizeof(SeedFam) % 16 == 0, "SeedFam arrays keep 16-byte alignment");

// Bucket entries: guide planes h, l (20 bits each); entry_idx holds the
// family-local guide index of each entry.
struct SeedArgs {
    const SeedFam *fams;
    const uint32_t *offsets;  // per bucket: entry start | count << 16
    const uint2 *entries;
    const uint16_t *entry_idx;
    int32_t n_fams, n_guides, n_offsets, n_lists;
};

// Prefiltered segment index (scan mode 2 with tuning.prefilter): per PAM
// family one byte per key of each tolerance-1 region (first <= kFilterKeyLen
// bases); the segment index itself stays in global memory.
constexpr int kFilterKeyLen = 7;
constexpr int kFilterColors = 7;

struct FilterArgs {
    const SeedFam *fams;       // the launch's families: fams[f - fam_begin]
    const uint32_t *offsets;   // segment index (tolerance 1) in global memory
    const uint2 *entries;
    const uint16_t *entry_idx;
    const uint8_t *tables;     // per launch family, tab_bytes each
    uint32_t *work;            // per launch family: next chunk to claim
    int *err;                  // bit 0: a chunk copy wait gave up
    const uint2 *fam_sizes;    // per launch family: (descriptors, list entries)
    int32_t tab_bytes;
    int32_t n_fams;
    // bytes of the largest launch family's index in shared memory (16-bit
    // descriptors, entry guide indices, guide planes); 0 = the index is read
    // from global memory
    int32_t idx_smem_bytes;
    int32_t pad;
};

// Segment-mask scan (scan mode 3): the segment index stored as guide bitmasks.
// Each family is cut into groups of at most kMaskGroupMax guides; for group g,
// segment j and key code c the table holds the bitmask of the group's guides
// whose segment-j key equals c, in 1, 2 or 4 words.
constexpr int kMaskThreads = 256;
constexpr int kMaskMaxK = 7;
constexpr int kMaskKeyLen = 4;     // bases per segment key: <= 256 codes
constexpr int kMaskGroupMax = 128;

struct MaskFam {
    uint16_t g0, g1;  // groups [g0, g1)
    uint8_t n_tests;  // PAM test program, as SeedFam
    uint8_t pam_shift[kMaxPam];
    uint8_t pad0;
    uint16_t pam_code[kMaxPam];
    uint32_t pad1[2];
};
static_assert(sizeof(MaskFam) % 16 == 0, "MaskFam arrays keep 16-byte alignment");

struct MaskGroup {
    uint32_t table_off;  // first table word (a multiple of the width)
    uint32_t guide_off;  // first entry of the group in the guide-plane array
    uint32_t gbeg;       // first row of the group in the family-sorted guide table
    uint16_t n;          // guides in the group
    uint8_t words;       // mask width in 32-bit words: 1, 2 or 4
    uint8_t pad;
};
static_assert(sizeof(MaskGroup) == 16, "MaskGroup is one 16-byte load");

struct MaskArgs {
    const MaskFam *fams;
    const MaskGroup *groups;
    const uint32_t *table;
    const uint2 *guides;  // (h, l) 20-bit planes per group entry
    int32_t n_fams, n_groups, table_words, n_guides;
    int32_t chunk_sites;  // positions per warp chunk: 1024 or 2048
    int32_t pad;
};

inline int64_t seed_tiles_for(int64_t total_bp, int chunk_sites = kSeedChunkSites) {
    int64_t valid = total_bp - kSiteSpan;
    return valid > 0 ? (valid + chunk_sites - 1) / chunk_sites : 0;
}

void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

// Plans and their indexes take device memory from one stream-ordered pool per
// device, so creating and destroying them never synchronises the device (a
// cudaFree waits for every stream, e.g. another serving slot's scan).
// pool_alloc returns memory any stream may use at once; pool_free returns
// memory that no queued work uses any more.
cudaError_t pool_alloc(int device, void **p, size_t bytes);
cudaError_t pool_free(int device, void *p);
// frees p once the work queued on `stream` so far is done (no host wait)
cudaError_t pool_free_after(int device, void *p, cudaStream_t stream);
// a disable-timing event of the device's recycled set, and its return
cudaError_t event_take(int device, cudaEvent_t *ev);
void event_give(int device, cudaEvent_t ev);

#define BGO_CUDA(call)                                              \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return ::bgo::cuda_fail(_e, #call);  \
    } while (0)

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Number of tiles covering the scanned positions [0, total_bp - 26).
inline int64_t tiles_for(int64_t total_bp) {
    int64_t valid = total_bp - kSiteSpan;
    return valid > 0 ? ceil_div(valid, kTileSites) : 0;
}

// Plane words needed so every tile load [t*256, t*256 + kTileWords) of the
// plain kernel and every 16-byte-aligned chunk copy of the segment-indexed
// and prefiltered kernels ([c*64, c*64 + 68) words for 2,048-position chunks,
// [c*128, c*128 + 132) for 4,096) is inside the buffer.
// N-plane words per bit of a strand's N summary (1,024 positions)
constexpr int kNSumGroup = 32;
// words of the N summary of a strand with `plane_words` plane words (one
// spare word, so that a reader may always load two consecutive words)
inline int64_t nsum_words_for(int64_t plane_words) {
    return (plane_words + 32 * kNSumGroup - 1) / (32 * kNSumGroup) + 1;
}

inline int64_t plane_words_for(int64_t total_bp) {
    int64_t t = tiles_for(total_bp);
    int64_t need = t * (kTileSites / 32) + kTileWords;
    int64_t valid = total_bp - kSiteSpan;
    int64_t chunks = valid > 0 ? ceil_div(valid, 2048) : 0;
    int64_t need2 = chunks * 64 + 68;
    int64_t chunks4 = valid > 0 ? ceil_div(valid, 4096) : 0;
    need2 = need2 > chunks4 * 128 + 132 ? need2 : chunks4 * 128 + 132;
    int64_t cover = ceil_div(total_bp > 0 ? total_bp : 1, 32) + 4;
    int64_t w = need > cover ? need : cover;
    w = w > need2 ? w : need2;
    return (w + 63) / 64 * 64;
}

}  // namespace bgo

struct bgo_genome {
    int device;
    int64_t total_bp;
    int32_t has_n;
    int64_t plane_words;
    uint32_t *d_planes;  // [3][plane_words]
    uint32_t *d_nsum;    // N summary (StrandDesc::nsum), nsum_words words; null without N
    int64_t nsum_words;
    int64_t bytes;
    unsigned char *d_stage = nullptr;  // packed words + N mask of bgo_genome_upload
    size_t stage_bytes = 0;
};

struct bgo_plan {
    int device;
    int32_t n_guides;        // rows given by the caller
    int32_t n_active;        // rows that can match (PAM length 1..6)
    int32_t n_families;
    bgo::FamilyDesc *d_fams;
    bgo::GuideRec *d_guides;
    bgo::FamilyDesc *h_fams;  // host copy (n_families)
    bgo::GuideRec *h_guides;  // host copy (n_active)
    // segment index for one (max_mismatches, tolerance) pair, built on first use
    int seed_k;               // -1000 = not built
    std::vector<int> seed_tols;  // tolerance per family the index was built with
    int seed_ok;              // 0: the filter does not apply to this K
    unsigned char *d_seed;    // device block: families | offsets | lists
    bgo::SeedArgs seed;
    std::vector<bgo::SeedArgs> seed_fam;  // the same index, one family per launch
    unsigned char *d_seed_fam;            // rebased per-family SeedFam copies
    std::vector<uint2> seed_sizes;        // per family: (descriptors, list entries)
    std::vector<uint32_t> seed_maxcnt;    // per family: largest bucket
    std::vector<uint32_t> seed_maxreg;    // per family: longest region list
    uint2 *d_seed_sizes = nullptr;
    // segment-mask index for one (max_mismatches, group size) pair
    int mask_k;               // -1000 = not built
    int mask_group;           // guides per group it was built with
    int mask_ok;
    unsigned char *d_mask;    // device block: families | groups | table | guides
    bgo::MaskArgs mask;
    bgo_tuning tuning;        // launch parameters chosen by the caller (zeros = defaults)
    std::vector<bgo_tuning> fam_tuning;  // per family (split launches); empty = tuning
    // recorded after the last work that reads the plan's device memory
    // (creation, scans, graph replays); destroy and index rebuilds wait on it
    cudaEvent_t done = nullptr;
    uint64_t index_gen = 0;   // bumped when an index block is replaced
    // prefilter tables (one block of filter_tab bytes per family) for filter_k
    int filter_k = -1000;
    uint32_t filter_tab = 0;
    unsigned char *d_filter = nullptr;
};

namespace bgo {
bool build_seed_index(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                      const std::vector<int> &tols,
                      std::vector<SeedFam> &out_fams, std::vector<uint32_t> &offsets,
                      std::vector<uint2> &entries, std::vector<uint16_t> &entry_idx);
size_t seed_smem_bytes(const SeedArgs &sa, int chunk_sites, int warps, bool walk);
// dynamic shared memory of the segment-index kernel form a tuning selects
size_t seed_tuning_smem(const SeedArgs &sa, const bgo_tuning &t);
int launch_seed_kernel(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                       int min_blocks, int tolerance, int inline_entries, int range_walk,
                       int ctas_per_sm, cudaStream_t s);
void pam_program(const FamilyDesc &F, SeedFam &sf);
bool build_mask_index(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                      int group_max, std::vector<MaskFam> &out_fams,
                      std::vector<MaskGroup> &groups, std::vector<uint32_t> &table,
                      std::vector<uint2> &guides);
size_t mask_smem_bytes(const MaskArgs &ma);
// Prefilter tables of families [0, n_fams) for K mismatches (tab_bytes per
// family); false when K is outside 0..7.
bool build_filter_tables(const FamilyDesc *fams, int n_fams, const GuideRec *recs, int K,
                         std::vector<uint8_t> &tables, uint32_t &tab_bytes);
uint32_t filter_tab_bytes(int K);
// dynamic shared memory of a prefiltered form besides the survivor index
size_t filter_smem_fixed_bytes(int K, int chunk_sites);
// dynamic shared memory a prefiltered launch may take
size_t filter_smem_limit();
int launch_filter_kernel(const ScanParams &p, const FilterArgs &fa, int sm_count, int chunk_sites,
                         cudaStream_t s);
int launch_mask_kernel(const ScanParams &p, const MaskArgs &ma, int sm_count, int ctas_per_sm,
                       cudaStream_t s);
}  // namespace bgo

struct bgo_engine {
    int device;
    uint64_t *d_keys;
    int64_t cap;
    unsigned long long *d_counter;
    int64_t launches;
    int launched;
    int sm_count;
    // epilogue: grow-only scratch and the device copy of the score-rank table
    unsigned char *d_epi = nullptr;
    size_t epi_bytes = 0;
    unsigned char *d_epi_rec = nullptr;   // candidate records, grouped by input row
    size_t epi_rec_bytes = 0;
    unsigned char *d_epi_out = nullptr;   // kept records, dense, for bgo_epilogue_fetch
    size_t epi_out_bytes = 0;
    int64_t epi_out_n = -1;               // records of the last epilogue (-1: none)
    uint32_t *d_rank = nullptr;
    std::vector<uint32_t> h_rank;   // host copy of what d_rank holds
    const uint32_t *rank_src = nullptr;  // caller's table address h_rank was taken from
    // bytes copied host -> device and device -> host by engine calls
    int64_t h2d_bytes = 0, d2h_bytes = 0;
    // bumped whenever d_keys / cap change (captured graphs re-capture then)
    uint64_t keys_gen = 0;
    // per launch family: the prefiltered kernel's next chunk to claim
    uint32_t *d_work = nullptr;
    // granule bitmap of keys dropped by the last scan (grow-only, from the pool)
    uint32_t *d_drop = nullptr;
    int64_t drop_words = 0;
    // 1 while every launch of the last scan takes a chunk list (segment
    // index, prefiltered), so that an overflow rescans dropped granules only
    int last_listable = 0;
    // a rescan in progress: the chunk lists per chunk length (1,024, 2,048,
    // 4,096 positions) on the device, and their lengths
    int rescan = 0;
    const uint32_t *rescan_list[3] = {nullptr, nullptr, nullptr};
    int64_t rescan_n[3] = {0, 0, 0};
    // recorded after the last work that reads or writes d_keys; a resize
    // waits on it (not on the device) before freeing the old buffer
    cudaEvent_t keys_done = nullptr;
};
// counters of d_counter: hits, pairs evaluated, error flags (bit 0: a chunk
// copy wait gave up), spare
constexpr int kEngineCounters = 4;
// families one prefiltered launch covers (its work counters)
constexpr int kWorkCap = 4096;
