// bgo_scan_noalloc: the off-target scan for callers that must not allocate
// device memory.
//
// Who needs it: a host application that embeds this library inside a larger
// GPU program whose own allocator already owns the device memory (a caching
// allocator that reserved the HBM up front, where a raw cudaMalloc would fail
// or fragment the pool), and latency-critical request loops where cudaMalloc /
// cudaFree would synchronise the whole device in the middle of a request.  The
// regular path (bgo_plan_create + bgo_scan_launch + bgo_scan_collect) allocates
// the guide tables per plan and grows the engine's hit buffer on demand; this
// entry point allocates no device memory, and on success no host memory
// either (its host-side family and guide tables are static arrays; a failing
// call records its error message in a host string).
//
// Instead, all the scratch it needs lives in one file-scope static __device__
// array (kNoallocBytes, about 8.1 MB): the hit counter and work counter, the
// PAM-family table, the guide table and a key buffer of kNoallocMaxHits keys.
// The CUDA runtime reserves this array on every GPU that loads this library and
// keeps it until the process exits.  Host code cannot use the array's name as a
// device address (in host code it names a host-side shadow), so the first call
// on each device looks the address up once with cudaGetSymbolAddress while that
// device is current, checks the result and caches it; make that first call
// before any stream capture.  Every later call on the device reuses the same
// array: each call clears the counters it relies on, and two calls whose work
// overlaps on the GPU (different streams) race on the same memory, so callers
// must serialise them.  Host threads are serialised here: a call holds a mutex
// from its checks to its last copy, since the static host tables are shared
// too.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "bgo_internal.cuh"

namespace bgo {

__global__ void scan_kernel(ScanParams p);

constexpr int64_t kNoallocMaxGuides = BGO_NOALLOC_MAX_GUIDES;
constexpr int64_t kNoallocMaxHits = BGO_NOALLOC_MAX_HITS;
constexpr size_t kCountersBytes = 256;
constexpr size_t kFamiliesOff = kCountersBytes;
constexpr size_t kGuidesOff = kFamiliesOff + sizeof(FamilyDesc) * kNoallocMaxGuides;
constexpr size_t kKeysOff = (kGuidesOff + sizeof(GuideRec) * kNoallocMaxGuides + 255) / 256 * 256;
constexpr size_t kNoallocBytes = kKeysOff + sizeof(uint64_t) * kNoallocMaxHits;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mutex;
static unsigned char *g_noalloc_ptr[kMaxDevices];
static int g_noalloc_blocks_per_sm[kMaxDevices];
static int g_noalloc_sms[kMaxDevices];
// host-side family and guide tables of a call (about 72 KB; static so that a
// call needs no heap and no large stack frame), guarded by g_noalloc_mutex
static FamilyDesc g_fams[kNoallocMaxGuides];
static GuideRec g_recs[kNoallocMaxGuides];
static int32_t g_fam_of[kNoallocMaxGuides];

// Device address of the scratch array on `device` (current), looked up once;
// the caller holds g_noalloc_mutex.
static int noalloc_setup(int device, unsigned char **out) {
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "bgo_scan_noalloc: cudaGetSymbolAddress");
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, scan_kernel, kTileThreads, 0);
        if (e != cudaSuccess) return cuda_fail(e, "bgo_scan_noalloc: occupancy");
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess) return cuda_fail(e, "bgo_scan_noalloc: SM count");
        g_noalloc_blocks_per_sm[device] = n > 0 ? n : 1;
        g_noalloc_sms[device] = sms;
        g_noalloc_ptr[device] = (unsigned char *)p;
    }
    *out = g_noalloc_ptr[device];
    return BGO_OK;
}

}  // namespace bgo

using namespace bgo;

extern "C" int bgo_scan_noalloc(const bgo_genome *const *strands, const int32_t *n_encoded,
                                int32_t n_strands, const uint64_t *guide_encoded,
                                const uint8_t *pam_masks, const uint8_t *pam_lens,
                                const uint8_t *pam_3prime, int32_t n_guides,
                                int32_t max_mismatches, uint64_t *keys, int64_t capacity,
                                int64_t *n_hits, void *stream) {
    if (!strands || !n_encoded || n_strands < 1 || n_strands > 2 || !n_hits || capacity < 0 ||
        n_guides < 0 || (n_guides > 0 && (!guide_encoded || !pam_masks || !pam_lens ||
                                          !pam_3prime))) {
        set_error("bgo_scan_noalloc: invalid argument");
        return BGO_ERR_ARG;
    }
    if (n_guides > kNoallocMaxGuides) {
        set_error("bgo_scan_noalloc: " + std::to_string(n_guides) +
                  " guide rows exceed the static limit of " + std::to_string(kNoallocMaxGuides) +
                  " (BGO_NOALLOC_MAX_GUIDES); split the rows or use bgo_plan_create");
        return BGO_ERR_ARG;
    }
    for (int i = 0; i < n_strands; ++i) {
        if (!strands[i] || n_encoded[i] < 0 || n_encoded[i] > 3 ||
            strands[i]->device != strands[0]->device) {
            set_error("bgo_scan_noalloc: bad strand or n_encoded");
            return BGO_ERR_ARG;
        }
    }
    const int device = strands[0]->device;
    if (device < 0 || device >= kMaxDevices) {
        set_error("bgo_scan_noalloc: device index out of range");
        return BGO_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    BGO_CUDA(cudaSetDevice(device));
    unsigned char *base = nullptr;
    int rc = noalloc_setup(device, &base);
    if (rc != BGO_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;

    // PAM families and guide planes built in the static host tables (no heap).
    FamilyDesc *fams = g_fams;
    GuideRec *recs = g_recs;
    int32_t *fam_of = g_fam_of;
    int n_fams = 0;
    for (int32_t i = 0; i < n_guides; ++i) {
        fam_of[i] = -1;
        const int plen = pam_lens[i];
        if (plen <= 0 || plen > kMaxPam) continue;
        FamilyDesc d{};
        for (int k = 0; k < plen; ++k) d.allowed[k] = pam_masks[i * kMaxPam + k] & 15u;
        d.plen = (uint8_t)plen;
        d.three_prime = pam_3prime[i] ? 1 : 0;
        int f = 0;
        for (; f < n_fams; ++f) {
            if (fams[f].plen == d.plen && fams[f].three_prime == d.three_prime &&
                std::equal(d.allowed, d.allowed + kMaxPam, fams[f].allowed))
                break;
        }
        if (f == n_fams) fams[n_fams++] = d;
        fam_of[i] = f;
    }
    int32_t n_recs = 0;
    for (int f = 0; f < n_fams; ++f) {
        fams[f].gbeg = n_recs;
        for (int32_t i = 0; i < n_guides; ++i) {
            if (fam_of[i] != f) continue;
            GuideRec r{};
            for (int k = 0; k < kGuideLen; ++k) {
                const uint32_t b = (uint32_t)((guide_encoded[i] >> (2 * k)) & 3u);
                r.h |= ((b >> 1) & 1u) << k;
                r.l |= (b & 1u) << k;
            }
            r.row = (uint32_t)i;
            recs[n_recs++] = r;
        }
        fams[f].gend = n_recs;
    }

    unsigned long long *d_counter = (unsigned long long *)base;
    FamilyDesc *d_fams = (FamilyDesc *)(base + kFamiliesOff);
    GuideRec *d_guides = (GuideRec *)(base + kGuidesOff);
    uint64_t *d_keys = (uint64_t *)(base + kKeysOff);
    BGO_CUDA(cudaMemsetAsync(d_counter, 0, 2 * sizeof(unsigned long long), s));
    if (n_fams > 0) {
        BGO_CUDA(cudaMemcpyAsync(d_fams, fams, sizeof(FamilyDesc) * n_fams,
                                 cudaMemcpyHostToDevice, s));
        BGO_CUDA(cudaMemcpyAsync(d_guides, recs, sizeof(GuideRec) * n_recs,
                                 cudaMemcpyHostToDevice, s));
        ScanParams p{};
        for (int i = 0; i < n_strands; ++i) {
            const bgo_genome *g = strands[i];
            StrandDesc &d = p.strand[i];
            d.H = g->d_planes;
            d.L = g->d_planes + g->plane_words;
            d.N = g->d_planes + 2 * g->plane_words;
            d.nsum = g->d_nsum;
            d.total_bp = g->total_bp;
            d.n_tiles = tiles_for(g->total_bp);
            d.has_n = g->has_n;
            d.n_encoded = n_encoded[i];
            d.slot = i;
        }
        p.n_strands = n_strands;
        p.tiles_total = p.strand[0].n_tiles + (n_strands > 1 ? p.strand[1].n_tiles : 0);
        p.fam_begin = 0;
        p.fam_end = n_fams;
        p.max_mm = max_mismatches;
        p.fams = d_fams;
        p.guides = d_guides;
        p.keys = d_keys;
        p.cap = kNoallocMaxHits;
        p.counter = d_counter;
        if (p.tiles_total > 0) {
            const int64_t grid = std::min<int64_t>(
                p.tiles_total, (int64_t)g_noalloc_sms[device] * g_noalloc_blocks_per_sm[device]);
            scan_kernel<<<(unsigned)grid, kTileThreads, 0, s>>>(p);
            BGO_CUDA(cudaGetLastError());
        }
    }
    unsigned long long n = 0;
    BGO_CUDA(cudaMemcpyAsync(&n, d_counter, sizeof(n), cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    *n_hits = (int64_t)n;
    if ((int64_t)n > kNoallocMaxHits) {
        set_error("bgo_scan_noalloc: " + std::to_string(n) + " hits exceed the static buffer of " +
                  std::to_string(kNoallocMaxHits) + " keys (BGO_NOALLOC_MAX_HITS); *n_hits "
                  "holds the exact count, use bgo_scan_launch for this search");
        return BGO_ERR_OOM;
    }
    if (keys && n > 0 && (int64_t)n <= capacity) {
        BGO_CUDA(cudaMemcpyAsync(keys, d_keys, (size_t)n * sizeof(uint64_t),
                                 cudaMemcpyDeviceToHost, s));
        BGO_CUDA(cudaStreamSynchronize(s));
        std::sort(keys, keys + n);
    }
    return BGO_OK;
}
