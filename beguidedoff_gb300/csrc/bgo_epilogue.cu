// Device epilogue of a scan: the per-hit part of the reference's host
// post-processing (beguidedoff/finder.py:193-244 decode / strand mapping /
// on-target exclusion, :405-472 mismatch positions / CCTOP / editable window /
// below-threshold count, :545-566 sort and top-N) for hit counts where a
// per-hit host loop is too slow.
//
// Scores.  The CCTOP score of a hit is a function of its 20-bit mismatch mask
// (guide vs decoded window).  The caller supplies rank_table[mask] = rank of
// that mask's exact score among all distinct scores (ascending), computed on
// the host with the reference's own summation, so ordering hits by score and
// testing "score <= threshold" become integer comparisons here and stay exact.
//
// Order.  The reference sorts a guide's hits by (score, chromosome name rank,
// local report position, strand).  A hit's order key packs exactly that:
// rank << 44 | name rank << 34 | (local + 2^32) << 1 | strand (20 + 10 + 33 +
// 1 bits; the local position is negative for junction windows the reference
// maps to chromosome -1).  With more than 1024 chromosomes the key is the
// rank alone and ties at the cut are all kept.
//
// Steps (one thread per hit in the passes over the engine's hit keys):
//   1. pass 1: per hit the window, mask, rank, report position and leftmost
//      position; per input row mapped to the hit's plan row: on-target
//      exclusion, editable-window test, below-threshold count, per-(plan row,
//      strand) hit count, and a histogram of rank >> 8 over the included hits;
//   2. per input row (one CTA): the histogram bin holding its n_top-th
//      included hit and the number of included hits up to that bin; an
//      exclusive scan gives every row a segment of that size;
//   3. pass 2: the included hits up to the cut bin are written to their
//      row's segment;
//   4. per input row (one CTA): radix select of the n_top smallest order keys
//      in the segment (8-bit digits, most significant first), compacted in
//      place; a scan and a gather make the kept records dense.
#include <cuda_runtime.h>

#include <cstring>

#include <algorithm>
#include <new>
#include <vector>

#include "bgo_internal.cuh"

namespace bgo {

constexpr int kRankShift = 8;
constexpr int kRankBins = (1 << 20) >> kRankShift;  // 4096
constexpr int kMaxChroms = 1 << 20;
constexpr int kExactChroms = 1024;
constexpr int kRowThreads = 256;

struct RowInfo {       // per plan row
    uint32_t h, l;     // guide planes
    int32_t plen;      // PAM length (3' PAM)
    int32_t in_beg;    // input rows [in_beg, in_end) in the CSR list
    int32_t in_end;
    int32_t pad;
};

struct EpiParams {
    const uint64_t *keys;
    int64_t n_hits;
    const uint32_t *H[2];
    const uint32_t *L[2];
    const RowInfo *rows;
    int32_t n_plan_rows;
    const int32_t *in_list;  // CSR: input row ids
    const bgo_input_row *inputs;
    int32_t n_inputs;
    const int64_t *chrom_off;
    const int64_t *chrom_len;
    const int32_t *chrom_rank;
    int32_t n_chroms;
    int32_t exact_order;
    const uint32_t *rank_table;
    unsigned long long *below;      // [n_inputs]
    unsigned long long *group_cnt;  // [n_plan_rows * 2]
    unsigned int *hist;             // [n_inputs * kRankBins]
    const int32_t *cut;             // [n_inputs]
    const int64_t *seg_off;         // [n_inputs]
    const int64_t *seg_cnt;         // [n_inputs]
    unsigned long long *fill;       // [n_inputs]
    bgo_record *recs;
};

// atomicAdd of 1 per lane, aggregated over the active lanes that target the
// same address (one atomic per distinct address per warp: hits of one dense
// guide land on the same few counters).
template <typename T>
__device__ __forceinline__ void aggregated_inc(T *addr) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, (unsigned long long)addr);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(addr, (T)__popc(peers));
}

// Fetch-and-increment with the same aggregation: every lane gets its own
// slot (the peers' base plus its rank among them).
template <typename T>
__device__ __forceinline__ T aggregated_fetch_inc(T *addr) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, (unsigned long long)addr);
    const int leader = __ffs(peers) - 1;
    const int lane = (int)(threadIdx.x & 31);
    T base = 0;
    if (lane == leader) base = atomicAdd(addr, (T)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (T)__popc(peers & ((1u << lane) - 1u));
}

// Index of the last chromosome whose offset is <= pos (-1 below the first,
// like Python's searchsorted(..., 'right') - 1).
__device__ __forceinline__ int chrom_of(const int64_t *off, int n, int64_t pos) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= pos) lo = mid + 1;
        else hi = mid;
    }
    return lo - 1;
}

template <int PASS>
__global__ void epilogue_kernel(EpiParams e) {
    const int64_t *__restrict__ off = e.chrom_off;
    const int64_t *__restrict__ len = e.chrom_len;
    const int nc = e.n_chroms;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < e.n_hits;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = e.keys[i];
        const int row = (int)(key >> 39);
        const int slot = (int)((key >> 38) & 1u);
        const int64_t pos = (int64_t)((key >> 6) & 0xFFFFFFFFull);
        if (row >= e.n_plan_rows) continue;
        const RowInfo R = e.rows[row];
        if (PASS == 2 && R.in_beg == R.in_end) continue;
        const uint32_t *H = slot ? e.H[1] : e.H[0];
        const uint32_t *L = slot ? e.L[1] : e.L[0];
        const int64_t w = pos >> 5;
        const uint32_t b = (uint32_t)(pos & 31);
        const uint32_t h20 = __funnelshift_r(H[w], H[w + 1], b) & 0xFFFFFu;
        const uint32_t l20 = __funnelshift_r(L[w], L[w + 1], b) & 0xFFFFFu;
        const uint32_t mask = (h20 ^ R.h) | (l20 ^ R.l);
        const uint32_t rank = e.rank_table[mask];
        const int64_t window = 20 + R.plen;
        int64_t leftmost = pos;
        if (slot) {
            const int ci = chrom_of(off, nc, pos);
            const int64_t local_rc = pos - off[ci];
            leftmost = off[ci] + (len[ci] - local_rc - window);
        }
        const int ot_ci = chrom_of(off, nc, leftmost);
        // Python indexes chromosome -1 as the last one
        const int64_t ot_local = leftmost - off[ot_ci >= 0 ? ot_ci : nc - 1];
        if (PASS == 1) aggregated_inc(e.group_cnt + 2 * row + slot);
        uint64_t order = (uint64_t)rank << 44;
        if (PASS == 2 && e.exact_order) {
            const int64_t report = slot ? leftmost + window - 1 : pos;
            int rc = chrom_of(off, nc, report);
            if (rc < 0) rc = nc - 1;
            const int64_t local = report - off[rc];
            order |= ((uint64_t)(uint32_t)e.chrom_rank[rc] << 34) |
                     ((uint64_t)(local + (1ll << 32)) << 1) | (uint64_t)slot;
        }
        for (int k = R.in_beg; k < R.in_end; ++k) {
            const int ir = e.in_list[k];
            const bgo_input_row in = e.inputs[ir];
            if (in.ot_chrom >= 0 && ot_ci == in.ot_chrom && ot_local == in.ot_local &&
                slot == in.ot_strand)
                continue;
            const uint32_t base_hit = in.target_base == 1 ? (~h20 & l20) : (~h20 & ~l20);
            const bool editable = (base_hit & in.window_mask & 0xFFFFFu) != 0u;
            const bool include = editable || (in.flags & BGO_ROW_RETURN_ALL);
            const uint32_t bin = rank >> kRankShift;
            if (PASS == 1) {
                if (in.threshold_rank >= 0 && editable && (int32_t)rank <= in.threshold_rank)
                    aggregated_inc(e.below + ir);
                if (include) aggregated_inc(e.hist + (size_t)ir * kRankBins + bin);
            } else if (include && (int32_t)bin <= e.cut[ir]) {
                const unsigned long long f = aggregated_fetch_inc(e.fill + ir);
                if ((int64_t)f < e.seg_cnt[ir]) {
                    bgo_record r;
                    r.key = key;
                    r.order = order;
                    r.input_row = ir;
                    r.rank = rank;
                    e.recs[e.seg_off[ir] + (int64_t)f] = r;
                }
            }
        }
    }
}

// Block-wide exclusive scan of one value per thread; returns the total.
// sWarp holds 33 values.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T &excl, T *sWarp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    T incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) sWarp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const T x = lane < nw ? sWarp[lane] : (T)0;
        T y = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T u = __shfl_up_sync(0xFFFFFFFFu, y, o);
            if (lane >= o) y += u;
        }
        if (lane < nw) sWarp[lane] = y - x;
        if (lane == 31) sWarp[32] = y;
    }
    __syncthreads();
    excl = sWarp[warp] + incl - v;
    const T total = sWarp[32];
    __syncthreads();
    return total;
}

// Per input row (one CTA of kRowThreads): cut bin and segment size.
__global__ void __launch_bounds__(kRowThreads) cut_kernel(const unsigned int *hist,
                                                          const bgo_input_row *inputs, int n_top,
                                                          int32_t *cut, int64_t *seg_cnt) {
    constexpr int kPer = kRankBins / kRowThreads;  // 16 bins per thread
    __shared__ long long sWarp[33];
    __shared__ int sFirst;
    const int r = blockIdx.x;
    const int t = threadIdx.x;
    const unsigned int *h = hist + (size_t)r * kRankBins + (size_t)t * kPer;
    unsigned int v[kPer];
    long long sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        v[k] = h[k];
        sum += v[k];
    }
    long long excl = 0;
    const long long total = block_exclusive_scan<long long>(sum, excl, sWarp);
    const bool all = (inputs[r].flags & BGO_ROW_RETURN_ALL) != 0;
    if (all || total <= (long long)n_top) {
        if (t == 0) {
            cut[r] = total > 0 ? kRankBins - 1 : -1;
            seg_cnt[r] = total;
        }
        return;
    }
    if (n_top <= 0) {
        if (t == 0) {
            cut[r] = -1;
            seg_cnt[r] = 0;
        }
        return;
    }
    if (t == 0) sFirst = kRowThreads;
    __syncthreads();
    if (excl < n_top && excl + sum >= n_top) atomicMin(&sFirst, t);
    __syncthreads();
    if (t == sFirst) {
        long long run = excl;
        int b = 0;
        for (; b < kPer; ++b) {
            run += v[b];
            if (run >= n_top) break;
        }
        cut[r] = t * kPer + b;
        seg_cnt[r] = run;
    }
}

// Exclusive scan of n int64 values by one CTA of 1024 threads; total in *total.
__global__ void __launch_bounds__(1024) scan_rows_kernel(const int64_t *in, int64_t *out, int n,
                                                         int64_t *total) {
    __shared__ long long sWarp[33];
    long long carry = 0;
    for (int base = 0; base < n; base += 1024) {
        const int i = base + (int)threadIdx.x;
        const long long v = i < n ? in[i] : 0;
        long long excl = 0;
        const long long tot = block_exclusive_scan<long long>(v, excl, sWarp);
        if (i < n) out[i] = carry + excl;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

// Per input row (one CTA): keep the n_top smallest order keys of its segment
// (every record when the row returns all), compacted to the segment start.
__global__ void __launch_bounds__(kRowThreads) select_kernel(bgo_record *recs,
                                                             const bgo_input_row *inputs,
                                                             const int64_t *seg_off,
                                                             const int64_t *seg_cnt,
                                                             const unsigned long long *fill,
                                                             int n_top, int64_t *kept) {
    __shared__ unsigned int sHist[256];
    __shared__ long long sWarp[33];
    __shared__ unsigned long long sPrefix;
    __shared__ long long sNeed;
    const int r = blockIdx.x;
    const int t = threadIdx.x;
    const int64_t cnt = min((int64_t)fill[r], seg_cnt[r]);
    bgo_record *seg = recs + seg_off[r];
    if ((inputs[r].flags & BGO_ROW_RETURN_ALL) || cnt <= (int64_t)n_top) {
        if (t == 0) kept[r] = cnt;
        return;
    }
    // radix select of the n_top-th smallest order key
    unsigned long long prefix = 0, pmask = 0;
    long long need = n_top;
    for (int d = 7; d >= 0; --d) {
        for (int i = t; i < 256; i += kRowThreads) sHist[i] = 0u;
        __syncthreads();
        for (int64_t i = t; i < cnt; i += kRowThreads) {
            const unsigned long long o = seg[i].order;
            if ((o & pmask) == prefix) atomicAdd(&sHist[(o >> (8 * d)) & 255u], 1u);
        }
        __syncthreads();
        if (t == 0) {
            long long acc = 0;
            int sel = 255;
            for (int b = 0; b < 256; ++b) {
                if (acc + (long long)sHist[b] >= need) {
                    sel = b;
                    break;
                }
                acc += sHist[b];
            }
            sPrefix = prefix | ((unsigned long long)sel << (8 * d));
            sNeed = need - acc;
        }
        __syncthreads();
        prefix = sPrefix;
        need = sNeed;
        pmask |= 255ull << (8 * d);
        __syncthreads();
    }
    // prefix is now the n_top-th smallest key: keep every record <= it
    long long running = 0;
    for (int64_t start = 0; start < cnt; start += kRowThreads) {
        const int64_t i = start + t;
        bgo_record rec{};
        bool keep = false;
        if (i < cnt) {
            rec = seg[i];
            keep = rec.order <= prefix;
        }
        long long excl = 0;
        const long long tot = block_exclusive_scan<long long>(keep ? 1 : 0, excl, sWarp);
        if (keep) seg[running + excl] = rec;  // never beyond the tile already read
        running += tot;
        __syncthreads();
    }
    if (t == 0) kept[r] = running;
}

// Dense copy of every row's kept records.
__global__ void gather_kernel(const bgo_record *recs, const int64_t *seg_off, const int64_t *kept,
                              const int64_t *kept_off, bgo_record *out) {
    const int r = blockIdx.x;
    const int64_t n = kept[r];
    const bgo_record *src = recs + seg_off[r];
    bgo_record *dst = out + kept_off[r];
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

static int grow(unsigned char *&buf, size_t &have, size_t need) {
    if (need <= have) return BGO_OK;
    if (buf) cudaFree(buf);
    buf = nullptr;
    have = 0;
    const size_t want = need + need / 4 + 256;
    BGO_CUDA(cudaMalloc(&buf, want));
    have = want;
    return BGO_OK;
}

}  // namespace bgo

using namespace bgo;

extern "C" int bgo_epilogue_run(bgo_engine *engine, const bgo_plan *plan,
                                const bgo_genome *const *strands, int32_t n_strands,
                                const bgo_input_row *inputs, int32_t n_inputs,
                                const int64_t *chrom_offsets, const int64_t *chrom_lengths,
                                const int32_t *chrom_rank, int32_t n_chroms,
                                const uint32_t *rank_table, int32_t n_top, int64_t *below,
                                int64_t *group_counts, int64_t *row_counts, int64_t *n_records,
                                void *stream) {
    if (!engine || !plan || !strands || n_strands < 1 || n_strands > 2 || n_inputs < 0 ||
        (n_inputs > 0 && (!inputs || !below || !row_counts)) || !chrom_offsets ||
        !chrom_lengths || !chrom_rank || n_chroms <= 0 || n_chroms > kMaxChroms || !rank_table ||
        !group_counts || !n_records || n_top < 0) {
        set_error("bgo_epilogue_run: invalid argument");
        return BGO_ERR_ARG;
    }
    if (!engine->launched) {
        set_error("bgo_epilogue_run: no scan to finish");
        return BGO_ERR_STATE;
    }
    engine->epi_out_n = -1;
    BGO_CUDA(cudaSetDevice(engine->device));
    cudaStream_t s = (cudaStream_t)stream;
    const int32_t n_rows = plan->n_guides;
    // per plan row: guide planes, PAM length, input-row list
    std::vector<RowInfo> rows((size_t)n_rows + 1);
    for (int f = 0; f < plan->n_families; ++f) {
        const FamilyDesc &F = plan->h_fams[f];
        for (int g = F.gbeg; g < F.gend; ++g) {
            const GuideRec &r = plan->h_guides[g];
            rows[r.row].h = r.h;
            rows[r.row].l = r.l;
            rows[r.row].plen = F.plen;
        }
    }
    std::vector<int32_t> count((size_t)n_rows + 1, 0), list((size_t)n_inputs + 1);
    for (int32_t i = 0; i < n_inputs; ++i) {
        if (inputs[i].plan_row < 0 || inputs[i].plan_row >= n_rows) {
            set_error("bgo_epilogue_run: input row refers to a missing plan row");
            return BGO_ERR_ARG;
        }
        count[(size_t)inputs[i].plan_row]++;
    }
    int32_t acc = 0;
    for (int32_t r = 0; r < n_rows; ++r) {
        rows[(size_t)r].in_beg = acc;
        acc += count[(size_t)r];
        rows[(size_t)r].in_end = rows[(size_t)r].in_beg;
    }
    for (int32_t i = 0; i < n_inputs; ++i) {
        RowInfo &R = rows[(size_t)inputs[i].plan_row];
        list[(size_t)R.in_end++] = i;
    }
    unsigned long long cnt[3] = {0, 0, 0};
    BGO_CUDA(cudaMemcpyAsync(cnt, engine->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    const int64_t n_hits = (int64_t)cnt[0];
    engine->d2h_bytes += (int64_t)sizeof(cnt);
    if (cnt[2] & 1u) {
        set_error("bgo_epilogue_run: a chunk copy of the last scan did not complete in time");
        return BGO_ERR_TIMEOUT;
    }
    if (n_hits > engine->cap) {
        set_error("bgo_epilogue_run: the last scan overflowed the hit buffer; reserve and rescan");
        return BGO_ERR_STATE;
    }
    // device scratch (grow-only, kept by the engine)
    const size_t ni = (size_t)n_inputs + 1;
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t b_rows = al(sizeof(RowInfo) * rows.size()), b_list = al(sizeof(int32_t) * ni);
    const size_t b_in = al(sizeof(bgo_input_row) * ni), b_chr = al(sizeof(int64_t) * n_chroms);
    const size_t b_crank = al(sizeof(int32_t) * n_chroms);
    const size_t b_below = al(sizeof(unsigned long long) * ni);
    const size_t b_grp = al(sizeof(unsigned long long) * (size_t)(2 * n_rows + 2));
    const size_t b_hist = al(sizeof(unsigned int) * ni * kRankBins);
    const size_t b_fill = al(sizeof(unsigned long long) * ni);
    const size_t b_i32 = al(sizeof(int32_t) * ni), b_i64 = al(sizeof(int64_t) * ni);
    const size_t b_tot = al(4 * sizeof(int64_t));
    const size_t zero_bytes = b_below + b_grp + b_hist + b_fill + b_tot;  // contiguous, zeroed
    const size_t total = b_rows + b_list + b_in + 2 * b_chr + b_crank + zero_bytes + b_i32 +
                         4 * b_i64;
    if (grow(engine->d_epi, engine->epi_bytes, total) != BGO_OK) return BGO_ERR_CUDA;
    const size_t rank_n = (size_t)1 << 20;
    if (!engine->d_rank) BGO_CUDA(cudaMalloc(&engine->d_rank, sizeof(uint32_t) * rank_n));
    // a table at the address of the last one is taken as unchanged (no 4 MB
    // compare per call); another address is compared and uploaded if it differs
    if (rank_table != engine->rank_src) {
        if (engine->h_rank.size() != rank_n ||
            memcmp(engine->h_rank.data(), rank_table, sizeof(uint32_t) * rank_n) != 0) {
            engine->h_rank.assign(rank_table, rank_table + rank_n);
            BGO_CUDA(cudaMemcpyAsync(engine->d_rank, engine->h_rank.data(),
                                     sizeof(uint32_t) * rank_n, cudaMemcpyHostToDevice, s));
            engine->h2d_bytes += (int64_t)(sizeof(uint32_t) * rank_n);
        }
        engine->rank_src = rank_table;
    }
    unsigned char *d = engine->d_epi;
    size_t o = 0;
    auto take = [&](size_t b) {
        unsigned char *p = d + o;
        o += b;
        return p;
    };
    RowInfo *d_rows = (RowInfo *)take(b_rows);
    int32_t *d_list = (int32_t *)take(b_list);
    bgo_input_row *d_in = (bgo_input_row *)take(b_in);
    int64_t *d_off = (int64_t *)take(b_chr);
    int64_t *d_len = (int64_t *)take(b_chr);
    int32_t *d_crank = (int32_t *)take(b_crank);
    unsigned char *d_zero = d + o;
    unsigned long long *d_below = (unsigned long long *)take(b_below);
    unsigned long long *d_grp = (unsigned long long *)take(b_grp);
    unsigned int *d_hist = (unsigned int *)take(b_hist);
    unsigned long long *d_fill = (unsigned long long *)take(b_fill);
    int64_t *d_tot = (int64_t *)take(b_tot);
    int32_t *d_cut = (int32_t *)take(b_i32);
    int64_t *d_seg_cnt = (int64_t *)take(b_i64);
    int64_t *d_seg_off = (int64_t *)take(b_i64);
    int64_t *d_kept = (int64_t *)take(b_i64);
    int64_t *d_kept_off = (int64_t *)take(b_i64);
    cudaError_t ce = cudaSuccess;
    auto step = [&](cudaError_t x) {
        if (ce == cudaSuccess) ce = x;
    };
    step(cudaMemcpyAsync(d_rows, rows.data(), sizeof(RowInfo) * rows.size(), cudaMemcpyHostToDevice,
                         s));
    if (n_inputs) {
        step(cudaMemcpyAsync(d_list, list.data(), sizeof(int32_t) * (size_t)n_inputs,
                             cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(d_in, inputs, sizeof(bgo_input_row) * (size_t)n_inputs,
                             cudaMemcpyHostToDevice, s));
    }
    step(cudaMemcpyAsync(d_off, chrom_offsets, sizeof(int64_t) * n_chroms, cudaMemcpyHostToDevice,
                         s));
    step(cudaMemcpyAsync(d_len, chrom_lengths, sizeof(int64_t) * n_chroms, cudaMemcpyHostToDevice,
                         s));
    step(cudaMemcpyAsync(d_crank, chrom_rank, sizeof(int32_t) * n_chroms, cudaMemcpyHostToDevice,
                         s));
    engine->h2d_bytes += (int64_t)(sizeof(RowInfo) * rows.size() +
                                   (sizeof(int32_t) + sizeof(bgo_input_row)) * (size_t)n_inputs +
                                   (2 * sizeof(int64_t) + sizeof(int32_t)) * (size_t)n_chroms);
    step(cudaMemsetAsync(d_zero, 0, zero_bytes, s));

    EpiParams e{};
    e.keys = engine->d_keys;
    e.n_hits = n_hits;
    for (int i = 0; i < 2; ++i) {
        const bgo_genome *g = strands[i < n_strands ? i : 0];
        e.H[i] = g->d_planes;
        e.L[i] = g->d_planes + g->plane_words;
    }
    e.rows = d_rows;
    e.n_plan_rows = n_rows;
    e.in_list = d_list;
    e.inputs = d_in;
    e.n_inputs = n_inputs;
    e.chrom_off = d_off;
    e.chrom_len = d_len;
    e.chrom_rank = d_crank;
    e.n_chroms = n_chroms;
    e.exact_order = n_chroms <= kExactChroms ? 1 : 0;
    e.rank_table = engine->d_rank;
    e.below = d_below;
    e.group_cnt = d_grp;
    e.hist = d_hist;
    e.cut = d_cut;
    e.seg_off = d_seg_off;
    e.seg_cnt = d_seg_cnt;
    e.fill = d_fill;
    const int threads = 256;
    const int64_t grid = std::max<int64_t>(
        1, std::min<int64_t>((n_hits + threads - 1) / threads, (int64_t)engine->sm_count * 8));
    if (ce == cudaSuccess && n_hits > 0) {
        epilogue_kernel<1><<<(unsigned)grid, threads, 0, s>>>(e);
        step(cudaGetLastError());
        engine->launches++;
    }
    if (ce == cudaSuccess && n_inputs > 0) {
        cut_kernel<<<(unsigned)n_inputs, kRowThreads, 0, s>>>(d_hist, d_in, n_top, d_cut,
                                                             d_seg_cnt);
        step(cudaGetLastError());
        scan_rows_kernel<<<1, 1024, 0, s>>>(d_seg_cnt, d_seg_off, n_inputs, d_tot);
        step(cudaGetLastError());
        engine->launches += 2;
    }
    int64_t n_cand = 0;
    step(cudaMemcpyAsync(&n_cand, d_tot, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    step(cudaStreamSynchronize(s));
    engine->d2h_bytes += 8;
    if (ce != cudaSuccess) return cuda_fail(ce, "bgo_epilogue_run");
    if (grow(engine->d_epi_rec, engine->epi_rec_bytes, sizeof(bgo_record) * (size_t)(n_cand + 1)) !=
        BGO_OK)
        return BGO_ERR_CUDA;
    e.recs = (bgo_record *)engine->d_epi_rec;
    if (n_hits > 0 && n_cand > 0) {
        epilogue_kernel<2><<<(unsigned)grid, threads, 0, s>>>(e);
        step(cudaGetLastError());
        engine->launches++;
    }
    if (ce == cudaSuccess && n_inputs > 0) {
        select_kernel<<<(unsigned)n_inputs, kRowThreads, 0, s>>>(e.recs, d_in, d_seg_off,
                                                                 d_seg_cnt, d_fill, n_top, d_kept);
        step(cudaGetLastError());
        scan_rows_kernel<<<1, 1024, 0, s>>>(d_kept, d_kept_off, n_inputs, d_tot + 1);
        step(cudaGetLastError());
        engine->launches += 2;
    }
    int64_t n_kept = 0;
    std::vector<unsigned long long> tmp_b(ni), tmp_g((size_t)2 * n_rows + 2);
    std::vector<int64_t> tmp_k(ni);
    step(cudaMemcpyAsync(&n_kept, d_tot + 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    step(cudaMemcpyAsync(tmp_b.data(), d_below, sizeof(unsigned long long) * ni,
                         cudaMemcpyDeviceToHost, s));
    step(cudaMemcpyAsync(tmp_g.data(), d_grp, sizeof(unsigned long long) * tmp_g.size(),
                         cudaMemcpyDeviceToHost, s));
    step(cudaMemcpyAsync(tmp_k.data(), d_kept, sizeof(int64_t) * ni, cudaMemcpyDeviceToHost, s));
    step(cudaStreamSynchronize(s));
    if (ce != cudaSuccess) return cuda_fail(ce, "bgo_epilogue_run");
    engine->d2h_bytes += (int64_t)(8 + 8 * (2 * ni + tmp_g.size()));
    if (grow(engine->d_epi_out, engine->epi_out_bytes, sizeof(bgo_record) * (size_t)(n_kept + 1)) !=
        BGO_OK)
        return BGO_ERR_CUDA;
    if (n_inputs > 0 && n_kept > 0) {
        gather_kernel<<<(unsigned)n_inputs, 128, 0, s>>>(e.recs, d_seg_off, d_kept, d_kept_off,
                                                         (bgo_record *)engine->d_epi_out);
        step(cudaGetLastError());
        step(cudaStreamSynchronize(s));
        engine->launches++;
        if (ce != cudaSuccess) return cuda_fail(ce, "bgo_epilogue_run");
    }
    for (int32_t i = 0; i < n_inputs; ++i) {
        below[i] = (int64_t)tmp_b[(size_t)i];
        row_counts[i] = tmp_k[(size_t)i];
    }
    for (int32_t i = 0; i < 2 * n_rows; ++i) group_counts[i] = (int64_t)tmp_g[(size_t)i];
    *n_records = n_kept;
    engine->epi_out_n = n_kept;
    return BGO_OK;
}

extern "C" int bgo_epilogue_fetch(bgo_engine *engine, bgo_record *records, int64_t capacity,
                                  void *stream) {
    if (!engine || capacity < 0 || (capacity > 0 && !records)) return BGO_ERR_ARG;
    if (engine->epi_out_n < 0) {
        set_error("bgo_epilogue_fetch: no epilogue results");
        return BGO_ERR_STATE;
    }
    if (capacity < engine->epi_out_n) {
        set_error("bgo_epilogue_fetch: capacity below the record count");
        return BGO_ERR_ARG;
    }
    if (engine->epi_out_n == 0) return BGO_OK;
    BGO_CUDA(cudaSetDevice(engine->device));
    cudaStream_t s = (cudaStream_t)stream;
    BGO_CUDA(cudaMemcpyAsync(records, engine->d_epi_out,
                             sizeof(bgo_record) * (size_t)engine->epi_out_n,
                             cudaMemcpyDeviceToHost, s));
    BGO_CUDA(cudaStreamSynchronize(s));
    engine->d2h_bytes += (int64_t)(sizeof(bgo_record) * (size_t)engine->epi_out_n);
    return BGO_OK;
}
