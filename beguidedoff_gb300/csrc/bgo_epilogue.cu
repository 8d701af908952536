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
// Passes over the engine's hit keys (unsorted, one thread per hit):
//   1. per hit: window from the strand's planes, mask, rank, report position
//      and chromosome, leftmost position for the on-target test; per input
//      row mapped to the hit's plan row: exclusion, editable-window test,
//      below-threshold count, per-(plan row, strand) hit count, and a
//      histogram of (rank >> kRankShift) over the included hits;
//   2. per input row: the histogram bin holding its n_top-th included hit
//      (all bins when every hit is returned);
//   3. per hit and input row: records for included hits whose bin is at or
//      below that cut.  The host sorts these few records exactly and keeps
//      n_top per row; the records are a superset of every row's top n_top.
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
    const int32_t *in_list;          // CSR: input row ids
    const bgo_input_row *inputs;
    int32_t n_inputs;
    const int64_t *chrom_off;
    const int64_t *chrom_len;
    int32_t n_chroms;
    const uint32_t *rank_table;
    int32_t threshold_rank;          // -1: no threshold
    int32_t return_all;
    unsigned long long *below;       // [n_inputs]
    unsigned long long *group_cnt;   // [n_plan_rows * 2]
    unsigned int *hist;              // [n_inputs * kRankBins]
    const int32_t *cut;              // [n_inputs]
    bgo_record *out;
    int64_t cap;
    unsigned long long *out_count;
};

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
    const int64_t *__restrict__ sOff = e.chrom_off;
    const int64_t *__restrict__ sLen = e.chrom_len;
    const int nc = e.n_chroms;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < e.n_hits;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = e.keys[i];
        const int row = (int)(key >> 39);
        const int slot = (int)((key >> 38) & 1u);
        const int64_t pos = (int64_t)((key >> 6) & 0xFFFFFFFFull);
        if (row >= e.n_plan_rows) continue;
        const RowInfo R = e.rows[row];
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
            const int ci = chrom_of(sOff, nc, pos);
            const int64_t local_rc = pos - sOff[ci];
            leftmost = sOff[ci] + (sLen[ci] - local_rc - window);
        }
        const int ot_ci = chrom_of(sOff, nc, leftmost);
        // Python indexes chromosome -1 as the last one
        const int64_t ot_local = leftmost - sOff[ot_ci >= 0 ? ot_ci : nc - 1];
        if (PASS == 1) atomicAdd(e.group_cnt + 2 * row + slot, 1ull);
        for (int k = R.in_beg; k < R.in_end; ++k) {
            const int ir = e.in_list[k];
            const bgo_input_row in = e.inputs[ir];
            if (in.ot_chrom >= 0 && ot_ci == in.ot_chrom && ot_local == in.ot_local &&
                slot == in.ot_strand)
                continue;
            const uint32_t base_hit = in.target_base == 1 ? (~h20 & l20) : (~h20 & ~l20);
            const bool editable = (base_hit & in.window_mask & 0xFFFFFu) != 0u;
            const bool include = editable || e.return_all;
            const uint32_t bin = rank >> kRankShift;
            if (PASS == 1) {
                if (e.threshold_rank >= 0 && editable && (int32_t)rank <= e.threshold_rank)
                    atomicAdd(e.below + ir, 1ull);
                if (include) atomicAdd(e.hist + (size_t)ir * kRankBins + bin, 1u);
            } else if (include && (int32_t)bin <= e.cut[ir]) {
                const unsigned long long slot_out = atomicAdd(e.out_count, 1ull);
                if ((int64_t)slot_out < e.cap) {
                    bgo_record r;
                    r.key = key;
                    r.input_row = ir;
                    r.rank = rank;
                    e.out[slot_out] = r;
                }
            }
        }
    }
}

// Per input row: the first bin at which the included hits reach n_top.
__global__ void cut_kernel(const unsigned int *hist, int n_inputs, int n_top, int return_all,
                           int32_t *cut) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n_inputs) return;
    if (return_all) {
        if (lane == 0) cut[warp] = kRankBins - 1;
        return;
    }
    const unsigned int *h = hist + (size_t)warp * kRankBins;
    unsigned long long run = 0;
    int found = kRankBins - 1;
    for (int b0 = 0; b0 < kRankBins; b0 += 32) {
        unsigned long long v = h[b0 + lane];
        unsigned long long incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += u;
        }
        const unsigned hitmask = __ballot_sync(0xFFFFFFFFu, run + incl >= (unsigned long long)n_top);
        if (hitmask) {
            found = b0 + __ffs(hitmask) - 1;
            break;
        }
        run += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) cut[warp] = n_top <= 0 ? -1 : found;
}

}  // namespace bgo

using namespace bgo;

extern "C" int bgo_epilogue_run(bgo_engine *engine, const bgo_plan *plan,
                                const bgo_genome *const *strands, int32_t n_strands,
                                const bgo_input_row *inputs, int32_t n_inputs,
                                const int64_t *chrom_offsets, const int64_t *chrom_lengths,
                                int32_t n_chroms, const uint32_t *rank_table,
                                int32_t threshold_rank, int32_t n_top, int32_t return_all,
                                int64_t *below, int64_t *group_counts, bgo_record *records,
                                int64_t capacity, int64_t *n_records, void *stream) {
    if (!engine || !plan || !strands || n_strands < 1 || n_strands > 2 || n_inputs < 0 ||
        (n_inputs > 0 && !inputs) || !chrom_offsets || !chrom_lengths || n_chroms <= 0 ||
        n_chroms > kMaxChroms || !rank_table || !below || !group_counts || !n_records ||
        capacity < 0 || (capacity > 0 && !records)) {
        set_error("bgo_epilogue_run: invalid argument");
        return BGO_ERR_ARG;
    }
    if (!engine->launched) {
        set_error("bgo_epilogue_run: no scan to finish");
        return BGO_ERR_STATE;
    }
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
    // device scratch: one block, freed on return
    const int64_t n_hits_host = [&] {
        unsigned long long n = 0;
        cudaMemcpyAsync(&n, engine->d_counter, sizeof(n), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        return (int64_t)n;
    }();
    engine->d2h_bytes += 8;
    if (n_hits_host > engine->cap) {
        set_error("bgo_epilogue_run: the last scan overflowed the hit buffer; reserve and rescan");
        return BGO_ERR_STATE;
    }
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t b_rows = al(sizeof(RowInfo) * rows.size());
    const size_t b_list = al(sizeof(int32_t) * list.size());
    const size_t b_in = al(sizeof(bgo_input_row) * (size_t)(n_inputs + 1));
    const size_t b_chr = al(sizeof(int64_t) * (size_t)n_chroms);
    const size_t b_below = al(sizeof(unsigned long long) * (size_t)(n_inputs + 1));
    const size_t b_grp = al(sizeof(unsigned long long) * (size_t)(2 * n_rows + 2));
    const size_t b_hist = al(sizeof(unsigned int) * (size_t)(n_inputs + 1) * kRankBins);
    const size_t b_cut = al(sizeof(int32_t) * (size_t)(n_inputs + 1));
    const size_t b_out = al(sizeof(bgo_record) * (size_t)(capacity + 1));
    const size_t b_cnt = al(sizeof(unsigned long long));
    const size_t total = b_rows + b_list + b_in + 2 * b_chr + b_below + b_grp + b_hist + b_cut +
                         b_out + b_cnt;
    // grow-only scratch and the rank table, kept by the engine across calls
    if (total > engine->epi_bytes) {
        if (engine->d_epi) cudaFree(engine->d_epi);
        engine->d_epi = nullptr;
        engine->epi_bytes = 0;
        const size_t want = total + total / 4;
        BGO_CUDA(cudaMalloc(&engine->d_epi, want));
        engine->epi_bytes = want;
    }
    const size_t rank_n = (size_t)1 << 20;
    if (!engine->d_rank) BGO_CUDA(cudaMalloc(&engine->d_rank, sizeof(uint32_t) * rank_n));
    if (engine->h_rank.size() != rank_n ||
        memcmp(engine->h_rank.data(), rank_table, sizeof(uint32_t) * rank_n) != 0) {
        engine->h_rank.assign(rank_table, rank_table + rank_n);
        BGO_CUDA(cudaMemcpyAsync(engine->d_rank, engine->h_rank.data(), sizeof(uint32_t) * rank_n,
                                 cudaMemcpyHostToDevice, s));
        engine->h2d_bytes += (int64_t)(sizeof(uint32_t) * rank_n);
    }
    unsigned char *d = engine->d_epi;
    size_t o = 0;
    auto take = [&](size_t b) {
        unsigned char *p = d + o;
        o += b;
        return p;
    };
    EpiParams e{};
    RowInfo *d_rows = (RowInfo *)take(b_rows);
    int32_t *d_list = (int32_t *)take(b_list);
    bgo_input_row *d_in = (bgo_input_row *)take(b_in);
    int64_t *d_off = (int64_t *)take(b_chr);
    int64_t *d_len = (int64_t *)take(b_chr);
    uint32_t *d_rank = engine->d_rank;
    unsigned long long *d_below = (unsigned long long *)take(b_below);
    unsigned long long *d_grp = (unsigned long long *)take(b_grp);
    unsigned int *d_hist = (unsigned int *)take(b_hist);
    int32_t *d_cut = (int32_t *)take(b_cut);
    bgo_record *d_out = (bgo_record *)take(b_out);
    unsigned long long *d_cnt = (unsigned long long *)take(b_cnt);
    int rc = BGO_OK;
    cudaError_t ce = cudaSuccess;
    auto step = [&](cudaError_t x) {
        if (ce == cudaSuccess) ce = x;
    };
    step(cudaMemcpyAsync(d_rows, rows.data(), sizeof(RowInfo) * rows.size(),
                         cudaMemcpyHostToDevice, s));
    if (n_inputs) {
        step(cudaMemcpyAsync(d_list, list.data(), sizeof(int32_t) * (size_t)n_inputs,
                             cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(d_in, inputs, sizeof(bgo_input_row) * (size_t)n_inputs,
                             cudaMemcpyHostToDevice, s));
    }
    step(cudaMemcpyAsync(d_off, chrom_offsets, sizeof(int64_t) * n_chroms, cudaMemcpyHostToDevice, s));
    step(cudaMemcpyAsync(d_len, chrom_lengths, sizeof(int64_t) * n_chroms, cudaMemcpyHostToDevice, s));
    engine->h2d_bytes += (int64_t)(sizeof(RowInfo) * rows.size() +
                                   (sizeof(int32_t) + sizeof(bgo_input_row)) * (size_t)n_inputs +
                                   2 * sizeof(int64_t) * (size_t)n_chroms);
    step(cudaMemsetAsync(d_below, 0, b_below + b_grp + b_hist, s));
    step(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), s));
    e.keys = engine->d_keys;
    e.n_hits = n_hits_host;
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
    e.n_chroms = n_chroms;
    e.rank_table = d_rank;
    e.threshold_rank = threshold_rank;
    e.return_all = return_all ? 1 : 0;
    e.below = d_below;
    e.group_cnt = d_grp;
    e.hist = d_hist;
    e.cut = d_cut;
    e.out = d_out;
    e.cap = capacity;
    e.out_count = d_cnt;
    const int threads = 256;
    const int64_t grid = std::max<int64_t>(
        1, std::min<int64_t>((n_hits_host + threads - 1) / threads, (int64_t)engine->sm_count * 8));
    if (ce == cudaSuccess && n_hits_host > 0) {
        epilogue_kernel<1><<<(unsigned)grid, threads, 0, s>>>(e);
        step(cudaGetLastError());
        if (n_inputs > 0) {
            cut_kernel<<<(unsigned)((n_inputs * 32 + 255) / 256), 256, 0, s>>>(
                d_hist, n_inputs, n_top, e.return_all, d_cut);
            step(cudaGetLastError());
        }
        epilogue_kernel<2><<<(unsigned)grid, threads, 0, s>>>(e);
        step(cudaGetLastError());
        engine->launches += 2 + (n_inputs > 0 ? 1 : 0);
    }
    unsigned long long n_out = 0;
    std::vector<unsigned long long> tmp_b((size_t)n_inputs + 1), tmp_g((size_t)2 * n_rows + 2);
    step(cudaMemcpyAsync(&n_out, d_cnt, sizeof(n_out), cudaMemcpyDeviceToHost, s));
    step(cudaMemcpyAsync(tmp_b.data(), d_below, sizeof(unsigned long long) * (size_t)(n_inputs + 1),
                         cudaMemcpyDeviceToHost, s));
    step(cudaMemcpyAsync(tmp_g.data(), d_grp, sizeof(unsigned long long) * (size_t)(2 * n_rows + 2),
                         cudaMemcpyDeviceToHost, s));
    step(cudaStreamSynchronize(s));
    engine->d2h_bytes += (int64_t)(sizeof(n_out) + sizeof(unsigned long long) *
                                                       (size_t)(n_inputs + 1 + 2 * n_rows + 2));
    if (ce == cudaSuccess && (int64_t)n_out <= capacity && n_out > 0) {
        step(cudaMemcpyAsync(records, d_out, sizeof(bgo_record) * (size_t)n_out,
                             cudaMemcpyDeviceToHost, s));
        step(cudaStreamSynchronize(s));
        engine->d2h_bytes += (int64_t)(sizeof(bgo_record) * n_out);
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "bgo_epilogue_run");
    for (int32_t i = 0; i < n_inputs; ++i) below[i] = (int64_t)tmp_b[(size_t)i];
    for (int32_t i = 0; i < 2 * n_rows; ++i) group_counts[i] = (int64_t)tmp_g[(size_t)i];
    *n_records = (int64_t)n_out;
    return rc;
}
