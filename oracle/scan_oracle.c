/*
 * ORACLE (test infrastructure only): a plain-C restatement of the reference's
 * extensive-mode scan kernel, used as the checker in tests/, by
 * __graft_entry__.smoke() and as the timed CPU baseline in bench.py.  The
 * product never links, loads or calls this file.
 *
 * It follows beguidedoff/cuda_search.py:163-314 (search_chunk_kernel) step by
 * step for one strand array:
 *   - positions pos in [0, total_bp - 26) regardless of PAM length (:211-213);
 *   - 26-bp N-gate over [pos, pos+26) from the little-bit-order N mask
 *     (:228-237); an empty mask disables gating;
 *   - 3' PAM: guide window at pos, PAM at pos+20; 5' PAM: PAM at pos, guide at
 *     pos+plen with the total_bp bounds check (:248-260);
 *   - PAM test per base with the IUPAC allowed-set nibble (:90-98, which the
 *     packed test of :267 is equivalent to for every code);
 *   - 40-bit XOR, (x | x>>1) & 0x5555555555, popcount (:272-275), reject
 *     above max_mismatches (:277);
 *   - N correction: guide-window N positions whose guide base equals
 *     n_encoded add one mismatch each, second reject (:290-308);
 *   - exact per-guide count; hits kept in genome order (the order the
 *     reference's atomic append produces when positions run in order).
 *
 * Hits are returned as 64-bit keys (guide << 40 | pos << 5 | mm), sorted
 * ascending, which is (guide, position) order.  A pass over disjoint position
 * ranges runs in parallel with OpenMP when compiled with -fopenmp.
 *
 * Parity pin: tests/test_oracle_golden.py checks every raw call recorded from
 * the reference into tests/golden/*.npz against this function.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_PAM 6

static inline uint32_t base_at(const uint32_t *packed, int64_t n_words, int64_t p) {
    int64_t w = p >> 4;
    if (w < 0 || w >= n_words) return 0;
    return (packed[w] >> ((p & 15) * 2)) & 3u;
}

static inline uint32_t nbit_at(const uint8_t *mask, int64_t n_bytes, int64_t p) {
    int64_t b = p >> 3;
    if (!mask || b < 0 || b >= n_bytes) return 0;
    return (mask[b] >> (p & 7)) & 1u;
}

static inline int popc64(uint64_t x) {
    int c = 0;
    while (x) { x &= x - 1; ++c; }
    return c;
}

/* 20 bases starting at `start` as the reference's 40-bit LSB-first window. */
static inline uint64_t window40(const uint32_t *packed, int64_t n_words, int64_t start) {
    uint64_t v = 0;
    for (int i = 0; i < 20; ++i) v |= (uint64_t)base_at(packed, n_words, start + i) << (2 * i);
    return v;
}

typedef struct {
    uint64_t *keys;
    int64_t n, cap;
} keybuf;

static int push(keybuf *kb, uint64_t k) {
    if (kb->n == kb->cap) {
        int64_t nc = kb->cap ? kb->cap * 2 : 1024;
        uint64_t *p = (uint64_t *)realloc(kb->keys, (size_t)nc * sizeof(uint64_t));
        if (!p) return -1;
        kb->keys = p;
        kb->cap = nc;
    }
    kb->keys[kb->n++] = k;
    return 0;
}

/* Scan positions [p0, p1) of one strand; append hit keys to kb; add counts. */
static int scan_range(const uint32_t *packed, int64_t n_words, int64_t total_bp,
                      const uint8_t *nmask, int64_t nmask_bytes,
                      const uint64_t *guides, const uint8_t *pam_masks, const uint8_t *pam_lens,
                      const uint8_t *pam_3prime, int32_t n_guides, int32_t max_mm,
                      int32_t n_encoded, int64_t p0, int64_t p1, int64_t *counts, keybuf *kb) {
    for (int64_t pos = p0; pos < p1; ++pos) {
        int need_n = 0;
        if (nmask && nmask_bytes > 0) {
            for (int i = 0; i < 26; ++i) need_n |= (int)nbit_at(nmask, nmask_bytes, pos + i);
        }
        for (int32_t g = 0; g < n_guides; ++g) {
            int plen = pam_lens[g];
            if (plen == 0 || plen > ORACLE_MAX_PAM) continue;
            int64_t guide_start, pam_start;
            if (pam_3prime[g]) {
                guide_start = pos;
                pam_start = pos + 20;
            } else {
                guide_start = pos + plen;
                pam_start = pos;
                if (guide_start + 20 > total_bp || pam_start + plen > total_bp) continue;
            }
            int pam_ok = 1;
            for (int i = 0; i < plen; ++i) {
                uint32_t nuc = base_at(packed, n_words, pam_start + i);
                if (((1u << nuc) & pam_masks[g * ORACLE_MAX_PAM + i]) == 0) { pam_ok = 0; break; }
            }
            if (!pam_ok) continue;
            uint64_t x = window40(packed, n_words, guide_start) ^ guides[g];
            int mm = popc64((x | (x >> 1)) & 0x5555555555ull);
            if (mm > max_mm) continue;
            int mm_final = mm;
            if (need_n) {
                int extra = 0;
                for (int i = 0; i < 20; ++i) {
                    if (nbit_at(nmask, nmask_bytes, guide_start + i) &&
                        ((guides[g] >> (2 * i)) & 3u) == (uint64_t)n_encoded)
                        ++extra;
                }
                mm_final = mm + extra;
                if (mm_final > max_mm) continue;
            }
            counts[g] += 1;
            if (push(kb, ((uint64_t)g << 40) | ((uint64_t)pos << 5) | (uint64_t)mm_final)) return -1;
        }
    }
    return 0;
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

/*
 * Scan one strand.  counts[n_guides] receives the exact per-guide hit count.
 * On success *keys_out points to a malloc'ed array of *n_out sorted keys
 * (free with oracle_free).  n_threads <= 0 uses every OpenMP thread.
 * Returns 0, or -1 on allocation failure.
 */
int oracle_scan_strand(const uint32_t *packed, int64_t n_words, int64_t total_bp,
                       const uint8_t *nmask, int64_t nmask_bytes, const uint64_t *guides,
                       const uint8_t *pam_masks, const uint8_t *pam_lens,
                       const uint8_t *pam_3prime, int32_t n_guides, int32_t max_mm,
                       int32_t n_encoded, int64_t pos_begin, int64_t pos_end, int n_threads,
                       int64_t *counts, uint64_t **keys_out, int64_t *n_out) {
    int64_t valid_end = total_bp - 26;
    if (pos_end > valid_end) pos_end = valid_end;
    if (pos_begin < 0) pos_begin = 0;
    memset(counts, 0, sizeof(int64_t) * (size_t)(n_guides > 0 ? n_guides : 0));
    *keys_out = NULL;
    *n_out = 0;
    if (pos_end <= pos_begin || n_guides <= 0) return 0;
    int nt = 1;
#ifdef _OPENMP
    nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#else
    (void)n_threads;
#endif
    int64_t span = pos_end - pos_begin;
    int64_t n_parts = (int64_t)nt * 8;
    if (n_parts > span) n_parts = span;
    keybuf *bufs = (keybuf *)calloc((size_t)n_parts, sizeof(keybuf));
    int64_t *part_counts = (int64_t *)calloc((size_t)n_parts * (size_t)n_guides, sizeof(int64_t));
    int err = (!bufs || !part_counts);
    if (!err) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) reduction(| : err)
#endif
        for (int64_t part = 0; part < n_parts; ++part) {
            int64_t a = pos_begin + span * part / n_parts;
            int64_t b = pos_begin + span * (part + 1) / n_parts;
            err |= scan_range(packed, n_words, total_bp, nmask, nmask_bytes, guides, pam_masks,
                              pam_lens, pam_3prime, n_guides, max_mm, n_encoded, a, b,
                              part_counts + part * n_guides, &bufs[part]);
        }
    }
    int64_t total = 0;
    if (!err) {
        for (int64_t part = 0; part < n_parts; ++part) {
            total += bufs[part].n;
            for (int32_t g = 0; g < n_guides; ++g) counts[g] += part_counts[part * n_guides + g];
        }
        uint64_t *keys = (uint64_t *)malloc((size_t)(total > 0 ? total : 1) * sizeof(uint64_t));
        if (!keys) {
            err = 1;
        } else {
            int64_t o = 0;
            for (int64_t part = 0; part < n_parts; ++part) {
                if (bufs[part].n) memcpy(keys + o, bufs[part].keys, (size_t)bufs[part].n * 8);
                o += bufs[part].n;
            }
            qsort(keys, (size_t)total, sizeof(uint64_t), cmp_u64);
            *keys_out = keys;
            *n_out = total;
        }
    }
    if (bufs)
        for (int64_t part = 0; part < n_parts; ++part) free(bufs[part].keys);
    free(bufs);
    free(part_counts);
    return err ? -1 : 0;
}

void oracle_free(void *p) { free(p); }

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
