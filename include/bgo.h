/*
 * bgo.h - C ABI of the GB300 (sm_103a) extensive off-target scan.
 *
 * Plain C types only: host pointers, sizes, and `void *stream` standing for a
 * cudaStream_t (NULL = the legacy default stream).  Every function returns an
 * int status (BGO_OK or a negative BGO_ERR_*); the message of the last failure
 * on the calling thread is available from bgo_last_error().
 *
 * Reference interfaces replaced (paths inside ltschmitt/BEguidedOFF):
 *   beguidedoff/cuda_search.py:384-488  search_genome_cuda(...)  -> bgo_search_genome
 *   beguidedoff/cuda_search.py:321-381  device genome / N-mask caches
 *                                       -> bgo_genome_create / bgo_genome_destroy
 *   beguidedoff/cuda_search.py:124-160  encode_pam_packed (host PAM precompile)
 *                                       -> bgo_plan_create (PAM families, guide planes)
 *   beguidedoff/cuda_search.py:163-314  search_chunk_kernel launches
 *                                       -> bgo_scan_launch / bgo_scan_collect
 *
 * Hit keys (uint64, ascending order = (guide, strand, position)):
 *   bits  0..5   mismatches after the N correction
 *   bits  6..37  0-based position in the scanned strand array
 *   bit  38      strand slot (index into the genome list given to the launch)
 *   bits 39..63  guide row index in the plan (input order)
 */
#ifndef BGO_H
#define BGO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BGO_OK 0
#define BGO_ERR_ARG (-1)      /* invalid argument                           */
#define BGO_ERR_CUDA (-2)     /* a CUDA runtime call failed                 */
#define BGO_ERR_OOM (-3)      /* device or host allocation failed           */
#define BGO_ERR_TIMEOUT (-4)  /* a bounded device wait gave up              */
#define BGO_ERR_STATE (-5)    /* call order violated (e.g. collect w/o launch) */

#define BGO_MAX_PAM_LEN 6
#define BGO_GUIDE_LEN 20

#define BGO_KEY_MM(k) ((int)((k) & 63u))
#define BGO_KEY_POS(k) ((int64_t)(((k) >> 6) & 0xFFFFFFFFull))
#define BGO_KEY_STRAND(k) ((int)(((k) >> 38) & 1u))
#define BGO_KEY_GUIDE(k) ((int64_t)((k) >> 39))

typedef struct bgo_genome bgo_genome;
typedef struct bgo_plan bgo_plan;
typedef struct bgo_engine bgo_engine;

/* Library version (major*10000 + minor*100 + patch). */
int bgo_version(void);

/* Copies the last error message of this thread (NUL-terminated, truncated). */
int bgo_last_error(char *buf, size_t len);

/* Number of CUDA devices visible to the process. */
int bgo_device_count(int *n);

/* Page-locked host buffers for fast host<->device copies. */
int bgo_host_alloc(void **ptr, size_t bytes);
int bgo_host_free(void *ptr);

/*
 * Uploads one strand array (the reference .npz layout: 2-bit bases A0 C1 G2 T3,
 * 16 per uint32, base i at bits 2*(i%16) of word i/16) and its N mask
 * (little bit order, bit i = position i; NULL or 0 bytes = no N gating, as the
 * reference does for genomes without N) to `device`, converting it to the
 * device layout (high-bit, low-bit and N planes, 32 positions per word).
 * Replaces the id()-keyed upload caches of beguidedoff/cuda_search.py:321-381.
 * The host buffers are only read during the call.  total_bp < 2^32.
 */
int bgo_genome_create(const uint32_t *packed, int64_t n_words, int64_t total_bp,
                      const uint8_t *n_mask_le, int64_t n_mask_bytes, int device,
                      void *stream, bgo_genome **out);
/*
 * Replaces a strand's contents with new arrays of the same total_bp (and the
 * same N-mask presence), reusing its device buffers: the copies and the
 * conversion are queued on `stream` with no allocation and no host
 * synchronisation.  No reference counterpart: the reference uploads a genome
 * once and keeps it (beguidedoff/finder.py:321-377).
 */
int bgo_genome_upload(bgo_genome *genome, const uint32_t *packed, int64_t n_words,
                      const uint8_t *n_mask_le, int64_t n_mask_bytes, void *stream);
int bgo_genome_destroy(bgo_genome *genome);
/* total_bp, whether an N mask is present, and the device bytes held. */
int bgo_genome_info(const bgo_genome *genome, int64_t *total_bp, int *has_n_mask,
                    int64_t *device_bytes);

/* Engine: per-device workspace (hit buffer, counters) reused across scans.
 * One engine serves one thread / stream at a time. */
int bgo_engine_create(int device, bgo_engine **out);
int bgo_engine_destroy(bgo_engine *engine);

/*
 * Guide plan: one row per scan key, in the reference's kernel-input form
 * (beguidedoff/finder.py:167-177): guide_encoded[i] = 20 bases, 2 bits each,
 * LSB first; pam_masks[i*6 + k] = IUPAC allowed-set nibble (bit0 A .. bit3 T)
 * of PAM position k; pam_lens[i] in 0..6 (0 or >6 = row never matches, as
 * encode_pam_packed leaves its length field 0); pam_3prime[i] 1 = PAM after
 * the guide, 0 = before.  Rows are grouped into PAM families on the device.
 * A plan's device memory (rows, segment indexes) comes from a stream-ordered
 * pool the library keeps per device: creating, rebuilding and destroying
 * plans does not synchronise the device.  bgo_plan_destroy waits for the
 * plan's last use (its creation, the last bgo_scan_launch or graph replay);
 * a caller that ran one plan on several streams at once synchronises the
 * others before destroying it.
 */
int bgo_plan_create(bgo_engine *engine, const uint64_t *guide_encoded, const uint8_t *pam_masks,
                    const uint8_t *pam_lens, const uint8_t *pam_3prime, int32_t n_guides,
                    void *stream, bgo_plan **out);
int bgo_plan_destroy(bgo_plan *plan);
/* Number of PAM families and rows of a plan. */
int bgo_plan_info(const bgo_plan *plan, int32_t *n_families, int32_t *n_guides);

/*
 * Enqueues the scan of `n_strands` (1 or 2) strand arrays against every plan
 * row on `stream`; no host synchronisation.  n_encoded[s] is the 2-bit value
 * an N encodes as on strand s (0 forward, 3 reverse complement).  Positions
 * scanned: [0, total_bp - 26) of each strand, as the reference kernel.
 * mode: 0 = one kernel per PAM family and strand (plain form),
 *       1 = one persistent launch over all families and strands, every guide
 *           compared at every PAM-passing position,
 *       2 = one launch with a segment index (pigeonhole over max_mismatches + 1
 *           segments, bucket lists of guides) for max_mismatches <= 7,
 *       3 = one launch with the segment index stored as guide bitmasks.
 * All modes return the same hits.  Modes 2 and 3 run as mode 1 when their
 * index does not apply (max_mismatches > 7 or an index too large for shared
 * memory).
 */
int bgo_scan_launch(bgo_engine *engine, const bgo_plan *plan, const bgo_genome *const *strands,
                    const int32_t *n_encoded, int32_t n_strands, int32_t max_mismatches,
                    int32_t mode, void *stream);

/*
 * Waits for the last launch of `engine`, then reports the exact number of hits
 * in *n_hits and, when keys != NULL and *n_hits <= capacity, copies all hit
 * keys to `keys` in ascending order.  If *n_hits > capacity nothing is copied;
 * call bgo_scan_launch again after bgo_engine_reserve(engine, *n_hits).
 */
int bgo_scan_collect(bgo_engine *engine, uint64_t *keys, int64_t capacity, int64_t *n_hits,
                     void *stream);

/*
 * Completes the last scan of `engine` (after bgo_scan_launch of the same
 * plan, strands and parameters, on the same stream) so that the hit buffer
 * holds every hit: *n_hits = the exact count.  When the scan overflowed the
 * buffer, the keys that did not fit have marked their 4,096-position granules;
 * the engine grows the buffer (without synchronising the device), keeps the
 * keys of the other granules and scans only the marked granules again (the
 * segment-index and prefiltered forms take a chunk list; the other forms scan
 * everything once more).  The reference's counterpart is the escalating
 * whole-genome re-scan of overflowed guides (beguidedoff/finder.py:568-638,
 * ceiling :100-116); here no hit is ever truncated.
 */
int bgo_scan_complete(bgo_engine *engine, const bgo_plan *plan, const bgo_genome *const *strands,
                      const int32_t *n_encoded, int32_t n_strands, int32_t max_mismatches,
                      int32_t mode, void *stream, int64_t *n_hits);

/* After the last launch completed: number of (PAM-passing position, guide
 * row) pairs whose mismatches were counted.  No reference counterpart: it is
 * the work figure of the roofline. */
int bgo_scan_stats(bgo_engine *engine, int64_t *pairs_evaluated, void *stream);

/*
 * Launch parameters of a plan (scan modes 2 and 3), normally chosen by the
 * autotuner (beguidedoff_gb300/autotune.py).  Zero fields keep the defaults.
 *   chunk_sites   modes 2/3: positions per warp chunk ("tile length"): 1024 or 2048
 *                 (4096 with prefilter)
 *   group_guides  mode 3: guides per mask group ("guides per block"): 32, 64
 *                 or 128; a family larger than this is cut into several groups
 *   ctas_per_sm   cap on resident CTAs per SM for the grid size (0 = the
 *                 occupancy maximum)
 *   split_families  mode 2: one launch per PAM family, each holding only its
 *                 family's index in shared memory (higher occupancy when the
 *                 combined index is large), instead of one launch for all
 *   min_blocks    mode 2: CTAs per SM the kernel is compiled for, 3 (up to 80
 *                 registers per thread) or 4 (up to 64) of 256 threads, or one
 *                 CTA sharing one copy of the index: 1 = 768 threads (24 warps),
 *                 2 = 512 threads (16 warps); 0 = 3.  A form that does not fit
 *                 in shared memory steps down to 1,024-position chunks and to
 *                 fewer warps
 *   tolerance     mode 2: mismatches allowed in a key region, 0 (K + 1 exact
 *                 regions) or 1 (K / 2 + 1 regions, guides also indexed under
 *                 every single-base substitution of their keys)
 *   inline_entries  mode 2: guides of each bucket compared inline before the
 *                 range queue or the walk, 1 or 2; 0 = 1 for tolerance 0 and
 *                 2 for tolerance 1
 *   range_walk    mode 2, tolerance 0 with one inline guide: the rest of a
 *                 bucket walked by its own lane (1) instead of spread over the
 *                 warp (0); tolerance 1 always walks
 *   prefilter     mode 2: 1 = the prefiltered form: per PAM-passing position a
 *                 lossless test on one byte per tolerance-1 region key
 *                 (shared memory) keeps the few positions that can hold a hit,
 *                 which then go through the tolerance-1 segment index in
 *                 global memory; chunks staged by 1-D bulk copies; one
 *                 persistent CTA per SM whose warps claim chunks of each
 *                 family from a counter (all families in one launch unless
 *                 split_families).  chunk_sites 2048 (default) or 4096;
 *                 min_blocks, inline_entries and range_walk do not apply, and
 *                 the index is always built with tolerance 1
 * Changing group_guides rebuilds the mask index at the next launch.  No
 * reference counterpart: the reference fixes 256 threads x 200 Mbp chunks.
 */
typedef struct bgo_tuning {
    int32_t chunk_sites;
    int32_t group_guides;
    int32_t ctas_per_sm;
    int32_t split_families;
    int32_t min_blocks;
    int32_t tolerance;
    int32_t family_form;   /* per-family tuning only: 0 segment index, 1 compare every guide */
    int32_t inline_entries;
    int32_t range_walk;
    int32_t prefilter;
    int32_t reserved[2];
} bgo_tuning;
int bgo_plan_set_tuning(bgo_plan *plan, const bgo_tuning *tuning);

/*
 * Per-family launch parameters for scan mode 2 with split_families: family f
 * gets its own form (segment index, or every guide compared as in mode 1),
 * tolerance, chunk_sites, min_blocks and ctas_per_sm.  Families are numbered
 * in first-seen order of their PAM pattern; bgo_plan_families writes each
 * plan row's family (-1 for rows that never match).  Families without their
 * own setting use the plan's.
 */
int bgo_plan_families(const bgo_plan *plan, int32_t *row_family);
int bgo_plan_set_family_tuning(bgo_plan *plan, int32_t family, const bgo_tuning *tuning);

/*
 * Times the scan: one untimed launch, then `reps` launches each bracketed by
 * CUDA events on `stream`; *ms_best = the fastest.  The autotuner's
 * measurement.  No reference counterpart.
 */
int bgo_scan_time(bgo_engine *engine, const bgo_plan *plan, const bgo_genome *const *strands,
                  const int32_t *n_encoded, int32_t n_strands, int32_t max_mismatches,
                  int32_t mode, int32_t reps, void *stream, double *ms_best);

/*
 * The same scan as bgo_scan_launch, captured once into a CUDA graph and
 * replayed by bgo_graph_launch (each replay resets the engine's counters and
 * rescans; collect with bgo_scan_collect).  Everything that allocates or
 * synchronises (the segment index, kernel attributes) happens at creation.
 * The graph refers to the engine, plan and strands: keep them alive and
 * unchanged while it exists.  After bgo_engine_reserve moved the hit buffer,
 * or after a launch of the plan with another max_mismatches or tolerance
 * rebuilt its index, the next bgo_graph_launch runs one ordinary scan and
 * captures the scan again before it replays.  No reference counterpart: the
 * reference launches one kernel per 200 Mbp chunk.
 */
typedef struct bgo_graph bgo_graph;
int bgo_graph_create(bgo_engine *engine, const bgo_plan *plan, const bgo_genome *const *strands,
                     const int32_t *n_encoded, int32_t n_strands, int32_t max_mismatches,
                     int32_t mode, bgo_graph **out);
int bgo_graph_launch(bgo_graph *graph, void *stream);
int bgo_graph_destroy(bgo_graph *graph);

/*
 * Device epilogue of the engine's last scan: the per-hit work of the
 * reference's host post-processing (beguidedoff/finder.py:193-244, :405-472,
 * :545-566) without a per-hit host loop.  One bgo_input_row per input guide row
 * (the reference's GuideInput after dedup to a plan row).
 *   rank_table[mask]  rank of the exact CCTOP score of each 20-bit mismatch
 *                     mask (bit p-1 = position p) among all distinct scores,
 *                     ascending; 2^20 entries, built on the host.  The
 *                     engine uploads it once and keeps the address: a table
 *                     at the last call's address is taken as unchanged, so
 *                     new contents go in a new buffer;
 *   chrom_rank[c]     rank of chromosome c's name in sorted name order (the
 *                     reference's tie order after the score);
 *   n_top             the reference's top-N rule.
 * A hit's order key is (score rank, chromosome name rank, local report
 * position, strand) packed in 64 bits - the reference's sort order.  Per input
 * row the epilogue keeps every included hit (editable, or any hit when the
 * row's flags ask for all; on-target excluded) among the row's n_top smallest
 * order keys, all of them when the row returns all.  With more than 1024
 * chromosomes the key holds the score rank only and all hits tied at the n_top
 * boundary are kept (the caller sorts them).
 * Outputs (host): below[n_inputs] = the reference's n_offtargets_below_threshold;
 * group_counts[2 * n_plan_rows] = hits per (plan row, strand slot);
 * row_counts[n_inputs] = records kept per input row; *n_records = their sum.
 * The records stay on the device, grouped by input row in row order, until
 * bgo_epilogue_fetch copies them.
 */
typedef struct {
    int32_t plan_row;       /* plan row of this input row's scan key             */
    uint32_t window_mask;   /* bit p-1: window position p is in the edit window  */
    int32_t target_base;    /* 0 = A (ABE), 1 = C (CBE, CGE)                      */
    int32_t ot_chrom;       /* on-target chromosome index, -1 = no exclusion      */
    int64_t ot_local;       /* on-target local leftmost position (0-based)        */
    int32_t ot_strand;      /* on-target strand slot: 0 '+', 1 '-'                */
    int32_t threshold_rank; /* hits with rank <= it count as below the threshold
                               (-1: no threshold)                                 */
    int32_t flags;          /* BGO_ROW_RETURN_ALL: keep every included hit        */
    int32_t pad;
} bgo_input_row;
#define BGO_ROW_RETURN_ALL 1

typedef struct {
    uint64_t key;      /* the hit key */
    uint64_t order;    /* the hit's order key for its input row */
    int32_t input_row; /* input row the hit is kept for */
    uint32_t rank;     /* rank of its CCTOP score */
} bgo_record;

int bgo_epilogue_run(bgo_engine *engine, const bgo_plan *plan, const bgo_genome *const *strands,
                     int32_t n_strands, const bgo_input_row *inputs, int32_t n_inputs,
                     const int64_t *chrom_offsets, const int64_t *chrom_lengths,
                     const int32_t *chrom_rank, int32_t n_chroms, const uint32_t *rank_table,
                     int32_t n_top, int64_t *below, int64_t *group_counts, int64_t *row_counts,
                     int64_t *n_records, void *stream);

/* Copies the records of the last bgo_epilogue_run (capacity >= its n_records). */
int bgo_epilogue_fetch(bgo_engine *engine, bgo_record *records, int64_t capacity, void *stream);

/* A non-blocking CUDA stream on `device` (no implicit synchronisation with
 * the legacy default stream), for callers without a CUDA runtime of their own:
 * one per concurrent engine lets searches overlap on the device. */
int bgo_stream_create(int device, void **stream);
int bgo_stream_destroy(void *stream);

/* Grows the engine's device hit buffer to at least `n_hits` keys. */
int bgo_engine_reserve(bgo_engine *engine, int64_t n_hits);

/*
 * Drop-in for search_genome_cuda (beguidedoff/cuda_search.py:384-488) on one
 * strand: hit_counts[g] = exact number of matches of row g (the reference's
 * counts dict), and rows g of hit_positions / hit_mismatches (row stride
 * results_per_guide) hold its first min(count, results_per_guide) hits in
 * genome order (the reference records them in atomic order).
 */
int bgo_search_genome(bgo_engine *engine, const bgo_genome *strand, const uint64_t *guide_encoded,
                      const uint8_t *pam_masks, const uint8_t *pam_lens,
                      const uint8_t *pam_3prime, int32_t n_guides, int32_t max_mismatches,
                      int32_t n_encoded, int64_t results_per_guide, int64_t *hit_counts,
                      int64_t *hit_positions, int8_t *hit_mismatches, void *stream);

/* Reserved device hit capacity (keys) and number of kernels launched since
 * creation (diagnostics); either pointer may be NULL. */
int bgo_engine_info(const bgo_engine *engine, int64_t *hit_capacity, int64_t *n_launches);

/* Bytes the engine's calls have copied host -> device (plans, segment
 * indexes, epilogue inputs and the score-rank table when it changes) and
 * device -> host (hit counts, keys, epilogue results) since creation.  Strand
 * uploads (bgo_genome_create) are not engine calls and are not counted. */
int bgo_engine_transfer(const bgo_engine *engine, int64_t *h2d_bytes, int64_t *d2h_bytes);

/*
 * The scan for callers that cannot allocate device memory: programs whose own
 * allocator already owns the GPU's memory, and latency-critical loops where a
 * cudaMalloc/cudaFree would synchronise the device.  No counterpart in the
 * reference.  It allocates no device memory: its guide tables, counters
 * and a key buffer live in one static device array of about 8.1 MB that every
 * GPU loading this library reserves until the process exits.  On the host it
 * works in static tables (no heap, small stack); only a failing call
 * allocates, to record its error message.  The first call on a device looks
 * the device array's address up (make it before any stream capture); calls
 * whose work overlaps on the GPU share the array and race, so serialise them
 * (concurrent host threads are serialised by the library).  Limits: n_guides
 * <= BGO_NOALLOC_MAX_GUIDES (larger values return BGO_ERR_ARG), at most
 * BGO_NOALLOC_MAX_HITS hits per call (more return BGO_ERR_OOM with the exact
 * count in *n_hits).  A call whose hits fit the static buffer but not
 * `capacity` returns BGO_OK with the exact count and leaves `keys` untouched:
 * compare *n_hits with capacity.  It runs the plain compare-every-guide scan
 * (scan mode 1), the form that needs no index memory.
 * Inputs and outputs are the caller's: strands as for bgo_scan_launch, guide
 * rows as for bgo_plan_create (host arrays); on success *n_hits is the exact
 * hit count and, when it is <= capacity, `keys` (host) receives all hit keys in
 * ascending order, the same keys bgo_scan_collect returns.
 */
#define BGO_NOALLOC_MAX_GUIDES 2048
#define BGO_NOALLOC_MAX_HITS (1 << 20)
int bgo_scan_noalloc(const bgo_genome *const *strands, const int32_t *n_encoded,
                     int32_t n_strands, const uint64_t *guide_encoded, const uint8_t *pam_masks,
                     const uint8_t *pam_lens, const uint8_t *pam_3prime, int32_t n_guides,
                     int32_t max_mismatches, uint64_t *keys, int64_t capacity, int64_t *n_hits,
                     void *stream);

/*
 * FASTA sequence bytes (all chromosomes concatenated, in file order) -> the
 * reference's .npz arrays on the device, as beguidedoff/genome_converter.py
 * :15-108 writes them: fwd_out ceil(total/16) words; rc_out (optional) the
 * per-chromosome reverse complement in the same layout; n_mask_big_out
 * (optional) ceil(total/8) bytes, N/n positions, np.packbits bit order.  Only
 * A/C/G/T (either case) have non-zero codes.
 */
int bgo_encode_genome(const uint8_t *seq, const int64_t *chrom_lengths, int32_t n_chroms,
                      int device, uint32_t *fwd_out, uint32_t *rc_out, uint8_t *n_mask_big_out);


#ifdef __cplusplus
}
#endif

#endif /* BGO_H */
