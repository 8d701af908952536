/*
 * Tools library of the benchmark and the tests (libbgo_tools.so, built beside
 * libbgo.so by beguidedoff_gb300/build.py and linked against it): seeded
 * synthetic genomes and the integer-pipe throughput probe.  Nothing here is
 * on the search path, and the reference has none of it.  Status codes and
 * bgo_last_error are libbgo's (include/bgo.h).
 */
#ifndef BGO_TOOLS_H
#define BGO_TOOLS_H

#include "bgo.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Seeded synthetic genome in the reference .npz layout (what
 * beguidedoff/genome_converter.py:15-108 writes for the equivalent FASTA):
 * chromosomes of the given lengths concatenated, bases drawn per position from
 * cumulative byte thresholds (A below t[0], C below t[1], G below t[2], else T),
 * N in the sorted disjoint half-open blocks [n_starts[i], n_ends[i]).
 * Outputs (host): fwd_out / rc_out ceil(total/16) words, n_mask_big_out
 * ceil(total/8) bytes in np.packbits (big) bit order.  No reference
 * counterpart: it stands in for the real assemblies the benchmarks used.
 */
int bgo_synth_genome(uint64_t seed, const int64_t *chrom_lengths, int32_t n_chroms,
                     const int64_t *n_starts, const int64_t *n_ends, int64_t n_blocks,
                     const uint8_t *thresholds, int device, uint32_t *fwd_out, uint32_t *rc_out,
                     uint8_t *n_mask_big_out);

/*
 * Repeat families inserted by bgo_synth_genome_repeats: the genome is cut
 * into n_copies equal regions; region r holds one copy of a seeded family at a
 * seeded offset and orientation, each base substituted with probability
 * divergence_65536 / 65536.  Families are uniform random ACGT of family_len bp.
 */
typedef struct bgo_repeat_spec {
    int32_t n_families;
    int32_t family_len;
    int64_t n_copies;
    uint32_t divergence_65536;
    uint32_t reserved;
    uint64_t seed;
} bgo_repeat_spec;

/*
 * bgo_synth_genome with repeat families (the hit-dense workload).
 * families_out receives n_families * family_len base codes (0-3 = ACGT).
 */
int bgo_synth_genome_repeats(uint64_t seed, const int64_t *chrom_lengths, int32_t n_chroms,
                             const int64_t *n_starts, const int64_t *n_ends, int64_t n_blocks,
                             const uint8_t *thresholds, const bgo_repeat_spec *repeats,
                             uint8_t *families_out, int device, uint32_t *fwd_out,
                             uint32_t *rc_out, uint8_t *n_mask_big_out);

/*
 * Measured throughput (Gop/s) of one integer instruction on `device`:
 * op 0 = LOP3, 1 = POPC, 2 = 32-bit add.  Independent chains, 8 CTAs of 256
 * threads per SM, best of 3 timed launches.  No reference counterpart: it is
 * the roofline denominator of the scan kernels.
 */
int bgo_probe_int_throughput(int device, int op, double *gops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* BGO_TOOLS_H */
