// Segment-indexed scan (scan mode 2) with tolerance 1: K / 2 + 1 key regions,
// each guide indexed under its key and every single-base substitution of it,
// so a position needs fewer lookups (3 instead of 6 at K = 5).  Buckets compare
// two guides inline (they rarely hold more).  Instantiated apart from the
// tolerance-0 forms so that they compile in parallel.
#include "bgo_seed_kernel.cuh"

namespace bgo {

int launch_seed_t1(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                   int min_blocks, int ctas_per_sm, cudaStream_t s) {
    return launch_form<1, 2, 1>(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
}

}  // namespace bgo
