// Segment-indexed scan (scan mode 2) with tolerance 1 and one inline guide
// per bucket, the rest walked by its lane: for families with few guides,
// whose substitution-expanded buckets are mostly empty, a second inline
// compare costs more than the rare walk it saves.  Instantiated in its own
// translation unit so that the forms compile in parallel.
#include "bgo_seed_kernel.cuh"

namespace bgo {

int launch_seed_t1i1(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                     int min_blocks, int ctas_per_sm, cudaStream_t s) {
    return launch_form<1, 1, 1>(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
}

}  // namespace bgo
