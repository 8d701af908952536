// Segment-indexed scan (scan mode 2), tolerance 0 with two guides of every
// bucket compared inline: fewer trips through the range queue when buckets
// often hold two guides.  Instantiated apart from the other forms so that they
// compile in parallel.
#include "bgo_seed_kernel.cuh"

namespace bgo {

int launch_seed_t0i2(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                     int min_blocks, int ctas_per_sm, cudaStream_t s) {
    return launch_form<0, 2, 0>(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
}

}  // namespace bgo
