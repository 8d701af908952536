// Segment-indexed scan (scan mode 2), tolerance 0 with one inline guide per
// bucket and the leftover entries of larger buckets walked by their own lane
// instead of the warp range queue (cheaper when larger buckets are rare).
// Instantiated apart from the other forms so that they compile in parallel.
#include "bgo_seed_kernel.cuh"

namespace bgo {

int launch_seed_t0walk(const ScanParams &p, const SeedArgs &sa, int sm_count, int chunk_sites,
                       int min_blocks, int ctas_per_sm, cudaStream_t s) {
    return launch_form<0, 1, 1>(p, sa, sm_count, chunk_sites, min_blocks, ctas_per_sm, s);
}

}  // namespace bgo
