// 4,096-position chunk forms of the prefiltered segment-index kernel with the
// survivor index in global memory (a separate translation unit so that the
// forms compile in parallel).
#include "bgo_filter_kernel.cuh"

namespace bgo {

int launch_filter_4k_g(const ScanParams &p, const FilterArgs &fa, int sm_count, cudaStream_t s) {
    return launch_filter_ch<4096, 0>(p, fa, sm_count, s);
}

}  // namespace bgo
