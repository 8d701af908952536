// 2,048-position chunk forms of the prefiltered segment-index kernel with the
// survivor index in global memory (a separate translation unit so that the
// forms compile in parallel).
#include "bgo_filter_kernel.cuh"

namespace bgo {

int launch_filter_2k_g(const ScanParams &p, const FilterArgs &fa, int sm_count, cudaStream_t s) {
    return launch_filter_ch<2048, 0>(p, fa, sm_count, s);
}

}  // namespace bgo
