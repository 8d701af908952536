// 4,096-position chunk forms of the prefiltered segment-index kernel (a
// separate translation unit so that the forms compile in parallel).
#include "bgo_filter_kernel.cuh"

namespace bgo {

int launch_filter_4k(const ScanParams &p, const FilterArgs &fa, int sm_count, cudaStream_t s) {
    return launch_filter_ch<4096>(p, fa, sm_count, s);
}

}  // namespace bgo
