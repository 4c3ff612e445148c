// k_gather_f32.cu -- the fused gather kernels instantiated for float (one
// translation unit per precision so the two compile in parallel).
#include "k_gather.cuh"

namespace qob {
namespace gather {
template void dispatch<float>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*,
                           int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
}  // namespace gather
}  // namespace qob
