// k_gather_df_real.cu -- the fused gather kernels in double-float arithmetic with real stored values
// (one translation unit per precision and value mode so they compile in parallel).
#include "k_gather.cuh"

namespace qob {
namespace gather {
template void dispatch_beta<DF, kReal, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
template void dispatch_beta<DF, kReal, false>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
}  // namespace gather
}  // namespace qob
