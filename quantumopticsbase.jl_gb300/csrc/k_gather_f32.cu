// k_gather_f32.cu -- dispatch of the fused gather for float; the kernels are
// instantiated per value mode in k_gather_f32_{real,phased,complex}.cu.
#include "k_gather.cuh"

namespace qob {
namespace gather {
extern template void dispatch_beta<float, kReal, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<float, kReal, false>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<float, kPhased, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<float, kComplex, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<float, kComplex, false>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
template void dispatch<float>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
}  // namespace gather
}  // namespace qob
