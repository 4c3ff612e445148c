// k_gather_df.cu -- dispatch of the fused gather in double-float arithmetic (ComplexF64
// data); the kernels are instantiated per value mode in k_gather_df_{real,phased,complex}.cu.
#include "k_gather.cuh"

namespace qob {
namespace gather {
extern template void dispatch_beta<DF, kReal, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<DF, kReal, false>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<DF, kPhased, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<DF, kComplex, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<DF, kComplex, false>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
template void dispatch<DF>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
}  // namespace gather
}  // namespace qob
