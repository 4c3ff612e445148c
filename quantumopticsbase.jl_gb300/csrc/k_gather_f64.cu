// k_gather_f64.cu -- dispatch of the fused gather for double; the kernels are
// instantiated per value mode in k_gather_f64_{real,phased,complex}.cu.
#include "k_gather.cuh"

namespace qob {
namespace gather {
extern template void dispatch_beta<double, kReal, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<double, kReal, false>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<double, kPhased, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<double, kComplex, true>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch_beta<double, kComplex, false>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
template void dispatch<double>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t, void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
}  // namespace gather
}  // namespace qob
