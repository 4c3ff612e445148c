// k_gather.cu -- the fused LazySum application kernel.
//
// One thread owns one output index J (and a tile of TC columns / kets).  It
// accumulates, in registers, the merged diagonal times x[J] plus every group's
// stored entries of its local row times the gathered x[base + coloff], then
// writes y[J] = alpha * acc + beta * y[J] once.  This replaces the reference's
// one pass per term over `result` (src/operators_lazysum.jl:189-200) and the
// recursive per-nonzero gather (src/operators_lazytensor.jl:652-685): the
// state is read once per entry from L1/L2 instead of once per term from
// memory, and y is read and written once.
//
// FP64 keeps the reference's arithmetic type; with real merged values (all
// the Hamiltonians built from number/ladder/Pauli factors with real
// coefficients) each stored entry costs two DFMA per column.  FP32 mode adds
// Kahan compensation across the accumulated contributions.
#include <cuda_runtime.h>

#include "qob_internal.h"

namespace qob {

namespace {

__device__ __forceinline__ uint32_t fdiv(uint32_t n, uint32_t d, uint64_t M) {
  return d == 1u ? n : (uint32_t)__umul64hi(M, (uint64_t)n);
}
__device__ __forceinline__ uint32_t fmodu(uint32_t n, uint32_t d, uint64_t M) {
  uint64_t low = M * (uint64_t)n;
  return (uint32_t)__umul64hi(low, (uint64_t)d);
}

template <typename R>
struct Cx;
template <>
struct Cx<double> {
  using T = double2;
};
template <>
struct Cx<float> {
  using T = float2;
};

template <typename R, bool REALV>
struct Val {
  using T = typename Cx<R>::T;
};
template <>
struct Val<double, true> {
  using T = double;
};
template <>
struct Val<float, true> {
  using T = float;
};

// FP64 accumulator: plain fused multiply-adds.
struct AccD {
  double re, im;
  __device__ void zero() { re = im = 0.0; }
  __device__ void mac(double v, double2 x) {
    re = fma(v, x.x, re);
    im = fma(v, x.y, im);
  }
  __device__ void mac(double2 v, double2 x) {
    re = fma(v.x, x.x, re);
    re = fma(-v.y, x.y, re);
    im = fma(v.x, x.y, im);
    im = fma(v.y, x.x, im);
  }
  __device__ double2 total() const { return make_double2(re, im); }
};

// FP32 accumulator with Kahan compensation (Kahan 1965): c carries the
// low-order part lost by each addition.
struct AccF {
  float re, im, cre, cim;
  __device__ void zero() { re = im = cre = cim = 0.f; }
  __device__ void add(float tr, float ti) {
    float yr = tr - cre;
    float sr = re + yr;
    cre = (sr - re) - yr;
    re = sr;
    float yi = ti - cim;
    float si = im + yi;
    cim = (si - im) - yi;
    im = si;
  }
  __device__ void mac(float v, float2 x) { add(v * x.x, v * x.y); }
  __device__ void mac(float2 v, float2 x) {
    add(__fmaf_rn(v.x, x.x, -v.y * x.y), __fmaf_rn(v.x, x.y, v.y * x.x));
  }
  __device__ float2 total() const { return make_float2(re - cre, im - cim); }
};

template <typename R>
struct AccOf;
template <>
struct AccOf<double> {
  using T = AccD;
};
template <>
struct AccOf<float> {
  using T = AccF;
};

__device__ __forceinline__ double2 ld(const double2* p) { return __ldg(p); }
__device__ __forceinline__ float2 ld(const float2* p) { return __ldg(p); }

// y = alpha * acc + beta * y with the reference's beta semantics:
// BMODE 0: beta == 0 (y is not read), 1: beta == 1, 2: general.
template <int BMODE>
__device__ __forceinline__ void combine(double2* yp, double2 a, double2 alpha, double2 beta) {
  double re = alpha.x * a.x - alpha.y * a.y;
  double im = alpha.x * a.y + alpha.y * a.x;
  if (BMODE == 1) {
    double2 o = *yp;
    re += o.x;
    im += o.y;
  } else if (BMODE == 2) {
    double2 o = *yp;
    re = fma(beta.x, o.x, fma(-beta.y, o.y, re));
    im = fma(beta.x, o.y, fma(beta.y, o.x, im));
  }
  *yp = make_double2(re, im);
}
template <int BMODE>
__device__ __forceinline__ void combine(float2* yp, float2 a, double2 alpha_d, double2 beta_d) {
  const float ar = (float)alpha_d.x, ai = (float)alpha_d.y;
  float re = ar * a.x - ai * a.y;
  float im = ar * a.y + ai * a.x;
  if (BMODE == 1) {
    float2 o = *yp;
    re += o.x;
    im += o.y;
  } else if (BMODE == 2) {
    const float br = (float)beta_d.x, bi = (float)beta_d.y;
    float2 o = *yp;
    re = __fmaf_rn(br, o.x, __fmaf_rn(-bi, o.y, re));
    im = __fmaf_rn(br, o.y, __fmaf_rn(bi, o.x, im));
  }
  *yp = make_float2(re, im);
}

__device__ __forceinline__ void load_groups(GGroup* sg, const GGroup* g, int n) {
  const uint64_t* src = reinterpret_cast<const uint64_t*>(g);
  uint64_t* dst = reinterpret_cast<uint64_t*>(sg);
  const int words = n * (int)(sizeof(GGroup) / 8);
  for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

// Local row and input base offset of output index J in group G.
template <bool SQUARE>
__device__ __forceinline__ bool group_row(const GGroup& G, const SiteTable& st, uint32_t J,
                                          uint32_t& r, int64_t& base) {
  r = 0;
  uint32_t sub = 0;
#pragma unroll
  for (int b = 0; b < kMaxBlocks; ++b) {
    if (b < G.nblk) {
      uint32_t q = fdiv(J, G.div[b], G.mdiv[b]);
      uint32_t d = fmodu(q, G.mod[b], G.mmod[b]);
      r += d * G.lstride[b];
      sub += d * G.div[b];
    }
  }
  if (SQUARE) {
    base = (int64_t)(J - sub);
    return true;
  }
  // non-square basis: identity (truncated) on the subsystems outside the support
  int64_t bs = 0;
  for (int s = 0; s < st.nsites; ++s) {
    const bool in_sup = s < 32 ? ((uint32_t)G.support_lo >> s) & 1u : (G.support_hi >> (s - 32)) & 1u;
    if (in_sup) continue;
    uint32_t js = fmodu(fdiv(J, st.sout[s], st.msout[s]), st.dout[s], st.mdout[s]);
    if (js >= st.din[s]) return false;
    bs += (int64_t)js * st.sin[s];
  }
  base = bs;
  return true;
}

template <typename R, bool REALV, bool SQUARE, int TC, int BMODE>
__global__ void __launch_bounds__(256) k_gather_j(GatherView g, SiteTable st,
                                                  const typename Cx<R>::T* __restrict__ x, int64_t xes,
                                                  int64_t xcs, typename Cx<R>::T* __restrict__ y,
                                                  int64_t yes, int64_t ycs, int ncols, double2 alpha,
                                                  double2 beta) {
  using CT = typename Cx<R>::T;
  using VT = typename Val<R, REALV>::T;
  using AT = typename AccOf<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GGroup* sg = reinterpret_cast<GGroup*>(smem_raw);
  load_groups(sg, g.groups, g.ngroups);

  const int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (J >= g.m) return;
  const int c0 = blockIdx.y * TC;
  const int nt = min(TC, ncols - c0);
  const CT* xb = x + (int64_t)c0 * xcs;
  const VT* vals = static_cast<const VT*>(g.vals);

  AT acc[TC];
#pragma unroll
  for (int t = 0; t < TC; ++t) acc[t].zero();

  if (g.has_diag) {
    const VT d = static_cast<const VT*>(g.diag)[J];
#pragma unroll
    for (int t = 0; t < TC; ++t)
      if (t < nt) acc[t].mac(d, ld(xb + J * xes + t * xcs));
  }
  for (int gi = 0; gi < g.ngroups; ++gi) {
    const GGroup& G = sg[gi];
    uint32_t r;
    int64_t base;
    if (!group_row<SQUARE>(G, st, (uint32_t)J, r, base)) continue;
    const int p0 = __ldg(g.rowptr + G.rowptr_off + r);
    const int p1 = __ldg(g.rowptr + G.rowptr_off + r + 1);
    for (int p = p0; p < p1; ++p) {
      const int64_t K = base + __ldg(g.coloff + p);
      const VT v = vals[p];
      const CT* xp = xb + K * xes;
#pragma unroll
      for (int t = 0; t < TC; ++t)
        if (t < nt) acc[t].mac(v, ld(xp + t * xcs));
    }
  }
  CT* yb = y + J * yes + (int64_t)c0 * ycs;
#pragma unroll
  for (int t = 0; t < TC; ++t)
    if (t < nt) combine<BMODE>(yb + t * ycs, acc[t].total(), alpha, beta);
}

// Rows-of-a-matrix form (Operator * op from the right with several rows): the
// vectors are the rows, contiguous across threads; all threads of a block share
// one output index J, so the group arithmetic is uniform.
template <typename R, bool REALV, bool SQUARE, int BMODE>
__global__ void __launch_bounds__(256) k_gather_c(GatherView g, SiteTable st,
                                                  const typename Cx<R>::T* __restrict__ x, int64_t xes,
                                                  int64_t xcs, typename Cx<R>::T* __restrict__ y,
                                                  int64_t yes, int64_t ycs, int ncols, double2 alpha,
                                                  double2 beta) {
  using CT = typename Cx<R>::T;
  using VT = typename Val<R, REALV>::T;
  using AT = typename AccOf<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GGroup* sg = reinterpret_cast<GGroup*>(smem_raw);
  load_groups(sg, g.groups, g.ngroups);

  const int64_t J = blockIdx.x;
  const int64_t c = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  const CT* xb = x + c * xcs;
  const VT* vals = static_cast<const VT*>(g.vals);
  AT acc;
  acc.zero();
  if (g.has_diag) acc.mac(static_cast<const VT*>(g.diag)[J], ld(xb + J * xes));
  for (int gi = 0; gi < g.ngroups; ++gi) {
    const GGroup& G = sg[gi];
    uint32_t r;
    int64_t base;
    if (!group_row<SQUARE>(G, st, (uint32_t)J, r, base)) continue;
    const int p0 = __ldg(g.rowptr + G.rowptr_off + r);
    const int p1 = __ldg(g.rowptr + G.rowptr_off + r + 1);
    for (int p = p0; p < p1; ++p) acc.mac(vals[p], ld(xb + (base + __ldg(g.coloff + p)) * xes));
  }
  combine<BMODE>(y + J * yes + c * ycs, acc.total(), alpha, beta);
}

// Merged diagonal: diag[J] = sum over groups of their local diagonal table.
template <typename R, bool REALV>
__global__ void k_build_diag(int64_t m, int ndg, const GGroup* __restrict__ dg,
                             const double2* __restrict__ dtab, void* diag) {
  const int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (J >= m) return;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < ndg; ++k) {
    const GGroup& G = dg[k];
    uint32_t r = 0;
    for (int b = 0; b < G.nblk; ++b) {
      uint32_t q = fdiv((uint32_t)J, G.div[b], G.mdiv[b]);
      r += fmodu(q, G.mod[b], G.mmod[b]) * G.lstride[b];
    }
    double2 v = dtab[G.rowptr_off + r];
    re += v.x;
    im += v.y;
  }
  using VT = typename Val<R, REALV>::T;
  VT* out = static_cast<VT*>(diag);
  if constexpr (REALV) {
    out[J] = (R)re;
  } else {
    typename Cx<R>::T o;
    o.x = (R)re;
    o.y = (R)im;
    out[J] = o;
  }
}

constexpr int kGroupsPerLaunch = 320;  // 320 * sizeof(GGroup) <= 48 KB of shared memory

template <typename R, bool REALV, bool SQUARE, int BMODE>
void dispatch_tc(const GatherView& v, const SiteTable& st, const void* x, int64_t xes, int64_t xcs,
                 void* y, int64_t yes, int64_t ycs, int64_t ncols, double2 a, double2 b,
                 cudaStream_t s) {
  using CT = typename Cx<R>::T;
  const size_t smem = (size_t)v.ngroups * sizeof(GGroup);
  if (xes == 1 || ncols == 1) {
    const int threads = 256;
    const unsigned gx = (unsigned)((v.m + threads - 1) / threads);
#define QOB_LAUNCH_J(TC_)                                                                        \
  k_gather_j<R, REALV, SQUARE, TC_, BMODE><<<dim3(gx, (unsigned)((ncols + TC_ - 1) / TC_)),    \
                                             threads, smem, s>>>(v, st, (const CT*)x, xes, xcs,  \
                                                                 (CT*)y, yes, ycs, (int)ncols, a, \
                                                                 b)
    if (ncols >= 8)
      QOB_LAUNCH_J(8);
    else if (ncols >= 4)
      QOB_LAUNCH_J(4);
    else if (ncols >= 2)
      QOB_LAUNCH_J(2);
    else
      QOB_LAUNCH_J(1);
#undef QOB_LAUNCH_J
  } else {
    const int threads = ncols >= 256 ? 256 : (int)((ncols + 31) / 32 * 32);
    dim3 grid((unsigned)v.m, (unsigned)((ncols + threads - 1) / threads));
    k_gather_c<R, REALV, SQUARE, BMODE><<<grid, threads, smem, s>>>(
        v, st, (const CT*)x, xes, xcs, (CT*)y, yes, ycs, (int)ncols, a, b);
  }
}

template <typename R, bool REALV, bool SQUARE>
void dispatch_beta(const GatherView& v, const SiteTable& st, const void* x, int64_t xes,
                   int64_t xcs, void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha,
                   c128 beta, cudaStream_t s) {
  double2 a = make_double2(alpha.re, alpha.im), b = make_double2(beta.re, beta.im);
  if (beta.re == 0.0 && beta.im == 0.0)
    dispatch_tc<R, REALV, SQUARE, 0>(v, st, x, xes, xcs, y, yes, ycs, ncols, a, b, s);
  else if (beta.re == 1.0 && beta.im == 0.0)
    dispatch_tc<R, REALV, SQUARE, 1>(v, st, x, xes, xcs, y, yes, ycs, ncols, a, b, s);
  else
    dispatch_tc<R, REALV, SQUARE, 2>(v, st, x, xes, xcs, y, yes, ycs, ncols, a, b, s);
}

template <typename R>
void dispatch_kind(const GatherView& v, const SiteTable& st, const void* x, int64_t xes,
                   int64_t xcs, void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha,
                   c128 beta, cudaStream_t s) {
  if (v.real_vals) {
    if (v.square)
      dispatch_beta<R, true, true>(v, st, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
    else
      dispatch_beta<R, true, false>(v, st, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
  } else {
    if (v.square)
      dispatch_beta<R, false, true>(v, st, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
    else
      dispatch_beta<R, false, false>(v, st, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
  }
}

}  // namespace

void launch_gather(const GatherPlan& g, int precision, const void* x, int64_t xes, int64_t xcs,
                   void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha, c128 beta,
                   cudaStream_t s) {
  GatherView v = g.view();
  // groups beyond one launch's shared-memory budget go in further launches
  // that accumulate into y (beta = 1, no diagonal)
  int g0 = 0;
  bool first = true;
  do {
    GatherView c = v;
    c.groups = v.groups + g0;
    c.ngroups = v.ngroups - g0 > kGroupsPerLaunch ? kGroupsPerLaunch : v.ngroups - g0;
    c.has_diag = first ? v.has_diag : 0;
    const c128 b = first ? beta : c128{1.0, 0.0};
    if (precision == QOB_C128)
      dispatch_kind<double>(c, g.sites, x, xes, xcs, y, yes, ycs, ncols, alpha, b, s);
    else
      dispatch_kind<float>(c, g.sites, x, xes, xcs, y, yes, ycs, ncols, alpha, b, s);
    QOB_LAUNCHED();
    g0 += c.ngroups;
    first = false;
  } while (g0 < v.ngroups);
}

void launch_build_diag(const GatherPlan& g, cudaStream_t s) {
  const int threads = 256;
  const unsigned blocks = (unsigned)((g.m + threads - 1) / threads);
  const GGroup* dg = (const GGroup*)g.dgroups.p;
  const double2* dt = (const double2*)g.dvals.p;
  if (g.precision == QOB_C128) {
    if (g.real_vals)
      k_build_diag<double, true><<<blocks, threads, 0, s>>>(g.m, g.ndgroups, dg, dt, g.diag.p);
    else
      k_build_diag<double, false><<<blocks, threads, 0, s>>>(g.m, g.ndgroups, dg, dt, g.diag.p);
  } else {
    if (g.real_vals)
      k_build_diag<float, true><<<blocks, threads, 0, s>>>(g.m, g.ndgroups, dg, dt, g.diag.p);
    else
      k_build_diag<float, false><<<blocks, threads, 0, s>>>(g.m, g.ndgroups, dg, dt, g.diag.p);
  }
  QOB_LAUNCHED();
}

}  // namespace qob
