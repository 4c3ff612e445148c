// k_gather.cu -- host entry of the fused LazySum gather (the kernels are in
// k_gather.cuh, instantiated per precision in k_gather_f64.cu / k_gather_f32.cu)
// and the merged-diagonal builder.
#include <cuda_runtime.h>

#include <type_traits>

#include "k_gather.cuh"

namespace qob {

namespace gather {
// explicit instantiations live in k_gather_f64.cu and k_gather_f32.cu
extern template void dispatch<double>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t,
                                      void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch<float>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t,
                                     void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
extern template void dispatch<DF>(const GatherView&, const SiteTable&, int, const void*, int64_t, int64_t,
                                  void*, int64_t, int64_t, int64_t, c128, c128, cudaStream_t);
}  // namespace gather

namespace {

constexpr int kGroupsPerLaunch = 256;  // 256 * sizeof(GGroup) = 44 KB of shared memory

// (hi, lo) float pair of a double: hi rounded to nearest, lo = the rest (not hot)
__device__ __forceinline__ float2 split_rn(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

// Merged diagonal: diag[J] = sum over groups of their local diagonal table.
template <typename R, bool REALV>
__global__ void k_build_diag(int64_t m, int ndg, const GGroup* __restrict__ dg,
                             const double2* __restrict__ dtab, void* diag) {
  const int64_t J = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (J >= m) return;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < ndg; ++k) {
    uint32_t r, sub;
    gather::local_row(dg[k], (uint32_t)J, r, sub);
    double2 v = dtab[dg[k].rowptr_off + r];
    re += v.x;
    im += v.y;
  }
  using VT = typename gather::Val<R, REALV>::T;
  VT* out = static_cast<VT*>(diag);
  if constexpr (std::is_same<R, gather::DF>::value) {
    if constexpr (REALV) {
      out[J] = split_rn(re);
    } else {
      const float2 a = split_rn(re), b = split_rn(im);
      out[J] = make_float4(a.x, a.y, b.x, b.y);
    }
  } else if constexpr (REALV) {
    out[J] = (R)re;
  } else {
    typename gather::Cx<R>::T o;
    o.x = (R)re;
    o.y = (R)im;
    out[J] = o;
  }
}

// Split of the input vectors into double-float quadruples (re hi, re lo, im
// hi, im lo), element e of vector c at e * es + c * cs in both arrays.  Each
// thread moves kSplitPer elements a block apart, their loads issued together.
constexpr int kSplitPer = 4;
__global__ void __launch_bounds__(256) k_ff_split(const double2* __restrict__ x, int64_t n, int64_t ncols,
                                                  int64_t es, int64_t cs, float4* __restrict__ out) {
  const int64_t total = n * ncols;
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x * kSplitPer + threadIdx.x;
  int64_t o[kSplitPer];
  double2 v[kSplitPer];
#pragma unroll
  for (int k = 0; k < kSplitPer; ++k) {
    const int64_t i = i0 + (int64_t)k * blockDim.x;
    o[k] = -1;
    if (i < total) {
      if (es == 1 && cs == n) {  // contiguous columns (kets): offset = index, no division
        o[k] = i;
      } else {
        int64_t c, e;
        udivmod(i, n, c, e);
        o[k] = e * es + c * cs;
      }
      v[k] = __ldg(x + o[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < kSplitPer; ++k)
    if (o[k] >= 0) {
      const float2 a = gather::ff_split(v[k].x), b = gather::ff_split(v[k].y);
      out[o[k]] = make_float4(a.x, a.y, b.x, b.y);
    }
}

// Stored values re-evaluated from the root LazySum's factors: one thread per
// merged slot, value = sum over its contributions of (f[top] * inner) * pv,
// summed in the order of the host record (the order of the LazySum's terms).
// The factor row is f_base + (2 * *step + off) * nf when `step` (a device
// counter of RK4 steps) is given, else f_base: recorded graphs read the row of
// the current step.
template <typename R, bool REALV>
__global__ void __launch_bounds__(256) k_td_values(int nslots, const TdSlot* __restrict__ slots,
                                                   const TdContrib* __restrict__ contrib,
                                                   const TdTerm* __restrict__ terms,
                                                   const double2* __restrict__ f_base,
                                                   const long long* __restrict__ step, long long off,
                                                   long long nf, void* vals, void* ell,
                                                   double2* __restrict__ dtab) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  const double2* f = step ? f_base + (2 * *step + off) * nf : f_base;
  const TdSlot sl = slots[s];
  double re = 0.0, im = 0.0;
  for (int k = 0; k < sl.count; ++k) {
    const TdContrib& c = contrib[sl.first + k];
    const TdTerm& t = terms[c.term];
    double cr = t.inner[0], ci = t.inner[1];
    if (t.top >= 0) {
      const double2 a = f[t.top];
      const double r2 = __dsub_rn(__dmul_rn(a.x, t.inner[0]), __dmul_rn(a.y, t.inner[1]));
      const double i2 = __dadd_rn(__dmul_rn(a.x, t.inner[1]), __dmul_rn(a.y, t.inner[0]));
      cr = r2;
      ci = i2;
    }
    re = __dadd_rn(re, __dsub_rn(__dmul_rn(cr, c.pv[0]), __dmul_rn(ci, c.pv[1])));
    im = __dadd_rn(im, __dadd_rn(__dmul_rn(cr, c.pv[1]), __dmul_rn(ci, c.pv[0])));
  }
  if (sl.dst_diag >= 0) dtab[sl.dst_diag] = make_double2(re, im);
  const double sv = sl.part ? im : re;  // the stored number of a real-storage plan
  if constexpr (std::is_same<R, gather::DF>::value) {
    const float2 a = split_rn(REALV ? sv : re), b = split_rn(im);
    if (sl.dst_val >= 0) {
      if constexpr (REALV)
        static_cast<float2*>(vals)[sl.dst_val] = a;
      else
        static_cast<float4*>(vals)[sl.dst_val] = make_float4(a.x, a.y, b.x, b.y);
    }
    if (sl.dst_ell >= 0) {
      if constexpr (REALV) {
        EllDF& e = static_cast<EllDF*>(ell)[sl.dst_ell];
        e.v[0] = a.x;
        e.v[1] = a.y;
      } else {
        EllZF& e = static_cast<EllZF*>(ell)[sl.dst_ell];
        e.v[0] = a.x;
        e.v[1] = a.y;
        e.v[2] = b.x;
        e.v[3] = b.y;
      }
    }
  } else {
    if (sl.dst_val >= 0) {
      if constexpr (REALV) {
        static_cast<R*>(vals)[sl.dst_val] = (R)sv;
      } else {
        typename gather::Cx<R>::T o;
        o.x = (R)re;
        o.y = (R)im;
        static_cast<typename gather::Cx<R>::T*>(vals)[sl.dst_val] = o;
      }
    }
    if (sl.dst_ell >= 0) {
      if constexpr (sizeof(R) == 8 && REALV) {
        static_cast<EllD*>(ell)[sl.dst_ell].v = sv;
      } else if constexpr (sizeof(R) == 8) {
        EllZ& e = static_cast<EllZ*>(ell)[sl.dst_ell];
        e.v[0] = re;
        e.v[1] = im;
      } else if constexpr (REALV) {
        static_cast<EllF*>(ell)[sl.dst_ell].v = (float)sv;
      } else {
        EllC& e = static_cast<EllC*>(ell)[sl.dst_ell];
        e.v[0] = (float)re;
        e.v[1] = (float)im;
      }
    }
  }
}

// Next RK4 step of a recorded time-dependent step graph.
__global__ void k_td_advance(long long* step) { *step += 1; }

}  // namespace

void launch_td_advance(long long* step, cudaStream_t s) {
  k_td_advance<<<1, 1, 0, s>>>(step);
  QOB_LAUNCHED();
}

void launch_td_values(const GatherPlan& g, const double2* factors_dev, cudaStream_t s, const long long* step,
                      long long off, long long nf) {
  if (g.td_nslots == 0) return;
  const int threads = 256;
  const unsigned blocks = (unsigned)((g.td_nslots + threads - 1) / threads);
  const TdSlot* sl = (const TdSlot*)g.td_slots.p;
  const TdContrib* co = (const TdContrib*)g.td_contrib.p;
  const TdTerm* te = (const TdTerm*)g.td_terms.p;
  double2* dt = (double2*)g.dvals.p;
  const bool store_real = g.real_vals || g.phased;
  if (g.ff) {
    if (store_real)
      k_td_values<gather::DF, true><<<blocks, threads, 0, s>>>(g.td_nslots, sl, co, te, factors_dev, step, off, nf, g.vals.p, g.ell.p, dt);
    else
      k_td_values<gather::DF, false><<<blocks, threads, 0, s>>>(g.td_nslots, sl, co, te, factors_dev, step, off, nf, g.vals.p, g.ell.p, dt);
  } else if (g.precision == QOB_C128) {
    if (store_real)
      k_td_values<double, true><<<blocks, threads, 0, s>>>(g.td_nslots, sl, co, te, factors_dev, step, off, nf, g.vals.p, g.ell.p, dt);
    else
      k_td_values<double, false><<<blocks, threads, 0, s>>>(g.td_nslots, sl, co, te, factors_dev, step, off, nf, g.vals.p, g.ell.p, dt);
  } else {
    if (store_real)
      k_td_values<float, true><<<blocks, threads, 0, s>>>(g.td_nslots, sl, co, te, factors_dev, step, off, nf, g.vals.p, g.ell.p, dt);
    else
      k_td_values<float, false><<<blocks, threads, 0, s>>>(g.td_nslots, sl, co, te, factors_dev, step, off, nf, g.vals.p, g.ell.p, dt);
  }
  QOB_LAUNCHED();
}

// Vectors per thread: the tuned choice, else the largest of 8 / 4 / 2 / 1 that
// the number of vectors fills.
int gather_tile(const GatherPlan& g, int64_t ncols) {
  int tc = g.tc;
  if (tc <= 0) tc = 8;
  while (tc > 1 && tc > ncols) tc >>= 1;
  return tc;
}

void launch_ff_split(const void* x, int64_t n, int64_t ncols, int64_t es, int64_t cs, void* out, cudaStream_t s) {
  const int64_t total = n * ncols;
  if (total == 0) return;
  const unsigned blocks = (unsigned)((total + 256 * kSplitPer - 1) / (256 * kSplitPer));
  k_ff_split<<<blocks, 256, 0, s>>>(static_cast<const double2*>(x), n, ncols, es, cs, static_cast<float4*>(out));
  QOB_LAUNCHED();
}

void launch_gather(const GatherPlan& g, int precision, const void* x, int64_t xes, int64_t xcs,
                   void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha, c128 beta,
                   cudaStream_t s, int64_t n, void* ff_x, bool pdl) {
  GatherView v = g.view();
  v.pdl = pdl ? 1 : 0;
  const int tc = gather_tile(g, ncols);
  if (g.ff) {
    // split x once; the gather then reads the quadruples with x's strides
    if (!ff_x || n <= 0) fail(QOB_ERR_ARG, "double-float gather without split buffer");
    launch_ff_split(x, n, ncols, xes, xcs, ff_x, s);
    x = ff_x;
  }
  // groups beyond one launch's shared-memory budget go in further launches
  // that accumulate into y (beta = 1, no diagonal)
  int g0 = 0;
  bool first = true;
  do {
    GatherView c = v;
    c.groups = v.groups + g0;
    if (v.fast) c.fastg = v.fastg + g0;
    c.ngroups = v.ngroups - g0 > kGroupsPerLaunch ? kGroupsPerLaunch : v.ngroups - g0;
    c.has_diag = first ? v.has_diag : 0;
    if (v.ngroups > kGroupsPerLaunch) c.ell_slots = 0;  // chunks read their slots from global memory
    const c128 b = first ? beta : c128{1.0, 0.0};
    if (g.ff)
      gather::dispatch<gather::DF>(c, g.sites, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, b, s);
    else if (precision == QOB_C128)
      gather::dispatch<double>(c, g.sites, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, b, s);
    else
      gather::dispatch<float>(c, g.sites, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, b, s);
    g0 += c.ngroups;
    first = false;
  } while (g0 < v.ngroups);
}

void launch_build_diag(const GatherPlan& g, cudaStream_t s) {
  const int threads = 256;
  const unsigned blocks = (unsigned)((g.m + threads - 1) / threads);
  const GGroup* dg = (const GGroup*)g.dgroups.p;
  const double2* dt = (const double2*)g.dvals.p;
  if (g.ff) {
    if (g.real_vals)
      k_build_diag<gather::DF, true><<<blocks, threads, 0, s>>>(g.m, g.ndgroups, dg, dt, g.diag.p);
    else
      k_build_diag<gather::DF, false><<<blocks, threads, 0, s>>>(g.m, g.ndgroups, dg, dt, g.diag.p);
  } else if (g.precision == QOB_C128) {
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
