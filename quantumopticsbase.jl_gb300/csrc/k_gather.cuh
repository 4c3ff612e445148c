// k_gather.cuh -- the fused LazySum application kernel (templates; instantiated
// per precision in k_gather_f64.cu and k_gather_f32.cu).
//
// One thread owns one output index J and a tile of TC vectors (kets, columns).
// It accumulates, in registers, the merged diagonal times x[J] plus every
// group's stored entries of its local row times the gathered x[base + coloff],
// then writes y[J] = alpha * acc + beta * y[J] once.  This replaces the
// reference's one pass per term over `result` (src/operators_lazysum.jl:189-200)
// and the recursive per-nonzero gather (src/operators_lazytensor.jl:652-685):
// the state is read once per entry from L1/L2 instead of once per term from
// memory, and y is read and written once.
//
// Groups whose rows hold at most kMaxEllWidth entries (every ladder / Pauli /
// number product) are read as fixed-width slots staged in shared memory with
// the group descriptors: one shared-memory load per entry instead of the
// dependent rowptr -> coloff -> value chain of the CSR form, which remains for
// wide groups (a full-space SparseOperator with long rows).  When every group
// has one slot per row (W1), the group loop is unrolled so the gathers of
// several groups are in flight together, and when every group is also one run
// of power-of-two subsystems (spin chains) a 16-byte compact record per group
// replaces the descriptor reads.
//
// Subsystems of power-of-two length (spin-1/2 chains) use shifts and masks for
// the index arithmetic, others Lemire's multiply-high division.
//
// FP64 keeps the reference's arithmetic type; with real merged values (all
// the Hamiltonians built from number/ladder/Pauli factors with real
// coefficients) each stored entry costs two DFMA per vector.  FP32 mode adds
// Kahan compensation across the accumulated contributions.  The double-float
// mode (R = DF) reads and writes ComplexF64 data but does the arithmetic as
// pairs of FP32 numbers on the FP32 pipes, which on GB300 issue 64x the FP64
// rate: x is split once into (hi, lo) float pairs by k_ff_split, the stored
// values are (hi, lo) pairs, and y is joined back to double by integer
// instructions.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <utility>

#include "launch.cuh"
#include "qob_internal.h"

namespace qob {
namespace gather {

// Bounds-checked build (-DQOB_DEBUG_BOUNDS): every slot index and gathered
// input index is checked before use; an out-of-range one is skipped and
// recorded in the context's device status word (bit kErrBoundsBit), which
// qob_device_status reports.  Off in the product build.
#ifdef QOB_DEBUG_BOUNDS
constexpr bool kDebugBounds = true;
#else
constexpr bool kDebugBounds = false;
#endif
constexpr unsigned kErrBoundsBit = 2u;
__device__ __forceinline__ bool out_of_range(int64_t i, int64_t n, unsigned* status) {
  if (i >= 0 && i < n) return false;
  if (status) atomicOr(status, kErrBoundsBit);
  return true;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, uint32_t d, uint64_t M) {
  return d == 1u ? n : (uint32_t)__umul64hi(M, (uint64_t)n);
}
__device__ __forceinline__ uint32_t fmodu(uint32_t n, uint32_t d, uint64_t M) {
  uint64_t low = M * (uint64_t)n;
  return (uint32_t)__umul64hi(low, (uint64_t)d);
}

// Precision tag of the double-float mode: ComplexF64 data, FP32-pair arithmetic.
struct DF {};
// The same arithmetic reading ComplexF64 vectors directly and splitting each
// element as it is loaded (the persistent batch kernel, whose items' vectors
// are read in place).
struct DFX {};

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
template <>
struct Cx<DF> {
  using T = double2;  // y and alpha / beta: ComplexF64
};
template <>
struct Cx<DFX> {
  using T = double2;
};

// element type of the input vectors as the kernels read them: the data type,
// or for DF the (re hi, re lo, im hi, im lo) quadruple written by k_ff_split
template <typename R>
struct In {
  using T = typename Cx<R>::T;
};
template <>
struct In<DF> {
  using T = float4;
};

template <typename R, int VM>
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
template <>
struct Val<DF, true> {
  using T = float2;  // (hi, lo)
};
template <>
struct Val<DF, false> {
  using T = float4;  // (re hi, re lo, im hi, im lo)
};
template <>
struct Val<DFX, true> {
  using T = float2;
};
template <>
struct Val<DFX, false> {
  using T = float4;
};

// fixed-width slot type per precision / realness, and its value
template <typename R, int VM>
struct Ell;
template <>
struct Ell<double, true> {
  using T = EllD;
  static __device__ __forceinline__ double v(const EllD& e) { return e.v; }
};
template <>
struct Ell<double, false> {
  using T = EllZ;
  static __device__ __forceinline__ double2 v(const EllZ& e) { return make_double2(e.v[0], e.v[1]); }
};
template <>
struct Ell<float, true> {
  using T = EllF;
  static __device__ __forceinline__ float v(const EllF& e) { return e.v; }
};
template <>
struct Ell<float, false> {
  using T = EllC;
  static __device__ __forceinline__ float2 v(const EllC& e) { return make_float2(e.v[0], e.v[1]); }
};
template <>
struct Ell<DF, true> {
  using T = EllDF;
  static __device__ __forceinline__ float2 v(const EllDF& e) { return make_float2(e.v[0], e.v[1]); }
};
template <>
struct Ell<DF, false> {
  using T = EllZF;
  static __device__ __forceinline__ float4 v(const EllZF& e) { return make_float4(e.v[0], e.v[1], e.v[2], e.v[3]); }
};
template <int RV>
struct Ell<DFX, RV> : Ell<DF, RV> {};

// Value modes of a plan: complex entries; real entries (and a real diagonal);
// real entries of groups that are either real or purely imaginary, with a
// per-group flag for the factor i, and a complex diagonal ("phased": e.g. the
// -i H and +i H parts of a Liouvillian beside its real dissipator).
constexpr int kComplex = 0, kReal = 1, kPhased = 2;

// Nonzero tests on the bit patterns (sign bit shifted out, so -0 counts as
// zero, NaN as nonzero): integer instructions, where a floating-point compare
// of a double would occupy the FP64 pipe that bounds the ComplexF64 kernels.
__device__ __forceinline__ bool nz(double v) { return ((unsigned long long)__double_as_longlong(v) << 1) != 0ull; }
__device__ __forceinline__ bool nz(float v) { return (__float_as_uint(v) << 1) != 0u; }
__device__ __forceinline__ bool nz(double2 v) {
  return ((unsigned long long)(__double_as_longlong(v.x) | __double_as_longlong(v.y)) << 1) != 0ull;
}
__device__ __forceinline__ bool nz(float2 v) { return ((__float_as_uint(v.x) | __float_as_uint(v.y)) << 1) != 0u; }
__device__ __forceinline__ bool nz(float4 v) {
  return ((__float_as_uint(v.x) | __float_as_uint(v.y) | __float_as_uint(v.z) | __float_as_uint(v.w)) << 1) != 0u;
}

// FP64 accumulator: plain fused multiply-adds.
struct AccD {
  double re, im;
  __device__ void zero() { re = im = 0.0; }
  __device__ void mac(double v, double2 x) {
    re = fma(v, x.x, re);
    im = fma(v, x.y, im);
  }
  // (i v) x for real v: the sign goes into the FMA operand
  __device__ void mac_i(double v, double2 x) {
    re = fma(-v, x.y, re);
    im = fma(v, x.x, im);
  }
  __device__ void mac_i(double2 v, double2 x) { mac(make_double2(-v.y, v.x), x); }
  __device__ void mac(double2 v, double2 x) {
    re = fma(v.x, x.x, re);
    re = fma(-v.y, x.y, re);
    im = fma(v.x, x.y, im);
    im = fma(v.y, x.x, im);
  }
  __device__ void set(double v, double2 x) {
    re = v * x.x;
    im = v * x.y;
  }
  __device__ void set(double2 v, double2 x) {
    re = fma(-v.y, x.y, v.x * x.x);
    im = fma(v.y, x.x, v.x * x.y);
  }
  __device__ double2 total() const { return make_double2(re, im); }
};

// FP32 accumulator with Kahan compensation (Kahan 1965): c carries the
// low-order part lost by each addition.  The term is formed with the
// compensation folded in, y = fma(v, x, -c) (one rounding), so a real
// multiply-add costs four FP32 operations: y, s = acc + y, c = (s - acc) - y.
struct AccF {
  float re, im, cre, cim;
  __device__ void zero() { re = im = cre = cim = 0.f; }
  // acc += y where y already holds term - c
  __device__ __forceinline__ void step(float& a, float& c, float y) {
    const float s = a + y;
    c = (s - a) - y;
    a = s;
  }
  __device__ void add(float tr, float ti) {
    step(re, cre, tr - cre);
    step(im, cim, ti - cim);
  }
  __device__ void mac(float v, float2 x) {
    step(re, cre, __fmaf_rn(v, x.x, -cre));
    step(im, cim, __fmaf_rn(v, x.y, -cim));
  }
  __device__ void mac_i(float v, float2 x) {
    step(re, cre, __fmaf_rn(-v, x.y, -cre));
    step(im, cim, __fmaf_rn(v, x.x, -cim));
  }
  __device__ void mac(float2 v, float2 x) {
    step(re, cre, __fmaf_rn(v.x, x.x, __fmaf_rn(-v.y, x.y, -cre)));
    step(im, cim, __fmaf_rn(v.x, x.y, __fmaf_rn(v.y, x.x, -cim)));
  }
  __device__ void mac_i(float2 v, float2 x) { mac(make_float2(-v.y, v.x), x); }
  __device__ void set(float v, float2 x) {
    re = v * x.x;
    im = v * x.y;
    cre = cim = 0.f;
  }
  __device__ void set(float2 v, float2 x) {
    re = __fmaf_rn(v.x, x.x, -v.y * x.y);
    im = __fmaf_rn(v.x, x.y, v.y * x.x);
    cre = cim = 0.f;
  }
  __device__ float2 total() const { return make_float2(re - cre, im - cim); }
};

// ---- double-float arithmetic (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2) ----
// A value is the unevaluated sum hi + lo of two floats.

// double -> (hi, lo) with integer instructions only: hi = the double truncated
// to 24 significant bits (exact), lo = the remaining 29 bits rounded to 24, so
// hi + lo is within 2^-48 relative of d.  Magnitudes in [2^-74, 2^128) keep
// both parts; in [2^-126, 2^-74) lo is dropped; below 2^-126 the value
// flushes to zero; above, hi is infinite (NaN stays NaN).
__device__ __forceinline__ float2 ff_split(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const uint32_t H = (uint32_t)(u >> 32), L = (uint32_t)u;
  const uint32_t sgn = H & 0x80000000u, ma = H & 0x7fffffffu;
  const uint32_t e = ma >> 20;  // biased binary exponent of the double
  float hi, lo;
  if (e >= 897u && e <= 1150u) {
    hi = __uint_as_float(sgn | ((ma - 0x38000000u) << 3) | (L >> 29));
  } else if (e > 1150u) {
    const bool nan = e == 2047u && ((ma & 0xfffffu) | L) != 0u;
    hi = __uint_as_float(sgn | 0x7f800000u | (nan ? 0x400000u : 0u));
  } else {
    hi = __uint_as_float(sgn);
  }
  if (e >= 949u && e <= 1150u) {
    // (L mod 2^29) * 2^(e - 1075); the power of two is a float with exponent field e - 948
    lo = __uint2float_rn(L & 0x1fffffffu) * __uint_as_float((e - 948u) << 23);
    lo = __uint_as_float(__float_as_uint(lo) | sgn);
  } else {
    lo = 0.f;
  }
  return make_float2(hi, lo);
}

// (hi, lo) -> double with integer instructions: renormalise with a two-sum,
// write hi's bits as a double and add lo in units of the double's last place.
__device__ __forceinline__ double ff_join(float h, float l) {
  const float s = h + l;
  const float bb = s - h;
  const float e = (h - (s - bb)) + (l - bb);  // s + e == h + l, |e| <= ulp(s) / 2
  const uint32_t S = __float_as_uint(s);
  const uint32_t E = (S >> 23) & 0xffu, M = S & 0x7fffffu;
  const unsigned long long sgn = (unsigned long long)(S & 0x80000000u) << 32;
  if (E == 0u) return __longlong_as_double((long long)sgn);  // zero (subnormal floats flush)
  if (E == 255u)
    return __longlong_as_double((long long)(sgn | 0x7ff0000000000000ull | (M ? 0x8000000000000ull : 0ull)));
  unsigned long long mag = ((unsigned long long)(E + 896u) << 52) | ((unsigned long long)M << 29);
  if (E >= 53u) {
    // e in units of the double's last place at s (2^(E - 179)); half that when
    // s is a power of two and e points below it (the next lower binade); the
    // scale 2^(179 - E) or 2^(180 - E) is a normal float for E >= 53, and
    // below that (|s| < 2^-74) e is dropped
    const bool toward = (__float_as_uint(e) ^ S) & 0x80000000u;
    const uint32_t sc = (M == 0u && toward) ? (307u - E) : (306u - E);
    const int n = __float2int_rn(fabsf(e) * __uint_as_float(sc << 23));
    mag = toward ? mag - (unsigned long long)n : mag + (unsigned long long)n;
  }
  return __longlong_as_double((long long)(sgn | mag));
}

// product of two double-float numbers (the lo * lo term is below 2^-48)
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float pe = __fmaf_rn(a.x, b.x, -p);
  pe = __fmaf_rn(a.x, b.y, pe);
  pe = __fmaf_rn(a.y, b.x, pe);
  return make_float2(p, pe);
}
// sum of two double-float numbers: two-sum of the high parts, the low parts added
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  const float s = a.x + b.x;
  const float bb = s - a.x;
  const float err = (a.x - (s - bb)) + (b.x - bb);
  return make_float2(s, err + (a.y + b.y));
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }

// Double-float accumulator of one complex value: acc += v * x with the
// product error (FMA) and the addition error (two-sum) carried in the low parts.
struct AccFF {
  float rh, rl, ih, il;
  static __device__ __forceinline__ void madd(float& h, float& l, float2 v, float xh, float xl) {
    const float p = v.x * xh;
    float pe = __fmaf_rn(v.x, xh, -p);
    pe = __fmaf_rn(v.x, xl, pe);
    pe = __fmaf_rn(v.y, xh, pe);
    const float s = h + p;
    const float bb = s - h;
    const float err = (h - (s - bb)) + (p - bb);
    l = l + (err + pe);
    h = s;
  }
  __device__ void zero() { rh = rl = ih = il = 0.f; }
  __device__ void mac(float2 v, float4 x) {
    madd(rh, rl, v, x.x, x.y);
    madd(ih, il, v, x.z, x.w);
  }
  // (i v) x for real v
  __device__ void mac_i(float2 v, float4 x) {
    madd(rh, rl, ff_neg(v), x.z, x.w);
    madd(ih, il, v, x.x, x.y);
  }
  __device__ void mac(float4 v, float4 x) {
    const float2 vr = make_float2(v.x, v.y), vi = make_float2(v.z, v.w);
    madd(rh, rl, vr, x.x, x.y);
    madd(rh, rl, ff_neg(vi), x.z, x.w);
    madd(ih, il, vr, x.z, x.w);
    madd(ih, il, vi, x.x, x.y);
  }
  __device__ void mac_i(float4 v, float4 x) { mac(make_float4(-v.z, -v.w, v.x, v.y), x); }
  __device__ void set(float2 v, float4 x) {
    const float2 r = ff_mul(v, make_float2(x.x, x.y)), i = ff_mul(v, make_float2(x.z, x.w));
    rh = r.x;
    rl = r.y;
    ih = i.x;
    il = i.y;
  }
  __device__ void set(float4 v, float4 x) {
    zero();
    mac(v, x);
  }
  __device__ float4 total() const { return make_float4(rh, rl, ih, il); }
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
template <>
struct AccOf<DF> {
  using T = AccFF;
};

// AccFF fed with ComplexF64 elements, split as they arrive (DFX)
__device__ __forceinline__ float4 ff_split4(double2 x) {
  const float2 a = ff_split(x.x), b = ff_split(x.y);
  return make_float4(a.x, a.y, b.x, b.y);
}
struct AccFFX : AccFF {
  __device__ void mac(float2 v, double2 x) { AccFF::mac(v, ff_split4(x)); }
  __device__ void mac_i(float2 v, double2 x) { AccFF::mac_i(v, ff_split4(x)); }
  __device__ void mac(float4 v, double2 x) { AccFF::mac(v, ff_split4(x)); }
  __device__ void mac_i(float4 v, double2 x) { AccFF::mac_i(v, ff_split4(x)); }
  __device__ void set(float2 v, double2 x) { AccFF::set(v, ff_split4(x)); }
  __device__ void set(float4 v, double2 x) { AccFF::set(v, ff_split4(x)); }
};
template <>
struct AccOf<DFX> {
  using T = AccFFX;
};

__device__ __forceinline__ double2 ld(const double2* p) { return __ldg(p); }
__device__ __forceinline__ float2 ld(const float2* p) { return __ldg(p); }
__device__ __forceinline__ float4 ld(const float4* p) { return __ldg(p); }

// y = alpha * acc + beta * y with the reference's beta semantics:
// BMODE 0: beta == 0 (y is not read), 2: general complex beta, 3: real beta.
template <int BMODE>
__device__ __forceinline__ void combine(double2* yp, double2 a, double2 alpha, double2 beta) {
  double re = alpha.x * a.x - alpha.y * a.y;
  double im = alpha.x * a.y + alpha.y * a.x;
  if (BMODE == 2) {
    double2 o = *yp;
    re = fma(beta.x, o.x, fma(-beta.y, o.y, re));
    im = fma(beta.x, o.y, fma(beta.y, o.x, im));
  } else if (BMODE == 3) {
    double2 o = *yp;
    re = fma(beta.x, o.x, re);
    im = fma(beta.x, o.y, im);
  }
  *yp = make_double2(re, im);
}
template <int BMODE>
__device__ __forceinline__ void combine(float2* yp, float2 a, float2 alpha, float2 beta) {
  float re = alpha.x * a.x - alpha.y * a.y;
  float im = alpha.x * a.y + alpha.y * a.x;
  if (BMODE == 2) {
    float2 o = *yp;
    re = __fmaf_rn(beta.x, o.x, __fmaf_rn(-beta.y, o.y, re));
    im = __fmaf_rn(beta.x, o.y, __fmaf_rn(beta.y, o.x, im));
  } else if (BMODE == 3) {
    float2 o = *yp;
    re = __fmaf_rn(beta.x, o.x, re);
    im = __fmaf_rn(beta.x, o.y, im);
  }
  *yp = make_float2(re, im);
}

// double-float: acc = (re hi, re lo, im hi, im lo), joined to double by
// integer instructions; alpha * acc + beta * y then in FP64 like the ComplexF64
// kernels (six FP64 operations per element, on the pipe the FP32-pair gather
// leaves idle)
template <int BMODE>
__device__ __forceinline__ void combine(double2* yp, float4 a, double2 alpha, double2 beta) {
  combine<BMODE>(yp, make_double2(ff_join(a.x, a.y), ff_join(a.z, a.w)), alpha, beta);
}

// Copy the group descriptors (then, for plans with the compact form, one int4
// per group; then, if requested, the fixed-width slots) to shared memory;
// returns the slot pointer to use.
template <typename ET>
__device__ __forceinline__ const ET* stage(unsigned char* smem, const GatherView& g) {
  GGroup* sg = reinterpret_cast<GGroup*>(smem);
  {
    const uint64_t* src = reinterpret_cast<const uint64_t*>(g.groups);
    uint64_t* dst = reinterpret_cast<uint64_t*>(sg);
    const int words = g.ngroups * (int)(sizeof(GGroup) / 8);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
  size_t off = (size_t)g.ngroups * sizeof(GGroup);
  if (g.fast) {
    int4* df = reinterpret_cast<int4*>(smem + off);
    for (int i = threadIdx.x; i < g.ngroups; i += blockDim.x) df[i] = g.fastg[i];
    off += (size_t)g.ngroups * sizeof(int4);
  }
  const ET* ell = static_cast<const ET*>(g.ell);
  if (g.ell_smem) {
    ET* se = reinterpret_cast<ET*>(smem + off);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(g.ell);
    uint32_t* dst = reinterpret_cast<uint32_t*>(se);
    const int words = g.ell_slots * (int)(sizeof(ET) / 4);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    ell = se;
  }
  __syncthreads();
  return ell;
}

// Local row r of output index J in group G, and sub = the part of J carried by
// the group's subsystems (so J - sub is the row's base index on a square basis).
__device__ __forceinline__ void local_row(const GGroup& G, uint32_t J, uint32_t& r, uint32_t& sub) {
  if (G.nblk == 1) {  // one run of consecutive subsystems (the common case)
    uint32_t d;
    if (G.pow2) {
      const uint32_t sh = G.shifts[0];
      d = (J >> (sh & 0xffu)) & (G.mod[0] - 1u);
      sub = d << (sh & 0xffu);
    } else {
      d = fmodu(fdiv(J, G.div[0], G.mdiv[0]), G.mod[0], G.mmod[0]);
      sub = d * G.div[0];
    }
    r = d;
    return;
  }
  r = 0;
  sub = 0;
  if (G.pow2) {  // shifts and masks (power-of-two subsystem lengths)
#pragma unroll
    for (int b = 0; b < kMaxBlocks; ++b) {
      if (b < G.nblk) {
        const uint32_t sh = G.shifts[b];
        const uint32_t sd = sh & 0xffu, sm = (sh >> 8) & 0xffu, sl = sh >> 16;
        const uint32_t d = (J >> sd) & ((1u << sm) - 1u);
        r += d << sl;
        sub += d << sd;
      }
    }
  } else {
#pragma unroll
    for (int b = 0; b < kMaxBlocks; ++b) {
      if (b < G.nblk) {
        const uint32_t q = fdiv(J, G.div[b], G.mdiv[b]);
        const uint32_t d = fmodu(q, G.mod[b], G.mmod[b]);
        r += d * G.lstride[b];
        sub += d * G.div[b];
      }
    }
  }
}

// Local row and input base offset of output index J in group G; false when a
// subsystem outside the support has no counterpart on the input side.
template <bool SQUARE>
__device__ __forceinline__ bool group_row(const GGroup& G, const SiteTable& st, uint32_t J,
                                          uint32_t& r, int64_t& base) {
  uint32_t sub;
  local_row(G, J, r, sub);
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

// acc[t] = (H x)[J] for the nt vectors starting at xb (element stride es,
// vector stride xcs).
template <typename R, int VM, bool SQUARE, bool W1, int TC>
__device__ __forceinline__ void accumulate(const GatherView& g, const SiteTable& st, const GGroup* sg,
                                           const typename Ell<R, VM != kComplex>::T* ell, uint32_t J,
                                           const typename In<R>::T* xb, int64_t es, int64_t xcs, int nt,
                                           typename AccOf<R>::T (&acc)[TC]) {
  using VT = typename Val<R, VM != kComplex>::T;  // stored entries
  using DT = typename Val<R, VM == kReal>::T;     // merged diagonal
  using ET = typename Ell<R, VM != kComplex>::T;
  using CT = typename In<R>::T;
  if (g.has_diag) {
    const DT d = static_cast<const DT*>(g.diag)[J];
    const CT* xp = xb + (int64_t)J * es;
#pragma unroll
    for (int t = 0; t < TC; ++t)
      if (t < nt) acc[t].set(d, ld(xp + t * xcs));
  } else {
#pragma unroll
    for (int t = 0; t < TC; ++t) acc[t].zero();
  }
  if (W1 && g.fast) {
    // every group: one run of power-of-two subsystems, one slot per row; its
    // shift, mask and first slot sit in one 16-byte word after the descriptors
    const int4* fg = reinterpret_cast<const int4*>(sg + g.ngroups);
#pragma unroll 4
    for (int gi = 0; gi < g.ngroups; ++gi) {
      const int4 f = fg[gi];
      const uint32_t r = (J >> f.x) & (uint32_t)f.y;
      if (kDebugBounds && out_of_range((int64_t)f.z + r, g.ell_slots, g.status)) continue;
      const ET s = ell[f.z + r];
      const VT v = Ell<R, VM != kComplex>::v(s);
      const CT* xp = xb + ((int64_t)(J - (r << f.x)) + s.col) * es;
      if (kDebugBounds && nz(v) && out_of_range((int64_t)(J - (r << f.x)) + s.col, g.n, g.status)) continue;
      if (nz(v)) {
        if (VM == kPhased && f.w != 0) {
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (t < nt) acc[t].mac_i(v, ld(xp + t * xcs));
        } else {
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (t < nt) acc[t].mac(v, ld(xp + t * xcs));
        }
      }
    }
    return;
  }
  if (W1) {
    // one slot per row in every group: unrolled, loads of several groups in flight
#pragma unroll 4
    for (int gi = 0; gi < g.ngroups; ++gi) {
      const GGroup& G = sg[gi];
      uint32_t r, sub;
      local_row(G, J, r, sub);
      if (kDebugBounds && out_of_range((int64_t)G.ell_off + r, g.ell_slots, g.status)) continue;
      const ET s = ell[G.ell_off + r];
      const VT v = Ell<R, VM != kComplex>::v(s);
      const CT* xp = xb + ((int64_t)(J - sub) + s.col) * es;
      if (kDebugBounds && nz(v) && out_of_range((int64_t)(J - sub) + s.col, g.n, g.status)) continue;
      if (nz(v)) {
        if (VM == kPhased && G.imag != 0) {
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (t < nt) acc[t].mac_i(v, ld(xp + t * xcs));
        } else {
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (t < nt) acc[t].mac(v, ld(xp + t * xcs));
        }
      }
    }
    return;
  }
  const VT* vals = static_cast<const VT*>(g.vals);
  for (int gi = 0; gi < g.ngroups; ++gi) {
    const GGroup& G = sg[gi];
    uint32_t r;
    int64_t base;
    if (!group_row<SQUARE>(G, st, J, r, base)) continue;
    const bool im = VM == kPhased && G.imag != 0;
    if (G.width > 0) {
      const ET* e = ell + G.ell_off + (int64_t)r * G.width;
      for (int k = 0; k < G.width; ++k) {
        if (kDebugBounds && out_of_range((int64_t)G.ell_off + (int64_t)r * G.width + k, g.ell_slots, g.status)) continue;
        const ET s = e[k];
        const VT v = Ell<R, VM != kComplex>::v(s);
        if (kDebugBounds && nz(v) && out_of_range(base + s.col, g.n, g.status)) continue;
        if (nz(v)) {
          const CT* xp = xb + (base + s.col) * es;
          if (im) {
#pragma unroll
            for (int t = 0; t < TC; ++t)
              if (t < nt) acc[t].mac_i(v, ld(xp + t * xcs));
          } else {
#pragma unroll
            for (int t = 0; t < TC; ++t)
              if (t < nt) acc[t].mac(v, ld(xp + t * xcs));
          }
        }
      }
    } else {
      const int p0 = __ldg(g.rowptr + G.rowptr_off + r);
      const int p1 = __ldg(g.rowptr + G.rowptr_off + r + 1);
      for (int p = p0; p < p1; ++p) {
        if (kDebugBounds && out_of_range(base + __ldg(g.coloff + p), g.n, g.status)) continue;
        const CT* xp = xb + (base + __ldg(g.coloff + p)) * es;
        const VT v = vals[p];
        if (im) {
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (t < nt) acc[t].mac_i(v, ld(xp + t * xcs));
        } else {
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (t < nt) acc[t].mac(v, ld(xp + t * xcs));
        }
      }
    }
  }
}

// Output index J fastest across threads: one thread per (J, tile of TC vectors);
// the vectors are contiguous (element stride 1).
template <typename R, int VM, bool SQUARE, bool W1, int TC, int BMODE>
__global__ void __launch_bounds__(256) k_gather_j(GatherView g, SiteTable st,
                                                  const typename In<R>::T* __restrict__ x, int64_t xcs,
                                                  typename Cx<R>::T* __restrict__ y, int64_t ycs, int ncols,
                                                  typename Cx<R>::T alpha, typename Cx<R>::T beta) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  using AT = typename AccOf<R>::T;
  using ET = typename Ell<R, VM != kComplex>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_enter();
  const ET* ell = stage<ET>(smem_raw, g);
  const GGroup* sg = reinterpret_cast<const GGroup*>(smem_raw);
  // lane split ls: a warp covers 32/ls consecutive output indices and ls
  // interleaved sets of TC vectors (vectors q, q + ls, ...), so operator
  // entries that vary with the low index bits diverge over fewer lanes; each
  // load still reads whole 32-byte sectors (32/ls consecutive elements per vector)
  // (ls is a power of two: shifts and masks, no integer division, which would
  // cost more than the work of a thread with one vector and few groups)
  const int ls = g.lane_split;
  const int lsh = __ffs(ls) - 1;  // log2(ls)
  const int jsh = 5 - lsh;        // log2(32 / ls)
  const int lane = threadIdx.x & 31;
  // block permutation: only grids of at most 4096 blocks use one (jmul < gridDim.x),
  // so the product fits 32 bits; jmul == 1 keeps the order without a modulo
  const int64_t blk = g.jmul == 1u ? (int64_t)blockIdx.x : (int64_t)((blockIdx.x * g.jmul) % gridDim.x);
  const int64_t J = blk * (int64_t)(blockDim.x >> lsh) + ((threadIdx.x >> 5) << jsh) + (lane & ((1 << jsh) - 1));
  if (J >= g.m) return;
  const int c0 = blockIdx.y * TC * ls + (lane >> jsh);
  // nt == 0 (a ket set past the last vector) skips every load and store below;
  // an early return here instead makes the FP64 single-vector kernels ~45 % slower
  const int nt = c0 < ncols ? min(TC, (ncols - c0 + ls - 1) >> lsh) : 0;
  const int64_t vs_x = (int64_t)ls * xcs, vs_y = (int64_t)ls * ycs;
  const XT* xb = x + (int64_t)c0 * xcs;
  AT acc[TC];
  accumulate<R, VM, SQUARE, W1, TC>(g, st, sg, ell, (uint32_t)J, xb, 1, vs_x, nt, acc);
  CT* yb = y + J + (int64_t)c0 * ycs;
#pragma unroll
  for (int t = 0; t < TC; ++t)
    if (t < nt) combine<BMODE>(yb + t * vs_y, acc[t].total(), alpha, beta);
}

// The two inputs of a pair of consecutive elements (the first at an even index):
// ComplexF32 in one 16-byte load, ComplexF64 (and its double-float split) in two.
__device__ __forceinline__ void ld_pair(const float2* p, float2& a, float2& b) {
  const float4 q = __ldg(reinterpret_cast<const float4*>(p));
  a = make_float2(q.x, q.y);
  b = make_float2(q.z, q.w);
}
__device__ __forceinline__ void ld_pair(const double2* p, double2& a, double2& b) {
  a = __ldg(p);
  b = __ldg(p + 1);
}
__device__ __forceinline__ void ld_pair(const float4* p, float4& a, float4& b) {  // double-float (hi, lo) pairs
  a = __ldg(p);
  b = __ldg(p + 1);
}
template <typename R, int VM>
struct PairsOk {
  static constexpr bool value =
      (std::is_same<R, double>::value || std::is_same<R, float>::value || std::is_same<R, DF>::value) && VM != kComplex;
};

// Two consecutive output indices per thread (J0 even and J0 + 1), for compact
// plans on kets (every group one run of power-of-two subsystems, one slot per
// row).  A group whose run starts above bit 0 maps both indices to the same
// local row, slot and value and to two consecutive inputs (an even first one),
// so its descriptor, slot lookup and index arithmetic serve two outputs and
// a ComplexF32 ket's two inputs arrive in one 16-byte load; the group on bit 0
// is taken index by index.  Lane split, block order and vector sets as
// k_gather_j, over pairs.
template <typename R, int VM, int TC, int BMODE>
__global__ void __launch_bounds__(256) k_gather_j2(GatherView g, const typename In<R>::T* __restrict__ x, int64_t xcs,
                                                   typename Cx<R>::T* __restrict__ y, int64_t ycs, int ncols,
                                                   typename Cx<R>::T alpha, typename Cx<R>::T beta) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  using AT = typename AccOf<R>::T;
  using ET = typename Ell<R, VM != kComplex>::T;
  using VT = typename Val<R, VM != kComplex>::T;
  using DT = typename Val<R, VM == kReal>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_enter();
  const ET* ell = stage<ET>(smem_raw, g);
  const int4* fg = reinterpret_cast<const int4*>(reinterpret_cast<const GGroup*>(smem_raw) + g.ngroups);
  const int ls = g.lane_split;
  const int lsh = __ffs(ls) - 1;
  const int jsh = 5 - lsh;
  const int lane = threadIdx.x & 31;
  const int64_t blk = g.jmul == 1u ? (int64_t)blockIdx.x : (int64_t)((blockIdx.x * g.jmul) % gridDim.x);
  const int64_t pair = blk * (int64_t)(blockDim.x >> lsh) + ((threadIdx.x >> 5) << jsh) + (lane & ((1 << jsh) - 1));
  if (2 * pair >= g.m) return;
  const uint32_t J0 = (uint32_t)(2 * pair);
  const int c0 = blockIdx.y * TC * ls + (lane >> jsh);
  const int nt = c0 < ncols ? min(TC, (ncols - c0 + ls - 1) >> lsh) : 0;
  const int64_t vs_x = (int64_t)ls * xcs, vs_y = (int64_t)ls * ycs;
  const XT* xb = x + (int64_t)c0 * xcs;
  AT a0[TC], a1[TC];
  if (g.has_diag) {
    const DT d0 = static_cast<const DT*>(g.diag)[J0], d1 = static_cast<const DT*>(g.diag)[J0 + 1];
#pragma unroll
    for (int t = 0; t < TC; ++t)
      if (t < nt) {
        XT u, w;
        ld_pair(xb + J0 + t * vs_x, u, w);
        a0[t].set(d0, u);
        a1[t].set(d1, w);
      }
  } else {
#pragma unroll
    for (int t = 0; t < TC; ++t) {
      a0[t].zero();
      a1[t].zero();
    }
  }
#pragma unroll 4
  for (int gi = 0; gi < g.ngroups; ++gi) {
    const int4 f = fg[gi];
    const bool im = VM == kPhased && f.w != 0;
    if (f.x == 0) {  // the group on bit 0: each index on its own
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const uint32_t J = J0 + (uint32_t)e;
        const uint32_t r = J & (uint32_t)f.y;
        if (kDebugBounds && out_of_range((int64_t)f.z + r, g.ell_slots, g.status)) continue;
        const ET s = ell[f.z + r];
        const VT v = Ell<R, VM != kComplex>::v(s);
        if (kDebugBounds && nz(v) && out_of_range((int64_t)(J - r) + s.col, g.n, g.status)) continue;
        if (nz(v)) {
          const XT* xp = xb + ((int64_t)(J - r) + s.col);
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (t < nt) {
              AT& acc = e == 0 ? a0[t] : a1[t];
              if (im)
                acc.mac_i(v, ld(xp + t * vs_x));
              else
                acc.mac(v, ld(xp + t * vs_x));
            }
        }
      }
    } else {
      const uint32_t r = (J0 >> f.x) & (uint32_t)f.y;
      if (kDebugBounds && out_of_range((int64_t)f.z + r, g.ell_slots, g.status)) continue;
      const ET s = ell[f.z + r];
      const VT v = Ell<R, VM != kComplex>::v(s);
      const int64_t p0 = (int64_t)(J0 - (r << f.x)) + s.col;  // even: every offset of the run is
      if (kDebugBounds && nz(v) && out_of_range(p0 + 1, g.n, g.status)) continue;  // a multiple of 2^f.x
      if (nz(v)) {
        const XT* xp = xb + p0;
#pragma unroll
        for (int t = 0; t < TC; ++t)
          if (t < nt) {
            XT u, w;
            ld_pair(xp + t * vs_x, u, w);
            if (im) {
              a0[t].mac_i(v, u);
              a1[t].mac_i(v, w);
            } else {
              a0[t].mac(v, u);
              a1[t].mac(v, w);
            }
          }
      }
    }
  }
  CT* yb = y + J0 + (int64_t)c0 * ycs;
#pragma unroll
  for (int t = 0; t < TC; ++t)
    if (t < nt) {
      combine<BMODE>(yb + t * vs_y, a0[t].total(), alpha, beta);
      combine<BMODE>(yb + 1 + t * vs_y, a1[t].total(), alpha, beta);
    }
}

// The same work as k_gather_j on a grid of exactly (SMs x resident blocks per
// SM): every block is resident at once, so every SM holds the same number of
// blocks, and block b takes the b-th equal share of the warp-sized chunks (32
// consecutive output indices x TC vectors).  With k_gather_j's grid of one
// wave or less the hardware may place up to the occupancy limit on some SMs
// and fewer on others; here the work per SM differs by at most one chunk per
// block.
template <typename R, int VM, bool SQUARE, bool W1, int TC, int BMODE>
__global__ void __launch_bounds__(256) k_gather_p(GatherView g, SiteTable st,
                                                  const typename In<R>::T* __restrict__ x, int64_t xcs,
                                                  typename Cx<R>::T* __restrict__ y, int64_t ycs, int ncols,
                                                  typename Cx<R>::T alpha, typename Cx<R>::T beta) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  using AT = typename AccOf<R>::T;
  using ET = typename Ell<R, VM != kComplex>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_enter();
  const ET* ell = stage<ET>(smem_raw, g);
  const GGroup* sg = reinterpret_cast<const GGroup*>(smem_raw);
  // chunks of (32/ls output indices x ls sets of TC vectors), one per warp at a
  // time, as in k_gather_j's lane split
  const int ls = g.lane_split;
  const int lsh = __ffs(ls) - 1, jsh = 5 - lsh;
  const int lane = threadIdx.x & 31;
  const int64_t nj = (g.m + (1 << jsh) - 1) >> jsh;
  const int64_t per_tile = (int64_t)TC * ls;
  const int64_t nchunks = nj * ((ncols + per_tile - 1) / per_tile);
  const int64_t lo = (int64_t)blockIdx.x * nchunks / gridDim.x;
  const int64_t hi = ((int64_t)blockIdx.x + 1) * nchunks / gridDim.x;
  const int64_t vs_x = (int64_t)ls * xcs, vs_y = (int64_t)ls * ycs;
  for (int64_t c = lo + (threadIdx.x >> 5); c < hi; c += blockDim.x >> 5) {
    int64_t tile, jc;
    udivmod(c, nj, tile, jc);
    if (g.jmul != 1u) {  // permuted order of the index chunks (jmul < nj, coprime)
      int64_t q;
      udivmod((int64_t)((uint64_t)jc * g.jmul), nj, q, jc);
    }
    const int64_t J = (jc << jsh) + (lane & ((1 << jsh) - 1));
    const int c0 = (int)(tile * per_tile) + (lane >> jsh);
    const int nt = c0 < ncols ? min(TC, (ncols - c0 + ls - 1) >> lsh) : 0;
    if (J < g.m) {
      const XT* xb = x + (int64_t)c0 * xcs;
      AT acc[TC];
      accumulate<R, VM, SQUARE, W1, TC>(g, st, sg, ell, (uint32_t)J, xb, 1, vs_x, nt, acc);
      CT* yb = y + J + (int64_t)c0 * ycs;
#pragma unroll
      for (int t = 0; t < TC; ++t)
        if (t < nt) combine<BMODE>(yb + t * vs_y, acc[t].total(), alpha, beta);
    }
  }
}

// Vectors with a stride between their elements (the rows of an operator
// multiplied from the right, a strided bra): the vectors run across threads,
// all threads of a block share one output index J.
template <typename R, int VM, bool SQUARE, int BMODE>
__global__ void __launch_bounds__(256) k_gather_c(GatherView g, SiteTable st,
                                                  const typename In<R>::T* __restrict__ x, int64_t xes,
                                                  int64_t xcs, typename Cx<R>::T* __restrict__ y,
                                                  int64_t yes, int64_t ycs, int ncols, typename Cx<R>::T alpha,
                                                  typename Cx<R>::T beta) {
  using AT = typename AccOf<R>::T;
  using ET = typename Ell<R, VM != kComplex>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_enter();
  const ET* ell = stage<ET>(smem_raw, g);
  const GGroup* sg = reinterpret_cast<const GGroup*>(smem_raw);
  const int64_t J = blockIdx.x;
  const int64_t c = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  AT acc[1];
  accumulate<R, VM, SQUARE, false, 1>(g, st, sg, ell, (uint32_t)J, x + c * xcs, xes, xcs, 1, acc);
  combine<BMODE>(y + J * yes + c * ycs, acc[0].total(), alpha, beta);
}

}  // namespace gather
}  // namespace qob

#include "k_tile.cuh"

namespace qob {
namespace gather {

// ---------------------------------------------------------------------------
// host-side dispatch (instantiated per precision)

constexpr size_t kSmemBudget = 96 * 1024;  // descriptors + staged slots per block
// Slots are staged per block only when the table is small: local operators
// (bonds, couplings) are read by every row, while a full-space sparse operator's
// table is read one block-sized slice per block and stays in L1/L2.
constexpr size_t kStageSlotsMax = 16 * 1024;
constexpr int kThreads = 256;

template <typename K>
void allow_smem(K kernel, size_t smem) {
  if (smem > 48 * 1024)
    QOB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
}

template <typename R, int VM, bool SQUARE, bool W1, int TC, int BMODE>
void launch_j(const GatherView& v, const SiteTable& st, const void* x, int64_t xcs, void* y, int64_t ycs,
              int64_t ncols, typename Cx<R>::T a, typename Cx<R>::T b, size_t smem, cudaStream_t s) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  // a tuned lane split wider than this call's vectors fill (fewer vectors than
  // the tuning, e.g. the chunks of a host call) is narrowed
  int ls = v.lane_split > 0 ? v.lane_split : 1;
  while (ls > 1 && (int64_t)TC * ls > ncols) ls >>= 1;
  if (v.block < 0 && ncols <= (int64_t)INT32_MAX) {
    // persistent grid: SMs x resident blocks of -v.block threads
    auto pk = k_gather_p<R, VM, SQUARE, W1, TC, BMODE>;
    allow_smem(pk, smem);
    const int threads = -v.block;
    int dev = 0, sms = 0, occ = 0;
    QOB_CUDA(cudaGetDevice(&dev));
    QOB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    QOB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk, threads, smem));
    if (occ > 0) {
      GatherView w = v;
      w.lane_split = ls;
      const int64_t jw = 32 / ls;
      w.jmul = chunk_multiplier((v.m + jw - 1) / jw);
      launch_kernel(v.pdl != 0, pk, dim3((unsigned)(sms * occ)), (unsigned)threads, smem, s, w, st, (const XT*)x,
                    xcs, (CT*)y, ycs, (int)ncols, a, b);
      QOB_LAUNCHED();
      return;
    }
  }
  auto kern = k_gather_j<R, VM, SQUARE, W1, TC, BMODE>;
  allow_smem(kern, smem);
  const int threads = v.block > 0 ? v.block : kThreads;
  const int64_t jpb = threads / ls;  // output indices per block
  const unsigned gx = (unsigned)((v.m + jpb - 1) / jpb);
  GatherView w = v;
  w.lane_split = ls;
  // a few waves of blocks: permuted so every SM's share mixes the whole index
  // range; many waves: in order (the hardware balances them, and neighbouring
  // blocks share the gathered input in L2)
  w.jmul = gx <= 4096 ? chunk_multiplier(gx) : 1;
  const int64_t per_y = (int64_t)TC * ls;  // vectors per grid row
  for (int64_t c0 = 0; c0 < ncols; c0 += (int64_t)65535 * per_y) {  // grid.y limit
    const int64_t nc = std::min<int64_t>(ncols - c0, (int64_t)65535 * per_y);
    launch_kernel(v.pdl != 0, kern, dim3(gx, (unsigned)((nc + per_y - 1) / per_y)), (unsigned)threads, smem, s, w,
                  st, (const XT*)x + c0 * xcs, xcs, (CT*)y + c0 * ycs, ycs, (int)nc, a, b);
    QOB_LAUNCHED();
  }
}

template <typename R, int VM, bool SQUARE, bool W1, int BMODE>
void launch_tc(const GatherView& v, const SiteTable& st, int tc, const void* x, int64_t xcs, void* y,
               int64_t ycs, int64_t ncols, typename Cx<R>::T a, typename Cx<R>::T b, size_t smem, cudaStream_t s) {
  switch (tc) {
    case 8:
      launch_j<R, VM, SQUARE, W1, 8, BMODE>(v, st, x, xcs, y, ycs, ncols, a, b, smem, s);
      break;
    case 4:
      launch_j<R, VM, SQUARE, W1, 4, BMODE>(v, st, x, xcs, y, ycs, ncols, a, b, smem, s);
      break;
    case 2:
      launch_j<R, VM, SQUARE, W1, 2, BMODE>(v, st, x, xcs, y, ycs, ncols, a, b, smem, s);
      break;
    default:
      launch_j<R, VM, SQUARE, W1, 1, BMODE>(v, st, x, xcs, y, ycs, ncols, a, b, smem, s);
  }
}

// k_gather_j2 (pairs of consecutive indices): grid over the m / 2 pairs as
// launch_j over indices.
template <typename R, int VM, int TC, int BMODE>
void launch_j2(const GatherView& v, const void* x, int64_t xcs, void* y, int64_t ycs, int64_t ncols,
               typename Cx<R>::T a, typename Cx<R>::T b, size_t smem, cudaStream_t s) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  int ls = v.lane_split > 0 ? v.lane_split : 1;
  while (ls > 1 && (int64_t)TC * ls > ncols) ls >>= 1;
  auto kern = k_gather_j2<R, VM, TC, BMODE>;
  allow_smem(kern, smem);
  const int threads = v.block > 0 ? v.block : kThreads;
  const int64_t ppb = threads / ls;  // pairs per block
  const unsigned gx = (unsigned)((v.m / 2 + ppb - 1) / ppb);
  GatherView w = v;
  w.lane_split = ls;
  w.jmul = gx <= 4096 ? chunk_multiplier(gx) : 1;
  const int64_t per_y = (int64_t)TC * ls;
  for (int64_t c0 = 0; c0 < ncols; c0 += (int64_t)65535 * per_y) {  // grid.y limit
    const int64_t nc = std::min<int64_t>(ncols - c0, (int64_t)65535 * per_y);
    launch_kernel(v.pdl != 0, kern, dim3(gx, (unsigned)((nc + per_y - 1) / per_y)), (unsigned)threads, smem, s, w,
                  (const XT*)x + c0 * xcs, xcs, (CT*)y + c0 * ycs, ycs, (int)nc, a, b);
    QOB_LAUNCHED();
  }
}

// Whether the pairs kernel can run this call: a compact plan of even size on
// contiguous vectors, 2 or 4 vectors per thread, and for ComplexF32 16-byte
// aligned pairs (an even vector stride on a 16-byte aligned base).
template <typename R>
bool pairs_fit(const GatherView& v, int tc, const void* x, int64_t xcs) {
  if (!v.pairs || !v.fast || v.m % 2 != 0 || (tc != 2 && tc != 4)) return false;
  if (sizeof(typename In<R>::T) == 8 && (((uintptr_t)x & 15) != 0 || (xcs & 1) != 0)) return false;
  return true;
}

// Shared memory of one staged-tile block at most (GB300: 227 KB per block)
constexpr size_t kTileSmemMax = 200 * 1024;

template <typename R, int VM, int BMODE>
void launch_tile_tc(const GatherView& v, int tc, const void* x, int64_t xcs, void* y, int64_t ycs, int64_t ncols,
                    typename Cx<R>::T a, typename Cx<R>::T b, cudaStream_t s) {
  switch (tc) {
    case 4:
      launch_t<R, VM, 4, BMODE>(v, x, xcs, y, ycs, ncols, a, b, s, v.status);
      break;
    case 2:
      launch_t<R, VM, 2, BMODE>(v, x, xcs, y, ycs, ncols, a, b, s, v.status);
      break;
    default:
      launch_t<R, VM, 1, BMODE>(v, x, xcs, y, ycs, ncols, a, b, s, v.status);
  }
}

template <typename R, int VM, bool SQUARE, int BMODE>
void dispatch_layout(const GatherView& v, const SiteTable& st, int tc, const void* x, int64_t xes,
                     int64_t xcs, void* y, int64_t yes, int64_t ycs, int64_t ncols, typename Cx<R>::T a, typename Cx<R>::T b,
                     cudaStream_t s) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  using ET = typename Ell<R, VM != kComplex>::T;
  GatherView w = v;
  size_t smem = (size_t)v.ngroups * (sizeof(GGroup) + (v.fast ? sizeof(int4) : 0));
  const size_t ell_bytes = (size_t)v.ell_slots * sizeof(ET);
  w.ell_smem = (v.ell_slots > 0 && ell_bytes <= kStageSlotsMax && smem + ell_bytes <= kSmemBudget) ? 1 : 0;
  if (w.ell_smem) smem += ell_bytes;
  if (xes == 1 && yes == 1) {
    if constexpr (SQUARE) {
      // staged tiles for compact plans (a tuned choice), when the tile and the
      // bulk copies fit this call; the slots are staged when the budget allows
      if (v.tile_bits > 0 && v.fast && tile_fits<R>(v, v.tile_bits, x, xcs, ncols)) {
        const int ttc = tc >= 4 ? 4 : tc;  // the tiled kernel takes 1, 2 or 4 vectors per thread
        int ls = v.lane_split > 0 ? v.lane_split : 1;
        while (ls > 1 && (int64_t)ttc * ls > ncols) ls >>= 1;
        GatherView t = v;
        t.ell_smem = 1;
        size_t need = tile_smem<XT, ET>(v.tile_bits, ttc * ls, v.ngroups, v.ell_slots, true);
        if (v.ell_slots <= 0 || (size_t)v.ell_slots * sizeof(ET) > kStageSlotsMax || need > kTileSmemMax) {
          t.ell_smem = 0;
          need = tile_smem<XT, ET>(v.tile_bits, ttc * ls, v.ngroups, v.ell_slots, false);
        }
        if (need <= kTileSmemMax) {
          launch_tile_tc<R, VM, BMODE>(t, ttc, x, xcs, y, ycs, ncols, a, b, s);
          return;
        }
      }
    }
    if constexpr (SQUARE && PairsOk<R, VM>::value) {
      if (v.all_w1 && pairs_fit<R>(v, tc, x, xcs)) {
        if (tc == 4)
          launch_j2<R, VM, 4, BMODE>(w, x, xcs, y, ycs, ncols, a, b, smem, s);
        else
          launch_j2<R, VM, 2, BMODE>(w, x, xcs, y, ycs, ncols, a, b, smem, s);
        return;
      }
    }
    if (SQUARE && v.all_w1)
      launch_tc<R, VM, SQUARE, true, BMODE>(w, st, tc, x, xcs, y, ycs, ncols, a, b, smem, s);
    else
      launch_tc<R, VM, SQUARE, false, BMODE>(w, st, tc, x, xcs, y, ycs, ncols, a, b, smem, s);
  } else {
    auto kern = k_gather_c<R, VM, SQUARE, BMODE>;
    allow_smem(kern, smem);
    const int threads = ncols >= 256 ? 256 : (int)((ncols + 31) / 32 * 32);
    for (int64_t c0 = 0; c0 < ncols; c0 += (int64_t)65535 * threads) {  // grid.y limit
      const int64_t nc = std::min<int64_t>(ncols - c0, (int64_t)65535 * threads);
      dim3 grid((unsigned)v.m, (unsigned)((nc + threads - 1) / threads));
      kern<<<grid, threads, smem, s>>>(w, st, (const XT*)x + c0 * xcs, xes, xcs, (CT*)y + c0 * ycs, yes, ycs,
                                       (int)nc, a, b);
      QOB_LAUNCHED();
    }
  }
}

template <typename R, int VM, bool SQUARE>
void dispatch_beta(const GatherView& v, const SiteTable& st, int tc, const void* x, int64_t xes, int64_t xcs,
                   void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha, c128 beta, cudaStream_t s) {
  typename Cx<R>::T a, b;
  using S = decltype(a.x);
  a.x = (S)alpha.re;
  a.y = (S)alpha.im;
  b.x = (S)beta.re;
  b.y = (S)beta.im;
  if (beta.re == 0.0 && beta.im == 0.0)
    dispatch_layout<R, VM, SQUARE, 0>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, a, b, s);
  else if (beta.im == 0.0)
    dispatch_layout<R, VM, SQUARE, 3>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, a, b, s);
  else
    dispatch_layout<R, VM, SQUARE, 2>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, a, b, s);
}

// One launch (or one column chunk per grid limit) of the fused gather in
// precision R.
template <typename R>
void dispatch(const GatherView& v, const SiteTable& st, int tc, const void* x, int64_t xes, int64_t xcs,
              void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha, c128 beta, cudaStream_t s) {
  if (v.real_vals) {
    if (v.square)
      dispatch_beta<R, kReal, true>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
    else
      dispatch_beta<R, kReal, false>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
  } else if (v.phased) {  // phased plans have a merged diagonal, hence a square basis
    dispatch_beta<R, kPhased, true>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
  } else {
    if (v.square)
      dispatch_beta<R, kComplex, true>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
    else
      dispatch_beta<R, kComplex, false>(v, st, tc, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, s);
  }
}

}  // namespace gather
}  // namespace qob
