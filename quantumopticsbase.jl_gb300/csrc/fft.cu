// fft.cu -- FFTOperator (src/particle.jl:196-535): the transform between a
// position grid and its momentum grid, applied to kets, bras and operators.
//
// The reference multiplies by a phase array (mul_before), runs FFTW's in-place
// fft!/bfft! over the transformed dimensions, and multiplies by a second phase
// array that includes 1/sqrt(N) (mul_after); bras and the rows of an operator
// multiplied from the right go through conj -> opposite-sign transform -> conj,
// which is the same-sign transform of the row with the two phase arrays
// swapped (the DFT matrix is symmetric).  Both phase arrays are Kronecker
// products of per-axis vectors, so a multi-dimensional transform is one pass per
// axis, each pass multiplying by its axis's phases.
//
// Each pass is one kernel: a block per line (the n elements of one axis of
// one vector), staged in shared memory; powers of two use the radix-2
// Stockham autosort FFT (Van Loan, Computational Frameworks for the FFT, 1992:
// log2 n stages, each reading one buffer and writing the other in natural
// order), other lengths a direct DFT over a twiddle table.  The last pass
// applies alpha and beta.
#include <cmath>
#include <type_traits>
#include <vector>

#include "k_gather.cuh"  // double-float helpers
#include "qob_internal.h"

namespace qob {
namespace {

using gather::DF;

// Element types per precision: G in memory (vectors, alpha, beta), S for the
// arithmetic (shared-memory lines, twiddles, phases).  The double-float form
// (ComplexF64 data) computes on (re hi, re lo, im hi, im lo) quadruples.
template <typename R>
struct FT;
template <>
struct FT<double> {
  using G = double2;
  using S = double2;
  static __device__ __forceinline__ S in(G g) { return g; }
};
template <>
struct FT<float> {
  using G = float2;
  using S = float2;
  static __device__ __forceinline__ S in(G g) { return g; }
};
template <>
struct FT<DF> {
  using G = double2;
  using S = float4;
  static __device__ __forceinline__ S in(G g) {
    const float2 a = gather::ff_split(g.x), b = gather::ff_split(g.y);
    return make_float4(a.x, a.y, b.x, b.y);
  }
};

template <typename CT>
__device__ __forceinline__ CT cm(CT a, CT b) {
  CT o;
  o.x = a.x * b.x - a.y * b.y;
  o.y = a.x * b.y + a.y * b.x;
  return o;
}
__device__ __forceinline__ float4 cm(float4 a, float4 b) {
  const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
  const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
  const float2 re = gather::ff_add(gather::ff_mul(ar, br), gather::ff_neg(gather::ff_mul(ai, bi)));
  const float2 im = gather::ff_add(gather::ff_mul(ar, bi), gather::ff_mul(ai, br));
  return make_float4(re.x, re.y, im.x, im.y);
}
template <typename CT>
__device__ __forceinline__ CT cadd(CT a, CT b) {
  CT o;
  o.x = a.x + b.x;
  o.y = a.y + b.y;
  return o;
}
template <typename CT>
__device__ __forceinline__ CT csub(CT a, CT b) {
  CT o;
  o.x = a.x - b.x;
  o.y = a.y - b.y;
  return o;
}
__device__ __forceinline__ float4 cadd(float4 a, float4 b) {
  const float2 re = gather::ff_add(make_float2(a.x, a.y), make_float2(b.x, b.y));
  const float2 im = gather::ff_add(make_float2(a.z, a.w), make_float2(b.z, b.w));
  return make_float4(re.x, re.y, im.x, im.y);
}
__device__ __forceinline__ float4 csub(float4 a, float4 b) { return cadd(a, make_float4(-b.x, -b.y, -b.z, -b.w)); }
// v times +i or -i exactly (a swap and a sign change)
template <typename CT>
__device__ __forceinline__ CT mul_i(CT v, bool plus) {
  CT o;
  o.x = plus ? -v.y : v.y;
  o.y = plus ? v.x : -v.x;
  return o;
}
__device__ __forceinline__ float4 mul_i(float4 v, bool plus) {
  return plus ? make_float4(-v.z, -v.w, v.x, v.y) : make_float4(v.z, v.w, -v.x, -v.y);
}
// the high part of the imaginary part (its sign)
__device__ __forceinline__ double im_hi(double2 v) { return v.y; }
__device__ __forceinline__ float im_hi(float2 v) { return v.y; }
__device__ __forceinline__ float im_hi(float4 v) { return v.z; }
template <typename CT>
__device__ __forceinline__ CT czero() {
  CT o;
  o.x = 0;
  o.y = 0;
  return o;
}
template <>
__device__ __forceinline__ float4 czero<float4>() {
  return make_float4(0.f, 0.f, 0.f, 0.f);
}

// Element k of line `line`: the line is (vector c, position p among the len/n
// lines of one vector); p = lo + stride * hi with lo < stride.
__device__ __forceinline__ int64_t line_base(int64_t line, int64_t lines_per_vec, int64_t stride, int64_t n,
                                             int64_t es, int64_t cs) {
  int64_t c, p, lo, hi;
  udivmod(line, lines_per_vec, c, p);
  udivmod(p, stride, hi, lo);
  return c * cs + (lo + hi * stride * n) * es;
}

template <typename R, bool FINAL, int BMODE>
__device__ __forceinline__ void store(typename FT<R>::G* y, typename FT<R>::S v, typename FT<R>::S post,
                                      typename FT<R>::G alpha, typename FT<R>::G beta) {
  using G = typename FT<R>::G;
  G o;
  if constexpr (std::is_same<R, DF>::value) {
    const float4 w = cm(v, post);  // double-float, then joined; alpha / beta in FP64
    o = make_double2(gather::ff_join(w.x, w.y), gather::ff_join(w.z, w.w));
  } else {
    o = cm(v, post);
  }
  if (FINAL) {
    o = cm(o, alpha);
    if (BMODE != 0) {
      const G b = cm(*y, beta);
      o.x += b.x;
      o.y += b.y;
    }
  }
  *y = o;
}

// Radix-2 Stockham FFT in shared memory: a holds n = 2^log2n inputs, b is
// scratch; twiddle m of the length-n transform is tw[m * tws].  Returns the
// buffer that holds the output (natural order).  The trivial twiddles (1 in
// every stage's first butterfly and in the first stage, +-i in the second
// stage) are applied without multiplications.
template <typename CT>
__device__ __forceinline__ CT* stockham(CT* a, CT* b, int64_t n, int log2n, const CT* __restrict__ tw,
                                        int64_t tws) {
  const int64_t half = n >> 1;
  // sign of the transform: w^(n/4) = +i (bfft) or -i (fft)
  const bool plus_i = log2n >= 2 ? im_hi(tw[(int64_t(1) << (log2n - 2)) * tws]) > 0 : true;
  for (int st = 0; st < log2n; ++st) {
    const int64_t ns = int64_t(1) << st;  // half-length of the sub-transforms being merged
    for (int64_t j = threadIdx.x; j < half; j += blockDim.x) {
      const int64_t k = j & (ns - 1);
      const CT u = a[j];
      CT v = a[j + half];
      if (st == 1 && k == 1) {
        v = mul_i(v, plus_i);  // twiddle w^(n/4) = +i or -i exactly
      } else if (st >= 2 && k != 0) {
        v = cm(v, tw[(k << (log2n - 1 - st)) * tws]);  // k == 0: twiddle 1
      }
      const int64_t i0 = 2 * j - k;
      b[i0] = cadd(u, v);
      b[i0 + ns] = csub(u, v);
    }
    __syncthreads();
    CT* t = a;
    a = b;
    b = t;
  }
  return a;
}

// Four-step FFT of long lines over many blocks (Bailey 1990): n = n1 * n2,
// element j = j2 + n2 * j1.  Pass A: for each (line, j2) the length-n1 FFT
// over j1, times w_n^(j2 k1), into scratch[line][j2 + n2 k1].  Pass B: for each
// (line, k1) the length-n2 FFT over j2 gives element k = k1 + n1 k2.
template <typename R>
__global__ void __launch_bounds__(256) k_fft4_a(int64_t n1, int log2n1, int64_t n2, int64_t stride,
                                                int64_t lines_per_vec, const typename FT<R>::G* __restrict__ x,
                                                int64_t xes, int64_t xcs, typename FT<R>::S* __restrict__ scratch,
                                                const typename FT<R>::S* __restrict__ twn,
                                                const typename FT<R>::S* __restrict__ pre) {
  using CT = typename FT<R>::S;
  extern __shared__ __align__(16) unsigned char smem[];
  CT* a = reinterpret_cast<CT*>(smem);
  CT* b = a + n1;
  const int64_t n = n1 * n2;
  const int64_t line = blockIdx.x / n2, j2 = blockIdx.x - line * n2;
  const typename FT<R>::G* xl = x + line_base(line, lines_per_vec, stride, n, xes, xcs);
  const int64_t se = stride * xes;
  for (int64_t j1 = threadIdx.x; j1 < n1; j1 += blockDim.x) {
    const int64_t j = j2 + n2 * j1;
    a[j1] = cm(FT<R>::in(xl[j * se]), pre[j]);
  }
  __syncthreads();
  const CT* r = stockham(a, b, n1, log2n1, twn, n2);
  CT* out = scratch + line * n;
  // n is a power of two on this path: the twiddle index wraps with a mask
  for (int64_t k1 = threadIdx.x; k1 < n1; k1 += blockDim.x) out[j2 + n2 * k1] = cm(r[k1], twn[(j2 * k1) & (n - 1)]);
}

template <typename R, int BMODE>
__global__ void __launch_bounds__(256) k_fft4_b(int64_t n1, int64_t n2, int log2n2, int64_t stride,
                                                int64_t lines_per_vec, const typename FT<R>::S* __restrict__ scratch,
                                                typename FT<R>::G* __restrict__ y, int64_t yes, int64_t ycs,
                                                const typename FT<R>::S* __restrict__ twn,
                                                const typename FT<R>::S* __restrict__ post, typename FT<R>::G alpha,
                                                typename FT<R>::G beta) {
  using CT = typename FT<R>::S;
  extern __shared__ __align__(16) unsigned char smem[];
  CT* a = reinterpret_cast<CT*>(smem);
  CT* b = a + n2;
  const int64_t n = n1 * n2;
  const int64_t line = blockIdx.x / n1, k1 = blockIdx.x - line * n1;
  const CT* in = scratch + line * n + n2 * k1;
  for (int64_t j2 = threadIdx.x; j2 < n2; j2 += blockDim.x) a[j2] = in[j2];
  __syncthreads();
  const CT* r = stockham(a, b, n2, log2n2, twn, n1);
  typename FT<R>::G* yl = y + line_base(line, lines_per_vec, stride, n, yes, ycs);
  const int64_t so = stride * yes;
  for (int64_t k2 = threadIdx.x; k2 < n2; k2 += blockDim.x) {
    const int64_t k = k1 + n1 * k2;
    store<R, true, BMODE>(yl + k * so, r[k2], post[k], alpha, beta);
  }
}

// Radix-2 Stockham FFT of one line in shared memory (n a power of two, n >= 2).
template <typename R, bool FINAL, int BMODE>
__global__ void __launch_bounds__(256) k_fft_pow2(int64_t n, int log2n, int64_t stride, int64_t lines_per_vec,
                                                  const typename FT<R>::G* __restrict__ x, int64_t xes, int64_t xcs,
                                                  typename FT<R>::G* __restrict__ y, int64_t yes, int64_t ycs,
                                                  const typename FT<R>::S* __restrict__ tw,
                                                  const typename FT<R>::S* __restrict__ pre,
                                                  const typename FT<R>::S* __restrict__ post, typename FT<R>::G alpha,
                                                  typename FT<R>::G beta) {
  using CT = typename FT<R>::S;
  extern __shared__ __align__(16) unsigned char smem[];
  CT* a = reinterpret_cast<CT*>(smem);
  CT* b = a + n;
  const int64_t line = blockIdx.x;
  const typename FT<R>::G* xl = x + line_base(line, lines_per_vec, stride, n, xes, xcs);
  const int64_t se = stride * xes;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) a[k] = cm(FT<R>::in(xl[k * se]), pre[k]);
  __syncthreads();
  a = stockham(a, b, n, log2n, tw, 1);
  typename FT<R>::G* yl = y + line_base(line, lines_per_vec, stride, n, yes, ycs);
  const int64_t so = stride * yes;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) store<R, FINAL, BMODE>(yl + k * so, a[k], post[k], alpha, beta);
}

// Direct DFT of one line (any n): out_k = sum_j in_j * w^((j k) mod n).
template <typename R, bool FINAL, int BMODE>
__global__ void __launch_bounds__(256) k_dft_line(int64_t n, int64_t stride, int64_t lines_per_vec,
                                                  const typename FT<R>::G* __restrict__ x, int64_t xes, int64_t xcs,
                                                  typename FT<R>::G* __restrict__ y, int64_t yes, int64_t ycs,
                                                  const typename FT<R>::S* __restrict__ tw,
                                                  const typename FT<R>::S* __restrict__ pre,
                                                  const typename FT<R>::S* __restrict__ post, typename FT<R>::G alpha,
                                                  typename FT<R>::G beta) {
  using CT = typename FT<R>::S;
  extern __shared__ __align__(16) unsigned char smem[];
  CT* a = reinterpret_cast<CT*>(smem);
  const int64_t line = blockIdx.x;
  const typename FT<R>::G* xl = x + line_base(line, lines_per_vec, stride, n, xes, xcs);
  const int64_t se = stride * xes;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) a[k] = cm(FT<R>::in(xl[k * se]), pre[k]);
  __syncthreads();
  typename FT<R>::G* yl = y + line_base(line, lines_per_vec, stride, n, yes, ycs);
  const int64_t so = stride * yes;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
    CT acc = czero<CT>();
    int64_t idx = 0;
    for (int64_t j = 0; j < n; ++j) {
      acc = cadd(acc, cm(a[j], tw[idx]));
      idx += k;
      if (idx >= n) idx -= n;
    }
    store<R, FINAL, BMODE>(yl + k * so, acc, post[k], alpha, beta);
  }
}

template <typename R, bool FINAL, int BMODE>
void launch_typed(const FftAxis& ax, int64_t len, const void* x, int64_t xes, int64_t xcs, void* y, int64_t yes,
                  int64_t ycs, int64_t ncols, c128 alpha, c128 beta, void* scratch, cudaStream_t s) {
  using G = typename FT<R>::G;  // vectors, alpha, beta
  using CT = typename FT<R>::S;  // twiddles, phases, shared memory, scratch
  G a, b;
  using E = decltype(a.x);
  a.x = (E)alpha.re;
  a.y = (E)alpha.im;
  b.x = (E)beta.re;
  b.y = (E)beta.im;
  const int64_t lines_per_vec = len / ax.n;
  int dev = 0, sms = 0;
  QOB_CUDA(cudaGetDevice(&dev));
  QOB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t lines = lines_per_vec * ncols;
  if (FINAL && ax.n1 > 0 && scratch && lines < sms && lines * ax.n2 <= INT32_MAX) {
    // few long lines: spread each over n2 + n1 blocks (two launches)
    int l1 = 0, l2 = 0;
    while ((int64_t(1) << l1) < ax.n1) ++l1;
    while ((int64_t(1) << l2) < ax.n2) ++l2;
    const int ta = (int)std::min<int64_t>(256, std::max<int64_t>(32, ax.n1 / 2));
    const int tb = (int)std::min<int64_t>(256, std::max<int64_t>(32, ax.n2 / 2));
    const size_t sa = 2 * (size_t)ax.n1 * sizeof(CT), sb = 2 * (size_t)ax.n2 * sizeof(CT);
    k_fft4_a<R><<<(unsigned)(lines * ax.n2), ta, sa, s>>>(ax.n1, l1, ax.n2, ax.stride, lines_per_vec, (const G*)x,
                                                         xes, xcs, (CT*)scratch, (const CT*)ax.tw_full.p,
                                                         (const CT*)ax.pre.p);
    QOB_LAUNCHED();
    k_fft4_b<R, BMODE><<<(unsigned)(lines * ax.n1), tb, sb, s>>>(ax.n1, ax.n2, l2, ax.stride, lines_per_vec,
                                                                 (const CT*)scratch, (G*)y, yes, ycs,
                                                                 (const CT*)ax.tw_full.p, (const CT*)ax.post.p, a, b);
    QOB_LAUNCHED();
    return;
  }
  const int threads = (int)std::min<int64_t>(256, std::max<int64_t>(32, ax.pow2 ? ax.n / 2 : ax.n));
  // whole vectors per launch, at most 2^31 - 1 lines (blocks)
  const int64_t vec_per_launch = std::max<int64_t>(1, (int64_t)INT32_MAX / lines_per_vec);
  for (int64_t c0 = 0; c0 < ncols; c0 += vec_per_launch) {
    const int64_t nl = std::min<int64_t>(ncols - c0, vec_per_launch) * lines_per_vec;
    const G* xs = (const G*)x + c0 * xcs;
    G* ys = (G*)y + c0 * ycs;
    if (ax.pow2) {
      const size_t smem = 2 * (size_t)ax.n * sizeof(CT);
      auto k = k_fft_pow2<R, FINAL, BMODE>;
      if (smem > 48 * 1024) QOB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int log2n = 0;
      while ((int64_t(1) << log2n) < ax.n) ++log2n;
      k<<<(unsigned)nl, threads, smem, s>>>(ax.n, log2n, ax.stride, lines_per_vec, xs, xes, xcs, ys, yes, ycs,
                                            (const CT*)ax.tw.p, (const CT*)ax.pre.p, (const CT*)ax.post.p, a, b);
    } else {
      const size_t smem = (size_t)ax.n * sizeof(CT);
      auto k = k_dft_line<R, FINAL, BMODE>;
      if (smem > 48 * 1024) QOB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k<<<(unsigned)nl, threads, smem, s>>>(ax.n, ax.stride, lines_per_vec, xs, xes, xcs, ys, yes, ycs,
                                            (const CT*)ax.tw.p, (const CT*)ax.pre.p, (const CT*)ax.post.p, a, b);
    }
    QOB_LAUNCHED();
  }
}

void upload_prec(DeviceBuf& d, const std::vector<c128>& v, int precision, bool ff) {
  if (ff) {  // (re hi, re lo, im hi, im lo)
    std::vector<float> q(4 * v.size());
    for (size_t i = 0; i < v.size(); ++i) {
      const float rh = (float)v[i].re, ih = (float)v[i].im;
      q[4 * i] = rh;
      q[4 * i + 1] = (float)(v[i].re - (double)rh);
      q[4 * i + 2] = ih;
      q[4 * i + 3] = (float)(v[i].im - (double)ih);
    }
    d.upload(q.data(), q.size() * sizeof(float));
  } else if (precision == QOB_C128) {
    d.upload(v.data(), v.size() * sizeof(c128));
  } else {
    std::vector<c64> f(v.size());
    for (size_t i = 0; i < v.size(); ++i) f[i] = {(float)v[i].re, (float)v[i].im};
    d.upload(f.data(), f.size() * sizeof(c64));
  }
}

}  // namespace

void launch_fft_pass(int precision, const FftAxis& ax, int64_t len, const void* x, int64_t xes, int64_t xcs,
                     void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha, c128 beta, bool final,
                     void* scratch, cudaStream_t s, bool ff) {
  const bool b0 = beta.re == 0.0 && beta.im == 0.0;
  if (ff) {
    if (!final) launch_typed<DF, false, 0>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
    else if (b0) launch_typed<DF, true, 0>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
    else launch_typed<DF, true, 2>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
  } else if (precision == QOB_C128) {
    if (!final) launch_typed<double, false, 0>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
    else if (b0) launch_typed<double, true, 0>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
    else launch_typed<double, true, 2>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
  } else {
    if (!final) launch_typed<float, false, 0>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
    else if (b0) launch_typed<float, true, 0>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
    else launch_typed<float, true, 2>(ax, len, x, xes, xcs, y, yes, ycs, ncols, alpha, beta, scratch, s);
  }
}

// LEFT (kets, operator columns): pre = before, post = after.  RIGHT (bras,
// operator rows): pre = after, post = before, same sign.
std::unique_ptr<Plan> compile_fft(const NodeP& op, int side, int precision_code) {
  const bool ff = precision_code == QOB_C128X;
  const int precision = ff ? QOB_C128 : precision_code;
  auto P = std::make_unique<Plan>();
  P->kind = Plan::Kind::Fft;
  P->side = side;
  P->precision = precision;
  P->ff = ff;
  P->m = side == QOB_RIGHT ? op->n : op->m;
  P->n = side == QOB_RIGHT ? op->m : op->n;
  P->root = op.get();
  const std::vector<int64_t>& shape = op->shape_l;
  int64_t off = 0;
  for (size_t a = 0; a < op->fft_sites.size(); ++a) {
    const int site = op->fft_sites[a];
    FftAxis ax;
    ax.n = shape[site];
    ax.stride = 1;
    for (int q = 0; q < site; ++q) ax.stride *= shape[q];
    ax.pow2 = (ax.n & (ax.n - 1)) == 0 && ax.n >= 2;
    const size_t esz = precision == QOB_C128 ? 16 : 8;
    const size_t smem = (ax.pow2 ? 2 : 1) * (size_t)ax.n * esz;
    if (smem > 200 * 1024) fail(QOB_ERR_UNSUPPORTED, "FFT axis too long for one block's shared memory");
    const double sgn = op->fft_sign[a] < 0 ? -1.0 : 1.0;
    const int64_t ntw = ax.pow2 ? ax.n / 2 : ax.n;
    std::vector<c128> tw((size_t)std::max<int64_t>(ntw, 1));
    for (int64_t m = 0; m < ntw; ++m) {
      const double th = 6.283185307179586476925286766559 * (double)m / (double)ax.n;
      tw[(size_t)m] = {std::cos(th), sgn * std::sin(th)};
    }
    std::vector<c128> before(op->fft_before.begin() + off, op->fft_before.begin() + off + ax.n);
    std::vector<c128> after(op->fft_after.begin() + off, op->fft_after.begin() + off + ax.n);
    off += ax.n;
    upload_prec(ax.tw, tw, precision, ff);
    if (ax.pow2 && ax.n >= 512) {
      int l = 0;
      while ((int64_t(1) << l) < ax.n) ++l;
      ax.n1 = int64_t(1) << (l / 2);
      ax.n2 = ax.n / ax.n1;
      std::vector<c128> full((size_t)ax.n);
      for (int64_t m = 0; m < ax.n; ++m) {
        const double th = 6.283185307179586476925286766559 * (double)m / (double)ax.n;
        full[(size_t)m] = {std::cos(th), sgn * std::sin(th)};
      }
      upload_prec(ax.tw_full, full, precision, ff);
    }
    upload_prec(ax.pre, side == QOB_RIGHT ? after : before, precision, ff);
    upload_prec(ax.post, side == QOB_RIGHT ? before : after, precision, ff);
    P->fft.push_back(std::move(ax));
  }
  return P;
}

}  // namespace qob

namespace {
qob_op* wrap_node(qob::NodeP n) {
  auto* h = new qob_op;
  h->node = std::move(n);
  return h;
}
}  // namespace

extern "C" int qob_op_fft(qob_ctx* ctx, int nsub, const int64_t* shape, int naxes, const int64_t* axes,
                          const int* sign, const double* before, const double* after, qob_op** out) {
  if (!ctx) return QOB_ERR_ARG;
  try {
    using namespace qob;
    if (!out || nsub < 1 || nsub > kMaxSites || !shape || naxes < 1 || naxes > nsub || !axes || !sign || !before ||
        !after)
      fail(QOB_ERR_ARG, "qob_op_fft: bad arguments");
    auto nd = std::make_shared<OpNode>();
    nd->kind = Kind::Fft;
    nd->shape_l.assign(shape, shape + nsub);
    nd->shape_r = nd->shape_l;
    int64_t len = 1;
    for (int i = 0; i < nsub; ++i) {
      if (shape[i] < 1) fail(QOB_ERR_ARG, "qob_op_fft: bad subsystem length");
      len *= shape[i];
    }
    if (len > INT32_MAX) fail(QOB_ERR_UNSUPPORTED, "dimension exceeds 2^31-1");
    nd->m = nd->n = len;
    int64_t total = 0;
    for (int a = 0; a < naxes; ++a) {
      if (axes[a] < 1 || axes[a] > nsub || (a > 0 && axes[a] <= axes[a - 1]))
        fail(QOB_ERR_ARG, "qob_op_fft: axes must be increasing 1-based subsystem indices");
      nd->fft_sites.push_back((int)axes[a] - 1);
      nd->fft_sign.push_back(sign[a] < 0 ? -1 : 1);
      total += shape[axes[a] - 1];
    }
    for (int64_t k = 0; k < total; ++k) {
      nd->fft_before.push_back({before[2 * k], before[2 * k + 1]});
      nd->fft_after.push_back({after[2 * k], after[2 * k + 1]});
    }
    *out = wrap_node(nd);
    return QOB_OK;
  } catch (const qob::Error& e) {
    ctx->c.err = e.msg;
    return e.code;
  }
}
