// k_misc.cu -- the smaller kernels of the application path:
//   * beta scaling / zero fill            (_zero_op_mul!, src/operators_lazysum.jl:179-186)
//   * y = alpha x + beta y                (_tp_sum_matmul! with no factors, :453-458)
//   * dense operator times vectors        (mul! -> BLAS, src/operators_dense.jl:394-396)
//   * one mode product of a factor        (_tp_matmul_first!/_mid!/_last!,
//                                          src/operators_lazytensor.jl:281-428)
//   * FP64 reductions: norm, dot          (src/states.jl:89, src/operators.jl:119)
#include <cuda_runtime.h>

#include <algorithm>

#include "k_gather.cuh"  // double-float helpers (ff_join, AccFF)
#include "qob_internal.h"

namespace qob {

namespace {

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

template <typename CT>
__device__ __forceinline__ CT mk(double re, double im) {
  CT o;
  o.x = (decltype(o.x))re;
  o.y = (decltype(o.y))im;
  return o;
}

// ---------------------------------------------------------------------------
template <typename CT>
__global__ void k_scale(CT* y, int64_t rows, int64_t cols, int64_t lr, int64_t lc, double br,
                        double bi) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  int64_t c, r;
  udivmod(i, rows, c, r);
  CT* p = y + r * lr + c * lc;
  if (br == 0.0 && bi == 0.0) {
    *p = mk<CT>(0.0, 0.0);
  } else {
    CT o = *p;
    double re = br * (double)o.x - bi * (double)o.y;
    double im = br * (double)o.y + bi * (double)o.x;
    *p = mk<CT>(re, im);
  }
}

// y[e, c] = alpha * x[e, c] + beta * y[e, c]   (beta == 0: y not read)
template <typename CT, typename R>
__global__ void k_axpby(const CT* __restrict__ x, int64_t xes, int64_t xcs, CT* __restrict__ y,
                        int64_t yes, int64_t ycs, int64_t len, int64_t ncols, double ar, double ai,
                        double br, double bi) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= len * ncols) return;
  int64_t c, e;
  udivmod(i, len, c, e);
  CT xv = x[e * xes + c * xcs];
  R re = (R)ar * xv.x - (R)ai * xv.y;
  R im = (R)ar * xv.y + (R)ai * xv.x;
  CT* yp = y + e * yes + c * ycs;
  if (br != 0.0 || bi != 0.0) {
    CT o = *yp;
    re += (R)br * o.x - (R)bi * o.y;
    im += (R)br * o.y + (R)bi * o.x;
  }
  *yp = mk<CT>(re, im);
}

// Dense operator (m x n, column-major) times ncols vectors.  A thread owns one
// row i and a tile of TC vectors (each A element it loads serves all of them);
// blocks split the columns k into kchunks ranges so that a tall-skinny product
// (one ket, m ~ 1000) still fills the GPU.  With one range the thread writes
// alpha * acc + beta * y; otherwise it writes its partial sum to part[z][c][i]
// and k_dense_reduce adds the ranges in order (deterministic) and combines.
template <typename CT, typename R, int TC>
__global__ void __launch_bounds__(128) k_dense(const CT* __restrict__ a, int64_t m, int64_t n,
                                               const CT* __restrict__ x, int64_t xes, int64_t xcs,
                                               CT* __restrict__ y, int64_t yes, int64_t ycs, int64_t ncols,
                                               int64_t kc, CT* __restrict__ part, double ar, double ai,
                                               double br, double bi) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.y * TC;
  if (i >= m) return;
  const int nt = (int)(ncols - c0 < TC ? ncols - c0 : TC);
  const int64_t k0 = (int64_t)blockIdx.z * kc, k1 = k0 + kc < n ? k0 + kc : n;
  R sre[TC], sim[TC];
#pragma unroll
  for (int t = 0; t < TC; ++t) sre[t] = sim[t] = 0;
  const CT* xc = x + c0 * xcs;
  for (int64_t k = k0; k < k1; ++k) {
    const CT av = a[i + k * m];
#pragma unroll
    for (int t = 0; t < TC; ++t) {
      if (t < nt) {
        const CT xv = xc[t * xcs + k * xes];
        sre[t] = fma(av.x, xv.x, sre[t]);
        sre[t] = fma(-av.y, xv.y, sre[t]);
        sim[t] = fma(av.x, xv.y, sim[t]);
        sim[t] = fma(av.y, xv.x, sim[t]);
      }
    }
  }
  if (part) {
#pragma unroll
    for (int t = 0; t < TC; ++t)
      if (t < nt) part[((int64_t)blockIdx.z * ncols + c0 + t) * m + i] = mk<CT>(sre[t], sim[t]);
    return;
  }
#pragma unroll
  for (int t = 0; t < TC; ++t) {
    if (t < nt) {
      R re = (R)ar * sre[t] - (R)ai * sim[t];
      R im = (R)ar * sim[t] + (R)ai * sre[t];
      CT* yp = y + i * yes + (c0 + t) * ycs;
      if (br != 0.0 || bi != 0.0) {
        const CT o = *yp;
        re += (R)br * o.x - (R)bi * o.y;
        im += (R)br * o.y + (R)bi * o.x;
      }
      *yp = mk<CT>(re, im);
    }
  }
}

// Double-float forms (ComplexF64 data, QOB_C128X): the operator factor is
// stored as (re hi, re lo, im hi, im lo) quadruples, x arrives split the same
// way (k_ff_split), the sums are FP32 pairs, joined to double for the FP64
// alpha / beta epilogue (or for the partial sums of a split product).
__device__ __forceinline__ double2 ff_total(const gather::AccFF& acc) {
  return make_double2(gather::ff_join(acc.rh, acc.rl), gather::ff_join(acc.ih, acc.il));
}
__device__ __forceinline__ void combine64(double2* yp, double2 v, double ar, double ai, double br, double bi) {
  double re = ar * v.x - ai * v.y;
  double im = ar * v.y + ai * v.x;
  if (br != 0.0 || bi != 0.0) {
    const double2 o = *yp;
    re += br * o.x - bi * o.y;
    im += br * o.y + bi * o.x;
  }
  *yp = make_double2(re, im);
}

template <int TC>
__global__ void __launch_bounds__(128) k_dense_ff(const float4* __restrict__ a, int64_t m, int64_t n,
                                                  const float4* __restrict__ x, int64_t xes, int64_t xcs,
                                                  double2* __restrict__ y, int64_t yes, int64_t ycs, int64_t ncols,
                                                  int64_t kc, double2* __restrict__ part, double ar, double ai,
                                                  double br, double bi) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.y * TC;
  if (i >= m) return;
  const int nt = (int)(ncols - c0 < TC ? ncols - c0 : TC);
  const int64_t k0 = (int64_t)blockIdx.z * kc, k1 = k0 + kc < n ? k0 + kc : n;
  gather::AccFF acc[TC];
#pragma unroll
  for (int t = 0; t < TC; ++t) acc[t].zero();
  const float4* xc = x + c0 * xcs;
  for (int64_t k = k0; k < k1; ++k) {
    const float4 av = a[i + k * m];
#pragma unroll
    for (int t = 0; t < TC; ++t)
      if (t < nt) acc[t].mac(av, xc[t * xcs + k * xes]);
  }
#pragma unroll
  for (int t = 0; t < TC; ++t) {
    if (t < nt) {
      const double2 v = ff_total(acc[t]);
      if (part)
        part[((int64_t)blockIdx.z * ncols + c0 + t) * m + i] = v;
      else
        combine64(y + i * yes + (c0 + t) * ycs, v, ar, ai, br, bi);
    }
  }
}

__global__ void k_modek_ff(const float4* __restrict__ A, int64_t s1, int64_t dout, int64_t din, int64_t s3,
                           const float4* __restrict__ x, int64_t xes, int64_t xcs, double2* __restrict__ y,
                           int64_t yes, int64_t ycs, int64_t ncols, double ar, double ai, double br, double bi) {
  const int64_t len = s1 * dout * s3;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = blockIdx.y;
  if (i >= len || c >= ncols) return;
  int64_t a, t, j, b;
  udivmod(i, s1, t, a);
  udivmod(t, dout, b, j);
  const float4* xc = x + c * xcs;
  gather::AccFF acc;
  acc.zero();
  for (int64_t k = 0; k < din; ++k) acc.mac(A[j + k * dout], xc[(a + s1 * (k + din * b)) * xes]);
  combine64(y + i * yes + c * ycs, ff_total(acc), ar, ai, br, bi);
}

// The k ranges' partial sums of k_dense added in order, then alpha / beta.
template <typename CT, typename R>
__global__ void k_dense_reduce(const CT* __restrict__ part, int kchunks, int64_t m, int64_t ncols,
                               CT* __restrict__ y, int64_t yes, int64_t ycs, double ar, double ai, double br,
                               double bi) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = blockIdx.y;
  if (i >= m) return;
  R sre = 0, sim = 0;
  for (int z = 0; z < kchunks; ++z) {
    const CT p = part[((int64_t)z * ncols + c) * m + i];
    sre += p.x;
    sim += p.y;
  }
  R re = (R)ar * sre - (R)ai * sim;
  R im = (R)ar * sim + (R)ai * sre;
  CT* yp = y + i * yes + c * ycs;
  if (br != 0.0 || bi != 0.0) {
    const CT o = *yp;
    re += (R)br * o.x - (R)bi * o.y;
    im += (R)br * o.y + (R)bi * o.x;
  }
  *yp = mk<CT>(re, im);
}

// One mode product: out[a, j, b] = alpha * sum_k A[j, k] in[a, k, b] + beta * out,
// a < s1, j < dout, b < s3; element e of vector c at x[e * xes + c * xcs].
// A non-square Eye is the truncated identity (src/operators_lazytensor.jl:348-371).
template <typename CT, typename R, bool EYE>
__global__ void k_modek(const CT* __restrict__ A, int64_t s1, int64_t dout, int64_t din, int64_t s3,
                        const CT* __restrict__ x, int64_t xes, int64_t xcs, CT* __restrict__ y,
                        int64_t yes, int64_t ycs, int64_t ncols, double ar, double ai, double br,
                        double bi) {
  const int64_t len = s1 * dout * s3;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = blockIdx.y;
  if (i >= len || c >= ncols) return;
  int64_t a, t, j, b;
  udivmod(i, s1, t, a);
  udivmod(t, dout, b, j);
  const CT* xc = x + c * xcs;
  R sre = 0, sim = 0;
  if (EYE) {
    if (j < din) {
      CT xv = xc[(a + s1 * (j + din * b)) * xes];
      sre = xv.x;
      sim = xv.y;
    }
  } else {
    for (int64_t k = 0; k < din; ++k) {
      CT av = A[j + k * dout];
      CT xv = xc[(a + s1 * (k + din * b)) * xes];
      sre = fma(av.x, xv.x, sre);
      sre = fma(-av.y, xv.y, sre);
      sim = fma(av.x, xv.y, sim);
      sim = fma(av.y, xv.x, sim);
    }
  }
  R re = (R)ar * sre - (R)ai * sim;
  R im = (R)ar * sim + (R)ai * sre;
  CT* yp = y + i * yes + c * ycs;
  if (br != 0.0 || bi != 0.0) {
    CT o = *yp;
    re += (R)br * o.x - (R)bi * o.y;
    im += (R)br * o.y + (R)bi * o.x;
  }
  *yp = mk<CT>(re, im);
}

// ---------------------------------------------------------------------------
// FP64 reductions in a fixed order: block partials (strided per thread, then a
// shared-memory tree), then one block sums the partials in index order.
constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 304;  // 2 x 152 SMs

template <typename CT>
__global__ void k_dot_partial(const CT* __restrict__ x, const CT* __restrict__ y, int64_t n,
                              double2* __restrict__ part) {
  __shared__ double sre[kRedThreads], sim[kRedThreads];
  double re = 0.0, im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kRedThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kRedThreads) {
    CT a = x[i], b = y[i];
    const double ax = a.x, ay = a.y, bx = b.x, by = b.y;
    // conj(a) * b
    re = fma(ax, bx, re);
    re = fma(ay, by, re);
    im = fma(ax, by, im);
    im = fma(-ay, bx, im);
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sre[threadIdx.x] += sre[threadIdx.x + w];
      sim[threadIdx.x] += sim[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sre[0], sim[0]);
}

// sum of x[i * stride] in the same fixed order as k_dot_partial
template <typename CT>
__global__ void k_strided_partial(const CT* __restrict__ x, int64_t n, int64_t stride, double2* __restrict__ part) {
  __shared__ double sre[kRedThreads], sim[kRedThreads];
  double re = 0.0, im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kRedThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kRedThreads) {
    const CT a = x[i * stride];
    re += (double)a.x;
    im += (double)a.y;
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sre[threadIdx.x] += sre[threadIdx.x + w];
      sim[threadIdx.x] += sim[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sre[0], sim[0]);
}

__global__ void k_dot_final(const double2* __restrict__ part, int nparts, double2* out) {
  __shared__ double sre[kRedThreads], sim[kRedThreads];
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < nparts; i += kRedThreads) {
    re += part[i].x;
    im += part[i].y;
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sre[threadIdx.x] += sre[threadIdx.x + w];
      sim[threadIdx.x] += sim[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = make_double2(sre[0], sim[0]);
}

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

void launch_scale(int precision, void* y, int64_t rows, int64_t cols, int64_t lr, int64_t lc,
                  c128 beta, cudaStream_t s) {
  if (beta.re == 1.0 && beta.im == 0.0) return;
  const int64_t n = rows * cols;
  if (n == 0) return;
  if (precision == QOB_C128)
    k_scale<double2><<<blocks_for(n, 256), 256, 0, s>>>((double2*)y, rows, cols, lr, lc, beta.re, beta.im);
  else
    k_scale<float2><<<blocks_for(n, 256), 256, 0, s>>>((float2*)y, rows, cols, lr, lc, beta.re, beta.im);
  QOB_LAUNCHED();
}

void launch_axpby(int precision, const void* x, int64_t xes, int64_t xcs, c128 alpha, void* y,
                  int64_t yes, int64_t ycs, c128 beta, int64_t len, int64_t ncols, cudaStream_t s) {
  const int64_t n = len * ncols;
  if (n == 0) return;
  if (precision == QOB_C128)
    k_axpby<double2, double><<<blocks_for(n, 256), 256, 0, s>>>(
        (const double2*)x, xes, xcs, (double2*)y, yes, ycs, len, ncols, alpha.re, alpha.im, beta.re, beta.im);
  else
    k_axpby<float2, float><<<blocks_for(n, 256), 256, 0, s>>>(
        (const float2*)x, xes, xcs, (float2*)y, yes, ycs, len, ncols, alpha.re, alpha.im, beta.re, beta.im);
  QOB_LAUNCHED();
}

namespace {
// k ranges per dense product: enough blocks for about eight per SM (fine
// enough that the last wave is short), sixteen for one ket per thread (a
// stream of the matrix, latency-bound: twice the warps in flight), each range
// at least 64 columns long
int dense_kchunks(int64_t m, int64_t n, int64_t ncols, int tc) {
  const int64_t blocks = ((m + 127) / 128) * ((ncols + tc - 1) / tc);
  const int64_t target = tc == 1 ? 2432 : 1216;
  int64_t kch = (target + blocks - 1) / blocks;
  kch = std::min<int64_t>(kch, std::max<int64_t>(1, n / 64));
  return (int)std::max<int64_t>(1, std::min<int64_t>(kch, 65535));
}

template <typename CT, typename R>
void dense_typed(const void* a, int64_t m, int64_t n, c128 alpha, const void* x, int64_t xes, int64_t xcs,
                 c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols, Workspace* ws, int slot,
                 cudaStream_t s) {
  const int tc = ncols >= 8 ? 8 : ncols >= 4 ? 4 : ncols >= 2 ? 2 : 1;
  int kch = ws ? dense_kchunks(m, n, ncols, tc) : 1;
  CT* part = nullptr;
  if (kch > 1) part = static_cast<CT*>(ws->get(slot, (size_t)kch * ncols * m * sizeof(CT)));
  const int64_t kc = (n + kch - 1) / kch;
  kch = (int)((n + kc - 1) / kc);
  const dim3 grid(blocks_for(m, 128), (unsigned)((ncols + tc - 1) / tc), (unsigned)kch);
  const CT* A = (const CT*)a;
  const CT* X = (const CT*)x;
  CT* Y = (CT*)y;
  switch (tc) {
    case 8:
      k_dense<CT, R, 8><<<grid, 128, 0, s>>>(A, m, n, X, xes, xcs, Y, yes, ycs, ncols, kc, part, alpha.re,
                                             alpha.im, beta.re, beta.im);
      break;
    case 4:
      k_dense<CT, R, 4><<<grid, 128, 0, s>>>(A, m, n, X, xes, xcs, Y, yes, ycs, ncols, kc, part, alpha.re,
                                             alpha.im, beta.re, beta.im);
      break;
    case 2:
      k_dense<CT, R, 2><<<grid, 128, 0, s>>>(A, m, n, X, xes, xcs, Y, yes, ycs, ncols, kc, part, alpha.re,
                                             alpha.im, beta.re, beta.im);
      break;
    default:
      k_dense<CT, R, 1><<<grid, 128, 0, s>>>(A, m, n, X, xes, xcs, Y, yes, ycs, ncols, kc, part, alpha.re,
                                             alpha.im, beta.re, beta.im);
  }
  QOB_LAUNCHED();
  if (part) {
    k_dense_reduce<CT, R><<<dim3(blocks_for(m, 128), (unsigned)ncols), 128, 0, s>>>(
        part, kch, m, ncols, Y, yes, ycs, alpha.re, alpha.im, beta.re, beta.im);
    QOB_LAUNCHED();
  }
}
void dense_ff(const void* a, int64_t m, int64_t n, c128 alpha, const void* x, int64_t xes, int64_t xcs,
              c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols, Workspace* ws, int slot,
              cudaStream_t s) {
  const int tc = ncols >= 4 ? 4 : ncols >= 2 ? 2 : 1;
  int kch = ws ? dense_kchunks(m, n, ncols, tc) : 1;
  double2* part = nullptr;
  if (kch > 1) part = static_cast<double2*>(ws->get(slot, (size_t)kch * ncols * m * sizeof(double2)));
  const int64_t kc = (n + kch - 1) / kch;
  kch = (int)((n + kc - 1) / kc);
  const dim3 grid(blocks_for(m, 128), (unsigned)((ncols + tc - 1) / tc), (unsigned)kch);
  const float4* A = (const float4*)a;
  const float4* X = (const float4*)x;
  double2* Y = (double2*)y;
  switch (tc) {
    case 4:
      k_dense_ff<4><<<grid, 128, 0, s>>>(A, m, n, X, xes, xcs, Y, yes, ycs, ncols, kc, part, alpha.re, alpha.im,
                                         beta.re, beta.im);
      break;
    case 2:
      k_dense_ff<2><<<grid, 128, 0, s>>>(A, m, n, X, xes, xcs, Y, yes, ycs, ncols, kc, part, alpha.re, alpha.im,
                                         beta.re, beta.im);
      break;
    default:
      k_dense_ff<1><<<grid, 128, 0, s>>>(A, m, n, X, xes, xcs, Y, yes, ycs, ncols, kc, part, alpha.re, alpha.im,
                                         beta.re, beta.im);
  }
  QOB_LAUNCHED();
  if (part) {
    k_dense_reduce<double2, double><<<dim3(blocks_for(m, 128), (unsigned)ncols), 128, 0, s>>>(
        part, kch, m, ncols, Y, yes, ycs, alpha.re, alpha.im, beta.re, beta.im);
    QOB_LAUNCHED();
  }
}
}  // namespace

void launch_dense(int precision, const void* a, int64_t m, int64_t n, c128 alpha, const void* x,
                  int64_t xes, int64_t xcs, c128 beta, void* y, int64_t yes, int64_t ycs,
                  int64_t ncols, cudaStream_t s, Workspace* ws, int slot, bool ff, bool dmma) {
  if (m == 0 || ncols == 0) return;
  const size_t esz = precision == QOB_C128 ? 16 : 8;
  if (ncols > 65535 * 8) {  // grid.y limit: split the vectors
    for (int64_t c0 = 0; c0 < ncols; c0 += 65535 * 8)
      launch_dense(precision, a, m, n, alpha, (const char*)x + c0 * xcs * esz, xes, xcs, beta,
                   (char*)y + c0 * ycs * esz, yes, ycs, std::min<int64_t>(65535 * 8, ncols - c0), s, ws, slot,
                   ff, dmma);
    return;
  }
  if (dmma && !ff && precision == QOB_C128 && n >= kDmmaMinK && ncols >= kDmmaMinCols) {
    launch_dense_dmma(a, m, n, alpha, x, xes, xcs, beta, y, yes, ycs, ncols, s, ws, slot);
    return;
  }
  if (ff)
    dense_ff(a, m, n, alpha, x, xes, xcs, beta, y, yes, ycs, ncols, ws, slot, s);
  else if (precision == QOB_C128)
    dense_typed<double2, double>(a, m, n, alpha, x, xes, xcs, beta, y, yes, ycs, ncols, ws, slot, s);
  else
    dense_typed<float2, float>(a, m, n, alpha, x, xes, xcs, beta, y, yes, ycs, ncols, ws, slot, s);
}

void launch_modek(int precision, const void* a, bool eye, int64_t s1, int64_t dout, int64_t din,
                  int64_t s3, c128 alpha, const void* x, int64_t xes, int64_t xcs, c128 beta,
                  void* y, int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s, bool ff, bool dmma) {
  const int64_t len = s1 * dout * s3;
  if (len == 0 || ncols == 0) return;
  if (dmma && !ff && !eye && precision == QOB_C128 && din >= kDmmaMinK && ncols >= kDmmaMinCols) {
    launch_modek_dmma(a, s1, dout, din, s3, alpha, x, xes, xcs, beta, y, yes, ycs, ncols, s);
    return;
  }
  const size_t esz = precision == QOB_C128 ? 16 : 8;
  if (ncols > 65535) {  // grid.y limit: split the vectors
    for (int64_t c0 = 0; c0 < ncols; c0 += 65535)
      launch_modek(precision, a, eye, s1, dout, din, s3, alpha, (const char*)x + c0 * xcs * esz, xes, xcs,
                   beta, (char*)y + c0 * ycs * esz, yes, ycs, std::min<int64_t>(65535, ncols - c0), s, ff, dmma);
    return;
  }
  dim3 grid(blocks_for(len, 256), (unsigned)ncols);
  if (ff && !eye) {
    k_modek_ff<<<grid, 256, 0, s>>>((const float4*)a, s1, dout, din, s3, (const float4*)x, xes, xcs, (double2*)y,
                                    yes, ycs, ncols, alpha.re, alpha.im, beta.re, beta.im);
  } else if (precision == QOB_C128) {
    if (eye)
      k_modek<double2, double, true><<<grid, 256, 0, s>>>(nullptr, s1, dout, din, s3, (const double2*)x, xes,
                                                          xcs, (double2*)y, yes, ycs, ncols, alpha.re,
                                                          alpha.im, beta.re, beta.im);
    else
      k_modek<double2, double, false><<<grid, 256, 0, s>>>((const double2*)a, s1, dout, din, s3,
                                                           (const double2*)x, xes, xcs, (double2*)y, yes,
                                                           ycs, ncols, alpha.re, alpha.im, beta.re, beta.im);
  } else {
    if (eye)
      k_modek<float2, float, true><<<grid, 256, 0, s>>>(nullptr, s1, dout, din, s3, (const float2*)x, xes, xcs,
                                                        (float2*)y, yes, ycs, ncols, alpha.re, alpha.im,
                                                        beta.re, beta.im);
    else
      k_modek<float2, float, false><<<grid, 256, 0, s>>>((const float2*)a, s1, dout, din, s3,
                                                         (const float2*)x, xes, xcs, (float2*)y, yes, ycs,
                                                         ncols, alpha.re, alpha.im, beta.re, beta.im);
  }
  QOB_LAUNCHED();
}

void reduce_strided_sum(Context& ctx, int precision, const void* x, int64_t n, int64_t stride, double* out,
                        cudaStream_t s) {
  if (ctx.reduce_buf.bytes < (kRedBlocks + 1) * sizeof(double2))
    ctx.reduce_buf.alloc((kRedBlocks + 1) * sizeof(double2));
  if (!ctx.reduce_host) QOB_CUDA(cudaMallocHost(&ctx.reduce_host, sizeof(double2)));
  double2* part = (double2*)ctx.reduce_buf.p;
  double2* res = part + kRedBlocks;
  if (precision == QOB_C128)
    k_strided_partial<double2><<<kRedBlocks, kRedThreads, 0, s>>>((const double2*)x, n, stride, part);
  else
    k_strided_partial<float2><<<kRedBlocks, kRedThreads, 0, s>>>((const float2*)x, n, stride, part);
  QOB_LAUNCHED();
  k_dot_final<<<1, kRedThreads, 0, s>>>(part, kRedBlocks, res);
  QOB_LAUNCHED();
  QOB_CUDA(cudaMemcpyAsync(ctx.reduce_host, res, sizeof(double2), cudaMemcpyDeviceToHost, s));
  QOB_CUDA(cudaStreamSynchronize(s));
  const double2 r = *(const double2*)ctx.reduce_host;
  out[0] = r.x;
  out[1] = r.y;
}

// result: interleaved complex dot (norm: sqrt of the real part in out[0]).
void reduce_dot(Context& ctx, int precision, const void* x, const void* y, int64_t n, bool norm,
                double* out, cudaStream_t s) {
  if (ctx.reduce_buf.bytes < (kRedBlocks + 1) * sizeof(double2))
    ctx.reduce_buf.alloc((kRedBlocks + 1) * sizeof(double2));
  if (!ctx.reduce_host) QOB_CUDA(cudaMallocHost(&ctx.reduce_host, sizeof(double2)));
  double2* part = (double2*)ctx.reduce_buf.p;
  double2* res = part + kRedBlocks;
  if (precision == QOB_C128)
    k_dot_partial<double2><<<kRedBlocks, kRedThreads, 0, s>>>((const double2*)x, (const double2*)y, n, part);
  else
    k_dot_partial<float2><<<kRedBlocks, kRedThreads, 0, s>>>((const float2*)x, (const float2*)y, n, part);
  QOB_LAUNCHED();
  k_dot_final<<<1, kRedThreads, 0, s>>>(part, kRedBlocks, res);
  QOB_LAUNCHED();
  QOB_CUDA(cudaMemcpyAsync(ctx.reduce_host, res, sizeof(double2), cudaMemcpyDeviceToHost, s));
  QOB_CUDA(cudaStreamSynchronize(s));
  const double2 r = *(const double2*)ctx.reduce_host;
  if (norm) {
    out[0] = sqrt(r.x);
  } else {
    out[0] = r.x;
    out[1] = r.y;
  }
}

}  // namespace qob
