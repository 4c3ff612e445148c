// k_dmma.cu -- ComplexF64 dense contractions on the FP64 tensor cores
// (DMMA: mma.sync.aligned.m8n8k4.row.col.f64), as one strided, batched complex
// GEMM that covers
//   * a DenseOperator times vectors  (mul! -> BLAS zgemm, src/operators_dense.jl:394-396)
//   * the mode products of a LazyTensor's dense factors
//                                    (_tp_matmul_first!/_mid!/_last!, src/operators_lazytensor.jl:281-428)
// D[i, j] = alpha * sum_k P[i, k] Q[k, j] + beta * D[i, j] for every batch
// entry z = z1 + nz1 * z2 (element strides given per operand and per batch
// index).  A complex product is four real DMMAs per 8 x 8 x 4 tile:
//   re += Pr Qr - Pi Qi,  im += Pr Qi + Pi Qr.
// A warp owns 8 rows x 8 NT columns (NT 8 x 8 accumulator tiles in two doubles
// per lane each, real and imaginary part apart); a block of four warps owns 32
// rows.  Products too small to fill the GPU split the k range over blocks; the
// partial sums are added in order by k_zgemm_reduce (deterministic).
//
// Used in place of the FMA kernels of k_misc.cu when the context option
// QOB_OPT_FP64_TENSOR is on and the contracted dimension is at least 64.
#include <cuda_runtime.h>

#include <algorithm>

#include "qob_internal.h"

namespace qob {

namespace {

struct ZGemm {
  const double2* p;
  int64_t ps_i, ps_k;
  const double2* q;
  int64_t qs_k, qs_j;
  double2* y;
  int64_t ys_i, ys_j;
  int64_t M, N, K;
  int64_t nz1;  // batch index z = z1 + nz1 * z2
  int64_t pz1, pz2, qz1, qz2, yz1, yz2;
  double ar, ai, br, bi;
  double2* part;  // k-split partial sums [kz][j][i] (batch of one only), or null
  int64_t kc;     // k range per block along grid.z when part != null
};

// D (8 x 8, two elements per lane) += A (8 x 4, one per lane) * B (4 x 8, one per lane)
__device__ __forceinline__ void dmma(double (&d)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
               : "+d"(d[0]), "+d"(d[1])
               : "d"(a), "d"(b));
}

template <int NT>
__global__ void __launch_bounds__(128) k_zgemm_dmma(ZGemm g) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, t4 = lane & 3;
  const int64_t i0 = ((int64_t)blockIdx.x * 4 + warp) * 8;
  if (i0 >= g.M) return;  // whole warps only: every lane of a live warp reaches each mma
  const int64_t j0 = (int64_t)blockIdx.y * 8 * NT;
  int64_t z = blockIdx.z, k0 = 0, k1 = g.K;
  if (g.part) {
    k0 = z * g.kc;
    k1 = k0 + g.kc < g.K ? k0 + g.kc : g.K;
    z = 0;
  }
  const int64_t z1 = z % g.nz1, z2 = z / g.nz1;
  const double2* P = g.p + z1 * g.pz1 + z2 * g.pz2;
  const double2* Q = g.q + z1 * g.qz1 + z2 * g.qz2;
  double cr[NT][2], ci[NT][2];
#pragma unroll
  for (int t = 0; t < NT; ++t) cr[t][0] = cr[t][1] = ci[t][0] = ci[t][1] = 0.0;
  const int64_t ia = i0 + gq;  // this lane's row of the A fragment
  const bool arow = ia < g.M;
  const double2* pa = P + ia * g.ps_i;
  for (int64_t k = k0; k < k1; k += 4) {
    const int64_t ka = k + t4;  // A fragment column = B fragment row
    const bool kin = ka < k1;
    double2 a = make_double2(0.0, 0.0);
    if (arow && kin) a = __ldg(pa + ka * g.ps_k);
    double2 b[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int64_t jb = j0 + 8 * t + gq;  // B fragment column
      b[t] = (kin && jb < g.N) ? __ldg(Q + ka * g.qs_k + jb * g.qs_j) : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      dmma(cr[t], a.x, b[t].x);
      dmma(cr[t], -a.y, b[t].y);
      dmma(ci[t], a.x, b[t].y);
      dmma(ci[t], a.y, b[t].x);
    }
  }
  // accumulator element e of tile t: row i0 + gq, column j0 + 8 t + 2 t4 + e
  const int64_t i = i0 + gq;
  if (i >= g.M) return;
#pragma unroll
  for (int t = 0; t < NT; ++t) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int64_t j = j0 + 8 * t + 2 * t4 + e;
      if (j >= g.N) continue;
      if (g.part) {
        g.part[((int64_t)blockIdx.z * g.N + j) * g.M + i] = make_double2(cr[t][e], ci[t][e]);
        continue;
      }
      double2* yp = g.y + z1 * g.yz1 + z2 * g.yz2 + i * g.ys_i + j * g.ys_j;
      double re = g.ar * cr[t][e] - g.ai * ci[t][e];
      double im = g.ar * ci[t][e] + g.ai * cr[t][e];
      if (g.br != 0.0 || g.bi != 0.0) {
        const double2 o = *yp;
        re += g.br * o.x - g.bi * o.y;
        im += g.br * o.y + g.bi * o.x;
      }
      *yp = make_double2(re, im);
    }
  }
}

// y[i, j] = alpha * (sum over the k ranges, in order) + beta * y[i, j]
__global__ void k_zgemm_reduce(const double2* __restrict__ part, int kchunks, int64_t M, int64_t N,
                               double2* __restrict__ y, int64_t ys_i, int64_t ys_j, double ar, double ai, double br,
                               double bi) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j = blockIdx.y;
  if (i >= M) return;
  double sre = 0.0, sim = 0.0;
  for (int z = 0; z < kchunks; ++z) {
    const double2 p = part[((int64_t)z * N + j) * M + i];
    sre += p.x;
    sim += p.y;
  }
  double re = ar * sre - ai * sim;
  double im = ar * sim + ai * sre;
  double2* yp = y + i * ys_i + j * ys_j;
  if (br != 0.0 || bi != 0.0) {
    const double2 o = *yp;
    re += br * o.x - bi * o.y;
    im += br * o.y + bi * o.x;
  }
  *yp = make_double2(re, im);
}

constexpr int kNT = 2;  // 16 columns per warp

void run_zgemm(ZGemm g, int64_t batch, Workspace* ws, int slot, cudaStream_t s) {
  const int64_t bx = (g.M + 31) / 32, by = (g.N + 8 * kNT - 1) / (8 * kNT);
  if (bx > 0x7fffffff || by > 65535) fail(QOB_ERR_UNSUPPORTED, "DMMA contraction too large for one grid");
  int64_t kch = 1;
  if (batch == 1 && ws) {
    // k ranges: about eight blocks per SM, each range at least 64 long
    kch = std::max<int64_t>(1, std::min<int64_t>((1216 + bx * by - 1) / (bx * by), g.K / 64));
    kch = std::min<int64_t>(kch, 65535);
  }
  if (kch > 1) {
    g.kc = ((g.K + kch - 1) / kch + 3) / 4 * 4;
    kch = (g.K + g.kc - 1) / g.kc;
    g.part = static_cast<double2*>(ws->get(slot, (size_t)kch * g.N * g.M * sizeof(double2)));
  }
  if (g.nz1 > 65535) fail(QOB_ERR_UNSUPPORTED, "DMMA contraction with more than 65535 inner batch entries");
  int64_t done = 0;
  const int64_t zmax = g.part ? kch : batch;
  const int64_t zstep = g.part ? 65535 : (65535 / g.nz1) * g.nz1;  // grid.z limit, whole inner batches
  do {
    const int64_t nz = std::min<int64_t>(zmax - done, zstep);
    ZGemm c = g;
    if (!g.part && done > 0) {  // shift the operands to batch entry `done` (z1 = 0 there)
      const int64_t z2 = done / g.nz1;
      c.p += z2 * g.pz2;
      c.q += z2 * g.qz2;
      c.y += z2 * g.yz2;
    }
    k_zgemm_dmma<kNT><<<dim3((unsigned)bx, (unsigned)by, (unsigned)nz), 128, 0, s>>>(c);
    QOB_LAUNCHED();
    done += nz;
  } while (done < zmax && !g.part);
  if (g.part) {
    if (g.N > 65535) fail(QOB_ERR_UNSUPPORTED, "DMMA reduction over more than 65535 columns");
    k_zgemm_reduce<<<dim3((unsigned)((g.M + 127) / 128), (unsigned)g.N), 128, 0, s>>>(
        g.part, (int)kch, g.M, g.N, g.y, g.ys_i, g.ys_j, g.ar, g.ai, g.br, g.bi);
    QOB_LAUNCHED();
  }
}

}  // namespace

void launch_dense_dmma(const void* a, int64_t m, int64_t n, c128 alpha, const void* x, int64_t xes, int64_t xcs,
                       c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s, Workspace* ws,
                       int slot) {
  if (m == 0 || ncols == 0) return;
  ZGemm g{};
  g.p = static_cast<const double2*>(a);
  g.ps_i = 1;
  g.ps_k = m;
  g.q = static_cast<const double2*>(x);
  g.qs_k = xes;
  g.qs_j = xcs;
  g.y = static_cast<double2*>(y);
  g.ys_i = yes;
  g.ys_j = ycs;
  g.M = m;
  g.N = ncols;
  g.K = n;
  g.nz1 = 1;
  g.ar = alpha.re;
  g.ai = alpha.im;
  g.br = beta.re;
  g.bi = beta.im;
  run_zgemm(g, 1, ws, slot, s);
}

// out[a, j, b] = alpha * sum_k A[j, k] in[a, k, b] + beta * out[a, j, b] for each
// vector c: rows j (dout); columns the longer of a (s1) and b (s3); the batch
// runs over the other one and the vectors.
void launch_modek_dmma(const void* A, int64_t s1, int64_t dout, int64_t din, int64_t s3, c128 alpha, const void* x,
                       int64_t xes, int64_t xcs, c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols,
                       cudaStream_t s) {
  if (s1 * dout * s3 == 0 || ncols == 0) return;
  ZGemm g{};
  g.p = static_cast<const double2*>(A);
  g.ps_i = 1;
  g.ps_k = dout;
  g.q = static_cast<const double2*>(x);
  g.y = static_cast<double2*>(y);
  g.M = dout;
  g.K = din;
  g.ar = alpha.re;
  g.ai = alpha.im;
  g.br = beta.re;
  g.bi = beta.im;
  if (s1 >= s3) {  // columns a, batch (b, c)
    g.N = s1;
    g.qs_k = s1 * xes;
    g.qs_j = xes;
    g.ys_i = s1 * yes;
    g.ys_j = yes;
    g.nz1 = s3;
    g.qz1 = s1 * din * xes;
    g.yz1 = s1 * dout * yes;
  } else {  // columns b, batch (a, c)
    g.N = s3;
    g.qs_k = s1 * xes;
    g.qs_j = s1 * din * xes;
    g.ys_i = s1 * yes;
    g.ys_j = s1 * dout * yes;
    g.nz1 = s1;
    g.qz1 = xes;
    g.yz1 = yes;
  }
  g.qz2 = xcs;
  g.yz2 = ycs;
  run_zgemm(g, g.nz1 * ncols, nullptr, 0, s);
}

}  // namespace qob
