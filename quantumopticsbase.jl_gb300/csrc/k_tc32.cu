// k_tc32.cu -- ComplexF32 dense operator times vectors on the 5th-generation
// tensor cores (tcgen05.mma kind::tf32, accumulator in tensor memory, operand
// tiles brought in by TMA), for mul! on a DenseOperator
// (src/operators_dense.jl:394-396, BLAS cgemm in the reference).
//
// The complex product is one real GEMM.  The operator is stored (built on
// first use) as the real matrix Ahat of 2m rows, K-major: row 2i holds
// Re A[i, :], row 2i + 1 holds Im A[i, :] (n rounded up to 32, zero padded).
// The vectors are split per call (k_tc_split_b) into Bhat of 2N rows, K-major:
// row j < N holds Re X[:, j], row N + j holds Im X[:, j].  Both are kept in
// memory as tiles (128 rows x 32 floats of Ahat, BN rows x 32 floats of Bhat),
// each tile one contiguous block laid out exactly as the MMA reads it from
// shared memory (rows of 128 bytes, 16-byte chunk c of row r at position
// c ^ (r mod 8): the 128-byte swizzle), so a stage arrives with one bulk copy
// per operand (cp.async.bulk) that streams a contiguous block.  Then
// D = Ahat Bhat^T (2m x 2N, FP32 in tensor memory) gives
//   Re Y[i, c] = D[2i, c] - D[2i+1, N+c],   Im Y[i, c] = D[2i+1, c] + D[2i, N+c]
// (in the kernel the imaginary rows of Bhat start at BN / 2, BN = the tile's
// column count, so N above stands for BN / 2).
// TF32 keeps 10 explicit mantissa bits, and an MMA of kind tf32 reads an FP32
// operand as TF32 by dropping its 13 low mantissa bits.  To reach FP32
// accuracy each operand x is used as its head hi (x itself, read truncated)
// and its tail lo = x - hi (exact in FP32, |lo| < 2^-10 |x|, read truncated in
// turn: within 2^-20 |x|), and D = Ahi Bhi + Ahi Blo + Alo Bhi (three MMAs per
// k step; the dropped Alo Blo is below 2^-20 of the product): about 1e-6
// relative.  The tails of Ahat are written into shared memory beside each tile
// as it arrives, those of Bhat once per call.
//
// Block (320 threads): warp 0 issues the bulk copies (a 5-, 4- or 3-stage ring
// of Ahat tiles and Bhat head / tail tiles); warps 2-9 write each Ahat tile's
// tail, add each k block's accumulator to registers (see k_tc_cgemm), then
// run the epilogue; warp 1 owns the tensor memory and one of its threads
// issues the MMAs (M = 128 rows, N = BN = 2 x kets, K = 8 per instruction).
// Blocks cover 64 complex rows each and, when that leaves SMs idle, a range of
// k blocks whose partial products k_tc_reduce adds in order; the grid is one
// wave (one block per SM by its shared memory).  Every wait is
// bounded: a wait that gives up records kTcErrTimeout in the status word, the
// block drains its copies and MMAs, frees its tensor memory and returns.
#include <cuda_runtime.h>

#include <algorithm>

#include "qob_internal.h"

namespace qob {

namespace {

constexpr int kTcBM = 128;     // rows of Ahat per block (64 complex rows)
constexpr int kTcBK = 32;      // floats per k block: one 128-byte swizzle span
constexpr int kTcThreads = 320;  // warp 0: copies, warp 1: MMAs, warps 2-9: splits + accumulators
constexpr int kTcWork = 256;     // threads of warps 2-9
constexpr unsigned kTcErrTimeout = 1u;
constexpr int kTcPolls = 1 << 21;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* b, unsigned n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ bool bar_test(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity) {
  for (int i = 0; i < kTcPolls; ++i) {
    if (bar_test(b, parity)) return true;
    if (i > 64) __nanosleep(32);
  }
  return false;
}
// bytes (a multiple of 16) from global src to shared dst, both 16-byte aligned, counted on b
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   saddr(dst)),
               "l"(src), "r"(bytes), "r"(saddr(b))
               : "memory");
}
// float offset of element (row r, column k) inside a swizzled tile of 32-float rows
__host__ __device__ __forceinline__ int swz(int r, int k) { return r * 32 + ((((k >> 2) ^ (r & 7)) << 2) | (k & 3)); }
// Shared-memory matrix descriptor of a K-major tile with the 128-byte swizzle:
// start address, stride between 8-row groups 1024 bytes, descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(const void* tile) {
  const uint64_t a = (saddr(tile) & 0x3FFFFu) >> 4;
  return a | (uint64_t(1) << 16) | (uint64_t(1024 >> 4) << 32) | (uint64_t(1) << 46) | (uint64_t(2) << 61);
}
__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(b))
               : "memory");
}
// x minus its TF32 truncation (the 13 low mantissa bits): the part of x that
// an MMA reading x as TF32 drops; exact in FP32
__device__ __forceinline__ float tf32_tail(float x) { return x - __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }
// 8 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
// 16 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int BN>
struct TcCfg {
  static constexpr int kStages = BN <= 32 ? 5 : (BN <= 64 ? 4 : 3);
  static constexpr int kATile = kTcBM * kTcBK * 4;  // 16 KB
  static constexpr int kBTile = BN * kTcBK * 4;
  static constexpr int kStage = 2 * kATile + 2 * kBTile;  // A (its head), A tail, B head, B tail
  static constexpr int kAcc = 4;                          // accumulators of BN columns, used in turn
  static constexpr int kGroup = 2;                        // k blocks summed in one accumulator
  static constexpr int kTmemCols = kAcc * BN;
  static constexpr size_t kSmem = 1024 /* alignment */ + (size_t)kStages * kStage + 256 /* barriers */;
};

// Y[i, c] (complex rows i < m, kets c < N) = alpha * (Ahat Bhat^T combined) + beta * Y,
// or the block's partial product into part[kz][c][i] when part != null.
//
// Accumulation: each group of kGroup k blocks (64 terms, 24 MMAs) starts a
// fresh accumulator in tensor memory, kAcc of them used in turn; the split
// warps read each finished one and add it to FP32 registers, rounding to
// nearest.  The tensor cores' own accumulation (which does not round to
// nearest) then spans 64 terms only, which keeps the FP32 accuracy of the
// ComplexF32 mode for long rows (the error no longer grows with n), and the
// MMAs of group q + kAcc wait only for the registers to take group q.
template <int BN>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_cgemm(const float* __restrict__ ahat, const float* __restrict__ bh_t, const float* __restrict__ bl_t,
               int64_t m, int N, int nkb, int kb_per, float2* y, int64_t yes, int64_t ycs, float2 alpha, float2 beta,
               float2* part, unsigned* status) {
  using C = TcCfg<BN>;
  constexpr int S = C::kStages;
  extern __shared__ __align__(16) unsigned char tc_smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + (size_t)S * C::kStage);
  uint64_t* full = bars;           // copies landed            (count 1 + tx)
  uint64_t* conv = bars + S;       // A tail written           (count kTcWork)
  uint64_t* empty = bars + 2 * S;  // MMAs read the stage      (count 1, tcgen05.commit)
  constexpr int NA = C::kAcc, G = C::kGroup;
  uint64_t* accf = bars + 3 * S;       // [NA] accumulator written (count 1, tcgen05.commit)
  uint64_t* acce = bars + 3 * S + NA;  // [NA] accumulator read    (count kTcWork)
  uint64_t* fin = bars + 3 * S + 2 * NA;  // every MMA issued has completed (count 1, tcgen05.commit)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3 * S + 2 * NA + 1);
  int* abort_flag = reinterpret_cast<int*>(bars + 3 * S + 2 * NA + 2);
  auto stageA = [&](int s) { return base + (size_t)s * C::kStage; };
  auto stageAl = [&](int s) { return base + (size_t)s * C::kStage + C::kATile; };
  auto stageBh = [&](int s) { return base + (size_t)s * C::kStage + 2 * C::kATile; };
  auto stageBl = [&](int s) { return base + (size_t)s * C::kStage + 2 * C::kATile + C::kBTile; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kb0 = blockIdx.y * kb_per;
  const int nk = min(nkb - kb0, kb_per);  // >= 1 (the host makes no empty ranges)
  const int row0 = blockIdx.x * kTcBM;    // first Ahat row of this block

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      bar_init(&full[s], 1);
      bar_init(&conv[s], kTcWork);
      bar_init(&empty[s], 1);
    }
    for (int b = 0; b < NA; ++b) {
      bar_init(&accf[b], 1);
      bar_init(&acce[b], kTcWork);
    }
    bar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                 "r"(C::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // producer
      int issued = 0;
      for (int it = 0; it < nk; ++it) {
        const int s = it % S;
        if (it >= S && !bar_wait(&empty[s], ((it / S) - 1) & 1)) {
          atomicExch(abort_flag, 1);
          break;
        }
        if (*(volatile int*)abort_flag) break;
        bar_expect(&full[s], 2 * C::kBTile + C::kATile);
        const int kb = kb0 + it;
        bulk_copy(stageA(s), ahat + ((int64_t)blockIdx.x * nkb + kb) * (C::kATile / 4), C::kATile, &full[s]);
        bulk_copy(stageBh(s), bh_t + (int64_t)kb * (C::kBTile / 4), C::kBTile, &full[s]);
        bulk_copy(stageBl(s), bl_t + (int64_t)kb * (C::kBTile / 4), C::kBTile, &full[s]);
        issued = it + 1;
      }
      // every copy issued has landed before the block's shared memory goes away
      for (int it = max(0, issued - S); it < issued; ++it) bar_wait(&full[it % S], (it / S) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      // kind::tf32, FP32 accumulator, A and B K-major, N = BN, M = 128
      const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
      for (int it = 0; it < nk; ++it) {
        const int s = it % S, q = it / G, b = q % NA;
        const bool first = it % G == 0, last = it % G == G - 1 || it == nk - 1;
        if (!bar_wait(&conv[s], (it / S) & 1) || (first && q >= NA && !bar_wait(&acce[b], ((q / NA) - 1) & 1))) {
          atomicExch(abort_flag, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(b * BN);
        const uint64_t ah = sw128_desc(stageA(s)), al = sw128_desc(stageAl(s));
        const uint64_t bh = sw128_desc(stageBh(s)), bl = sw128_desc(stageBl(s));
#pragma unroll
        for (int kk = 0; kk < kTcBK / 8; ++kk) {  // 8 TF32 = 32 bytes = 2 descriptor units per step
          const uint64_t o = (uint64_t)(2 * kk);
          mma_tf32(d, ah + o, bh + o, idesc, (kk > 0 || !first) ? 1u : 0u);
          mma_tf32(d, ah + o, bl + o, idesc, 1u);
          mma_tf32(d, al + o, bh + o, idesc, 1u);
        }
        mma_commit(&empty[s]);
        if (last) mma_commit(&accf[b]);
      }
      mma_commit(fin);  // also after an early exit: fires when every MMA above has completed
    }
  } else {
    // warps 2-9: write each A tile's tail; after each k block, add the
    // accumulator to registers.  Warps w and w + 4 share tensor-memory lanes
    // 32 * (w % 4) ..; warp half h keeps the kets [h * BN/4, (h + 1) * BN/4):
    // their real-part columns and, BN/2 further, their imaginary-part columns.
    const int ct = threadIdx.x - 64;
    const int q4 = warp & 3;
    const int half = (warp - 2) >> 2;
    constexpr int KQ = BN / 4;  // kets per warp half
    const uint32_t lane_addr = tmem + ((uint32_t)(q4 * 32) << 16);
    float acc_re[KQ], acc_im[KQ];
#pragma unroll
    for (int c = 0; c < KQ; ++c) acc_re[c] = acc_im[c] = 0.f;
    bool ok = true;
    auto drain = [&](int q) {  // accumulator of k-block group q
      const int b = q % NA;
      if (!__all_sync(0xffffffffu, bar_wait(&accf[b], (q / NA) & 1) && !*(volatile int*)abort_flag)) {
        ok = false;
        return;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t col = lane_addr + (uint32_t)(b * BN + half * KQ);
#pragma unroll
      for (int c0 = 0; c0 < KQ; c0 += 8) {
        float v[8], w[8];
        tmem_ld8(col + (uint32_t)c0, v);
        tmem_ld8(col + (uint32_t)(BN / 2 + c0), w);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          acc_re[c0 + t] += v[t];
          acc_im[c0 + t] += w[t];
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      bar_arrive(&acce[b]);
    };
    for (int it = 0; it < nk && ok; ++it) {
      const int s = it % S;
      if (*(volatile int*)abort_flag || !bar_wait(&full[s], (it / S) & 1)) {
        ok = false;
        break;
      }
      // the MMAs read the raw tile as TF32 (its head, truncated); the tail goes beside it
      const float4* a = reinterpret_cast<const float4*>(stageA(s));
      float4* al = reinterpret_cast<float4*>(stageAl(s));
#pragma unroll
      for (int q = 0; q < C::kATile / 16 / kTcWork; ++q) {
        const int idx = ct + kTcWork * q;
        const float4 v = a[idx];
        al[idx] = make_float4(tf32_tail(v.x), tf32_tail(v.y), tf32_tail(v.z), tf32_tail(v.w));
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bar_arrive(&conv[s]);
      if (it % G == 0 && it >= G) drain(it / G - 1);  // the previous group, once this one has begun
    }
    if (ok) drain((nk - 1) / G);  // the last group (the one before it was drained in the loop)
    ok = __all_sync(0xffffffffu, ok && !*(volatile int*)abort_flag);
    if (!ok) {
      atomicExch(abort_flag, 1);
      if (lane == 0 && status) atomicOr(status, kTcErrTimeout);
    } else {
      const int r = q4 * 32 + lane;  // accumulator row = Ahat row row0 + r
      const int64_t i = (int64_t)(row0 + r) >> 1;
      const bool even = (lane & 1) == 0;
#pragma unroll
      for (int t = 0; t < KQ; ++t) {
        const int c = half * KQ + t;
        const float other = __shfl_xor_sync(0xffffffffu, acc_im[t], 1);
        const float v = even ? acc_re[t] - other : acc_re[t] + other;  // even lane: Re Y, odd lane: Im Y
        const float w = __shfl_xor_sync(0xffffffffu, v, 1);
        if (even && i < m && c < N) {
          if (part) {
            part[((int64_t)blockIdx.y * N + c) * m + i] = make_float2(v, w);
          } else {
            float2* yp = y + i * yes + (int64_t)c * ycs;
            float re = alpha.x * v - alpha.y * w;
            float im = alpha.x * w + alpha.y * v;
            if (beta.x != 0.f || beta.y != 0.f) {
              const float2 o = *yp;
              re = __fmaf_rn(beta.x, o.x, __fmaf_rn(-beta.y, o.y, re));
              im = __fmaf_rn(beta.x, o.y, __fmaf_rn(beta.y, o.x, im));
            }
            *yp = make_float2(re, im);
          }
        }
      }
    }
  }
  // every MMA issued has completed before the tensor memory is freed
  if (warp == 1 && lane == 0) bar_wait(fin, 0);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::kTmemCols) : "memory");
  }
}

// Bhat head and tail: row j = Re X[:, j], row H + j = Im X[:, j] (j < the
// kets, H = half the tile's BN columns), value and TF32 tail, as swizzled tiles of BN
// rows x 32 floats, one per k block (zero beyond n).
__global__ void k_tc_split_b(const float2* __restrict__ x, int64_t n, int64_t xes, int64_t xcs, int BN, int64_t nkb,
                             float* __restrict__ bh, float* __restrict__ bl) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (k >= nkb * kTcBK) return;
  float2 v = make_float2(0.f, 0.f);
  if (k < n) v = x[k * xes + (int64_t)j * xcs];
  const int64_t tile = (k / kTcBK) * (int64_t)BN * kTcBK;
  const int kk = (int)(k % kTcBK);
  const int64_t o_re = tile + swz(j, kk), o_im = tile + swz(BN / 2 + j, kk);
  bh[o_re] = v.x;  // read as TF32 by the MMA: its truncated head
  bl[o_re] = tf32_tail(v.x);
  bh[o_im] = v.y;
  bl[o_im] = tf32_tail(v.y);
}

// y[i, c] = alpha * (sum of the k ranges' partial products, in order) + beta * y[i, c]
__global__ void k_tc_reduce(const float2* __restrict__ part, int kchunks, int64_t m, int N, float2* __restrict__ y,
                            int64_t yes, int64_t ycs, float2 alpha, float2 beta) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= m) return;
  float sr = 0.f, si = 0.f;
  for (int z = 0; z < kchunks; ++z) {
    const float2 p = part[((int64_t)z * N + c) * m + i];
    sr += p.x;
    si += p.y;
  }
  float2* yp = y + i * yes + (int64_t)c * ycs;
  float re = alpha.x * sr - alpha.y * si;
  float im = alpha.x * si + alpha.y * sr;
  if (beta.x != 0.f || beta.y != 0.f) {
    const float2 o = *yp;
    re = __fmaf_rn(beta.x, o.x, __fmaf_rn(-beta.y, o.y, re));
    im = __fmaf_rn(beta.x, o.y, __fmaf_rn(beta.y, o.x, im));
  }
  *yp = make_float2(re, im);
}

template <int BN>
void run_tc(const TcDense& d, int64_t n, const float2* x, int64_t xes, int64_t xcs, int N, float2* y, int64_t yes,
            int64_t ycs, float2 alpha, float2 beta, Workspace* ws, int slot, cudaStream_t s, unsigned* status,
            int num_sms) {
  using C = TcCfg<BN>;
  const int64_t nkb = d.ldk / kTcBK;
  // split vectors: head and tail tiles of Bhat (rows N .. BN/2 - 1 and BN/2 + N .. BN - 1 stay zero)
  const size_t bbytes = (size_t)nkb * C::kBTile;
  char* w = static_cast<char*>(ws->get(slot, 2 * bbytes + 256));
  float* bh = reinterpret_cast<float*>(w);
  float* bl = reinterpret_cast<float*>(w + bbytes);
  if (N < BN / 2) QOB_CUDA(cudaMemsetAsync(w, 0, 2 * bbytes, s));
  k_tc_split_b<<<dim3((unsigned)((d.ldk + 255) / 256), (unsigned)N), 256, 0, s>>>(x, n, xes, xcs, BN, nkb, bh, bl);
  QOB_LAUNCHED();
  const int mt = (int)d.mtiles;
  // k ranges so that the blocks fill the SMs in one wave (each range at least 4 k blocks)
  int kchunks = (int)std::max<int64_t>(1, std::min<int64_t>(num_sms / std::max(1, mt), nkb / 4));
  const int kb_per = (int)((nkb + kchunks - 1) / kchunks);
  kchunks = (int)((nkb + kb_per - 1) / kb_per);
  float2* part = nullptr;
  if (kchunks > 1) part = static_cast<float2*>(ws->get(slot + 1, (size_t)kchunks * N * d.m * sizeof(float2)));
  auto kern = k_tc_cgemm<BN>;
  QOB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::kSmem));
  kern<<<dim3((unsigned)mt, (unsigned)kchunks), kTcThreads, C::kSmem, s>>>(
      static_cast<const float*>(d.ahat.p), bh, bl, d.m, N, (int)nkb, kb_per, y, yes, ycs, alpha, beta, part, status);
  QOB_LAUNCHED();
  if (part) {
    k_tc_reduce<<<dim3((unsigned)((d.m + 127) / 128), (unsigned)N), 128, 0, s>>>(part, kchunks, d.m, N, y, yes, ycs,
                                                                                alpha, beta);
    QOB_LAUNCHED();
  }
}

// Ahat of the stored ComplexF32 matrix (column-major m x n, on the device) as
// swizzled 128 x 32 tiles, tile (t, b) at float offset (t * nkb + b) * 4096:
// row 2i = Re A[i, :], row 2i + 1 = Im A[i, :]; zero beyond the matrix.
__global__ void k_tc_build_ahat(const float2* __restrict__ a, int64_t m, int64_t n, int64_t nkb, float* __restrict__ ah) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // complex row
  const int64_t k = blockIdx.y;
  const int64_t mpad = (2 * m + kTcBM - 1) / kTcBM * kTcBM / 2;
  if (i >= mpad || k >= nkb * kTcBK) return;
  const float2 v = (i < m && k < n) ? a[i + k * m] : make_float2(0.f, 0.f);
  const int64_t r = 2 * i;  // Ahat row of the real part; the imaginary part is the next row of the same tile
  const int64_t tile = ((r / kTcBM) * nkb + k / kTcBK) * (int64_t)(kTcBM * kTcBK);
  const int rr = (int)(r % kTcBM), kk = (int)(k % kTcBK);
  ah[tile + swz(rr, kk)] = v.x;
  ah[tile + swz(rr + 1, kk)] = v.y;
}

}  // namespace

void tc_dense_build(TcDense& d, const void* a, int64_t m, int64_t n, cudaStream_t s) {
  d.m = m;
  d.n = n;
  d.ldk = (n + kTcBK - 1) / kTcBK * kTcBK;
  d.mtiles = (2 * m + kTcBM - 1) / kTcBM;
  if (d.ldk > 65535) fail(QOB_ERR_UNSUPPORTED, "tensor-core dense path: more than 65535 columns");
  const int64_t nkb = d.ldk / kTcBK;
  d.ahat.alloc((size_t)d.mtiles * nkb * kTcBM * kTcBK * sizeof(float));
  const int64_t mpad = d.mtiles * kTcBM / 2;
  k_tc_build_ahat<<<dim3((unsigned)((mpad + 127) / 128), (unsigned)d.ldk), 128, 0, s>>>(
      static_cast<const float2*>(a), m, n, nkb, static_cast<float*>(d.ahat.p));
  QOB_LAUNCHED();
  d.ready = true;
}

bool launch_dense_tc(const TcDense& d, c128 alpha, const void* x, int64_t xes, int64_t xcs, c128 beta, void* y,
                     int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s, Workspace* ws, int slot,
                     unsigned* status, int num_sms) {
  if (!d.ready || ncols < 1) return false;
  const float2 a = make_float2((float)alpha.re, (float)alpha.im), b = make_float2((float)beta.re, (float)beta.im);
  for (int64_t c0 = 0; c0 < ncols; c0 += 64) {  // up to 64 kets per pass (BN = 128 columns)
    const int N = (int)std::min<int64_t>(64, ncols - c0);
    const float2* xc = static_cast<const float2*>(x) + c0 * xcs;
    float2* yc = static_cast<float2*>(y) + c0 * ycs;
    if (N <= 16)
      run_tc<32>(d, d.n, xc, xes, xcs, N, yc, yes, ycs, a, b, ws, slot, s, status, num_sms);
    else if (N <= 32)
      run_tc<64>(d, d.n, xc, xes, xcs, N, yc, yes, ycs, a, b, ws, slot, s, status, num_sms);
    else
      run_tc<128>(d, d.n, xc, xes, xcs, N, yc, yes, ycs, a, b, ws, slot, s, status, num_sms);
  }
  return true;
}

}  // namespace qob
