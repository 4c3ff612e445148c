// k_tc32.cu -- ComplexF32 dense operator times vectors on the 5th-generation
// tensor cores (tcgen05.mma kind::tf32, accumulator and A operand in tensor
// memory, B tiles brought in by bulk copies), for mul! on a DenseOperator
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
// c ^ (r mod 8): the 128-byte swizzle), so a B stage arrives with one bulk
// copy per tile (cp.async.bulk) that streams a contiguous block.  Then
// D = Ahat Bhat^T (2m x 2N, FP32 in tensor memory) gives
//   Re Y[i, c] = D[2i, c] - D[2i+1, N+c],   Im Y[i, c] = D[2i+1, c] + D[2i, N+c]
// (in the kernel the imaginary rows of Bhat start at BN / 2, BN = the tile's
// column count, so N above stands for BN / 2).
// TF32 keeps 10 explicit mantissa bits, and an MMA of kind tf32 reads an FP32
// operand as TF32 by dropping its 13 low mantissa bits.  To reach FP32
// accuracy each operand x is used as its head hi (x itself, read truncated)
// and its tail lo = x - hi (exact in FP32, |lo| < 2^-10 |x|, read truncated in
// turn: within 2^-20 |x|), and D = Ahi Bhi + Ahi Blo + Alo Bhi (three products
// per k step, two MMAs when B's head and tail tiles are one operand of twice
// the columns; the dropped Alo Blo is below 2^-20 of the product): about 1e-6
// relative.  Each Ahat tile is loaded from global memory into registers and
// stored into tensor memory, value and tail side by side, and the MMAs read A
// from there; the tails of Bhat are made once per call, beside its values.
//
// Block (320 threads): warp 0 issues the bulk copies of the ring of Bhat head /
// tail tiles; warps 2-9 load each Ahat tile (one k block ahead) and store it
// into tensor memory, add each group's accumulator to registers (see
// k_tc_cgemm), then run the epilogue; warp 1 owns the tensor memory and one of
// its threads issues the MMAs (M = 128 rows, N = BN or 2 x BN, K = 8 per
// instruction).
// Work is split stream-K style: the (row tile of 64 complex rows, k block)
// units, row tile major, are cut into equal runs, one per block, so that the
// grid fills every SM in one wave (two blocks per SM for up to 16 kets, each
// with half of the SM's tensor memory, else one with all of it).  A block's run holds one or more segments
// (the part of one row tile's k range in the run); a segment that covers a
// whole row tile writes y, the others write partial products that
// k_tc_reduce adds in k order.  Every wait is bounded: a wait that gives up
// records kTcErrTimeout in the status word, the block drains its copies and
// MMAs, frees its tensor memory and returns.
#include <cuda_runtime.h>

#include <algorithm>

#include "launch.cuh"
#include "qob_internal.h"

namespace qob {

namespace {

constexpr int kTcBM = 128;     // rows of Ahat per block (64 complex rows)
constexpr int kTcBK = 32;      // floats per k block: one 128-byte swizzle span
constexpr int kTcThreads = 320;  // warp 0: copies, warp 1: MMAs, warps 2-9: splits + accumulators
constexpr int kTcWork = 256;     // threads of warps 2-9
constexpr int kTcTmemCols = 512;  // the tensor memory of one SM
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
// element offset of column c of a column map (no division for a plain stride;
// 32-bit divisions: column counts and the map's extents stay below 2^31)
__host__ __device__ __forceinline__ int64_t tc_col_offset(const TcColMap& m, int64_t c) {
  if (m.s1 == 1 && m.s3 == 1) return c * m.st;
  const uint32_t cc = (uint32_t)c, s1 = (uint32_t)m.s1, s3 = (uint32_t)m.s3;
  const uint32_t a = cc % s1, q = cc / s1;
  return (int64_t)a * m.sa + (int64_t)(q % s3) * m.sb + (int64_t)(q / s3) * m.st;
}
// Consecutive columns of a column map: the offset of column c, then of c + 1, ...
struct TcColCursor {
  int64_t a, b, off;
  __device__ __forceinline__ TcColCursor(const TcColMap& m, int64_t c) {
    const uint32_t cc = (uint32_t)c, s1 = (uint32_t)m.s1, s3 = (uint32_t)m.s3;
    a = cc % s1;
    const uint32_t q = cc / s1;
    b = q % s3;
    off = a * m.sa + b * m.sb + (int64_t)(q / s3) * m.st;
  }
  __device__ __forceinline__ void next(const TcColMap& m) {
    if (++a < m.s1) {
      off += m.sa;
      return;
    }
    a = 0;
    off -= (m.s1 - 1) * m.sa;
    if (++b < m.s3) {
      off += m.sb;
      return;
    }
    b = 0;
    off += m.st - (m.s3 - 1) * m.sb;
  }
};
// Shared-memory matrix descriptor of a K-major tile with the 128-byte swizzle:
// start address, stride between 8-row groups 1024 bytes, descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(const void* tile) {
  const uint64_t a = (saddr(tile) & 0x3FFFFu) >> 4;
  return a | (uint64_t(1) << 16) | (uint64_t(1024 >> 4) << 32) | (uint64_t(1) << 46) | (uint64_t(2) << 61);
}
// D (tensor memory) += A B^T with A read from tensor memory (a_tmem: the column
// of A's first K element, lane 0) and B from shared memory (descriptor bd)
__device__ __forceinline__ void mma_tf32_ts(uint32_t tmem, uint32_t a_tmem, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem),
      "r"(a_tmem), "l"(bd), "r"(idesc), "r"(acc)
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
// 16 consecutive columns of this warp's 32 lanes from registers (completion: tcgen05.wait::st)
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
}
template <int BN>
struct TcCfg {
  // head x [B head | B tail] as one MMA of N = 2 BN (the MMA's time is flat up
  // to N = 64: about 55 cycles for M = 128, K = 8), the tail product beside it
  static constexpr bool kMerge = BN <= 64;
  static constexpr int kAccCols = kMerge ? 2 * BN : BN;  // columns of one accumulator
  // two blocks per SM for up to 16 kets (each with half the tensor memory and
  // shared memory): one block's MMA issue waits for its own k blocks' copies
  // and MMAs while the other's MMAs run (kernel 40.5 against 45.4 us on n = 4096, 16 kets)
  static constexpr int kPerSM = BN <= 32 ? 2 : 1;
  static constexpr int kTmemCols = kTcTmemCols / kPerSM;  // allocated per block
  static constexpr int kAcc = 2;                         // accumulators, used in turn
  static constexpr int kGroup = 2;                       // k blocks summed in one accumulator
  static constexpr int kSlots = BN <= 32 ? 2 : 4;        // B stages = tensor-memory A slots
  static constexpr int kSlotCol0 = kAcc * kAccCols;      // first column of the A slots (64 each)
  static constexpr int kATile = kTcBM * kTcBK * 4;       // 16 KB
  static constexpr int kBTile = BN * kTcBK * 4;
  static constexpr int kBStage = 2 * kBTile;             // B head tile, then B tail tile
  static constexpr int kAStages = BN <= 32 ? 5 : (BN <= 64 ? 8 : 5);  // A ring (ARING)
  static constexpr int kBarBytes = 512;
  static constexpr size_t smem(bool aring) {
    return 1024 /* alignment */ + (aring ? (size_t)kAStages * kATile : 0) + (size_t)kSlots * kBStage + kBarBytes;
  }
  static_assert(kSlotCol0 + 64 * kSlots <= kTmemCols, "tensor-memory budget");
  static_assert(kPerSM * (smem(true) + 1024) <= 228 * 1024, "shared memory of kPerSM blocks on one SM");
  static_assert(8 * (2 * kAStages + 3 * kSlots + 2 * kAcc + 1) + 8 <= kBarBytes, "barrier area");
  static_assert(smem(true) <= 227 * 1024, "shared-memory budget of one block");
};

// Y[i, c] (complex rows i < m, kets c < N) = alpha * (Ahat Bhat^T combined) + beta * Y
// for the segments of the block's run that cover a whole row tile; for the
// others their partial products, part[row tile][segment][c][row in the tile].
//
// Pipeline.  The split warps store each Ahat tile into a tensor-memory slot:
// its value, read by the MMA as the TF32 head, and its tail, 32 + 32 columns.
// They take the tile from a ring of kAStages shared-memory stages filled by
// bulk copies (ARING: a matrix streamed once from memory, larger than half
// the L2, which these copies stream fastest; each stage released as soon as
// it is read), or load it themselves from global memory into registers two
// k blocks ahead (a matrix read from L2, as the mode products and the smaller
// operators re-read theirs, where 16-byte loads that each cover 512 bytes of
// a warp are faster).  The Bhat tiles of a k block, brought into shared
// memory by bulk copies, and the tensor-memory slot share an index in a ring
// of kSlots, released by the MMAs' commit.  The MMAs read A from tensor
// memory and B from shared memory.
//
// Accumulation: each group of kGroup k blocks (64 terms) starts a fresh
// accumulator in tensor memory, kAcc of them used in turn; the split warps
// read each finished one and add it to FP32 registers, rounding to nearest.
// The tensor cores' own accumulation (which does not round to nearest) then
// spans 64 terms only, which keeps the FP32 accuracy of the ComplexF32 mode
// for long rows (the error does not grow with n).
// COLS: more than one column tile or a column map other than one stride
// (mode products); without it the kernel keeps one column tile and y's
// columns one stride apart, which the common dense case compiles leaner for.
template <int BN, bool COLS, bool ARING>
__global__ void __launch_bounds__(kTcThreads, TcCfg<BN>::kPerSM)
    k_tc_cgemm(const float* __restrict__ ahat, const float* __restrict__ bh_t, const float* __restrict__ bl_t,
               int64_t m, int mt, int64_t ncols, int nkb, int per, int64_t units, int smax, float2* y, int64_t yes,
               TcColMap ym, float2 alpha, float2 beta, float2* part, unsigned* status) {
  using C = TcCfg<BN>;
  constexpr int SA = ARING ? C::kAStages : 0, K = C::kSlots, NA = C::kAcc, G = C::kGroup;
  extern __shared__ __align__(16) unsigned char tc_smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + (size_t)SA * C::kATile + (size_t)K * C::kBStage);
  uint64_t* afull = bars;                            // [SA] A tile landed          (count 1 + tx)
  uint64_t* aempty = afull + SA;                     // [SA] A tile read            (count kTcWork)
  uint64_t* bfull = aempty + SA;                     // [K] B tiles landed          (count 1 + tx)
  uint64_t* conv = bfull + K;                        // [K] A slot written          (count kTcWork)
  uint64_t* done = conv + K;                         // [K] MMAs of the slot done   (count 1, tcgen05.commit)
  uint64_t* accf = done + K;                         // [NA] accumulator written    (count 1, tcgen05.commit)
  uint64_t* acce = accf + NA;                        // [NA] accumulator read       (count kTcWork)
  uint64_t* fin = acce + NA;                         // every MMA issued has completed (count 1, tcgen05.commit)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fin + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  auto stageA = [&](int s) { return base + (size_t)s * C::kATile; };
  auto stageB = [&](int t) { return base + (size_t)SA * C::kATile + (size_t)t * C::kBStage; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t u0 = (int64_t)blockIdx.x * per;           // first unit of this block
  const int nk = (int)(units - u0 < (int64_t)per ? units - u0 : (int64_t)per);  // >= 1 (the host makes no empty runs)
  // The loops below walk the run with (kb, p): the k block of unit it and its
  // position in its segment; an accumulator group is kGroup k blocks of one
  // segment (it opens one when p % kGroup == 0, closes one at
  // p % kGroup == kGroup - 1 or at the segment's end).
  const int kb_start = (int)(u0 % nkb);

  if (threadIdx.x == 0) {
    for (int s = 0; s < SA; ++s) {
      bar_init(&afull[s], 1);
      bar_init(&aempty[s], kTcWork);
    }
    for (int t = 0; t < K; ++t) {
      bar_init(&bfull[t], 1);
      bar_init(&conv[t], kTcWork);
      bar_init(&done[t], 1);
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
  // with programmatic dependent launch the set-up above overlaps the split
  // kernel; nothing in global memory is touched before this point
  pdl_enter();

  if (warp == 0) {
    if (lane == 0) {  // producer: the B tiles, and the A tiles with ARING
      int issued_a = 0, issued_b = 0;
      int64_t rt = u0 / nkb;                  // combined row tile: column tile * mt + row tile
      int mti = (int)(rt % mt);               // row tile
      int64_t ct = rt / mt;                   // column tile
      for (int it = 0, kb = kb_start; it < nk; ++it) {
        const int t = it % K;
        if constexpr (ARING) {
          const int s = it % SA;
          if (it >= SA && !bar_wait(&aempty[s], ((it / SA) - 1) & 1)) {
            atomicExch(abort_flag, 1);
            break;
          }
          if (*(volatile int*)abort_flag) break;
          bar_expect(&afull[s], C::kATile);
          bulk_copy(stageA(s), ahat + ((int64_t)mti * nkb + kb) * (C::kATile / 4), C::kATile, &afull[s]);
          issued_a = it + 1;
        }
        if (*(volatile int*)abort_flag) break;
        if (it >= K && !bar_wait(&done[t], ((it / K) - 1) & 1)) {
          atomicExch(abort_flag, 1);
          break;
        }
        bar_expect(&bfull[t], C::kBStage);
        const int64_t bt = ((COLS ? ct * nkb : 0) + kb) * (C::kBTile / 4);  // the column tile's Bhat tile of k block kb
        bulk_copy(stageB(t), bh_t + bt, C::kBTile, &bfull[t]);
        bulk_copy(stageB(t) + C::kBTile, bl_t + bt, C::kBTile, &bfull[t]);
        issued_b = it + 1;
        if (++kb == nkb) {
          kb = 0;
          if (++mti == mt) {
            mti = 0;
            ++ct;
          }
        }
      }
      // every copy issued has landed before the block's shared memory goes away
      for (int it = max(0, issued_a - SA); it < issued_a; ++it) bar_wait(&afull[it % SA], (it / SA) & 1);
      for (int it = max(0, issued_b - K); it < issued_b; ++it) bar_wait(&bfull[it % K], (it / K) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      // kind::tf32, FP32 accumulator, A (tensor memory) and B K-major, M = 128, N = BN or 2 BN
      const uint32_t idesc1 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
      const uint32_t idesc2 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)((2 * BN) >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
      int q = -1;  // accumulator group
      for (int it = 0, kb = kb_start, p = 0; it < nk; ++it) {
        const bool first = p % G == 0, last = p % G == G - 1 || kb == nkb - 1 || it == nk - 1;
        if (++kb == nkb) {
          kb = 0;
          p = 0;
        } else {
          ++p;
        }
        if (first) ++q;
        const int t = it % K, b = q % NA;
        if (!bar_wait(&conv[t], (it / K) & 1) || !bar_wait(&bfull[t], (it / K) & 1) ||
            (first && q >= NA && !bar_wait(&acce[b], ((q / NA) - 1) & 1))) {
          atomicExch(abort_flag, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(b * C::kAccCols);
        const uint32_t ta = tmem + (uint32_t)(C::kSlotCol0 + t * 64);  // head columns; the tail 32 further
        const uint64_t bh = sw128_desc(stageB(t)), bl = sw128_desc(stageB(t) + C::kBTile);
#pragma unroll
        for (int kk = 0; kk < kTcBK / 8; ++kk) {  // 8 TF32 = 32 bytes = 2 descriptor units per step
          const uint64_t o = (uint64_t)(2 * kk);
          const uint32_t a_hi = ta + (uint32_t)(8 * kk), a_lo = a_hi + 32;
          const uint32_t acc = (kk > 0 || !first) ? 1u : 0u;
          if (C::kMerge) {
            mma_tf32_ts(d, a_hi, bh + o, idesc2, acc);  // head x [B head | B tail]: columns [0, 2 BN)
            mma_tf32_ts(d, a_lo, bh + o, idesc1, 1u);   // tail x B head: columns [0, BN)
          } else {
            mma_tf32_ts(d, a_hi, bh + o, idesc1, acc);
            mma_tf32_ts(d, a_hi, bl + o, idesc1, 1u);
            mma_tf32_ts(d, a_lo, bh + o, idesc1, 1u);
          }
        }
        mma_commit(&done[t]);
        if (last) mma_commit(&accf[b]);
      }
      mma_commit(fin);  // also after an early exit: fires when every MMA above has completed
    }
  } else {
    // warps 2-9: move each A tile into tensor memory (value and tail); after
    // each group, add the accumulator to registers.  Warps w and w + 4 share
    // tensor-memory lanes 32 * (w % 4) .. (the A rows of those lanes): warp
    // half h moves the tile's columns [16 h, 16 h + 16) and keeps the kets
    // [h * BN/4, (h + 1) * BN/4): their real-part columns and, BN/2 further,
    // their imaginary-part columns.
    const int q4 = warp & 3;
    const int half = (warp - 2) >> 2;
    constexpr int KQ = BN / 4;  // kets per warp half
    const uint32_t lane_addr = tmem + ((uint32_t)(q4 * 32) << 16);
    const int r = q4 * 32 + lane;  // A row of this thread = its tensor-memory lane
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
      const uint32_t col = lane_addr + (uint32_t)(b * C::kAccCols + half * KQ);
#pragma unroll
      for (int c0 = 0; c0 < KQ; c0 += 8) {
        float v[8], w[8];
        tmem_ld8(col + (uint32_t)c0, v);
        tmem_ld8(col + (uint32_t)(BN / 2 + c0), w);
        if (C::kMerge) {
          float v2[8], w2[8];
          tmem_ld8(col + (uint32_t)(BN + c0), v2);
          tmem_ld8(col + (uint32_t)(BN + BN / 2 + c0), w2);
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            v[u] += v2[u];
            w[u] += w2[u];
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          acc_re[c0 + u] += v[u];
          acc_im[c0 + u] += w[u];
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      bar_arrive(&acce[b]);
    };
    // the segment of row tile mt, its k blocks drained into acc_re / acc_im: y
    // when it covers the whole row tile, else its partial product; then the
    // registers start again from zero
    auto epilogue = [&](int64_t rt, bool whole) {
      const int il = r >> 1;                          // complex row in the row tile
      const uint32_t rt32 = (uint32_t)rt;             // units (rt * nkb) stay below 2^31 (the host checks)
      const int64_t i = (int64_t)(rt32 % (uint32_t)mt) * (kTcBM / 2) + il;
      const int64_t c0 = (int64_t)(rt32 / (uint32_t)mt) * (BN / 2);  // first column of the column tile
      const int64_t j = (int64_t)blockIdx.x - (int64_t)((rt32 * (uint32_t)nkb) / (uint32_t)per);  // segment in the row tile
      const bool even = (lane & 1) == 0;
      TcColCursor cur(ym, COLS ? c0 + half * KQ : 0);  // y offset of this thread's first column (COLS)
#pragma unroll
      for (int u = 0; u < KQ; ++u) {
        const int c = half * KQ + u;
        const float other = __shfl_xor_sync(0xffffffffu, acc_im[u], 1);
        const float v = even ? acc_re[u] - other : acc_re[u] + other;  // even lane: Re Y, odd lane: Im Y
        const float w = __shfl_xor_sync(0xffffffffu, v, 1);
        if (even && i < m && c0 + c < ncols) {
          if (!whole) {
            part[((rt * smax + j) * (BN / 2) + c) * (kTcBM / 2) + il] = make_float2(v, w);
          } else {
            float2* yp = y + i * yes + (COLS ? cur.off : (int64_t)c * ym.st);
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
        acc_re[u] = acc_im[u] = 0.f;
        if (COLS) cur.next(ym);
      }
    };
    int q = -1;                                  // accumulator group
    int64_t seg_tile = u0 / nkb;                 // row tile of the current segment
    bool seg_from_zero = kb_start == 0;          // the current segment starts at k block 0
    int kb = kb_start, p = 0;
    // row r, columns [16 half, 16 half + 16) of a tile: four 16-byte loads j,
    // each of the warp's a run of 512 bytes (the tile order of a_slot), from
    // the shared-memory stage (ARING) or from global memory, where the tile
    // of unit (row tile mti, k block kb) starts at float4 (mti * nkb + kb) * 1024
    const int aoff = (q4 * 2 + half) * 4 * 32 + lane;
    const float4* __restrict__ arow = reinterpret_cast<const float4*>(ahat) + aoff;
    // direct loads: two tiles in flight, units it + 1 (nx) and it + 2 (nx2), while unit it is stored
    int fmti = (int)((uint32_t)seg_tile % (uint32_t)mt), fkb = kb_start;  // the unit last loaded
    auto load = [&](float4 (&v)[4]) {
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = __ldg(arow + ((int64_t)fmti * nkb + fkb) * (C::kATile / 16) + 32 * j);
    };
    auto advance = [&] {
      if (++fkb == nkb) {
        fkb = 0;
        if (++fmti == mt) fmti = 0;
      }
    };
    float4 nx[4], nx2[4];
    if constexpr (!ARING) {
      load(nx);
      if (nk > 1) {
        advance();
        load(nx2);
      }
    }
    for (int it = 0; it < nk && ok; ++it) {
      const int s = ARING ? it % SA : 0, t = it % K;
      float hv[16];
      if constexpr (!ARING) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          hv[4 * j] = nx[j].x;
          hv[4 * j + 1] = nx[j].y;
          hv[4 * j + 2] = nx[j].z;
          hv[4 * j + 3] = nx[j].w;
          nx[j] = nx2[j];
        }
        if (it + 2 < nk) {  // the unit after next, loaded while this one is stored
          advance();
          load(nx2);
        }
      }
      // warp-uniform, as the tensor-memory stores below need the whole warp
      if (!__all_sync(0xffffffffu, !*(volatile int*)abort_flag && (!ARING || bar_wait(&afull[s], (it / SA) & 1)) &&
                                       (it < K || bar_wait(&done[t], ((it / K) - 1) & 1)))) {
        ok = false;
        break;
      }
      if constexpr (ARING) {
        const float4* a = reinterpret_cast<const float4*>(stageA(s)) + aoff;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float4 x = a[32 * j];
          hv[4 * j] = x.x;
          hv[4 * j + 1] = x.y;
          hv[4 * j + 2] = x.z;
          hv[4 * j + 3] = x.w;
        }
        bar_arrive(&aempty[s]);  // the stage may be refilled
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // the MMAs read the value as TF32 (its head, truncated); the tail 32 columns further
      const uint32_t ta = lane_addr + (uint32_t)(C::kSlotCol0 + t * 64 + 16 * half);
      tmem_st16(ta, hv);
#pragma unroll
      for (int j = 0; j < 16; ++j) hv[j] = tf32_tail(hv[j]);
      tmem_st16(ta + 32, hv);
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      bar_arrive(&conv[t]);
      if (p % G == 0) {
        ++q;
        if (q > 0) {
          drain(q - 1);  // the previous group, once this one has begun
          if (ok && kb == 0 && it > 0) {  // ... which closed the previous segment, a whole row tile's tail
            epilogue(seg_tile, seg_from_zero);
            ++seg_tile;
            seg_from_zero = true;
          }
        }
      }
      if (++kb == nkb) {
        kb = 0;
        p = 0;
      } else {
        ++p;
      }
    }
    if (ok) drain(q);  // the last group
    if (ok) epilogue(seg_tile, seg_from_zero && kb == 0);  // whole when the run ended at the tile's last k block
    ok = __all_sync(0xffffffffu, ok && !*(volatile int*)abort_flag);
    if (!ok) {
      atomicExch(abort_flag, 1);
      if (lane == 0 && status) atomicOr(status, kTcErrTimeout);
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

// Bhat head and tail of the ncols columns (x's column c at element offset
// tc_col_offset(xm, c), elements k * xes apart) in column tiles of H = BN / 2
// columns: in tile ct, row j = Re X[:, ct * H + j], row H + j = Im X[:, ct * H + j],
// value and TF32 tail, as swizzled tiles of BN rows x 32 floats, tile
// (ct, k block) at float offset (ct * nkb + k block) * BN * 32 (zero beyond n).
template <int BN>
__global__ void k_tc_split_b(const float2* __restrict__ x, int64_t n, int64_t xes, TcColMap xm, int64_t ncols,
                             int64_t nkb, float* __restrict__ bh, float* __restrict__ bl) {
  constexpr int H = BN / 2;
  pdl_enter();
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nkb * kTcBK) return;
  const int kk = (int)(k % kTcBK);
  for (uint32_t cg = blockIdx.y; cg < (uint32_t)ncols; cg += gridDim.y) {
    float2 v = make_float2(0.f, 0.f);
    if (k < n) v = x[k * xes + tc_col_offset(xm, cg)];
    const uint32_t ct = cg / H;
    const int j = (int)(cg % H);
    const int64_t tile = ((int64_t)ct * nkb + k / kTcBK) * (int64_t)BN * kTcBK;
    const int64_t o_re = tile + swz(j, kk), o_im = tile + swz(H + j, kk);
    bh[o_re] = v.x;  // read as TF32 by the MMA: its truncated head
    bl[o_re] = tf32_tail(v.x);
    bh[o_im] = v.y;
    bl[o_im] = tf32_tail(v.y);
  }
}

// y[i, c] = alpha * (sum of the segments' partial products of (i, c)'s
// combined row tile, in k order) + beta * y[i, c], for the row tiles split over
// more than one block (a row tile that one block covered was written by that
// block); c's column tile is c / H, its combined row tile column tile * mt + i / 64.
template <int BN>
__global__ void k_tc_reduce(const float2* __restrict__ part, int mt, int nkb, int per, int smax, int64_t m,
                            int64_t ncols, float2* __restrict__ y, int64_t yes, TcColMap ym, float2 alpha,
                            float2 beta) {
  constexpr int H = BN / 2;
  pdl_enter();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int il = (int)(i % (kTcBM / 2));
  const uint32_t mti = (uint32_t)(i / (kTcBM / 2));
  for (uint32_t cg = blockIdx.y; cg < (uint32_t)ncols; cg += gridDim.y) {
    const uint32_t rt = (cg / H) * (uint32_t)mt + mti;  // units (rt * nkb) stay below 2^31 (the host checks)
    const int c = (int)(cg % H);
    const uint32_t b0 = (rt * (uint32_t)nkb) / (uint32_t)per, b1 = (rt * (uint32_t)nkb + nkb - 1) / (uint32_t)per;
    if (b1 == b0) continue;
    float sr = 0.f, si = 0.f;
    for (uint32_t j = 0; j <= b1 - b0; ++j) {
      const float2 p = part[(((int64_t)rt * smax + j) * H + c) * (kTcBM / 2) + il];
      sr += p.x;
      si += p.y;
    }
    float2* yp = y + i * yes + tc_col_offset(ym, cg);
    float re = alpha.x * sr - alpha.y * si;
    float im = alpha.x * si + alpha.y * sr;
    if (beta.x != 0.f || beta.y != 0.f) {
      const float2 o = *yp;
      re = __fmaf_rn(beta.x, o.x, __fmaf_rn(-beta.y, o.y, re));
      im = __fmaf_rn(beta.x, o.y, __fmaf_rn(beta.y, o.x, im));
    }
    *yp = make_float2(re, im);
  }
}

template <int BN>
void run_tc(const TcDense& d, const float2* x, int64_t xes, const TcColMap& xm, int64_t ncols, float2* y,
            int64_t yes, const TcColMap& ym, float2 alpha, float2 beta, Workspace* ws, int slot, cudaStream_t s,
            unsigned* status, int num_sms, bool pdl) {
  using C = TcCfg<BN>;
  constexpr int H = BN / 2;
  const int64_t nkb = d.ldk / kTcBK;
  const int64_t ncolt = (ncols + H - 1) / H;
  // split vectors: head and tail tiles of Bhat (the rows of a last column tile's missing columns stay zero)
  const size_t bbytes = (size_t)ncolt * nkb * C::kBTile;
  char* w = static_cast<char*>(ws->get(slot, 2 * bbytes + 256));
  float* bh = reinterpret_cast<float*>(w);
  float* bl = reinterpret_cast<float*>(w + bbytes);
  if (ncols % H != 0) QOB_CUDA(cudaMemsetAsync(w, 0, 2 * bbytes, s));
  const unsigned gy = (unsigned)std::min<int64_t>(ncols, 65535);
  launch_kernel(pdl, k_tc_split_b<BN>, dim3((unsigned)((d.ldk + 255) / 256), gy), 256u, 0, s, x, d.n, xes, xm, ncols,
                nkb, bh, bl);
  QOB_LAUNCHED();
  const int64_t mt = d.mtiles;
  // units (column tile, row tile, k block), in that order of significance:
  // whole row tiles when they fill the SMs, else equal runs over exactly one
  // wave of blocks (each at least 4 k blocks)
  const int64_t rtiles = ncolt * mt, units = rtiles * nkb, wave = (int64_t)C::kPerSM * num_sms;
  const int per = rtiles >= wave ? (int)nkb : (int)std::max<int64_t>(4, (units + wave - 1) / wave);
  const int64_t blocks = (units + per - 1) / per;
  const int smax = (int)((nkb - 1) / per + 2);  // segments of one row tile, at most
  float2* part = nullptr;
  if (per % nkb != 0)
    part = static_cast<float2*>(ws->get(slot + 1, (size_t)rtiles * smax * H * (kTcBM / 2) * sizeof(float2)));
  const bool cols = ncolt > 1 || ym.s1 != 1 || ym.s3 != 1;
  // the A ring for a matrix streamed once from memory (one column tile, larger
  // than half the L2), direct loads for one read from L2
  const bool aring = !cols && d.stream_a;
  auto kern = cols ? k_tc_cgemm<BN, true, false> : aring ? k_tc_cgemm<BN, false, true> : k_tc_cgemm<BN, false, false>;
  const size_t smem = C::smem(aring);
  QOB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  launch_kernel(pdl, kern, dim3((unsigned)blocks), (unsigned)kTcThreads, smem, s,
                static_cast<const float*>(d.ahat.p), (const float*)bh, (const float*)bl, d.m, (int)mt, ncols, (int)nkb,
                per, units, smax, y, yes, ym, alpha, beta, part, status);
  QOB_LAUNCHED();
  if (part) {
    launch_kernel(pdl, k_tc_reduce<BN>, dim3((unsigned)((d.m + 127) / 128), gy), 128u, 0, s, (const float2*)part,
                  (int)mt, (int)nkb, per, smax, d.m, ncols, y, yes, ym, alpha, beta);
    QOB_LAUNCHED();
  }
}

// Position of element (row rr, column kk) in an Ahat tile: the order in which
// the split warps load it.  Warp half h of the warps that own tensor-memory
// lanes 32 q .. 32 q + 31 loads columns [16 h, 16 h + 16) of those rows as
// four 16-byte loads j (columns 16 h + 4 j .. + 3), lane l for row 32 q + l, so
// that each load of a warp reads 512 consecutive bytes.
__device__ __forceinline__ int a_slot(int rr, int kk) {
  const int q = rr >> 5, l = rr & 31, h = kk >> 4, jj = (kk >> 2) & 3, e = kk & 3;
  return ((((q * 2 + h) * 4 + jj) * 32 + l) << 2) + e;
}

// Ahat of the stored ComplexF32 matrix (column-major m x n, on the device) as
// 128 x 32 tiles, tile (t, b) at float offset (t * nkb + b) * 4096, each in the
// order the split warps of k_tc_cgemm load it (a_slot): row 2i = Re A[i, :],
// row 2i + 1 = Im A[i, :]; zero beyond the matrix.
__global__ void k_tc_build_ahat(const float2* __restrict__ a, int64_t m, int64_t n, int64_t nkb, float* __restrict__ ah) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // complex row
  const int64_t k = blockIdx.y;
  const int64_t mpad = (2 * m + kTcBM - 1) / kTcBM * kTcBM / 2;
  if (i >= mpad || k >= nkb * kTcBK) return;
  const float2 v = (i < m && k < n) ? a[i + k * m] : make_float2(0.f, 0.f);
  const int64_t r = 2 * i;  // Ahat row of the real part; the imaginary part is the next row of the same tile
  const int64_t tile = ((r / kTcBM) * nkb + k / kTcBK) * (int64_t)(kTcBM * kTcBK);
  const int rr = (int)(r % kTcBM), kk = (int)(k % kTcBK);
  ah[tile + a_slot(rr, kk)] = v.x;
  ah[tile + a_slot(rr + 1, kk)] = v.y;
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
  int dev = 0, l2 = 0;
  QOB_CUDA(cudaGetDevice(&dev));
  QOB_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
  d.stream_a = d.ahat.bytes > (size_t)l2 / 2;
  const int64_t mpad = d.mtiles * kTcBM / 2;
  k_tc_build_ahat<<<dim3((unsigned)((mpad + 127) / 128), (unsigned)d.ldk), 128, 0, s>>>(
      static_cast<const float2*>(a), m, n, nkb, static_cast<float*>(d.ahat.p));
  QOB_LAUNCHED();
  d.ready = true;
}

bool launch_gemm_tc(const TcDense& d, c128 alpha, const void* x, int64_t xes, const TcColMap& xm, c128 beta,
                    void* y, int64_t yes, const TcColMap& ym, int64_t ncols, cudaStream_t s, Workspace* ws, int slot,
                    unsigned* status, int num_sms, bool pdl) {
  if (!d.ready || ncols < 1) return false;
  // (column tile, row tile, k block) units and column indices are counted in 32 bits
  if (ncols >= ((int64_t)1 << 31) ||
      (int64_t)(d.mtiles * ((ncols + 15) / 16)) > ((int64_t)1 << 31) / (d.ldk / kTcBK))
    fail(QOB_ERR_UNSUPPORTED, "tensor-core product: too many tiles");
  const float2 a = make_float2((float)alpha.re, (float)alpha.im), b = make_float2((float)beta.re, (float)beta.im);
  const float2* xc = static_cast<const float2*>(x);
  float2* yc = static_cast<float2*>(y);
  if (ncols <= 16)
    run_tc<32>(d, xc, xes, xm, ncols, yc, yes, ym, a, b, ws, slot, s, status, num_sms, pdl);
  else if (ncols <= 32)
    run_tc<64>(d, xc, xes, xm, ncols, yc, yes, ym, a, b, ws, slot, s, status, num_sms, pdl);
  else  // column tiles of 64 (BN = 128 rows of Bhat), all in one launch
    run_tc<128>(d, xc, xes, xm, ncols, yc, yes, ym, a, b, ws, slot, s, status, num_sms, pdl);
  return true;
}

bool launch_dense_tc(const TcDense& d, c128 alpha, const void* x, int64_t xes, int64_t xcs, c128 beta, void* y,
                     int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s, Workspace* ws, int slot,
                     unsigned* status, int num_sms, bool pdl) {
  TcColMap xm, ym;  // kets: column c at c * (column stride)
  xm.st = xcs;
  ym.st = ycs;
  return launch_gemm_tc(d, alpha, x, xes, xm, beta, y, yes, ym, ncols, s, ws, slot, status, num_sms, pdl);
}

}  // namespace qob
