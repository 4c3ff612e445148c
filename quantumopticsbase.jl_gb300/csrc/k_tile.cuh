// k_tile.cuh -- the fused LazySum gather with the input staged in shared
// memory, for plans in the compact form (every merged group one run of
// power-of-two subsystems with one stored entry per row: spin chains and
// other two-level systems) on kets stored one after another.
//
// A block owns a tile of P = 2^tbits consecutive output indices J of up to
// TC x ls kets.  One thread copies the tile's input rows x[J0 .. J0 + P) of
// those kets into shared memory with bulk asynchronous copies (cp.async.bulk,
// completion counted on an mbarrier); meanwhile the block stages the groups'
// compact records and slots.  A group whose index bits all lie below tbits
// maps every J of the tile to a partner J' = J - (r << shift) + col inside the
// same tile, so its gathers read shared memory; the others (the bonds between
// the high subsystems) gather from global memory, where the partner tile is
// another block's input and sits in L2.  The arithmetic and its order are those
// of k_gather_j: the merged diagonal first, then the groups in plan order, then
// y = alpha * acc + beta * y (the two agree to rounding: the compiler may fuse a
// multiply and an add differently in the two kernels).
//
// Threads: a warp covers 32 / ls consecutive J x ls sets of TC kets (ket q + k
// * ls of the block for set q), as in k_gather_j's lane split; the staged rows
// are padded by 64 bytes so that the sets of a warp fall in different banks.
//
// The wait for the copies is bounded: after kTileWaitPolls polls the block
// records kErrWaitTimeout in the context's device status word, waits (again
// bounded) for its copies to land, and returns without computing.
// Included by k_gather.cuh (after the accumulators, before the host dispatch).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

namespace qob {
namespace gather {

constexpr unsigned kErrWaitTimeout = 1u;  // device status bits (Context::status); kErrBoundsBit = 2
constexpr int kTileWaitPolls = 1 << 20;   // x >= 64 ns sleep between polls: > 60 ms in all
constexpr int kTilePadBytes = 64;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Polls the barrier's phase `parity` at most kTileWaitPolls times.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < kTileWaitPolls; ++i) {
    if (mbar_test(bar, parity)) return true;
    __nanosleep(64);
  }
  return false;
}
// bytes (a multiple of 16) from global src to shared dst, both 16-byte aligned,
// counted on bar
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

template <typename XT>
__host__ __device__ constexpr int tile_pad() {
  return kTilePadBytes / (int)sizeof(XT);
}

// Shared memory of one block: the mbarrier (16 bytes), the staged rows, the
// groups' compact records, the slots when staged.
template <typename XT, typename ET>
__host__ __device__ inline size_t tile_smem(int tbits, int kpc, int ngroups, int ell_slots, bool ell_smem) {
  const size_t rows = (size_t)kpc * (((size_t)1 << tbits) + tile_pad<XT>()) * sizeof(XT);
  return 16 + rows + (size_t)ngroups * sizeof(int4) + (ell_smem ? (size_t)ell_slots * sizeof(ET) : 0);
}

template <typename R, int VM, int TC, int BMODE>
__global__ void __launch_bounds__(256) k_gather_t(GatherView g, const typename In<R>::T* __restrict__ x, int64_t xcs,
                                                  typename Cx<R>::T* __restrict__ y, int64_t ycs, int ncols,
                                                  typename Cx<R>::T alpha, typename Cx<R>::T beta, int tbits,
                                                  unsigned* status) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  using AT = typename AccOf<R>::T;
  using ET = typename Ell<R, VM != kComplex>::T;
  using VT = typename Val<R, VM != kComplex>::T;
  using DT = typename Val<R, VM == kReal>::T;
  extern __shared__ __align__(16) unsigned char tile_smem_raw[];
  const uint32_t P = 1u << tbits;
  const int ls = g.lane_split;
  const int lsh = __ffs(ls) - 1, jsh = 5 - lsh;
  const int kpc = TC * ls;  // kets per block
  const int rowlen = (int)P + tile_pad<XT>();
  const uint32_t ntiles = (uint32_t)(g.m >> tbits);
  const uint32_t tile = blockIdx.x % ntiles;
  const int c_base = (int)(blockIdx.x / ntiles) * kpc;
  const int nk = min(kpc, ncols - c_base);  // kets of this block (>= 1)
  const uint32_t J0 = tile << tbits;

  uint64_t* bar = reinterpret_cast<uint64_t*>(tile_smem_raw);
  XT* xs = reinterpret_cast<XT*>(tile_smem_raw + 16);
  size_t off = 16 + (size_t)kpc * rowlen * sizeof(XT);
  int4* rec = reinterpret_cast<int4*>(tile_smem_raw + off);
  off += (size_t)g.ngroups * sizeof(int4);

  pdl_enter();
  if (threadIdx.x == 0) mbar_init(bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t row_bytes = P * (uint32_t)sizeof(XT);
    mbar_expect_tx(bar, row_bytes * (uint32_t)nk);
    for (int t = 0; t < nk; ++t) bulk_to_smem(xs + (size_t)t * rowlen, x + (int64_t)(c_base + t) * xcs + J0, row_bytes, bar);
  }
  // compact records with a flag (bit 1 of w) for groups inside the tile, and the
  // slots, while the rows are in flight
  for (int i = threadIdx.x; i < g.ngroups; i += blockDim.x) {
    int4 f = g.fastg[i];
    const uint32_t top = (uint32_t)f.y << f.x;  // the group's largest index offset
    f.w = (f.w & 1) | (top < P ? 2 : 0);
    rec[i] = f;
  }
  const ET* ell = static_cast<const ET*>(g.ell);
  if (g.ell_smem) {
    ET* se = reinterpret_cast<ET*>(tile_smem_raw + off);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(g.ell);
    uint32_t* dst = reinterpret_cast<uint32_t*>(se);
    const int words = g.ell_slots * (int)(sizeof(ET) / 4);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    ell = se;
  }
  __syncthreads();
  if (!mbar_wait_bounded(bar, 0)) {
    if (status) atomicOr(status, kErrWaitTimeout);
    mbar_wait_bounded(bar, 0);  // let the copies land before the block's shared memory goes away
    return;
  }

  const int lane = threadIdx.x & 31;
  const int q = lane >> jsh;  // ket set of this lane
  const int nt = q < nk ? min(TC, (nk - q + ls - 1) >> lsh) : 0;
  const int nwarps = blockDim.x >> 5;
  const XT* xrow = xs + (size_t)q * rowlen;
  const XT* xglob = x + (int64_t)(c_base + q) * xcs;
  const int64_t vs_s = (int64_t)ls * rowlen, vs_x = (int64_t)ls * xcs, vs_y = (int64_t)ls * ycs;
  CT* ybase = y + (int64_t)(c_base + q) * ycs;
  for (uint32_t jb = (uint32_t)(threadIdx.x >> 5) << jsh; jb < P; jb += (uint32_t)nwarps << jsh) {
    const uint32_t j = jb + (uint32_t)(lane & ((1 << jsh) - 1));
    const uint32_t J = J0 + j;
    AT acc[TC];
    if (g.has_diag) {
      const DT d = static_cast<const DT*>(g.diag)[J];
#pragma unroll
      for (int t = 0; t < TC; ++t)
        if (t < nt) acc[t].set(d, xrow[j + t * vs_s]);
    } else {
#pragma unroll
      for (int t = 0; t < TC; ++t) acc[t].zero();
    }
#pragma unroll 4
    for (int gi = 0; gi < g.ngroups; ++gi) {
      const int4 f = rec[gi];
      const uint32_t r = (J >> f.x) & (uint32_t)f.y;
      if (kDebugBounds && out_of_range((int64_t)f.z + r, g.ell_slots, g.status)) continue;
      const ET s = ell[f.z + r];
      const VT v = Ell<R, VM != kComplex>::v(s);
      if (nz(v)) {
        const uint32_t Jp = J - (r << f.x) + (uint32_t)s.col;
        if (kDebugBounds && ((f.w & 2) ? out_of_range((int64_t)Jp - J0, P, g.status)
                                       : out_of_range((int64_t)Jp, g.n, g.status)))
          continue;
        const bool im = VM == kPhased && (f.w & 1);
        if (f.w & 2) {  // partner inside the tile: shared memory
          const XT* xp = xrow + (Jp - J0);
          if (im) {
#pragma unroll
            for (int t = 0; t < TC; ++t)
              if (t < nt) acc[t].mac_i(v, xp[t * vs_s]);
          } else {
#pragma unroll
            for (int t = 0; t < TC; ++t)
              if (t < nt) acc[t].mac(v, xp[t * vs_s]);
          }
        } else {  // partner in another tile: global memory (L2)
          const XT* xp = xglob + Jp;
          if (im) {
#pragma unroll
            for (int t = 0; t < TC; ++t)
              if (t < nt) acc[t].mac_i(v, ld(xp + t * vs_x));
          } else {
#pragma unroll
            for (int t = 0; t < TC; ++t)
              if (t < nt) acc[t].mac(v, ld(xp + t * vs_x));
          }
        }
      }
    }
    CT* yp = ybase + J;
#pragma unroll
    for (int t = 0; t < TC; ++t)
      if (t < nt) combine<BMODE>(yp + t * vs_y, acc[t].total(), alpha, beta);
  }
}

// Whether a launch of the tiled kernel fits this call (checked on the host).
template <typename R>
bool tile_fits(const GatherView& v, int tbits, const void* x, int64_t xcs, int64_t ncols) {
  using XT = typename In<R>::T;
  if (!v.fast || !v.square || tbits < 6 || v.m <= 0 || v.m > (int64_t(1) << 31)) return false;
  if ((v.m & (v.m - 1)) != 0 || (v.m >> tbits) < 1) return false;  // a power-of-two length, whole tiles
  // 16-byte alignment of every bulk copy's source
  if (((uintptr_t)x & 15u) != 0 || ((xcs * (int64_t)sizeof(XT)) & 15) != 0) return false;
  (void)ncols;
  return true;
}

template <typename R, int VM, int TC, int BMODE>
void launch_t(const GatherView& v, const void* x, int64_t xcs, void* y, int64_t ycs, int64_t ncols,
              typename Cx<R>::T a, typename Cx<R>::T b, cudaStream_t s, unsigned* status) {
  using CT = typename Cx<R>::T;
  using XT = typename In<R>::T;
  using ET = typename Ell<R, VM != kComplex>::T;
  int ls = v.lane_split > 0 ? v.lane_split : 1;
  while (ls > 1 && (int64_t)TC * ls > ncols) ls >>= 1;
  GatherView w = v;
  w.lane_split = ls;
  const int kpc = TC * ls;
  const int tbits = v.tile_bits;
  const size_t smem = tile_smem<XT, ET>(tbits, kpc, v.ngroups, v.ell_slots, v.ell_smem != 0);
  auto kern = k_gather_t<R, VM, TC, BMODE>;
  QOB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int threads = v.block > 0 ? v.block : 256;
  const int64_t ntiles = v.m >> tbits;
  // column groups of at most 2^31 / ntiles blocks per launch
  const int64_t groups_per_launch = std::max<int64_t>(1, (int64_t(1) << 31) / ntiles - 1);
  for (int64_t c0 = 0; c0 < ncols; c0 += groups_per_launch * kpc) {
    const int64_t nc = std::min<int64_t>(ncols - c0, groups_per_launch * kpc);
    const int64_t blocks = ntiles * ((nc + kpc - 1) / kpc);
    launch_kernel(v.pdl != 0, kern, dim3((unsigned)blocks), (unsigned)threads, smem, s, w, (const XT*)x + c0 * xcs,
                  xcs, (CT*)y + c0 * ycs, ycs, (int)nc, a, b, tbits, status);
    QOB_LAUNCHED();
  }
}

}  // namespace gather
}  // namespace qob
