// noalloc.cu -- qob_dot_noalloc: the FP64 inner product <x|y> without any
// device allocation.
//
// Who needs it: callers that must not call cudaMalloc / cudaFree while they
// work.  Examples: a host program whose memory pool already owns the device's
// memory and enforces its own budget; code that issues work while a stream is
// being captured into a CUDA graph, where an allocation would break or
// serialise the capture; a Julia finalizer or callback that must not trigger
// allocation.  The ordinary qob_dot stages its per-block partial sums in a
// context buffer that grows with cudaMalloc and returns the result through
// pinned host memory; this entry point keeps the partial sums in a fixed
// file-scope device array and writes the result to device memory the caller
// already owns.
//
// Limits and sharing:
//   * the scratch array holds kNaMaxPartials partial sums (128 KiB), loaded
//     with the library and held on every GPU that loads it until the process
//     exits; one partial covers kNaPerBlock elements, so n is limited to
//     kNaMaxElements = 16,777,216; larger n is rejected with QOB_ERR_ARG;
//   * every call shares the one array: calls that overlap on the GPU (two
//     streams, or two host threads) race on it and give wrong results.  Issue
//     them on one stream, or order them;
//   * each call writes every partial it later reads, so nothing in the array
//     has to start at zero and the previous call's leftovers are never read;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it; make that
//     first call before any stream capture.
#include <cuda_runtime.h>

#include <exception>
#include <mutex>
#include <new>

#include "qob_internal.h"

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaItems = 8;
constexpr int64_t kNaPerBlock = (int64_t)kNaThreads * kNaItems;  // 2048 elements per partial
constexpr int kNaMaxPartials = 8192;                                // 8192 x 16 B = 128 KiB
constexpr int64_t kNaMaxElements = kNaPerBlock * kNaMaxPartials;   // 16,777,216
constexpr int kNaMaxDevices = 64;

// File-scope scratch.  Host code must not pass g_na_partials itself to a
// kernel: in host code the name is a host-side stand-in, not a device address.
__device__ __align__(256) double2 g_na_partials[kNaMaxPartials];

std::mutex g_na_mutex;
void* g_na_ptr[kNaMaxDevices] = {};

// Block b sums conj(x[i]) * y[i] over its 2048 elements (coalesced: thread t
// reads i = b * 2048 + k * 256 + t), then a shared-memory tree.
template <typename CT>
__global__ void __launch_bounds__(kNaThreads) k_na_partial(const CT* __restrict__ x, const CT* __restrict__ y,
                                                          int64_t n, double2* __restrict__ part) {
  __shared__ double sre[kNaThreads], sim[kNaThreads];
  double re = 0.0, im = 0.0;
  const int64_t base = (int64_t)blockIdx.x * kNaPerBlock + threadIdx.x;
#pragma unroll
  for (int k = 0; k < kNaItems; ++k) {
    const int64_t i = base + (int64_t)k * kNaThreads;
    if (i < n) {
      const CT a = x[i], b = y[i];
      const double ax = a.x, ay = a.y, bx = b.x, by = b.y;
      re = fma(ax, bx, re);
      re = fma(ay, by, re);
      im = fma(ax, by, im);
      im = fma(-ay, bx, im);
    }
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int w = kNaThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sre[threadIdx.x] += sre[threadIdx.x + w];
      sim[threadIdx.x] += sim[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sre[0], sim[0]);
}

// One block adds the nparts partials in a fixed order and writes (re, im).
__global__ void __launch_bounds__(kNaThreads) k_na_final(const double2* __restrict__ part, int nparts,
                                                        double* __restrict__ out) {
  __shared__ double sre[kNaThreads], sim[kNaThreads];
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < nparts; i += kNaThreads) {
    re += part[i].x;
    im += part[i].y;
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int w = kNaThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sre[threadIdx.x] += sre[threadIdx.x + w];
      sim[threadIdx.x] += sim[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sre[0];
    out[1] = sim[0];
  }
}

// Device address of the scratch array on the current device, looked up once.
double2* scratch_on(int device) {
  if (device < 0 || device >= kNaMaxDevices) qob::fail(QOB_ERR_ARG, "qob_dot_noalloc: device index out of range");
  std::lock_guard<std::mutex> lk(g_na_mutex);
  if (!g_na_ptr[device]) {
    void* p = nullptr;
    QOB_CUDA(cudaGetSymbolAddress(&p, g_na_partials));
    if (!p) qob::fail(QOB_ERR_CUDA, "qob_dot_noalloc: scratch array has no device address");
    g_na_ptr[device] = p;
  }
  return static_cast<double2*>(g_na_ptr[device]);
}

}  // namespace

extern "C" int qob_dot_noalloc(qob_ctx* ctx, int dtype, const void* x, const void* y, int64_t n, double* result,
                               void* stream) {
  if (!ctx) return QOB_ERR_ARG;
  try {
    QOB_CUDA(cudaSetDevice(ctx->c.device));
    if (dtype != QOB_C128 && dtype != QOB_C64) qob::fail(QOB_ERR_ARG, "qob_dot_noalloc: dtype must be QOB_C128 or QOB_C64");
    if (!result || n < 0 || (n > 0 && (!x || !y))) qob::fail(QOB_ERR_ARG, "qob_dot_noalloc: bad arguments");
    if (n > kNaMaxElements)
      qob::fail(QOB_ERR_ARG,
                "qob_dot_noalloc: n exceeds the 16777216-element limit of its 128 KiB static scratch; use qob_dot");
    double2* part = scratch_on(ctx->c.device);
    const int nparts = (int)((n + kNaPerBlock - 1) / kNaPerBlock);
    cudaStream_t s = (cudaStream_t)stream;
    if (nparts > 0) {
      if (dtype == QOB_C128)
        k_na_partial<double2><<<nparts, kNaThreads, 0, s>>>((const double2*)x, (const double2*)y, n, part);
      else
        k_na_partial<float2><<<nparts, kNaThreads, 0, s>>>((const float2*)x, (const float2*)y, n, part);
      QOB_LAUNCHED();
    }
    k_na_final<<<1, kNaThreads, 0, s>>>(part, nparts, result);
    QOB_LAUNCHED();
    return QOB_OK;
  } catch (const qob::Error& e) {
    ctx->c.err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    ctx->c.err = "host out of memory";
    return QOB_ERR_OOM;
  } catch (const std::exception& e) {  // e.g. std::system_error from locking the mutex
    ctx->c.err = e.what();
    return QOB_ERR_ARG;
  }
}
