// batch.cu -- many operator applications of uneven size in one persistent launch.
//
// A batch holds items (op, x, y, alpha, beta): y = alpha * op * x + beta * y for
// one ket per item, each item with its own operator and Hilbert-space
// dimension (e.g. 256 two-mode cavities with dimensions 81 ... 4225).  The
// reference would issue one mul! per model (src/operators_lazysum.jl:189-200);
// here the fused gather of every item runs in ONE launch: the items' output
// index ranges are cut into equal tiles, a device table lists (item, first
// index) per tile, and a persistent grid of blocks walks the tiles, staging
// each tile's group tables in shared memory.  The launch only reads device
// tables that stay in place, so it can be captured in a CUDA graph and
// replayed; qob_batch_tune picks the tile length by timing.
//
// Items whose operator has parts outside the fused gather (large dense
// factors, dense full-space terms, LazyProducts) or a non-square basis, and
// real-valued items in a batch that also holds complex-valued ones, run as
// ordinary per-item applications after the persistent launch.
//
// The same tables drive the serving engine's batched RK4 stages (evolve.cu).
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "batch.h"
#include "k_gather.cuh"

namespace qob {

namespace {

// k of an RK4 stage into the stage combination (the arithmetic of
// k_rk4_stage, element by element): 1: acc = k, tmp = psi + dt/2 k; 2, 3:
// acc += 2 k, tmp = psi + (dt/2 | dt) k; 4: psi += dt/6 (acc + k)
template <typename CT, typename S>
__device__ __forceinline__ void rk4_stage_element(const BatchItemDev& it, int64_t j, CT kv, int stage) {
  CT* psi = (CT*)it.psi;
  CT* acc = (CT*)it.acc;
  CT* tmp = (CT*)it.tmp_out;
  const S dt = (S)it.dt;
  if (stage == 1) {
    const CT p = psi[j];
    const S c = dt * (S)0.5;
    acc[j] = kv;
    CT o;
    o.x = p.x + c * kv.x;
    o.y = p.y + c * kv.y;
    tmp[j] = o;
  } else if (stage == 2 || stage == 3) {
    const CT p = psi[j];
    const S c = stage == 2 ? dt * (S)0.5 : dt;
    CT a = acc[j];
    a.x += (S)2 * kv.x;
    a.y += (S)2 * kv.y;
    acc[j] = a;
    CT o;
    o.x = p.x + c * kv.x;
    o.y = p.y + c * kv.y;
    tmp[j] = o;
  } else {
    const CT a = acc[j];
    CT p = psi[j];
    const S c = dt / (S)6;
    p.x += c * (a.x + kv.x);
    p.y += c * (a.y + kv.y);
    psi[j] = p;
  }
}

// RK4 instantiates the fused-stage epilogue (stage 1..4 at run time); the
// plain instantiation keeps the y = alpha k + beta y epilogue alone, so the
// batched product does not carry the stage code's registers and branches.
template <typename R, bool REALV, bool RK4>
__global__ void __launch_bounds__(256) k_gather_batch(const BatchItemDev* __restrict__ items,
                                                      const int2* __restrict__ tiles, int ntiles, int tile,
                                                      int stage) {
  using CT = typename gather::Cx<R>::T;
  using AT = typename gather::AccOf<R>::T;
  using ET = typename gather::Ell<R, REALV>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SiteTable st;  // not read: fused items are square
  st.nsites = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int2 td = tiles[t];
    const BatchItemDev& it = items[td.x];
    __syncthreads();  // the previous tile is done with the staged tables
    const ET* ell = gather::stage<ET>(smem_raw, it.v);
    const GGroup* sg = reinterpret_cast<const GGroup*>(smem_raw);
    const int64_t jend = min((int64_t)td.y + tile, it.v.m);
    for (int64_t J = td.y + threadIdx.x; J < jend; J += blockDim.x) {
      AT acc[1];
      gather::accumulate<R, REALV ? gather::kReal : gather::kComplex, true, false, 1>(
          it.v, st, sg, ell, (uint32_t)J, (const CT*)it.x, 1, 0, 1, acc);
      if constexpr (RK4) {  // k = alpha * acc, as combine<0> computes it, then the stage combination
        CT kv;
        if constexpr (std::is_same<R, gather::DFX>::value || sizeof(R) == 8) {
          gather::combine<0>(&kv, acc[0].total(), it.alpha, it.beta);
          rk4_stage_element<CT, double>(it, J, kv, stage);
        } else {
          const float2 a = make_float2((float)it.alpha.x, (float)it.alpha.y);
          gather::combine<0>(&kv, acc[0].total(), a, a);
          rk4_stage_element<CT, float>(it, J, kv, stage);
        }
      } else {
        CT* yp = (CT*)it.y + J;
        // beta == 0 overwrites y without reading it (NaN in y is ignored)
        const bool bz = it.beta.x == 0.0 && it.beta.y == 0.0;
        if constexpr (std::is_same<R, gather::DFX>::value || sizeof(R) == 8) {
          if (bz)
            gather::combine<0>(yp, acc[0].total(), it.alpha, it.beta);
          else
            gather::combine<2>(yp, acc[0].total(), it.alpha, it.beta);
        } else {
          const float2 a = make_float2((float)it.alpha.x, (float)it.alpha.y);
          const float2 b = make_float2((float)it.beta.x, (float)it.beta.y);
          if (bz)
            gather::combine<0>(yp, acc[0].total(), a, b);
          else
            gather::combine<2>(yp, acc[0].total(), a, b);
        }
      }
    }
  }
}

constexpr size_t kBatchSmemBudget = 96 * 1024;

size_t ell_size(int prec, bool real) {
  if (prec == QOB_C128) return real ? sizeof(EllD) : sizeof(EllZ);
  return real ? sizeof(EllF) : sizeof(EllC);
}

template <bool RK4>
const void* batch_kernel(int prec, bool real, bool ff) {
  if (ff)
    return real ? (const void*)k_gather_batch<gather::DFX, true, RK4> : (const void*)k_gather_batch<gather::DFX, false, RK4>;
  return prec == QOB_C128
             ? (real ? (const void*)k_gather_batch<double, true, RK4> : (const void*)k_gather_batch<double, false, RK4>)
             : (real ? (const void*)k_gather_batch<float, true, RK4> : (const void*)k_gather_batch<float, false, RK4>);
}

template <bool RK4>
void launch_batch(const BatchTables& T, const BatchItemDev* it, const int2* tl, cudaStream_t s, int stage) {
  const int grid = RK4 ? T.grid_rk4 : T.grid;
  if (T.ff) {
    if (T.real)
      k_gather_batch<gather::DFX, true, RK4><<<grid, 256, T.smem, s>>>(it, tl, T.ntiles, T.tile, stage);
    else
      k_gather_batch<gather::DFX, false, RK4><<<grid, 256, T.smem, s>>>(it, tl, T.ntiles, T.tile, stage);
  } else if (T.prec == QOB_C128) {
    if (T.real)
      k_gather_batch<double, true, RK4><<<grid, 256, T.smem, s>>>(it, tl, T.ntiles, T.tile, stage);
    else
      k_gather_batch<double, false, RK4><<<grid, 256, T.smem, s>>>(it, tl, T.ntiles, T.tile, stage);
  } else {
    if (T.real)
      k_gather_batch<float, true, RK4><<<grid, 256, T.smem, s>>>(it, tl, T.ntiles, T.tile, stage);
    else
      k_gather_batch<float, false, RK4><<<grid, 256, T.smem, s>>>(it, tl, T.ntiles, T.tile, stage);
  }
}

}  // namespace

bool plan_fusable(const Plan& P) {
  return P.kind == Plan::Kind::Sum && P.gather && P.dense.empty() && P.modek.empty() && P.subs.empty() &&
         P.gather->square && !P.gather->phased && P.gather->ngroups <= 256 && P.nterms_total > 0;
}

void build_tables(Context& ctx, BatchTables& T, const std::vector<BatchSpec>& specs, int prec, int tile) {
  prec = prec == QOB_C128X ? QOB_C128 : prec;  // ComplexF64 data; the items' plans say double-float
  std::vector<BatchItemDev> dev;
  std::vector<int2> tiles;
  T.prec = prec;
  T.real = true;
  T.ff = false;
  T.smem = 0;
  T.fused.assign(specs.size(), false);
  for (size_t i = 0; i < specs.size(); ++i) {
    T.fused[i] = plan_fusable(*specs[i].plan);
    if (T.fused[i]) T.real &= specs[i].plan->gather->real_vals;
    if (T.fused[i]) T.ff |= specs[i].plan->gather->ff;
  }
  for (size_t i = 0; i < specs.size(); ++i) {
    if (!T.fused[i]) continue;
    const GatherPlan& g = *specs[i].plan->gather;
    // real items in a batch with complex ones, and FP64 items beside
    // double-float ones, run apart
    if (g.real_vals != T.real || g.ff != T.ff) {
      T.fused[i] = false;
      continue;
    }
    BatchItemDev d;
    d.v = g.view();
    size_t smem = (size_t)d.v.ngroups * (sizeof(GGroup) + (d.v.fast ? sizeof(int4) : 0));
    const size_t eb = (size_t)d.v.ell_slots * ell_size(prec, T.real);
    d.v.ell_smem = (d.v.ell_slots > 0 && eb <= gather::kStageSlotsMax && smem + eb <= kBatchSmemBudget) ? 1 : 0;
    if (d.v.ell_smem) smem += eb;
    T.smem = std::max(T.smem, smem);
    d.x = specs[i].x;
    d.y = specs[i].y;
    d.alpha = make_double2(specs[i].alpha.re, specs[i].alpha.im);
    d.beta = make_double2(specs[i].beta.re, specs[i].beta.im);
    d.psi = specs[i].psi;
    d.acc = specs[i].acc;
    d.tmp_out = specs[i].tmp_out;
    d.dt = specs[i].dt;
    const int idx = (int)dev.size();
    dev.push_back(d);
    for (int64_t j0 = 0; j0 < g.m; j0 += tile) tiles.push_back(make_int2(idx, (int)j0));
  }
  T.nfused = (int)dev.size();
  T.ntiles = (int)tiles.size();
  T.tile = tile;
  if (!dev.empty()) {
    T.items.upload(dev.data(), dev.size() * sizeof(BatchItemDev));
    T.tiles.upload(tiles.data(), tiles.size() * sizeof(int2));
  }
  // persistent grids: as many 256-thread blocks as are resident at once
  auto resident = [&](const void* kern) {
    int n = 1;
    if (T.smem > 48 * 1024)
      QOB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T.smem));
    QOB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, 256, T.smem));
    return std::max(1, std::min(T.ntiles, ctx.num_sms * std::max(n, 1)));
  };
  T.grid = T.grid_rk4 = 1;
  if (T.ntiles > 0) {
    T.grid = resident(batch_kernel<false>(prec, T.real, T.ff));
    T.grid_rk4 = resident(batch_kernel<true>(prec, T.real, T.ff));
  }
}

bool all_fused(const BatchTables& T) {
  for (bool f : T.fused)
    if (!f) return false;
  return true;
}

void launch_tables(Context& ctx, const BatchTables& T, const std::vector<BatchSpec>& specs, cudaStream_t s,
                   int stage) {
  if (stage != 0 && !all_fused(T)) fail(QOB_ERR_STATE, "launch_tables: a fused RK4 stage with items outside the launch");
  if (T.ntiles > 0) {
    const BatchItemDev* it = (const BatchItemDev*)T.items.p;
    const int2* tl = (const int2*)T.tiles.p;
    if (stage != 0)
      launch_batch<true>(T, it, tl, s, stage);
    else
      launch_batch<false>(T, it, tl, s, stage);
    QOB_LAUNCHED();
  }
  for (size_t i = 0; i < specs.size(); ++i) {  // items outside the fused launch
    if (T.fused[i]) continue;
    Plan& P = *specs[i].plan;
    apply_plan(ctx, P, specs[i].alpha, specs[i].x, 1, P.n, specs[i].beta, specs[i].y, 1, P.m, 1, s, 0);
  }
}

}  // namespace qob

struct qob_batch {
  int dtype = QOB_C128;
  bool built = false;
  int tile = 256;
  std::vector<qob_op*> ops;
  std::vector<qob::BatchSpec> specs;
  qob::BatchTables tables;
};

namespace {

template <class F>
int bguard(qob_ctx* ctx, F&& f) {
  if (!ctx) return QOB_ERR_ARG;
  try {
    QOB_CUDA(cudaSetDevice(ctx->c.device));
    f();
    return QOB_OK;
  } catch (const qob::Error& e) {
    ctx->c.err = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    ctx->c.err = e.what();
    return QOB_ERR_ARG;
  }
}

// (Re)compile the items' plans and the device tables.
void rebuild(qob_ctx* ctx, qob_batch* b, int tile) {
  for (size_t i = 0; i < b->ops.size(); ++i) b->specs[i].plan = &qob::batch_plan(ctx->c, b->ops[i], b->dtype);
  qob::build_tables(ctx->c, b->tables, b->specs, b->dtype, tile);
  b->tile = tile;
  b->built = true;
}

bool plans_current(qob_batch* b) {
  for (size_t i = 0; i < b->ops.size(); ++i) {
    const auto& slot = b->ops[i]->plans[QOB_LEFT][b->dtype];
    if (!slot || slot.get() != b->specs[i].plan || !qob::plan_is_current(*slot)) return false;
  }
  return true;
}

}  // namespace

extern "C" {

int qob_batch_create(qob_ctx* ctx, int dtype, qob_batch** out) {
  return bguard(ctx, [&] {
    if (!out || (dtype != QOB_C128 && dtype != QOB_C64 && dtype != QOB_C128X))
      qob::fail(QOB_ERR_ARG, "qob_batch_create: bad arguments");
    auto* b = new qob_batch;
    b->dtype = dtype;
    *out = b;
  });
}

int qob_batch_add(qob_ctx* ctx, qob_batch* b, qob_op* op, double alpha_re, double alpha_im, const void* x, void* y,
                  double beta_re, double beta_im) {
  return bguard(ctx, [&] {
    if (!b || !op || !x || !y) qob::fail(QOB_ERR_ARG, "qob_batch_add: bad arguments");
    const size_t esz = b->dtype == QOB_C64 ? 8 : 16;
    const char* px = static_cast<const char*>(x);
    const char* py = static_cast<const char*>(y);
    if (px < py + op->node->m * esz && py < px + op->node->n * esz)
      qob::fail(QOB_ERR_ALIAS, "output matrix must not be aliased with input matrix");
    qob::BatchSpec s;
    s.plan = nullptr;
    s.x = x;
    s.y = y;
    s.alpha = {alpha_re, alpha_im};
    s.beta = {beta_re, beta_im};
    b->ops.push_back(op);
    b->specs.push_back(s);
    b->built = false;
  });
}

int qob_batch_run(qob_ctx* ctx, qob_batch* b, void* stream) {
  return bguard(ctx, [&] {
    if (!b) qob::fail(QOB_ERR_ARG, "null batch");
    if (!b->built || !plans_current(b)) rebuild(ctx, b, b->tile);
    qob::launch_tables(ctx->c, b->tables, b->specs, (cudaStream_t)stream);
  });
}

int qob_batch_tune(qob_ctx* ctx, qob_batch* b, double* times_ms, int* chosen) {
  return bguard(ctx, [&] {
    if (!b) qob::fail(QOB_ERR_ARG, "null batch");
    const int tiles[4] = {128, 256, 512, 1024};
    double best_t = 1e300;
    int best = 256;
    cudaEvent_t e0, e1;
    QOB_CUDA(cudaEventCreate(&e0));
    QOB_CUDA(cudaEventCreate(&e1));
    for (int k = 0; k < 4; ++k) {
      rebuild(ctx, b, tiles[k]);
      for (int i = 0; i < 2; ++i) qob::launch_tables(ctx->c, b->tables, b->specs, 0);
      QOB_CUDA(cudaEventRecord(e0, 0));
      for (int i = 0; i < 5; ++i) qob::launch_tables(ctx->c, b->tables, b->specs, 0);
      QOB_CUDA(cudaEventRecord(e1, 0));
      QOB_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      QOB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (times_ms) times_ms[k] = ms / 5.0;
      if (ms < best_t) {
        best_t = ms;
        best = tiles[k];
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    rebuild(ctx, b, best);
    if (chosen) *chosen = best;
  });
}

int qob_batch_set_tile(qob_ctx* ctx, qob_batch* b, int tile) {
  return bguard(ctx, [&] {
    if (!b) qob::fail(QOB_ERR_ARG, "null batch");
    if (tile != 128 && tile != 256 && tile != 512 && tile != 1024)
      qob::fail(QOB_ERR_ARG, "qob_batch_set_tile: tile must be 128, 256, 512 or 1024");
    rebuild(ctx, b, tile);
  });
}

int qob_batch_info(qob_ctx* ctx, qob_batch* b, int64_t* info) {
  return bguard(ctx, [&] {
    if (!b || !info) qob::fail(QOB_ERR_ARG, "qob_batch_info: bad arguments");
    if (!b->built || !plans_current(b)) rebuild(ctx, b, b->tile);
    info[0] = (int64_t)b->specs.size();
    info[1] = b->tables.nfused;
    info[2] = b->tables.ntiles;
    info[3] = b->tables.tile;
    info[4] = b->tables.grid;
  });
}

int qob_batch_free(qob_ctx* ctx, qob_batch* b) {
  return bguard(ctx, [&] { delete b; });
}

}  // extern "C"

// One-shot form of the batch API: n applications y_i = alpha_i op_i x_i + beta_i y_i
// (kets, device memory) in one fused launch where the plans allow.  The batch's
// tables are built and freed inside the call; synchronous on `stream`.
extern "C" int qob_apply_batched(qob_ctx* ctx, int dtype, int n, qob_op* const* ops, const void* const* xs,
                                 void* const* ys, const double* alphas, const double* betas, void* stream) {
  if (!ctx) return QOB_ERR_ARG;
  if (n < 0 || (n > 0 && (!ops || !xs || !ys || !alphas || !betas))) {
    ctx->c.err = "qob_apply_batched: bad arguments";
    return QOB_ERR_ARG;
  }
  qob_batch* b = nullptr;
  int rc = qob_batch_create(ctx, dtype, &b);
  for (int i = 0; rc == QOB_OK && i < n; ++i)
    rc = qob_batch_add(ctx, b, ops[i], alphas[2 * i], alphas[2 * i + 1], xs[i], ys[i], betas[2 * i], betas[2 * i + 1]);
  if (rc == QOB_OK && n > 0) rc = qob_batch_run(ctx, b, stream);
  if (rc == QOB_OK) {
    const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) {
      ctx->c.err = cudaGetErrorString(e);
      rc = QOB_ERR_CUDA;
    }
  }
  if (b) qob_batch_free(ctx, b);
  return rc;
}
