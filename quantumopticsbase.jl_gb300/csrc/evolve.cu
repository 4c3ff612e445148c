// evolve.cu -- fixed-step RK4 time evolution on the device and the
// continuous-batching request server built on it.
//
// Time evolution is the reference's main consumer of mul!: an ODE solver
// calls mul!(dpsi, H, psi, -im, 0) on every right-hand-side evaluation
// (QuantumOptics.jl's timeevolution on top of src/operators_lazysum.jl:189).
// One RK4 step of dpsi/dt = -i H psi is four applications of H plus the
// stage combinations:
//   k1 = -iH psi,           acc = k1,        tmp = psi + dt/2 k1
//   k2 = -iH tmp,           acc += 2 k2,     tmp = psi + dt/2 k2
//   k3 = -iH tmp,           acc += 2 k3,     tmp = psi + dt k3
//   k4 = -iH tmp,           psi += dt/6 (acc + k4)
// Every application of all states in flight runs as one launch (the batch
// tables of batch.cu).  When every state's operator is in the fused launch,
// each application does its stage combination in the same kernel (k stays in
// registers: four launches per step, and the k buffer serves as the second
// tmp buffer the stages then alternate with); otherwise the stage
// combinations run as launches of their own (eight per step).  The optional renormalisation
// computes |psi| in FP64 with a per-request reduction of fixed order, so a
// request's result does not depend on which other requests share its launches.
//
// The server (qob_server_*) keeps states and operators resident on the
// device, admits queued requests when a slot and device memory (its own
// budget and cudaMemGetInfo) allow, advances every active request by RK4
// steps -- replayed from a CUDA graph of one step of the current ensemble,
// up to 16 per iteration on the worker thread (4 while requests wait, never
// past a request's last step), one per qob_server_step -- and retires finished
// ones with their latency record.  Requests that arrive while others run join
// at the next iteration.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "batch.h"

namespace qob {

struct StageItemDev {
  void* psi;
  void* k;
  void* acc;
  void* tmp;
  int64_t n;
  double dt;
  int32_t part0;  // first FP64 partial of this item (renormalisation)
  int32_t nparts;
};

namespace {

constexpr int kStageTile = 1024;

// Stage combination over all items, tile by tile (element-wise, so the
// result of an element does not depend on the tiling).
template <typename CT, typename R>
__global__ void __launch_bounds__(256) k_rk4_stage(const StageItemDev* __restrict__ items,
                                                   const int2* __restrict__ tiles, int ntiles, int mode) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int2 td = tiles[t];
    const StageItemDev& it = items[td.x];
    const int64_t end = min((int64_t)td.y + kStageTile, it.n);
    CT* psi = (CT*)it.psi;
    const CT* k = (const CT*)it.k;
    CT* acc = (CT*)it.acc;
    CT* tmp = (CT*)it.tmp;
    const R dt = (R)it.dt;
    for (int64_t j = td.y + threadIdx.x; j < end; j += blockDim.x) {
      const CT kv = k[j];
      if (mode == 1) {
        const CT p = psi[j];
        const R c = dt * (R)0.5;
        acc[j] = kv;
        CT o;
        o.x = p.x + c * kv.x;
        o.y = p.y + c * kv.y;
        tmp[j] = o;
      } else if (mode == 2 || mode == 3) {
        const CT p = psi[j];
        const R c = mode == 2 ? dt * (R)0.5 : dt;
        CT a = acc[j];
        a.x += (R)2 * kv.x;
        a.y += (R)2 * kv.y;
        acc[j] = a;
        CT o;
        o.x = p.x + c * kv.x;
        o.y = p.y + c * kv.y;
        tmp[j] = o;
      } else {
        const CT a = acc[j];
        CT p = psi[j];
        const R c = dt / (R)6;
        p.x += c * (a.x + kv.x);
        p.y += c * (a.y + kv.y);
        psi[j] = p;
      }
    }
  }
}

// |psi|^2 partials in FP64: one partial per (item, tile), tree order fixed.
template <typename CT>
__global__ void __launch_bounds__(256) k_norm_partial(const StageItemDev* __restrict__ items,
                                                      const int2* __restrict__ tiles, int ntiles,
                                                      double* __restrict__ part) {
  __shared__ double s[256];
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int2 td = tiles[t];
    const StageItemDev& it = items[td.x];
    const int64_t end = min((int64_t)td.y + kStageTile, it.n);
    const CT* psi = (const CT*)it.psi;
    double a = 0.0;
    for (int64_t j = td.y + threadIdx.x; j < end; j += blockDim.x) {
      const CT p = psi[j];
      a = fma((double)p.x, (double)p.x, a);
      a = fma((double)p.y, (double)p.y, a);
    }
    __syncthreads();
    s[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[it.part0 + (td.y / kStageTile)] = s[0];
  }
}

// psi /= |psi| per item; the item's partials are added in index order.
template <typename CT, typename R>
__global__ void __launch_bounds__(256) k_renormalise(const StageItemDev* __restrict__ items,
                                                     const int2* __restrict__ tiles, int ntiles,
                                                     const double* __restrict__ part) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int2 td = tiles[t];
    const StageItemDev& it = items[td.x];
    double nn = 0.0;
    for (int q = 0; q < it.nparts; ++q) nn += part[it.part0 + q];
    const R inv = nn > 0.0 ? (R)(1.0 / sqrt(nn)) : (R)1;
    const int64_t end = min((int64_t)td.y + kStageTile, it.n);
    CT* psi = (CT*)it.psi;
    for (int64_t j = td.y + threadIdx.x; j < end; j += blockDim.x) {
      CT p = psi[j];
      p.x *= inv;
      p.y *= inv;
      psi[j] = p;
    }
  }
}

}  // namespace

// Device tables of an ensemble of states being evolved together.
struct Ensemble {
  int prec = QOB_C128;
  std::vector<BatchSpec> from_psi, from_tmp;  // k = -i H psi  /  k = -i H tmp
  BatchTables g_psi, g_tmp;
  // fused steps: stage s applies H to its input and combines in place, the
  // stages' inputs and outputs alternating psi -> tmp -> k -> tmp -> psi
  bool fused = false;
  std::vector<BatchSpec> stage_specs[4];
  BatchTables g_stage[4];
  DeviceBuf stage_items, stage_tiles, partials;
  int stage_ntiles = 0;
  int grid = 1;
  bool renormalise = false;
};

struct EvolveState {
  Plan* plan;
  void* psi;
  void* k;
  void* acc;
  void* tmp;
  int64_t n;
  double dt;
};

void ensemble_build(Context& ctx, Ensemble& E, const std::vector<EvolveState>& states, int prec) {
  // QOB_C128X: ComplexF64 states (FP64 stage kernels), operators in double-float
  prec = prec == QOB_C128X ? QOB_C128 : prec;
  E.prec = prec;
  E.from_psi.clear();
  E.from_tmp.clear();
  std::vector<StageItemDev> items;
  std::vector<int2> tiles;
  int32_t nparts = 0;
  for (size_t i = 0; i < states.size(); ++i) {
    const EvolveState& s = states[i];
    E.from_psi.push_back({s.plan, s.psi, s.k, {0.0, -1.0}, {0.0, 0.0}});
    E.from_tmp.push_back({s.plan, s.tmp, s.k, {0.0, -1.0}, {0.0, 0.0}});
    StageItemDev d;
    d.psi = s.psi;
    d.k = s.k;
    d.acc = s.acc;
    d.tmp = s.tmp;
    d.n = s.n;
    d.dt = s.dt;
    d.part0 = nparts;
    d.nparts = (int32_t)((s.n + kStageTile - 1) / kStageTile);
    nparts += d.nparts;
    for (int64_t j = 0; j < s.n; j += kStageTile) tiles.push_back(make_int2((int)i, (int)j));
    items.push_back(d);
  }
  // fused stages when every operator is in the fused launch
  for (int st = 0; st < 4; ++st) E.stage_specs[st].clear();
  for (const EvolveState& s : states) {
    const double dt = s.dt;
    E.stage_specs[0].push_back({s.plan, s.psi, s.k, {0.0, -1.0}, {0.0, 0.0}, s.psi, s.acc, s.tmp, dt});
    E.stage_specs[1].push_back({s.plan, s.tmp, s.k, {0.0, -1.0}, {0.0, 0.0}, s.psi, s.acc, s.k, dt});
    E.stage_specs[2].push_back({s.plan, s.k, s.tmp, {0.0, -1.0}, {0.0, 0.0}, s.psi, s.acc, s.tmp, dt});
    E.stage_specs[3].push_back({s.plan, s.tmp, s.k, {0.0, -1.0}, {0.0, 0.0}, s.psi, s.acc, nullptr, dt});
  }
  E.fused = false;
  if (!states.empty()) {
    build_tables(ctx, E.g_stage[0], E.stage_specs[0], prec, 256);
    E.fused = all_fused(E.g_stage[0]);
  }
  if (E.fused) {
    for (int st = 1; st < 4; ++st) build_tables(ctx, E.g_stage[st], E.stage_specs[st], prec, 256);
  } else {
    build_tables(ctx, E.g_psi, E.from_psi, prec, 256);
    build_tables(ctx, E.g_tmp, E.from_tmp, prec, 256);
  }
  E.stage_ntiles = (int)tiles.size();
  if (!items.empty()) {
    E.stage_items.upload(items.data(), items.size() * sizeof(StageItemDev));
    E.stage_tiles.upload(tiles.data(), tiles.size() * sizeof(int2));
    if (E.partials.bytes < (size_t)nparts * sizeof(double)) E.partials.alloc((size_t)std::max(nparts, 1) * sizeof(double));
  }
  E.grid = std::max(1, std::min(E.stage_ntiles, ctx.num_sms * 8));
}

// One RK4 step of every state; before_stage(mode), when given, runs before the
// application of each stage (time-dependent operators refresh their values there).
void ensemble_step(Context& ctx, Ensemble& E, cudaStream_t s,
                   const std::function<void(int)>* before_stage = nullptr) {
  if (E.stage_ntiles == 0) return;
  const StageItemDev* it = (const StageItemDev*)E.stage_items.p;
  const int2* tl = (const int2*)E.stage_tiles.p;
  for (int mode = 1; mode <= 4; ++mode) {
    if (before_stage) (*before_stage)(mode);
    if (E.fused) {
      launch_tables(ctx, E.g_stage[mode - 1], E.stage_specs[mode - 1], s, mode);
      continue;
    }
    launch_tables(ctx, mode == 1 ? E.g_psi : E.g_tmp, mode == 1 ? E.from_psi : E.from_tmp, s);
    if (E.prec == QOB_C128)
      k_rk4_stage<double2, double><<<E.grid, 256, 0, s>>>(it, tl, E.stage_ntiles, mode);
    else
      k_rk4_stage<float2, float><<<E.grid, 256, 0, s>>>(it, tl, E.stage_ntiles, mode);
    QOB_LAUNCHED();
  }
  if (E.renormalise) {
    double* part = (double*)E.partials.p;
    if (E.prec == QOB_C128) {
      k_norm_partial<double2><<<E.grid, 256, 0, s>>>(it, tl, E.stage_ntiles, part);
      QOB_LAUNCHED();
      k_renormalise<double2, double><<<E.grid, 256, 0, s>>>(it, tl, E.stage_ntiles, part);
    } else {
      k_norm_partial<float2><<<E.grid, 256, 0, s>>>(it, tl, E.stage_ntiles, part);
      QOB_LAUNCHED();
      k_renormalise<float2, float><<<E.grid, 256, 0, s>>>(it, tl, E.stage_ntiles, part);
    }
    QOB_LAUNCHED();
  }
}

}  // namespace qob

// ---------------------------------------------------------------------------
// server
// ---------------------------------------------------------------------------
namespace {

using Clock = std::chrono::steady_clock;
double now_s() { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); }

struct Request {
  int64_t id = 0;
  qob_op* op = nullptr;
  int64_t n = 0;
  int nsteps = 0;
  int step = 0;
  double dt = 0.0;
  int status = 0;  // 0 queued, 1 active, 2 done, negative: error code
  bool cancel = false;    // cancelled while active: retired at the next engine iteration
  int alloc_failures = 0;  // refused allocations while nothing else was active
  std::vector<char> psi0, result;
  double t_submit = 0, t_admit = 0, t_done = 0;
  void* dev = nullptr;
  size_t bytes = 0;
  qob::Plan* plan = nullptr;
  // time-dependent requests: a plan of their own (its values follow the
  // request's coefficient rows), the rows on the device, a device step counter
  bool td = false;
  std::vector<double> rows_host;  // (2*nsteps+1) x nf interleaved complex
  int64_t nf = 0;
  std::unique_ptr<qob::Plan> own_plan;
  qob::DeviceBuf rows, step_ctr;
};

}  // namespace

struct qob_server {
  qob_ctx* ctx = nullptr;
  int dtype = QOB_C128;
  size_t budget = 0;
  int max_active = 64;
  bool renormalise = false;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Request*> queue;
  std::vector<Request*> active;
  std::unordered_map<int64_t, std::unique_ptr<Request>> all;
  int64_t next_id = 1;
  size_t mem_used = 0;
  cudaStream_t stream = nullptr;
  qob::Ensemble ens;
  bool dirty = true;
  // one RK4 step of the current ensemble as a CUDA graph: recorded on the
  // second iteration after a rebuild (the first sizes every buffer), replayed after
  int graph_state = 0;  // 0: next step runs directly, 1: next step is recorded, 2: replay
  cudaGraphExec_t graph = nullptr;
  std::vector<Request*> td_members;  // time-dependent requests of the current ensemble
  std::thread worker;
  bool stop = false;
  bool running = false;
  int64_t steps_run = 0, iterations = 0, rejected = 0, completed = 0, cancelled = 0, alloc_refusals = 0;
  int last_error = 0;
  std::string last_msg;
  // host-side allocation hook, asked before every admission's device allocation
  int (*alloc_hook)(void* user, size_t bytes) = nullptr;
  void* alloc_user = nullptr;
};

namespace {

size_t elem_bytes(int dtype) { return dtype == QOB_C64 ? 8 : 16; }

// Consecutive refused allocations, with no other request active, after which a
// queued request is rejected (nothing in this server will free memory for it).
constexpr int kMaxAllocFailures = 3;

// A request leaves the server with a final status (lock held): its device
// memory is released and waiters are woken.
void retire(qob_server* S, Request* r, int status) {
  if (r->dev) {
    cudaFreeAsync(r->dev, S->stream);  // best effort: after a failed iteration the stream may carry the error
    cudaGetLastError();
    S->mem_used -= r->bytes;
    r->dev = nullptr;
  }
  r->own_plan.reset();
  r->rows = qob::DeviceBuf();
  r->step_ctr = qob::DeviceBuf();
  r->rows_host.clear();
  r->status = status;
  r->t_done = now_s();
  S->cv.notify_all();
}

// Admit queued requests while a slot and memory are free (lock held).  An
// allocation that the hook refuses or that the device cannot serve leaves the
// request queued while other requests run (their memory comes back when they
// finish); with nothing active it is retried at the next iterations and the
// request is rejected with -QOB_ERR_OOM after kMaxAllocFailures refusals.
void admit(qob_server* S) {
  while (!S->queue.empty() && (int)S->active.size() < S->max_active) {
    Request* r = S->queue.front();
    const size_t need = 4 * (size_t)r->n * elem_bytes(S->dtype);
    size_t free_b = 0, total_b = 0;
    QOB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (S->mem_used + need > S->budget || need + (size_t(256) << 20) > free_b) break;  // wait for memory
    cudaError_t ae = cudaErrorMemoryAllocation;
    if (!S->alloc_hook || S->alloc_hook(S->alloc_user, need) == 0) ae = cudaMallocAsync(&r->dev, need, S->stream);
    if (ae != cudaSuccess) {
      if (ae != cudaErrorMemoryAllocation) QOB_CUDA(ae);
      cudaGetLastError();
      r->dev = nullptr;
      S->alloc_refusals++;
      if (S->active.empty() && ++r->alloc_failures >= kMaxAllocFailures) {
        S->queue.pop_front();
        S->rejected++;
        retire(S, r, -QOB_ERR_OOM);
        continue;
      }
      break;  // stays queued
    }
    r->alloc_failures = 0;
    r->bytes = need;
    S->mem_used += need;
    QOB_CUDA(cudaMemcpyAsync(r->dev, r->psi0.data(), r->psi0.size(), cudaMemcpyHostToDevice, S->stream));
    if (r->td) {
      try {
        qob::Context& c = S->ctx->c;
        r->own_plan = qob::compile_plan(c, r->op->node, QOB_LEFT, S->dtype);
        qob::Plan& P = *r->own_plan;
        if (P.kind != qob::Plan::Kind::Sum || !P.dense.empty() || !P.modek.empty() || !P.subs.empty() || !P.gather)
          qob::fail(QOB_ERR_UNSUPPORTED, "time-dependent requests need every term in the fused gather");
        qob::prepare_factor_rows(P, *r->op->node, r->rows_host.data(), 2 * (int64_t)r->nsteps + 1);
        r->rows.upload(r->rows_host.data(), std::max<size_t>(r->rows_host.size(), 2) * sizeof(double));
        const long long zero = 0;
        r->step_ctr.upload(&zero, sizeof(zero));
        // the values of row 0 (stage 1 of the first step)
        qob::device_refresh(*P.gather, (const double2*)r->rows.p, S->stream, (const long long*)r->step_ctr.p, 0,
                            (long long)r->nf);
        r->plan = &P;
      } catch (const qob::Error& e) {  // this request fails, the server goes on
        QOB_CUDA(cudaFreeAsync(r->dev, S->stream));
        r->dev = nullptr;
        S->mem_used -= need;
        r->own_plan.reset();
        r->status = -e.code;
        r->t_done = now_s();
        S->rejected++;
        S->queue.pop_front();
        S->cv.notify_all();
        continue;
      }
    } else {
      r->plan = &qob::batch_plan(S->ctx->c, r->op, S->dtype);
    }
    r->status = 1;
    r->t_admit = now_s();
    S->queue.pop_front();
    S->active.push_back(r);
    S->dirty = true;
  }
}

void drop_graph(qob_server* S) {
  if (S->graph) cudaGraphExecDestroy(S->graph);
  S->graph = nullptr;
  S->graph_state = 0;
}

// The launches of one RK4 step: time-dependent members re-evaluate their values
// before stages 2 and 4 (rows 2s+1, 2s+2 by their device step counters) and
// advance the counters at the end.
void step_launches(qob_server* S) {
  qob::Context& ctx = S->ctx->c;
  if (S->td_members.empty()) {
    qob::ensemble_step(ctx, S->ens, S->stream);
    return;
  }
  std::function<void(int)> hook = [&](int mode) {
    if (mode != 2 && mode != 4) return;
    for (Request* r : S->td_members)
      qob::device_refresh(*r->own_plan->gather, (const double2*)r->rows.p, S->stream,
                          (const long long*)r->step_ctr.p, mode == 2 ? 1 : 2, (long long)r->nf);
  };
  qob::ensemble_step(ctx, S->ens, S->stream, &hook);
  for (Request* r : S->td_members) qob::launch_td_advance(static_cast<long long*>(r->step_ctr.p), S->stream);
}

// One RK4 step of the ensemble: directly, recorded into a graph, or replayed.
void run_step(qob_server* S) {
  if (S->graph_state == 2) {
    QOB_CUDA(cudaGraphLaunch(S->graph, S->stream));
    return;
  }
  if (S->graph_state == 0) {
    step_launches(S);
    S->graph_state = 1;
    return;
  }
  cudaGraph_t g = nullptr;
  QOB_CUDA(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
  try {
    step_launches(S);
  } catch (...) {
    cudaStreamEndCapture(S->stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  QOB_CUDA(cudaStreamEndCapture(S->stream, &g));
  const cudaError_t e = cudaGraphInstantiate(&S->graph, g, 0);
  cudaGraphDestroy(g);
  QOB_CUDA(e);
  S->graph_state = 2;
  QOB_CUDA(cudaGraphLaunch(S->graph, S->stream));
}

// One engine iteration: admit, up to max_steps RK4 steps of every active
// request (never past a request's last step), retire.  Returns the number of
// active requests after the iteration.
int iterate(qob_server* S, int max_steps) {
  std::vector<Request*> act;
  bool waiting = false;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    // requests cancelled while active leave between iterations
    bool any = false;
    for (Request* r : S->active) any |= r->cancel;
    if (any) {
      QOB_CUDA(cudaStreamSynchronize(S->stream));
      drop_graph(S);
      std::vector<Request*> keep;
      for (Request* r : S->active) {
        if (r->cancel) {
          S->cancelled++;
          retire(S, r, -QOB_ERR_CANCELLED);
        } else {
          keep.push_back(r);
        }
      }
      S->active.swap(keep);
      S->dirty = true;
    }
    admit(S);
    act = S->active;
    waiting = !S->queue.empty();
  }
  if (act.empty()) return 0;
  qob::Context& ctx = S->ctx->c;
  if (S->dirty) {
    std::vector<qob::EvolveState> states;
    for (Request* r : act) {
      const size_t sz = (size_t)r->n * elem_bytes(S->dtype);
      char* base = static_cast<char*>(r->dev);
      states.push_back({r->plan, base, base + sz, base + 2 * sz, base + 3 * sz, r->n, r->dt});
    }
    S->ens.renormalise = S->renormalise;
    drop_graph(S);
    S->td_members.clear();
    for (Request* r : act)
      if (r->td) S->td_members.push_back(r);
    qob::ensemble_build(ctx, S->ens, states, S->dtype);
    S->dirty = false;
  }
  int k = waiting ? std::min(max_steps, 4) : max_steps;  // queued requests join soon
  for (Request* r : act) k = std::min(k, r->nsteps - r->step);
  k = std::max(k, 1);
  for (int i = 0; i < k; ++i) run_step(S);
  QOB_CUDA(cudaStreamSynchronize(S->stream));
  S->iterations++;
  std::vector<Request*> finished;
  for (Request* r : act) {
    r->step += k;
    S->steps_run += k;
    if (r->step >= r->nsteps) finished.push_back(r);
  }
  for (Request* r : finished) {
    r->result.resize(r->psi0.size());
    QOB_CUDA(cudaMemcpyAsync(r->result.data(), r->dev, r->result.size(), cudaMemcpyDeviceToHost, S->stream));
  }
  if (!finished.empty()) {
    QOB_CUDA(cudaStreamSynchronize(S->stream));
    std::lock_guard<std::mutex> lk(S->mu);
    const double t = now_s();
    for (Request* r : finished) {
      QOB_CUDA(cudaFreeAsync(r->dev, S->stream));
      S->mem_used -= r->bytes;
      r->dev = nullptr;
      r->own_plan.reset();  // the step graph that used it is dropped before the next step
      r->rows = qob::DeviceBuf();
      r->step_ctr = qob::DeviceBuf();
      r->rows_host.clear();
      r->status = 2;
      r->t_done = t;
      S->completed++;
      S->active.erase(std::find(S->active.begin(), S->active.end(), r));
    }
    S->dirty = true;
    S->cv.notify_all();
  }
  std::lock_guard<std::mutex> lk(S->mu);
  return (int)S->active.size();
}

void worker_loop(qob_server* S) {
  cudaSetDevice(S->ctx->c.device);
  while (true) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv.wait_for(lk, std::chrono::milliseconds(2),
                     [&] { return S->stop || !S->queue.empty() || !S->active.empty(); });
      if (S->stop) break;
      if (S->queue.empty() && S->active.empty()) continue;
    }
    int code = 0;
    std::string msg;
    try {
      iterate(S, 16);
    } catch (const qob::Error& e) {
      code = e.code;
      msg = e.msg;
    } catch (const std::exception& e) {
      code = QOB_ERR_ARG;
      msg = e.what();
    }
    if (code) {
      std::lock_guard<std::mutex> lk(S->mu);
      S->last_error = code;
      S->last_msg = msg;
      // fail the requests in flight and give their memory back; the server
      // keeps serving new ones
      drop_graph(S);
      for (Request* r : S->active) retire(S, r, -code);
      S->active.clear();
      S->dirty = true;
    }
  }
}

template <class F>
int sguard(qob_server* S, F&& f) {
  if (!S || !S->ctx) return QOB_ERR_ARG;
  try {
    QOB_CUDA(cudaSetDevice(S->ctx->c.device));
    f();
    return QOB_OK;
  } catch (const qob::Error& e) {
    S->ctx->c.err = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    S->ctx->c.err = e.what();
    return QOB_ERR_ARG;
  }
}

}  // namespace

extern "C" {

int qob_server_create(qob_ctx* ctx, int dtype, size_t mem_budget, int max_active, int renormalise,
                      qob_server** out) {
  if (!ctx || !out || (dtype != QOB_C128 && dtype != QOB_C64 && dtype != QOB_C128X) || max_active < 1)
    return QOB_ERR_ARG;
  auto* S = new qob_server;
  S->ctx = ctx;
  S->dtype = dtype;
  S->budget = mem_budget;
  S->max_active = max_active;
  S->renormalise = renormalise != 0;
  int rc = sguard(S, [&] { QOB_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking)); });
  if (rc) {
    delete S;
    return rc;
  }
  *out = S;
  return QOB_OK;
}

int qob_server_submit(qob_server* S, qob_op* H, const void* psi0, int64_t n, int nsteps, double dt,
                      int64_t* id) {
  return sguard(S, [&] {
    if (!H || !psi0 || n < 1 || nsteps < 0 || !id) qob::fail(QOB_ERR_ARG, "qob_server_submit: bad arguments");
    if (H->node->m != n || H->node->n != n) qob::fail(QOB_ERR_DIM, "Hamiltonian and state dimensions differ");
    auto r = std::make_unique<Request>();
    r->op = H;
    r->n = n;
    r->nsteps = nsteps;
    r->dt = dt;
    const size_t bytes = (size_t)n * elem_bytes(S->dtype);
    r->psi0.assign(static_cast<const char*>(psi0), static_cast<const char*>(psi0) + bytes);
    r->t_submit = now_s();
    std::lock_guard<std::mutex> lk(S->mu);
    r->id = S->next_id++;
    *id = r->id;
    if (4 * bytes > S->budget) {  // can never be admitted
      r->status = -QOB_ERR_OOM;
      r->t_done = r->t_submit;
      S->rejected++;
    } else {
      S->queue.push_back(r.get());
    }
    S->all[r->id] = std::move(r);
    S->cv.notify_all();
  });
}

int qob_server_submit_td(qob_server* S, qob_op* H, const void* psi0, int64_t n, int nsteps, double dt,
                         const double* factors, int64_t nrows, int64_t* id) {
  return sguard(S, [&] {
    if (!H || !psi0 || n < 1 || nsteps < 0 || !id) qob::fail(QOB_ERR_ARG, "qob_server_submit_td: bad arguments");
    if (H->node->kind != qob::Kind::LazySum) qob::fail(QOB_ERR_ARG, "time-dependent requests need a LazySum");
    if (nrows != 2 * (int64_t)nsteps + 1) qob::fail(QOB_ERR_ARG, "qob_server_submit_td: nrows must be 2*nsteps+1");
    const int64_t nf = (int64_t)H->node->factors.size();
    if (nf > 0 && !factors) qob::fail(QOB_ERR_ARG, "qob_server_submit_td: null factor table");
    if (H->node->m != n || H->node->n != n) qob::fail(QOB_ERR_DIM, "Hamiltonian and state dimensions differ");
    auto r = std::make_unique<Request>();
    r->op = H;
    r->n = n;
    r->nsteps = nsteps;
    r->dt = dt;
    r->td = true;
    r->nf = nf;
    if (nf > 0) r->rows_host.assign(factors, factors + 2 * nrows * nf);
    const size_t bytes = (size_t)n * elem_bytes(S->dtype);
    r->psi0.assign(static_cast<const char*>(psi0), static_cast<const char*>(psi0) + bytes);
    r->t_submit = now_s();
    std::lock_guard<std::mutex> lk(S->mu);
    r->id = S->next_id++;
    *id = r->id;
    if (4 * bytes > S->budget) {
      r->status = -QOB_ERR_OOM;
      r->t_done = r->t_submit;
      S->rejected++;
    } else {
      S->queue.push_back(r.get());
    }
    S->all[r->id] = std::move(r);
    S->cv.notify_all();
  });
}

int qob_server_step(qob_server* S, int* nactive) {
  return sguard(S, [&] {
    if (S->running) qob::fail(QOB_ERR_STATE, "the server's worker thread is running");
    const int a = iterate(S, 1);
    if (nactive) *nactive = a;
  });
}

int qob_server_start(qob_server* S) {
  return sguard(S, [&] {
    if (S->running) return;
    S->stop = false;
    S->running = true;
    S->worker = std::thread(worker_loop, S);
  });
}

int qob_server_stop(qob_server* S) {
  return sguard(S, [&] {
    if (!S->running) return;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->stop = true;
      S->cv.notify_all();
    }
    S->worker.join();
    S->running = false;
  });
}

int qob_server_poll(qob_server* S, int64_t id, void* psi_out, double* times, int* status) {
  return sguard(S, [&] {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) qob::fail(QOB_ERR_ARG, "unknown request id");
    Request* r = it->second.get();
    if (status) *status = r->status;
    if (times) {
      times[0] = r->t_submit;
      times[1] = r->t_admit;
      times[2] = r->t_done;
    }
    if (r->status == 2 && psi_out) std::memcpy(psi_out, r->result.data(), r->result.size());
  });
}

int qob_server_wait(qob_server* S, int64_t id, double timeout_s, int* status) {
  return sguard(S, [&] {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) qob::fail(QOB_ERR_ARG, "unknown request id");
    Request* r = it->second.get();
    const bool ok = S->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return r->status >= 2 || r->status < 0; });
    if (status) *status = r->status;
    if (!ok) qob::fail(QOB_ERR_TIMEOUT, "request did not finish in time");
  });
}

int qob_server_stats(qob_server* S, int64_t* out) {
  return sguard(S, [&] {
    std::lock_guard<std::mutex> lk(S->mu);
    out[0] = (int64_t)S->queue.size();
    out[1] = (int64_t)S->active.size();
    out[2] = S->completed;
    out[3] = S->rejected;
    out[4] = S->steps_run;
    out[5] = S->iterations;
    out[6] = (int64_t)S->mem_used;
    out[7] = S->last_error;
  });
}

int qob_server_stats2(qob_server* S, int64_t* out) {
  return sguard(S, [&] {
    if (!out) qob::fail(QOB_ERR_ARG, "qob_server_stats2: null output");
    std::lock_guard<std::mutex> lk(S->mu);
    out[0] = S->cancelled;
    out[1] = S->alloc_refusals;
  });
}

int qob_server_cancel(qob_server* S, int64_t id) {
  return sguard(S, [&] {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) qob::fail(QOB_ERR_ARG, "unknown request id");
    Request* r = it->second.get();
    if (r->status == 0) {  // queued: leaves at once
      S->queue.erase(std::find(S->queue.begin(), S->queue.end(), r));
      S->cancelled++;
      retire(S, r, -QOB_ERR_CANCELLED);
    } else if (r->status == 1) {  // running: leaves before the engine's next iteration
      r->cancel = true;
      S->cv.notify_all();
    } else {
      qob::fail(QOB_ERR_STATE, "the request has already finished");
    }
  });
}

int qob_server_set_alloc_hook(qob_server* S, int (*hook)(void* user, size_t bytes), void* user) {
  return sguard(S, [&] {
    std::lock_guard<std::mutex> lk(S->mu);
    S->alloc_hook = hook;
    S->alloc_user = user;
  });
}

int qob_server_destroy(qob_server* S) {
  if (!S) return QOB_ERR_ARG;
  qob_server_stop(S);
  cudaSetDevice(S->ctx->c.device);
  for (Request* r : S->active)
    if (r->dev) cudaFreeAsync(r->dev, S->stream);
  drop_graph(S);
  if (S->stream) {
    cudaStreamSynchronize(S->stream);
    cudaStreamDestroy(S->stream);
  }
  delete S;
  return QOB_OK;
}

// Single-state RK4: nsteps steps of dpsi/dt = -i H psi on device state psi.
int qob_rk4(qob_ctx* ctx, qob_op* H, int dtype, void* psi, int64_t n, double dt, int nsteps, int renormalise,
            void* stream) {
  if (!ctx) return QOB_ERR_ARG;
  try {
    QOB_CUDA(cudaSetDevice(ctx->c.device));
    if (!H || !psi || n < 1 || (dtype != QOB_C128 && dtype != QOB_C64 && dtype != QOB_C128X))
      qob::fail(QOB_ERR_ARG, "qob_rk4: bad arguments");
    if (H->node->m != n || H->node->n != n) qob::fail(QOB_ERR_DIM, "Hamiltonian and state dimensions differ");
    const size_t sz = (size_t)n * (dtype == QOB_C64 ? 8 : 16);
    char* w = static_cast<char*>(ctx->c.ws.get(20, 3 * sz));
    qob::Plan& P = qob::batch_plan(ctx->c, H, dtype);
    qob::Ensemble E;
    E.renormalise = renormalise != 0;
    qob::ensemble_build(ctx->c, E, {qob::EvolveState{&P, psi, w, w + sz, w + 2 * sz, n, dt}}, dtype);
    cudaStream_t st = (cudaStream_t)stream;
    // the first step runs directly (it sizes every buffer); the rest replay a
    // CUDA graph of one step on the context's own stream (the call is
    // synchronous, so the caller's stream is drained first)
    int s = 0;
    if (nsteps > 0) {
      qob::ensemble_step(ctx->c, E, st);
      s = 1;
    }
    if (nsteps - s >= 4) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      QOB_CUDA(cudaStreamIsCapturing(st, &cs));
      if (cs == cudaStreamCaptureStatusNone) {
        QOB_CUDA(cudaStreamSynchronize(st));
        if (!ctx->c.copy_stream[1]) QOB_CUDA(cudaStreamCreateWithFlags(&ctx->c.copy_stream[1], cudaStreamNonBlocking));
        st = ctx->c.copy_stream[1];
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        QOB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
          qob::ensemble_step(ctx->c, E, st);
        } catch (...) {
          cudaStreamEndCapture(st, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        QOB_CUDA(cudaStreamEndCapture(st, &g));
        const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        QOB_CUDA(e);
        for (; s < nsteps; ++s) {
          const cudaError_t le = cudaGraphLaunch(ge, st);
          if (le != cudaSuccess) {
            cudaGraphExecDestroy(ge);
            QOB_CUDA(le);
          }
        }
        QOB_CUDA(cudaStreamSynchronize(st));
        cudaGraphExecDestroy(ge);
      }
    }
    for (; s < nsteps; ++s) qob::ensemble_step(ctx->c, E, st);
    QOB_CUDA(cudaStreamSynchronize(st));
    return QOB_OK;
  } catch (const qob::Error& e) {
    ctx->c.err = e.msg;
    return e.code;
  }
}

// RK4 with time-dependent LazySum factors: row r of `factors` holds the factors
// at t0 + r*dt/2.  Stage 1 of step s uses row 2s, stages 2 and 3 row 2s+1,
// stage 4 row 2s+2; the values are re-evaluated on the device before each
// stage whose row differs from the previous one, from a device-side step
// counter, so steps after the first replay one recorded CUDA graph.
int qob_rk4_td(qob_ctx* ctx, qob_op* H, int dtype, void* psi, int64_t n, double dt, int nsteps,
               const double* factors, int64_t nrows, int renormalise, void* stream) {
  if (!ctx) return QOB_ERR_ARG;
  try {
    QOB_CUDA(cudaSetDevice(ctx->c.device));
    if (!H || !psi || n < 1 || nsteps < 0 || (dtype != QOB_C128 && dtype != QOB_C64 && dtype != QOB_C128X))
      qob::fail(QOB_ERR_ARG, "qob_rk4_td: bad arguments");
    if (H->node->kind != qob::Kind::LazySum) qob::fail(QOB_ERR_ARG, "qob_rk4_td needs a LazySum");
    if (nrows != 2 * (int64_t)nsteps + 1) qob::fail(QOB_ERR_ARG, "qob_rk4_td: nrows must be 2*nsteps+1");
    const size_t nf = H->node->factors.size();
    if (nf > 0 && !factors) qob::fail(QOB_ERR_ARG, "qob_rk4_td: null factor table");
    if (H->node->m != n || H->node->n != n) qob::fail(QOB_ERR_DIM, "Hamiltonian and state dimensions differ");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t sz = (size_t)n * (dtype == QOB_C64 ? 8 : 16);
    char* w = static_cast<char*>(ctx->c.ws.get(20, 3 * sz));
    qob::Plan& P = qob::batch_plan(ctx->c, H, dtype);
    if (P.kind != qob::Plan::Kind::Sum || !P.dense.empty() || !P.modek.empty() || !P.subs.empty())
      qob::fail(QOB_ERR_UNSUPPORTED, "qob_rk4_td: every term must compile into the fused gather");
    if (nsteps == 0) return QOB_OK;
    qob::prepare_factor_rows(P, *H->node, factors, nrows);
    qob::DeviceBuf table;
    table.upload(factors, std::max<size_t>((size_t)nrows * nf, 1) * 16);
    const double2* rows = (const double2*)table.p;
    qob::Ensemble E;
    E.renormalise = renormalise != 0;
    qob::ensemble_build(ctx->c, E, {qob::EvolveState{&P, psi, w, w + sz, w + 2 * sz, n, dt}}, dtype);
    // the step counter lives on the device, so a recorded step reads the rows
    // of the step it runs in: stage 2 row 2s+1, stage 4 row 2s+2 (stage 1
    // keeps row 2s from the previous step's stage 4; step 0 refreshes it)
    qob::DeviceBuf stepbuf;
    const long long zero = 0;
    stepbuf.upload(&zero, sizeof(zero));
    long long* dstep = static_cast<long long*>(stepbuf.p);
    bool first = true;
    std::function<void(int)> hook = [&](int mode) {
      if (!P.gather) return;
      if (mode == 1 && first) qob::device_refresh(*P.gather, rows, st, dstep, 0, (long long)nf);
      if (mode == 2) qob::device_refresh(*P.gather, rows, st, dstep, 1, (long long)nf);
      if (mode == 4) qob::device_refresh(*P.gather, rows, st, dstep, 2, (long long)nf);
    };
    auto one_step = [&](cudaStream_t s2) {
      qob::ensemble_step(ctx->c, E, s2, &hook);
      qob::launch_td_advance(dstep, s2);
    };
    int s = 0;
    if (nsteps > 0) {
      one_step(st);
      first = false;
      s = 1;
    }
    if (nsteps - s >= 4) {  // the rest: replays of a recorded step on the context's stream
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      QOB_CUDA(cudaStreamIsCapturing(st, &cs));
      if (cs == cudaStreamCaptureStatusNone) {
        QOB_CUDA(cudaStreamSynchronize(st));
        if (!ctx->c.copy_stream[1]) QOB_CUDA(cudaStreamCreateWithFlags(&ctx->c.copy_stream[1], cudaStreamNonBlocking));
        st = ctx->c.copy_stream[1];
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        QOB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
          one_step(st);
        } catch (...) {
          cudaStreamEndCapture(st, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        QOB_CUDA(cudaStreamEndCapture(st, &g));
        const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        QOB_CUDA(e);
        for (; s < nsteps; ++s) {
          const cudaError_t le = cudaGraphLaunch(ge, st);
          if (le != cudaSuccess) {
            cudaGraphExecDestroy(ge);
            QOB_CUDA(le);
          }
        }
        QOB_CUDA(cudaStreamSynchronize(st));
        cudaGraphExecDestroy(ge);
      }
    }
    for (; s < nsteps; ++s) one_step(st);
    QOB_CUDA(cudaStreamSynchronize(st));
    // the values now belong to the last row: the next use re-evaluates them
    // from the operator's own factors
    for (auto& d : P.deps)
      if (d.first == H->node.get()) d.second = ~uint64_t(0);
    return QOB_OK;
  } catch (const qob::Error& e) {
    ctx->c.err = e.msg;
    return e.code;
  }
}

}  // extern "C"
