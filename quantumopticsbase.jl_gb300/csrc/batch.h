// batch.h -- device work tables for applying many (uneven) operators in one
// persistent launch; used by qob_batch_* and by the serving engine.
#pragma once

#include <vector>

#include "qob_internal.h"

namespace qob {

// One fused item as the persistent kernel reads it.  With an RK4 stage
// (launch_tables' stage 1 .. 4) the item's k = alpha * plan * x goes straight
// into the stage combination of psi, acc and tmp_out instead of into y.
struct BatchItemDev {
  GatherView v;
  const void* x;
  void* y;
  double2 alpha, beta;
  void* psi;
  void* acc;
  void* tmp_out;
  double dt;
};

// One application y = alpha * plan * x + beta * y (one ket, element stride 1);
// psi, acc, tmp_out and dt for a fused RK4 stage.
struct BatchSpec {
  Plan* plan;
  const void* x;
  void* y;
  c128 alpha, beta;
  void* psi = nullptr;
  void* acc = nullptr;
  void* tmp_out = nullptr;
  double dt = 0.0;
};

struct BatchTables {
  DeviceBuf items, tiles;
  std::vector<bool> fused;  // per spec: in the persistent launch
  int prec = QOB_C128;
  int ntiles = 0;
  int nfused = 0;
  int tile = 256;
  bool real = true;
  bool ff = false;  // double-float items (ComplexF64 data): the kernel splits x as it loads
  size_t smem = 0;
  int grid = 1;      // persistent grid of the plain product
  int grid_rk4 = 1;  // and of the fused RK4 stages
};

// The LEFT-side plan of an operator, compiled or refreshed on demand (capi.cu).
Plan& batch_plan(Context& ctx, qob_op* op, int prec);
bool plan_fusable(const Plan& P);
void build_tables(Context& ctx, BatchTables& T, const std::vector<BatchSpec>& specs, int prec, int tile);
// stage 0: y = alpha * plan * x + beta * y for every item; 1 .. 4: the fused
// items run RK4 stage `stage` with k = alpha * plan * x (every item must be in
// the fused launch: all_fused)
void launch_tables(Context& ctx, const BatchTables& T, const std::vector<BatchSpec>& specs, cudaStream_t s,
                   int stage = 0);
bool all_fused(const BatchTables& T);

}  // namespace qob
