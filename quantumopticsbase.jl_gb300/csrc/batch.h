// batch.h -- device work tables for applying many (uneven) operators in one
// persistent launch; used by qob_batch_* and by the serving engine.
#pragma once

#include <vector>

#include "qob_internal.h"

namespace qob {

// One fused item as the persistent kernel reads it.
struct BatchItemDev {
  GatherView v;
  const void* x;
  void* y;
  double2 alpha, beta;
};

// One application y = alpha * plan * x + beta * y (one ket, element stride 1).
struct BatchSpec {
  Plan* plan;
  const void* x;
  void* y;
  c128 alpha, beta;
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
  int grid = 1;
};

// The LEFT-side plan of an operator, compiled or refreshed on demand (capi.cu).
Plan& batch_plan(Context& ctx, qob_op* op, int prec);
bool plan_fusable(const Plan& P);
void build_tables(Context& ctx, BatchTables& T, const std::vector<BatchSpec>& specs, int prec, int tile);
void launch_tables(Context& ctx, const BatchTables& T, const std::vector<BatchSpec>& specs, cudaStream_t s);

}  // namespace qob
