// capi.cu -- the C ABI (include/qobgpu.h): operator handles, plan cache,
// execution of compiled plans, and the FP64 reductions.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <new>

#include "qob_internal.h"

namespace qob {

void fail(int code, const std::string& msg) { throw Error{code, msg}; }

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  cudaGetLastError();  // clear a sticky-free error so the context stays usable
  if (e == cudaErrorMemoryAllocation) fail(QOB_ERR_OOM, std::string(what) + ": out of device memory");
  fail(QOB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

DeviceBuf::~DeviceBuf() {
  if (p) cudaFree(p);
}
void DeviceBuf::alloc(size_t b) {
  if (p) {
    cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  QOB_CUDA(cudaMalloc(&p, b));
  bytes = b;
}
void DeviceBuf::upload(const void* host, size_t b) {
  if (!p || bytes < b) alloc(b);
  QOB_CUDA(cudaMemcpy(p, host, b, cudaMemcpyHostToDevice));
}

void* Workspace::get(size_t slot, size_t bytes) {
  if (slots.size() <= slot) slots.resize(slot + 1);
  DeviceBuf& d = slots[slot];
  if (d.bytes < bytes) {
    // buffers are reused across calls; wait for work that may still use the old one
    QOB_CUDA(cudaDeviceSynchronize());
    d.alloc(bytes + bytes / 4);
  }
  return d.p;
}

Context::~Context() {
  if (reduce_host) cudaFreeHost(reduce_host);
  for (auto s : copy_stream)
    if (s) cudaStreamDestroy(s);
  for (int k = 0; k < kPipeChunks; ++k) {
    if (pipe_in[k]) cudaEventDestroy(pipe_in[k]);
    if (pipe_done[k]) cudaEventDestroy(pipe_done[k]);
  }
  for (auto e : stage_free)
    if (e) cudaEventDestroy(e);
  for (auto e : ticket_done)
    if (e) cudaEventDestroy(e);
}

namespace {

c128 coefval(const TermCoef& c, const OpNode* root) {
  if (c.top < 0) return c.inner;
  return cmul(root->factors[c.top], c.inner);
}

int64_t prod_range(const std::vector<int64_t>& v, size_t lo, size_t hi) {
  int64_t p = 1;
  for (size_t i = lo; i < hi; ++i) p *= v[i];
  return p;
}

}  // namespace

// Runs a compiled plan: y = alpha * op * x + beta * y on ncols vectors whose
// element e of vector c lives at x[e * xes + c * xcs].
void apply_plan(Context& ctx, Plan& P, c128 alpha, const void* x, int64_t xes, int64_t xcs,
                c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s,
                int ws) {
  const size_t esz = P.precision == QOB_C128 ? 16 : 8;
  const c128 one{1.0, 0.0}, zero{0.0, 0.0};
  if (P.kind == Plan::Kind::Sum) {
    // LazySum with no terms or alpha == 0: _zero_op_mul! (src/operators_lazysum.jl:190-192)
    if (is_zero(alpha) || P.nterms_total == 0) {
      launch_scale(P.precision, y, P.m, ncols, yes, ycs, beta, s);
      return;
    }
    c128 b = beta;  // the first pass applies beta, the rest accumulate (:194-197)
    if (P.gather) {
      // a double-float gather splits x into slot ws first (free here: x and y
      // of a nested call live in the caller's slots)
      void* ffx = P.gather->ff
                      ? ctx.ws.get(ws, (size_t)((P.n - 1) * xes + (ncols - 1) * xcs + 1) * 16)
                      : nullptr;
      launch_gather(*P.gather, P.precision, x, xes, xcs, y, yes, ycs, ncols, alpha, b, s, P.n, ffx, ctx.pdl);
      b = one;
    }
    for (auto& d : P.dense) {
      // partial sums of a split product in slot ws (free here, as for the split input above);
      // a double-float plan splits x into slot ws + 1 first
      const void* xin = x;
      if (P.ff) {
        void* xs = ctx.ws.get(ws + 1, (size_t)((P.n - 1) * xes + (ncols - 1) * xcs + 1) * 16);
        launch_ff_split(x, P.n, ncols, xes, xcs, xs, s);
        xin = xs;
      }
      const c128 ad = cmul(alpha, coefval(d.coef, P.root));
      if (ctx.fp32_tensor && P.precision == QOB_C64 && !P.ff && d.m >= kDmmaMinK && d.n >= kDmmaMinK) {
        if (!d.tc.ready) tc_dense_build(d.tc, d.a.p, d.m, d.n, s);
        launch_dense_tc(d.tc, ad, xin, xes, xcs, b, y, yes, ycs, ncols, s, &ctx.ws, ws,
                        static_cast<unsigned*>(ctx.status.p), ctx.num_sms, ctx.pdl);
      } else {
        launch_dense(P.precision, d.a.p, d.m, d.n, ad, xin, xes, xcs, b, y, yes, ycs, ncols, s, &ctx.ws, ws, P.ff,
                     ctx.fp64_tensor);
      }
      b = one;
    }
    for (auto& mk : P.modek) {
      const c128 a = cmul(alpha, coefval(mk.coef, P.root));
      const size_t nst = mk.steps.size();
      if (nst == 0) {
        launch_axpby(P.precision, x, xes, xcs, a, y, yes, ycs, b, P.m, ncols, s);
        b = one;
        continue;
      }
      std::vector<int64_t> cur = mk.shape_in;
      const void* src = x;
      int64_t ses = xes, scs = xcs;
      for (size_t k = 0; k < nst; ++k) {
        ModekStep& st = mk.steps[k];
        std::vector<int64_t> next = cur;
        next[st.site] = st.dout;
        const int64_t s1 = prod_range(cur, 0, st.site), s3 = prod_range(cur, st.site + 1, cur.size());
        const c128 ak = (k == 0) ? a : one;
        // a double-float plan splits each step's input into slot ws + 2 (the
        // step's temporaries use ws and ws + 1; sub-plans, which use ws + 2, run after)
        const bool ffs = P.ff && !st.eye;
        const void* sin = src;
        if (ffs) {
          const int64_t len_in = prod_range(cur, 0, cur.size());
          void* xs = ctx.ws.get(ws + 2, (size_t)((len_in - 1) * ses + (ncols - 1) * scs + 1) * 16);
          launch_ff_split(src, len_in, ncols, ses, scs, xs, s);
          sin = xs;
        }
        // ComplexF32 dense factors on the tensor cores: one product with the
        // (before, after, ket) index triples as columns, contracted dimension din
        const bool tc = ctx.fp32_tensor && P.precision == QOB_C64 && !ffs && !st.eye && st.din >= kDmmaMinK &&
                        st.dout >= kDmmaMinK;
        auto mode_product = [&](c128 bk, void* out, int64_t oes, int64_t ocs) {
          if (tc) {
            if (!st.tc.ready) tc_dense_build(st.tc, st.a.p, st.dout, st.din, s);
            TcColMap xm, ym;
            xm.s1 = ym.s1 = s1;
            xm.s3 = ym.s3 = s3;
            xm.sa = ses;
            xm.sb = s1 * st.din * ses;
            xm.st = scs;
            ym.sa = oes;
            ym.sb = s1 * st.dout * oes;
            ym.st = ocs;
            launch_gemm_tc(st.tc, ak, sin, s1 * ses, xm, bk, out, s1 * oes, ym, s1 * s3 * ncols, s, &ctx.ws, ws + 3,
                           static_cast<unsigned*>(ctx.status.p), ctx.num_sms, ctx.pdl);
          } else {
            launch_modek(P.precision, st.a.p, st.eye, s1, st.dout, st.din, s3, ak, sin, ses, scs, bk, out, oes, ocs,
                         ncols, s, ffs, ctx.fp64_tensor);
          }
        };
        if (k + 1 == nst) {
          mode_product(b, y, yes, ycs);
        } else {
          const int64_t len = prod_range(next, 0, next.size());
          void* t = ctx.ws.get(ws + (k % 2), (size_t)len * ncols * esz);
          mode_product(zero, t, 1, len);
          src = t;
          ses = 1;
          scs = len;
        }
        cur = next;
      }
      b = one;
    }
    for (auto& sp : P.subs) {
      apply_plan(ctx, *sp.plan, cmul(alpha, coefval(sp.coef, P.root)), x, xes, xcs, b, y, yes, ycs, ncols, s,
                 ws + 2);
      b = one;
    }
    return;
  }
  if (P.kind == Plan::Kind::Fft) {
    // FFTOperator mul! (src/particle.jl:438-535): one pass per transformed axis;
    // the first reads x, the last writes alpha * ... + beta * y
    const size_t na = P.fft.size();
    const void* src = x;
    int64_t ses = xes, scs = xcs;
    for (size_t a = 0; a < na; ++a) {
      if (a + 1 == na) {
        void* scratch = P.fft[a].n1 > 0 ? ctx.ws.get(ws + 2, (size_t)P.m * ncols * esz) : nullptr;
        launch_fft_pass(P.precision, P.fft[a], P.m, src, ses, scs, y, yes, ycs, ncols, alpha, beta, true, scratch,
                        s, P.ff);
      } else {
        void* t = ctx.ws.get(ws + (a % 2), (size_t)P.m * ncols * esz);
        launch_fft_pass(P.precision, P.fft[a], P.m, src, ses, scs, t, 1, P.m, ncols, one, zero, false, nullptr, s,
                        P.ff);
        src = t;
        ses = 1;
        scs = P.m;
      }
    }
    return;
  }
  // LazyProduct (src/operators_lazyproduct.jl:103-164)
  if (is_zero(alpha)) {
    launch_scale(P.precision, y, P.m, ncols, yes, ycs, beta, s);
    return;
  }
  const size_t n = P.chain.size();
  if (n == 1) {
    apply_plan(ctx, *P.chain[0], cmul(P.pfactor, alpha), x, xes, xcs, beta, y, yes, ycs, ncols, s, ws);
    return;
  }
  const void* src = x;
  int64_t ses = xes, scs = xcs;
  for (size_t i = 0; i < n; ++i) {
    Plan& Q = *P.chain[i];
    if (i + 1 == n) {
      apply_plan(ctx, Q, alpha, src, ses, scs, beta, y, yes, ycs, ncols, s, ws + 2);
    } else {
      void* t = ctx.ws.get(ws + (i % 2), (size_t)Q.m * ncols * esz);
      apply_plan(ctx, Q, i == 0 ? P.pfactor : one, src, ses, scs, zero, t, 1, Q.m, ncols, s, ws + 2);
      src = t;
      ses = 1;
      scs = Q.m;
    }
  }
}

}  // namespace qob

using namespace qob;

namespace {

template <class F>
int guard(qob_ctx* ctx, F&& f) {
  try {
    if (ctx) QOB_CUDA(cudaSetDevice(ctx->c.device));
    f();
    return QOB_OK;
  } catch (const Error& e) {
    if (ctx) ctx->c.err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->c.err = "host out of memory";
    return QOB_ERR_OOM;
  } catch (const std::exception& e) {
    if (ctx) ctx->c.err = e.what();
    return QOB_ERR_ARG;
  }
}

c128 read_c(const void* p, int dtype, int64_t i) {
  if (dtype == QOB_C128) {
    const double* d = static_cast<const double*>(p);
    return {d[2 * i], d[2 * i + 1]};
  }
  const float* f = static_cast<const float*>(p);
  return {(double)f[2 * i], (double)f[2 * i + 1]};
}

void check_dtype(int dtype) {
  if (dtype != QOB_C128 && dtype != QOB_C64) fail(QOB_ERR_ARG, "dtype must be QOB_C128 or QOB_C64");
}
// qob_mul and its relatives also take the double-float form of ComplexF64
void check_mul_dtype(int dtype) {
  if (dtype != QOB_C128 && dtype != QOB_C64 && dtype != QOB_C128X)
    fail(QOB_ERR_ARG, "dtype must be QOB_C128, QOB_C64 or QOB_C128X");
}
size_t elem_size(int dtype) { return dtype == QOB_C64 ? 8 : 16; }

qob_op* wrap(NodeP n) {
  auto* h = new qob_op;
  h->node = std::move(n);
  return h;
}

bool is_leaf(const OpNode& n) { return n.kind == Kind::Sparse || n.kind == Kind::Dense || n.kind == Kind::Eye; }

Plan& get_plan(Context& ctx, qob_op* op, int side, int prec) {
  auto& slot = op->plans[side][prec];
  if (slot && !plan_is_current(*slot)) {
    bool only_root = true;
    for (auto& d : slot->deps)
      if (d.first != op->node.get() && d.first->factors_version != d.second) only_root = false;
    if (only_root && op->node->kind == Kind::LazySum)
      refresh_coefficients(*slot, *op->node);
    else
      slot.reset();
  }
  if (!slot) slot = compile_plan(ctx, op->node, side, prec);
  return *slot;
}

}  // namespace

namespace qob {
// The LEFT-side plan of an operator, compiled or refreshed on demand (batch.cu).
Plan& batch_plan(Context& ctx, qob_op* op, int prec) { return get_plan(ctx, op, QOB_LEFT, prec); }
}  // namespace qob

namespace {

bool overlaps(const void* a, size_t abytes, const void* b, size_t bbytes) {
  const char* pa = static_cast<const char*>(a);
  const char* pb = static_cast<const char*>(b);
  return pa < pb + bbytes && pb < pa + abytes;
}

}  // namespace

extern "C" {

int qob_version(void) { return 10000; }

int64_t qob_kernel_launches(void) { return (int64_t)g_launches.load(std::memory_order_relaxed); }

int qob_create(qob_ctx** ctx, int device, unsigned flags) {
  (void)flags;
  if (!ctx) return QOB_ERR_ARG;
  *ctx = nullptr;
  auto* c = new qob_ctx;
  c->c.device = device;
  int rc = guard(c, [&] {
    int n = 0;
    QOB_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) fail(QOB_ERR_ARG, "no such CUDA device");
    QOB_CUDA(cudaDeviceGetAttribute(&c->c.num_sms, cudaDevAttrMultiProcessorCount, device));
    QOB_CUDA(cudaSetDevice(device));
    c->c.status.alloc(16);
    QOB_CUDA(cudaMemset(c->c.status.p, 0, 16));
  });
  if (rc) {
    delete c;
    return rc;
  }
  *ctx = c;
  return QOB_OK;
}

int qob_destroy(qob_ctx* ctx) {
  if (!ctx) return QOB_ERR_ARG;
  cudaSetDevice(ctx->c.device);
  delete ctx;
  return QOB_OK;
}

const char* qob_last_error(qob_ctx* ctx) { return ctx ? ctx->c.err.c_str() : "null context"; }

int qob_op_sparse(qob_ctx* ctx, int64_t m, int64_t n, const int64_t* colptr, const int64_t* rowval,
                  const void* nzval, int dtype, int adjoint, qob_op** out) {
  return guard(ctx, [&] {
    if (!out || !colptr || m < 0 || n < 0) fail(QOB_ERR_ARG, "qob_op_sparse: bad arguments");
    check_dtype(dtype);
    auto nd = std::make_shared<OpNode>();
    nd->kind = Kind::Sparse;
    nd->sm = m;
    nd->sn = n;
    nd->adjoint = adjoint != 0;
    nd->m = nd->adjoint ? n : m;
    nd->n = nd->adjoint ? m : n;
    nd->src_dtype = dtype;
    if (colptr[0] != 1) fail(QOB_ERR_ARG, "CSC colptr must start at 1");
    nd->colptr.resize(n + 1);
    for (int64_t c = 0; c <= n; ++c) {
      nd->colptr[c] = colptr[c] - 1;
      if (c > 0 && nd->colptr[c] < nd->colptr[c - 1]) fail(QOB_ERR_ARG, "CSC colptr must be non-decreasing");
    }
    const int64_t nnz = nd->colptr[n];
    if (nnz > 0 && (!rowval || !nzval)) fail(QOB_ERR_ARG, "CSC with entries needs rowval and nzval");
    nd->rowval.resize(nnz);
    nd->vals.resize(nnz);
    for (int64_t p = 0; p < nnz; ++p) {
      if (rowval[p] < 1 || rowval[p] > m) fail(QOB_ERR_ARG, "CSC row index out of range");
      nd->rowval[p] = rowval[p] - 1;
      nd->vals[p] = read_c(nzval, dtype, p);
    }
    *out = wrap(nd);
  });
}

int qob_op_dense(qob_ctx* ctx, int64_t m, int64_t n, const void* data, int64_t ld, int dtype, int adjoint,
                 qob_op** out) {
  return guard(ctx, [&] {
    if (!out || (m * n > 0 && !data) || m < 0 || n < 0 || ld < std::max<int64_t>(m, 1))
      fail(QOB_ERR_ARG, "qob_op_dense: bad arguments");
    check_dtype(dtype);
    auto nd = std::make_shared<OpNode>();
    nd->kind = Kind::Dense;
    nd->sm = m;
    nd->sn = n;
    nd->adjoint = adjoint != 0;
    nd->m = nd->adjoint ? n : m;
    nd->n = nd->adjoint ? m : n;
    nd->src_dtype = dtype;
    nd->vals.resize(m * n);
    for (int64_t c = 0; c < n; ++c)
      for (int64_t r = 0; r < m; ++r) nd->vals[r + c * m] = read_c(data, dtype, r + c * ld);
    *out = wrap(nd);
  });
}

int qob_op_eye(qob_ctx* ctx, int64_t m, int64_t n, qob_op** out) {
  return guard(ctx, [&] {
    if (!out || m < 0 || n < 0) fail(QOB_ERR_ARG, "qob_op_eye: bad arguments");
    auto nd = std::make_shared<OpNode>();
    nd->kind = Kind::Eye;
    nd->sm = nd->m = m;
    nd->sn = nd->n = n;
    *out = wrap(nd);
  });
}

int qob_op_lazytensor(qob_ctx* ctx, int nsub, const int64_t* shape_l, const int64_t* shape_r, int nfac,
                      const int64_t* indices, qob_op* const* factors, double factor_re, double factor_im,
                      qob_op** out) {
  return guard(ctx, [&] {
    if (!out || nsub < 1 || !shape_l || !shape_r || nfac < 0 || (nfac > 0 && (!indices || !factors)))
      fail(QOB_ERR_ARG, "qob_op_lazytensor: bad arguments");
    auto nd = std::make_shared<OpNode>();
    nd->kind = Kind::LazyTensor;
    nd->shape_l.assign(shape_l, shape_l + nsub);
    nd->shape_r.assign(shape_r, shape_r + nsub);
    nd->m = nd->n = 1;
    for (int i = 0; i < nsub; ++i) {
      if (shape_l[i] < 1 || shape_r[i] < 1) fail(QOB_ERR_ARG, "subsystem lengths must be positive");
      nd->m *= shape_l[i];
      nd->n *= shape_r[i];
    }
    nd->factor = {factor_re, factor_im};
    for (int k = 0; k < nfac; ++k) {
      const int64_t idx = indices[k];
      if (idx < 1 || idx > nsub) fail(QOB_ERR_ARG, "LazyTensor index out of range");
      if (k > 0 && idx <= indices[k - 1]) fail(QOB_ERR_ARG, "LazyTensor indices must be sorted and unique");
      if (!factors[k]) fail(QOB_ERR_ARG, "null factor");
      const NodeP& f = factors[k]->node;
      if (!is_leaf(*f))
        fail(QOB_ERR_UNSUPPORTED, "gemm! of LazyTensor is not implemented for a non-data operator factor");
      if (f->m != shape_l[idx - 1] || f->n != shape_r[idx - 1])
        fail(QOB_ERR_DIM, "factor shape does not match its subsystem");
      nd->sites.push_back((int)(idx - 1));
      nd->ops.push_back(f);
    }
    *out = wrap(nd);
  });
}

int qob_op_lazysum(qob_ctx* ctx, int64_t m, int64_t n, int nterms, const double* factors, qob_op* const* ops,
                   qob_op** out) {
  return guard(ctx, [&] {
    if (!out || nterms < 0 || (nterms > 0 && (!factors || !ops)) || m < 0 || n < 0)
      fail(QOB_ERR_ARG, "qob_op_lazysum: bad arguments");
    auto nd = std::make_shared<OpNode>();
    nd->kind = Kind::LazySum;
    nd->m = m;
    nd->n = n;
    for (int k = 0; k < nterms; ++k) {
      if (!ops[k]) fail(QOB_ERR_ARG, "null term");
      const NodeP& t = ops[k]->node;
      if (t->m != m || t->n != n) fail(QOB_ERR_DIM, "LazySum term shape does not match the sum (IncompatibleBases)");
      nd->ops.push_back(t);
      nd->factors.push_back({factors[2 * k], factors[2 * k + 1]});
    }
    *out = wrap(nd);
  });
}

int qob_op_lazyproduct(qob_ctx* ctx, int nops, qob_op* const* ops, double factor_re, double factor_im,
                       qob_op** out) {
  return guard(ctx, [&] {
    if (!out || nops < 1 || !ops) fail(QOB_ERR_ARG, "LazyProduct needs at least one operator");
    auto nd = std::make_shared<OpNode>();
    nd->kind = Kind::LazyProduct;
    for (int k = 0; k < nops; ++k) {
      if (!ops[k]) fail(QOB_ERR_ARG, "null operator");
      if (k > 0 && ops[k - 1]->node->n != ops[k]->node->m)
        fail(QOB_ERR_DIM, "LazyProduct operators are not multiplicable");
      nd->ops.push_back(ops[k]->node);
    }
    nd->m = nd->ops.front()->m;
    nd->n = nd->ops.back()->n;
    nd->factor = {factor_re, factor_im};
    *out = wrap(nd);
  });
}

int qob_op_set_factors(qob_ctx* ctx, qob_op* op, const double* factors) {
  return guard(ctx, [&] {
    if (!op || (!factors && !op->node->factors.empty())) fail(QOB_ERR_ARG, "qob_op_set_factors: bad arguments");
    if (op->node->kind != Kind::LazySum) fail(QOB_ERR_ARG, "set_factors needs a LazySum");
    for (size_t k = 0; k < op->node->factors.size(); ++k) op->node->factors[k] = {factors[2 * k], factors[2 * k + 1]};
    op->node->factors_version++;
  });
}

int qob_op_free(qob_ctx* ctx, qob_op* op) {
  return guard(ctx, [&] { delete op; });
}

int qob_op_shape(qob_ctx* ctx, const qob_op* op, int64_t* rows, int64_t* cols) {
  return guard(ctx, [&] {
    if (!op) fail(QOB_ERR_ARG, "null operator");
    if (rows) *rows = op->node->m;
    if (cols) *cols = op->node->n;
  });
}

int qob_op_prepare(qob_ctx* ctx, qob_op* op, int side, int dtype, int64_t* info) {
  return guard(ctx, [&] {
    if (!ctx || !op || (side != QOB_LEFT && side != QOB_RIGHT)) fail(QOB_ERR_ARG, "qob_op_prepare: bad arguments");
    check_mul_dtype(dtype);
    Plan& P = get_plan(ctx->c, op, side, dtype);
    if (info) {
      info[0] = P.gather ? P.gather->ngroups : 0;
      info[1] = P.gather && P.gather->has_diag ? 1 : 0;
      info[2] = P.gather ? P.gather->nentries : 0;
      info[3] = (int64_t)(P.dense.size() + P.modek.size() + P.subs.size() + P.chain.size());
    }
  });
}

namespace {
// The autotuner; writes min(times_len, 58) timings.
int tune_impl(qob_ctx* ctx, qob_op* op, int side, int dtype, int64_t ncols, double* times_ms, int times_len,
              int* chosen) {
  return guard(ctx, [&] {
    if (!ctx || !op || ncols < 1 || (side != QOB_LEFT && side != QOB_RIGHT) || times_len < 0)
      fail(QOB_ERR_ARG, "qob_op_tune: bad arguments");
    check_mul_dtype(dtype);
    Plan& P = get_plan(ctx->c, op, side, dtype);
    const int tiles[4] = {1, 2, 4, 8};
    // launch shapes: 128 / 256 threads, the persistent grid of 256-thread
    // blocks, and 128 / 256 threads with 4, 8 or 16 vector sets per warp
    constexpr int kShapes = 9;
    const int blocks[kShapes] = {128, 256, -256, 128, 256, 128, 256, 128, 256};
    const int splits[kShapes] = {1, 1, 1, 4, 4, 8, 8, 16, 16};
    // staged tiles (compact plans, vectors from the left): 2^bits indices x
    // vectors per thread x vector sets per warp, 256 threads
    constexpr int kTileShapes = 12;
    const int tbits_c[kTileShapes] = {10, 10, 9, 11, 11, 12, 9, 8, 8, 9, 10, 7};
    const int ttc_c[kTileShapes] = {1, 2, 4, 1, 2, 1, 1, 1, 2, 2, 1, 2};
    const int tls_c[kTileShapes] = {1, 1, 1, 1, 1, 1, 4, 16, 8, 4, 4, 16};
    // two consecutive indices per thread (compact plans, vectors from the
    // left): vectors per thread x threads x vector sets per warp
    constexpr int kPairShapes = 10;
    const int ptc_c[kPairShapes] = {2, 4, 2, 4, 2, 4, 2, 4, 2, 4};
    const int pblk_c[kPairShapes] = {256, 256, 128, 128, 256, 128, 128, 128, 128, 128};
    const int pls_c[kPairShapes] = {1, 1, 1, 1, 4, 4, 8, 8, 16, 16};
    constexpr int kCands = 4 * kShapes + kTileShapes + kPairShapes;
    double t[kCands];
    for (double& v : t) v = -1.0;
    int best = 0, best_block = 256, best_split = 1, best_tile = 0, best_pairs = 0;
    if (P.gather && P.kind == Plan::Kind::Sum) {
      GatherPlan& g = *P.gather;
      const size_t esz = elem_size(dtype);
      // Vector sets of 16 MB or more are tuned as a stream of such sets would
      // run -- inputs not in L2: up to 16 copies, at least 256 MB in all, used
      // in turn; smaller sets are tuned L2-resident, as they would be used.
      const size_t xsz = (size_t)P.n * ncols * esz, ysz = (size_t)P.m * ncols * esz;
      const size_t set = xsz + ysz;
      const int copies = set >= (size_t(16) << 20) ? (int)std::min<size_t>(16, ((size_t(256) << 20) + set - 1) / set) : 1;
      DeviceBuf x, y;
      x.alloc(xsz * copies);
      y.alloc(ysz * copies);
      // timed on a stream of the context's own, the launches replayed from a
      // CUDA graph: no host launch overhead in the times, as in a recorded loop
      if (!ctx->c.copy_stream[1]) QOB_CUDA(cudaStreamCreateWithFlags(&ctx->c.copy_stream[1], cudaStreamNonBlocking));
      cudaStream_t ts = ctx->c.copy_stream[1];
      QOB_CUDA(cudaMemsetAsync(x.p, 0, x.bytes, ts));
      QOB_CUDA(cudaMemsetAsync(y.p, 0, y.bytes, ts));
      auto xc = [&](int i) { return static_cast<char*>(x.p) + (size_t)(i % copies) * xsz; };
      auto yc = [&](int i) { return static_cast<char*>(y.p) + (size_t)(i % copies) * ysz; };
      // vectors as the reference lays them out: columns for LEFT, rows for RIGHT
      const int64_t xes = side == QOB_LEFT ? 1 : ncols, xcs = side == QOB_LEFT ? P.n : 1;
      const int64_t yes = side == QOB_LEFT ? 1 : ncols, ycs = side == QOB_LEFT ? P.m : 1;
      int mbits = 0;
      while ((int64_t(1) << mbits) < g.m) ++mbits;
      const bool tiles_ok = g.fast && g.square && side == QOB_LEFT && (int64_t(1) << mbits) == g.m;
      const bool pairs_ok = g.fast && g.square && side == QOB_LEFT && g.all_w1 && g.m % 2 == 0;
      cudaEvent_t e0, e1;
      QOB_CUDA(cudaEventCreate(&e0));
      QOB_CUDA(cudaEventCreate(&e1));
      double best_t = 1e300;
      for (int k = 0; k < kCands; ++k) {
        int tc, blk, ls, tb = 0, pr = 0;
        if (k < 4 * kShapes) {
          tc = tiles[k / kShapes];
          blk = blocks[k % kShapes];
          ls = splits[k % kShapes];
          if (tc > ncols || (tc > 1 && side == QOB_RIGHT && ncols > 1)) continue;
          if (ls > 1 && (tc * ls > ncols || side == QOB_RIGHT)) continue;
        } else if (k < 4 * kShapes + kTileShapes) {
          const int i = k - 4 * kShapes;
          tc = ttc_c[i];
          blk = 256;
          ls = tls_c[i];
          tb = tbits_c[i];
          if (!tiles_ok || tb > mbits || tc * ls > ncols) continue;
        } else {
          const int i = k - 4 * kShapes - kTileShapes;
          tc = ptc_c[i];
          blk = pblk_c[i];
          ls = pls_c[i];
          pr = 1;
          if (!pairs_ok || tc * ls > ncols) continue;
        }
        g.tc = tc;
        g.block = blk;
        g.lane_split = ls;
        g.tile_bits = tb;
        g.pairs = pr;
        for (int i = 0; i < 2; ++i)
          apply_plan(ctx->c, P, {1.0, 0.0}, xc(i), xes, xcs, {0.3, 0.0}, yc(i), yes, ycs, ncols, ts, 0);
        const int reps = std::max(8, copies);
        cudaGraph_t gr = nullptr;
        QOB_CUDA(cudaStreamBeginCapture(ts, cudaStreamCaptureModeThreadLocal));
        try {
          for (int i = 0; i < reps; ++i)
            apply_plan(ctx->c, P, {1.0, 0.0}, xc(i + 2), xes, xcs, {0.3, 0.0}, yc(i + 2), yes, ycs, ncols, ts, 0);
        } catch (...) {
          cudaStreamEndCapture(ts, &gr);  // leave the stream usable
          if (gr) cudaGraphDestroy(gr);
          throw;
        }
        QOB_CUDA(cudaStreamEndCapture(ts, &gr));
        cudaGraphExec_t ge = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&ge, gr, 0);
        cudaGraphDestroy(gr);
        QOB_CUDA(ie);
        QOB_CUDA(cudaGraphLaunch(ge, ts));  // untimed replay
        QOB_CUDA(cudaEventRecord(e0, ts));
        QOB_CUDA(cudaGraphLaunch(ge, ts));
        QOB_CUDA(cudaEventRecord(e1, ts));
        const cudaError_t se = cudaEventSynchronize(e1);
        cudaGraphExecDestroy(ge);
        QOB_CUDA(se);
        float ms = 0.f;
        QOB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        t[k] = ms / reps;
        if (t[k] < best_t) {
          best_t = t[k];
          best = tc;
          best_block = blk;
          best_split = ls;
          best_tile = tb;
          best_pairs = pr;
        }
      }
      g.tc = best;
      g.block = best_block;
      g.lane_split = best_split;
      g.tile_bits = best_tile;
      g.pairs = best_pairs;
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
    }
    if (times_ms)
      for (int k = 0; k < kCands && k < times_len; ++k) times_ms[k] = t[k];
    int lg = 0;
    while ((1 << lg) < best_split) ++lg;
    if (chosen)
      *chosen = best | (best_pairs << 7) | (best_tile << 8) | ((best_block < 0 ? -best_block : best_block) << 16) |
                (lg << 26) | (best_block < 0 ? (1 << 30) : 0);
  });
}
}  // namespace

int qob_op_tune(qob_ctx* ctx, qob_op* op, int side, int dtype, int64_t ncols, double* times_ms, int* chosen) {
  return tune_impl(ctx, op, side, dtype, ncols, times_ms, 36, chosen);
}

int qob_op_tune_ex(qob_ctx* ctx, qob_op* op, int side, int dtype, int64_t ncols, double* times_ms, int times_len,
                   int* chosen) {
  return tune_impl(ctx, op, side, dtype, ncols, times_ms, times_len, chosen);
}

int qob_op_set_launch(qob_ctx* ctx, qob_op* op, int side, int dtype, int vectors_per_thread, int block,
                      int lane_split) {
  return guard(ctx, [&] {
    if (!ctx || !op || (side != QOB_LEFT && side != QOB_RIGHT)) fail(QOB_ERR_ARG, "qob_op_set_launch: bad arguments");
    check_mul_dtype(dtype);
    if (vectors_per_thread != 1 && vectors_per_thread != 2 && vectors_per_thread != 4 && vectors_per_thread != 8)
      fail(QOB_ERR_ARG, "vectors per thread must be 1, 2, 4 or 8");
    if (block != 128 && block != 256 && block != -256) fail(QOB_ERR_ARG, "block must be 128, 256 or -256");
    if (lane_split < 1 || lane_split > 32 || (lane_split & (lane_split - 1)) != 0)
      fail(QOB_ERR_ARG, "lane_split must be 1, 2, 4, 8, 16 or 32");
    Plan& P = get_plan(ctx->c, op, side, dtype);
    if (P.gather) {
      P.gather->tc = vectors_per_thread;
      P.gather->block = block;
      P.gather->lane_split = lane_split;
      P.gather->tile_bits = 0;
      P.gather->pairs = 0;
    }
  });
}

int qob_op_set_pairs(qob_ctx* ctx, qob_op* op, int side, int dtype, int vectors_per_thread, int block,
                     int lane_split) {
  return guard(ctx, [&] {
    if (!ctx || !op || (side != QOB_LEFT && side != QOB_RIGHT)) fail(QOB_ERR_ARG, "qob_op_set_pairs: bad arguments");
    check_mul_dtype(dtype);
    if (vectors_per_thread != 2 && vectors_per_thread != 4)
      fail(QOB_ERR_ARG, "vectors per thread must be 2 or 4 for index pairs");
    if (block != 128 && block != 256) fail(QOB_ERR_ARG, "block must be 128 or 256");
    if (lane_split < 1 || lane_split > 32 || (lane_split & (lane_split - 1)) != 0)
      fail(QOB_ERR_ARG, "lane_split must be 1, 2, 4, 8, 16 or 32");
    Plan& P = get_plan(ctx->c, op, side, dtype);
    if (P.gather) {
      P.gather->tc = vectors_per_thread;
      P.gather->block = block;
      P.gather->lane_split = lane_split;
      P.gather->tile_bits = 0;
      P.gather->pairs = 1;
    }
  });
}

int qob_op_set_tile(qob_ctx* ctx, qob_op* op, int side, int dtype, int vectors_per_thread, int lane_split,
                    int tile_bits) {
  return guard(ctx, [&] {
    if (!ctx || !op || (side != QOB_LEFT && side != QOB_RIGHT)) fail(QOB_ERR_ARG, "qob_op_set_tile: bad arguments");
    check_mul_dtype(dtype);
    if (vectors_per_thread != 1 && vectors_per_thread != 2 && vectors_per_thread != 4)
      fail(QOB_ERR_ARG, "vectors per thread must be 1, 2 or 4 for staged tiles");
    if (lane_split < 1 || lane_split > 32 || (lane_split & (lane_split - 1)) != 0)
      fail(QOB_ERR_ARG, "lane_split must be 1, 2, 4, 8, 16 or 32");
    if (tile_bits < 6 || tile_bits > 16) fail(QOB_ERR_ARG, "tile_bits must be in 6 .. 16");
    Plan& P = get_plan(ctx->c, op, side, dtype);
    if (P.gather) {
      P.gather->tc = vectors_per_thread;
      P.gather->block = 256;
      P.gather->lane_split = lane_split;
      P.gather->tile_bits = tile_bits;
      P.gather->pairs = 0;
    }
  });
}

#ifdef QOB_DEBUG_BOUNDS
// Bounds-checked build only: moves the input offset of the first stored entry
// with a nonzero value of op's compiled gather (side, dtype) by col_shift, so
// that a test can watch the device checks catch an index out of range.
int qob_debug_shift_slot(qob_ctx* ctx, qob_op* op, int side, int dtype, int col_shift) {
  return guard(ctx, [&] {
    if (!ctx || !op || (side != QOB_LEFT && side != QOB_RIGHT)) fail(QOB_ERR_ARG, "qob_debug_shift_slot: bad arguments");
    check_mul_dtype(dtype);
    Plan& P = get_plan(ctx->c, op, side, dtype);
    if (!P.gather || P.gather->ell_slots <= 0) fail(QOB_ERR_UNSUPPORTED, "no fixed-width slots in this plan");
    GatherPlan& g = *P.gather;
    const size_t n = (size_t)g.ell_slots;
    const size_t sz = g.ell.bytes / n;  // slot size: col (int32) first, the value after the padding
    std::vector<unsigned char> h(n * sz);
    QOB_CUDA(cudaDeviceSynchronize());
    QOB_CUDA(cudaMemcpy(h.data(), g.ell.p, h.size(), cudaMemcpyDeviceToHost));
    const size_t voff = sz >= 16 ? 8 : 4;
    for (size_t i = 0; i < n; ++i) {
      unsigned char* e = h.data() + i * sz;
      bool nonzero = false;
      for (size_t b = voff; b < sz; ++b) nonzero |= e[b] != 0;
      if (!nonzero) continue;
      int32_t col;
      std::memcpy(&col, e, 4);
      col += col_shift;
      std::memcpy(e, &col, 4);
      QOB_CUDA(cudaMemcpy(g.ell.p, h.data(), h.size(), cudaMemcpyHostToDevice));
      return;
    }
    fail(QOB_ERR_UNSUPPORTED, "no stored entry with a nonzero value");
  });
}
#endif

int qob_set_option(qob_ctx* ctx, int option, int64_t value) {
  return guard(ctx, [&] {
    if (!ctx) fail(QOB_ERR_ARG, "qob_set_option: bad arguments");
    if (option == QOB_OPT_FP64_TENSOR)
      ctx->c.fp64_tensor = value != 0;
    else if (option == QOB_OPT_PDL)
      ctx->c.pdl = value != 0;
    else if (option == QOB_OPT_FP32_TENSOR)
      ctx->c.fp32_tensor = value != 0;
    else
      fail(QOB_ERR_ARG, "qob_set_option: unknown option");
  });
}

int qob_device_status(qob_ctx* ctx, void* stream, unsigned* flags) {
  return guard(ctx, [&] {
    if (!ctx) fail(QOB_ERR_ARG, "qob_device_status: bad arguments");
    unsigned w = 0;
    const cudaStream_t s = (cudaStream_t)stream;
    QOB_CUDA(cudaMemcpyAsync(&w, ctx->c.status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QOB_CUDA(cudaStreamSynchronize(s));
    if (flags) *flags = w;
    if (w) {
      QOB_CUDA(cudaMemsetAsync(ctx->c.status.p, 0, sizeof(unsigned), s));
      QOB_CUDA(cudaStreamSynchronize(s));
      if (w & 2u)
        fail(QOB_ERR_ARG, "device status: a kernel met an out-of-range index (bounds-checked build) and skipped it");
      fail(QOB_ERR_TIMEOUT, "device status: a kernel's bounded wait gave up; its output is incomplete");
    }
  });
}

namespace {

// The vector layout of y = alpha * op * x + beta * y: vectors are the columns
// of x and y (side LEFT, kets) or their rows (side RIGHT, bras); checks the
// dimensions as the reference's mul! does (src/operators.jl).
struct MulShape {
  int64_t ncols = 0, xes = 1, xcs = 1, yes = 1, ycs = 1;
  bool empty = false;
};

MulShape mul_shape(const qob_op* op, int side, int is_vector, int64_t x_rows, int64_t x_cols, int64_t x_ld,
                   int64_t y_rows, int64_t y_cols, int64_t y_ld) {
  if (!op) fail(QOB_ERR_ARG, "null context or operator");
  if (side != QOB_LEFT && side != QOB_RIGHT) fail(QOB_ERR_ARG, "side must be QOB_LEFT or QOB_RIGHT");
  const int64_t m = op->node->m, n = op->node->n;
  MulShape sh;
  if (side == QOB_LEFT) {
    if (x_rows != n) fail(QOB_ERR_DIM, "A and B dimensions do not match. Can't do `A*B`");
    if (y_rows != m || y_cols != x_cols) fail(QOB_ERR_DIM, "Output dimensions do not match A*B. Can't do `R.=A*B`");
    if (is_vector && x_cols != 1) fail(QOB_ERR_ARG, "a Ket has one column");
    if (x_ld < std::max<int64_t>(x_rows, 1) || y_ld < std::max<int64_t>(y_rows, 1))
      fail(QOB_ERR_ARG, "leading dimension smaller than the number of rows");
    sh.ncols = x_cols;
    sh.xcs = x_ld;
    sh.ycs = y_ld;
  } else {
    if (x_cols != m) fail(QOB_ERR_DIM, "A and B dimensions do not match. Can't do `A*B`");
    if (y_cols != n || y_rows != x_rows) fail(QOB_ERR_DIM, "Output dimensions do not match A*B. Can't do `R.=A*B`");
    if (is_vector && x_rows != 1) fail(QOB_ERR_ARG, "a Bra has one row");
    if (x_ld < std::max<int64_t>(x_rows, 1) || y_ld < std::max<int64_t>(y_rows, 1))
      fail(QOB_ERR_ARG, "leading dimension smaller than the number of rows");
    sh.ncols = x_rows;
    sh.xes = x_ld;
    sh.yes = y_ld;
  }
  sh.empty = sh.ncols == 0 || (side == QOB_LEFT ? m : n) == 0;
  if (!sh.empty && sh.ncols > 65535 && side == QOB_RIGHT) fail(QOB_ERR_UNSUPPORTED, "more than 65535 rows");
  return sh;
}

// Enqueues one host call: copies in on copy_stream[0], the application on
// copy_stream[1], the copy of y back on copy_stream[2], linked per chunk by
// events.  With `chunks` (a call waited on alone), several kets from the left
// go through in up to four chunks of columns, so that the copies of one chunk
// overlap the kernels of another; otherwise (a stream of calls, which overlap
// one another) and for other shapes in one piece, with the fewest copies.  The
// call uses staging set (host_calls % 2) once the copy out of the call before
// the previous one has left it.  Returns the call's ticket.
uint64_t enqueue_host(Context& c, int side, int is_vector, qob_op* op, int dtype, c128 alpha, const void* x,
                      int64_t x_rows, int64_t x_cols, c128 beta, void* y, int64_t y_rows, int64_t y_cols,
                      bool chunks) {
  check_mul_dtype(dtype);
  const MulShape sh = mul_shape(op, side, is_vector, x_rows, x_cols, std::max<int64_t>(x_rows, 1), y_rows, y_cols,
                                std::max<int64_t>(y_rows, 1));
  const bool has_beta = beta.re != 0.0 || beta.im != 0.0;
  {
    const size_t esz = elem_size(dtype);
    if (!sh.empty && overlaps(x, (size_t)x_rows * x_cols * esz, y, (size_t)y_rows * y_cols * esz))
      fail(QOB_ERR_ALIAS, "output matrix must not be aliased with input matrix");
  }
  for (int k = 0; k < 3; ++k)
    if (!c.copy_stream[k]) QOB_CUDA(cudaStreamCreateWithFlags(&c.copy_stream[k], cudaStreamNonBlocking));
  for (int k = 0; k < Context::kPipeChunks; ++k) {
    if (!c.pipe_in[k]) QOB_CUDA(cudaEventCreateWithFlags(&c.pipe_in[k], cudaEventDisableTiming));
    if (!c.pipe_done[k]) QOB_CUDA(cudaEventCreateWithFlags(&c.pipe_done[k], cudaEventDisableTiming));
  }
  for (int k = 0; k < 2; ++k)
    if (!c.stage_free[k]) QOB_CUDA(cudaEventCreateWithFlags(&c.stage_free[k], cudaEventDisableTiming));
  for (int k = 0; k < Context::kTickets; ++k)
    if (!c.ticket_done[k]) QOB_CUDA(cudaEventCreateWithFlags(&c.ticket_done[k], cudaEventDisableTiming));
  cudaStream_t sin = c.copy_stream[0], scomp = c.copy_stream[1], sout = c.copy_stream[2];
  const uint64_t ticket = c.host_calls + 1;
  if (!sh.empty) {
    if (!x || !y) fail(QOB_ERR_ARG, "null data pointer");
    const int st = (int)(c.host_calls & 1);
    const size_t esz = elem_size(dtype);
    const size_t xb = (size_t)x_rows * x_cols * esz, yb = (size_t)y_rows * y_cols * esz;
    if (c.stage_x[st].bytes < xb || c.stage_y[st].bytes < yb) {
      // a larger set: the calls in flight finish before the old one is freed
      for (int k = 0; k < 3; ++k) QOB_CUDA(cudaStreamSynchronize(c.copy_stream[k]));
      if (c.stage_x[st].bytes < xb) c.stage_x[st].alloc(xb);
      if (c.stage_y[st].bytes < yb) c.stage_y[st].alloc(yb);
    }
    Plan& P = get_plan(c, op, side, dtype);
    if (c.stage_used[st]) QOB_CUDA(cudaStreamWaitEvent(sin, c.stage_free[st], 0));
    const bool chunked = chunks && side == QOB_LEFT && x_cols >= 8;
    const int64_t nchunk = chunked ? std::min<int64_t>(4, x_cols / 4) : 1;
    const int64_t per = chunked ? (x_cols + nchunk - 1) / nchunk : x_cols;
    int64_t k = 0;
    for (int64_t c0 = 0; c0 < x_cols; c0 += per, ++k) {
      const int64_t nc = std::min(per, x_cols - c0);
      char* dx = static_cast<char*>(c.stage_x[st].p) + (size_t)c0 * x_rows * esz;
      char* dy = static_cast<char*>(c.stage_y[st].p) + (size_t)c0 * y_rows * esz;
      const char* hx = static_cast<const char*>(x) + (size_t)c0 * x_rows * esz;
      char* hy = static_cast<char*>(y) + (size_t)c0 * y_rows * esz;
      QOB_CUDA(cudaMemcpyAsync(dx, hx, (size_t)nc * x_rows * esz, cudaMemcpyHostToDevice, sin));
      if (has_beta) QOB_CUDA(cudaMemcpyAsync(dy, hy, (size_t)nc * y_rows * esz, cudaMemcpyHostToDevice, sin));
      QOB_CUDA(cudaEventRecord(c.pipe_in[k], sin));
      QOB_CUDA(cudaStreamWaitEvent(scomp, c.pipe_in[k], 0));
      if (chunked)
        apply_plan(c, P, alpha, dx, 1, x_rows, beta, dy, 1, y_rows, nc, scomp, 24);
      else
        apply_plan(c, P, alpha, dx, sh.xes, sh.xcs, beta, dy, sh.yes, sh.ycs, sh.ncols, scomp, 24);
      QOB_CUDA(cudaEventRecord(c.pipe_done[k], scomp));
      QOB_CUDA(cudaStreamWaitEvent(sout, c.pipe_done[k], 0));
      QOB_CUDA(cudaMemcpyAsync(hy, dy, (size_t)nc * y_rows * esz, cudaMemcpyDeviceToHost, sout));
    }
    QOB_CUDA(cudaEventRecord(c.stage_free[st], sout));
    c.stage_used[st] = true;
  }
  QOB_CUDA(cudaEventRecord(c.ticket_done[(ticket - 1) % Context::kTickets], sout));
  c.host_calls = ticket;
  return ticket;
}

}  // namespace

int qob_mul(qob_ctx* ctx, int side, int is_vector, qob_op* op, int dtype, double alpha_re, double alpha_im,
            const void* x, int64_t x_rows, int64_t x_cols, int64_t x_ld, double beta_re, double beta_im, void* y,
            int64_t y_rows, int64_t y_cols, int64_t y_ld, void* stream) {
  return guard(ctx, [&] {
    if (!ctx) fail(QOB_ERR_ARG, "null context or operator");
    check_mul_dtype(dtype);
    const MulShape sh = mul_shape(op, side, is_vector, x_rows, x_cols, x_ld, y_rows, y_cols, y_ld);
    if (sh.empty) return;
    if (!x || !y) fail(QOB_ERR_ARG, "null data pointer");
    const size_t esz = elem_size(dtype);
    const size_t xbytes = (size_t)(x_ld * (x_cols - 1) + x_rows) * esz;
    const size_t ybytes = (size_t)(y_ld * (y_cols - 1) + y_rows) * esz;
    if (overlaps(x, xbytes, y, ybytes)) fail(QOB_ERR_ALIAS, "output matrix must not be aliased with input matrix");
    Plan& P = get_plan(ctx->c, op, side, dtype);
    apply_plan(ctx->c, P, {alpha_re, alpha_im}, x, sh.xes, sh.xcs, {beta_re, beta_im}, y, sh.yes, sh.ycs, sh.ncols,
               (cudaStream_t)stream, 0);
  });
}

int qob_mul_host(qob_ctx* ctx, int side, int is_vector, qob_op* op, int dtype, double alpha_re, double alpha_im,
                 const void* x, int64_t x_rows, int64_t x_cols, double beta_re, double beta_im, void* y,
                 int64_t y_rows, int64_t y_cols) {
  return guard(ctx, [&] {
    if (!ctx) fail(QOB_ERR_ARG, "null context or operator");
    const uint64_t t = enqueue_host(ctx->c, side, is_vector, op, dtype, {alpha_re, alpha_im}, x, x_rows, x_cols,
                                    {beta_re, beta_im}, y, y_rows, y_cols, true);
    QOB_CUDA(cudaEventSynchronize(ctx->c.ticket_done[(t - 1) % Context::kTickets]));
  });
}

int qob_mul_host_async(qob_ctx* ctx, int side, int is_vector, qob_op* op, int dtype, double alpha_re,
                       double alpha_im, const void* x, int64_t x_rows, int64_t x_cols, double beta_re,
                       double beta_im, void* y, int64_t y_rows, int64_t y_cols, uint64_t* ticket) {
  return guard(ctx, [&] {
    if (!ctx || !ticket) fail(QOB_ERR_ARG, "null context or ticket");
    *ticket = enqueue_host(ctx->c, side, is_vector, op, dtype, {alpha_re, alpha_im}, x, x_rows, x_cols,
                           {beta_re, beta_im}, y, y_rows, y_cols, false);
  });
}

int qob_host_wait(qob_ctx* ctx, uint64_t ticket) {
  return guard(ctx, [&] {
    if (!ctx) fail(QOB_ERR_ARG, "null context");
    if (ticket > ctx->c.host_calls) fail(QOB_ERR_ARG, "qob_host_wait: ticket not handed out");
    if (ticket == 0) return;
    // a slot recorded again by a later call ends later: waiting on it is safe
    QOB_CUDA(cudaEventSynchronize(ctx->c.ticket_done[(ticket - 1) % Context::kTickets]));
  });
}

int qob_norm(qob_ctx* ctx, int dtype, const void* x, int64_t n, double* result, void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !x || !result || n < 0) fail(QOB_ERR_ARG, "qob_norm: bad arguments");
    check_dtype(dtype);
    reduce_dot(ctx->c, dtype, x, x, n, true, result, (cudaStream_t)stream);
  });
}

int qob_dot(qob_ctx* ctx, int dtype, const void* x, const void* y, int64_t n, double* result, void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !x || !y || !result || n < 0) fail(QOB_ERR_ARG, "qob_dot: bad arguments");
    check_dtype(dtype);
    reduce_dot(ctx->c, dtype, x, y, n, false, result, (cudaStream_t)stream);
  });
}

struct qob_graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
};

int qob_graph_begin(qob_ctx* ctx, void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !stream) fail(QOB_ERR_ARG, "capture needs a context and a non-default stream");
    QOB_CUDA(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
  });
}

int qob_graph_end(qob_ctx* ctx, void* stream, qob_graph** out) {
  return guard(ctx, [&] {
    if (!ctx || !stream || !out) fail(QOB_ERR_ARG, "qob_graph_end: bad arguments");
    auto* gr = new qob_graph;
    cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &gr->g);
    if (e != cudaSuccess) {
      delete gr;
      cuda_check(e, "cudaStreamEndCapture");
    }
    e = cudaGraphInstantiate(&gr->e, gr->g, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(gr->g);
      delete gr;
      cuda_check(e, "cudaGraphInstantiate");
    }
    *out = gr;
  });
}

int qob_graph_launch(qob_ctx* ctx, qob_graph* graph, void* stream) {
  return guard(ctx, [&] {
    if (!graph) fail(QOB_ERR_ARG, "null graph");
    QOB_CUDA(cudaGraphLaunch(graph->e, (cudaStream_t)stream));
  });
}

int qob_graph_free(qob_ctx* ctx, qob_graph* graph) {
  return guard(ctx, [&] {
    if (!graph) return;
    if (graph->e) cudaGraphExecDestroy(graph->e);
    if (graph->g) cudaGraphDestroy(graph->g);
    delete graph;
  });
}

int qob_expect(qob_ctx* ctx, qob_op* op, int dtype, const void* psi, int64_t n, double* result, void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !op || !psi || !result) fail(QOB_ERR_ARG, "qob_expect: bad arguments");
    check_dtype(dtype);
    if (op->node->m != n || op->node->n != n) fail(QOB_ERR_DIM, "expect needs a square operator matching the state");
    const size_t esz = dtype == QOB_C128 ? 16 : 8;
    void* t = ctx->c.ws.get(15, (size_t)n * esz);
    Plan& P = get_plan(ctx->c, op, QOB_LEFT, dtype);
    apply_plan(ctx->c, P, {1.0, 0.0}, psi, 1, n, {0.0, 0.0}, t, 1, n, 1, (cudaStream_t)stream, 16);
    reduce_dot(ctx->c, dtype, psi, t, n, false, result, (cudaStream_t)stream);
  });
}

int qob_expect_dm(qob_ctx* ctx, qob_op* op, int dtype, const void* rho, int64_t n, int64_t ld, double* result,
                  void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !op || !rho || !result || n < 0) fail(QOB_ERR_ARG, "qob_expect_dm: bad arguments");
    check_dtype(dtype);
    if (op->node->m != n || op->node->n != n) fail(QOB_ERR_DIM, "expect needs a square operator matching the state");
    if (ld < std::max<int64_t>(n, 1)) fail(QOB_ERR_ARG, "leading dimension smaller than the number of rows");
    if (n == 0) {
      result[0] = result[1] = 0.0;
      return;
    }
    const size_t esz = dtype == QOB_C128 ? 16 : 8;
    const cudaStream_t s = (cudaStream_t)stream;
    // t = op * rho[:, c0 : c0 + w] for column blocks of rho (every column a
    // vector), then the block's share of tr(op rho) = sum_ij op[i,j] rho[j,i]:
    // t[c0 + j, j] for j < w.  The workspace holds one block of at most
    // kExpectDmWorkspace bytes (at least one column); the blocks' sums are
    // added in block order in FP64.
    constexpr size_t kExpectDmWorkspace = 256ull << 20;
    const int64_t w = std::max<int64_t>(1, std::min<int64_t>(n, (int64_t)(kExpectDmWorkspace / ((size_t)n * esz))));
    void* t = ctx->c.ws.get(13, (size_t)n * w * esz);
    Plan& P = get_plan(ctx->c, op, QOB_LEFT, dtype);
    double re = 0.0, im = 0.0;
    for (int64_t c0 = 0; c0 < n; c0 += w) {
      const int64_t nc = std::min<int64_t>(w, n - c0);
      const char* rb = static_cast<const char*>(rho) + (size_t)c0 * ld * esz;
      apply_plan(ctx->c, P, {1.0, 0.0}, rb, 1, ld, {0.0, 0.0}, t, 1, n, nc, s, 16);
      double part[2];
      reduce_strided_sum(ctx->c, dtype, static_cast<const char*>(t) + (size_t)c0 * esz, nc, n + 1, part, s);
      re += part[0];
      im += part[1];
    }
    result[0] = re;
    result[1] = im;
  });
}

int qob_variance(qob_ctx* ctx, qob_op* op, int dtype, const void* psi, int64_t n, double* result, void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !op || !psi || !result) fail(QOB_ERR_ARG, "qob_variance: bad arguments");
    check_dtype(dtype);
    if (op->node->m != n || op->node->n != n) fail(QOB_ERR_DIM, "variance needs a square operator matching the state");
    const size_t esz = dtype == QOB_C128 ? 16 : 8;
    const cudaStream_t s = (cudaStream_t)stream;
    void* x = ctx->c.ws.get(14, (size_t)n * esz);
    void* z = ctx->c.ws.get(15, (size_t)n * esz);
    Plan& P = get_plan(ctx->c, op, QOB_LEFT, dtype);
    // x = op psi, z = op x (the reference's op*state, op*x)
    apply_plan(ctx->c, P, {1.0, 0.0}, psi, 1, n, {0.0, 0.0}, x, 1, n, 1, s, 16);
    apply_plan(ctx->c, P, {1.0, 0.0}, x, 1, n, {0.0, 0.0}, z, 1, n, 1, s, 16);
    double e2[2], e1[2];
    reduce_dot(ctx->c, dtype, psi, z, n, false, e2, s);
    reduce_dot(ctx->c, dtype, psi, x, n, false, e1, s);
    // <psi|op^2|psi> - <psi|op|psi>^2 in complex arithmetic, as the reference's
    // state.data' * (op*x).data - (state.data' * x.data)^2
    result[0] = e2[0] - (e1[0] * e1[0] - e1[1] * e1[1]);
    result[1] = e2[1] - 2.0 * e1[0] * e1[1];
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// device states for callers without their own device memory management: a
// state is dim x ncols complex values of one dtype, column-major
// ---------------------------------------------------------------------------
extern "C" {

int qob_state_alloc(qob_ctx* ctx, int dtype, int64_t dim, int64_t ncols, void** out) {
  return guard(ctx, [&] {
    if (!ctx || !out || dim < 0 || ncols < 0) fail(QOB_ERR_ARG, "qob_state_alloc: bad arguments");
    check_dtype(dtype);
    QOB_CUDA(cudaSetDevice(ctx->c.device));
    const size_t bytes = std::max<size_t>((size_t)dim * ncols * (dtype == QOB_C128 ? 16 : 8), 16);
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      fail(QOB_ERR_OOM, "qob_state_alloc: out of device memory");
    }
    QOB_CUDA(e);
    QOB_CUDA(cudaMemset(p, 0, bytes));
    *out = p;
  });
}

int qob_state_free(qob_ctx* ctx, void* state) {
  return guard(ctx, [&] {
    if (state) QOB_CUDA(cudaFree(state));
  });
}

int qob_state_upload(qob_ctx* ctx, int dtype, void* state, const void* host, int64_t dim, int64_t ncols,
                     void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !state || (!host && dim * ncols > 0)) fail(QOB_ERR_ARG, "qob_state_upload: bad arguments");
    check_dtype(dtype);
    const size_t bytes = (size_t)dim * ncols * (dtype == QOB_C128 ? 16 : 8);
    QOB_CUDA(cudaMemcpyAsync(state, host, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    QOB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  });
}

int qob_state_download(qob_ctx* ctx, int dtype, const void* state, void* host, int64_t dim, int64_t ncols,
                       void* stream) {
  return guard(ctx, [&] {
    if (!ctx || !state || (!host && dim * ncols > 0)) fail(QOB_ERR_ARG, "qob_state_download: bad arguments");
    check_dtype(dtype);
    const size_t bytes = (size_t)dim * ncols * (dtype == QOB_C128 ? 16 : 8);
    QOB_CUDA(cudaMemcpyAsync(host, state, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    QOB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  });
}

}  // extern "C"
