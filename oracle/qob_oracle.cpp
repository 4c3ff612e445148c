// qob_oracle.cpp -- CPU restatement of QuantumOpticsBase.jl v0.5.13's 5-argument
// mul! for LazySum / LazyTensor / LazyProduct / SparseOperator / DenseOperator.
//
// TEST INFRASTRUCTURE ONLY: the parity checker for the GPU library and the timed
// CPU baseline.  Nothing in the product path links or calls this file.
//
// Every function restates one reference function, cited by file:line within the
// QuantumOpticsBase.jl source tree.  Loop orders follow the reference so that the
// per-element accumulation order is the reference's.  Complex arithmetic is
// written out as Julia's Base does it (no Annex-G NaN recovery) and the file is
// compiled with -ffp-contract=off so no multiply-add is fused.
//
// Dense products go through BLAS in the reference (third-party, unpinned: the
// package has no Manifest).  They are restated here with the loop orders of the
// netlib reference BLAS zgemm/zgemv; the reference's own tests pin dense paths
// only to a tolerance (test/test_operators_dense.jl:354-419), so parity there is
// tolerance-level by construction.
#include "qob_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

struct cd {
  double re, im;
};
inline cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
inline cd cconj(cd a) { return {a.re, -a.im}; }
inline bool iszero(cd a) { return a.re == 0.0 && a.im == 0.0; }
inline bool isone(cd a) { return a.re == 1.0 && a.im == 0.0; }
const cd kOne{1.0, 0.0};
const cd kZero{0.0, 0.0};

enum Kind { K_SPARSE, K_DENSE, K_EYE, K_LT, K_LS, K_LP, K_FFT };

thread_local std::string g_err;

struct Err {
  int code;
};
[[noreturn]] void fail(int code, const std::string& msg) {
  g_err = msg;
  throw Err{code};
}
constexpr int E_DIM = 1, E_ALIAS = 2, E_UNSUP = 3;

}  // namespace

struct oref_node {
  Kind kind;
  int64_t m = 0, n = 0;  // operator shape after adjoint: length(basis_l) x length(basis_r)
  bool adjoint = false;
  // sparse: stored (pre-adjoint) CSC, converted to 0-based
  int64_t sm = 0, sn = 0;
  std::vector<int64_t> colptr, rowval;
  std::vector<cd> nzval;
  // dense: stored sm x sn, column-major
  std::vector<cd> dense;
  // lazy operators
  std::vector<int64_t> shape_l, shape_r, indices;  // indices 1-based
  std::vector<oref_node*> ops;
  cd factor{1.0, 0.0};
  std::vector<cd> factors;
  // FFTOperator: transformed subsystems (0-based), the sign of the transform a
  // ket sees (fft_r!), and the full phase arrays mul_before / mul_after
  std::vector<int> fft_axes;
  int fft_sign = -1;
  std::vector<cd> mul_before, mul_after;
};

namespace {

using Node = oref_node;

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

// _strides (src/operators_dense.jl:296-308): column-major strides of a shape.
std::vector<int64_t> strides_of(const std::vector<int64_t>& shape) {
  std::vector<int64_t> s(shape.size());
  int64_t t = 1;
  for (size_t i = 0; i < shape.size(); ++i) {
    s[i] = t;
    t *= shape[i];
  }
  return s;
}

int64_t prod(const std::vector<int64_t>& v) {
  int64_t p = 1;
  for (auto x : v) p *= x;
  return p;
}

// _zero_op_mul! (src/operators_lazysum.jl:179-186)
void zero_op_mul(cd* y, int64_t len, cd beta) {
  if (iszero(beta)) {
    for (int64_t i = 0; i < len; ++i) y[i] = kZero;
  } else if (!isone(beta)) {
    for (int64_t i = 0; i < len; ++i) y[i] = cmul(y[i], beta);
  }
}

// beta pre-scaling used by _gemm_puresparse (src/operators_lazytensor.jl:719-723,
// 731-735) and gemm!/gemv! (src/sparsematrix.jl:103-107, 194-198).
void prescale(cd* y, int64_t len, cd beta) { zero_op_mul(y, len, beta); }

// Element (i, j) of a leaf data operator, adjoint applied.
cd leaf_at(const Node* f, int64_t i, int64_t j) {
  switch (f->kind) {
    case K_DENSE:
      return f->adjoint ? cconj(f->dense[j + i * f->sm]) : f->dense[i + j * f->sm];
    case K_EYE:
      return (i == j) ? kOne : kZero;
    case K_SPARSE: {
      int64_t r = f->adjoint ? j : i, c = f->adjoint ? i : j;
      for (int64_t p = f->colptr[c]; p < f->colptr[c + 1]; ++p)
        if (f->rowval[p] == r) return f->adjoint ? cconj(f->nzval[p]) : f->nzval[p];
      return kZero;
    }
    default:
      fail(E_UNSUP, "leaf_at on a non-data operator");
  }
}

// A dense column-major copy of a leaf factor, optionally transposed (the
// op_transform of _tpops_tuple, src/operators_lazytensor.jl:523-537).
struct Mat {
  int64_t r, c;
  bool eye;
  std::vector<cd> a;
  cd at(int64_t i, int64_t j) const { return a[i + j * r]; }
};
Mat materialise(const Node* f, bool transpose) {
  Mat M;
  int64_t r = transpose ? f->n : f->m, c = transpose ? f->m : f->n;
  M.r = r;
  M.c = c;
  M.eye = (f->kind == K_EYE);
  M.a.assign(r * c, kZero);
  for (int64_t j = 0; j < c; ++j)
    for (int64_t i = 0; i < r; ++i) M.a[i + j * r] = transpose ? leaf_at(f, j, i) : leaf_at(f, i, j);
  return M;
}

// ---------------------------------------------------------------------------
// forward declarations
// ---------------------------------------------------------------------------
void mul_left(bool vec, const Node* op, cd alpha, const cd* x, int64_t xr, int64_t xc, cd beta,
              cd* y, int64_t yr, int64_t yc);
void mul_right(bool vec, const Node* op, cd alpha, const cd* x, int64_t xr, int64_t xc, cd beta,
               cd* y, int64_t yr, int64_t yc);

// ---------------------------------------------------------------------------
// sparse kernels (src/sparsematrix.jl)
// ---------------------------------------------------------------------------

// gemv!(alpha, M, v, beta, result) (src/sparsematrix.jl:190-214)
void gemv_sp(cd alpha, const Node* M, const cd* v, cd beta, cd* res) {
  prescale(res, M->sm, beta);
  if (isone(alpha)) {
    for (int64_t col = 0; col < M->sn; ++col) {
      cd vj = v[col];
      for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i)
        res[M->rowval[i]] = cadd(res[M->rowval[i]], cmul(M->nzval[i], vj));
    }
  } else {
    for (int64_t col = 0; col < M->sn; ++col) {
      cd vj = cmul(alpha, v[col]);
      for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i)
        res[M->rowval[i]] = cadd(res[M->rowval[i]], cmul(M->nzval[i], vj));
    }
  }
}

// gemv!(alpha, v, M, beta, result) -- bra times sparse (src/sparsematrix.jl:216-238)
void gemv_sp_bra(cd alpha, const cd* v, const Node* M, cd beta, cd* res) {
  prescale(res, M->sn, beta);
  if (isone(alpha)) {
    for (int64_t col = 0; col < M->sn; ++col)
      for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i)
        res[col] = cadd(res[col], cmul(M->nzval[i], v[M->rowval[i]]));
  } else {
    for (int64_t col = 0; col < M->sn; ++col)
      for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i)
        res[col] = cadd(res[col], cmul(cmul(M->nzval[i], alpha), v[M->rowval[i]]));
  }
}

// gemm!(alpha, M::SparseMatrixCSC, B, beta, result) (src/sparsematrix.jl:99-113)
// with gemm_sp_dense_small (:1-23) and gemm_sp_dense_big (:25-47).
void gemm_sp_dense(cd alpha, const Node* M, const cd* B, int64_t bcols, cd beta, cd* R) {
  const int64_t br = M->sn, rr = M->sm;
  prescale(R, rr * bcols, beta);
  int64_t nnz = M->colptr[M->sn];
  if (nnz > 550) {
    for (int64_t j = 0; j < bcols; ++j)
      for (int64_t col = 0; col < M->sn; ++col) {
        cd m2 = isone(alpha) ? B[col + j * br] : cmul(alpha, B[col + j * br]);
        for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i) {
          int64_t row = M->rowval[i];
          R[row + j * rr] = cadd(R[row + j * rr], cmul(M->nzval[i], m2));
        }
      }
  } else {
    for (int64_t col = 0; col < M->sn; ++col)
      for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i) {
        int64_t row = M->rowval[i];
        cd val = isone(alpha) ? M->nzval[i] : cmul(alpha, M->nzval[i]);
        for (int64_t j = 0; j < bcols; ++j)
          R[row + j * rr] = cadd(R[row + j * rr], cmul(val, B[col + j * br]));
      }
  }
}

// gemm!(alpha, B, M::SparseMatrixCSC, beta, result) (src/sparsematrix.jl:115-146)
void gemm_dense_sp(cd alpha, const cd* B, int64_t brows, const Node* M, cd beta, cd* R) {
  prescale(R, brows * M->sn, beta);
  for (int64_t col = 0; col < M->sn; ++col)
    for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i) {
      cd mi = isone(alpha) ? M->nzval[i] : cmul(M->nzval[i], alpha);
      int64_t mrow = M->rowval[i];
      for (int64_t j = 0; j < brows; ++j)
        R[j + col * brows] = cadd(R[j + col * brows], cmul(mi, B[j + mrow * brows]));
    }
}

// gemm_adj_sp_dense_small (src/sparsematrix.jl:73-96), used by
// gemm!(alpha, M', B, beta, result) when nnz <= 550 (:148-163).  For nnz > 550 the
// reference calls SparseArrays' adjoint mul!, restated as a row-dot per output
// row in the same column order.
void gemm_adjsp_dense(cd alpha, const Node* M, const cd* B, int64_t bcols, cd beta, cd* R) {
  // M' is sn x sm; B is sm x bcols; R is sn x bcols
  const int64_t br = M->sm, rr = M->sn;
  int64_t nnz = M->colptr[M->sn];
  if (nnz > 550) {
    for (int64_t j = 0; j < bcols; ++j)
      for (int64_t col = 0; col < M->sn; ++col) {
        cd s = kZero;
        for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i)
          s = cadd(s, cmul(cconj(M->nzval[i]), B[M->rowval[i] + j * br]));
        cd v = cmul(alpha, s);
        R[col + j * rr] = iszero(beta) ? v : cadd(v, cmul(beta, R[col + j * rr]));
      }
    return;
  }
  prescale(R, rr * bcols, beta);
  for (int64_t col = 0; col < M->sn; ++col)
    for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i) {
      cd mi = isone(alpha) ? cconj(M->nzval[i]) : cmul(cconj(M->nzval[i]), alpha);
      int64_t mrow = M->rowval[i];
      for (int64_t j = 0; j < bcols; ++j)
        R[col + j * rr] = cadd(R[col + j * rr], cmul(mi, B[mrow + j * br]));
    }
}

// gemm_dense_adj_sp (src/sparsematrix.jl:49-71) via gemm!(alpha, B, M', ...) (:165-175)
void gemm_dense_adjsp(cd alpha, const cd* B, int64_t brows, const Node* M, cd beta, cd* R) {
  // B is brows x sn ; M' is sn x sm ; R is brows x sm
  prescale(R, brows * M->sm, beta);
  for (int64_t col = 0; col < M->sn; ++col)
    for (int64_t i = M->colptr[col]; i < M->colptr[col + 1]; ++i) {
      int64_t row = M->rowval[i];
      cd val = isone(alpha) ? cconj(M->nzval[i]) : cmul(alpha, cconj(M->nzval[i]));
      for (int64_t j = 0; j < brows; ++j)
        R[j + row * brows] = cadd(R[j + row * brows], cmul(val, B[j + col * brows]));
    }
}

// ---------------------------------------------------------------------------
// dense products: LinearAlgebra.mul! -> BLAS (src/operators_dense.jl:394-396),
// restated with netlib zgemm / zgemv loop orders.
// ---------------------------------------------------------------------------

// C (m x nc) = alpha * op(A) * B + beta * C, with op(A) = leaf operator f (m x k).
void dense_left(const Node* f, cd alpha, const cd* B, int64_t nc, cd beta, cd* C) {
  const int64_t m = f->m, k = f->n;
  for (int64_t j = 0; j < nc; ++j) {
    cd* c = C + j * m;
    if (iszero(beta))
      for (int64_t i = 0; i < m; ++i) c[i] = kZero;
    else if (!isone(beta))
      for (int64_t i = 0; i < m; ++i) c[i] = cmul(beta, c[i]);
    for (int64_t l = 0; l < k; ++l) {
      cd temp = cmul(alpha, B[l + j * k]);
      for (int64_t i = 0; i < m; ++i) c[i] = cadd(c[i], cmul(temp, leaf_at(f, i, l)));
    }
  }
}

// Bra: result = alpha * transpose(A) * x + beta * result (src/operators_dense.jl:396),
// netlib zgemv 'T' order (dot product per output entry).
void dense_bra(const Node* f, cd alpha, const cd* x, cd beta, cd* y) {
  for (int64_t j = 0; j < f->n; ++j) {
    cd temp = kZero;
    for (int64_t i = 0; i < f->m; ++i) temp = cadd(temp, cmul(leaf_at(f, i, j), x[i]));
    cd v = cmul(alpha, temp);
    y[j] = iszero(beta) ? v : cadd(cmul(beta, y[j]), v);
  }
}

// C (r x n) = alpha * X (r x m) * A (m x n) + beta * C, netlib zgemm order.
void dense_right(const Node* f, cd alpha, const cd* X, int64_t r, cd beta, cd* C) {
  const int64_t m = f->m, n = f->n;
  for (int64_t j = 0; j < n; ++j) {
    cd* c = C + j * r;
    if (iszero(beta))
      for (int64_t i = 0; i < r; ++i) c[i] = kZero;
    else if (!isone(beta))
      for (int64_t i = 0; i < r; ++i) c[i] = cmul(beta, c[i]);
    for (int64_t l = 0; l < m; ++l) {
      cd temp = cmul(alpha, leaf_at(f, l, j));
      for (int64_t i = 0; i < r; ++i) c[i] = cadd(c[i], cmul(temp, X[i + l * r]));
    }
  }
}

// ---------------------------------------------------------------------------
// LazyTensor
// ---------------------------------------------------------------------------

// _is_pure_sparse (src/operators_lazytensor.jl:520)
bool is_pure_sparse(const Node* h) {
  if (h->ops.empty()) return false;
  for (auto* o : h->ops)
    if (!((o->kind == K_SPARSE && !o->adjoint) || o->kind == K_EYE)) return false;
  return true;
}

const Node* suboperator(const Node* h, int64_t site1) {
  for (size_t i = 0; i < h->indices.size(); ++i)
    if (h->indices[i] == site1) return h->ops[i];
  return nullptr;
}

struct Rec {
  const Node* h;
  std::vector<int64_t> shape, sk, sj;
  std::vector<const Node*> fac;  // per site, nullptr if none
  const cd* op;
  cd* res;
  int64_t ncols, op_ld, res_ld;
};

// _gemm_recursive_lazy_dense (src/operators_lazytensor.jl:652-685):
// result[J, I] += val * op[K, I]; K walks the input (basis_r) strides, J the
// output (basis_l) strides.
void rec_lazy_dense(const Rec& R, size_t ik, int64_t K, int64_t J, cd val) {
  if (ik == R.shape.size()) {
    for (int64_t I = 0; I < R.ncols; ++I)
      R.res[J + I * R.res_ld] = cadd(R.res[J + I * R.res_ld], cmul(val, R.op[K + I * R.op_ld]));
    return;
  }
  const Node* f = R.fac[ik];
  if (f && f->kind == K_SPARSE) {
    for (int64_t k = 0; k < f->sn; ++k) {
      int64_t K_ = K + R.sk[ik] * k;
      for (int64_t p = f->colptr[k]; p < f->colptr[k + 1]; ++p) {
        int64_t j = f->rowval[p];
        int64_t J_ = J + R.sj[ik] * j;
        rec_lazy_dense(R, ik + 1, K_, J_, cmul(val, f->nzval[p]));
      }
    }
    return;
  }
  for (int64_t k = 0; k < R.shape[ik]; ++k)
    rec_lazy_dense(R, ik + 1, K + R.sk[ik] * k, J + R.sj[ik] * k, val);
}

// _gemm_recursive_dense_lazy (src/operators_lazytensor.jl:613-648):
// result[I, K] += val * op[I, J] (bra / operator from the right).
void rec_dense_lazy(const Rec& R, size_t ik, int64_t K, int64_t J, cd val) {
  if (ik == R.shape.size()) {
    // rows I of the left operand are the batch; op_ld/res_ld are their strides
    for (int64_t I = 0; I < R.ncols; ++I)
      R.res[I + K * R.res_ld] = cadd(R.res[I + K * R.res_ld], cmul(val, R.op[I + J * R.op_ld]));
    return;
  }
  const Node* f = R.fac[ik];
  if (f && f->kind == K_SPARSE) {
    for (int64_t k = 0; k < f->sn; ++k) {
      int64_t K_ = K + R.sk[ik] * k;
      for (int64_t p = f->colptr[k]; p < f->colptr[k + 1]; ++p) {
        int64_t j = f->rowval[p];
        int64_t J_ = J + R.sj[ik] * j;
        rec_dense_lazy(R, ik + 1, K_, J_, cmul(val, f->nzval[p]));
      }
    }
    return;
  }
  for (int64_t k = 0; k < R.shape[ik]; ++k)
    rec_dense_lazy(R, ik + 1, K + R.sk[ik] * k, J + R.sj[ik] * k, val);
}

// _get_shape_and_strides (src/operators_lazytensor.jl:741-746)
void shape_and_strides(const Node* h, Rec& R) {
  const size_t N = h->shape_l.size();
  R.shape.resize(N);
  for (size_t i = 0; i < N; ++i) R.shape[i] = std::min(h->shape_l[i], h->shape_r[i]);
  R.sj = strides_of(h->shape_l);
  R.sk = strides_of(h->shape_r);
  R.fac.assign(N, nullptr);
  for (size_t i = 0; i < N; ++i) R.fac[i] = suboperator(h, (int64_t)i + 1);
}

// _gemm_puresparse(alpha, h, op, beta, result) (src/operators_lazytensor.jl:729-739)
void puresparse_left(const Node* h, cd alpha, const cd* x, int64_t ncols, cd beta, cd* y) {
  if (x == y) fail(E_ALIAS, "output matrix must not be aliased with input matrix");
  prescale(y, h->m * ncols, beta);
  Rec R;
  R.h = h;
  shape_and_strides(h, R);
  R.op = x;
  R.res = y;
  R.ncols = ncols;
  R.op_ld = h->n;
  R.res_ld = h->m;
  rec_lazy_dense(R, 0, 0, 0, cmul(alpha, h->factor));
}

// _gemm_puresparse(alpha, op, h, beta, result) (src/operators_lazytensor.jl:711-727)
void puresparse_right(const Node* h, cd alpha, const cd* x, int64_t nrows, cd beta, cd* y) {
  if (x == y) fail(E_ALIAS, "output matrix must not be aliased with input matrix");
  prescale(y, nrows * h->n, beta);
  Rec R;
  R.h = h;
  shape_and_strides(h, R);
  // For the right product the roles of the strides are as in the reference call
  // _gemm_recursive_dense_lazy(1, N, 1, 1, alpha*h.factor, shape, strides_k, strides_j, ...)
  // with strides_j = strides(shape_l) (the input, basis_l side) and
  // strides_k = strides(shape_r) (the output, basis_r side).
  R.op = x;
  R.res = y;
  R.ncols = nrows;
  R.op_ld = nrows;
  R.res_ld = nrows;
  rec_dense_lazy(R, 0, 0, 0, cmul(alpha, h->factor));
}

// One mode product of _tp_matmul! (src/operators_lazytensor.jl:406-428):
// result = alpha * A (applied to mode loc of b) + beta * result, with the
// non-square Eye branch of _tp_matmul_mid! (:348-371).  First/last/middle
// positions only differ in how the reference lays the GEMM out in memory; the
// arithmetic per element is the same dot product.
void tp_matmul(cd* res, const std::vector<int64_t>& shape_res, const Mat& A, size_t loc,
               const cd* b, const std::vector<int64_t>& shape_b, cd alpha, cd beta) {
  int64_t s1 = 1, s3 = 1;
  for (size_t i = 0; i < loc; ++i) s1 *= shape_b[i];
  for (size_t i = loc + 1; i < shape_b.size(); ++i) s3 *= shape_b[i];
  const int64_t din = shape_b[loc], dout = shape_res[loc];
  if (A.r != dout || A.c != din) fail(E_DIM, "Dimensions of factor do not match subspace dimensions.");
  if (A.eye) {
    const int64_t len = s1 * dout * s3;
    if (iszero(beta)) {
      for (int64_t i = 0; i < len; ++i) res[i] = kZero;
    } else {
      for (int64_t i = 0; i < len; ++i) res[i] = cmul(res[i], beta);
    }
    const int64_t d = std::min(A.r, A.c);
    for (int64_t c3 = 0; c3 < s3; ++c3)
      for (int64_t j = 0; j < d; ++j)
        for (int64_t c1 = 0; c1 < s1; ++c1) {
          int64_t ir = c1 + s1 * (j + dout * c3), ib = c1 + s1 * (j + din * c3);
          res[ir] = cadd(res[ir], cmul(alpha, b[ib]));
        }
    return;
  }
  for (int64_t c3 = 0; c3 < s3; ++c3)
    for (int64_t j = 0; j < dout; ++j)
      for (int64_t c1 = 0; c1 < s1; ++c1) {
        cd s = kZero;
        for (int64_t k = 0; k < din; ++k) s = cadd(s, cmul(A.at(j, k), b[c1 + s1 * (k + din * c3)]));
        int64_t ir = c1 + s1 * (j + dout * c3);
        cd v = cmul(alpha, s);
        res[ir] = iszero(beta) ? v : cadd(v, cmul(beta, res[ir]));
      }
}

struct TpOp {
  Mat A;
  size_t loc;
};

// _tpops_tuple + _explicit_isometries (src/operators_lazytensor.jl:491-537).
// transpose selects the Bra / right-product form.
std::vector<TpOp> tp_ops(const Node* h, bool transpose) {
  std::vector<TpOp> ops;
  for (size_t i = 0; i < h->ops.size(); ++i) {
    const Node* f = h->ops[i];
    if (f->kind == K_EYE && f->m == f->n) continue;  // _is_square_eye filter
    ops.push_back({materialise(f, transpose), (size_t)(h->indices[i] - 1)});
  }
  const auto& sl = transpose ? h->shape_r : h->shape_l;  // output side
  const auto& sr = transpose ? h->shape_l : h->shape_r;  // input side
  if (sl != sr) {
    for (size_t i = 0; i < sl.size(); ++i) {
      bool used = false;
      for (auto idx : h->indices) used |= (idx - 1 == (int64_t)i);
      if (sl[i] != sr[i] && !used) {
        Mat E;
        E.r = sl[i];
        E.c = sr[i];
        E.eye = true;
        ops.push_back({E, i});
      }
    }
  }
  return ops;
}

// _tp_sum_matmul! (src/operators_lazytensor.jl:443-488) for one vector.
void tp_sum_matmul_vec(const std::vector<TpOp>& ops, const std::vector<int64_t>& shape_out,
                       const std::vector<int64_t>& shape_in, cd* res, const cd* b, cd alpha,
                       cd beta) {
  const size_t n_ops = ops.size();
  const int64_t len_out = prod(shape_out);
  if (n_ops == 0) {
    for (int64_t i = 0; i < len_out; ++i) {
      cd v = cmul(alpha, b[i]);
      res[i] = iszero(beta) ? v : cadd(v, cmul(beta, res[i]));
    }
    return;
  }
  if (n_ops == 1) {
    tp_matmul(res, shape_out, ops[0].A, ops[0].loc, b, shape_in, alpha, beta);
    return;
  }
  std::vector<int64_t> sh1 = shape_in;
  sh1[ops[0].loc] = ops[0].A.r;
  std::vector<cd> tmp1(prod(sh1));
  tp_matmul(tmp1.data(), sh1, ops[0].A, ops[0].loc, b, shape_in, alpha, kZero);
  for (size_t i = 1; i + 1 < n_ops; ++i) {
    std::vector<int64_t> sh2 = sh1;
    sh2[ops[i].loc] = ops[i].A.r;
    std::vector<cd> tmp2(prod(sh2));
    tp_matmul(tmp2.data(), sh2, ops[i].A, ops[i].loc, tmp1.data(), sh1, kOne, kZero);
    tmp1.swap(tmp2);
    sh1 = sh2;
  }
  tp_matmul(res, shape_out, ops[n_ops - 1].A, ops[n_ops - 1].loc, tmp1.data(), sh1, kOne, beta);
}

// mul!(::Ket, ::LazyTensor, ::Ket) and mul!(::DenseOpType, ::LazyTensor, ::DenseOpType)
// (src/operators_lazytensor.jl:539-557, 576-591)
void lazytensor_left(const Node* h, cd alpha, const cd* x, int64_t ncols, cd beta, cd* y) {
  if (iszero(alpha)) {
    zero_op_mul(y, h->m * ncols, beta);
    return;
  }
  if (is_pure_sparse(h)) {
    puresparse_left(h, alpha, x, ncols, beta, y);
    return;
  }
  auto ops = tp_ops(h, false);
  cd a = cmul(alpha, h->factor);
  for (int64_t c = 0; c < ncols; ++c)
    tp_sum_matmul_vec(ops, h->shape_l, h->shape_r, y + c * h->m, x + c * h->n, a, beta);
}

// mul!(::Bra, ::Bra, ::LazyTensor) and mul!(::DenseOpType, ::DenseOpType, ::LazyTensor)
// (src/operators_lazytensor.jl:559-574, 593-609).  Each row of the left operand
// is one bra.
void lazytensor_right(const Node* h, cd alpha, const cd* x, int64_t nrows, cd beta, cd* y) {
  if (iszero(alpha)) {
    zero_op_mul(y, nrows * h->n, beta);
    return;
  }
  if (is_pure_sparse(h)) {
    puresparse_right(h, alpha, x, nrows, beta, y);
    return;
  }
  auto ops = tp_ops(h, true);
  cd a = cmul(alpha, h->factor);
  std::vector<cd> xin(h->m), yout(h->n);
  for (int64_t r = 0; r < nrows; ++r) {
    for (int64_t j = 0; j < h->m; ++j) xin[j] = x[r + j * nrows];
    for (int64_t j = 0; j < h->n; ++j) yout[j] = y[r + j * nrows];
    tp_sum_matmul_vec(ops, h->shape_r, h->shape_l, yout.data(), xin.data(), a, beta);
    for (int64_t j = 0; j < h->n; ++j) y[r + j * nrows] = yout[j];
  }
}

// ---------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------

void eye_left(const Node* f, cd alpha, const cd* x, int64_t nc, cd beta, cd* y) {
  const int64_t d = std::min(f->m, f->n);
  for (int64_t c = 0; c < nc; ++c)
    for (int64_t i = 0; i < f->m; ++i) {
      cd v = (i < d) ? cmul(alpha, x[i + c * f->n]) : kZero;
      cd& o = y[i + c * f->m];
      o = iszero(beta) ? v : cadd(v, cmul(beta, o));
    }
}
void eye_right(const Node* f, cd alpha, const cd* x, int64_t nr, cd beta, cd* y) {
  const int64_t d = std::min(f->m, f->n);
  for (int64_t j = 0; j < f->n; ++j)
    for (int64_t r = 0; r < nr; ++r) {
      cd v = (j < d) ? cmul(alpha, x[r + j * nr]) : kZero;
      cd& o = y[r + j * nr];
      o = iszero(beta) ? v : cadd(v, cmul(beta, o));
    }
}

// ---------------------------------------------------------------------------
// FFTOperator (src/particle.jl:438-535).  FFTW's fft!/bfft! over a set of
// dimensions compute the unnormalised multi-dimensional DFT
// X_k = sum_j x_j exp(sign 2 pi i j.k / N) (sign -1: fft, +1: bfft); restated
// here as direct sums, one dimension after the other (the DFT is separable).
// ---------------------------------------------------------------------------

// In-place DFT along dimension `dim` of an array of shape `shape` (column-major).
void dft_dim(cd* a, const std::vector<int64_t>& shape, size_t dim, int sign) {
  const int64_t n = shape[dim];
  int64_t inner = 1, outer = 1;
  for (size_t q = 0; q < dim; ++q) inner *= shape[q];
  for (size_t q = dim + 1; q < shape.size(); ++q) outer *= shape[q];
  std::vector<cd> w(n), line(n);
  for (int64_t m = 0; m < n; ++m) {
    const double th = 6.283185307179586476925286766559 * (double)m / (double)n;
    w[m] = {std::cos(th), sign * std::sin(th)};
  }
  for (int64_t o = 0; o < outer; ++o)
    for (int64_t i = 0; i < inner; ++i) {
      cd* base = a + i + o * inner * n;
      for (int64_t j = 0; j < n; ++j) line[j] = base[j * inner];
      for (int64_t k = 0; k < n; ++k) {
        cd acc = kZero;
        int64_t idx = 0;
        for (int64_t j = 0; j < n; ++j) {
          acc = cadd(acc, cmul(line[j], w[idx]));
          idx += k;
          if (idx >= n) idx -= n;
        }
        base[k * inner] = acc;
      }
    }
}

// fft over the transformed dimensions of an array whose leading (or trailing)
// dimensions are the operator's composite shape.
void fft_dims(const Node* f, cd* a, const std::vector<int64_t>& shape, size_t offset, int sign) {
  for (int ax : f->fft_axes) dft_dim(a, shape, offset + ax, sign);
}

// Ket (vec) and Operator (columns) from the left: :438-457, :504-535
void fft_left(bool vec, const Node* f, cd alpha, const cd* x, int64_t xc, cd beta, cd* y) {
  const int64_t N = f->m;
  const std::vector<int64_t>& sh = f->shape_l;
  if (vec) {
    if (iszero(beta)) {
      for (int64_t i = 0; i < N; ++i) y[i] = cmul(f->mul_before[i], x[i]);
      fft_dims(f, y, sh, 0, f->fft_sign);
      for (int64_t i = 0; i < N; ++i) y[i] = cmul(y[i], cmul(f->mul_after[i], alpha));
    } else {
      std::vector<cd> p(x, x + N);
      for (int64_t i = 0; i < N; ++i) p[i] = cmul(p[i], f->mul_before[i]);
      fft_dims(f, p.data(), sh, 0, f->fft_sign);
      for (int64_t i = 0; i < N; ++i) y[i] = cadd(cmul(beta, y[i]), cmul(cmul(alpha, p[i]), f->mul_after[i]));
    }
    return;
  }
  std::vector<cd> d(x, x + N * xc);
  for (int64_t j = 0; j < xc; ++j)
    for (int64_t i = 0; i < N; ++i) d[i + j * N] = cmul(d[i + j * N], f->mul_before[i]);
  std::vector<int64_t> sh2 = sh;
  sh2.push_back(xc);
  fft_dims(f, d.data(), sh2, 0, f->fft_sign);
  for (int64_t j = 0; j < xc; ++j)
    for (int64_t i = 0; i < N; ++i) d[i + j * N] = cmul(d[i + j * N], f->mul_after[i]);
  if (!isone(alpha))
    for (cd& v : d) v = cmul(alpha, v);
  if (iszero(beta)) {
    std::copy(d.begin(), d.end(), y);
  } else {
    for (int64_t k = 0; k < N * xc; ++k) y[k] = cadd(cmul(y[k], beta), d[k]);
  }
}

// Bra (vec) and Operator (rows) from the right: :459-478, :481-502
void fft_right(bool vec, const Node* f, cd alpha, const cd* x, int64_t xr, cd beta, cd* y) {
  const int64_t N = f->m;
  const std::vector<int64_t>& sh = f->shape_l;
  if (vec) {
    if (iszero(beta)) {
      for (int64_t i = 0; i < N; ++i) y[i] = cmul(cconj(f->mul_after[i]), cconj(x[i]));
      fft_dims(f, y, sh, 0, -f->fft_sign);
      for (int64_t i = 0; i < N; ++i) y[i] = cmul(cmul(cconj(y[i]), f->mul_before[i]), alpha);
    } else {
      std::vector<cd> p(N);
      for (int64_t i = 0; i < N; ++i) p[i] = cmul(cconj(x[i]), cconj(f->mul_after[i]));
      fft_dims(f, p.data(), sh, 0, -f->fft_sign);
      for (int64_t i = 0; i < N; ++i)
        y[i] = cadd(cmul(beta, y[i]), cmul(cmul(alpha, cconj(p[i])), f->mul_before[i]));
    }
    return;
  }
  std::vector<cd> d(x, x + xr * N);
  for (int64_t j = 0; j < N; ++j)
    for (int64_t i = 0; i < xr; ++i) d[i + j * xr] = cconj(cmul(d[i + j * xr], f->mul_after[j]));
  std::vector<int64_t> sh2{xr};
  sh2.insert(sh2.end(), sh.begin(), sh.end());
  fft_dims(f, d.data(), sh2, 1, -f->fft_sign);
  for (int64_t j = 0; j < N; ++j)
    for (int64_t i = 0; i < xr; ++i) d[i + j * xr] = cmul(cconj(d[i + j * xr]), f->mul_before[j]);
  if (!isone(alpha))
    for (cd& v : d) v = cmul(alpha, v);
  if (iszero(beta)) {
    std::copy(d.begin(), d.end(), y);
  } else {
    for (int64_t k = 0; k < xr * N; ++k) y[k] = cadd(cmul(y[k], beta), d[k]);
  }
}

void mul_left(bool vec, const Node* op, cd alpha, const cd* x, int64_t xr, int64_t xc, cd beta,
              cd* y, int64_t yr, int64_t yc) {
  // _check_mul!_dim_compatibility (src/operators_lazytensor.jl:695-703)
  if (op->n != xr) fail(E_DIM, "A and B dimensions do not match. Can't do `A*B`");
  if (op->m != yr || xc != yc) fail(E_DIM, "Output dimensions do not match A*B. Can't do `R.=A*B`");
  switch (op->kind) {
    case K_LS: {  // src/operators_lazysum.jl:189-200, 215-226
      if (op->ops.empty() || iszero(alpha)) {
        zero_op_mul(y, yr * yc, beta);
        return;
      }
      mul_left(vec, op->ops[0], cmul(alpha, op->factors[0]), x, xr, xc, beta, y, yr, yc);
      for (size_t i = 1; i < op->ops.size(); ++i)
        mul_left(vec, op->ops[i], cmul(alpha, op->factors[i]), x, xr, xc, kOne, y, yr, yc);
      return;
    }
    case K_LT:
      lazytensor_left(op, alpha, x, xc, beta, y);
      return;
    case K_FFT:
      fft_left(vec, op, alpha, x, xc, beta, y);
      return;
    case K_LP: {  // src/operators_lazyproduct.jl:103-115, 131-146
      if (iszero(alpha)) {
        zero_op_mul(y, yr * yc, beta);
        return;
      }
      const size_t n = op->ops.size();
      if (n == 1) {
        mul_left(vec, op->ops[0], cmul(op->factor, alpha), x, xr, xc, beta, y, yr, yc);
        return;
      }
      // ket_l[i] lives in operators[i+1].basis_l (0-based i = 0 .. n-2)
      std::vector<std::vector<cd>> kl(n - 1);
      for (size_t i = 0; i + 1 < n; ++i) kl[i].assign(op->ops[i + 1]->m * xc, kZero);
      mul_left(vec, op->ops[n - 1], op->factor, x, xr, xc, kZero, kl[n - 2].data(), op->ops[n - 1]->m, xc);
      for (int64_t i = (int64_t)n - 3; i >= 0; --i)
        mul_left(vec, op->ops[i + 1], kOne, kl[i + 1].data(), op->ops[i + 2]->m, xc, kZero,
                 kl[i].data(), op->ops[i + 1]->m, xc);
      mul_left(vec, op->ops[0], alpha, kl[0].data(), op->ops[1]->m, xc, beta, y, yr, yc);
      return;
    }
    case K_SPARSE:
      if (!op->adjoint) {
        if (vec)  // src/operators_sparse.jl:201 -> gemv!
          gemv_sp(alpha, op, x, beta, y);
        else  // src/operators_sparse.jl:199 -> gemm!
          gemm_sp_dense(alpha, op, x, xc, beta, y);
      } else {
        // Ket: LinearAlgebra.mul! on an Adjoint{SparseMatrixCSC}; Operator:
        // gemm!(alpha, M', B, ...) (src/sparsematrix.jl:148-163).  Both are the
        // adjoint product restated by gemm_adjsp_dense.
        gemm_adjsp_dense(alpha, op, x, xc, beta, y);
      }
      return;
    case K_DENSE:
      dense_left(op, alpha, x, xc, beta, y);
      return;
    case K_EYE:
      eye_left(op, alpha, x, xc, beta, y);
      return;
  }
}

void mul_right(bool vec, const Node* op, cd alpha, const cd* x, int64_t xr, int64_t xc, cd beta,
               cd* y, int64_t yr, int64_t yc) {
  if (op->m != xc) fail(E_DIM, "A and B dimensions do not match. Can't do `A*B`");
  if (op->n != yc || xr != yr) fail(E_DIM, "Output dimensions do not match A*B. Can't do `R.=A*B`");
  switch (op->kind) {
    case K_LS: {  // src/operators_lazysum.jl:202-213, 227-238
      if (op->ops.empty() || iszero(alpha)) {
        zero_op_mul(y, yr * yc, beta);
        return;
      }
      mul_right(vec, op->ops[0], cmul(alpha, op->factors[0]), x, xr, xc, beta, y, yr, yc);
      for (size_t i = 1; i < op->ops.size(); ++i)
        mul_right(vec, op->ops[i], cmul(alpha, op->factors[i]), x, xr, xc, kOne, y, yr, yc);
      return;
    }
    case K_LT:
      lazytensor_right(op, alpha, x, xr, beta, y);
      return;
    case K_FFT:
      fft_right(vec, op, alpha, x, xr, beta, y);
      return;
    case K_LP: {  // src/operators_lazyproduct.jl:117-129, 148-163
      if (iszero(alpha)) {
        zero_op_mul(y, yr * yc, beta);
        return;
      }
      const size_t n = op->ops.size();
      if (n == 1) {
        mul_right(vec, op->ops[0], cmul(op->factor, alpha), x, xr, xc, beta, y, yr, yc);
        return;
      }
      // bra_r[i] lives in operators[i].basis_r (0-based i = 0 .. n-2)
      std::vector<std::vector<cd>> br(n - 1);
      for (size_t i = 0; i + 1 < n; ++i) br[i].assign(xr * op->ops[i]->n, kZero);
      mul_right(vec, op->ops[0], op->factor, x, xr, xc, kZero, br[0].data(), xr, op->ops[0]->n);
      for (size_t i = 1; i + 1 < n; ++i)
        mul_right(vec, op->ops[i], kOne, br[i - 1].data(), xr, op->ops[i - 1]->n, kZero,
                  br[i].data(), xr, op->ops[i]->n);
      mul_right(vec, op->ops[n - 1], alpha, br[n - 2].data(), xr, op->ops[n - 2]->n, beta, y, yr, yc);
      return;
    }
    case K_SPARSE:
      if (!op->adjoint) {
        if (vec)  // src/operators_sparse.jl:202 -> gemv! (bra)
          gemv_sp_bra(alpha, x, op, beta, y);
        else  // src/operators_sparse.jl:200 -> gemm!(alpha, B, M, ...)
          gemm_dense_sp(alpha, x, xr, op, beta, y);
      } else {
        if (vec) {
          // Bra times adjoint sparse: LinearAlgebra.mul!(result, transpose(M'), a)
          // (src/operators_dense.jl:396): result[i] = sum_j conj(M[i, j]) a[j].
          std::vector<cd> acc(op->n, kZero);
          for (int64_t col = 0; col < op->sn; ++col)
            for (int64_t p = op->colptr[col]; p < op->colptr[col + 1]; ++p) {
              int64_t row = op->rowval[p];
              acc[row] = cadd(acc[row], cmul(cconj(op->nzval[p]), x[col]));
            }
          for (int64_t i = 0; i < op->n; ++i) {
            cd v = cmul(alpha, acc[i]);
            y[i] = iszero(beta) ? v : cadd(cmul(beta, y[i]), v);
          }
        } else {
          gemm_dense_adjsp(alpha, x, xr, op, beta, y);
        }
      }
      return;
    case K_DENSE:
      if (vec)
        dense_bra(op, alpha, x, beta, y);
      else
        dense_right(op, alpha, x, xr, beta, y);
      return;
    case K_EYE:
      eye_right(op, alpha, x, xr, beta, y);
      return;
  }
}

// ---------------------------------------------------------------------------
// product states (src/states_lazyket.jl)
// ---------------------------------------------------------------------------

// LinearAlgebra's dot(x, A, y) for a data operator (src/operators_dense.jl:219-221):
// column by column, s += (sum_i conj(x_i) A_ij) * y_j.
cd dot3(const cd* x, const Node* A, const cd* y, int64_t d) {
  cd s = kZero;
  for (int64_t j = 0; j < d; ++j) {
    if (iszero(y[j])) continue;
    cd t = kZero;
    for (int64_t i = 0; i < d; ++i) t = cadd(t, cmul(cconj(x[i]), leaf_at(A, i, j)));
    s = cadd(s, cmul(t, y[j]));
  }
  return s;
}

cd dotc(const std::vector<cd>& a, const std::vector<cd>& b) {
  cd s = kZero;
  for (size_t i = 0; i < a.size(); ++i) s = cadd(s, cmul(cconj(a[i]), b[i]));
  return s;
}

bool is_leaf(const Node* f) { return f->kind == K_SPARSE || f->kind == K_DENSE || f->kind == K_EYE; }

// mul!(y::LazyKet, op::LazyTensor, x::LazyKet, alpha, 0) (src/states_lazyket.jl:131-150)
void lazyket_mul(const Node* op, cd alpha, const std::vector<std::vector<cd>>& x,
                 std::vector<std::vector<cd>>& y) {
  if (op->kind != K_LT) fail(E_UNSUP, "mul! on a LazyKet needs a LazyTensor");
  for (size_t i = 0; i < x.size(); ++i) {
    int fi = -1;
    for (size_t q = 0; q < op->indices.size(); ++q)
      if (op->indices[q] == (int64_t)i + 1) fi = (int)q;
    if (fi >= 0) {
      const Node* f = op->ops[fi];
      if (!is_leaf(f)) fail(E_UNSUP, "LazyKet factors must be data operators");
      mul_left(true, f, kOne, x[i].data(), (int64_t)x[i].size(), 1, kZero, y[i].data(), (int64_t)y[i].size(), 1);
    } else {
      y[i] = x[i];
    }
  }
  const cd s = cmul(op->factor, alpha);
  for (cd& v : y[0]) v = cmul(v, s);
}

cd expect_lazyket(const Node* op, const std::vector<std::vector<cd>>& kets) {
  switch (op->kind) {
    case K_LT: {  // :64-84
      cd e = op->factor;
      for (size_t i = 0; i < op->ops.size(); ++i) {
        const Node* f = op->ops[i];
        if (!is_leaf(f)) fail(E_UNSUP, "LazyKet factors must be data operators");
        const auto& k = kets[op->indices[i] - 1];
        e = cmul(e, dot3(k.data(), f, k.data(), (int64_t)k.size()));
      }
      for (size_t i = 0; i < kets.size(); ++i) {
        bool in = false;
        for (int64_t q : op->indices) in |= (q == (int64_t)i + 1);
        if (!in) e = cmul(e, dotc(kets[i], kets[i]));
      }
      return e;
    }
    case K_LP: {  // :86-107
      std::vector<std::vector<cd>> t1 = kets, t2 = kets;
      for (int64_t i = (int64_t)op->ops.size() - 1; i >= 0; --i) {
        lazyket_mul(op->ops[i], kOne, t1, t2);
        t1 = t2;
      }
      cd e = op->factor;
      for (size_t j = 0; j < kets.size(); ++j) e = cmul(e, dotc(kets[j], t2[j]));
      return e;
    }
    case K_LS: {  // :109-120
      cd e = kZero;
      for (size_t k = 0; k < op->ops.size(); ++k) e = cadd(e, cmul(op->factors[k], expect_lazyket(op->ops[k], kets)));
      return e;
    }
    default:
      fail(E_UNSUP, "expect on a LazyKet needs a LazyTensor, LazySum or LazyProduct");
  }
  return kZero;
}

template <class F>
int guarded(F&& f) {
  try {
    f();
    return 0;
  } catch (const Err& e) {
    return e.code;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 4;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

oref_node* oref_sparse(int64_t m, int64_t n, const int64_t* colptr, const int64_t* rowval,
                       const double* nzval, int adjoint) {
  auto* f = new Node;
  f->kind = K_SPARSE;
  f->sm = m;
  f->sn = n;
  f->adjoint = adjoint != 0;
  f->m = f->adjoint ? n : m;
  f->n = f->adjoint ? m : n;
  f->colptr.resize(n + 1);
  for (int64_t i = 0; i <= n; ++i) f->colptr[i] = colptr[i] - 1;
  int64_t nnz = f->colptr[n];
  f->rowval.resize(nnz);
  f->nzval.resize(nnz);
  for (int64_t i = 0; i < nnz; ++i) {
    f->rowval[i] = rowval[i] - 1;
    f->nzval[i] = {nzval[2 * i], nzval[2 * i + 1]};
  }
  return f;
}

oref_node* oref_dense(int64_t m, int64_t n, const double* data, int adjoint) {
  auto* f = new Node;
  f->kind = K_DENSE;
  f->sm = m;
  f->sn = n;
  f->adjoint = adjoint != 0;
  f->m = f->adjoint ? n : m;
  f->n = f->adjoint ? m : n;
  f->dense.resize(m * n);
  for (int64_t i = 0; i < m * n; ++i) f->dense[i] = {data[2 * i], data[2 * i + 1]};
  return f;
}

oref_node* oref_eye(int64_t m, int64_t n) {
  auto* f = new Node;
  f->kind = K_EYE;
  f->sm = f->m = m;
  f->sn = f->n = n;
  return f;
}

oref_node* oref_lazytensor(int nsub, const int64_t* shape_l, const int64_t* shape_r, int nfac,
                           const int64_t* indices, oref_node* const* factors, double factor_re,
                           double factor_im) {
  auto* h = new Node;
  h->kind = K_LT;
  h->shape_l.assign(shape_l, shape_l + nsub);
  h->shape_r.assign(shape_r, shape_r + nsub);
  h->indices.assign(indices, indices + nfac);
  h->ops.assign(factors, factors + nfac);
  h->factor = {factor_re, factor_im};
  h->m = prod(h->shape_l);
  h->n = prod(h->shape_r);
  return h;
}

oref_node* oref_lazysum(int64_t m, int64_t n, int nterms, const double* factors,
                        oref_node* const* ops) {
  auto* s = new Node;
  s->kind = K_LS;
  s->m = m;
  s->n = n;
  s->ops.assign(ops, ops + nterms);
  for (int i = 0; i < nterms; ++i) s->factors.push_back({factors[2 * i], factors[2 * i + 1]});
  return s;
}

oref_node* oref_lazyproduct(int nops, oref_node* const* ops, double factor_re, double factor_im) {
  auto* p = new Node;
  p->kind = K_LP;
  p->ops.assign(ops, ops + nops);
  p->factor = {factor_re, factor_im};
  p->m = ops[0]->m;
  p->n = ops[nops - 1]->n;
  return p;
}

oref_node* oref_fft(int nsub, const int64_t* shape, int naxes, const int64_t* axes, int sign,
                    const double* mul_before, const double* mul_after) {
  auto* p = new Node;
  p->kind = K_FFT;
  p->shape_l.assign(shape, shape + nsub);
  p->shape_r = p->shape_l;
  p->m = p->n = prod(p->shape_l);
  for (int a = 0; a < naxes; ++a) p->fft_axes.push_back((int)axes[a] - 1);
  p->fft_sign = sign < 0 ? -1 : 1;
  for (int64_t k = 0; k < p->m; ++k) {
    p->mul_before.push_back({mul_before[2 * k], mul_before[2 * k + 1]});
    p->mul_after.push_back({mul_after[2 * k], mul_after[2 * k + 1]});
  }
  return p;
}

int oref_lazysum_set_factors(oref_node* s, const double* factors) {
  if (s->kind != K_LS) return E_UNSUP;
  for (size_t i = 0; i < s->factors.size(); ++i) s->factors[i] = {factors[2 * i], factors[2 * i + 1]};
  return 0;
}

void oref_free(oref_node* node) { delete node; }
int64_t oref_rows(const oref_node* node) { return node->m; }
int64_t oref_cols(const oref_node* node) { return node->n; }

int oref_mul(int side, int is_vector, const oref_node* op, double alpha_re, double alpha_im,
             const double* x, int64_t x_rows, int64_t x_cols, double beta_re, double beta_im,
             double* y, int64_t y_rows, int64_t y_cols) {
  return guarded([&] {
    const cd* xc = reinterpret_cast<const cd*>(x);
    cd* yc = reinterpret_cast<cd*>(y);
    if (side == 0)
      mul_left(is_vector != 0, op, {alpha_re, alpha_im}, xc, x_rows, x_cols, {beta_re, beta_im}, yc,
               y_rows, y_cols);
    else
      mul_right(is_vector != 0, op, {alpha_re, alpha_im}, xc, x_rows, x_cols, {beta_re, beta_im},
                yc, y_rows, y_cols);
  });
}

int oref_mul_kets_threaded(const oref_node* op, double alpha_re, double alpha_im, const double* x,
                           double beta_re, double beta_im, double* y, int64_t nvec, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  std::vector<int> rc(nthreads, 0);
  std::vector<std::string> errs(nthreads);
  auto work = [&](int t) {
    for (int64_t v = t; v < nvec; v += nthreads) {
      int r = oref_mul(0, 1, op, alpha_re, alpha_im, x + 2 * v * op->n, op->n, 1, beta_re, beta_im,
                       y + 2 * v * op->m, op->m, 1);
      if (r) {
        rc[t] = r;
        errs[t] = g_err;
        return;
      }
    }
  };
  if (nthreads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
    for (auto& t : th) t.join();
  }
  for (int t = 0; t < nthreads; ++t)
    if (rc[t]) {
      g_err = errs[t];
      return rc[t];
    }
  return 0;
}

// expect(op, ψ::LazyKet) (src/states_lazyket.jl:64-125); kets: nsites site kets,
// concatenated.  A LazyTensor's factors must be data operators.
int oref_expect_lazyket(const oref_node* op, int nsites, const int64_t* dims, const double* kets,
                        double* result) {
  return guarded([&] {
    std::vector<std::vector<cd>> psi(nsites);
    const cd* k = reinterpret_cast<const cd*>(kets);
    for (int i = 0; i < nsites; ++i) {
      psi[i].assign(k, k + dims[i]);
      k += dims[i];
    }
    const cd e = expect_lazyket(op, psi);
    result[0] = e.re;
    result[1] = e.im;
  });
}

const char* oref_last_error(void) { return g_err.c_str(); }

}  // extern "C"
