/*
 * qob_oracle.h -- CPU restatement of QuantumOpticsBase.jl's operator-application
 * path (the 5-argument mul! on Ket/Bra/Operator with LazySum, LazyTensor,
 * LazyProduct, SparseOperator and DenseOperator).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * library and the timed CPU baseline; it is never part of the product path.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
 * load it.
 *
 * Parity status: the reference (Julia) cannot run on this machine, so the
 * restatement is pinned against the identities the reference's own tests
 * check (lazy operator == dense materialisation, alpha/beta, NaN-killing with
 * beta == 0, isometries, adjoints, empty sums) and against known-answer values
 * of the factor constructors; not against outputs of the reference itself.
 *
 * Data conventions (same as the reference): complex values are interleaved
 * (re, im) doubles, matrices are column-major, CSC index arrays are 1-based
 * (Julia's SparseMatrixCSC), composite bases are ordered first-subsystem
 * fastest (src/states.jl:105).
 */
#ifndef QOB_ORACLE_H
#define QOB_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct oref_node oref_node;

/* Leaf data operators.  (m, n) are the dimensions of the STORED matrix; with
 * adjoint != 0 the operator is its conjugate transpose (n x m), as
 * Operator{BL,BR,<:Adjoint} in src/operators_sparse.jl:5-7 and
 * src/operators_dense.jl:49-52. */
oref_node* oref_sparse(int64_t m, int64_t n, const int64_t* colptr, const int64_t* rowval,
                       const double* nzval, int adjoint);
oref_node* oref_dense(int64_t m, int64_t n, const double* data, int adjoint);
/* FillArrays.Eye(m, n) data (src/operators_sparse.jl:86-88). */
oref_node* oref_eye(int64_t m, int64_t n);

/* LazyTensor(basis_l, basis_r, indices, operators, factor)
 * (src/operators_lazytensor.jl:15-36).  indices are 1-based and sorted. */
oref_node* oref_lazytensor(int nsub, const int64_t* shape_l, const int64_t* shape_r, int nfac,
                           const int64_t* indices, oref_node* const* factors, double factor_re,
                           double factor_im);
/* LazySum(basis_l, basis_r, factors, operators) (src/operators_lazysum.jl:41-51). */
oref_node* oref_lazysum(int64_t m, int64_t n, int nterms, const double* factors,
                        oref_node* const* ops);
/* LazyProduct(operators, factor) (src/operators_lazyproduct.jl:33-52). */
oref_node* oref_lazyproduct(int nops, oref_node* const* ops, double factor_re, double factor_im);
/* FFTOperator (src/particle.jl:196-535) on a composite shape of nsub
 * subsystems: the transformed subsystems axes (1-based, increasing), the sign
 * of the transform applied to kets (fft_r!: -1 fft, +1 bfft) and the full
 * phase arrays mul_before / mul_after (prod(shape) complex values each). */
oref_node* oref_fft(int nsub, const int64_t* shape, int naxes, const int64_t* axes, int sign,
                    const double* mul_before, const double* mul_after);
/* Rewrite the factors of a LazySum in place (TimeDependentSum's
 * update_static_coefficients!, src/time_dependent_operator.jl:279-290). */
int oref_lazysum_set_factors(oref_node* sum, const double* factors);
void oref_free(oref_node* node);
int64_t oref_rows(const oref_node* node);
int64_t oref_cols(const oref_node* node);

/* side 0: y (m x ncols) = alpha * op * x + beta * y       (Ket / Operator from the left)
 * side 1: y (nrows x n) = alpha * x * op + beta * y       (Bra / Operator from the right)
 * x, y contiguous column-major.  is_vector != 0 means x and y are a Ket (side
 * 0) or a Bra (side 1) rather than an Operator; it selects gemv! over gemm!
 * exactly as the reference's dispatch does.  Returns 0 on success, non-zero on
 * the reference's error cases (DimensionMismatch = 1, aliasing ArgumentError =
 * 2, unsupported = 3); oref_last_error() gives the message. */
int oref_mul(int side, int is_vector, const oref_node* op, double alpha_re, double alpha_im,
             const double* x, int64_t x_rows, int64_t x_cols, double beta_re, double beta_im,
             double* y, int64_t y_rows, int64_t y_cols);

/* nvec independent left-applications (one Ket each, contiguous, stride = rows)
 * spread over nthreads host threads.  Used as the timed CPU baseline. */
int oref_mul_kets_threaded(const oref_node* op, double alpha_re, double alpha_im, const double* x,
                           double beta_re, double beta_im, double* y, int64_t nvec, int nthreads);

/* expect(op, LazyKet(basis, kets)) (src/states_lazyket.jl:64-125): kets are
 * the nsites site kets (lengths dims) concatenated; result = one complex. */
int oref_expect_lazyket(const oref_node* op, int nsites, const int64_t* dims, const double* kets,
                        double* result);

const char* oref_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
