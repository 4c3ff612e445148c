/*
 * qobgpu.h -- C ABI of libqobgpu.so, the GB300 (sm_103a) implementation of
 * QuantumOpticsBase.jl's operator-application path.
 *
 * The library replaces the reference's 5-argument mul!
 *     mul!(result, a, b, alpha, beta)      result = alpha*a*b + beta*result
 * for Ket / Bra / Operator results with LazySum, LazyTensor, LazyProduct,
 * SparseOperator and DenseOperator operands.  A host language (Julia through
 * ccall, Python through ctypes, C/C++ directly) builds operator handles that
 * mirror the reference's operator objects, then calls qob_mul on device
 * buffers.  There is no CPU fallback: every qob_mul runs CUDA kernels.
 *
 * Conventions (the reference's):
 *   - complex data is interleaved (re, im); dtype QOB_C128 = ComplexF64,
 *     QOB_C64 = ComplexF32;
 *   - matrices are column-major; CSC index arrays are 1-based (Julia's
 *     SparseMatrixCSC colptr / rowval) and are converted on upload;
 *   - composite bases are ordered first subsystem fastest (src/states.jl:105);
 *   - LazyTensor indices are 1-based and sorted (src/operators_lazytensor.jl:15-36).
 *
 * Every function returns a status (QOB_OK = 0); qob_last_error(ctx) gives a
 * message for the last failure on that context.  All work is stream-ordered
 * on the stream passed in (NULL = the legacy default stream).  A context is
 * not thread-safe: use one per host thread.
 */
#ifndef QOBGPU_H
#define QOBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define QOB_OK 0
#define QOB_ERR_DIM 1         /* DimensionMismatch (src/operators_lazytensor.jl:695-703) */
#define QOB_ERR_ALIAS 2       /* ArgumentError: output aliased with input (:704-708) */
#define QOB_ERR_UNSUPPORTED 3 /* ArgumentError / MethodError: unsupported operand (:640,677) */
#define QOB_ERR_ARG 4         /* invalid argument: null pointer, malformed CSC, bad index */
#define QOB_ERR_CUDA 5        /* a CUDA runtime call failed */
#define QOB_ERR_OOM 6         /* device memory exhausted / admission refused */
#define QOB_ERR_TIMEOUT 7     /* a bounded device-side wait gave up */
#define QOB_ERR_STATE 8       /* call not valid in the object's current state */
#define QOB_ERR_CANCELLED 9   /* the request was cancelled (qob_server_cancel) */

/* element types */
#define QOB_C128 0 /* ComplexF64 */
#define QOB_C64 1  /* ComplexF32 */
/* ComplexF64 data with the fused LazySum part, dense operators, mode
 * products and FFT operators applied in double-float arithmetic (each number the unevaluated
 * sum of two FP32 numbers, about 48 significant bits) on the FP32 pipes, which
 * on GB300 issue far faster than its FP64 pipe (FFT passes too).  Results
 * agree with QOB_C128 to about 1e-14 relative (l2).  Magnitudes of vector
 * elements, operator entries, alpha and beta in [2^-74, 2^128) keep full
 * precision; smaller ones keep 24 bits and below 2^-126 flush to zero; larger
 * ones become infinite.  Accepted by qob_mul, qob_mul_host, qob_mul_host_async,
 * qob_op_prepare, qob_op_tune, qob_op_set_launch, qob_batch_create,
 * qob_apply_batched, qob_rk4, qob_rk4_td and qob_server_create (ComplexF64
 * states, stage arithmetic and norms in FP64); the other entry points take
 * QOB_C128 or QOB_C64. */
#define QOB_C128X 2

/* sides of qob_mul */
#define QOB_LEFT 0  /* y = alpha * op * x + beta * y   (Ket, or Operator from the left)  */
#define QOB_RIGHT 1 /* y = alpha * x * op + beta * y   (Bra, or Operator from the right) */

typedef struct qob_ctx qob_ctx;
typedef struct qob_op qob_op;

int qob_version(void);

/* Number of CUDA kernels this library has launched in the process so far
 * (diagnostics: lets a caller count the device work behind a call). */
int64_t qob_kernel_launches(void);

/* Diagnostics: the device's fused multiply-add rate in TFLOP/s (2 flops per
 * FMA), which = 0 for FP64, 1 for FP32, measured with 16 independent chains of
 * FMAs per thread over one full wave of 256-thread blocks (SMs x the blocks the
 * occupancy calculator admits per SM; one untimed launch, the best of three
 * timed with CUDA events; a few ms).  No counterpart in the reference.
 * Synchronous; allocates and frees a few KB of device memory. */
int qob_probe_peak(qob_ctx* ctx, int which, double* tflops);

/* qob_probe_peak with two more figures of the same best launch (either pointer
 * may be NULL): lanes_per_clock = FMA lanes per SM clock (per SM: the FMAs of
 * its blocks over the span of the SM's cycle counter, median over the SMs),
 * independent of the clock the launch ran at; sm_mhz = the SM clock of that
 * launch (the longest SM span in cycles over the event time).  The roofline of
 * an FP64-bound kernel is lanes_per_clock x 2 x SMs x the SM clock it ran at. */
int qob_probe_peak_ex(qob_ctx* ctx, int which, double* tflops, double* lanes_per_clock, double* sm_mhz);

/* Context on one CUDA device.  flags: reserved, pass 0. */
int qob_create(qob_ctx** ctx, int device, unsigned flags);
int qob_destroy(qob_ctx* ctx);
const char* qob_last_error(qob_ctx* ctx);

/* Context options (no counterpart in the reference, whose BLAS picks its own
 * kernels).  QOB_OPT_FP64_TENSOR, value 0 (default) or 1: ComplexF64 dense
 * operators and mode products of dense LazyTensor factors whose contracted
 * dimension is at least 64, applied to at least 8 kets, run on the FP64 tensor
 * cores (DMMA, mma.sync.m8n8k4.f64: four real products per complex 8 x 8 x 4
 * tile) instead of the FMA kernels; results agree to rounding (1e-15
 * relative).  On GB300 the FMA kernels are faster (about 1.2 against 1.0
 * TFLOP/s); the option is kept for parts with a faster FP64 tensor pipe. */
#define QOB_OPT_FP64_TENSOR 1
/* QOB_OPT_PDL, value 0 (default) or 1: the fused gather kernels, and the
 * split, GEMM and reduce kernels of the tensor-core path (QOB_OPT_FP32_TENSOR),
 * are launched with programmatic dependent launch, so that an application's
 * blocks are scheduled while the previous kernel on the stream finishes (each
 * waits for that kernel's completion before it touches memory; the GEMM sets up
 * its barriers and tensor memory first).  Shortens back-to-back applications,
 * e.g. replayed steps; a grid of far fewer blocks than SMs may run slower with
 * it, its blocks placed on the SMs that the previous kernel frees first. */
#define QOB_OPT_PDL 2
/* QOB_OPT_FP32_TENSOR, value 0 (default) or 1: ComplexF32 dense operators whose
 * sides are both at least 64, and the mode products of ComplexF32 dense
 * LazyTensor factors of at least 64 x 64, run on the 5th-generation tensor cores
 * (tcgen05.mma kind::tf32; operand tiles brought into shared memory by bulk
 * asynchronous copies, the matrix's tiles moved on into tensor memory beside
 * the accumulators) with every operand split into a TF32 head and tail and
 * three products per k step, which keeps FP32 accuracy (relative error ~1e-7);
 * a real, tiled copy of the matrix (the size of the complex one, rounded up to
 * 64 rows x 32 columns) is built on first use.  Each block holds its share of
 * the SM's tensor memory (all of it, or half for up to 16 kets) while it runs. */
#define QOB_OPT_FP32_TENSOR 3
int qob_set_option(qob_ctx* ctx, int option, int64_t value);

/* ---------------------------------------------------------------------------
 * Operator handles.  Data is copied from host memory at construction; child
 * handles may be freed after being used in a parent (the parent keeps its own
 * reference).
 * ------------------------------------------------------------------------- */

/* SparseOperator: Operator{BL,BR,<:SparseMatrixCSC} (src/operators_sparse.jl:5-7).
 * (m, n, colptr[n+1], rowval[nnz], nzval[nnz]) is the stored CSC matrix with
 * 1-based indices; adjoint != 0 makes the operator its conjugate transpose
 * (SparseOpAdjType). */
int qob_op_sparse(qob_ctx* ctx, int64_t m, int64_t n, const int64_t* colptr,
                  const int64_t* rowval, const void* nzval, int dtype, int adjoint, qob_op** out);

/* DenseOperator: Operator{BL,BR,<:Matrix} (src/operators_dense.jl:12-20,49-52);
 * column-major m x n with leading dimension ld; adjoint as above. */
int qob_op_dense(qob_ctx* ctx, int64_t m, int64_t n, const void* data, int64_t ld, int dtype,
                 int adjoint, qob_op** out);

/* identityoperator data: FillArrays Eye(m, n) (src/operators_sparse.jl:86-88,180-183). */
int qob_op_eye(qob_ctx* ctx, int64_t m, int64_t n, qob_op** out);

/* LazyTensor(basis_l, basis_r, indices, operators, factor)
 * (src/operators_lazytensor.jl:15-36).  shape_l / shape_r: the subsystem
 * lengths of the composite bases (_comp_size, :517-518); indices: nfac
 * 1-based, strictly increasing subsystem numbers; factors: sparse, dense or
 * eye handles whose shapes match their subsystems. */
int qob_op_lazytensor(qob_ctx* ctx, int nsub, const int64_t* shape_l, const int64_t* shape_r,
                      int nfac, const int64_t* indices, qob_op* const* factors, double factor_re,
                      double factor_im, qob_op** out);

/* LazySum(basis_l, basis_r, factors, operators) (src/operators_lazysum.jl:41-51);
 * factors: nterms interleaved complex doubles; an empty sum (nterms == 0) is
 * allowed and needs (m, n). */
int qob_op_lazysum(qob_ctx* ctx, int64_t m, int64_t n, int nterms, const double* factors,
                   qob_op* const* ops, qob_op** out);

/* FFTOperator (src/particle.jl:196-535): the transform between position and
 * momentum grids on a composite shape of nsub subsystems (lengths shape[]).
 * The naxes subsystems axes[] (1-based, increasing) are transformed; axis a
 * has the sign sign[a] of the transform a ket sees (-1: FFTW's fft!,
 * e^{-2 pi i jk/N}; +1: bfft!) and per-axis phase vectors before[a] and
 * after[a] (shape[axes[a]-1] complex values each, concatenated in axis order;
 * the reference's mul_before / mul_after are their Kronecker products, with
 * ones on untransformed subsystems, and after includes 1/sqrt(N)).  qob_mul
 * applies it to kets and operator columns (LEFT: after .* DFT(before .* x)) and
 * to bras and operator rows (RIGHT: the same transform of the row with the two
 * phase vectors swapped, as the reference's conj / opposite-sign / conj
 * sequence gives); it may be a term of a LazySum or a factor of a LazyProduct.
 * Power-of-two axes use a radix-2 FFT, other lengths a direct DFT. */
int qob_op_fft(qob_ctx* ctx, int nsub, const int64_t* shape, int naxes, const int64_t* axes, const int* sign,
               const double* before, const double* after, qob_op** out);

/* LazyProduct(operators, factor) (src/operators_lazyproduct.jl:33-52). */
int qob_op_lazyproduct(qob_ctx* ctx, int nops, qob_op* const* ops, double factor_re,
                       double factor_im, qob_op** out);

/* Rewrite a LazySum's factors in place, as TimeDependentSum's
 * update_static_coefficients! does (src/time_dependent_operator.jl:279-290).
 * The compiled device forms are updated at their next use without recompiling:
 * while the stored pattern holds the new values, the factors are copied to the
 * device and the values re-evaluated there in the order of the next call's
 * stream (no synchronisation); a value that becomes nonzero outside the stored
 * pattern, or complex in a real-valued form, rebuilds the structure. */
int qob_op_set_factors(qob_ctx* ctx, qob_op* sum, const double* factors);

int qob_op_free(qob_ctx* ctx, qob_op* op);

/* Shape of an operator: rows = length(basis_l), cols = length(basis_r). */
int qob_op_shape(qob_ctx* ctx, const qob_op* op, int64_t* rows, int64_t* cols);

/* Compile (and cache) the device form of op for one side and dtype ahead of
 * the first qob_mul; qob_mul does this on demand otherwise.  Reports the
 * compiled structure for diagnostics: info[0] = gather groups, info[1] = 1 if a
 * merged diagonal is used, info[2] = total stored entries of the groups,
 * info[3] = number of extra (non-fused) passes.  info may be NULL. */
int qob_op_prepare(qob_ctx* ctx, qob_op* op, int side, int dtype, int64_t* info);

/* Autotuner: time the fused kernel with 1, 2, 4 and 8 vectors per thread and
 * nine launch shapes for applications of op to ncols vectors (side, dtype as
 * in qob_mul) and keep the fastest for later calls with this operator, side
 * and dtype.  Shapes b: 0 / 1 = blocks of 128 / 256 threads over the output
 * indices; 2 = a persistent grid of (SMs x resident blocks) 256-thread blocks
 * that split the work evenly; 3 / 4 = blocks of 128 / 256 threads whose warps
 * cover 8 output indices x 4 sets of vectors, 5 / 6 = 4 output indices x 8
 * sets, 7 / 8 = 2 output indices x 16 sets (entries that vary with the low
 * index bits then diverge over fewer lanes).  times_ms[9k + b] = milliseconds
 * per application with 2^k vectors per thread and shape b, -1 when not tried
 * (36 entries).  For plans in the compact form (every merged group one run of
 * power-of-two subsystems with one entry per row, e.g. spin chains) applied to
 * kets from the left, twelve staged-tile shapes are timed as well (their times
 * are reported by qob_op_tune_ex).  *chosen = vectors per thread | (tile bits
 * << 8, 0 when untiled) | (threads per block << 16) | (log2 vector sets per
 * warp << 26) | (1 << 30 when persistent), 0 when the operator has no fused
 * part.  Either pointer may be NULL.  Vector sets (x and y) of 16 MB or more
 * are timed with inputs not in L2 (up to 16 scratch copies, at least 256 MB in
 * all, used in turn), smaller ones L2-resident.  Each shape is timed over
 * launches replayed from a CUDA graph on a stream of the context's own (no host
 * launch overhead in the times, as in the recorded loops of qob_rk4 / the
 * server).  Allocates and frees the scratch arrays; synchronous. */
int qob_op_tune(qob_ctx* ctx, qob_op* op, int side, int dtype, int64_t ncols, double* times_ms,
                int* chosen);

/* qob_op_tune with the length of times_ms given: writes min(times_len, 58)
 * times, the 36 of qob_op_tune, the twelve staged-tile shapes
 * (times_ms[36 + i]) and ten index-pair shapes (times_ms[48 + i], compact
 * plans on kets from the left: two consecutive
 * output indices per thread, see qob_op_set_pairs), (vectors per thread,
 * threads, vector sets per warp) = (2,256,1) (4,256,1) (2,128,1) (4,128,1)
 * (2,256,4) (4,128,4) (2,128,8) (4,128,8) (2,128,16) (4,128,16); *chosen has
 * bit 7 set when an index-pair shape won.  The staged tiles: blocks of 256 threads that copy tiles of 2^bits
 * consecutive indices of their kets into shared memory, for (bits, vectors per
 * thread, vector sets per warp) = (10,1,1) (10,2,1) (9,4,1) (11,1,1) (11,2,1)
 * (12,1,1) (9,1,4) (8,1,16) (8,2,8) (9,2,4) (10,1,4) (7,2,16); -1 when not
 * tried. */
int qob_op_tune_ex(qob_ctx* ctx, qob_op* op, int side, int dtype, int64_t ncols, double* times_ms, int times_len,
                   int* chosen);

/* Fix the launch shape instead of tuning: vectors_per_thread 1, 2, 4 or 8;
 * block 128 or 256 threads, or -256 for the persistent grid; lane_split 1, 2,
 * 4, 8, 16 or 32 vector sets per warp (32 / lane_split output indices per
 * warp; not used by the persistent grid).  Kept until
 * the next tune or recompilation. */
int qob_op_set_launch(qob_ctx* ctx, qob_op* op, int side, int dtype, int vectors_per_thread, int block,
                      int lane_split);

/* Fix a staged-tile shape instead of tuning (compact plans, kets from the
 * left; other calls keep the untiled kernel with the same vectors per thread
 * and lane split): tiles of 2^tile_bits indices (6 .. 16), vectors_per_thread
 * 1, 2 or 4, lane_split as above, 256 threads.  A call whose tile does not fit
 * (input not 16-byte aligned, or the tile's shared memory over 200 KB) runs the
 * untiled kernel. */
int qob_op_set_tile(qob_ctx* ctx, qob_op* op, int side, int dtype, int vectors_per_thread, int lane_split,
                    int tile_bits);

/* Fix an index-pair shape instead of tuning: compact plans (every group one
 * run of power-of-two subsystems with one entry per row, e.g. spin chains) of
 * even size, applied to kets from the left (ComplexF64, ComplexF32 or
 * double-float), run
 * with two consecutive output indices per thread (a group above bit 0 then
 * serves both with one slot lookup, and a ComplexF32 ket's two inputs arrive in
 * one 16-byte load); vectors_per_thread 2 or 4, block 128 or 256 threads,
 * lane_split as above.  Other calls (other plans, dtypes or sides, ComplexF32
 * vectors not 16-byte aligned or with an odd stride) run the one-index kernel
 * with the same shape. */
int qob_op_set_pairs(qob_ctx* ctx, qob_op* op, int side, int dtype, int vectors_per_thread, int block,
                     int lane_split);

/* Device status of the context: kernels with bounded waits (the staged-tile
 * gather's wait for its copies) record a wait that gave up, and a library built
 * with QOB_DEBUG_BOUNDS records gathered indices outside their vectors (the
 * access is skipped), in a status word instead of faulting.  Reads the word
 * (synchronising `stream`) into *flags (may be NULL) and clears it: 0 and
 * QOB_OK when nothing was recorded; else QOB_ERR_TIMEOUT (bit 0: a wait gave
 * up) or QOB_ERR_ARG (bit 1: an index was out of range), with the message in
 * qob_last_error.  No counterpart in the reference, which only throws on the
 * host. */
int qob_device_status(qob_ctx* ctx, void* stream, unsigned* flags);

/* ---------------------------------------------------------------------------
 * Application: the 5-argument mul!.
 *
 * side QOB_LEFT : y (m x ncols) = alpha * op * x (n x ncols) + beta * y
 *   Ket:       mul!(::Ket, op, ::Ket, alpha, beta)        ncols = 1
 *   Operator:  mul!(::Operator, op, ::Operator, ...)      ncols = columns
 * side QOB_RIGHT: y (nrows x n) = alpha * x (nrows x m) * op + beta * y
 *   Bra:       mul!(::Bra, ::Bra, op, alpha, beta)        nrows = 1
 *   Operator:  mul!(::Operator, ::Operator, op, ...)      nrows = rows
 *
 * x and y are DEVICE pointers to column-major arrays with leading dimensions
 * x_ld, y_ld (elements).  is_vector selects the Ket/Bra form of the
 * reference's dispatch (gemv! rather than gemm!).  beta == 0 overwrites y
 * without reading it (NaN in y is ignored, src/operators_lazysum.jl:179-186).
 * Errors: QOB_ERR_DIM on shape mismatch, QOB_ERR_ALIAS when y overlaps x.
 * ------------------------------------------------------------------------- */
int qob_mul(qob_ctx* ctx, int side, int is_vector, qob_op* op, int dtype, double alpha_re,
            double alpha_im, const void* x, int64_t x_rows, int64_t x_cols, int64_t x_ld,
            double beta_re, double beta_im, void* y, int64_t y_rows, int64_t y_cols, int64_t y_ld,
            void* stream);

/* Same as qob_mul for HOST x and y (column-major, leading dimension = rows):
 * the library copies x (and y when beta != 0) to the device, applies the
 * operator and copies y back -- the path a caller without device buffers uses.
 * Several kets from the left go through in up to four chunks of columns whose
 * copies and kernels overlap.  Synchronous: returns with y written. */
int qob_mul_host(qob_ctx* ctx, int side, int is_vector, qob_op* op, int dtype, double alpha_re,
                 double alpha_im, const void* x, int64_t x_rows, int64_t x_cols, double beta_re,
                 double beta_im, void* y, int64_t y_rows, int64_t y_cols);

/* Stream-ordered qob_mul_host for a stream of batches: enqueues the copies
 * in, the application and the copy of y back out, and returns at once with a
 * ticket.  After qob_host_wait(ctx, ticket) returns, y holds the result and x
 * and y may be reused; until then the caller leaves both untouched.  Calls run
 * in the order made, and each call's copies in overlap the previous call's
 * kernels and copy out (two device staging sets are used in turn), so a stream
 * of batches moves at the host link's rate; a call's own copies and kernels
 * run one after another (no chunks: fewer copies), so a single call waited on
 * alone is slower than qob_mul_host.  With page-locked host memory the
 * copies are asynchronous; with pageable memory the driver stages them and the
 * call returns once they are done.  Errors of the argument checks return at
 * once; errors of the device work return from qob_host_wait. */
int qob_mul_host_async(qob_ctx* ctx, int side, int is_vector, qob_op* op, int dtype, double alpha_re,
                       double alpha_im, const void* x, int64_t x_rows, int64_t x_cols, double beta_re,
                       double beta_im, void* y, int64_t y_rows, int64_t y_cols, uint64_t* ticket);

/* Blocks until the qob_mul_host_async call that returned `ticket` and every
 * earlier one have finished.  Ticket 0 returns at once; a ticket not yet handed
 * out is QOB_ERR_ARG. */
int qob_host_wait(qob_ctx* ctx, uint64_t ticket);

/* ---------------------------------------------------------------------------
 * FP64 reductions (norm, inner product, expectation value) on device vectors;
 * deterministic order.  Results are written to HOST memory (synchronous).
 * x of dtype QOB_C128 or QOB_C64; accumulation is always in double.
 * ------------------------------------------------------------------------- */
/* norm(x) (src/states.jl:89) */
int qob_norm(qob_ctx* ctx, int dtype, const void* x, int64_t n, double* result, void* stream);
/* dot(x, y) = sum conj(x_i) y_i, result interleaved complex */
int qob_dot(qob_ctx* ctx, int dtype, const void* x, const void* y, int64_t n, double* result,
            void* stream);
/* expect(op, psi) = <psi|op|psi> (src/operators.jl:119) */
int qob_expect(qob_ctx* ctx, qob_op* op, int dtype, const void* psi, int64_t n, double* result,
               void* stream);
/* expect(op, rho) = sum_ij op[i,j] rho[j,i] = tr(op rho) for a density
 * operator rho (n x n, column-major, leading dimension ld, on the device)
 * (src/operators_dense.jl:223-230, src/operators_sparse.jl:36-46; here for
 * every operator kind): op applied to blocks of rho's columns, then the
 * blocks' shares of the trace of the product summed in FP64 in block order.
 * The workspace holds one block, at most 256 MiB (at least one column), and
 * stays with the context until qob_destroy. */
int qob_expect_dm(qob_ctx* ctx, qob_op* op, int dtype, const void* rho, int64_t n, int64_t ld, double* result,
                  void* stream);
/* variance(op, psi) = <psi|op (op psi)> - <psi|op psi>^2 (src/operators.jl:139-142):
 * two applications of op, two FP64 inner products; result interleaved complex
 * (real for a Hermitian op up to rounding). */
int qob_variance(qob_ctx* ctx, qob_op* op, int dtype, const void* psi, int64_t n, double* result,
                 void* stream);

/* qob_dot_noalloc: the inner product of qob_dot for callers that cannot
 * allocate device memory while they run (their memory pool owns the device, or
 * they issue work during a stream capture).  No counterpart in the reference:
 * it is an addition of this library.
 *   - allocates nothing: partial sums live in a 128 KiB static device array held
 *     by every GPU that loads the library until exit; the result (two doubles,
 *     re and im) is written to DEVICE memory `result` owned by the caller,
 *     stream-ordered on `stream`, without synchronising;
 *   - n is limited to 16,777,216 elements; larger n returns QOB_ERR_ARG;
 *   - all calls share the one array: calls that overlap on the GPU race; order
 *     them (one stream);
 *   - the first call on a device looks up the array's address; make it before
 *     any stream capture. */
int qob_dot_noalloc(qob_ctx* ctx, int dtype, const void* x, const void* y, int64_t n,
                    double* result, void* stream);

/* ---------------------------------------------------------------------------
 * Batches of uneven applications in one launch (no counterpart in the
 * reference, which would issue one mul! per operator).  Each item is
 * y = alpha * op * x + beta * y for one ket (x: op cols, y: op rows, DEVICE
 * pointers in the batch's dtype); the items may have different operators and
 * dimensions.  qob_batch_run applies all items: the fused parts of every item
 * in one persistent launch over equal tiles of their output indices, the rest
 * per item.  Pointers are captured at qob_batch_add; a run reads the current
 * contents, so a run recorded in a CUDA graph can be replayed after refilling
 * the same buffers.
 * ------------------------------------------------------------------------- */
typedef struct qob_batch qob_batch;
int qob_batch_create(qob_ctx* ctx, int dtype, qob_batch** out);
int qob_batch_add(qob_ctx* ctx, qob_batch* batch, qob_op* op, double alpha_re, double alpha_im,
                  const void* x, void* y, double beta_re, double beta_im);
int qob_batch_run(qob_ctx* ctx, qob_batch* batch, void* stream);
/* One-shot batched application (creates, runs and frees a batch):
 * y_i = alpha_i op_i x_i + beta_i y_i for i < n on device kets of `dtype`;
 * alphas / betas: n interleaved complex doubles each.  Synchronous on stream. */
int qob_apply_batched(qob_ctx* ctx, int dtype, int n, qob_op* const* ops, const void* const* xs,
                      void* const* ys, const double* alphas, const double* betas, void* stream);
/* Time tile lengths 128 / 256 / 512 / 1024 (times_ms[0..3]) and keep the
 * fastest; runs the batch 28 times, so the outputs are overwritten. */
int qob_batch_tune(qob_ctx* ctx, qob_batch* batch, double* times_ms, int* chosen);
/* Set the tile length (128, 256, 512 or 1024 output indices) without timing,
 * e.g. to the one a previous qob_batch_tune chose; QOB_ERR_ARG otherwise. */
int qob_batch_set_tile(qob_ctx* ctx, qob_batch* batch, int tile);
/* info[0] items, [1] items in the fused launch, [2] tiles, [3] tile length,
 * [4] blocks of the persistent grid. */
int qob_batch_info(qob_ctx* ctx, qob_batch* batch, int64_t* info);
int qob_batch_free(qob_ctx* ctx, qob_batch* batch);

/* ---------------------------------------------------------------------------
 * Device states for callers that do not manage device memory themselves
 * (the reference's arrays are Julia-owned; a C caller can use these instead of
 * CUDA calls of its own).  A state holds dim x ncols complex values of dtype,
 * column-major, zero-initialised; uploads and downloads are synchronous on
 * `stream`.
 * ------------------------------------------------------------------------- */
int qob_state_alloc(qob_ctx* ctx, int dtype, int64_t dim, int64_t ncols, void** state);
int qob_state_free(qob_ctx* ctx, void* state);
int qob_state_upload(qob_ctx* ctx, int dtype, void* state, const void* host, int64_t dim, int64_t ncols,
                     void* stream);
int qob_state_download(qob_ctx* ctx, int dtype, const void* state, void* host, int64_t dim, int64_t ncols,
                       void* stream);

/* ---------------------------------------------------------------------------
 * Expectation values on product states (LazyKet, src/states_lazyket.jl:64-125).
 * op: a LazyTensor, a LazySum (nested sums allowed) of LazyTensors and
 * LazyProducts of LazyTensors, on the square composite basis whose nsites
 * subsystems have the lengths site_dims.  kets: nstates product states on the
 * device in dtype, one after another, each the concatenation of its site kets
 * (state s, site i at element s * sum(site_dims) + sum_{j<i} site_dims[j]).
 * result: nstates complex doubles on the device,
 *   result[s] = expect(op, LazyKet(basis, (psi_s1, ..., psi_sn))):
 *   for a LazyTensor  factor * prod_{i in indices} <psi_i|A_i|psi_i> * prod_{i not in indices} <psi_i|psi_i>,
 *   for a LazyProduct factor * (factors of its LazyTensors) * prod_i <psi_i|F_1i ... F_ni|psi_i>,
 *   for a LazySum     sum_k f_k * (its terms).
 * Computed in FP64 for both dtypes.  Synchronous on `stream`. */
int qob_expect_lazyket(qob_ctx* ctx, qob_op* op, int dtype, int nsites, const int64_t* site_dims,
                       const void* kets, int64_t nstates, double* result, void* stream);

/* ---------------------------------------------------------------------------
 * Time evolution.  qob_rk4 advances a device state by nsteps fixed RK4 steps
 * of dpsi/dt = -i H psi (the right-hand side QuantumOptics.jl's Schroedinger
 * solver evaluates with mul!(dpsi, H, psi, -im, 0) on top of this package).
 * renormalise != 0 rescales psi to unit FP64 norm after every step.
 * Synchronous on `stream`.
 * ------------------------------------------------------------------------- */
int qob_rk4(qob_ctx* ctx, qob_op* H, int dtype, void* psi, int64_t n, double dt, int nsteps,
            int renormalise, void* stream);

/* RK4 of dpsi/dt = -i H(t) psi for a TimeDependentSum: H is the LazySum of its
 * operators and row r of `factors` (nrows = 2*nsteps + 1 rows of nterms
 * interleaved complex doubles, host memory) holds the coefficients at
 * t0 + r*dt/2, i.e. what set_time!(H, t) writes through
 * update_static_coefficients! (src/time_dependent_operator.jl:162-171,279-290)
 * before each right-hand-side evaluation.  The table is copied to the device
 * once; before each stage the compiled values are re-evaluated on the device
 * from its row, so no host round trip happens inside the steps.  Every term
 * must compile into the fused gather (QOB_ERR_UNSUPPORTED otherwise).
 * Synchronous on `stream`. */
int qob_rk4_td(qob_ctx* ctx, qob_op* H, int dtype, void* psi, int64_t n, double dt, int nsteps,
               const double* factors, int64_t nrows, int renormalise, void* stream);

/* ---------------------------------------------------------------------------
 * Request server with continuous batching (no counterpart in the reference).
 * A request = (H, psi0 on the HOST, nsteps, dt): nsteps RK4 steps of
 * dpsi/dt = -i H psi.  States and operators stay resident on the device; a
 * queued request is admitted when fewer than max_active run and its device
 * memory (4 state vectors) fits both mem_budget and the free device memory;
 * requests larger than mem_budget are rejected (status -QOB_ERR_OOM).  A step
 * of every active request is four batched launches (each RK4 stage's
 * combination done in the batched gather's epilogue; eight, the combinations
 * apart, when an operator does not compile into the fused gather), recorded
 * once per set of active requests into a CUDA graph and replayed; an engine iteration on the
 * worker thread (qob_server_start / _stop) runs up to 16 steps (4 while
 * requests wait, never past a request's last step), qob_server_step runs one.
 * Requests that arrive while others run join at the next iteration.  A
 * request's result does not depend on the others in flight.
 * status: 0 queued, 1 running, 2 done, < 0 failed (-error code).
 * times[0..2]: submit, admit and completion time (seconds, steady clock).
 * stats[0..7]: queued, active, completed, rejected, request-steps, engine
 * iterations, device bytes held, last engine error code.
 * ------------------------------------------------------------------------- */
typedef struct qob_server qob_server;
int qob_server_create(qob_ctx* ctx, int dtype, size_t mem_budget, int max_active, int renormalise,
                      qob_server** out);
int qob_server_submit(qob_server* server, qob_op* H, const void* psi0, int64_t n, int nsteps,
                      double dt, int64_t* id);
/* A request with a time-dependent H (TimeDependentSum): H is the LazySum of its
 * operators and factors holds its coefficients at t0 + r*dt/2 for r = 0 ..
 * 2*nsteps (nrows rows of nterms interleaved complex doubles, host memory), as
 * qob_rk4_td takes them.  The request gets a compiled form of its own; its
 * values are re-evaluated on the device inside the recorded steps.  Every term
 * must compile into the fused gather (else the request fails with
 * -QOB_ERR_UNSUPPORTED at admission). */
int qob_server_submit_td(qob_server* server, qob_op* H, const void* psi0, int64_t n, int nsteps, double dt,
                         const double* factors, int64_t nrows, int64_t* id);
int qob_server_step(qob_server* server, int* nactive);
int qob_server_start(qob_server* server);
int qob_server_stop(qob_server* server);
int qob_server_poll(qob_server* server, int64_t id, void* psi_out, double* times, int* status);
int qob_server_wait(qob_server* server, int64_t id, double timeout_s, int* status);
int qob_server_stats(qob_server* server, int64_t* stats);
/* stats[0..1]: requests cancelled, allocations refused (by the hook or the device). */
int qob_server_stats2(qob_server* server, int64_t* stats);
/* Cancel a request (no counterpart in the reference).  A queued request leaves
 * at once; a running one leaves before the engine's next iteration (at most 16
 * steps later), its device memory released.  Its status becomes
 * -QOB_ERR_CANCELLED and qob_server_wait returns for it.  QOB_ERR_STATE when the
 * request has already finished or failed. */
int qob_server_cancel(qob_server* server, int64_t id);
/* Host-side allocation hook (no counterpart in the reference): hook(user,
 * bytes) is called, with the server's lock held, before the device memory of
 * each admission is allocated; a nonzero return refuses the allocation as if
 * the device were out of memory.  A refused admission leaves the request queued
 * while other requests run (they free memory when they finish); with nothing
 * else active it is retried at the next iterations and rejected with
 * -QOB_ERR_OOM after three refusals in a row.  Device allocation failures take
 * the same path.  NULL removes the hook.  The hook must not call the server. */
int qob_server_set_alloc_hook(qob_server* server, int (*hook)(void* user, size_t bytes), void* user);
int qob_server_destroy(qob_server* server);

/* ---------------------------------------------------------------------------
 * CUDA graphs of library calls.  Between qob_graph_begin and qob_graph_end the
 * qob_* calls issued on `stream` (a non-default stream) are recorded instead of
 * run; qob_graph_launch replays them.  Operators used inside must have been
 * applied (or qob_op_prepare'd) once with the same shapes before capture, so
 * that no allocation or upload happens while recording.
 * ------------------------------------------------------------------------- */
typedef struct qob_graph qob_graph;
int qob_graph_begin(qob_ctx* ctx, void* stream);
int qob_graph_end(qob_ctx* ctx, void* stream, qob_graph** out);
int qob_graph_launch(qob_ctx* ctx, qob_graph* graph, void* stream);
int qob_graph_free(qob_ctx* ctx, qob_graph* graph);

#ifdef __cplusplus
}
#endif
#endif /* QOBGPU_H */
