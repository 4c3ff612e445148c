// qob_internal.h -- internal types of libqobgpu: the operator tree mirrored
// from the reference's operator objects, and the compiled device form
// ("plan") that the kernels execute.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "qobgpu.h"

namespace qob {

// ---------------------------------------------------------------------------
// complex scalars (interleaved re, im), usable on host and device
// ---------------------------------------------------------------------------
struct c128 {
  double re, im;
};
struct c64 {
  float re, im;
};

__host__ __device__ inline c128 cmul(c128 a, c128 b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ inline c128 cadd(c128 a, c128 b) { return {a.re + b.re, a.im + b.im}; }
inline bool is_zero(c128 a) { return a.re == 0.0 && a.im == 0.0; }
inline bool is_one(c128 a) { return a.re == 1.0 && a.im == 0.0; }
inline c128 cconj(c128 a) { return {a.re, -a.im}; }

// ---------------------------------------------------------------------------
// errors: thrown inside the library, turned into status codes at the C ABI
// ---------------------------------------------------------------------------
struct Error {
  int code;
  std::string msg;
};
[[noreturn]] void fail(int code, const std::string& msg);
void cuda_check(cudaError_t e, const char* what);
#define QOB_CUDA(call) ::qob::cuda_check((call), #call)
// Every kernel launch of the library is checked and counted (qob_kernel_launches).
void count_launch();
#define QOB_LAUNCHED()                  \
  do {                                  \
    QOB_CUDA(cudaGetLastError());       \
    ::qob::count_launch();              \
  } while (0)

// ---------------------------------------------------------------------------
// operator tree (host)
// ---------------------------------------------------------------------------
enum class Kind { Sparse, Dense, Eye, LazyTensor, LazySum, LazyProduct, Fft };

struct OpNode {
  Kind kind;
  int64_t m = 0, n = 0;  // shape after adjoint: length(basis_l) x length(basis_r)
  bool adjoint = false;
  int src_dtype = QOB_C128;
  // Sparse: stored CSC (0-based), pre-adjoint; Dense: stored column-major.
  int64_t sm = 0, sn = 0;
  std::vector<int64_t> colptr, rowval;
  std::vector<c128> vals;
  // lazy operators
  std::vector<int64_t> shape_l, shape_r;  // composite shapes (LazyTensor)
  std::vector<int> sites;                 // 0-based subsystem of each factor
  std::vector<std::shared_ptr<OpNode>> ops;
  c128 factor{1.0, 0.0};
  std::vector<c128> factors;  // LazySum
  uint64_t factors_version = 0;
  // Fft: DFT along fft_sites (0-based, increasing) of the composite shape shape_l,
  // with per-axis sign (-1: e^{-2 pi i jk/N}, +1: e^{+2 pi i jk/N}) and phase
  // vectors applied before / after (concatenated in axis order)
  std::vector<int> fft_sites, fft_sign;
  std::vector<c128> fft_before, fft_after;
};
using NodeP = std::shared_ptr<OpNode>;

// ---------------------------------------------------------------------------
// compiled device form
// ---------------------------------------------------------------------------
constexpr int kMaxBlocks = 4;   // runs of consecutive subsystems per group
constexpr int kMaxSites = 32;   // subsystems of a composite basis on the device

// One merged local operator: all LazyTensor terms with the same support.
// The local row of output index J is sum_b ((J / div_b) % mod_b) * lstride_b;
// its stored entries give input offsets relative to the row's base index.
struct GGroup {
  int32_t nblk;
  int32_t nrows;
  int32_t rowptr_off;  // into rowptr[]; rowptr values are absolute entry indices
  int32_t support_lo;  // bit mask of support subsystems (non-square bases)
  uint32_t div[kMaxBlocks];
  uint32_t mod[kMaxBlocks];
  uint32_t lstride[kMaxBlocks];
  uint32_t support_hi;
  int32_t width;    // > 0: rows stored as fixed-width (ELL) slots in ell[]; 0: CSR
  int32_t ell_off;  // first ELL slot of this group (slot = one (coloff, value) pair)
  int32_t pow2;     // 1: every div and mod is a power of two (shifts[] are valid)
  uint64_t mdiv[kMaxBlocks];  // Lemire magic numbers of div / mod
  uint64_t mmod[kMaxBlocks];
  uint32_t shifts[kMaxBlocks];  // log2 div | log2 mod << 8 | log2 lstride << 16
  int32_t imag;  // phased plans: 1 when the group's stored (real) values stand for i times them
  int32_t pad_[3];
};

// Fixed-width row slots: a row's entries padded with value 0 to the group's
// width (at most kMaxEllWidth).  One 8/16/32-byte load per slot.
constexpr int kMaxEllWidth = 8;
struct EllD {  // FP64, real value
  int32_t col;
  int32_t pad;
  double v;
};
struct EllZ {  // FP64, complex value
  int32_t col;
  int32_t pad[3];
  double v[2];
};
struct EllF {  // FP32, real value
  int32_t col;
  float v;
};
struct EllC {  // FP32, complex value
  int32_t col;
  int32_t pad;
  float v[2];
};
struct EllDF {  // double-float, real value (hi, lo): the size of EllD
  int32_t col;
  int32_t pad;
  float v[2];
};
struct EllZF {  // double-float, complex value (re hi, re lo, im hi, im lo): the size of EllZ
  int32_t col;
  int32_t pad[3];
  float v[4];
};
static_assert(sizeof(EllDF) == sizeof(EllD) && sizeof(EllZF) == sizeof(EllZ), "double-float slots keep the FP64 sizes");

static_assert(sizeof(GGroup) % 16 == 0,
              "GGroup is copied to shared memory in 8-byte words and the 16-byte items staged after the "
              "descriptors (compact int4 records, ELL slots) must stay 16-byte aligned");

// Per-subsystem data for bases whose left and right shapes differ.
struct SiteTable {
  int32_t nsites;
  uint32_t dout[kMaxSites];
  uint32_t sout[kMaxSites];
  uint32_t din[kMaxSites];
  uint32_t sin[kMaxSites];
  uint64_t msout[kMaxSites];
  uint64_t mdout[kMaxSites];
};

// Kernel-side view of a gather plan for one scalar type.
struct GatherView {
  int64_t m;  // output length
  int64_t n;  // input length
  int32_t ngroups;
  int32_t square;
  int32_t real_vals;
  int32_t has_diag;
  const GGroup* groups;
  const int32_t* rowptr;
  const int32_t* coloff;
  const void* vals;  // double / double2 / float / float2 by precision and real_vals
  const void* diag;  // same element type as vals, length m
  const void* ell;   // EllD / EllZ / EllF / EllC slots of the fixed-width groups
  int32_t ell_slots; // number of ELL slots (all groups)
  int32_t ell_smem;  // 1: stage the ELL slots in shared memory with the descriptors
  int32_t all_ell;   // 1: every group has fixed-width slots
  int32_t all_w1;    // 1: every group has exactly one slot per row
  int32_t fast;      // 1: fastg holds {log2 div, mod - 1, first slot, 0} per group
  const int4* fastg; // compact form: one run of power-of-two subsystems, width 1 (w: the group's imag flag)
  int32_t phased;    // 1: real stored values with per-group imag flags, complex diagonal
  int32_t block;     // threads per block of the index-lanes kernel (0: 256; < 0: persistent grid of -block)
  // Blocks of output indices (k_gather_j) or warp-sized chunks (k_gather_p) are visited in the
  // order c -> (c * jmul) mod count (jmul coprime to count, set per launch): consecutive blocks
  // cover index ranges far apart, so the cost of a block -- which depends on the high index
  // bits through the operator's sparsity -- averages out over the blocks an SM runs.
  uint32_t jmul;
  int32_t lane_split;  // k_gather_j: vector sets per warp (1, 2, 4 or 8; 32/lane_split indices per warp)
  int32_t tile_bits;   // > 0: compact plans on kets use k_gather_t with tiles of 2^tile_bits indices
  int32_t pairs;       // 1: compact plans on kets use k_gather_j2 (two consecutive indices per thread)
  int32_t pdl;         // 1: launched with programmatic stream serialization (QOB_OPT_PDL)
  unsigned* status;    // the context's device status word (bounded waits that gave up, failed checks)
};

// A host-side record of how each stored entry is made from the terms, so a
// change of the LazySum factors only re-evaluates values (set_factors).
struct Contribution {
  int32_t term;   // flattened term index
  int32_t slot;   // entry index (>= 0) or -(diag slot + 1)
  c128 pv;        // product of factor values (without the term coefficient)
};

struct TermCoef {
  int32_t top;    // index into the root LazySum's factors, or -1
  c128 inner;     // product of inner factors (LazyTensor factor, nested sums)
};

// Device copy of the contribution record: every stored value re-evaluated on
// the device from the root LazySum's factors (time-dependent sums), written
// to its places in vals[], ell[] and the local diagonal tables.
struct TdSlot {
  int32_t first, count;  // range in the TdContrib array
  int32_t dst_val;       // index into vals[] or -1
  int32_t dst_ell;       // ELL slot or -1
  int32_t dst_diag;      // index into the local diagonal tables or -1
  int32_t part;          // phased plans: 1 stores the imaginary part in vals[] / ell[]
};
struct TdContrib {
  int32_t term;
  int32_t pad[3];
  double pv[2];
};
struct TdTerm {
  int32_t top;  // factor index or -1
  int32_t pad[3];
  double inner[2];
};

struct DeviceBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DeviceBuf() = default;
  DeviceBuf(const DeviceBuf&) = delete;
  DeviceBuf& operator=(const DeviceBuf&) = delete;
  DeviceBuf(DeviceBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DeviceBuf& operator=(DeviceBuf&& o) noexcept {
    std::swap(p, o.p);
    std::swap(bytes, o.bytes);
    return *this;
  }
  ~DeviceBuf();
  void alloc(size_t b);
  void upload(const void* host, size_t b);
};

struct GatherPlan {
  int64_t m = 0, n = 0;
  bool square = true;
  bool real_vals = true;
  bool phased = false;  // real stored values, per-group imag flags, complex diagonal
  bool ff = false;      // ComplexF64 plan whose values are stored and applied as double-float pairs
  bool has_diag = false;
  int precision = QOB_C128;
  int ngroups = 0;
  int64_t nentries = 0;
  // device arrays
  DeviceBuf groups, rowptr, coloff, vals, diag, ell;
  int32_t ell_slots = 0;
  bool all_ell = true;
  bool all_w1 = true;
  bool fast = false;
  DeviceBuf fastg;
  int tc = 0;     // vectors per thread chosen by qob_op_tune (0: automatic)
  int block = 0;  // threads per block chosen by qob_op_tune (0: 256; < 0: persistent grid of -block)
  int lane_split = 1;  // vector sets per warp chosen by qob_op_tune
  int tile_bits = 0;   // > 0: staged tiles of 2^tile_bits indices (k_gather_t), chosen by qob_op_tune
  int pairs = 0;       // 1: two consecutive indices per thread (k_gather_j2), chosen by qob_op_tune
  unsigned* status = nullptr;  // the owning context's device status word
  DeviceBuf dgroups, dvals;  // diagonal sources: groups + local diagonal tables
  int ndgroups = 0;
  SiteTable sites{};
  // host record for coefficient updates
  std::vector<TermCoef> terms;
  std::vector<Contribution> contrib;
  std::vector<int64_t> dslot_count;
  int64_t ndslots = 0;
  std::shared_ptr<void> host_rec;  // merged-slot record used by set_factors
  // device re-evaluation (built on first use; the structure stays as it is)
  DeviceBuf td_slots, td_contrib, td_terms, td_factors;
  int32_t td_nslots = 0;
  int32_t td_nfactors = 0;
  bool td_ready = false;
  GatherView view() const;
};

// The tensor-core form of a ComplexF32 dense pass (k_tc32.cu): the matrix as
// a real K-major array of 2m rows (rows 2i / 2i + 1: real / imaginary parts of
// row i, n padded to ldk), stored as swizzled 128 x 32 tiles; built on first use.
struct TcDense {
  int64_t m = 0, n = 0, ldk = 0, mtiles = 0;
  DeviceBuf ahat;
  bool stream_a = false;  // the tiled matrix is larger than half the L2 (streamed from memory on each call)
  bool ready = false;
};

// Columns of a tensor-core product's operand: column c = a + s1 * (b + s3 * t)
// sits at element offset a * sa + b * sb + t * st (a dense operator's kets:
// s1 = s3 = 1, st = the ket stride; a mode product: a and b index the
// subsystems before and after the contracted one, t the ket).
struct TcColMap {
  int64_t s1 = 1, s3 = 1, sa = 0, sb = 0, st = 0;
};

// Dense full-space term (GEMM / GEMV pass) or a mode-k sequence.
struct DensePass {
  TermCoef coef;
  int64_t m, n;
  DeviceBuf a;  // m x n column-major in the plan's precision (already transposed for RIGHT)
  TcDense tc;   // ComplexF32 plans: the tensor-core form (QOB_OPT_FP32_TENSOR)
};


struct ModekStep {
  int site;
  int64_t dout, din;
  DeviceBuf a;  // dout x din column-major
  bool eye = false;
  TcDense tc;   // ComplexF32 plans: the tensor-core form (QOB_OPT_FP32_TENSOR)
};
struct ModekPass {
  TermCoef coef;
  std::vector<int64_t> shape_in, shape_out;
  std::vector<ModekStep> steps;
};

struct Plan;
struct SubPass {
  TermCoef coef;
  std::unique_ptr<Plan> plan;
};

// One axis of an FFT plan: lines of n elements at stride `stride` (in vector
// elements); pre / post phases on the side's order; twiddles of the sign.
struct FftAxis {
  int64_t n = 0, stride = 1;
  bool pow2 = true;
  DeviceBuf tw, pre, post;  // plan precision: n/2 (power of two) or n twiddles; n phases each
  // four-step split n = n1 * n2 for long power-of-two axes (0: none); all n twiddles
  int64_t n1 = 0, n2 = 0;
  DeviceBuf tw_full;
};

struct Plan {
  enum class Kind { Sum, Product, Fft } kind = Kind::Sum;
  int side = QOB_LEFT;
  int precision = QOB_C128;
  bool ff = false;  // QOB_C128X: gather, dense and mode-product passes in double-float arithmetic
  int64_t m = 0, n = 0;  // rows of the output vectors / of the input vectors
  // Sum
  std::unique_ptr<GatherPlan> gather;
  std::vector<DensePass> dense;
  std::vector<ModekPass> modek;
  std::vector<SubPass> subs;
  int nterms_total = 0;
  // Product
  c128 pfactor{1.0, 0.0};
  std::vector<std::unique_ptr<Plan>> chain;  // in application order
  // Fft
  std::vector<FftAxis> fft;
  // dependency record: (node, factors_version) of every LazySum inside
  std::vector<std::pair<const OpNode*, uint64_t>> deps;
  const OpNode* root = nullptr;
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct Workspace {
  std::vector<DeviceBuf> slots;
  void* get(size_t slot, size_t bytes);
};

struct Context {
  int device = 0;
  int num_sms = 0;
  std::string err;
  Workspace ws;
  DeviceBuf reduce_buf;
  void* reduce_host = nullptr;  // pinned
  // qob_mul_host's pipeline: copies in, kernels, copies out on three streams,
  // linked per chunk by events
  cudaStream_t copy_stream[3] = {nullptr, nullptr, nullptr};
  static constexpr int kPipeChunks = 8;
  cudaEvent_t pipe_in[kPipeChunks] = {}, pipe_done[kPipeChunks] = {};
  // two device staging sets for host calls, used in turn; stage_free[s] marks
  // the last copy out of the call that used set s
  DeviceBuf stage_x[2], stage_y[2];
  cudaEvent_t stage_free[2] = {};
  bool stage_used[2] = {false, false};
  // tickets of qob_mul_host_async: call t's last copy out is ticket_done[(t-1) % kTickets]
  static constexpr int kTickets = 16;
  cudaEvent_t ticket_done[kTickets] = {};
  uint64_t host_calls = 0;
  // QOB_OPT_FP64_TENSOR: ComplexF64 dense and mode-product passes whose
  // contracted dimension is >= kDmmaMinK run on the FP64 tensor cores
  bool fp64_tensor = false;
  // QOB_OPT_PDL: fused gathers launched with programmatic dependent launch
  bool pdl = false;
  // QOB_OPT_FP32_TENSOR: ComplexF32 dense operators with both sides >= 64 run
  // on the tensor cores (tcgen05, TF32 head + tail split)
  bool fp32_tensor = false;
  // device status word (one unsigned, zeroed at creation): kernels record
  // bounded waits that gave up and failed debug checks; read by qob_device_status
  DeviceBuf status;
  ~Context();
};

// plan.cu
std::unique_ptr<Plan> compile_plan(Context& ctx, const NodeP& op, int side, int precision);
void refresh_coefficients(Plan& plan, const OpNode& root, cudaStream_t s = 0);
bool plan_is_current(const Plan& plan);
// Make the gather structure hold every row of a factor table (rows x nfactors,
// interleaved complex) and build the device re-evaluation tables.
void prepare_factor_rows(Plan& plan, const OpNode& root, const double* rows, int64_t nrows);
// Re-evaluate the gather values on the device from factors in device memory
// (nfactors complex values) and rebuild the merged diagonal, on stream s.
void device_refresh(GatherPlan& g, const double2* factors_dev, cudaStream_t s, const long long* step = nullptr,
                    long long off = 0, long long nf = 0);

// kernels (launchers)
// ff_x: for a double-float plan, room for the split input (the span of x's
// elements, 16 bytes each); unused otherwise.  n = x's length.
void launch_gather(const GatherPlan& g, int precision, const void* x, int64_t xes, int64_t xcs,
                   void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha, c128 beta,
                   cudaStream_t s, int64_t n = 0, void* ff_x = nullptr, bool pdl = false);
void launch_build_diag(const GatherPlan& g, cudaStream_t s);
// Factors at factors_dev, or, with a device step counter, at row 2 * *step + off
// of the table factors_dev (nf factors per row).
void launch_td_values(const GatherPlan& g, const double2* factors_dev, cudaStream_t s,
                      const long long* step = nullptr, long long off = 0, long long nf = 0);
void launch_td_advance(long long* step, cudaStream_t s);
// One FFT pass along an axis of every vector: y = alpha * post .* DFT(pre .* x) + beta * y
// (beta ignored when final == false: y is overwritten).
// scratch (len * ncols elements, may be null) lets few long lines run as a
// four-step FFT over many blocks.
void launch_fft_pass(int precision, const FftAxis& ax, int64_t len, const void* x, int64_t xes, int64_t xcs,
                     void* y, int64_t yes, int64_t ycs, int64_t ncols, c128 alpha, c128 beta, bool final,
                     void* scratch, cudaStream_t s, bool ff = false);
std::unique_ptr<Plan> compile_fft(const NodeP& op, int side, int precision);
int gather_tile(const GatherPlan& g, int64_t ncols);
void launch_scale(int precision, void* y, int64_t rows, int64_t cols, int64_t ld_row,
                  int64_t ld_col, c128 beta, cudaStream_t s);
// ws / slot: room for the partial sums of a product split over column ranges
// (no split without it)
// ff: double-float form (a: (hi, lo) quadruples, x split by launch_ff_split)
void launch_dense(int precision, const void* a, int64_t m, int64_t n, c128 alpha, const void* x,
                  int64_t xes, int64_t xcs, c128 beta, void* y, int64_t yes, int64_t ycs,
                  int64_t ncols, cudaStream_t s, Workspace* ws = nullptr, int slot = 0, bool ff = false,
                  bool dmma = false);
// The same on the FP64 tensor cores (k_dmma.cu; ComplexF64 only).
void launch_dense_dmma(const void* a, int64_t m, int64_t n, c128 alpha, const void* x, int64_t xes, int64_t xcs,
                       c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s, Workspace* ws,
                       int slot);
void launch_modek_dmma(const void* A, int64_t s1, int64_t dout, int64_t din, int64_t s3, c128 alpha, const void* x,
                       int64_t xes, int64_t xcs, c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols,
                       cudaStream_t s);
void tc_dense_build(TcDense& d, const void* a, int64_t m, int64_t n, cudaStream_t s);
// y = alpha * A x + beta * y for ComplexF32 vectors on the tensor cores;
// false when d is not built.  Workspace slots slot, slot + 1.  pdl: the
// split, GEMM and reduce kernels are launched with programmatic dependent
// launch (QOB_OPT_PDL).
bool launch_dense_tc(const TcDense& d, c128 alpha, const void* x, int64_t xes, int64_t xcs, c128 beta, void* y,
                     int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s, Workspace* ws, int slot,
                     unsigned* status, int num_sms, bool pdl = false);
// The same with general column maps (xm, ym) over ncols columns, elements xes /
// yes apart along the contracted / output dimension: mode products of
// ComplexF32 dense LazyTensor factors.
bool launch_gemm_tc(const TcDense& d, c128 alpha, const void* x, int64_t xes, const TcColMap& xm, c128 beta,
                    void* y, int64_t yes, const TcColMap& ym, int64_t ncols, cudaStream_t s, Workspace* ws, int slot,
                    unsigned* status, int num_sms, bool pdl = false);
// contracted dimension and kets from which the FP64 tensor-core option
// applies (an 8 x 8 x 4 tile covers 8 kets: on one ket the FMA kernels are
// about 15x faster at n = 4096)
constexpr int64_t kDmmaMinK = 64;
constexpr int64_t kDmmaMinCols = 8;
// Split of ncols vectors of n ComplexF64 elements (element stride es, vector
// stride cs) into double-float quadruples at the same offsets of out.
void launch_ff_split(const void* x, int64_t n, int64_t ncols, int64_t es, int64_t cs, void* out, cudaStream_t s);
void launch_modek(int precision, const void* a, bool eye, int64_t s1, int64_t dout, int64_t din,
                  int64_t s3, c128 alpha, const void* x, int64_t xes, int64_t xcs, c128 beta,
                  void* y, int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s, bool ff = false,
                  bool dmma = false);
void launch_axpby(int precision, const void* x, int64_t xes, int64_t xcs, c128 alpha, void* y,
                  int64_t yes, int64_t ycs, c128 beta, int64_t len, int64_t ncols,
                  cudaStream_t s);
void reduce_dot(Context& ctx, int precision, const void* x, const void* y, int64_t n, bool norm,
                double* out, cudaStream_t s);
// sum of x[i * stride], i < n, in FP64 (a trace: stride = leading dimension + 1)
void reduce_strided_sum(Context& ctx, int precision, const void* x, int64_t n, int64_t stride, double* out,
                        cudaStream_t s);

// execution (capi.cu)
void apply_plan(Context& ctx, Plan& plan, c128 alpha, const void* x, int64_t xes, int64_t xcs,
                c128 beta, void* y, int64_t yes, int64_t ycs, int64_t ncols, cudaStream_t s,
                int ws_base);

#ifdef __CUDACC__
// Quotient and remainder of non-negative 64-bit values, in 32-bit arithmetic
// when both fit: a 64-bit division is a long instruction sequence, more than an
// elementwise kernel's own work per element.
__device__ __forceinline__ void udivmod(int64_t a, int64_t b, int64_t& q, int64_t& r) {
  if ((((uint64_t)a | (uint64_t)b) >> 32) == 0) {
    const uint32_t q32 = (uint32_t)a / (uint32_t)b;
    q = q32;
    r = (int64_t)((uint32_t)a - q32 * (uint32_t)b);
  } else {
    q = a / b;
    r = a - q * b;
  }
}
#endif

// A multiplier coprime to n near n * (sqrt(5) - 1) / 2: c -> (c * mul) mod n
// visits 0 .. n-1 in an order where neighbours are far apart (1 for n <= 2).
inline uint32_t chunk_multiplier(int64_t n) {
  if (n <= 2) return 1;
  int64_t a = (int64_t)((double)n * 0.6180339887498949) | 1;
  auto gcd = [](int64_t x, int64_t y) {
    while (y) {
      int64_t t = x % y;
      x = y;
      y = t;
    }
    return x;
  };
  while (gcd(a, n) != 1) a += 2;
  return (uint32_t)(a % n);
}

// Lemire, Kaser & Kurz (2019) "Faster remainder by direct computation":
// for 32-bit n and d > 1, n / d == umulhi64(M, n) and n % d ==
// umulhi64((M * n) mod 2^64, d) with M = floor((2^64 - 1) / d) + 1.
inline uint64_t lemire_magic(uint32_t d) { return d <= 1 ? 0 : (~uint64_t(0)) / d + 1; }

}  // namespace qob

struct qob_ctx {
  qob::Context c;
};
struct qob_op {
  qob::NodeP node;
  std::unique_ptr<qob::Plan> plans[2][3];  // [side][dtype: QOB_C128, QOB_C64, QOB_C128X]
};
