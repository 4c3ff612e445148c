// lazyket.cu -- expectation values on product states (LazyKet,
// src/states_lazyket.jl:64-125), many states per launch.
//
// The reference evaluates expect(op, ψ::LazyKet) term by term on the host:
// for a LazyTensor, factor * Π_{i in indices} <ψ_i|A_i|ψ_i> * Π_{i not in
// indices} <ψ_i|ψ_i> (:64-84); for a LazyProduct of LazyTensors it applies the
// factors site by site to a copy of ψ and multiplies the site overlaps (:86-107,
// with the LazyTensor factors multiplied into the first site, :127-150); a
// LazySum adds f_k times its terms (:109-120).  Here the operator is compiled
// once into terms c_k * Π_{sites} <ψ_i|M_ki|ψ_i>, where M_ki is the site
// factor (or the product of a LazyProduct's site factors) and sites without a
// factor contribute <ψ_i|ψ_i>; distinct (site, matrix) pairs are evaluated once
// per state.  One block per state: the site overlaps go to shared memory, then
// the terms are multiplied out and summed in a fixed order (FP64 throughout).
#include <algorithm>
#include <map>
#include <vector>

#include "qob_internal.h"

namespace qob {
namespace {

using DenseM = std::vector<c128>;  // d x d, column-major

struct SiteObs {
  int32_t site;
  int32_t row0;   // first row pointer of the matrix (into rowptr)
  int32_t dim;
  int32_t pad;
};

struct KetTerm {
  double coef[2];
  int32_t first, count;  // range of observable indices in term_obs
  uint32_t mask_lo, mask_hi;  // sites covered by observables (others contribute <ψ_i|ψ_i>)
};

DenseM leaf_dense(const OpNode& f) {
  const int64_t m = f.m, n = f.n;
  DenseM a((size_t)(m * n), c128{0.0, 0.0});
  auto put = [&](int64_t r, int64_t c, c128 v) {  // (r, c) of the stored matrix
    if (f.adjoint) a[(size_t)(c + r * m)] = cconj(v);
    else a[(size_t)(r + c * m)] = v;
  };
  switch (f.kind) {
    case Kind::Sparse:
      for (int64_t c = 0; c < f.sn; ++c)
        for (int64_t p = f.colptr[c]; p < f.colptr[c + 1]; ++p) put(f.rowval[p], c, f.vals[p]);
      break;
    case Kind::Dense:
      for (int64_t c = 0; c < f.sn; ++c)
        for (int64_t r = 0; r < f.sm; ++r) put(r, c, f.vals[r + c * f.sm]);
      break;
    case Kind::Eye:
      for (int64_t k = 0; k < std::min(m, n); ++k) a[(size_t)(k + k * m)] = {1.0, 0.0};
      break;
    default:
      fail(QOB_ERR_UNSUPPORTED, "expect on a LazyKet: LazyTensor factors must be data operators");
  }
  return a;
}

DenseM matmul(const DenseM& a, const DenseM& b, int64_t d) {
  DenseM c((size_t)(d * d), c128{0.0, 0.0});
  for (int64_t j = 0; j < d; ++j)
    for (int64_t k = 0; k < d; ++k) {
      const c128 bk = b[(size_t)(k + j * d)];
      if (bk.re == 0.0 && bk.im == 0.0) continue;
      for (int64_t i = 0; i < d; ++i) c[(size_t)(i + j * d)] = cadd(c[(size_t)(i + j * d)], cmul(a[(size_t)(i + k * d)], bk));
    }
  return c;
}

struct Builder {
  std::vector<int64_t> dims;
  std::vector<int32_t> rowptr, col;
  std::vector<c128> val;
  std::vector<SiteObs> obs;
  std::map<std::pair<int, std::vector<double>>, int32_t> seen;
  std::vector<KetTerm> terms;
  std::vector<int32_t> term_obs;

  int32_t add_obs(int site, const DenseM& m) {
    std::vector<double> key(2 * m.size());
    for (size_t k = 0; k < m.size(); ++k) {
      key[2 * k] = m[k].re;
      key[2 * k + 1] = m[k].im;
    }
    auto it = seen.find({site, key});
    if (it != seen.end()) return it->second;
    const int64_t d = dims[site];
    SiteObs o{};
    o.site = site;
    o.row0 = (int32_t)rowptr.size();
    o.dim = (int32_t)d;
    rowptr.push_back((int32_t)col.size());
    for (int64_t r = 0; r < d; ++r) {
      for (int64_t c = 0; c < d; ++c) {
        const c128 v = m[(size_t)(r + c * d)];
        if (v.re != 0.0 || v.im != 0.0) {
          col.push_back((int32_t)c);
          val.push_back(v);
        }
      }
      rowptr.push_back((int32_t)col.size());
    }
    const int32_t id = (int32_t)obs.size();
    obs.push_back(o);
    seen[{site, key}] = id;
    return id;
  }

  void add_term(c128 coef, const std::map<int, DenseM>& site_mats) {
    KetTerm t{};
    t.coef[0] = coef.re;
    t.coef[1] = coef.im;
    t.first = (int32_t)term_obs.size();
    for (auto& sm : site_mats) {
      term_obs.push_back(add_obs(sm.first, sm.second));
      if (sm.first < 32) t.mask_lo |= 1u << sm.first;
      else t.mask_hi |= 1u << (sm.first - 32);
    }
    t.count = (int32_t)(term_obs.size() - t.first);
    terms.push_back(t);
  }

  // site factors of a LazyTensor on the state's composite basis
  std::map<int, DenseM> site_factors(const OpNode& lt) {
    if (lt.shape_l != lt.shape_r) fail(QOB_ERR_UNSUPPORTED, "expect on a LazyKet needs a square LazyTensor");
    if (lt.shape_l.size() != dims.size() || !std::equal(dims.begin(), dims.end(), lt.shape_l.begin()))
      fail(QOB_ERR_DIM, "LazyTensor and LazyKet bases differ");
    std::map<int, DenseM> out;
    for (size_t i = 0; i < lt.ops.size(); ++i) {
      const int s = lt.sites[i];
      DenseM a = leaf_dense(*lt.ops[i]);
      auto it = out.find(s);
      if (it == out.end()) out[s] = std::move(a);
      else it->second = matmul(it->second, a, dims[s]);
    }
    return out;
  }

  void walk(const OpNode& op, c128 coef) {
    switch (op.kind) {
      case Kind::LazySum:
        for (size_t k = 0; k < op.ops.size(); ++k) walk(*op.ops[k], cmul(coef, op.factors[k]));
        return;
      case Kind::LazyTensor:
        add_term(cmul(coef, op.factor), site_factors(op));
        return;
      case Kind::LazyProduct: {
        // M_i = F_1,i F_2,i ... F_n,i: the last operator acts first (:94-100)
        c128 c = cmul(coef, op.factor);
        std::map<int, DenseM> acc;
        for (size_t k = 0; k < op.ops.size(); ++k) {
          const OpNode& lt = *op.ops[k];
          if (lt.kind != Kind::LazyTensor)
            fail(QOB_ERR_UNSUPPORTED, "expect(LazyProduct, LazyKet) needs LazyTensor factors");
          c = cmul(c, lt.factor);
          for (auto& sf : site_factors(lt)) {
            auto it = acc.find(sf.first);
            if (it == acc.end()) acc[sf.first] = sf.second;
            else it->second = matmul(it->second, sf.second, dims[sf.first]);
          }
        }
        add_term(c, acc);
        return;
      }
      default:
        fail(QOB_ERR_UNSUPPORTED, "expect on a LazyKet needs a LazyTensor, LazySum or LazyProduct");
    }
  }
};

constexpr int kKetThreads = 128;

template <typename CT>
__global__ void __launch_bounds__(kKetThreads) k_lazyket_expect(
    const CT* __restrict__ kets, int64_t stride, int nsites, const int64_t* __restrict__ site_off,
    const int64_t* __restrict__ site_dim, int nobs, const SiteObs* __restrict__ obs,
    const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col, const double2* __restrict__ val,
    int nterms, const KetTerm* __restrict__ terms, const int32_t* __restrict__ term_obs,
    double2* __restrict__ result) {
  extern __shared__ __align__(16) unsigned char sm[];
  // 16-byte items first, then the 8-byte norms (every array stays aligned)
  double2* e = reinterpret_cast<double2*>(sm);             // nobs
  double2* part = e + nobs;                                // kKetThreads
  double* nrm = reinterpret_cast<double*>(part + kKetThreads);  // nsites
  const CT* psi = kets + (int64_t)blockIdx.x * stride;
  // <ψ_i|M|ψ_i> per observable, row by row: sum_r conj(ψ_r) sum_p M_rp ψ_p
  for (int u = threadIdx.x; u < nobs; u += blockDim.x) {
    const SiteObs o = obs[u];
    const CT* p = psi + site_off[o.site];
    double re = 0.0, im = 0.0;
    for (int r = 0; r < o.dim; ++r) {
      double tr = 0.0, ti = 0.0;
      for (int q = rowptr[o.row0 + r]; q < rowptr[o.row0 + r + 1]; ++q) {
        const double2 v = val[q];
        const CT x = p[col[q]];
        tr += v.x * (double)x.x - v.y * (double)x.y;
        ti += v.x * (double)x.y + v.y * (double)x.x;
      }
      const CT a = p[r];
      re += (double)a.x * tr + (double)a.y * ti;
      im += (double)a.x * ti - (double)a.y * tr;
    }
    e[u] = make_double2(re, im);
  }
  for (int i = threadIdx.x; i < nsites; i += blockDim.x) {
    const CT* p = psi + site_off[i];
    double s = 0.0;
    for (int64_t r = 0; r < site_dim[i]; ++r) s += (double)p[r].x * (double)p[r].x + (double)p[r].y * (double)p[r].y;
    nrm[i] = s;
  }
  __syncthreads();
  double pr = 0.0, pi = 0.0;
  for (int k = threadIdx.x; k < nterms; k += blockDim.x) {
    const KetTerm t = terms[k];
    double vr = t.coef[0], vi = t.coef[1];
    for (int q = 0; q < t.count; ++q) {
      const double2 a = e[term_obs[t.first + q]];
      const double r2 = vr * a.x - vi * a.y;
      vi = vr * a.y + vi * a.x;
      vr = r2;
    }
    for (int i = 0; i < nsites; ++i) {
      const bool cov = i < 32 ? ((t.mask_lo >> i) & 1u) : ((t.mask_hi >> (i - 32)) & 1u);
      if (!cov) {
        vr *= nrm[i];
        vi *= nrm[i];
      }
    }
    pr += vr;
    pi += vi;
  }
  part[threadIdx.x] = make_double2(pr, pi);
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr = 0.0, si = 0.0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      sr += part[t].x;
      si += part[t].y;
    }
    result[blockIdx.x] = make_double2(sr, si);
  }
}

}  // namespace
}  // namespace qob

extern "C" int qob_expect_lazyket(qob_ctx* ctx, qob_op* op, int dtype, int nsites, const int64_t* site_dims,
                                  const void* kets, int64_t nstates, double* result, void* stream) {
  if (!ctx) return QOB_ERR_ARG;
  try {
    using namespace qob;
    QOB_CUDA(cudaSetDevice(ctx->c.device));
    if (!op || nsites < 1 || nsites > 64 || !site_dims || nstates < 0 || (nstates > 0 && (!kets || !result)) ||
        (dtype != QOB_C128 && dtype != QOB_C64))
      fail(QOB_ERR_ARG, "qob_expect_lazyket: bad arguments");
    if (nstates > INT32_MAX) fail(QOB_ERR_ARG, "qob_expect_lazyket: too many states");
    Builder B;
    B.dims.assign(site_dims, site_dims + nsites);
    for (int64_t d : B.dims)
      if (d < 1 || d > INT32_MAX) fail(QOB_ERR_ARG, "qob_expect_lazyket: bad site dimension");
    B.walk(*op->node, c128{1.0, 0.0});
    std::vector<int64_t> off(nsites);
    int64_t stride = 0;
    for (int i = 0; i < nsites; ++i) {
      off[i] = stride;
      stride += B.dims[i];
    }
    if (nstates == 0) return QOB_OK;
    const size_t smem = B.obs.size() * 16 + kKetThreads * 16 + (size_t)nsites * 8;
    if (smem > 200 * 1024) fail(QOB_ERR_UNSUPPORTED, "qob_expect_lazyket: too many distinct site observables");
    DeviceBuf d_off, d_dim, d_obs, d_rp, d_col, d_val, d_terms, d_tobs;
    d_off.upload(off.data(), off.size() * 8);
    d_dim.upload(B.dims.data(), B.dims.size() * 8);
    auto up = [](DeviceBuf& b, const void* p, size_t n) {
      if (n == 0) b.alloc(16);
      else b.upload(p, n);
    };
    up(d_obs, B.obs.data(), B.obs.size() * sizeof(SiteObs));
    up(d_rp, B.rowptr.data(), B.rowptr.size() * 4);
    up(d_col, B.col.data(), B.col.size() * 4);
    up(d_val, B.val.data(), B.val.size() * 16);
    up(d_terms, B.terms.data(), B.terms.size() * sizeof(KetTerm));
    up(d_tobs, B.term_obs.data(), B.term_obs.size() * 4);
    cudaStream_t s = (cudaStream_t)stream;
    if (smem > 48 * 1024) {
      if (dtype == QOB_C128)
        QOB_CUDA(cudaFuncSetAttribute(k_lazyket_expect<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      else
        QOB_CUDA(cudaFuncSetAttribute(k_lazyket_expect<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
#define QOB_KET_ARGS                                                                                          \
  stride, nsites, (const int64_t*)d_off.p, (const int64_t*)d_dim.p, (int)B.obs.size(), (const SiteObs*)d_obs.p, \
      (const int32_t*)d_rp.p, (const int32_t*)d_col.p, (const double2*)d_val.p, (int)B.terms.size(),        \
      (const KetTerm*)d_terms.p, (const int32_t*)d_tobs.p, (double2*)result
    if (dtype == QOB_C128)
      k_lazyket_expect<double2><<<(unsigned)nstates, kKetThreads, smem, s>>>((const double2*)kets, QOB_KET_ARGS);
    else
      k_lazyket_expect<float2><<<(unsigned)nstates, kKetThreads, smem, s>>>((const float2*)kets, QOB_KET_ARGS);
#undef QOB_KET_ARGS
    QOB_LAUNCHED();
    // the tables are freed on return: wait for the kernel
    QOB_CUDA(cudaStreamSynchronize(s));
    return QOB_OK;
  } catch (const qob::Error& e) {
    ctx->c.err = e.msg;
    return e.code;
  }
}
