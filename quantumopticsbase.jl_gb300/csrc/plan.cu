// plan.cu -- compiles an operator tree into the device form the kernels run.
//
// The reference evaluates mul!(out, H::LazySum, psi, a, b) as one pass over
// `out` per term (src/operators_lazysum.jl:189-200), each term a recursive
// gather over the subsystems (src/operators_lazytensor.jl:652-685) or a chain
// of mode products (:443-488).  Here every term whose factors are small is
// folded into one fused gather:
//
//   * terms are flattened through nested LazySums with their coefficients;
//   * each LazyTensor term becomes a local operator on its support (the
//     subsystems carrying non-identity factors), expanded as a Kronecker
//     product of the factors' row lists;
//   * terms with the same support are summed into one local operator ("group");
//   * on bases whose left and right shapes agree, every diagonal entry of every
//     group is moved into one merged diagonal, built on the device;
//   * a full-space SparseOperator is a group whose support is every subsystem,
//     i.e. a CSR SpMV / SpMM.
//
// The values are linear in the LazySum factors, so each stored value keeps the
// list of (term, product) contributions it came from; set_factors re-evaluates
// them without re-expanding the terms.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

#include "qob_internal.h"

namespace qob {

namespace {

struct RowList {
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> ptr;  // rows + 1
  std::vector<int64_t> col;
  std::vector<c128> val;
};

// Row-gather (CSR) form of a leaf factor as it acts on the given side:
// LEFT uses F, RIGHT uses transpose(F) (no conjugation: the `op_transform =
// transpose` of src/operators_lazytensor.jl:569,604).  F is the stored matrix,
// conjugate-transposed when the operator is an adjoint.
RowList leaf_rows(const OpNode& f, bool transpose) {
  struct Tr {
    int64_t i, j;
    c128 v;
  };
  std::vector<Tr> t;
  auto push = [&](int64_t r, int64_t c, c128 v) {
    // (r, c) of the stored matrix -> (i, j) of F -> (i, j) of the side's matrix
    int64_t i = r, j = c;
    if (f.adjoint) {
      std::swap(i, j);
      v = cconj(v);
    }
    if (transpose) std::swap(i, j);
    t.push_back({i, j, v});
  };
  switch (f.kind) {
    case Kind::Sparse:
      for (int64_t c = 0; c < f.sn; ++c)
        for (int64_t p = f.colptr[c]; p < f.colptr[c + 1]; ++p) push(f.rowval[p], c, f.vals[p]);
      break;
    case Kind::Dense:
      for (int64_t c = 0; c < f.sn; ++c)
        for (int64_t r = 0; r < f.sm; ++r) {
          c128 v = f.vals[r + c * f.sm];
          if (v.re != 0.0 || v.im != 0.0) push(r, c, v);
        }
      break;
    case Kind::Eye:
      for (int64_t k = 0; k < std::min(f.sm, f.sn); ++k) push(k, k, {1.0, 0.0});
      break;
    default:
      fail(QOB_ERR_UNSUPPORTED, "gemm! of LazyTensor is not implemented for this factor type");
  }
  RowList R;
  R.rows = transpose ? f.n : f.m;
  R.cols = transpose ? f.m : f.n;
  std::stable_sort(t.begin(), t.end(), [](const Tr& a, const Tr& b) {
    return a.i != b.i ? a.i < b.i : a.j < b.j;
  });
  R.ptr.assign(R.rows + 1, 0);
  for (auto& e : t) R.ptr[e.i + 1]++;
  for (int64_t i = 0; i < R.rows; ++i) R.ptr[i + 1] += R.ptr[i];
  for (auto& e : t) {
    R.col.push_back(e.j);
    R.val.push_back(e.v);
  }
  return R;
}

RowList identity_rows(int64_t dout, int64_t din) {
  RowList R;
  R.rows = dout;
  R.cols = din;
  R.ptr.assign(dout + 1, 0);
  for (int64_t j = 0; j < dout; ++j) {
    R.ptr[j + 1] = R.ptr[j];
    if (j < din) {
      R.col.push_back(j);
      R.val.push_back({1.0, 0.0});
      R.ptr[j + 1]++;
    }
  }
  return R;
}

struct FlatTerm {
  TermCoef coef;
  const OpNode* node;
  NodeP keep;
};

c128 coef_value(const TermCoef& c, const OpNode* root) {
  if (c.top < 0) return c.inner;
  return cmul(root->factors[c.top], c.inner);
}

void collect_deps(const OpNode* n, std::vector<std::pair<const OpNode*, uint64_t>>& deps) {
  if (n->kind == Kind::LazySum) deps.push_back({n, n->factors_version});
  if (n->kind == Kind::LazySum || n->kind == Kind::LazyProduct)
    for (auto& c : n->ops) collect_deps(c.get(), deps);
}

void flatten(const NodeP& node, TermCoef coef, bool is_root, std::vector<FlatTerm>& out) {
  if (node->kind == Kind::LazySum) {
    for (size_t k = 0; k < node->ops.size(); ++k) {
      TermCoef c2 = coef;
      if (is_root) {
        c2.top = (int32_t)k;
        c2.inner = {1.0, 0.0};
      } else {
        c2.inner = cmul(c2.inner, node->factors[k]);
      }
      flatten(node->ops[k], c2, false, out);
    }
    return;
  }
  out.push_back({coef, node.get(), node});
}

// A group under construction.
struct GroupBuild {
  std::vector<int> support;        // original support (sorted subsystems)
  std::vector<int> ext;            // support with gaps filled (S')
  std::vector<std::pair<int, int>> runs;  // [lo, hi] subsystem runs of ext
  int64_t nrows = 1;
  struct Raw {
    int64_t r, coloff;
    int32_t term;
    c128 pv;
  };
  std::vector<Raw> raw;
};

struct Shapes {
  std::vector<int64_t> dout, din, sout, sin;
  bool square = true;
};

Shapes make_shapes(const std::vector<int64_t>& out, const std::vector<int64_t>& in) {
  Shapes S;
  S.dout = out;
  S.din = in;
  S.sout.resize(out.size());
  S.sin.resize(in.size());
  int64_t a = 1, b = 1;
  for (size_t i = 0; i < out.size(); ++i) {
    S.sout[i] = a;
    S.sin[i] = b;
    a *= out[i];
    b *= in[i];
  }
  S.square = (out == in);
  return S;
}

// Runs of consecutive subsystems; more than kMaxBlocks runs are merged across
// the cheapest gaps (the gap subsystems then carry identity factors).
void make_runs(GroupBuild& g, const Shapes& S) {
  std::vector<std::pair<int, int>> runs;
  for (int s : g.support) {
    if (!runs.empty() && runs.back().second + 1 == s)
      runs.back().second = s;
    else
      runs.push_back({s, s});
  }
  if (runs.empty()) runs.clear();
  while ((int)runs.size() > kMaxBlocks) {
    size_t best = 0;
    double bestcost = 1e300;
    for (size_t i = 0; i + 1 < runs.size(); ++i) {
      double c = 1;
      for (int s = runs[i].second + 1; s < runs[i + 1].first; ++s) c *= (double)S.dout[s];
      if (c < bestcost) {
        bestcost = c;
        best = i;
      }
    }
    runs[best].second = runs[best + 1].second;
    runs.erase(runs.begin() + best + 1);
  }
  g.runs = runs;
  g.ext.clear();
  for (auto& r : runs)
    for (int s = r.first; s <= r.second; ++s) g.ext.push_back(s);
  g.nrows = 1;
  for (int s : g.ext) g.nrows *= S.dout[s];
}

// Expand a term's Kronecker product over the group's extended support.
void expand_term(GroupBuild& g, const Shapes& S, const std::vector<const RowList*>& rl, int32_t term) {
  const size_t ns = g.ext.size();
  std::vector<int64_t> lstr(ns);
  int64_t a = 1;
  for (size_t i = 0; i < ns; ++i) {
    lstr[i] = a;
    a *= S.dout[g.ext[i]];
  }
  // iterate over local output rows r (mixed radix over ext, first fastest)
  std::vector<int64_t> digit(ns, 0);
  for (int64_t r = 0; r < g.nrows; ++r) {
    // decompose r
    int64_t t = r;
    for (size_t i = 0; i < ns; ++i) {
      digit[i] = t % S.dout[g.ext[i]];
      t /= S.dout[g.ext[i]];
    }
    // nested loop over entries of each factor's row digit[i]
    std::vector<int64_t> pos(ns), end(ns), beg(ns);
    bool empty = false;
    for (size_t i = 0; i < ns; ++i) {
      beg[i] = rl[i]->ptr[digit[i]];
      end[i] = rl[i]->ptr[digit[i] + 1];
      pos[i] = beg[i];
      if (beg[i] == end[i]) empty = true;
    }
    if (empty) continue;
    while (true) {
      int64_t coloff = 0;
      c128 pv{1.0, 0.0};
      for (size_t i = 0; i < ns; ++i) {
        coloff += rl[i]->col[pos[i]] * S.sin[g.ext[i]];
        pv = cmul(pv, rl[i]->val[pos[i]]);
      }
      if (pv.re != 0.0 || pv.im != 0.0) g.raw.push_back({r, coloff, term, pv});
      // advance (first subsystem fastest, the order of the reference's recursion
      // does not matter for one output row: each (row, col) pair is unique)
      size_t i = 0;
      for (; i < ns; ++i) {
        if (++pos[i] < end[i]) break;
        pos[i] = beg[i];
      }
      if (i == ns) break;
    }
  }
}

template <class T>
void upload_vec(DeviceBuf& b, const std::vector<T>& v) {
  if (v.empty()) {
    b.alloc(16);
    return;
  }
  b.upload(v.data(), v.size() * sizeof(T));
}

GGroup make_desc(const GroupBuild& g, const Shapes& S, int32_t rowptr_off) {
  GGroup d;
  std::memset(&d, 0, sizeof(d));
  d.nblk = (int32_t)g.runs.size();
  d.nrows = (int32_t)g.nrows;
  d.rowptr_off = rowptr_off;
  int64_t ls = 1;
  for (size_t b = 0; b < g.runs.size(); ++b) {
    int64_t mod = 1;
    for (int s = g.runs[b].first; s <= g.runs[b].second; ++s) mod *= S.dout[s];
    d.div[b] = (uint32_t)S.sout[g.runs[b].first];
    d.mod[b] = (uint32_t)mod;
    d.lstride[b] = (uint32_t)ls;
    d.mdiv[b] = lemire_magic(d.div[b]);
    d.mmod[b] = lemire_magic(d.mod[b]);
    ls *= mod;
  }
  // power-of-two strides (spin-1/2 chains, qubit registers): shifts and masks
  auto log2_exact = [](uint64_t v) -> int {
    if (v == 0 || (v & (v - 1))) return -1;
    int k = 0;
    while ((uint64_t(1) << k) < v) ++k;
    return k;
  };
  d.pow2 = 1;
  for (int b = 0; b < d.nblk; ++b) {
    const int a = log2_exact(d.div[b]), m = log2_exact(d.mod[b]), l = log2_exact(d.lstride[b]);
    if (a < 0 || m < 0 || l < 0) {
      d.pow2 = 0;
      break;
    }
    d.shifts[b] = (uint32_t)a | ((uint32_t)m << 8) | ((uint32_t)l << 16);
  }
  for (int s : g.ext) {
    if (s < 32)
      d.support_lo |= (1u << s);
    else
      d.support_hi |= (1u << (s - 32));
  }
  return d;
}

}  // namespace

// ---------------------------------------------------------------------------
// gather plan construction
// ---------------------------------------------------------------------------

namespace {

struct GatherBuilder {
  Shapes S;
  std::vector<GroupBuild> groups;
  std::map<std::vector<int>, int> by_support;
  std::vector<TermCoef> terms;

  int group_for(const std::vector<int>& support) {
    auto it = by_support.find(support);
    if (it != by_support.end()) return it->second;
    GroupBuild g;
    g.support = support;
    make_runs(g, S);
    groups.push_back(std::move(g));
    by_support[support] = (int)groups.size() - 1;
    return (int)groups.size() - 1;
  }
};

// Slot of the merged structure: all contributions to one (group, row, coloff).
struct Slot {
  int group;
  int64_t r, coloff;
  bool diag;
  int64_t first, count;  // range in the sorted contribution array
};

}  // namespace

static void finalize_gather(GatherPlan& gp, GatherBuilder& B, const OpNode* root, int precision,
                            int64_t m, int64_t n);

// Evaluate slot values from contributions and (re)upload the device arrays.
// Structure (rowptr / coloff) is rebuilt when the set of nonzero slots changes.
struct GatherHost {
  std::vector<GroupBuild> groups;  // runs / ext kept; raw emptied after sorting
  std::vector<Slot> slots;
  std::vector<Contribution> contrib;  // sorted by slot
  Shapes S;
  std::vector<uint8_t> live;  // current nonzero pattern of off-diagonal slots
  // where each slot's value is stored on the device (-1: not stored)
  std::vector<int32_t> dst_val, dst_ell, dst_diag;
  std::vector<uint8_t> group_imag;  // phased plans: group stores imaginary parts
};

// ---------------------------------------------------------------------------

static std::vector<c128> eval_slots(const GatherHost& H, const std::vector<TermCoef>& terms,
                                    const OpNode* root) {
  std::vector<c128> coef(terms.size());
  for (size_t t = 0; t < terms.size(); ++t) coef[t] = coef_value(terms[t], root);
  std::vector<c128> v(H.slots.size(), c128{0.0, 0.0});
  for (size_t s = 0; s < H.slots.size(); ++s) {
    c128 acc{0.0, 0.0};
    for (int64_t k = 0; k < H.slots[s].count; ++k) {
      const Contribution& c = H.contrib[H.slots[s].first + k];
      acc = cadd(acc, cmul(coef[c.term], c.pv));
    }
    v[s] = acc;
  }
  return v;
}


// keep: off-diagonal slots stored even where their value is zero (a factor
// table's union pattern); complex: store complex values even if all are real.
static void upload_structure(GatherPlan& gp, GatherHost& H, const std::vector<c128>& val_in,
                             int precision, const std::vector<uint8_t>* keep = nullptr,
                             bool complex = false) {
  const bool square = H.S.square;
  const std::vector<c128>& val = val_in;
  // live pattern of off-diagonal slots
  H.live.assign(H.slots.size(), 0);
  for (size_t s = 0; s < H.slots.size(); ++s)
    if (!H.slots[s].diag && (val[s].re != 0.0 || val[s].im != 0.0 || (keep && (*keep)[s]))) H.live[s] = 1;
  H.dst_val.assign(H.slots.size(), -1);
  H.dst_ell.assign(H.slots.size(), -1);
  H.dst_diag.assign(H.slots.size(), -1);
  // realness
  bool real = !complex;
  for (size_t s = 0; s < H.slots.size(); ++s)
    if (val[s].im != 0.0) real = false;
  gp.real_vals = real;
  gp.td_ready = false;  // destinations change with the structure
  // phased: every group's stored values either all real or all imaginary (the
  // diagonal may be complex); the stored value is then one real number
  H.group_imag.assign(H.groups.size(), 0);
  bool phased = !real && !complex && square;
  if (phased) {
    std::vector<uint8_t> has_re(H.groups.size(), 0), has_im(H.groups.size(), 0);
    for (size_t s = 0; s < H.slots.size(); ++s) {
      if (H.slots[s].diag || !H.live[s]) continue;
      if (val[s].re != 0.0) has_re[H.slots[s].group] = 1;
      if (val[s].im != 0.0) has_im[H.slots[s].group] = 1;
    }
    for (size_t gi = 0; gi < H.groups.size() && phased; ++gi) {
      if (has_re[gi] && has_im[gi]) phased = false;
      H.group_imag[gi] = has_im[gi];
    }
    if (!phased) H.group_imag.assign(H.groups.size(), 0);
  }
  gp.phased = phased;
  const bool store_real = real || phased;
  // the stored number of each off-diagonal slot (phased: the imaginary part in imaginary groups)
  auto stored = [&](size_t s) -> c128 {
    if (phased && !H.slots[s].diag) return H.group_imag[H.slots[s].group] ? c128{val[s].im, 0.0} : c128{val[s].re, 0.0};
    return val[s];
  };
  // per group: live entries ordered by (r, coloff)
  std::vector<GGroup> descs;
  std::vector<int32_t> rowptr, coloff, pos_slot;
  std::vector<c128> vals;
  struct EllHost {
    int32_t col;
    c128 v;
  };
  std::vector<EllHost> ell;
  // the device tables index entries, rows and slots with 32-bit integers
  constexpr int64_t kMaxTable = INT32_MAX;
  if ((int64_t)H.slots.size() > kMaxTable) fail(QOB_ERR_UNSUPPORTED, "more than 2^31-1 stored entries");
  size_t s0 = 0;
  for (size_t gi = 0; gi < H.groups.size(); ++gi) {
    size_t s1 = s0;
    while (s1 < H.slots.size() && H.slots[s1].group == (int)gi) ++s1;
    int64_t nlive = 0;
    for (size_t s = s0; s < s1; ++s) nlive += H.live[s];
    if (nlive > 0) {
      const GroupBuild& g = H.groups[gi];
      if ((int64_t)coloff.size() + nlive > kMaxTable || (int64_t)rowptr.size() + g.nrows + 1 > kMaxTable)
        fail(QOB_ERR_UNSUPPORTED, "more than 2^31-1 stored entries or rows in the compiled tables");
      GGroup d = make_desc(g, H.S, (int32_t)rowptr.size());
      d.imag = H.group_imag[gi];
      std::vector<int32_t> cnt(g.nrows + 1, 0);
      for (size_t s = s0; s < s1; ++s)
        if (H.live[s]) cnt[H.slots[s].r + 1]++;
      int32_t base = (int32_t)coloff.size();
      for (int64_t r = 0; r < g.nrows; ++r) cnt[r + 1] += cnt[r];
      for (int64_t r = 0; r <= g.nrows; ++r) rowptr.push_back(base + cnt[r]);
      for (size_t s = s0; s < s1; ++s)
        if (H.live[s]) {
          H.dst_val[s] = (int32_t)vals.size();
          pos_slot.push_back((int32_t)s);
          coloff.push_back((int32_t)H.slots[s].coloff);
          vals.push_back(stored(s));
        }
      // rows with at most kMaxEllWidth entries also get fixed-width slots
      int32_t width = 0;
      for (int64_t r = 0; r < g.nrows; ++r) width = std::max<int32_t>(width, cnt[r + 1] - cnt[r]);
      if (width <= kMaxEllWidth && (int64_t)ell.size() + g.nrows * width < (int64_t(1) << 30)) {
        d.width = width;
        d.ell_off = (int32_t)ell.size();
        for (int64_t r = 0; r < g.nrows; ++r) {
          int32_t k = 0;
          for (int32_t p = cnt[r]; p < cnt[r + 1]; ++p, ++k) {
            H.dst_ell[pos_slot[base + p]] = (int32_t)ell.size();
            ell.push_back({coloff[base + p], vals[base + p]});
          }
          for (; k < width; ++k) ell.push_back({0, c128{0.0, 0.0}});
        }
      }
      descs.push_back(d);
    }
    s0 = s1;
  }
  gp.ngroups = (int)descs.size();
  gp.nentries = (int64_t)coloff.size();
  gp.all_ell = true;
  gp.all_w1 = true;
  for (auto& d : descs) {
    gp.all_ell &= (d.width > 0);
    gp.all_w1 &= (d.width == 1);
  }
  // compact form: every group one run of power-of-two subsystems with one slot per row
  gp.fast = square && !descs.empty();
  std::vector<int4> fastg;
  for (auto& d : descs) {
    if (!(d.pow2 && d.nblk == 1 && d.width == 1)) gp.fast = false;
    fastg.push_back(make_int4((int)(d.shifts[0] & 0xffu), (int)(d.mod[0] - 1u), d.ell_off, d.imag));
  }
  if (gp.fast) upload_vec(gp.fastg, fastg);
  gp.square = square;
  upload_vec(gp.groups, descs);
  upload_vec(gp.rowptr, rowptr);
  upload_vec(gp.coloff, coloff);
  // values in the plan precision, real or complex; double-float plans store
  // (hi, lo) float pairs in the same sizes
  auto split = [](double v) {
    const float h = (float)v;
    return std::pair<float, float>(h, (float)(v - (double)h));
  };
  if (gp.ff) {
    if (store_real) {
      std::vector<float> v(2 * vals.size());
      for (size_t i = 0; i < vals.size(); ++i) std::tie(v[2 * i], v[2 * i + 1]) = split(vals[i].re);
      upload_vec(gp.vals, v);
    } else {
      std::vector<float> v(4 * vals.size());
      for (size_t i = 0; i < vals.size(); ++i) {
        std::tie(v[4 * i], v[4 * i + 1]) = split(vals[i].re);
        std::tie(v[4 * i + 2], v[4 * i + 3]) = split(vals[i].im);
      }
      upload_vec(gp.vals, v);
    }
  } else if (precision == QOB_C128) {
    if (store_real) {
      std::vector<double> v(vals.size());
      for (size_t i = 0; i < vals.size(); ++i) v[i] = vals[i].re;
      upload_vec(gp.vals, v);
    } else {
      upload_vec(gp.vals, vals);
    }
  } else {
    if (store_real) {
      std::vector<float> v(vals.size());
      for (size_t i = 0; i < vals.size(); ++i) v[i] = (float)vals[i].re;
      upload_vec(gp.vals, v);
    } else {
      std::vector<c64> v(vals.size());
      for (size_t i = 0; i < vals.size(); ++i) v[i] = {(float)vals[i].re, (float)vals[i].im};
      upload_vec(gp.vals, v);
    }
  }
  // fixed-width slots in the plan precision
  gp.ell_slots = (int32_t)ell.size();
  if (gp.ff) {
    if (store_real) {
      std::vector<EllDF> e(ell.size());
      for (size_t i = 0; i < ell.size(); ++i) {
        e[i] = {ell[i].col, 0, {0.f, 0.f}};
        std::tie(e[i].v[0], e[i].v[1]) = split(ell[i].v.re);
      }
      upload_vec(gp.ell, e);
    } else {
      std::vector<EllZF> e(ell.size());
      for (size_t i = 0; i < ell.size(); ++i) {
        e[i] = {ell[i].col, {0, 0, 0}, {0.f, 0.f, 0.f, 0.f}};
        std::tie(e[i].v[0], e[i].v[1]) = split(ell[i].v.re);
        std::tie(e[i].v[2], e[i].v[3]) = split(ell[i].v.im);
      }
      upload_vec(gp.ell, e);
    }
  } else if (precision == QOB_C128) {
    if (store_real) {
      std::vector<EllD> e(ell.size());
      for (size_t i = 0; i < ell.size(); ++i) e[i] = {ell[i].col, 0, ell[i].v.re};
      upload_vec(gp.ell, e);
    } else {
      std::vector<EllZ> e(ell.size());
      for (size_t i = 0; i < ell.size(); ++i) e[i] = {ell[i].col, {0, 0, 0}, {ell[i].v.re, ell[i].v.im}};
      upload_vec(gp.ell, e);
    }
  } else {
    if (store_real) {
      std::vector<EllF> e(ell.size());
      for (size_t i = 0; i < ell.size(); ++i) e[i] = {ell[i].col, (float)ell[i].v.re};
      upload_vec(gp.ell, e);
    } else {
      std::vector<EllC> e(ell.size());
      for (size_t i = 0; i < ell.size(); ++i) e[i] = {ell[i].col, 0, {(float)ell[i].v.re, (float)ell[i].v.im}};
      upload_vec(gp.ell, e);
    }
  }
  // diagonal sources: one descriptor + local table per group that has diagonal slots
  if (square) {
    std::vector<GGroup> dd;
    std::vector<c128> dtab;
    size_t t0 = 0;
    for (size_t gi = 0; gi < H.groups.size(); ++gi) {
      size_t t1 = t0;
      bool any = false;
      while (t1 < H.slots.size() && H.slots[t1].group == (int)gi) {
        any |= H.slots[t1].diag;
        ++t1;
      }
      if (any) {
        const GroupBuild& g = H.groups[gi];
        if ((int64_t)dtab.size() + g.nrows > INT32_MAX)
          fail(QOB_ERR_UNSUPPORTED, "more than 2^31-1 rows in the diagonal tables");
        GGroup d = make_desc(g, H.S, (int32_t)dtab.size());  // rowptr_off = table offset
        std::vector<c128> tab(g.nrows, c128{0.0, 0.0});
        for (size_t s = t0; s < t1; ++s)
          if (H.slots[s].diag) {
            tab[H.slots[s].r] = val[s];
            H.dst_diag[s] = (int32_t)(dtab.size() + H.slots[s].r);
          }
        dtab.insert(dtab.end(), tab.begin(), tab.end());
        dd.push_back(d);
      }
      t0 = t1;
    }
    gp.ndgroups = (int)dd.size();
    gp.has_diag = gp.ndgroups > 0;
    if (gp.has_diag) {
      upload_vec(gp.dgroups, dd);
      upload_vec(gp.dvals, dtab);
      size_t esz = precision == QOB_C128 ? (real ? 8 : 16) : (real ? 4 : 8);
      if (gp.diag.bytes < (size_t)gp.m * esz) gp.diag.alloc((size_t)gp.m * esz);
      launch_build_diag(gp, 0);
      QOB_CUDA(cudaStreamSynchronize(0));
    }
  } else {
    gp.has_diag = false;
    gp.ndgroups = 0;
  }
}

// ---------------------------------------------------------------------------
// plan compilation
// ---------------------------------------------------------------------------

// Merge a LazyTensor's factors into one local operator (fused gather) or keep
// the mode-product chain.  A merged row holds the product of the factors' row
// widths, the chain costs their sum per element plus one pass over the state
// per factor: merge while the product stays within max(16, 2 x sum) -- every
// Pauli / ladder / number product, single dense factors of any size -- and
// chain for several wide (dense) factors, e.g. 64 x 64 and 16 x 16 dense
// factors: 1024 entries per merged row against 80 multiply-adds per element.
// A complex matrix in the plan's storage: ComplexF64, ComplexF32, or for a
// double-float plan (hi, lo) float pairs of the real and imaginary parts.
static void upload_matrix(DeviceBuf& d, const std::vector<c128>& a, const Plan& P) {
  if (P.ff) {
    std::vector<float> q(4 * a.size());
    for (size_t k = 0; k < a.size(); ++k) {
      const float rh = (float)a[k].re, ih = (float)a[k].im;
      q[4 * k] = rh;
      q[4 * k + 1] = (float)(a[k].re - (double)rh);
      q[4 * k + 2] = ih;
      q[4 * k + 3] = (float)(a[k].im - (double)ih);
    }
    upload_vec(d, q);
  } else if (P.precision == QOB_C128) {
    upload_vec(d, a);
  } else {
    std::vector<c64> a32(a.size());
    for (size_t k = 0; k < a.size(); ++k) a32[k] = {(float)a[k].re, (float)a[k].im};
    upload_vec(d, a32);
  }
}

static bool gatherable_factor_sizes(const std::vector<const RowList*>& rl, int64_t nrows) {
  double entries = (double)nrows, prod = 1.0, sum = 0.0;
  for (auto* r : rl) {
    int64_t mx = 0;
    for (int64_t i = 0; i < r->rows; ++i) mx = std::max(mx, r->ptr[i + 1] - r->ptr[i]);
    entries *= (double)std::max<int64_t>(mx, 1);
    prod *= (double)std::max<int64_t>(mx, 1);
    sum += (double)std::max<int64_t>(mx, 1);
  }
  return nrows <= (int64_t(1) << 24) && entries <= double(int64_t(1) << 25) && prod <= std::max(16.0, 2.0 * sum);
}

std::unique_ptr<Plan> compile_plan(Context& ctx, const NodeP& op, int side, int precision);

static std::unique_ptr<Plan> compile_sum(Context& ctx, const NodeP& root, int side, int precision) {
  auto P = std::make_unique<Plan>();
  P->kind = Plan::Kind::Sum;
  P->side = side;
  P->precision = precision == QOB_C128X ? QOB_C128 : precision;
  P->ff = precision == QOB_C128X;
  const bool tr = (side == QOB_RIGHT);
  P->m = tr ? root->n : root->m;  // output vector length
  P->n = tr ? root->m : root->n;  // input vector length
  P->root = root.get();
  collect_deps(root.get(), P->deps);

  std::vector<FlatTerm> terms;
  if (root->kind == Kind::LazySum)
    flatten(root, TermCoef{-1, {1.0, 0.0}}, true, terms);
  else
    terms.push_back({TermCoef{-1, {1.0, 0.0}}, root.get(), root});
  P->nterms_total = (int)terms.size();

  // composite shape: from the LazyTensor terms, else a single subsystem
  std::vector<int64_t> shp_out, shp_in;
  for (auto& t : terms)
    if (t.node->kind == Kind::LazyTensor) {
      const auto& so = tr ? t.node->shape_r : t.node->shape_l;
      const auto& si = tr ? t.node->shape_l : t.node->shape_r;
      if (shp_out.empty()) {
        shp_out = so;
        shp_in = si;
      } else if (so != shp_out || si != shp_in) {
        fail(QOB_ERR_DIM, "LazySum terms act on different composite bases");
      }
    }
  if (shp_out.empty()) {
    shp_out = {P->m};
    shp_in = {P->n};
  }
  if ((int)shp_out.size() > kMaxSites)
    fail(QOB_ERR_UNSUPPORTED, "more than 32 subsystems in one composite basis");
  if (P->m > INT32_MAX || P->n > INT32_MAX) fail(QOB_ERR_UNSUPPORTED, "dimension exceeds 2^31-1");

  GatherBuilder B;
  B.S = make_shapes(shp_out, shp_in);
  std::vector<std::unique_ptr<RowList>> keep;
  const int nsites = (int)shp_out.size();

  for (auto& t : terms) {
    const OpNode* nd = t.node;
    TermCoef coef = t.coef;
    switch (nd->kind) {
      case Kind::LazyTensor: {
        coef.inner = cmul(coef.inner, nd->factor);
        // support: subsystems with factors other than square Eyes
        std::vector<int> support;
        std::vector<const OpNode*> fac_of(nsites, nullptr);
        for (size_t i = 0; i < nd->ops.size(); ++i) {
          const OpNode* f = nd->ops[i].get();
          if (f->kind == Kind::Eye && f->m == f->n) continue;
          if (f->kind != Kind::Sparse && f->kind != Kind::Dense && f->kind != Kind::Eye)
            fail(QOB_ERR_UNSUPPORTED, "gemm! of LazyTensor is not implemented for a lazy factor");
          support.push_back(nd->sites[i]);
          fac_of[nd->sites[i]] = f;
        }
        int gi = B.group_for(support);
        GroupBuild& g = B.groups[gi];
        std::vector<const RowList*> rl;
        for (int s : g.ext) {
          if (fac_of[s]) {
            keep.push_back(std::make_unique<RowList>(leaf_rows(*fac_of[s], tr)));
          } else {
            keep.push_back(std::make_unique<RowList>(identity_rows(B.S.dout[s], B.S.din[s])));
          }
          rl.push_back(keep.back().get());
        }
        if (!gatherable_factor_sizes(rl, g.nrows)) {
          // large dense factors: mode-product chain (the _tp_sum_matmul! structure)
          ModekPass mp;
          mp.coef = coef;
          mp.shape_in = shp_in;
          mp.shape_out = shp_out;
          std::vector<int64_t> cur = shp_in;
          for (size_t i = 0; i < nd->ops.size(); ++i) {
            const OpNode* f = nd->ops[i].get();
            if (f->kind == Kind::Eye && f->m == f->n) continue;
            ModekStep st;
            st.site = nd->sites[i];
            RowList r = leaf_rows(*f, tr);
            st.dout = r.rows;
            st.din = r.cols;
            st.eye = (f->kind == Kind::Eye);
            std::vector<c128> a(st.dout * st.din, c128{0.0, 0.0});
            for (int64_t row = 0; row < r.rows; ++row)
              for (int64_t p = r.ptr[row]; p < r.ptr[row + 1]; ++p) a[row + r.col[p] * st.dout] = r.val[p];
            upload_matrix(st.a, a, *P);
            mp.steps.push_back(std::move(st));
          }
          // non-square subsystems without factors: explicit isometries (:491-514)
          for (int s = 0; s < nsites; ++s) {
            bool used = false;
            for (int q : nd->sites) used |= (q == s);
            if (!used && shp_out[s] != shp_in[s]) {
              ModekStep st;
              st.site = s;
              st.dout = shp_out[s];
              st.din = shp_in[s];
              st.eye = true;
              mp.steps.push_back(std::move(st));
            }
          }
          P->modek.push_back(std::move(mp));
          g.raw.shrink_to_fit();
          break;
        }
        B.terms.push_back(coef);
        expand_term(g, B.S, rl, (int32_t)B.terms.size() - 1);
        break;
      }
      case Kind::Sparse:
      case Kind::Eye:
      case Kind::Dense: {
        bool small_dense = nd->kind == Kind::Dense && nd->m <= 256 && nd->n <= 256;
        if (nd->kind == Kind::Dense && !small_dense) {
          DensePass dp;
          dp.coef = coef;
          dp.m = tr ? nd->n : nd->m;
          dp.n = tr ? nd->m : nd->n;
          std::vector<c128> a(dp.m * dp.n);
          for (int64_t j = 0; j < dp.n; ++j)
            for (int64_t i = 0; i < dp.m; ++i) {
              // element (i, j) of the side's matrix
              int64_t r = i, c = j;
              if (tr) std::swap(r, c);  // transpose(F)
              c128 v;
              if (nd->adjoint)
                v = cconj(nd->vals[c + r * nd->sm]);
              else
                v = nd->vals[r + c * nd->sm];
              a[i + j * dp.m] = v;
            }
          upload_matrix(dp.a, a, *P);
          P->dense.push_back(std::move(dp));
          break;
        }
        // full-space term: support is every subsystem
        std::vector<int> support(nsites);
        for (int s = 0; s < nsites; ++s) support[s] = s;
        int gi = B.group_for(support);
        GroupBuild& g = B.groups[gi];
        RowList r = leaf_rows(*nd, tr);
        if (r.rows != P->m || r.cols != P->n) fail(QOB_ERR_DIM, "operator shape does not match the sum");
        B.terms.push_back(coef);
        int32_t term = (int32_t)B.terms.size() - 1;
        for (int64_t row = 0; row < r.rows; ++row)
          for (int64_t p = r.ptr[row]; p < r.ptr[row + 1]; ++p)
            if (r.val[p].re != 0.0 || r.val[p].im != 0.0) g.raw.push_back({row, r.col[p], term, r.val[p]});
        break;
      }
      case Kind::Fft:
      case Kind::LazyProduct: {
        SubPass sp;
        sp.coef = coef;
        sp.plan = compile_plan(ctx, t.keep, side, precision);
        P->subs.push_back(std::move(sp));
        break;
      }
      case Kind::LazySum:
        fail(QOB_ERR_ARG, "internal: unflattened LazySum");
    }
  }

  bool any_raw = false;
  for (auto& g : B.groups) any_raw |= !g.raw.empty();
  if (any_raw) {
    P->gather = std::make_unique<GatherPlan>();
    P->gather->status = static_cast<unsigned*>(ctx.status.p);
    finalize_gather(*P->gather, B, root.get(), precision, P->m, P->n);
  }
  return P;
}

static void finalize_gather(GatherPlan& gp, GatherBuilder& B, const OpNode* root, int precision,
                            int64_t m, int64_t n) {
  gp.m = m;
  gp.n = n;
  gp.precision = precision == QOB_C128X ? QOB_C128 : precision;
  gp.ff = precision == QOB_C128X;
  gp.terms = B.terms;
  auto hp = std::make_shared<GatherHost>();
  GatherHost& H = *hp;
  H.S = B.S;
  gp.sites.nsites = (int32_t)B.S.dout.size();
  for (size_t s = 0; s < B.S.dout.size(); ++s) {
    gp.sites.dout[s] = (uint32_t)B.S.dout[s];
    gp.sites.sout[s] = (uint32_t)B.S.sout[s];
    gp.sites.din[s] = (uint32_t)B.S.din[s];
    gp.sites.sin[s] = (uint32_t)B.S.sin[s];
    gp.sites.msout[s] = lemire_magic(gp.sites.sout[s]);
    gp.sites.mdout[s] = lemire_magic(gp.sites.dout[s]);
  }
  // sort contributions per group by (r, coloff), keeping term order
  for (size_t gi = 0; gi < B.groups.size(); ++gi) {
    auto& raw = B.groups[gi].raw;
    std::stable_sort(raw.begin(), raw.end(), [](const GroupBuild::Raw& a, const GroupBuild::Raw& b) {
      return a.r != b.r ? a.r < b.r : a.coloff < b.coloff;
    });
    const GroupBuild& g = B.groups[gi];
    // row offset of a local row on a square basis: sum of the block digits times div
    auto rowoff = [&](int64_t r) {
      int64_t off = 0, t = r;
      for (auto& run : g.runs) {
        int64_t mod = 1;
        for (int s = run.first; s <= run.second; ++s) mod *= B.S.dout[s];
        off += (t % mod) * B.S.sout[run.first];
        t /= mod;
      }
      return off;
    };
    for (size_t k = 0; k < raw.size();) {
      size_t e = k;
      while (e < raw.size() && raw[e].r == raw[k].r && raw[e].coloff == raw[k].coloff) ++e;
      Slot s;
      s.group = (int)gi;
      s.r = raw[k].r;
      s.coloff = raw[k].coloff;
      s.diag = B.S.square && raw[k].coloff == rowoff(raw[k].r);
      s.first = (int64_t)H.contrib.size();
      s.count = (int64_t)(e - k);
      for (size_t q = k; q < e; ++q) H.contrib.push_back({raw[q].term, 0, raw[q].pv});
      H.slots.push_back(s);
      k = e;
    }
    raw.clear();
    raw.shrink_to_fit();
  }
  for (auto& g : B.groups) H.groups.push_back(g);
  std::vector<c128> val = eval_slots(H, gp.terms, root);
  upload_structure(gp, H, val, gp.precision);
  gp.host_rec = hp;
}

// precision QOB_C128X: a ComplexF64 plan (P->precision QOB_C128) whose fused
// gathers store and apply their values in double-float arithmetic
std::unique_ptr<Plan> compile_plan(Context& ctx, const NodeP& op, int side, int precision) {
  const int layout = precision == QOB_C128X ? QOB_C128 : precision;
  if (op->kind == Kind::Fft) return compile_fft(op, side, precision);
  if (op->kind == Kind::LazyProduct) {
    auto P = std::make_unique<Plan>();
    P->kind = Plan::Kind::Product;
    P->side = side;
    P->precision = layout;
    P->ff = precision == QOB_C128X;
    const bool tr = (side == QOB_RIGHT);
    P->m = tr ? op->n : op->m;
    P->n = tr ? op->m : op->n;
    P->pfactor = op->factor;
    P->root = op.get();
    collect_deps(op.get(), P->deps);
    const size_t k = op->ops.size();
    for (size_t i = 0; i < k; ++i) {
      // LEFT applies the last operator first; RIGHT the first
      const NodeP& c = tr ? op->ops[i] : op->ops[k - 1 - i];
      P->chain.push_back(compile_plan(ctx, c, side, precision));
    }
    P->nterms_total = (int)k;
    return P;
  }
  return compile_sum(ctx, op, side, precision);
}

bool plan_is_current(const Plan& plan) {
  for (auto& d : plan.deps)
    if (d.first->factors_version != d.second) return false;
  return true;
}

// The contribution record on the device (once per structure).
static void build_td_tables(GatherPlan& gp, const GatherHost& H, size_t nfactors) {
  if (gp.td_ready && gp.td_nfactors == (int32_t)nfactors) return;
  std::vector<TdSlot> sl;
  std::vector<TdContrib> co;
  for (size_t s = 0; s < H.slots.size(); ++s) {
    if (H.dst_val[s] < 0 && H.dst_ell[s] < 0 && H.dst_diag[s] < 0) continue;
    TdSlot d{};
    d.first = (int32_t)co.size();
    d.count = (int32_t)H.slots[s].count;
    d.dst_val = H.dst_val[s];
    d.dst_ell = H.dst_ell[s];
    d.dst_diag = H.dst_diag[s];
    d.part = (gp.phased && !H.slots[s].diag && H.group_imag[H.slots[s].group]) ? 1 : 0;
    for (int64_t k = 0; k < H.slots[s].count; ++k) {
      const Contribution& c = H.contrib[H.slots[s].first + k];
      TdContrib t{};
      t.term = c.term;
      t.pv[0] = c.pv.re;
      t.pv[1] = c.pv.im;
      co.push_back(t);
    }
    sl.push_back(d);
  }
  std::vector<TdTerm> te(gp.terms.size());
  for (size_t t = 0; t < gp.terms.size(); ++t) {
    te[t] = TdTerm{};
    te[t].top = gp.terms[t].top;
    te[t].inner[0] = gp.terms[t].inner.re;
    te[t].inner[1] = gp.terms[t].inner.im;
  }
  upload_vec(gp.td_slots, sl);
  upload_vec(gp.td_contrib, co);
  upload_vec(gp.td_terms, te);
  if (gp.td_factors.bytes < std::max<size_t>(nfactors, 1) * 16) gp.td_factors.alloc(std::max<size_t>(nfactors, 1) * 16);
  gp.td_nslots = (int32_t)sl.size();
  gp.td_nfactors = (int32_t)nfactors;
  gp.td_ready = true;
}

void device_refresh(GatherPlan& g, const double2* factors_dev, cudaStream_t s, const long long* step,
                    long long off, long long nf) {
  if (!g.td_ready) fail(QOB_ERR_STATE, "device refresh without its tables");
  launch_td_values(g, factors_dev, s, step, off, nf);
  if (g.has_diag) launch_build_diag(g, s);
}

// Whether the current structure holds these values: every nonzero
// off-diagonal slot is stored and complex values have complex storage.
static bool structure_holds(const GatherPlan& gp, const GatherHost& H, const std::vector<c128>& val) {
  for (size_t s = 0; s < H.slots.size(); ++s) {
    if (gp.real_vals && val[s].im != 0.0) return false;
    if (!H.slots[s].diag && !H.live[s] && (val[s].re != 0.0 || val[s].im != 0.0)) return false;
    if (gp.phased && !H.slots[s].diag) {
      const bool im = H.group_imag[H.slots[s].group] != 0;
      if (im ? val[s].re != 0.0 : val[s].im != 0.0) return false;
    }
  }
  return true;
}

// Only the root LazySum's factors changed: re-evaluate the gather values.  When
// the stored pattern still holds them, the factors go to the device and the
// values are re-evaluated there, in stream order (no structure upload, no
// synchronisation); otherwise the structure is rebuilt.
void refresh_coefficients(Plan& plan, const OpNode& root, cudaStream_t s) {
  if (plan.gather) {
    GatherPlan& gp = *plan.gather;
    if (!gp.host_rec) fail(QOB_ERR_STATE, "gather plan lost its host record");
    GatherHost& H = *static_cast<GatherHost*>(gp.host_rec.get());
    std::vector<c128> val = eval_slots(H, gp.terms, &root);
    if (structure_holds(gp, H, val)) {
      build_td_tables(gp, H, root.factors.size());
      if (!root.factors.empty())
        QOB_CUDA(cudaMemcpyAsync(gp.td_factors.p, root.factors.data(), root.factors.size() * sizeof(c128),
                                 cudaMemcpyHostToDevice, s));
      device_refresh(gp, (const double2*)gp.td_factors.p, s);
    } else {
      upload_structure(gp, H, val, plan.precision);
    }
  }
  for (auto& d : plan.deps)
    if (d.first == &root) d.second = root.factors_version;
}

void prepare_factor_rows(Plan& plan, const OpNode& root, const double* rows, int64_t nrows) {
  if (!plan.gather) return;
  GatherPlan& gp = *plan.gather;
  if (!gp.host_rec) fail(QOB_ERR_STATE, "gather plan lost its host record");
  GatherHost& H = *static_cast<GatherHost*>(gp.host_rec.get());
  const size_t nf = root.factors.size();
  // union of the nonzero patterns and realness over all rows
  OpNode tmp;
  tmp.factors.resize(nf);
  std::vector<uint8_t> keep(H.slots.size(), 0);
  bool complex = false;
  for (int64_t r = 0; r < nrows; ++r) {
    for (size_t k = 0; k < nf; ++k) tmp.factors[k] = {rows[2 * (r * nf + k)], rows[2 * (r * nf + k) + 1]};
    std::vector<c128> v = eval_slots(H, gp.terms, &tmp);
    for (size_t s = 0; s < v.size(); ++s) {
      if (v[s].re != 0.0 || v[s].im != 0.0) keep[s] = 1;
      if (v[s].im != 0.0) complex = true;
    }
  }
  bool holds = !(gp.real_vals && complex);
  for (size_t s = 0; s < H.slots.size() && holds; ++s)
    if (!H.slots[s].diag && keep[s] && !H.live[s]) holds = false;
  if (!holds) {
    std::vector<c128> val = eval_slots(H, gp.terms, &root);
    upload_structure(gp, H, val, plan.precision, &keep, complex);
  }
  build_td_tables(gp, H, nf);
}

GatherView GatherPlan::view() const {
  GatherView v;
  v.jmul = chunk_multiplier((m + 31) / 32);
  v.m = m;
  v.n = n;
  v.ngroups = ngroups;
  v.square = square ? 1 : 0;
  v.real_vals = real_vals ? 1 : 0;
  v.phased = phased ? 1 : 0;
  v.has_diag = has_diag ? 1 : 0;
  v.groups = (const GGroup*)groups.p;
  v.rowptr = (const int32_t*)rowptr.p;
  v.coloff = (const int32_t*)coloff.p;
  v.vals = vals.p;
  v.diag = diag.p;
  v.ell = ell.p;
  v.ell_slots = ell_slots;
  v.ell_smem = 0;  // decided per launch from the shared-memory budget
  v.all_ell = all_ell ? 1 : 0;
  v.all_w1 = all_w1 ? 1 : 0;
  v.fast = fast ? 1 : 0;
  v.fastg = (const int4*)fastg.p;
  v.block = block;
  v.lane_split = lane_split;
  v.tile_bits = tile_bits;
  v.pairs = pairs;
  v.status = status;
  v.pdl = 0;
  return v;
}

}  // namespace qob
