// Operator networks from sums of product terms, and the finite-difference
// stencils built from them, behind the C ABI (so a caller without this
// package's host code gets the same operators).
//
// Reference: ITensorNetworks' ttn(OpSum, s; cutoff) as the reference calls it
// (src/elementary_operators.jl:114,119,151), the carry-string shift OpSums
// (:59-103) with their boundary terms (:32-57), and stencil (:122-160).
//
// A term is a coefficient and a set of site factors (a base x base matrix
// M[out, in] on one digit leg; identity elsewhere).  The terms become a
// block-diagonal direct sum (bond dimension = number of terms; the
// coefficient sits on vertex 0), built on the host, uploaded, and compressed
// on the device by the truncation sweep with the relative cutoff.  Long term
// lists go in blocks of 64: each block is compressed, then added to the
// running sum, which is compressed again, so no uncompressed bond exceeds a
// block plus the running rank.
#include <cstring>
#include <map>
#include <vector>

#include "common.cuh"

namespace tnfa {

Topo topo_from_abi(const tnfa_topology* t);                                          // core.cu
tnfa_net* direct_sum(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g);            // algebra.cu
tnfa_net* truncate_net(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_trunc_params& p);  // ttn.cu

namespace {

constexpr int kOpBlock = 64;

struct Factor {
  int leg;                 // global leg index of the function topology
  std::vector<double> m;   // base x base, row-major M[out, in]
};
struct Term {
  double coef;
  std::vector<Factor> f;
};

struct NetOwn {
  tnfa_net* p = nullptr;
  explicit NetOwn(tnfa_net* q = nullptr) : p(q) {}
  NetOwn(const NetOwn&) = delete;
  NetOwn& operator=(const NetOwn&) = delete;
  ~NetOwn() {
    if (p) tnfa_net_destroy(p);
  }
  tnfa_net* release() {
    tnfa_net* q = p;
    p = nullptr;
    return q;
  }
};

// The operator topology on the function's tree: every digit leg becomes a
// fused (out, in) leg of dim base^2, every bond has dim `bond` (1 at roots).
Topo op_topo(const Topo& F, int bond) {
  Topo O = F;
  for (int l = 0; l < F.leg_off[F.V]; ++l) {
    O.leg_dim[l] = F.leg_dim[l] * F.leg_dim[l];
    O.leg_kind[l] = TNFA_LEG_OPERATOR;
  }
  for (int v = 0; v < F.V; ++v) O.link[v] = F.parent[v] < 0 ? 1 : bond;
  O.finalize();
  return O;
}

// Direct sum of the terms [t0, t1) as an uncompressed operator network.
tnfa_net* terms_direct_sum(tnfa_ctx* ctx, const Topo& F, const std::vector<Term>& terms, size_t t0,
                           size_t t1) {
  const int T = (int)(t1 - t0);
  const Topo O = op_topo(F, T);
  std::vector<double> h((size_t)O.n_elem, 0.0);
  for (int v = 0; v < F.V; ++v) {
    const int l0 = F.leg_off[v], nl = F.leg_off[v + 1] - l0;
    const int64_t sd = O.site_dim[v];
    const int nch = (int)F.children[v].size();
    const bool root = F.parent[v] < 0;
    // bond strides of the canonical layout [sites][parent][children...]
    int64_t bstride = 1;  // stride of the last child bond
    std::vector<int64_t> cstride(nch);
    for (int c = nch - 1; c >= 0; --c) {
      cstride[c] = bstride;
      bstride *= T;
    }
    const int64_t pstride = bstride;            // parent bond stride
    const int64_t sstride = pstride * (root ? 1 : T);  // site index stride
    std::vector<double> site((size_t)sd);
    for (int t = 0; t < T; ++t) {
      const Term& tm = terms[t0 + t];
      // the term's site tensor at v: outer product over v's legs of the fused
      // (out, in) factor (identity where the term has none)
      std::fill(site.begin(), site.end(), 0.0);
      site[0] = 1.0;
      int64_t cur = 1;
      for (int k = 0; k < nl; ++k) {
        const int leg = l0 + k, b = F.leg_dim[leg];
        std::vector<double> m((size_t)b * b, 0.0);
        bool found = false;
        for (const Factor& fc : tm.f)
          if (fc.leg == leg) {
            m = fc.m;
            found = true;
          }
        if (!found)
          for (int i = 0; i < b; ++i) m[(size_t)i * b + i] = 1.0;
        std::vector<double> nxt((size_t)cur * b * b);
        for (int64_t i = 0; i < cur; ++i)
          for (int j = 0; j < b * b; ++j) nxt[(size_t)(i * b * b + j)] = site[(size_t)i] * m[(size_t)j];
        std::copy(nxt.begin(), nxt.end(), site.begin());
        cur *= (int64_t)b * b;
      }
      const double cf = v == 0 ? tm.coef : 1.0;
      int64_t bo = root ? 0 : (int64_t)t * pstride;
      for (int c = 0; c < nch; ++c) bo += (int64_t)t * cstride[c];
      for (int64_t s = 0; s < sd; ++s) h[(size_t)(O.off[v] + s * sstride + bo)] += site[(size_t)s] * cf;
    }
  }
  tnfa_net* out = new_net(ctx, O, TNFA_F64);
  TNFA_CUDA(cudaMemcpyAsync(out->d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  return out;
}

tnfa_net* compress(tnfa_ctx* ctx, const tnfa_net* op, double cutoff) {
  const tnfa_trunc_params p{cutoff, 0, 1, 0, TNFA_PREC_F64};
  return truncate_net(ctx, op, p);
}

// The terms as one compressed operator network; vertices in `scale_v` are
// multiplied by `scale` (the stencil's base^power) before the last
// compression.
tnfa_net* build_operator(tnfa_ctx* ctx, const Topo& F, const std::vector<Term>& terms, double cutoff,
                         const std::vector<int>& scale_v, double scale) {
  TNFA_CHECK(!terms.empty(), TNFA_ERR_INVALID_ARGUMENT, "an empty term list has no operator");
  auto scale_all = [&](tnfa_net* n) {
    for (int v : scale_v) TNFA_CHECK(tnfa_net_scale(ctx, n, v, scale, 0.0) == TNFA_OK, TNFA_ERR_CUDA, "scale");
  };
  if (terms.size() <= (size_t)kOpBlock) {
    NetOwn op(terms_direct_sum(ctx, F, terms, 0, terms.size()));
    scale_all(op.p);
    if (terms.size() == 1) return op.release();
    return compress(ctx, op.p, cutoff);
  }
  NetOwn acc;
  for (size_t b0 = 0; b0 < terms.size(); b0 += kOpBlock) {
    const size_t b1 = std::min(terms.size(), b0 + kOpBlock);
    NetOwn part(terms_direct_sum(ctx, F, terms, b0, b1));
    if (b1 - b0 > 1) {
      NetOwn c(compress(ctx, part.p, cutoff));
      std::swap(part.p, c.p);
    }
    if (!acc.p) {
      std::swap(acc.p, part.p);
    } else {
      NetOwn sum(direct_sum(ctx, acc.p, part.p));
      NetOwn c(compress(ctx, sum.p, cutoff));
      std::swap(acc.p, c.p);
    }
  }
  scale_all(acc.p);
  return acc.release();
}

// ------------------------------------------------ stencil OpSum terms ----
const double kDplus[4] = {0, 1, 0, 0};  // M[out, in] (src/digit_inds.jl:35-58)
const double kDminus[4] = {0, 0, 1, 0};
const double kDdn[4] = {1, 0, 0, 0};
const double kDup[4] = {0, 0, 0, 1};

struct Digits {
  std::map<int, int> leg_of;  // digit -> global leg of variable `dim`
  int L = 0;
};

Digits digits_of(const Topo& F, int dim) {
  Digits D;
  for (int l = 0; l < F.leg_off[F.V]; ++l)
    if (F.leg_var[l] == dim && F.leg_kind[l] == TNFA_LEG_REAL) {
      TNFA_CHECK(F.leg_dim[l] == 2, TNFA_ERR_UNSUPPORTED, "shift operators need base 2");
      TNFA_CHECK(D.leg_of.count(F.leg_digit[l]) == 0, TNFA_ERR_TOPOLOGY, "a digit appears twice");
      D.leg_of[F.leg_digit[l]] = l;
    }
  D.L = (int)D.leg_of.size();
  TNFA_CHECK(D.L >= 1, TNFA_ERR_INVALID_ARGUMENT, "the variable has no digits");
  for (int k = 1; k <= D.L; ++k)
    TNFA_CHECK(D.leg_of.count(k) == 1, TNFA_ERR_TOPOLOGY, "digits of the variable are not 1..L");
  return D;
}

Factor fac(const Digits& D, int digit, const double* m) {
  return Factor{D.leg_of.at(digit), std::vector<double>(m, m + 4)};
}

// f(x + (n+1) delta) (forward) or f(x - (n+1) delta) with carries, and the
// boundary term (src/elementary_operators.jl:32-103).
void shift_terms(const Digits& D, int n, bool fwd, int boundary, double w, std::vector<Term>& out) {
  const double* up = fwd ? kDplus : kDminus;
  const double* down = fwd ? kDminus : kDplus;
  const int top = D.L - n;
  TNFA_CHECK(top >= 1, TNFA_ERR_INVALID_ARGUMENT, "shift longer than the grid");
  std::map<int, const double*> str{{top, up}};
  auto emit = [&](double c, const std::map<int, const double*>& s) {
    Term t{c, {}};
    for (auto& kv : s) t.f.push_back(fac(D, kv.first, kv.second));
    out.push_back(t);
  };
  emit(w, str);
  for (int i = top; i > 1; --i) {
    str[i] = down;
    str[i - 1] = up;
    emit(w, str);
  }
  if (boundary == TNFA_BC_NEUMANN || boundary == TNFA_BC_PERIODIC) {
    std::map<int, const double*> b;
    const double* m = boundary == TNFA_BC_NEUMANN ? (fwd ? kDup : kDdn) : (fwd ? kDminus : kDplus);
    for (int j = 1; j <= top; ++j) b[j] = m;
    emit(w, b);
  } else {
    TNFA_CHECK(boundary == TNFA_BC_DIRICHLET, TNFA_ERR_INVALID_ARGUMENT, "unknown boundary condition");
  }
}

}  // namespace
}  // namespace tnfa

using namespace tnfa;

int tnfa_op_from_terms(tnfa_ctx* ctx, const tnfa_topology* topo, int32_t n_terms, const double* coefs,
                       const int32_t* n_factors, const int32_t* factor_leg, const double* factor_mat,
                       double cutoff, tnfa_net** op) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CHECK(topo && op && coefs && n_factors && n_terms >= 1, TNFA_ERR_INVALID_ARGUMENT,
             "op_from_terms: null argument or no terms");
  TNFA_CHECK(cutoff >= 0, TNFA_ERR_INVALID_ARGUMENT, "negative cutoff");
  const Topo F = topo_from_abi(topo);
  const int nlegs = F.leg_off[F.V];
  for (int l = 0; l < nlegs; ++l)
    TNFA_CHECK(F.leg_kind[l] != TNFA_LEG_OPERATOR, TNFA_ERR_INVALID_ARGUMENT,
               "op_from_terms takes the function's topology (digit legs), not an operator's");
  std::vector<Term> terms(n_terms);
  int64_t k = 0, moff = 0;
  for (int t = 0; t < n_terms; ++t) {
    TNFA_CHECK(n_factors[t] >= 0, TNFA_ERR_INVALID_ARGUMENT, "negative factor count");
    TNFA_CHECK(n_factors[t] == 0 || (factor_leg && factor_mat), TNFA_ERR_INVALID_ARGUMENT, "null factors");
    terms[t].coef = coefs[t];
    for (int f = 0; f < n_factors[t]; ++f, ++k) {
      const int leg = factor_leg[k];
      TNFA_CHECK(leg >= 0 && leg < nlegs, TNFA_ERR_INVALID_ARGUMENT, "factor leg out of range");
      for (const Factor& o : terms[t].f)
        TNFA_CHECK(o.leg != leg, TNFA_ERR_INVALID_ARGUMENT, "two factors of one term on the same leg");
      const int b = F.leg_dim[leg];
      terms[t].f.push_back(Factor{leg, std::vector<double>(factor_mat + moff, factor_mat + moff + (int64_t)b * b)});
      moff += (int64_t)b * b;
    }
  }
  *op = build_operator(ctx, F, terms, cutoff, {}, 1.0);
  TNFA_API_END
}

namespace {
// The stencil's product terms (src/elementary_operators.jl:122-160, before
// the base^power scaling, which acts on vertices).
std::vector<Term> stencil_terms(const Topo& F, int dim, const double* weights, int left_bc, int right_bc) {
  TNFA_CHECK(F.roots().size() == 1, TNFA_ERR_UNSUPPORTED, "shift operators need a tree");
  const Digits D = digits_of(F, dim);
  std::vector<Term> terms;
  terms.push_back(Term{weights[2], {}});  // the identity, always present (possibly 0)
  for (int i = 0; i < 2; ++i)
    if (weights[i] != 0) shift_terms(D, i == 0 ? 1 : 0, true, right_bc, weights[i], terms);
  for (int i = 3; i < 5; ++i)
    if (weights[i] != 0) shift_terms(D, i == 4 ? 1 : 0, false, left_bc, weights[i], terms);
  return terms;
}
}  // namespace

int tnfa_op_stencil_terms(const tnfa_topology* topo, int32_t dim, const double* weights, int32_t left_bc,
                          int32_t right_bc, int32_t max_terms, int32_t max_factors, double* coefs,
                          int32_t* n_factors, int32_t* factor_leg, double* factor_mat, int32_t* n_terms,
                          int32_t* n_factors_total) {
  TNFA_API_BEGIN(nullptr);
  TNFA_CHECK(topo && weights && n_terms && n_factors_total, TNFA_ERR_INVALID_ARGUMENT,
             "op_stencil_terms: null argument");
  const Topo F = topo_from_abi(topo);
  const std::vector<Term> terms = stencil_terms(F, dim, weights, left_bc, right_bc);
  int64_t nf = 0;
  for (const Term& t : terms) nf += (int64_t)t.f.size();
  *n_terms = (int32_t)terms.size();
  *n_factors_total = (int32_t)nf;
  if (max_terms < (int)terms.size() || max_factors < nf) return TNFA_OK;  // sizes only
  TNFA_CHECK(coefs && n_factors && (nf == 0 || (factor_leg && factor_mat)), TNFA_ERR_INVALID_ARGUMENT,
             "op_stencil_terms: null output");
  int64_t k = 0;
  for (size_t t = 0; t < terms.size(); ++t) {
    coefs[t] = terms[t].coef;
    n_factors[t] = (int32_t)terms[t].f.size();
    for (const Factor& f : terms[t].f) {
      factor_leg[k] = f.leg;
      std::copy(f.m.begin(), f.m.end(), factor_mat + 4 * k);  // base 2: 2 x 2 each
      ++k;
    }
  }
  TNFA_API_END
}

int tnfa_op_build_stencil(tnfa_ctx* ctx, const tnfa_topology* topo, int32_t dim, const double* weights,
                          int32_t delta_power, int32_t left_bc, int32_t right_bc, int32_t scale, double cutoff,
                          tnfa_net** op) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CHECK(topo && weights && op, TNFA_ERR_INVALID_ARGUMENT, "op_build_stencil: null argument");
  TNFA_CHECK(cutoff >= 0 && delta_power >= 0, TNFA_ERR_INVALID_ARGUMENT, "negative cutoff or power");
  const Topo F = topo_from_abi(topo);
  // shifts [x+2d, x+d, x, x-d, x-2d] (src/elementary_operators.jl:122-160)
  const std::vector<Term> terms = stencil_terms(F, dim, weights, left_bc, right_bc);
  std::vector<int> sv;
  if (scale)
    for (int v = 0; v < F.V; ++v)
      for (int l = F.leg_off[v]; l < F.leg_off[v + 1]; ++l)
        if (F.leg_var[l] == dim && F.leg_kind[l] == TNFA_LEG_REAL) {
          sv.push_back(v);
          break;
        }
  *op = build_operator(ctx, F, terms, cutoff, sv, std::ldexp(1.0, delta_power));
  TNFA_API_END
}
