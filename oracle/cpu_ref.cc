// CPU restatement of the reference's expectation + adjoint-gradient loops,
// used as the timed CPU baseline (TEST INFRASTRUCTURE, never the product).
//
// Follows, per circuit, in complex64 like the reference's simulator:
//   forward ............ tfq_simulate_expectation_op.cc:196-243 (gate by gate)
//   expectation ........ util_qsim.h:142-188: per Pauli term copy the state,
//                        apply the term's Pauli factors, real inner product
//   lambda ............. util_qsim.h:362-414 AccumulateOperators
//   adjoint sweep ...... tfq_adj_grad_op.cc:199-276: psi <- G^dag psi, copy,
//                        zero non-matching controls, apply gradient gate,
//                        2 Re<scratch|lambda>, lambda <- G^dag lambda
// Circuits run in parallel over host threads (ComputeSmall's ParallelFor).
// Gate matrices come in precomputed (the oracle builds them); the reference
// additionally fuses neighbouring gates, which this restatement does not.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Gate {
  int nq, b0, b1;
  uint32_t cmask, cval;
  const float* m;    // 2*D*D floats
  int ngrad;
  const float* dm;   // ngrad * 32 floats
  const int* cols;   // ngrad
};

inline uint32_t ins0(uint32_t i, int b) {
  return ((i >> b) << (b + 1)) | (i & ((1u << b) - 1u));
}

void apply(float* s, int n, const Gate& g, const float* m, bool dagger,
           bool controls = true) {
  const int D = 1 << g.nq;
  float mm[32];
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) {
      int src = dagger ? (c * D + r) : (r * D + c);
      mm[2 * (r * D + c)] = m[2 * src];
      mm[2 * (r * D + c) + 1] = dagger ? -m[2 * src + 1] : m[2 * src + 1];
    }
  const uint32_t cnt = 1u << (n - g.nq);
  for (uint32_t i = 0; i < cnt; ++i) {
    uint32_t idx[4];
    if (g.nq == 1) {
      idx[0] = ins0(i, g.b0);
      idx[1] = idx[0] | (1u << g.b0);
    } else {
      int lo = g.b0 < g.b1 ? g.b0 : g.b1, hi = g.b0 < g.b1 ? g.b1 : g.b0;
      uint32_t b = ins0(ins0(i, lo), hi);
      idx[0] = b;
      idx[1] = b | (1u << g.b1);
      idx[2] = b | (1u << g.b0);
      idx[3] = b | (1u << g.b0) | (1u << g.b1);
    }
    if (controls && (idx[0] & g.cmask) != g.cval) continue;
    float ar[4], ai[4];
    for (int k = 0; k < D; ++k) {
      ar[k] = s[2 * idx[k]];
      ai[k] = s[2 * idx[k] + 1];
    }
    for (int r = 0; r < D; ++r) {
      float re = 0.f, im = 0.f;
      for (int k = 0; k < D; ++k) {
        float mr = mm[2 * (r * D + k)], mi = mm[2 * (r * D + k) + 1];
        re += mr * ar[k] - mi * ai[k];
        im += mr * ai[k] + mi * ar[k];
      }
      s[2 * idx[r]] = re;
      s[2 * idx[r] + 1] = im;
    }
  }
}

// Applies one Pauli factor on bit b (X, Y or Z) as a full pass.
void apply_pauli(float* s, int n, int b, char p) {
  const uint32_t cnt = 1u << (n - 1);
  for (uint32_t i = 0; i < cnt; ++i) {
    uint32_t i0 = ins0(i, b), i1 = i0 | (1u << b);
    float r0 = s[2 * i0], m0 = s[2 * i0 + 1], r1 = s[2 * i1], m1 = s[2 * i1 + 1];
    if (p == 'X') {
      s[2 * i0] = r1; s[2 * i0 + 1] = m1; s[2 * i1] = r0; s[2 * i1 + 1] = m0;
    } else if (p == 'Y') {  // Y = [[0,-i],[i,0]]
      s[2 * i0] = m1; s[2 * i0 + 1] = -r1; s[2 * i1] = -m0; s[2 * i1 + 1] = r0;
    } else {
      s[2 * i1] = -r1; s[2 * i1 + 1] = -m1;
    }
  }
}

double real_inner(const float* a, const float* b, uint32_t N) {
  double acc = 0.0;
  for (uint32_t x = 0; x < N; ++x) acc += double(a[2 * x]) * b[2 * x] + double(a[2 * x + 1]) * b[2 * x + 1];
  return acc;
}

}  // namespace

extern "C" {

// rows: circuits.  Per row r: n[r]; gates [gate_off[r], gate_off[r+1]) with
// per-gate nq, b0, b1, cmask, cval, ngrad, grad_cols (2 per gate);
// matrices 32 floats per gate, derivative matrices 64 floats per gate.
// Terms [term_off[r], term_off[r+1]): term_op, term_coef, and the Pauli
// factors [fac_off[t], fac_off[t+1]) as (bit, char).
int cpuref_expect_adj(int rows, const int* n, const int64_t* gate_off,
                      const int* nq, const int* b0, const int* b1,
                      const uint32_t* cmask, const uint32_t* cval,
                      const float* mats, const int* ngrad,
                      const int* grad_cols, const float* dmats,
                      const int64_t* term_off, const int* term_op,
                      const float* term_coef, const int64_t* fac_off,
                      const int* fac_bit, const char* fac_type, int n_ops,
                      int num_symbols, const float* dgrads, float* out_exp,
                      float* out_grad, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int r = 0; r < rows; ++r) {
    const int nn = n[r];
    const uint32_t N = 1u << nn;
    std::vector<float> psi(2 * N), scratch(2 * N), scratch2(2 * N);
    std::vector<Gate> gates;
    for (int64_t g = gate_off[r]; g < gate_off[r + 1]; ++g)
      gates.push_back(Gate{nq[g], b0[g], b1[g], cmask[g], cval[g], mats + 32 * g,
                           ngrad[g], dmats + 64 * g, grad_cols + 2 * g});
    auto forward = [&]() {
      std::fill(psi.begin(), psi.end(), 0.f);
      psi[0] = 1.f;
      for (const Gate& g : gates) apply(psi.data(), nn, g, g.m, false);
    };
    // expectation op (ComputeSmall of tfq_simulate_expectation_op.cc)
    forward();
    for (int j = 0; j < n_ops; ++j) out_exp[int64_t(r) * n_ops + j] = 0.f;
    for (int64_t t = term_off[r]; t < term_off[r + 1]; ++t) {
      float& o = out_exp[int64_t(r) * n_ops + term_op[t]];
      if (fac_off[t] == fac_off[t + 1]) { o += term_coef[t]; continue; }
      scratch = psi;
      for (int64_t f = fac_off[t]; f < fac_off[t + 1]; ++f)
        apply_pauli(scratch.data(), nn, fac_bit[f], fac_type[f]);
      o += term_coef[t] * float(real_inner(psi.data(), scratch.data(), N));
    }
    // adjoint op (ComputeSmall of tfq_adj_grad_op.cc)
    forward();
    std::vector<float> lam(2 * N, 0.f);
    scratch = psi;
    for (int64_t t = term_off[r]; t < term_off[r + 1]; ++t) {
      float w = dgrads[int64_t(r) * n_ops + term_op[t]] * term_coef[t];
      if (fabsf(w) < 1e-5f) continue;
      for (int64_t f = fac_off[t]; f < fac_off[t + 1]; ++f)
        apply_pauli(scratch.data(), nn, fac_bit[f], fac_type[f]);
      for (uint32_t x = 0; x < 2 * N; ++x) lam[x] += w * scratch[x];
      scratch = psi;
    }
    float* grad = out_grad + int64_t(r) * num_symbols;
    for (int k = 0; k < num_symbols; ++k) grad[k] = 0.f;
    for (int gi = int(gates.size()) - 1; gi >= 0; --gi) {
      const Gate& g = gates[gi];
      apply(psi.data(), nn, g, g.m, true);
      for (int k = 0; k < g.ngrad; ++k) {
        scratch2 = psi;
        if (g.cmask)
          for (uint32_t x = 0; x < N; ++x)
            if ((x & g.cmask) != g.cval) scratch2[2 * x] = scratch2[2 * x + 1] = 0.f;
        apply(scratch2.data(), nn, g, g.dm + 32 * k, false, false);
        grad[g.cols[k]] += float(2.0 * real_inner(scratch2.data(), lam.data(), N));
      }
      apply(lam.data(), nn, g, g.m, true);
    }
  }
  return 0;
}

int cpuref_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
