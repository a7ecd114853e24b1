// CPU restatement of the reference's expectation + adjoint-gradient loops,
// used as the timed CPU baseline (TEST INFRASTRUCTURE, never the product).
//
// Follows, per circuit, in complex64 like the reference's simulator:
//   fusion ............. circuit_parser_qsim.cc:857-859: the circuit is fused
//                        before it is simulated; here every run of
//                        uncontrolled one-qubit gates on a qubit is folded
//                        into the next uncontrolled two-qubit gate on that
//                        qubit (leftovers run as one fused one-qubit gate),
//                        the <=2-qubit blocks of a basic gate fuser
//   forward ............ tfq_simulate_expectation_op.cc:196-243
//   expectation ........ util_qsim.h:142-188: per Pauli term copy the state,
//                        apply the term's Pauli factors, real inner product
//   lambda ............. util_qsim.h:362-414 AccumulateOperators
//   adjoint sweep ...... tfq_adj_grad_op.cc:199-276: the forward state from
//                        the fused circuit; then backward, the gates between
//                        gradient gates as fused partial blocks
//                        (adj_util.cc:155-172) applied daggered to psi and
//                        lambda; per gradient gate psi <- G^dag psi, copy,
//                        zero non-matching controls, apply the gradient gate,
//                        2 Re<scratch|lambda>, lambda <- G^dag lambda
// Circuits run in parallel over host threads (ComputeSmall's ParallelFor).
// States are split into real and imaginary float arrays so that the
// amplitude loops of one- and two-qubit gates vectorize (the reference's
// simulator likewise runs vector lanes over amplitudes).  Gate matrices come
// in bound to the symbol values (the oracle builds them before the timed
// call; binding is a few hundred 2x2 / 4x4 matrices per circuit).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Gate {
  int nq, b0, b1;    // matrix index bit 1 (MSB) <-> b0, bit 0 <-> b1
  uint32_t cmask, cval;
  float m[32];       // interleaved complex, D x D row-major
  int ngrad;
  const float* dm;   // ngrad * 32 floats
  const int* cols;   // ngrad
};

struct State {
  std::vector<float> re, im;
  explicit State(uint32_t N) : re(N), im(N) {}
};

inline uint32_t ins0(uint32_t i, int b) {
  return ((i >> b) << (b + 1)) | (i & ((1u << b) - 1u));
}

// c = a * b for D x D interleaved complex matrices
void matmul(const float* a, const float* b, float* c, int D) {
  for (int r = 0; r < D; ++r)
    for (int k = 0; k < D; ++k) {
      float re = 0.f, im = 0.f;
      for (int j = 0; j < D; ++j) {
        const float ar = a[2 * (r * D + j)], ai = a[2 * (r * D + j) + 1];
        const float br = b[2 * (j * D + k)], bi = b[2 * (j * D + k) + 1];
        re += ar * br - ai * bi;
        im += ar * bi + ai * br;
      }
      c[2 * (r * D + k)] = re;
      c[2 * (r * D + k) + 1] = im;
    }
}

void dagger(const float* m, float* out, int D) {
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) {
      out[2 * (r * D + c)] = m[2 * (c * D + r)];
      out[2 * (r * D + c) + 1] = -m[2 * (c * D + r) + 1];
    }
}

// one-qubit matrix on bit b, contiguous inner runs of 2^b amplitudes
void apply1(State& s, int n, int b, const float* m) {
  const float m00r = m[0], m00i = m[1], m01r = m[2], m01i = m[3];
  const float m10r = m[4], m10i = m[5], m11r = m[6], m11i = m[7];
  float* __restrict__ re = s.re.data();
  float* __restrict__ im = s.im.data();
  const uint32_t N = 1u << n, h = 1u << b;
  if (h >= 4) {
    for (uint32_t base = 0; base < N; base += 2 * h) {
      float* __restrict__ r0 = re + base;
      float* __restrict__ i0 = im + base;
      float* __restrict__ r1 = re + base + h;
      float* __restrict__ i1 = im + base + h;
      for (uint32_t l = 0; l < h; ++l) {
        const float ar = r0[l], ai = i0[l], br = r1[l], bi = i1[l];
        r0[l] = m00r * ar - m00i * ai + m01r * br - m01i * bi;
        i0[l] = m00r * ai + m00i * ar + m01r * bi + m01i * br;
        r1[l] = m10r * ar - m10i * ai + m11r * br - m11i * bi;
        i1[l] = m10r * ai + m10i * ar + m11r * bi + m11i * br;
      }
    }
    return;
  }
  for (uint32_t i = 0; i < N / 2; ++i) {
    const uint32_t x0 = ins0(i, b), x1 = x0 | h;
    const float ar = re[x0], ai = im[x0], br = re[x1], bi = im[x1];
    re[x0] = m00r * ar - m00i * ai + m01r * br - m01i * bi;
    im[x0] = m00r * ai + m00i * ar + m01r * bi + m01i * br;
    re[x1] = m10r * ar - m10i * ai + m11r * br - m11i * bi;
    im[x1] = m10r * ai + m10i * ar + m11r * bi + m11i * br;
  }
}

// two-qubit matrix (index bit 1 <-> b0, bit 0 <-> b1), contiguous inner runs
// of 2^min(b0, b1) amplitudes
void apply2(State& s, int n, int b0, int b1, const float* m) {
  float* __restrict__ re = s.re.data();
  float* __restrict__ im = s.im.data();
  const uint32_t N = 1u << n;
  const int lo = b0 < b1 ? b0 : b1, hi = b0 < b1 ? b1 : b0;
  const uint32_t o1 = 1u << b1, o2 = 1u << b0, o3 = o1 | o2;
  float mr[16], mi[16];
  for (int k = 0; k < 16; ++k) {
    mr[k] = m[2 * k];
    mi[k] = m[2 * k + 1];
  }
  const uint32_t hl = 1u << lo;
  if (hl >= 4) {
    for (uint32_t a = 0; a < N; a += 2u << hi)
      for (uint32_t mid = 0; mid < (1u << hi); mid += 2 * hl) {
        const uint32_t base = a + mid;
        float* __restrict__ r0 = re + base;
        float* __restrict__ i0 = im + base;
        for (uint32_t l = 0; l < hl; ++l) {
          const float xr0 = r0[l], xi0 = i0[l], xr1 = r0[l + o1], xi1 = i0[l + o1];
          const float xr2 = r0[l + o2], xi2 = i0[l + o2], xr3 = r0[l + o3], xi3 = i0[l + o3];
#define ROW(k, dr, di)                                                               \
  const float dr = mr[4 * k] * xr0 - mi[4 * k] * xi0 + mr[4 * k + 1] * xr1 -       \
                   mi[4 * k + 1] * xi1 + mr[4 * k + 2] * xr2 - mi[4 * k + 2] * xi2 + \
                   mr[4 * k + 3] * xr3 - mi[4 * k + 3] * xi3;                        \
  const float di = mr[4 * k] * xi0 + mi[4 * k] * xr0 + mr[4 * k + 1] * xi1 +       \
                   mi[4 * k + 1] * xr1 + mr[4 * k + 2] * xi2 + mi[4 * k + 2] * xr2 + \
                   mr[4 * k + 3] * xi3 + mi[4 * k + 3] * xr3;
          ROW(0, yr0, yi0)
          ROW(1, yr1, yi1)
          ROW(2, yr2, yi2)
          ROW(3, yr3, yi3)
          r0[l] = yr0; i0[l] = yi0;
          r0[l + o1] = yr1; i0[l + o1] = yi1;
          r0[l + o2] = yr2; i0[l + o2] = yi2;
          r0[l + o3] = yr3; i0[l + o3] = yi3;
        }
      }
    return;
  }
  for (uint32_t i = 0; i < N / 4; ++i) {
    const uint32_t base = ins0(ins0(i, lo), hi);
    float* r0 = re + base;
    float* i0 = im + base;
    const uint32_t l = 0;
    const float xr0 = r0[l], xi0 = i0[l], xr1 = r0[l + o1], xi1 = i0[l + o1];
    const float xr2 = r0[l + o2], xi2 = i0[l + o2], xr3 = r0[l + o3], xi3 = i0[l + o3];
    ROW(0, yr0, yi0)
    ROW(1, yr1, yi1)
    ROW(2, yr2, yi2)
    ROW(3, yr3, yi3)
#undef ROW
    r0[l] = yr0; i0[l] = yi0;
    r0[l + o1] = yr1; i0[l + o1] = yi1;
    r0[l + o2] = yr2; i0[l + o2] = yi2;
    r0[l + o3] = yr3; i0[l + o3] = yi3;
  }
}

// general path: controls (only amplitudes with (x & cmask) == cval change)
void apply_ctrl(State& s, int n, const Gate& g, const float* m) {
  const int D = 1 << g.nq;
  const uint32_t cnt = 1u << (n - g.nq);
  for (uint32_t i = 0; i < cnt; ++i) {
    uint32_t idx[4];
    if (g.nq == 1) {
      idx[0] = ins0(i, g.b0);
      idx[1] = idx[0] | (1u << g.b0);
    } else {
      const int lo = g.b0 < g.b1 ? g.b0 : g.b1, hi = g.b0 < g.b1 ? g.b1 : g.b0;
      const uint32_t b = ins0(ins0(i, lo), hi);
      idx[0] = b;
      idx[1] = b | (1u << g.b1);
      idx[2] = b | (1u << g.b0);
      idx[3] = b | (1u << g.b0) | (1u << g.b1);
    }
    if ((idx[0] & g.cmask) != g.cval) continue;
    float ar[4], ai[4];
    for (int k = 0; k < D; ++k) {
      ar[k] = s.re[idx[k]];
      ai[k] = s.im[idx[k]];
    }
    for (int r = 0; r < D; ++r) {
      float re = 0.f, im = 0.f;
      for (int k = 0; k < D; ++k) {
        const float mr = m[2 * (r * D + k)], mi = m[2 * (r * D + k) + 1];
        re += mr * ar[k] - mi * ai[k];
        im += mr * ai[k] + mi * ar[k];
      }
      s.re[idx[r]] = re;
      s.im[idx[r]] = im;
    }
  }
}

void apply(State& s, int n, const Gate& g, const float* m, bool controls = true) {
  if (controls && g.cmask) return apply_ctrl(s, n, g, m);
  if (g.nq == 1) return apply1(s, n, g.b0, m);
  apply2(s, n, g.b0, g.b1, m);
}

void apply_dagger(State& s, int n, const Gate& g) {
  float md[32];
  dagger(g.m, md, 1 << g.nq);
  apply(s, n, g, md);
}

// Fuses a gate range into <=2-qubit blocks: runs of uncontrolled one-qubit
// gates on a qubit fold into the next uncontrolled two-qubit gate on it;
// controlled gates flush the pending runs of every qubit they touch.
std::vector<Gate> fuse(const Gate* begin, const Gate* end, int n) {
  std::vector<Gate> out;
  std::vector<int> has(n, 0);
  std::vector<float> pend(size_t(n) * 8);
  auto flush = [&](int b) {
    if (!has[b]) return;
    Gate g{};
    g.nq = 1;
    g.b0 = b;
    memcpy(g.m, &pend[size_t(b) * 8], 8 * sizeof(float));
    out.push_back(g);
    has[b] = 0;
  };
  for (const Gate* p = begin; p != end; ++p) {
    const Gate& g = *p;
    if (g.cmask) {
      flush(g.b0);
      if (g.nq == 2) flush(g.b1);
      for (int b = 0; b < n; ++b)
        if ((g.cmask >> b) & 1u) flush(b);
      Gate c = g;
      c.ngrad = 0;
      out.push_back(c);
    } else if (g.nq == 1) {
      float* P = &pend[size_t(g.b0) * 8];
      if (has[g.b0]) {
        float t[8];
        matmul(g.m, P, t, 2);
        memcpy(P, t, sizeof(t));
      } else {
        memcpy(P, g.m, 8 * sizeof(float));
        has[g.b0] = 1;
      }
    } else {
      // M = G (P_b0 (x) P_b1), identity where nothing is pending
      float K[32];
      const float I2[8] = {1, 0, 0, 0, 0, 0, 1, 0};
      const float* A = has[g.b0] ? &pend[size_t(g.b0) * 8] : I2;
      const float* B = has[g.b1] ? &pend[size_t(g.b1) * 8] : I2;
      for (int r0 = 0; r0 < 2; ++r0)
        for (int r1 = 0; r1 < 2; ++r1)
          for (int c0 = 0; c0 < 2; ++c0)
            for (int c1 = 0; c1 < 2; ++c1) {
              const float ar = A[2 * (r0 * 2 + c0)], ai = A[2 * (r0 * 2 + c0) + 1];
              const float br = B[2 * (r1 * 2 + c1)], bi = B[2 * (r1 * 2 + c1) + 1];
              const int k = (r0 * 2 + r1) * 4 + (c0 * 2 + c1);
              K[2 * k] = ar * br - ai * bi;
              K[2 * k + 1] = ar * bi + ai * br;
            }
      Gate f = g;
      f.ngrad = 0;
      if (has[g.b0] || has[g.b1]) matmul(g.m, K, f.m, 4);
      has[g.b0] = has[g.b1] = 0;
      out.push_back(f);
    }
  }
  for (int b = 0; b < n; ++b) flush(b);
  return out;
}

void copy(const State& a, State& b) {
  memcpy(b.re.data(), a.re.data(), a.re.size() * sizeof(float));
  memcpy(b.im.data(), a.im.data(), a.im.size() * sizeof(float));
}

// Applies one Pauli factor on bit b (X, Y or Z) as a full pass.
void apply_pauli(State& s, int n, int b, char p) {
  const float X[8] = {0, 0, 1, 0, 1, 0, 0, 0};
  const float Y[8] = {0, 0, 0, -1, 0, 1, 0, 0};
  const float Z[8] = {1, 0, 0, 0, 0, 0, -1, 0};
  apply1(s, n, b, p == 'X' ? X : p == 'Y' ? Y : Z);
}

double real_inner(const State& a, const State& b) {
  const size_t N = a.re.size();
  const float* __restrict__ ar = a.re.data();
  const float* __restrict__ ai = a.im.data();
  const float* __restrict__ br = b.re.data();
  const float* __restrict__ bi = b.im.data();
  // float partial sums over runs of 64 amplitudes, accumulated in double
  double acc = 0.0;
  for (size_t x0 = 0; x0 < N; x0 += 64) {
    const size_t x1 = x0 + 64 < N ? x0 + 64 : N;
    float part = 0.f;
    for (size_t x = x0; x < x1; ++x) part += ar[x] * br[x] + ai[x] * bi[x];
    acc += part;
  }
  return acc;
}

}  // namespace

extern "C" {

// rows: circuits.  Per row r: n[r]; gates [gate_off[r], gate_off[r+1]) with
// per-gate nq, b0, b1, cmask, cval, ngrad, grad_cols (2 per gate);
// matrices 32 floats per gate, derivative matrices 64 floats per gate.
// Terms [term_off[r], term_off[r+1]): term_op, term_coef, and the Pauli
// factors [fac_off[t], fac_off[t+1]) as (bit, char).  do_expect / do_adj
// select the two ops (the benchmark step runs both).
int cpuref_run(int rows, const int* n, const int64_t* gate_off, const int* nq,
               const int* b0, const int* b1, const uint32_t* cmask, const uint32_t* cval,
               const float* mats, const int* ngrad, const int* grad_cols,
               const float* dmats, const int64_t* term_off, const int* term_op,
               const float* term_coef, const int64_t* fac_off, const int* fac_bit,
               const char* fac_type, int n_ops, int num_symbols, const float* dgrads,
               float* out_exp, float* out_grad, int threads, int do_expect, int do_adj) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int r = 0; r < rows; ++r) {
    const int nn = n[r];
    const uint32_t N = 1u << nn;
    std::vector<Gate> gates;
    for (int64_t g = gate_off[r]; g < gate_off[r + 1]; ++g) {
      Gate x{};
      x.nq = nq[g];
      x.b0 = b0[g];
      x.b1 = b1[g];
      x.cmask = cmask[g];
      x.cval = cval[g];
      memcpy(x.m, mats + 32 * g, 32 * sizeof(float));
      x.ngrad = ngrad[g];
      x.dm = dmats + 64 * g;
      x.cols = grad_cols + 2 * g;
      gates.push_back(x);
    }
    if (do_expect) {
      // expectation op (ComputeSmall of tfq_simulate_expectation_op.cc)
      for (int j = 0; j < n_ops; ++j) out_exp[int64_t(r) * n_ops + j] = 0.f;
      if (gates.empty()) {
        for (int j = 0; j < n_ops; ++j) out_exp[int64_t(r) * n_ops + j] = -2.f;
      } else {
        State psi(N), scratch(N);
        const std::vector<Gate> fused = fuse(gates.data(), gates.data() + gates.size(), nn);
        psi.re[0] = 1.f;
        for (const Gate& g : fused) apply(psi, nn, g, g.m);
        for (int64_t t = term_off[r]; t < term_off[r + 1]; ++t) {
          float& o = out_exp[int64_t(r) * n_ops + term_op[t]];
          if (fac_off[t] == fac_off[t + 1]) {
            o += term_coef[t];
            continue;
          }
          copy(psi, scratch);
          for (int64_t f = fac_off[t]; f < fac_off[t + 1]; ++f)
            apply_pauli(scratch, nn, fac_bit[f], fac_type[f]);
          o += term_coef[t] * float(real_inner(psi, scratch));
        }
      }
    }
    if (!do_adj) continue;
    // adjoint op (ComputeSmall of tfq_adj_grad_op.cc)
    float* grad = out_grad + int64_t(r) * num_symbols;
    for (int k = 0; k < num_symbols; ++k) grad[k] = 0.f;
    if (gates.empty()) continue;
    State psi(N), scratch(N), scratch2(N), lam(N);
    {
      const std::vector<Gate> fused = fuse(gates.data(), gates.data() + gates.size(), nn);
      psi.re[0] = 1.f;
      for (const Gate& g : fused) apply(psi, nn, g, g.m);
    }
    // partial fuses: the gates between consecutive gradient gates
    std::vector<int> grad_idx;
    for (size_t i = 0; i < gates.size(); ++i)
      if (gates[i].ngrad > 0) grad_idx.push_back(int(i));
    std::vector<std::vector<Gate>> partial(grad_idx.size() + 1);
    {
      int left = 0;
      for (size_t i = 0; i < grad_idx.size(); ++i) {
        partial[i] = fuse(gates.data() + left, gates.data() + grad_idx[i], nn);
        left = grad_idx[i] + 1;
      }
      partial[grad_idx.size()] = fuse(gates.data() + left, gates.data() + gates.size(), nn);
    }
    // AccumulateOperators
    copy(psi, scratch);
    for (int64_t t = term_off[r]; t < term_off[r + 1]; ++t) {
      const float w = dgrads[int64_t(r) * n_ops + term_op[t]] * term_coef[t];
      if (fabsf(w) < 1e-5f) continue;
      for (int64_t f = fac_off[t]; f < fac_off[t + 1]; ++f)
        apply_pauli(scratch, nn, fac_bit[f], fac_type[f]);
      for (uint32_t x = 0; x < N; ++x) {
        lam.re[x] += w * scratch.re[x];
        lam.im[x] += w * scratch.im[x];
      }
      copy(psi, scratch);
    }
    for (int j = int(partial.size()) - 1; j >= 0; --j) {
      for (int k = int(partial[j].size()) - 1; k >= 0; --k) {
        apply_dagger(psi, nn, partial[j][k]);
        apply_dagger(lam, nn, partial[j][k]);
      }
      if (j == 0) break;
      const Gate& g = gates[grad_idx[j - 1]];
      apply_dagger(psi, nn, g);
      for (int k = 0; k < g.ngrad; ++k) {
        copy(psi, scratch2);
        if (g.cmask)
          for (uint32_t x = 0; x < N; ++x)
            if ((x & g.cmask) != g.cval) scratch2.re[x] = scratch2.im[x] = 0.f;
        apply(scratch2, nn, g, g.dm + 32 * k, false);
        grad[g.cols[k]] += float(2.0 * real_inner(scratch2, lam));
      }
      apply_dagger(lam, nn, g);
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
