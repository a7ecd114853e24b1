// Gate matrices of the TFQ gate set, usable on host and device.
//
// The formulas are the published definitions of the cirq gate families that
// the reference parses (circuit_parser_qsim.cc:154-562 builds them through
// qsim's cirq gate constructors):
//   EigenGate G^t with global shift s:  sum_k exp(i pi t (lambda_k + s)) P_k
//   PhasedXPow(p, t, s) = Z^p X^t Z^-p * exp(i pi t s)
//   FSim(theta, phi), PhasedISwapPow(p, t) = (Z^-p x Z^p) ISWAP^t (Z^p x Z^-p)
// Matrices are row-major, complex, 2x2 (4 entries) or 4x4 (16 entries); for
// two-qubit gates the first listed qubit is the most significant index bit.
//
// Everything is templated on the real type R: `double` gives the matrix,
// `Dual` (value + derivative) gives the matrix and its exact derivative with
// respect to one parameter in the same evaluation.
#pragma once
#include <math.h>
#include "tfqg_types.h"

#ifdef __CUDACC__
#define TFQG_HD __host__ __device__ __forceinline__
#else
#define TFQG_HD inline
#endif

namespace tfqg {

struct Dual {
  double v, d;
  TFQG_HD Dual() : v(0), d(0) {}
  TFQG_HD Dual(double x) : v(x), d(0) {}
  TFQG_HD Dual(double x, double dx) : v(x), d(dx) {}
};
TFQG_HD Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
TFQG_HD Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
TFQG_HD Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
TFQG_HD Dual operator*(Dual a, Dual b) {
  return Dual(a.v * b.v, a.d * b.v + a.v * b.d);
}
TFQG_HD Dual dcos(Dual a) { return Dual(cos(a.v), -sin(a.v) * a.d); }
TFQG_HD Dual dsin(Dual a) { return Dual(sin(a.v), cos(a.v) * a.d); }
TFQG_HD double dcos(double a) { return cos(a); }
TFQG_HD double dsin(double a) { return sin(a); }

template <class R>
struct Cx {
  R re, im;
  TFQG_HD Cx() : re(0.0), im(0.0) {}
  TFQG_HD Cx(R r, R i) : re(r), im(i) {}
};
template <class R>
TFQG_HD Cx<R> operator+(Cx<R> a, Cx<R> b) { return Cx<R>(a.re + b.re, a.im + b.im); }
template <class R>
TFQG_HD Cx<R> operator-(Cx<R> a, Cx<R> b) { return Cx<R>(a.re - b.re, a.im - b.im); }
template <class R>
TFQG_HD Cx<R> operator*(Cx<R> a, Cx<R> b) {
  return Cx<R>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class R>
TFQG_HD Cx<R> cscale(Cx<R> a, R s) { return Cx<R>(a.re * s, a.im * s); }
template <class R>
TFQG_HD Cx<R> expi(R x) { return Cx<R>(dcos(x), dsin(x)); }
template <class R>
TFQG_HD Cx<R> mul_i(Cx<R> a) { return Cx<R>(-a.im, a.re); }  // i*a

constexpr double kPi = 3.14159265358979323846;

// m <- (1+a)/2 * I + (1-a)/2 * P   for P with entries given by `pent`
// (used for the eigen gates with eigenvalues {0, 1} of a Pauli-like P).
template <class R>
TFQG_HD void eigen_pauli(Cx<R> a, const Cx<R>* pent, int dim, Cx<R>* m) {
  const R half(0.5);
  Cx<R> one(R(1.0), R(0.0));
  Cx<R> p = cscale(one + a, half);
  Cx<R> q = cscale(one - a, half);
  for (int i = 0; i < dim * dim; ++i) m[i] = q * pent[i];
  for (int i = 0; i < dim; ++i) m[i * dim + i] = m[i * dim + i] + p;
}

// Matrix of gate `kind` for effective parameters:
//   eigen gates: e0 = exponent t, e1 = global shift s
//   PXP: e0 = phase exponent p, e1 = exponent t, e2 = global shift s
//   FSIM: e0 = theta, e1 = phi;  PISP: e0 = phase exponent p, e1 = exponent t
// Returns the number of qubits (1 or 2); writes 4 or 16 entries.
template <class R>
TFQG_HD int gate_matrix(int kind, R e0, R e1, R e2, Cx<R>* m) {
  const R zero(0.0), one(1.0);
  const Cx<R> c0(zero, zero), c1(one, zero);
  if (kind == GK_I1) {
    m[0] = c1; m[1] = c0; m[2] = c0; m[3] = c1;
    return 1;
  }
  if (kind == GK_I2) {
    for (int i = 0; i < 16; ++i) m[i] = c0;
    m[0] = m[5] = m[10] = m[15] = c1;
    return 2;
  }
  const R pi(kPi);
  if (kind == GK_PXP) {
    R p = e0, t = e1, s = e2;
    Cx<R> a = expi<R>(pi * t);
    Cx<R> g = expi<R>(pi * t * s);
    const R half(0.5);
    Cx<R> d = cscale(c1 + a, half);
    Cx<R> o = cscale(c1 - a, half);
    Cx<R> z = expi<R>(pi * p);
    Cx<R> zc = expi<R>(-(pi * p));
    m[0] = g * d;
    m[1] = g * (o * zc);
    m[2] = g * (o * z);
    m[3] = g * d;
    return 1;
  }
  if (kind == GK_FSIM) {
    R c = dcos(e0), s = dsin(e0);
    for (int i = 0; i < 16; ++i) m[i] = c0;
    m[0] = c1;
    m[5] = Cx<R>(c, zero);
    m[6] = Cx<R>(zero, -s);
    m[9] = Cx<R>(zero, -s);
    m[10] = Cx<R>(c, zero);
    m[15] = expi<R>(-e1);
    return 2;
  }
  if (kind == GK_PISP) {
    const R half(0.5);
    R c = dcos(pi * e1 * half), s = dsin(pi * e1 * half);
    Cx<R> f = expi<R>(R(2.0) * pi * e0);
    Cx<R> fc = expi<R>(-(R(2.0) * pi * e0));
    for (int i = 0; i < 16; ++i) m[i] = c0;
    m[0] = c1;
    m[15] = c1;
    m[5] = Cx<R>(c, zero);
    m[10] = Cx<R>(c, zero);
    m[6] = mul_i(cscale(f, s));
    m[9] = mul_i(cscale(fc, s));
    return 2;
  }
  // Eigen gates.
  R t = e0, s = e1;
  Cx<R> a = expi<R>(pi * t);
  Cx<R> g = expi<R>(pi * t * s);
  int nq = 1;
  switch (kind) {
    case GK_XP: {
      Cx<R> P[4] = {c0, c1, c1, c0};
      eigen_pauli(a, P, 2, m);
      break;
    }
    case GK_YP: {
      Cx<R> P[4] = {c0, Cx<R>(zero, -one), Cx<R>(zero, one), c0};
      eigen_pauli(a, P, 2, m);
      break;
    }
    case GK_ZP: {
      m[0] = c1; m[1] = c0; m[2] = c0; m[3] = a;
      break;
    }
    case GK_HP: {
      const R r(0.70710678118654752440);
      Cx<R> P[4] = {Cx<R>(r, zero), Cx<R>(r, zero), Cx<R>(r, zero),
                    Cx<R>(-r, zero)};
      eigen_pauli(a, P, 2, m);
      break;
    }
    case GK_XXP: {
      Cx<R> P[16];
      for (int i = 0; i < 16; ++i) P[i] = c0;
      P[3] = P[6] = P[9] = P[12] = c1;
      eigen_pauli(a, P, 4, m);
      nq = 2;
      break;
    }
    case GK_YYP: {
      Cx<R> P[16];
      for (int i = 0; i < 16; ++i) P[i] = c0;
      Cx<R> mone(-one, zero);
      P[3] = mone; P[6] = c1; P[9] = c1; P[12] = mone;
      eigen_pauli(a, P, 4, m);
      nq = 2;
      break;
    }
    case GK_ZZP: {
      for (int i = 0; i < 16; ++i) m[i] = c0;
      m[0] = c1; m[5] = a; m[10] = a; m[15] = c1;
      nq = 2;
      break;
    }
    case GK_CZP: {
      for (int i = 0; i < 16; ++i) m[i] = c0;
      m[0] = c1; m[5] = c1; m[10] = c1; m[15] = a;
      nq = 2;
      break;
    }
    case GK_CNP: {
      const R half(0.5);
      for (int i = 0; i < 16; ++i) m[i] = c0;
      m[0] = c1; m[5] = c1;
      Cx<R> d = cscale(c1 + a, half), o = cscale(c1 - a, half);
      m[10] = d; m[11] = o; m[14] = o; m[15] = d;
      nq = 2;
      break;
    }
    case GK_SP: {
      const R half(0.5);
      for (int i = 0; i < 16; ++i) m[i] = c0;
      m[0] = c1; m[15] = c1;
      Cx<R> d = cscale(c1 + a, half), o = cscale(c1 - a, half);
      m[5] = d; m[6] = o; m[9] = o; m[10] = d;
      nq = 2;
      break;
    }
    case GK_ISP: {
      const R half(0.5);
      for (int i = 0; i < 16; ++i) m[i] = c0;
      m[0] = c1; m[15] = c1;
      R c = dcos(pi * t * half), sn = dsin(pi * t * half);
      m[5] = Cx<R>(c, zero); m[10] = Cx<R>(c, zero);
      m[6] = Cx<R>(zero, sn); m[9] = Cx<R>(zero, sn);
      nq = 2;
      break;
    }
    default:
      m[0] = c1; m[1] = c0; m[2] = c0; m[3] = c1;
      return 1;
  }
  int dim = nq == 1 ? 4 : 16;
  for (int i = 0; i < dim; ++i) m[i] = g * m[i];
  return nq;
}

// True for gates whose matrix is diagonal for every parameter value.
TFQG_HD bool gate_is_diagonal(int kind) {
  return kind == GK_ZP || kind == GK_ZZP || kind == GK_CZP || kind == GK_I1 ||
         kind == GK_I2;
}

TFQG_HD int gate_num_qubits(int kind) {
  switch (kind) {
    case GK_I1: case GK_XP: case GK_YP: case GK_ZP: case GK_HP: case GK_PXP:
      return 1;
    default:
      return 2;
  }
}

// Effective parameters of a template for given raw parameter values
// (raw0, raw1) in fp32, exactly as the reference combines them
// (circuit_parser_qsim.cc:229,278,426,480,537: fp32 `value * scalar`).
TFQG_HD void effective_params(const GateTemplate& g, float raw0, float raw1,
                              float* e0, float* e1, float* e2) {
  switch (g.kind) {
    case GK_PXP:
      *e0 = raw0 * g.a[1]; *e1 = raw1 * g.a[3]; *e2 = g.a[4];
      break;
    case GK_FSIM: case GK_PISP:
      *e0 = raw0 * g.a[1]; *e1 = raw1 * g.a[3]; *e2 = 0.f;
      break;
    default:
      *e0 = raw0 * g.a[1]; *e1 = g.a[2]; *e2 = 0.f;
      break;
  }
}

// Matrix of one template with its parameters bound: a[i] is replaced by
// row_values[src[i]] where the template names a symbol column.
TFQG_HD int bound_matrix(const GateTemplate& gt, const float* row_values,
                         Cx<double>* m) {
  GateTemplate gv = gt;
  for (int i = 0; i < 5; ++i)
    if (gt.src[i] >= 0) gv.a[i] = row_values[gt.src[i]];
  float e0, e1, e2;
  effective_params(gv, gv.a[0], gv.a[2], &e0, &e1, &e2);
  return gate_matrix<double>(gt.kind, e0, e1, e2, m);
}

// Matrix of a GK_FUSED gate: the product of its members' matrices in time
// order (the last member leftmost), each member embedded into the fused
// gate's space (2x2 for nq == 1, 4x4 with b0 as MSB for nq == 2) by its
// FusePos.  Members come as fp32 matrices from `load(k, m)` (k = template
// index) and are multiplied in fp32, as qsim multiplies the fp32 matrices of
// the gates it fuses.  `gates` is the program's template array.
template <class Load>
TFQG_HD void fused_product(const GateTemplate* gates, const GateTemplate& f,
                           Load load, Cx<float>* F) {
  const int D = f.nq == 1 ? 2 : 4;
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c)
      F[r * D + c] = Cx<float>(r == c ? 1.f : 0.f, 0.f);
  int k = f.link;
  for (int guard = 0; k >= 0 && guard < kMaxFuseMembers; ++guard) {
    const GateTemplate& g = gates[k];
    Cx<float> m[16], out[16];
    load(k, m);
    if (D == 2 || g.fpos == FP_HIGH || g.fpos == FP_LOW) {
      // 1-qubit member: row r mixes with the row that differs in its bit
      const int s = D == 2 ? 1 : (g.fpos == FP_HIGH ? 2 : 1);
      for (int r = 0; r < D; ++r) {
        const int rb = (r & s) ? 1 : 0, r0 = r & ~s;
        for (int c = 0; c < D; ++c)
          out[r * D + c] = m[rb * 2] * F[r0 * D + c] + m[rb * 2 + 1] * F[(r0 | s) * D + c];
      }
    } else {
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
          Cx<float> acc(0.f, 0.f);
          for (int j = 0; j < 4; ++j) {
            const int rr = g.fpos == FP_SAME ? r : ((r & 1) << 1 | r >> 1);
            const int jj = g.fpos == FP_SAME ? j : ((j & 1) << 1 | j >> 1);
            acc = acc + m[rr * 4 + jj] * F[j * 4 + c];
          }
          out[r * 4 + c] = acc;
        }
    }
    for (int i = 0; i < D * D; ++i) F[i] = out[i];
    k = g.link;
  }
}

// Column j of the 32 x 32 matrix of a tensor-core block (TcBlock): the
// basis state |j> of the block's 5 bits, with every member gate applied in
// time order, in Cx<R> (complex128 or complex64).  A member's targets and
// controls map to block
// positions (index bit i of the column is bit blk.tgt[i]); a 2-qubit
// member's matrix has b0 as its most significant index bit, and the gate
// acts where the control bits hold their required values.  `load(k, m)`
// gives member k's matrix (4 or 16 entries).
template <class R, class Load>
TFQG_HD void tc_block_column(const GateTemplate* gates, const int32_t* members,
                             const TcBlock& blk, int j, Load load, Cx<R>* col) {
  for (int i = 0; i < 32; ++i) col[i] = Cx<R>(R(i == j ? 1 : 0), R(0));
  for (uint32_t mi = blk.member_begin; mi < blk.member_end; ++mi) {
    const GateTemplate& g = gates[members[mi]];
    int pos[32];
    for (int b = 0; b < 32; ++b) pos[b] = -1;
    for (int i = 0; i < kTcBits; ++i) pos[blk.tgt[i]] = i;
    uint32_t cm = 0, cv = 0;
    for (int b = 0; b < 32; ++b)
      if ((g.cmask >> b) & 1u) {
        cm |= 1u << pos[b];
        if ((g.cval >> b) & 1u) cv |= 1u << pos[b];
      }
    Cx<R> m[16];
    load(members[mi], m);
    if (g.nq == 1) {
      const uint32_t s = 1u << pos[g.b0];
      for (uint32_t i = 0; i < 32; ++i) {
        if ((i & s) || (i & cm) != cv) continue;
        const Cx<R> a = col[i], c = col[i | s];
        col[i] = m[0] * a + m[1] * c;
        col[i | s] = m[2] * a + m[3] * c;
      }
    } else {
      const uint32_t s0 = 1u << pos[g.b0], s1 = 1u << pos[g.b1];
      for (uint32_t i = 0; i < 32; ++i) {
        if ((i & (s0 | s1)) || (i & cm) != cv) continue;
        const uint32_t idx[4] = {i, i | s1, i | s0, i | s0 | s1};
        Cx<R> v[4], w[4];
        for (int k = 0; k < 4; ++k) v[k] = col[idx[k]];
        for (int r = 0; r < 4; ++r) {
          w[r] = Cx<R>(R(0), R(0));
          for (int k = 0; k < 4; ++k) w[r] = w[r] + m[r * 4 + k] * v[k];
        }
        for (int k = 0; k < 4; ++k) col[idx[k]] = w[k];
      }
    }
  }
}

}  // namespace tfqg
