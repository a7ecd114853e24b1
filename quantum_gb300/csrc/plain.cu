// Plain comparison path: one kernel launch per gate (and per Pauli term, per
// gradient inner product) over all rows' states held in HBM, no fusion and
// no shared-memory residency.  It is the "one gate per pass" GPU design the
// fused/batched kernels are measured against; it computes the same
// expectation + adjoint gradient (tfq_adj_grad_op.cc:199-276 structure).
#include <cuda_runtime.h>
#include <stdint.h>

#include "plain.h"

namespace tfqg {
namespace {

__device__ __forceinline__ float2 pcfma(float2 m, float2 a, float2 acc) {
  acc.x = fmaf(m.x, a.x, fmaf(-m.y, a.y, acc.x));
  acc.y = fmaf(m.x, a.y, fmaf(m.y, a.x, acc.y));
  return acc;
}
__device__ __forceinline__ uint32_t pins0(uint32_t i, int b) {
  return ((i >> b) << (b + 1)) | (i & ((1u << b) - 1u));
}

__global__ void plain_init(float2* psi, int64_t total, int n) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= total) return;
  psi[t] = make_float2((t & ((int64_t(1) << n) - 1)) == 0 ? 1.f : 0.f, 0.f);
}

__global__ void plain_zero(float2* v, int64_t total) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < total) v[t] = make_float2(0.f, 0.f);
}

// Applies gate g (or its adjoint) of every row to psi [rows][2^n].
__global__ void plain_gate(const GateTemplate gt, const float2* mats,
                           int64_t mat_stride, int g, float2* psi, int rows,
                           int n, int dagger) {
  const int nq = gt.nq;
  const int64_t per = int64_t(1) << (n - nq);
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= per * rows) return;
  const int r = int(t / per);
  const uint32_t i = uint32_t(t - int64_t(r) * per);
  float2* s = psi + (int64_t(r) << n);
  const float2* m = mats + int64_t(r) * mat_stride * 16 + int64_t(g) * 16;
  const int D = 1 << nq;
  uint32_t idx[4];
  if (nq == 1) {
    idx[0] = pins0(i, gt.b0);
    idx[1] = idx[0] | (1u << gt.b0);
  } else {
    int lo = gt.b0 < gt.b1 ? gt.b0 : gt.b1, hi = gt.b0 < gt.b1 ? gt.b1 : gt.b0;
    uint32_t b = pins0(pins0(i, lo), hi);
    idx[0] = b;
    idx[1] = b | (1u << gt.b1);
    idx[2] = b | (1u << gt.b0);
    idx[3] = b | (1u << gt.b0) | (1u << gt.b1);
  }
  if ((idx[0] & gt.cmask) != gt.cval) return;
  float2 a[4], o[4];
  for (int k = 0; k < D; ++k) a[k] = s[idx[k]];
  for (int rr = 0; rr < D; ++rr) {
    float2 acc = make_float2(0.f, 0.f);
    for (int k = 0; k < D; ++k) {
      float2 mm = dagger ? make_float2(m[k * D + rr].x, -m[k * D + rr].y)
                         : m[rr * D + k];
      acc = pcfma(mm, a[k], acc);
    }
    o[rr] = acc;
  }
  for (int k = 0; k < D; ++k) s[idx[k]] = o[k];
}

// acc[r] += Re(i^ny sum_x conj(psi_x) sign psi_{x^flip}) for one term
__global__ void plain_term(DevTerm t, const float2* psi, int rows, int n,
                           double* acc, int acc_stride) {
  const int64_t N = int64_t(1) << n;
  int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t.identity) {
    if (g < N * rows && (g & (N - 1)) == 0)
      atomicAdd(acc + (g >> n) * acc_stride + t.op, double(t.coef));
    return;
  }
  float re = 0.f, im = 0.f;
  int r = -1;
  if (g < N * rows) {
    r = int(g >> n);
    uint32_t x = uint32_t(g & (N - 1)), y = x ^ t.flip;
    const float2* s = psi + (int64_t(r) << n);
    float2 a = s[x], b = s[y];
    float sg = (__popc(y & t.zy) & 1) ? -1.f : 1.f;
    re = sg * (a.x * b.x + a.y * b.y);
    im = sg * (a.x * b.y - a.y * b.x);
  }
  // blocks never straddle rows when N >= blockDim
  for (int o = 16; o; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if ((threadIdx.x & 31) == 0 && r >= 0) {
    double v;
    switch (t.ny & 3) {
      case 0: v = re; break;
      case 1: v = -im; break;
      case 2: v = -re; break;
      default: v = im; break;
    }
    atomicAdd(acc + int64_t(r) * acc_stride + t.op, double(t.coef) * v);
  }
}

// lam += w P psi for one term (w = downstream_grads[r, op] * coef)
__global__ void plain_lambda(DevTerm t, const float2* psi, float2* lam,
                             const float* dgrads, int n_ops, int rows, int n) {
  const int64_t N = int64_t(1) << n;
  int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= N * rows) return;
  int r = int(g >> n);
  float w = dgrads[int64_t(r) * n_ops + t.op] * t.coef;
  if (fabsf(w) < 1e-5f) return;
  uint32_t x = uint32_t(g & (N - 1));
  const float2* s = psi + (int64_t(r) << n);
  float2 p;
  if (t.identity) {
    p = s[x];
  } else {
    uint32_t y = x ^ t.flip;
    p = s[y];
    if (__popc(y & t.zy) & 1) w = -w;
    switch (t.ny & 3) {
      case 1: p = make_float2(-p.y, p.x); break;
      case 2: p = make_float2(-p.x, -p.y); break;
      case 3: p = make_float2(p.y, -p.x); break;
      default: break;
    }
  }
  float2* l = lam + (int64_t(r) << n);
  l[x].x += w * p.x;
  l[x].y += w * p.y;
}

// grad[r, col] += 2 Re<lam | dG P_c | psi> for derivative slot k of gate g
__global__ void plain_grad(const GateTemplate gt, const float2* dmats,
                           int64_t dmat_stride, int slot, const float2* psi,
                           const float2* lam, int rows, int n, double* acc,
                           int acc_stride, int col) {
  const int nq = gt.nq;
  const int64_t per = int64_t(1) << (n - nq);
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float part = 0.f;
  int r = -1;
  if (t < per * rows) {
    r = int(t / per);
    const uint32_t i = uint32_t(t - int64_t(r) * per);
    const float2* s = psi + (int64_t(r) << n);
    const float2* l = lam + (int64_t(r) << n);
    const float2* d = dmats + int64_t(r) * dmat_stride * 16 + int64_t(slot) * 16;
    const int D = 1 << nq;
    uint32_t idx[4];
    if (nq == 1) {
      idx[0] = pins0(i, gt.b0);
      idx[1] = idx[0] | (1u << gt.b0);
    } else {
      int lo = gt.b0 < gt.b1 ? gt.b0 : gt.b1, hi = gt.b0 < gt.b1 ? gt.b1 : gt.b0;
      uint32_t b = pins0(pins0(i, lo), hi);
      idx[0] = b;
      idx[1] = b | (1u << gt.b1);
      idx[2] = b | (1u << gt.b0);
      idx[3] = b | (1u << gt.b0) | (1u << gt.b1);
    }
    if ((idx[0] & gt.cmask) == gt.cval) {
      float2 a[4];
      for (int k = 0; k < D; ++k) a[k] = s[idx[k]];
      for (int rr = 0; rr < D; ++rr) {
        float2 dv = make_float2(0.f, 0.f);
        for (int k = 0; k < D; ++k) dv = pcfma(d[rr * D + k], a[k], dv);
        float2 lv = l[idx[rr]];
        part += lv.x * dv.x + lv.y * dv.y;
      }
    }
  }
  for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0 && r >= 0)
    atomicAdd(acc + int64_t(r) * acc_stride + col, 2.0 * double(part));
}

__global__ void plain_to_float(const double* src, float* dst, int64_t total) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < total) dst[t] = float(src[t]);
}

inline unsigned blocks_for(int64_t work, int threads) {
  return unsigned((work + threads - 1) / threads);
}

}  // namespace

cudaError_t plain_expect_adjoint(const PlainJob& j, cudaStream_t s,
                                 int64_t* launches) {
  const int T = 256;
  const int n = j.n;
  const int64_t N = int64_t(1) << n;
  const int64_t total = N * j.rows;
  int64_t L = 0;
  plain_init<<<blocks_for(total, T), T, 0, s>>>(j.psi, total, n); ++L;
  for (int g = 0; g < j.num_gates; ++g) {
    const GateTemplate& gt = j.gates[g];
    if (gt.kind == GK_FUSED) continue;  // its members run one by one
    plain_gate<<<blocks_for((N >> gt.nq) * j.rows, T), T, 0, s>>>(
        gt, j.mats, j.num_gates, g, j.psi, j.rows, n, 0);
    ++L;
  }
  for (int t = 0; t < j.num_terms; ++t) {
    const DevTerm& tm = j.terms[t];
    plain_term<<<blocks_for(total, T), T, 0, s>>>(tm, j.psi, j.rows, n,
                                                  j.acc_exp, j.n_ops);
    ++L;
  }
  plain_zero<<<blocks_for(total, T), T, 0, s>>>(j.lam, total); ++L;
  for (int t = 0; t < j.num_terms; ++t) {
    plain_lambda<<<blocks_for(total, T), T, 0, s>>>(j.terms[t], j.psi, j.lam,
                                                    j.dgrads, j.n_ops, j.rows, n);
    ++L;
  }
  for (int g = j.num_gates - 1; g >= 0; --g) {
    const GateTemplate& gt = j.gates[g];
    if (gt.kind == GK_FUSED) continue;
    const int64_t work = (N >> gt.nq) * j.rows;
    plain_gate<<<blocks_for(work, T), T, 0, s>>>(gt, j.mats, j.num_gates, g,
                                                 j.psi, j.rows, n, 1);
    ++L;
    for (int k = 0; k < gt.ngrad; ++k) {
      plain_grad<<<blocks_for(work, T), T, 0, s>>>(
          gt, j.dmats, j.num_grads, gt.grad_slot + k, j.psi, j.lam, j.rows, n,
          j.acc_grad, j.num_symbols, j.grad_cols[gt.grad_slot + k]);
      ++L;
    }
    plain_gate<<<blocks_for(work, T), T, 0, s>>>(gt, j.mats, j.num_gates, g,
                                                 j.lam, j.rows, n, 1);
    ++L;
  }
  const int64_t ng = int64_t(j.rows) * j.num_symbols;
  plain_to_float<<<blocks_for(ng, T), T, 0, s>>>(j.acc_grad, j.out_grad, ng); ++L;
  const int64_t ne = int64_t(j.rows) * j.n_ops;
  plain_to_float<<<blocks_for(ne, T), T, 0, s>>>(j.acc_exp, j.out_exp, ne); ++L;
  if (launches) *launches = L;
  return cudaGetLastError();
}

}  // namespace tfqg
