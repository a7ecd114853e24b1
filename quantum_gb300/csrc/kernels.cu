// sm_103a kernels of the TFQ state-vector hot path.
//
//  build_matrices_kernel   binds symbol values: one thread per (row, gate)
//                          computes the complex64 gate matrix and, for the
//                          adjoint, the derivative matrix of each symbolic
//                          parameter (reference finite difference with
//                          eps = 5e-3, adj_util.cc:32,175-302, or exact).
//  simulate_<mode>_kernel  the simulation kernels, one translation unit per
//                          mode (sim_mode.cuh, sim_<mode>.cu).
//  noisy_finalize_kernel   divides the trajectory sums by their counts.
//  wide_*                  rows too large for one CTA (kWideMinQubits and
//                          up): measurement passes, expectation finalize,
//                          probability chunk sums and sampling over a state
//                          in global memory that every CTA works on (the
//                          forward passes are sim_wide.cu).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "gate_math.cuh"
#include "sim_device.cuh"

namespace tfqg {
namespace {

// matrix build
// ---------------------------------------------------------------------------
__device__ __forceinline__ void store_mat(float2* dst, const Cx<double>* m,
                                          int nq) {
  int dim = nq == 1 ? 4 : 16;
  for (int i = 0; i < 16; ++i)
    dst[i] = i < dim ? make_float2(float(m[i].re), float(m[i].im))
                     : make_float2(0.f, 0.f);
}

// phase 0: every gate's own matrix (and derivatives); phase 1: GK_FUSED
// gates, as products of their members' matrices written in phase 0.
__global__ void build_matrices_kernel(BatchDevice b, RunArgs a, int with_grads,
                                      int phase) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= b.total_gates) return;
  // locate the row: rows are laid out with increasing mat_offset
  int lo = 0, hi = b.num_rows - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (int64_t(b.rows[mid].mat_offset) <= t) lo = mid; else hi = mid - 1;
  }
  const DevRow row = b.rows[lo];
  const DevProgram prog = b.programs[row.program];
  int g = int(t - int64_t(row.mat_offset));
  if (g >= prog.num_gates) return;
  const GateTemplate gt = b.gates[prog.gate_begin + g];
  if ((gt.kind == GK_FUSED) != (phase == 1)) return;
  if (phase == 1) {
    const float2* mats = a.mats + int64_t(row.mat_offset) * 16;
    Cx<float> f[16];
    fused_product(b.gates + prog.gate_begin, gt,
                  [&](int k, Cx<float>* m) {
                    const float2* src = mats + int64_t(k) * 16;
                    for (int i = 0; i < 16; ++i) m[i] = Cx<float>(src[i].x, src[i].y);
                  },
                  f);
    float2* dst = a.mats + int64_t(t) * 16;
    const int dim = gt.nq == 1 ? 4 : 16;
    for (int i = 0; i < 16; ++i)
      dst[i] = i < dim ? make_float2(f[i].re, f[i].im) : make_float2(0.f, 0.f);
    return;
  }
  float v[5];
  for (int i = 0; i < 5; ++i)
    v[i] = gt.src[i] >= 0 ? a.values[int64_t(lo) * b.num_symbols + gt.src[i]]
                          : gt.a[i];
  // effective parameters, fp32 products as in circuit_parser_qsim.cc
  GateTemplate gv = gt;
  for (int i = 0; i < 5; ++i) gv.a[i] = v[i];
  float e0, e1, e2;
  effective_params(gv, v[0], v[2], &e0, &e1, &e2);
  Cx<double> m[16];
  int nq = gate_matrix<double>(gt.kind, e0, e1, e2, m);
  store_mat(a.mats + int64_t(t) * 16, m, nq);
  if (!with_grads || gt.ngrad == 0) return;
  for (int k = 0; k < gt.ngrad; ++k) {
    const int p = gt.gparam[k];
    float2* dst = a.dmats + (int64_t(row.dmat_offset) + gt.grad_slot + k) * 16;
    Cx<double> d[16];
    if (a.grad_rule == 0) {
      // (G(x + eps) - G(x - eps)) * 0.5 / eps with fp32 parameter
      // arithmetic (adj_util.cc:175-186).
      const float eps = 5e-3f;
      const float raw = v[2 * p];
      float rp = raw + eps, rm = raw - eps;
      float ep0, ep1, ep2, em0, em1, em2;
      effective_params(gv, p == 0 ? rp : v[0], p == 1 ? rp : v[2], &ep0, &ep1, &ep2);
      effective_params(gv, p == 0 ? rm : v[0], p == 1 ? rm : v[2], &em0, &em1, &em2);
      Cx<double> gp[16], gm[16];
      gate_matrix<double>(gt.kind, ep0, ep1, ep2, gp);
      gate_matrix<double>(gt.kind, em0, em1, em2, gm);
      const double f = 0.5 / double(eps);
      for (int i = 0; i < 16; ++i)
        d[i] = Cx<double>((gp[i].re - gm[i].re) * f, (gp[i].im - gm[i].im) * f);
    } else {
      // exact derivative: dual numbers through the same gate formulas
      Dual d0(e0), d1(e1), d2(e2);
      double scale = gv.a[2 * p + 1];
      if (p == 0) d0 = Dual(e0, scale); else d1 = Dual(e1, scale);
      Cx<Dual> md[16];
      gate_matrix<Dual>(gt.kind, d0, d1, d2, md);
      for (int i = 0; i < 16; ++i) d[i] = Cx<double>(md[i].re.d, md[i].im.d);
    }
    store_mat(dst, d, nq);
  }
}

__global__ void noisy_finalize_kernel(BatchDevice b, RunArgs a) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(b.num_rows) * b.num_ops) return;
  int row = int(t / b.num_ops);
  const DevRow r = b.rows[row];
  const DevProgram p = b.programs[r.program];
  if (p.n == 0 || p.fwd_pass_begin == p.fwd_pass_end) {
    a.out_f[t] = -2.f;
    return;
  }
  int reps = a.reps[t];
  a.out_f[t] = reps > 0 ? float(a.acc[t] / double(reps)) : 0.f;
}

// ---- sampled expectation ------------------------------------------------------

// One warp per (row, op) (tfq_simulate_sampled_expectation_op.cc:139-312,
// util_qsim.h:199-270).  The reference rotates a copy of the state into the
// measurement basis of each Pauli term, draws N bitstrings and adds
// float(parity_total) * coef / float(N).  The parity of one such sample is
// +1 with probability (1 + <P>)/2, independently per sample, so this kernel
// draws the N parities directly as Bernoulli trials from the exact <P>
// (same distribution of the result) and combines them with the reference's
// float arithmetic, term by term in pauli-sum order.  Identity terms add
// their coefficient; empty programs give -2.
__global__ void sampled_expectation_kernel(BatchDevice b, RunArgs a,
                                           const int32_t* num_samples) {
  const int64_t wid = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= int64_t(b.num_rows) * b.num_ops) return;
  const int row = int(wid / b.num_ops), op = int(wid % b.num_ops);
  const DevRow r = b.rows[row];
  const DevProgram p = b.programs[r.program];
  float* out = a.out_f + wid;
  if (p.n == 0 || p.fwd_pass_begin == p.fwd_pass_end) {
    if (lane == 0) *out = -2.f;
    return;
  }
  const int N = num_samples[wid];
  float ev = 0.f;
  for (uint32_t t = r.term_begin; t < r.term_end; ++t) {
    const DevTerm term = b.terms[t];
    if (term.op != op) continue;
    if (term.identity) {
      ev += term.coef;
      continue;
    }
    const double v = a.term_vals[int64_t(row) * a.term_stride + (t - r.term_begin)];
    const double pp = fmin(fmax(0.5 + 0.5 * v, 0.0), 1.0);  // P(parity = +1)
    const double thr = pp * 4294967296.0;
    int k = 0;
    for (int s0 = 4 * lane; s0 < N; s0 += 128) {
      const uint4 u = philox(make_uint4(uint32_t(row), t, uint32_t(s0 >> 2), 0x5EA7u),
                             make_uint2(uint32_t(a.seed), uint32_t(a.seed >> 32)));
      k += (double(u.x) < thr) + (s0 + 1 < N && double(u.y) < thr) +
           (s0 + 2 < N && double(u.z) < thr) + (s0 + 3 < N && double(u.w) < thr);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    const int parity_total = 2 * k - N;
    ev += static_cast<float>(parity_total) * term.coef / static_cast<float>(N);
  }
  if (lane == 0) *out = ev;
}

// ---- inner products -----------------------------------------------------------

constexpr int kInnerChunkBits = 14;  // amplitudes per CTA of the inner product

// CTA t: pair p = t / nchunks (reference row i = p / others, paired row
// main_rows + p), chunk c = t % nchunks of 2^kInnerChunkBits amplitudes;
// adds sum_x conj(psi_i[x]) phi_p[x] over its chunk to acc[2p], acc[2p + 1]
// (ss.InnerProduct, tfq_inner_product.cc:180-199).
__global__ void __launch_bounds__(256)
inner_product_kernel(BatchDevice b, const float2* states, int64_t stride, int main_rows,
                     int others, int nchunks, double* acc) {
  __shared__ double part[2][8];
  const int64_t t = blockIdx.x;
  const int64_t p = t / nchunks;
  const int c = int(t % nchunks);
  const int i = int(p / others);
  const int n = b.rows[i].n;
  const int64_t N = int64_t(1) << n;
  const int64_t x0 = int64_t(c) << kInnerChunkBits;
  if (x0 >= N) return;  // uniform per CTA
  const int64_t x1 = min(N, x0 + (int64_t(1) << kInnerChunkBits));
  const float2* psi = states + int64_t(i) * stride;
  const float2* phi = states + (int64_t(main_rows) + p) * stride;
  float re = 0.f, im = 0.f;
  for (int64_t x = x0 + threadIdx.x; x < x1; x += blockDim.x) {
    const float2 a = psi[x], v = phi[x];
    re = fmaf(a.x, v.x, fmaf(a.y, v.y, re));
    im = fmaf(a.x, v.y, fmaf(-a.y, v.x, im));
  }
  re = warp_sum(re);
  im = warp_sum(im);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    part[0][w] = re;
    part[1][w] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < int(blockDim.x >> 5); ++k) {
      sr += part[0][k];
      si += part[1][k];
    }
    atomicAdd(acc + 2 * p, sr);
    atomicAdd(acc + 2 * p + 1, si);
  }
}

__global__ void inner_product_finalize_kernel(BatchDevice b, int main_rows, int others,
                                              const double* acc, float2* out) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= int64_t(main_rows) * others) return;
  const DevProgram pr = b.programs[b.rows[p / others].program];
  const bool empty = pr.n == 0 || pr.fwd_pass_begin == pr.fwd_pass_end;
  out[p] = empty ? make_float2(1.f, 0.f)
                 : make_float2(float(acc[2 * p]), float(acc[2 * p + 1]));
}

__global__ void paired_sum_kernel(BatchDevice b, float2* states, int64_t stride,
                                  int main_rows, int others, const float* grads, int row0) {
  const int i = row0 + int(blockIdx.y);
  const int64_t N = int64_t(1) << b.rows[i].n;
  float2* chi = states + int64_t(i) * stride;
  for (int64_t x = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; x < N;
       x += int64_t(gridDim.x) * blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    for (int j = 0; j < others; ++j) {
      const float g = grads[int64_t(i) * others + j];
      const float2 v = states[(int64_t(main_rows) + int64_t(i) * others + j) * stride + x];
      acc.x = fmaf(g, v.x, acc.x);
      acc.y = fmaf(g, v.y, acc.y);
    }
    chi[x] = acc;
  }
}

__global__ void conj_combine_kernel(const float* re, const float* im, float2* out, int64_t n) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) out[k] = make_float2(re[k], -im[k]);
}

// ---- wide rows --------------------------------------------------------------

__global__ void __launch_bounds__(kWideThreads, 2)
wide_measure_kernel(BatchDevice b, RunArgs a, int row, int mp, const float2* psi,
                    double* wacc, int term0, int state_amps) {
  wide_measure_body(b, a, row, mp, psi, wacc, term0, state_amps);
}

// Combines the term sums of a wide row into out_f[row, :] in double, with the
// measure_passes rules: Re(i^ny * sum) times the coefficient, identity terms
// contribute their coefficient (util_qsim.h:152-186).
__device__ void expect_finalize_body(const BatchDevice& b, const RunArgs& a, int row,
                                     const double* wacc, int term0, double* acc) {
  const DevRow r = b.rows[row];
  for (int j = threadIdx.x; j < b.num_ops; j += blockDim.x) acc[j] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (uint32_t mp = r.meas_begin; mp < r.meas_end; ++mp) {
      const DevMeas M = b.meas[mp];
      for (uint32_t i = M.begin; i < M.end; ++i) {
        const DevTerm t = b.terms[b.meas_terms[i].term];
        double v = 1.0;
        if (!t.identity) {
          const double sre = wacc[2 * (int64_t(i) - term0)];
          const double sim = wacc[2 * (int64_t(i) - term0) + 1];
          switch (t.ny & 3) {
            case 0: v = sre; break;
            case 1: v = -sim; break;
            case 2: v = -sre; break;
            default: v = sim; break;
          }
        }
        acc[t.op] += double(t.coef) * v;
        if (a.term_vals)
          a.term_vals[int64_t(row) * a.term_stride +
                      (b.meas_terms[i].term - r.term_begin)] = v;
      }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < b.num_ops; j += blockDim.x)
    a.out_f[int64_t(row) * b.num_ops + j] = float(acc[j]);
}

__global__ void wide_expect_finalize_kernel(BatchDevice b, RunArgs a, int row,
                                            const double* wacc, int term0,
                                            double* acc) {
  expect_finalize_body(b, a, row, wacc, term0, acc);
}

// *out = sum of |psi|^2 over the 2^13 amplitudes at `chunk` (256 threads;
// `part` is shared scratch of 8 doubles).
__device__ void chunk_sum_body(const float2* chunk, double* out, double* part) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const float4* p = reinterpret_cast<const float4*>(chunk);
  float f = 0.f;
  for (uint32_t k = threadIdx.x; k < (1u << (kTile - 1)); k += blockDim.x) {
    const float4 v = __ldcg(p + k);
    f = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, f))));
  }
  double d = f;
  for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  if (lane == 0) part[w] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) t += part[i];
    *out = t;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256)
wide_chunk_sums_kernel(const float2* psi, int n, double* csum) {
  __shared__ double part[8];
  const uint32_t nch = 1u << (n - kTile);
  for (uint32_t c = blockIdx.x; c < nch; c += gridDim.x)
    chunk_sum_body(psi + (size_t(c) << kTile), csum + c, part);
}

// One CTA: inclusive scan of the chunk sums, then one thread per sample finds
// its chunk by binary search and its index by a scan inside the chunk
// (StateSpace::Sample semantics: index x with probability |psi_x|^2; bit k
// of x goes to column max_n - k - 1, tfq_simulate_samples_op.cc:226-243).
// Samples of one row from its chunk sums (chunks of 2^cbits amplitudes).
__device__ void sample_row_body(const BatchDevice& b, const RunArgs& a, int row,
                                const float2* psi, int n, double* csum, double* seg,
                                int cbits = kTile) {
  const uint32_t nch = 1u << (n - cbits);
  const uint32_t per = (nch + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(threadIdx.x * per, nch), hi = min(lo + per, nch);
  double run = 0.0;
  for (uint32_t i = lo; i < hi; ++i) {
    run += csum[i];
    csum[i] = run;
  }
  seg[threadIdx.x] = run;
  __syncthreads();
  if (threadIdx.x == 0) {
    double off = 0.0;
    for (uint32_t t = 0; t < blockDim.x; ++t) {
      const double v = seg[t];
      seg[t] = off;
      off += v;
    }
  }
  __syncthreads();
  for (uint32_t i = lo; i < hi; ++i) csum[i] += seg[threadIdx.x];
  __syncthreads();
  const double total = csum[nch - 1];
  const int maxn = b.max_n, S = a.num_samples;
  const uint32_t L = 1u << cbits;
  int8_t* out = a.out_samples + int64_t(row) * S * maxn;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    const double u = uniform01(a.seed, uint32_t(row), uint32_t(s), 0x5A3Fu) * total;
    uint32_t c0 = 0, c1 = nch - 1;
    while (c0 < c1) {
      const uint32_t mid = (c0 + c1) >> 1;
      if (csum[mid] > u) c1 = mid; else c0 = mid + 1;
    }
    double acc = c0 ? csum[c0 - 1] : 0.0;
    const size_t first = size_t(c0) * L;
    size_t x = first, last_nz = first;
    bool found = false;
    for (uint32_t j = 0; j < L; ++j) {
      const float2 v = psi[first + j];
      const double p = double(v.x) * v.x + double(v.y) * v.y;
      if (p > 0.0) last_nz = first + j;
      acc += p;
      if (acc > u && p > 0.0) { x = first + j; found = true; break; }
    }
    if (!found) x = last_nz;
    int8_t* o = out + int64_t(s) * maxn;
    for (int c = 0; c < maxn; ++c) {
      const int k = maxn - 1 - c;
      o[c] = k >= n ? int8_t(-2) : int8_t((x >> k) & 1);
    }
  }
}

__global__ void __launch_bounds__(512)
wide_sample_kernel(BatchDevice b, RunArgs a, int row, const float2* psi, int n,
                   double* csum) {
  __shared__ double seg[512];
  sample_row_body(b, a, row, psi, n, csum, seg);
}

// ---- lockstep rows ------------------------------------------------------------
// Rows of one lockstep group run side by side, each over its own state
// (arena + off); every launch covers the tiles or chunks of all the group's
// rows, `items` giving each row's first global tile or chunk (prefix) in
// ascending order.

__device__ __forceinline__ int lock_find(const LockItem* items, int nitems, int64_t T) {
  int lo = 0, hi = nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].prefix <= T) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// First batch-wide measurement-term index of a row (0 for a row without
// measurement passes).
__device__ __forceinline__ int row_first_term(const BatchDevice& b, const DevRow& r) {
  return r.meas_begin < r.meas_end ? int(b.meas[r.meas_begin].begin) : 0;
}

// Measurement pass items[i].pass of every row: each tile's term sums go to
// wacc[2 * (acc + t) + {0, 1}], t the term's index within its row's
// measurement terms and acc the row's first accumulator.
__global__ void __launch_bounds__(kWideThreads, 2)
lock_measure_kernel(BatchDevice b, RunArgs a, const LockItem* items, int nitems,
                    int64_t ntiles, const float2* arena, double* wacc, int state_amps) {
  const Smem sm = carve_smem<kModeState>(state_amps, 1);
  for (int64_t T = blockIdx.x; T < ntiles; T += gridDim.x) {
    const LockItem it = items[lock_find(items, nitems, T)];
    RowCtx rc;
    rc.row = it.row;
    rc.traj = 0;
    rc.r = b.rows[it.row];
    rc.p = b.programs[rc.r.program];
    const int n = rc.p.n;
    const DevMeas M = b.meas[it.pass];
    const int nt = int(M.end - M.begin);
    stage_terms(b, a, sm, rc, M, false);
    for (int i = threadIdx.x; i < 2 * nt; i += blockDim.x) sm.macc[i] = 0.0;
    build_hi_table(sm.hi, M.tile_mask);
    __syncthreads();
    const uint32_t all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
    const uint32_t base = deposit(uint32_t(T - it.prefix), all & ~M.tile_mask);
    tile_load_async(sm.psi, arena + it.off, sm.hi, base);
    tile_load_wait();
    __syncthreads();
    measure_tile(sm, nt, 1u << kTile, base, false);
    __syncthreads();
    double* dst = wacc + 2 * (int64_t(it.acc) + (int64_t(M.begin) - row_first_term(b, rc.r)));
    for (int i = threadIdx.x; i < 2 * nt; i += blockDim.x)
      if (sm.macc[i] != 0.0) atomicAdd(dst + i, sm.macc[i]);
    __syncthreads();
  }
}

// out_f of every row of the group: one CTA per row (acc: num_ops doubles per row)
__global__ void lock_expect_finalize_kernel(BatchDevice b, RunArgs a, const LockItem* rows,
                                            const double* wacc, double* acc) {
  const LockItem it = rows[blockIdx.x];
  expect_finalize_body(b, a, it.row, wacc + 2 * int64_t(it.acc),
                       row_first_term(b, b.rows[it.row]), acc + int64_t(blockIdx.x) * b.num_ops);
}

// Sampling of lockstep rows uses chunks of 2^kLockChunkBits (kernels.h)
// amplitudes, so that a sample's search ends in a short scan (the chunk)
// after a binary search over the row's chunk sums.
// chunk sums of every row, one warp per chunk: chunk C of the launch (row
// item i: its chunks from rows[i].prefix) -> csum[C]
__global__ void __launch_bounds__(256)
lock_chunk_sums_kernel(const LockItem* rows, int nrows, int64_t nchunks, const float2* arena,
                       double* csum) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t C = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); C < nchunks;
       C += warps) {
    const LockItem it = rows[lock_find(rows, nrows, C)];
    const float4* p = reinterpret_cast<const float4*>(
        arena + it.off + ((C - it.prefix) << kLockChunkBits));
    float f = 0.f;
#pragma unroll
    for (int k = 0; k < (1 << (kLockChunkBits - 1)) / 32; ++k) {
      const float4 v = __ldcg(p + lane + 32 * k);
      f = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, f))));
    }
    double d = f;
    for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) csum[C] = d;
  }
}

// samples of every row: one CTA per row
__global__ void __launch_bounds__(512)
lock_sample_kernel(BatchDevice b, RunArgs a, const LockItem* rows, const float2* arena,
                   double* csum) {
  __shared__ double seg[512];
  const LockItem it = rows[blockIdx.x];
  sample_row_body(b, a, it.row, arena + it.off, it.n, csum + it.prefix, seg, kLockChunkBits);
}

// -2 padding of the state rows: amplitudes [2^n, 2^max_n) of every row
__global__ void lock_pad_kernel(BatchDevice b, RunArgs a, const LockItem* rows) {
  const LockItem it = rows[blockIdx.y];
  float2* out = a.out_state + (int64_t(it.row) << b.max_n);
  const int64_t lo = int64_t(1) << it.n, hi = int64_t(1) << b.max_n;
  for (int64_t k = lo + int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < hi;
       k += int64_t(gridDim.x) * blockDim.x)
    out[k] = make_float2(-2.f, 0.f);
}

// |0...0> in every row of `rows`, one warp per chunk of 2^kLockChunkBits
// amplitudes (16-byte stores)
__global__ void __launch_bounds__(256)
lock_zero_kernel(float2* state, int row_shift, const LockItem* rows, int nrows,
                 int64_t nchunks) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t C = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); C < nchunks;
       C += warps) {
    const LockItem it = rows[lock_find(rows, nrows, C)];
    float2* psi = state + (row_shift >= 0 ? (int64_t(it.row) << row_shift) : it.off);
    const int64_t c = C - it.prefix;
    float4* p = reinterpret_cast<float4*>(psi + (c << kLockChunkBits));
#pragma unroll
    for (int k = 0; k < (1 << (kLockChunkBits - 1)) / 32; ++k) {
      const int q = lane + 32 * k;
      __stcg(p + q, make_float4(c == 0 && q == 0 ? 1.f : 0.f, 0.f, 0.f, 0.f));
    }
  }
}

// One CTA per row: the row's outputs become markers when *status is set.
__global__ void lock_tc_poison_kernel(BatchDevice b, RunArgs a, int mode, const LockItem* rows,
                                      const int* status) {
  if (*status == 0) return;
  const LockItem it = rows[blockIdx.x];
  const float nan = __int_as_float(0x7fc00000);
  if (mode == kModeExpect) {
    for (int j = threadIdx.x; j < b.num_ops; j += blockDim.x)
      a.out_f[int64_t(it.row) * b.num_ops + j] = nan;
    if (a.term_vals) {
      const DevRow r = b.rows[it.row];
      for (uint32_t t = threadIdx.x; t < r.term_end - r.term_begin; t += blockDim.x)
        a.term_vals[int64_t(it.row) * a.term_stride + t] = nan;
    }
  } else if (mode == kModeState) {
    float2* out = a.out_state + (int64_t(it.row) << b.max_n);
    for (int64_t k = threadIdx.x; k < (int64_t(1) << it.n); k += blockDim.x)
      out[k] = make_float2(nan, nan);
  } else {
    int8_t* out = a.out_samples + int64_t(it.row) * a.num_samples * b.max_n;
    for (int64_t k = threadIdx.x; k < int64_t(a.num_samples) * b.max_n; k += blockDim.x)
      out[k] = -1;
  }
}

__global__ void fill_kernel(float2* p, int64_t count, float2 first, float2 rest) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count;
       i += int64_t(gridDim.x) * blockDim.x)
    p[i] = i == 0 ? first : rest;
}

const void* kernel_for(int mode) {
  switch (mode) {
    case kModeExpect: return sim_kernel_expect();
    case kModeState: return sim_kernel_state();
    case kModeSample: return sim_kernel_sample();
    case kModeAdjoint: return sim_kernel_adjoint();
    default: return sim_kernel_noisy();
  }
}

}  // namespace

cudaError_t launch_build_matrices(const BatchDevice& b, const RunArgs& a,
                                  bool with_grads, cudaStream_t s) {
  if (b.total_gates == 0) return cudaSuccess;
  const int threads = 128;
  int64_t blocks = (b.total_gates + threads - 1) / threads;
  build_matrices_kernel<<<unsigned(blocks), threads, 0, s>>>(b, a, with_grads ? 1 : 0, 0);
  if (b.any_fused)
    build_matrices_kernel<<<unsigned(blocks), threads, 0, s>>>(b, a, 0, 1);
  return cudaGetLastError();
}

int sim_state_amps(int max_resident_n, bool any_streamed) {
  int amps = max_resident_n >= 0 ? (1 << max_resident_n) : 0;
  if (any_streamed && amps < (1 << kTile)) amps = 1 << kTile;
  return amps < kRA ? kRA : amps;
}

size_t sim_smem_bytes(int mode, int max_resident_n, bool any_streamed,
                      int max_grads) {
  size_t amps = size_t(sim_state_amps(max_resident_n, any_streamed));
  int nstates = mode == kModeAdjoint ? 2 : 1;
  size_t bytes = amps * nstates * sizeof(float2);
  bytes += 2 * sizeof(Stage) + sizeof(RedBuf);
  bytes += (1u << kHiBits) * sizeof(uint32_t);
  bytes += 2 * 4 * kWarps * sizeof(double);
  if (mode == kModeSample || mode == kModeNoisy) bytes += kMaxChunks * sizeof(double);
  bytes += 2 * kMaxMeasTermsDev * sizeof(double) + kMaxMeasTermsDev * 16;
  if (mode == kModeExpect) bytes += kMaxOpsSmem * sizeof(double);
  if (mode == kModeAdjoint) bytes += size_t(max_grads) * sizeof(double);
  return bytes;
}

int sim_grid_size(int mode, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* k = kernel_for(mode);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kSimThreads, smem);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

cudaError_t launch_simulate(int mode, const BatchDevice& b, const RunArgs& a,
                            int grid, size_t smem, int state_amps,
                            cudaStream_t s) {
  const int nstates = mode == kModeAdjoint ? 2 : 1;
  switch (mode) {
    case kModeExpect: return sim_launch_expect(b, a, grid, smem, state_amps, nstates, s);
    case kModeState: return sim_launch_state(b, a, grid, smem, state_amps, nstates, s);
    case kModeSample: return sim_launch_sample(b, a, grid, smem, state_amps, nstates, s);
    case kModeAdjoint: return sim_launch_adjoint(b, a, grid, smem, state_amps, nstates, s);
    default: return sim_launch_noisy(b, a, grid, smem, state_amps, nstates, s);
  }
}

cudaError_t launch_sampled_expectation(const BatchDevice& b, const RunArgs& a,
                                       const int32_t* num_samples, cudaStream_t s) {
  const int64_t warps = int64_t(b.num_rows) * b.num_ops;
  if (warps == 0) return cudaSuccess;
  const int threads = 256;
  const int64_t blocks = (warps * 32 + threads - 1) / threads;
  sampled_expectation_kernel<<<unsigned(blocks), threads, 0, s>>>(b, a, num_samples);
  return cudaGetLastError();
}

cudaError_t launch_inner_products(const BatchDevice& b, const float2* states,
                                  int64_t stride, int main_rows, int others,
                                  double* acc, float2* out, cudaStream_t s) {
  const int64_t pairs = int64_t(main_rows) * others;
  if (pairs == 0) return cudaSuccess;
  const int nchunks = int(std::max<int64_t>(1, stride >> kInnerChunkBits));
  inner_product_kernel<<<unsigned(pairs * nchunks), 256, 0, s>>>(b, states, stride, main_rows,
                                                                  others, nchunks, acc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  inner_product_finalize_kernel<<<unsigned((pairs + 255) / 256), 256, 0, s>>>(
      b, main_rows, others, acc, out);
  return cudaGetLastError();
}

cudaError_t launch_paired_sum(const BatchDevice& b, float2* states, int64_t stride,
                              int main_rows, int others, const float* grads,
                              cudaStream_t s) {
  if (main_rows == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((stride + 255) / 256, 1024);
  for (int row0 = 0; row0 < main_rows; row0 += 65535) {  // grid.y limit
    const int rows = std::min(65535, main_rows - row0);
    paired_sum_kernel<<<dim3(unsigned(blocks), unsigned(rows)), 256, 0, s>>>(
        b, states, stride, main_rows, others, grads, row0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_conj_combine(const float* re, const float* im, float2* out, int64_t n,
                                cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  conj_combine_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(re, im, out, n);
  return cudaGetLastError();
}

cudaError_t launch_noisy_finalize(const BatchDevice& b, const RunArgs& a,
                                  cudaStream_t s) {
  int64_t total = int64_t(b.num_rows) * b.num_ops;
  if (total == 0) return cudaSuccess;
  noisy_finalize_kernel<<<unsigned((total + 255) / 256), 256, 0, s>>>(b, a);
  return cudaGetLastError();
}

const void* wide_measure_kernel_ptr() {
  return reinterpret_cast<const void*>(&wide_measure_kernel);
}

cudaError_t launch_wide_measure(const BatchDevice& b, const RunArgs& a, int row, int mp,
                                const float2* psi, double* wacc, int term0, int grid,
                                size_t smem, int state_amps, cudaStream_t s) {
  wide_measure_kernel<<<grid, kWideThreads, smem, s>>>(b, a, row, mp, psi, wacc, term0,
                                                      state_amps);
  return cudaGetLastError();
}

cudaError_t launch_wide_expect_finalize(const BatchDevice& b, const RunArgs& a, int row,
                                        const double* wacc, int term0, double* scratch,
                                        cudaStream_t s) {
  wide_expect_finalize_kernel<<<1, 256, 0, s>>>(b, a, row, wacc, term0, scratch);
  return cudaGetLastError();
}

cudaError_t launch_wide_chunk_sums(const float2* psi, int n, double* csum, int grid,
                                   cudaStream_t s) {
  wide_chunk_sums_kernel<<<grid, 256, 0, s>>>(psi, n, csum);
  return cudaGetLastError();
}

cudaError_t launch_wide_sample(const BatchDevice& b, const RunArgs& a, int row,
                               const float2* psi, int n, double* csum, cudaStream_t s) {
  wide_sample_kernel<<<1, 512, 0, s>>>(b, a, row, psi, n, csum);
  return cudaGetLastError();
}

const void* lock_measure_kernel_ptr() {
  return reinterpret_cast<const void*>(&lock_measure_kernel);
}

cudaError_t launch_lock_measure(const BatchDevice& b, const RunArgs& a, const LockItem* items,
                                int nitems, int64_t ntiles, const float2* arena,
                                double* wacc, int grid, size_t smem, int state_amps,
                                cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  lock_measure_kernel<<<grid, kWideThreads, smem, s>>>(b, a, items, nitems, ntiles, arena,
                                                      wacc, state_amps);
  return cudaGetLastError();
}

cudaError_t launch_lock_expect_finalize(const BatchDevice& b, const RunArgs& a,
                                        const LockItem* rows, int nrows, const double* wacc,
                                        double* scratch, cudaStream_t s) {
  if (nrows <= 0) return cudaSuccess;
  lock_expect_finalize_kernel<<<nrows, 256, 0, s>>>(b, a, rows, wacc, scratch);
  return cudaGetLastError();
}

cudaError_t launch_lock_chunk_sums(const LockItem* rows, int nrows, int64_t nchunks,
                                   const float2* arena, double* csum, int grid,
                                   cudaStream_t s) {
  if (nchunks <= 0) return cudaSuccess;
  lock_chunk_sums_kernel<<<grid, 256, 0, s>>>(rows, nrows, nchunks, arena, csum);
  return cudaGetLastError();
}

cudaError_t launch_lock_sample(const BatchDevice& b, const RunArgs& a, const LockItem* rows,
                               int nrows, const float2* arena, double* csum,
                               cudaStream_t s) {
  if (nrows <= 0) return cudaSuccess;
  lock_sample_kernel<<<nrows, 512, 0, s>>>(b, a, rows, arena, csum);
  return cudaGetLastError();
}

cudaError_t launch_lock_pad(const BatchDevice& b, const RunArgs& a, const LockItem* rows,
                            int nrows, cudaStream_t s) {
  if (nrows <= 0) return cudaSuccess;
  lock_pad_kernel<<<dim3(8, unsigned(nrows)), 256, 0, s>>>(b, a, rows);
  return cudaGetLastError();
}

cudaError_t launch_lock_zero(float2* state, int row_shift, const LockItem* rows, int nrows,
                             int64_t nchunks, int grid, cudaStream_t s) {
  if (nrows <= 0 || nchunks <= 0) return cudaSuccess;
  lock_zero_kernel<<<grid, 256, 0, s>>>(state, row_shift, rows, nrows, nchunks);
  return cudaGetLastError();
}

cudaError_t launch_lock_tc_poison(const BatchDevice& b, const RunArgs& a, int mode,
                                  const LockItem* rows, int nrows, const int* status,
                                  cudaStream_t s) {
  if (nrows <= 0) return cudaSuccess;
  lock_tc_poison_kernel<<<nrows, 256, 0, s>>>(b, a, mode, rows, status);
  return cudaGetLastError();
}

cudaError_t launch_fill(float2* p, int64_t count, float2 first, float2 rest, int grid,
                        cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  fill_kernel<<<grid, 256, 0, s>>>(p, count, first, rest);
  return cudaGetLastError();
}

}  // namespace tfqg
