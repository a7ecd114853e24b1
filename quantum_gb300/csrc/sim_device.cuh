// Device code of the simulation kernels, shared by the precompiled library
// (kernels.cu) and by batch-specialized code compiled at run time (jit.cc):
// state layout helpers, register-level gate application, sub-pass staging,
// tile passes, measurement, lambda, sampling and the per-row driver.
#pragma once
#ifdef __CUDACC_RTC__
#include "rtc_types.h"
#else
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "kernels.h"
#include "tfqg_types.h"

namespace tfqg {
namespace {


// Dynamic shared memory of the simulation kernel (layout set up in
// simulate_kernel); device functions address it by byte offset so every
// access compiles to a shared-space load/store.
extern __shared__ __align__(16) unsigned char smem_raw[];

constexpr int kTile = 13;              // streamed tile bits (matches host)
constexpr int kHiBits = kTile - 5;     // tile bits above the 5 lane bits
constexpr int kMaxChunks = 1024;       // sampler prefix chunks
constexpr int kWarps = kSimThreads / 32;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cfma(float2 m, float2 a, float2 acc) {
  acc.x = fmaf(m.x, a.x, fmaf(-m.y, a.y, acc.x));
  acc.y = fmaf(m.x, a.y, fmaf(m.y, a.x, acc.y));
  return acc;
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ uint32_t ins0(uint32_t i, int b) {
  return ((i >> b) << (b + 1)) | (i & ((1u << b) - 1u));
}
// Shared-memory position of amplitude x: the index nibbles above bit 3 are
// XOR-folded into the low nibble, so the 16 lanes of a half warp that walk
// any 4 index bits hit 16 distinct bank pairs.  Linear over GF(2):
// swz(a ^ b) = swz(a) ^ swz(b); an involution.
__device__ __forceinline__ uint32_t swz(uint32_t x) {
  return x ^ ((x >> 4) & 15u) ^ ((x >> 8) & 15u) ^ ((x >> 12) & 15u);
}
__device__ __forceinline__ uint32_t sidx(uint32_t x, bool shared) {
  return shared ? swz(x) : x;
}

// Re(conj(a) * b)
__device__ __forceinline__ float re_conj_mul(float2 a, float2 b) {
  return fmaf(a.x, b.x, a.y * b.y);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp sums of P values at once (P a power of two, <= 32) by a transposing
// butterfly: at each of the first log2(P) steps a lane keeps half of its
// values, sends the other half to its partner lane and adds what it gets
// back, so the value count halves while the lanes holding one value double.
// Then value j of the warp total sits in the lanes whose bits 4, 3, ... spell
// j; the remaining low lane bits are summed with plain butterflies.  Lane
// (j << (5 - log2 P)) returns value j; the result in other lanes is partial.
// Costs (P - 1) + (5 - log2 P) shuffles instead of 5 P.
template <int P>
__device__ __forceinline__ float warp_sum_many(float (&v)[P], int lane) {
  static_assert(P >= 1 && P <= 32 && (P & (P - 1)) == 0, "P: power of two <= 32");
  int m = P;
#pragma unroll
  for (int off = 16; off >= 1 && m > 1; off >>= 1) {
    const bool up = lane & off;
    m >>= 1;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (j < m) {
        const float send = up ? v[j] : v[j + m];
        const float keep = up ? v[j + m] : v[j];
        v[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
      }
    }
  }
  float s = v[0];
  constexpr int kSteps = (P >= 32) ? 5 : (P >= 16) ? 4 : (P >= 8) ? 3 : (P >= 4) ? 2 : (P >= 2) ? 1 : 0;
#pragma unroll
  for (int off = 16 >> kSteps; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}
// Uniform double in [0, 1) with 53 random bits.
__device__ __forceinline__ double uniform01(uint64_t seed, uint32_t a,
                                            uint32_t b, uint32_t c) {
  uint4 r = philox(make_uint4(a, b, c, 0x9A7Eu),
                   make_uint2(uint32_t(seed), uint32_t(seed >> 32)));
  return (double(r.x >> 5) * 67108864.0 + double(r.y >> 6)) *
         (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// simulation building blocks (all threads of the CTA take part)
// ---------------------------------------------------------------------------
constexpr int kRB = 4;            // register bits of forward sub-passes
constexpr int kRA = 1 << kRB;     // amplitudes per forward thread group
constexpr int kMaxOps = 32;       // ops per sub-pass (host kMaxSubOps)

// One sub-pass staged in shared memory: descriptors, matrices and
// derivative matrices.  Two of these alternate, so that sub-pass k + 1 is
// staged while sub-pass k runs and one barrier separates them.
struct Stage {
  uint32_t code[kMaxOps];
  uint32_t lcmask[kMaxOps], lcval[kMaxOps], gcmask[kMaxOps], gcval[kMaxOps];
  float2 mat[kMaxOps][16];
  float2 dmat[kMaxOps][2][16];
};

// Gradient partials of the adjoint's sub-passes.  Sub-pass k writes its
// per-warp partials to red[k & 1]; after the barrier that ends it, the
// partials are summed into the accumulators while sub-pass k + 1 runs and
// sub-pass k + 2 is staged, so the slot lists rotate through three buffers.
struct RedBuf {
  float red[2][2 * kMaxOps][kWarps];  // [k & 1][grad entry of the sub-pass][warp]
  int32_t red_slot[3][2 * kMaxOps];   // [k % 3]: derivative slot of each entry
  int32_t nred[3];
  int32_t pad;
};
// carve_smem places sections back to back: every section size must keep the
// 16-byte alignment of the next (float4 staging, double scratch)
static_assert(sizeof(Stage) % 16 == 0, "Stage size must be a multiple of 16");
static_assert(sizeof(RedBuf) % 16 == 0, "RedBuf size must be a multiple of 16");

struct Smem {
  float2* psi;        // resident state / tile
  float2* lam;        // adjoint state / tile
  uint32_t* hi;       // tile-local high bits -> global offsets
  double* red;        // [2][4][kWarps] reduction scratch (terms, channels)
  double* csum;       // sampler chunk prefix sums
  double* grad;       // adjoint accumulators
  Stage* st;          // [2] staged sub-passes
  RedBuf* rb;
  double* macc;       // [2 * kMaxMeasTerms] term sums (re, im)
  // ny: bits 0-1 the Y count mod 4, bit 2 parity(flip & zy) (global bits)
  struct MTerm { float w; uint32_t lflip, zy; uint16_t op; uint8_t ny, identity; }* mterm;
  double* oacc;       // [kMaxOpsSmem] per-op sums (expectation mode)
};
constexpr int kMaxMeasTermsDev = 128;  // host kMaxMeasTerms
constexpr int kMaxOpsSmem = 1024;

__device__ __forceinline__ void warp_partials(double* red, int buf,
                                              const float* vals, int nv) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int v = 0; v < nv; ++v) {
    float s = warp_sum(vals[v]);
    if (lane == 0) red[(buf * 4 + v) * kWarps + w] = double(s);
  }
}

__device__ __forceinline__ double red_total(const double* red, int buf, int v) {
  double s = 0.0;
  const int nw = int(blockDim.x >> 5);  // kernels run with <= kWarps warps
  for (int w = 0; w < nw; ++w) s += red[(buf * 4 + v) * kWarps + w];
  return s;
}

// ---- register-level gate application ----
// Every function reads `in` and writes every element of `out` (ping-pong
// arrays): results land directly in their final registers, so consecutive
// gates need no register shuffling.  J is the target's register bit.
#define TFQG_PAIRS_IO(J, ...)                                           \
  _Pragma("unroll") for (int k = 0; k < NA; ++k) {                      \
    if (k & (1 << (J))) continue;                                       \
    const int k1 = k | (1 << (J));                                      \
    if ((k & kmask) == kval) { __VA_ARGS__ } else { out[k] = in[k]; out[k1] = in[k1]; } \
  }

template <int J, int NA>
__device__ __forceinline__ void f1_general(const float2 (&in)[NA], float2 (&out)[NA],
                                           const float2* m, int kmask, int kval) {
  const float2 m0 = m[0], m1 = m[1], m2 = m[2], m3 = m[3];
  const float2 z = make_float2(0.f, 0.f);
  TFQG_PAIRS_IO(J, {
    out[k] = cfma(m1, in[k1], cfma(m0, in[k], z));
    out[k1] = cfma(m3, in[k1], cfma(m2, in[k], z));
  })
}

template <int J, int NA>
__device__ __forceinline__ void f1_real(const float2 (&in)[NA], float2 (&out)[NA],
                                        const float2* m, int kmask, int kval) {
  const float m0 = m[0].x, m1 = m[1].x, m2 = m[2].x, m3 = m[3].x;
  TFQG_PAIRS_IO(J, {
    const float2 x = in[k], y = in[k1];
    out[k] = make_float2(fmaf(m0, x.x, m1 * y.x), fmaf(m0, x.y, m1 * y.y));
    out[k1] = make_float2(fmaf(m2, x.x, m3 * y.x), fmaf(m2, x.y, m3 * y.y));
  })
}

template <int J, int NA>
__device__ __forceinline__ void f1_diag(const float2 (&in)[NA], float2 (&out)[NA],
                                        const float2* m, int kmask, int kval) {
  const float2 d0 = m[0], d1 = m[3];
  TFQG_PAIRS_IO(J, {
    out[k] = cmul(d0, in[k]);
    out[k1] = cmul(d1, in[k1]);
  })
}

template <int J, int NA>
__device__ __forceinline__ void f1_x(const float2 (&in)[NA], float2 (&out)[NA],
                                     int kmask, int kval) {
  TFQG_PAIRS_IO(J, {
    out[k] = in[k1];
    out[k1] = in[k];
  })
}

// X on register bit J controlled by register bit C having value V.
template <int J, int C, int V, int NA>
__device__ __forceinline__ void f1_cx(const float2 (&in)[NA], float2 (&out)[NA]) {
#pragma unroll
  for (int k = 0; k < NA; ++k)
    out[k] = (((k >> C) & 1) == V) ? in[k ^ (1 << J)] : in[k];
}

template <int NA>
__device__ __forceinline__ void copy_regs(const float2 (&in)[NA], float2 (&out)[NA]) {
#pragma unroll
  for (int k = 0; k < NA; ++k) out[k] = in[k];
}

#define TFQG_QUADS_IO(J0, J1, ...)                                                \
  _Pragma("unroll") for (int k = 0; k < NA; ++k) {                                \
    if (k & ((1 << (J0)) | (1 << (J1)))) continue;                                \
    const int idx[4] = {k, k | (1 << (J1)), k | (1 << (J0)), k | (1 << (J0)) | (1 << (J1))}; \
    if ((k & kmask) == kval) { __VA_ARGS__ } else {                               \
      _Pragma("unroll") for (int q = 0; q < 4; ++q) out[idx[q]] = in[idx[q]];     \
    }                                                                             \
  }

template <int J0, int J1, int NA>
__device__ __forceinline__ void f2_general(const float2 (&in)[NA], float2 (&out)[NA],
                                           const float2* m, int kmask, int kval) {
  TFQG_QUADS_IO(J0, J1, {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < 4; ++q) acc = cfma(m[r * 4 + q], in[idx[q]], acc);
      out[idx[r]] = acc;
    }
  })
}

template <int J0, int J1, int NA>
__device__ __forceinline__ void f2_diag(const float2 (&in)[NA], float2 (&out)[NA],
                                        const float2* m, int kmask, int kval) {
  const float2 d[4] = {m[0], m[5], m[10], m[15]};
  TFQG_QUADS_IO(J0, J1, {
#pragma unroll
    for (int q = 0; q < 4; ++q) out[idx[q]] = cmul(d[q], in[idx[q]]);
  })
}

// Adjoint step on a 1-qubit gate: psi <- G^dag psi; part[g] += Re <lam| dG_g
// psi>; lam <- G^dag lam (tfq_adj_grad_op.cc:225-275).
template <int J, int CLS, int NA, int NG>
__device__ __forceinline__ void b1(const float2 (&a)[NA], const float2 (&l)[NA],
                                   float2 (&ao)[NA], float2 (&lo)[NA],
                                   const float2* m, const float2* dm, int kmask,
                                   int kval, float* part) {
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    if (k & (1 << J)) continue;
    const int k1 = k | (1 << J);
    if ((k & kmask) != kval) {
      ao[k] = a[k]; ao[k1] = a[k1]; lo[k] = l[k]; lo[k1] = l[k1];
      continue;
    }
    const float2 x = a[k], y = a[k1], u = l[k], v = l[k1];
    const float2 z = make_float2(0.f, 0.f);
    float2 p0, p1, q0, q1;
    if (CLS == GC_X) {
      p0 = y; p1 = x; q0 = v; q1 = u;
    } else if (CLS == GC_DIAG) {
      const float2 d0 = cconj(m[0]), d1 = cconj(m[3]);
      p0 = cmul(d0, x); p1 = cmul(d1, y);
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float2* D = dm + g * 16;
        part[g] += re_conj_mul(u, cmul(D[0], p0)) + re_conj_mul(v, cmul(D[3], p1));
      }
      q0 = cmul(d0, u); q1 = cmul(d1, v);
    } else if (CLS == GC_REAL) {
      const float h0 = m[0].x, h1 = m[2].x, h2 = m[1].x, h3 = m[3].x;  // G^T
      p0 = make_float2(fmaf(h0, x.x, h1 * y.x), fmaf(h0, x.y, h1 * y.y));
      p1 = make_float2(fmaf(h2, x.x, h3 * y.x), fmaf(h2, x.y, h3 * y.y));
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float2* D = dm + g * 16;
        float2 e0 = make_float2(fmaf(D[0].x, p0.x, D[1].x * p1.x), fmaf(D[0].x, p0.y, D[1].x * p1.y));
        float2 e1 = make_float2(fmaf(D[2].x, p0.x, D[3].x * p1.x), fmaf(D[2].x, p0.y, D[3].x * p1.y));
        part[g] += re_conj_mul(u, e0) + re_conj_mul(v, e1);
      }
      q0 = make_float2(fmaf(h0, u.x, h1 * v.x), fmaf(h0, u.y, h1 * v.y));
      q1 = make_float2(fmaf(h2, u.x, h3 * v.x), fmaf(h2, u.y, h3 * v.y));
    } else {
      const float2 h0 = cconj(m[0]), h1 = cconj(m[2]), h2 = cconj(m[1]), h3 = cconj(m[3]);
      p0 = cfma(h1, y, cfma(h0, x, z));
      p1 = cfma(h3, y, cfma(h2, x, z));
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float2* D = dm + g * 16;
        float2 e0 = cfma(D[1], p1, cfma(D[0], p0, z));
        float2 e1 = cfma(D[3], p1, cfma(D[2], p0, z));
        part[g] += re_conj_mul(u, e0) + re_conj_mul(v, e1);
      }
      q0 = cfma(h1, v, cfma(h0, u, z));
      q1 = cfma(h3, v, cfma(h2, u, z));
    }
    ao[k] = p0; ao[k1] = p1; lo[k] = q0; lo[k1] = q1;
  }
}

template <int J0, int J1, int CLS, int NA, int NG>
__device__ __forceinline__ void b2(const float2 (&a)[NA], const float2 (&l)[NA],
                                   float2 (&ao)[NA], float2 (&lo)[NA],
                                   const float2* m, const float2* dm, int kmask,
                                   int kval, float* part) {
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    if (k & ((1 << J0) | (1 << J1))) continue;
    const int idx[4] = {k, k | (1 << J1), k | (1 << J0), k | (1 << J0) | (1 << J1)};
    if ((k & kmask) != kval) {
#pragma unroll
      for (int q = 0; q < 4; ++q) { ao[idx[q]] = a[idx[q]]; lo[idx[q]] = l[idx[q]]; }
      continue;
    }
    float2 x[4], u[4], p[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) { x[q] = a[idx[q]]; u[q] = l[idx[q]]; }
    if (CLS == GC_DIAG) {
#pragma unroll
      for (int q = 0; q < 4; ++q) p[q] = cmul(cconj(m[5 * q]), x[q]);
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float2* D = dm + g * 16;
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) acc += re_conj_mul(u[q], cmul(D[5 * q], p[q]));
        part[g] += acc;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ao[idx[q]] = p[q];
        lo[idx[q]] = cmul(cconj(m[5 * q]), u[q]);
      }
    } else {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < 4; ++q) acc = cfma(cconj(m[q * 4 + r]), x[q], acc);
        p[r] = acc;
      }
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float2* D = dm + g * 16;
        float acc = 0.f;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          float2 dv = make_float2(0.f, 0.f);
#pragma unroll
          for (int q = 0; q < 4; ++q) dv = cfma(D[r * 4 + q], p[q], dv);
          acc += re_conj_mul(u[r], dv);
        }
        part[g] += acc;
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < 4; ++q) acc = cfma(cconj(m[q * 4 + r]), u[q], acc);
        ao[idx[r]] = p[r];
        lo[idx[r]] = acc;
      }
    }
  }
}

// Dispatch on the runtime register bits; every case is fully unrolled.
#define TFQG_J4(F, ...)                        \
  switch (j0) {                                \
    case 0: F<0, NA>(__VA_ARGS__); break;      \
    case 1: F<1, NA>(__VA_ARGS__); break;      \
    case 2: F<2, NA>(__VA_ARGS__); break;      \
    default: F<3, NA>(__VA_ARGS__); break;     \
  }
#define TFQG_J12(F, ...)                       \
  switch (j0 * 4 + j1) {                       \
    case 1: F<0, 1, NA>(__VA_ARGS__); break;   \
    case 2: F<0, 2, NA>(__VA_ARGS__); break;   \
    case 3: F<0, 3, NA>(__VA_ARGS__); break;   \
    case 4: F<1, 0, NA>(__VA_ARGS__); break;   \
    case 6: F<1, 2, NA>(__VA_ARGS__); break;   \
    case 7: F<1, 3, NA>(__VA_ARGS__); break;   \
    case 8: F<2, 0, NA>(__VA_ARGS__); break;   \
    case 9: F<2, 1, NA>(__VA_ARGS__); break;   \
    case 11: F<2, 3, NA>(__VA_ARGS__); break;  \
    case 12: F<3, 0, NA>(__VA_ARGS__); break;  \
    case 13: F<3, 1, NA>(__VA_ARGS__); break;  \
    default: F<3, 2, NA>(__VA_ARGS__); break;  \
  }
#define TFQG_CX(NA_, I, O)                                                      \
  switch ((j0 * 4 + jc) * 2 + cv) {                                            \
    case 2: f1_cx<0, 1, 0, NA_>(I, O); break;  case 3: f1_cx<0, 1, 1, NA_>(I, O); break; \
    case 4: f1_cx<0, 2, 0, NA_>(I, O); break;  case 5: f1_cx<0, 2, 1, NA_>(I, O); break; \
    case 6: f1_cx<0, 3, 0, NA_>(I, O); break;  case 7: f1_cx<0, 3, 1, NA_>(I, O); break; \
    case 8: f1_cx<1, 0, 0, NA_>(I, O); break;  case 9: f1_cx<1, 0, 1, NA_>(I, O); break; \
    case 12: f1_cx<1, 2, 0, NA_>(I, O); break; case 13: f1_cx<1, 2, 1, NA_>(I, O); break; \
    case 14: f1_cx<1, 3, 0, NA_>(I, O); break; case 15: f1_cx<1, 3, 1, NA_>(I, O); break; \
    case 16: f1_cx<2, 0, 0, NA_>(I, O); break; case 17: f1_cx<2, 0, 1, NA_>(I, O); break; \
    case 18: f1_cx<2, 1, 0, NA_>(I, O); break; case 19: f1_cx<2, 1, 1, NA_>(I, O); break; \
    case 22: f1_cx<2, 3, 0, NA_>(I, O); break; case 23: f1_cx<2, 3, 1, NA_>(I, O); break; \
    case 24: f1_cx<3, 0, 0, NA_>(I, O); break; case 25: f1_cx<3, 0, 1, NA_>(I, O); break; \
    case 26: f1_cx<3, 1, 0, NA_>(I, O); break; case 27: f1_cx<3, 1, 1, NA_>(I, O); break; \
    case 28: f1_cx<3, 2, 0, NA_>(I, O); break; default: f1_cx<3, 2, 1, NA_>(I, O); break; \
  }
#define TFQG_B3(F, NG_, ...)                          \
  switch (j0) {                                       \
    case 0: F<0, NA, NG_>(__VA_ARGS__); break;        \
    case 1: F<1, NA, NG_>(__VA_ARGS__); break;        \
    default: F<2, NA, NG_>(__VA_ARGS__); break;       \
  }
#define TFQG_B6(F, NG_, ...)                          \
  switch (j0 * 4 + j1) {                              \
    case 1: F<0, 1, NA, NG_>(__VA_ARGS__); break;     \
    case 2: F<0, 2, NA, NG_>(__VA_ARGS__); break;     \
    case 4: F<1, 0, NA, NG_>(__VA_ARGS__); break;     \
    case 6: F<1, 2, NA, NG_>(__VA_ARGS__); break;     \
    case 8: F<2, 0, NA, NG_>(__VA_ARGS__); break;     \
    default: F<2, 1, NA, NG_>(__VA_ARGS__); break;    \
  }

#define TFQG_B1_WRAP(NAME, CLS)                                                  \
  template <int J, int NA, int NG>                                               \
  __device__ __forceinline__ void NAME(const float2 (&a)[NA], const float2 (&l)[NA], \
                                       float2 (&ao)[NA], float2 (&lo)[NA],       \
                                       const float2* m, const float2* dm,        \
                                       int kmask, int kval, float* part) {       \
    b1<J, CLS, NA, NG>(a, l, ao, lo, m, dm, kmask, kval, part);                  \
  }
TFQG_B1_WRAP(b1_x, GC_X)
TFQG_B1_WRAP(b1_diag, GC_DIAG)
TFQG_B1_WRAP(b1_real, GC_REAL)
TFQG_B1_WRAP(b1_general, GC_GENERAL)
#define TFQG_B2_WRAP(NAME, CLS)                                                  \
  template <int J0, int J1, int NA, int NG>                                      \
  __device__ __forceinline__ void NAME(const float2 (&a)[NA], const float2 (&l)[NA], \
                                       float2 (&ao)[NA], float2 (&lo)[NA],       \
                                       const float2* m, const float2* dm,        \
                                       int kmask, int kval, float* part) {       \
    b2<J0, J1, CLS, NA, NG>(a, l, ao, lo, m, dm, kmask, kval, part);             \
  }
TFQG_B2_WRAP(b2_diag, GC_DIAG)
TFQG_B2_WRAP(b2_general, GC_GENERAL)

constexpr int kFwdRB = 4;  // register bits of forward sub-passes
constexpr int kBwdRB = 3;  // register bits of adjoint sub-passes (psi + lambda)

// One forward gate: in -> out (every element of out written).
__device__ __forceinline__ void apply_forward(uint32_t code,
                                              const float2 (&in)[1 << kFwdRB],
                                              float2 (&out)[1 << kFwdRB],
                                              const float2* m) {
  constexpr int NA = 1 << kFwdRB;
  const int type = code & 7, cls = (code >> 3) & 7, j0 = (code >> 6) & 3,
            j1 = (code >> 8) & 3, kmask = (code >> 10) & 15, kval = (code >> 14) & 15;
  if (type == OP_F1 || type == OP_MCH) {
    if (cls == GC_SKIP) { copy_regs(in, out); return; }
    if (kmask == 0) {
      switch (cls) {
        case GC_REAL: TFQG_J4(f1_real, in, out, m, 0, 0); break;
        case GC_DIAG: TFQG_J4(f1_diag, in, out, m, 0, 0); break;
        case GC_X: TFQG_J4(f1_x, in, out, 0, 0); break;
        default: TFQG_J4(f1_general, in, out, m, 0, 0); break;
      }
    } else if (cls == GC_X && ((code >> 21) & 1)) {
      const int jc = (code >> 22) & 3, cv = (code >> 24) & 1;
      TFQG_CX(NA, in, out);
    } else {
      switch (cls) {
        case GC_REAL: TFQG_J4(f1_real, in, out, m, kmask, kval); break;
        case GC_DIAG: TFQG_J4(f1_diag, in, out, m, kmask, kval); break;
        case GC_X: TFQG_J4(f1_x, in, out, kmask, kval); break;
        default: TFQG_J4(f1_general, in, out, m, kmask, kval); break;
      }
    }
  } else {
    if (cls == GC_DIAG) {
      if (kmask == 0) { TFQG_J12(f2_diag, in, out, m, 0, 0); }
      else { TFQG_J12(f2_diag, in, out, m, kmask, kval); }
    } else {
      if (kmask == 0) { TFQG_J12(f2_general, in, out, m, 0, 0); }
      else { TFQG_J12(f2_general, in, out, m, kmask, kval); }
    }
  }
}

// One adjoint step: (a, l) -> (ao, lo).
__device__ __forceinline__ void apply_backward(uint32_t code,
                                               const float2 (&a)[1 << kBwdRB],
                                               const float2 (&l)[1 << kBwdRB],
                                               float2 (&ao)[1 << kBwdRB],
                                               float2 (&lo)[1 << kBwdRB],
                                               const float2* m,
                                               const float2* dm, float* part) {
  constexpr int NA = 1 << kBwdRB;
  const int type = code & 7, cls = (code >> 3) & 7, j0 = (code >> 6) & 3,
            j1 = (code >> 8) & 3, kmask = (code >> 10) & 15, kval = (code >> 14) & 15;
  const int ng = (code >> 18) & 3;
  if (type == OP_B1) {
    if (cls == GC_X && ((code >> 21) & 1)) {
      // X is its own adjoint and has no parameters: permute psi and lambda
      const int jc = (code >> 22) & 3, cv = (code >> 24) & 1;
      TFQG_CX(NA, a, ao);
      TFQG_CX(NA, l, lo);
      return;
    }
#define TFQG_B1_ALL(NG_, KM, KV)                                                   \
    switch (cls) {                                                                 \
      case GC_X: TFQG_B3(b1_x, NG_, a, l, ao, lo, m, dm, KM, KV, part); break;     \
      case GC_DIAG: TFQG_B3(b1_diag, NG_, a, l, ao, lo, m, dm, KM, KV, part); break; \
      case GC_REAL: TFQG_B3(b1_real, NG_, a, l, ao, lo, m, dm, KM, KV, part); break; \
      default: TFQG_B3(b1_general, NG_, a, l, ao, lo, m, dm, KM, KV, part); break; \
    }
    if (kmask == 0) {
      if (ng == 0) { TFQG_B1_ALL(0, 0, 0) }
      else if (ng == 1) { TFQG_B1_ALL(1, 0, 0) }
      else { TFQG_B1_ALL(2, 0, 0) }
    } else {
      if (ng == 0) { TFQG_B1_ALL(0, kmask, kval) }
      else if (ng == 1) { TFQG_B1_ALL(1, kmask, kval) }
      else { TFQG_B1_ALL(2, kmask, kval) }
    }
#undef TFQG_B1_ALL
  } else {
#define TFQG_B2_ALL(NG_, KM, KV)                                                   \
    if (cls == GC_DIAG) {                                                          \
      TFQG_B6(b2_diag, NG_, a, l, ao, lo, m, dm, KM, KV, part);                    \
    } else {                                                                       \
      TFQG_B6(b2_general, NG_, a, l, ao, lo, m, dm, KM, KV, part);                 \
    }
    if (kmask == 0) {
      if (ng == 0) { TFQG_B2_ALL(0, 0, 0) }
      else if (ng == 1) { TFQG_B2_ALL(1, 0, 0) }
      else { TFQG_B2_ALL(2, 0, 0) }
    } else {
      if (ng == 0) { TFQG_B2_ALL(0, kmask, kval) }
      else if (ng == 1) { TFQG_B2_ALL(1, kmask, kval) }
      else { TFQG_B2_ALL(2, kmask, kval) }
    }
#undef TFQG_B2_ALL
  }
}

__device__ __forceinline__ uint32_t group_base(uint32_t g, uint32_t rbits, int rb) {
  // insert zeros at the register bits, lowest first
  for (int j = 0; j < rb; ++j) g = ins0(g, int((rbits >> (8 * j)) & 0xFF));
  return g;
}

__device__ __forceinline__ bool op_active(const Stage* st, int i, uint32_t code,
                                          uint32_t gb, uint32_t base) {
  return !((code >> 20) & 1) ||
         ((gb & st->lcmask[i]) == st->lcval[i] && (base & st->gcmask[i]) == st->gcval[i]);
}

#ifndef TFQG_JIT
// Forward sub-pass: each thread group loads the 16 amplitudes spanning the
// register bits, applies the staged ops in registers (ping-pong between two
// arrays), stores once.  Compiled once and shared by every kernel mode.
__device__ __noinline__ void exec_forward(uint32_t s_off, int T, uint32_t base,
                                          uint32_t st_off, int nops,
                                          uint32_t rbits) {
  constexpr int RB = kFwdRB, NA = 1 << RB;
  float2* s = reinterpret_cast<float2*>(smem_raw + s_off);
  const Stage* st = reinterpret_cast<const Stage*>(smem_raw + st_off);
  uint32_t soff[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    uint32_t o = 0;
#pragma unroll
    for (int j = 0; j < RB; ++j)
      if (k >> j & 1) o |= 1u << ((rbits >> (8 * j)) & 0xFF);
    soff[k] = swz(o);
  }
  const uint32_t ngroups = 1u << (T - RB);
  for (uint32_t g = threadIdx.x; g < ngroups; g += blockDim.x) {
    const uint32_t gb = group_base(g, rbits, RB);
    const uint32_t sgb = swz(gb);
    float2 A[NA], B[NA];
#pragma unroll
    for (int k = 0; k < NA; ++k) A[k] = s[sgb ^ soff[k]];
    int i = 0;
    for (;;) {
      if (i >= nops) {
#pragma unroll
        for (int k = 0; k < NA; ++k) s[sgb ^ soff[k]] = A[k];
        break;
      }
      {
        const uint32_t code = st->code[i];
        if (op_active(st, i, code, gb, base)) apply_forward(code, A, B, st->mat[i]);
        else copy_regs(A, B);
      }
      if (++i >= nops) {
#pragma unroll
        for (int k = 0; k < NA; ++k) s[sgb ^ soff[k]] = B[k];
        break;
      }
      {
        const uint32_t code = st->code[i];
        if (op_active(st, i, code, gb, base)) apply_forward(code, B, A, st->mat[i]);
        else copy_regs(B, A);
      }
      ++i;
    }
  }
}

#endif  // TFQG_JIT

// One adjoint op of the sub-pass: (a, l) -> (ao, lo) plus warp-reduced
// gradient partials into rb->red.
__device__ __forceinline__ void backward_op(const Stage* st, RedBuf* rb, int i, uint32_t gb,
                                            uint32_t base, bool active, int it,
                                            int rbuf, int& gi,
                                            const float2 (&a)[1 << kBwdRB],
                                            const float2 (&l)[1 << kBwdRB],
                                            float2 (&ao)[1 << kBwdRB],
                                            float2 (&lo)[1 << kBwdRB]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t code = st->code[i];
  const bool on = active && op_active(st, i, code, gb, base);
  const int ng = (code >> 18) & 3;
  float part[2] = {0.f, 0.f};
  if (on) {
    apply_backward(code, a, l, ao, lo, st->mat[i], &st->dmat[i][0][0], part);
  } else {
    copy_regs(a, ao);
    copy_regs(l, lo);
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    if (q < ng) {
      float v = warp_sum(part[q]);
      if (lane == 0) {
        if (it == 0) rb->red[rbuf][gi + q][warp] = v;
        else rb->red[rbuf][gi + q][warp] += v;
      }
    }
  }
  gi += ng;
}

#ifndef TFQG_JIT
// Adjoint sub-pass on psi (s) and lambda (l) with 3 register bits.
__device__ __noinline__ void exec_backward(uint32_t s_off, uint32_t l_off, int T,
                                           uint32_t base, uint32_t st_off,
                                           uint32_t rb_off, int nops, uint32_t rbits,
                                           int rbuf) {
  constexpr int RB = kBwdRB, NA = 1 << RB;
  float2* s = reinterpret_cast<float2*>(smem_raw + s_off);
  float2* l = reinterpret_cast<float2*>(smem_raw + l_off);
  const Stage* st = reinterpret_cast<const Stage*>(smem_raw + st_off);
  RedBuf* rb = reinterpret_cast<RedBuf*>(smem_raw + rb_off);
  uint32_t soff[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    uint32_t o = 0;
#pragma unroll
    for (int j = 0; j < RB; ++j)
      if (k >> j & 1) o |= 1u << ((rbits >> (8 * j)) & 0xFF);
    soff[k] = swz(o);
  }
  const uint32_t ngroups = 1u << (T - RB);
  const uint32_t iters = (ngroups + blockDim.x - 1) / blockDim.x;
  for (uint32_t it = 0; it < iters; ++it) {
    const uint32_t g = it * blockDim.x + threadIdx.x;
    const bool active = g < ngroups;
    const uint32_t gb = group_base(active ? g : 0u, rbits, RB);
    const uint32_t sgb = swz(gb);
    float2 A[NA], LA[NA], B[NA], LB[NA];
    if (active) {
#pragma unroll
      for (int k = 0; k < NA; ++k) { A[k] = s[sgb ^ soff[k]]; LA[k] = l[sgb ^ soff[k]]; }
    } else {
#pragma unroll
      for (int k = 0; k < NA; ++k) { A[k] = make_float2(0.f, 0.f); LA[k] = A[k]; }
    }
    int gi = 0, i = 0;
    for (;;) {
      if (i >= nops) {
        if (active) {
#pragma unroll
          for (int k = 0; k < NA; ++k) { s[sgb ^ soff[k]] = A[k]; l[sgb ^ soff[k]] = LA[k]; }
        }
        break;
      }
      backward_op(st, rb, i, gb, base, active, int(it), rbuf, gi, A, LA, B, LB);
      if (++i >= nops) {
        if (active) {
#pragma unroll
          for (int k = 0; k < NA; ++k) { s[sgb ^ soff[k]] = B[k]; l[sgb ^ soff[k]] = LB[k]; }
        }
        break;
      }
      backward_op(st, rb, i, gb, base, active, int(it), rbuf, gi, B, LB, A, LA);
      ++i;
    }
  }
}

#endif  // TFQG_JIT

// Amplitude accessors of a channel: a swizzled shared-memory tile, or a
// whole state in global memory (read through L2, as tiles are).
struct SharedAmps {
  float2* s;
  __device__ float2 ld(uint32_t i) const { return s[swz(i)]; }
  __device__ void st(uint32_t i, float2 v) const { s[swz(i)] = v; }
};
struct GlobalAmps {
  float2* g;
  __device__ float2 ld(uint32_t i) const { return __ldcg(g + i); }
  __device__ void st(uint32_t i, float2 v) const { __stcg(g + i, v); }
};

// Any channel on bit t0 of a 2^T-amplitude state (qsim
// QuantumTrajectorySimulator semantics: mixed-unitary channels draw the
// branch from fixed probabilities, others from |K_k psi|^2, then renormalize).
template <class Amps>
__device__ void apply_channel(Amps A, int T, int t0, const DevChannel& ch,
                              const float2* kraus, double u, double* red) {
  const uint32_t np = 1u << (T - 1), bit = 1u << t0;
  int k = ch.nk - 1;
  float scale = 1.f;
  if (ch.mixed_unitary) {
    for (int j = 0; j < ch.nk; ++j)
      if (u < ch.cum[j]) { k = j; break; }
    if ((ch.ident_mask >> k) & 1) return;  // identity branch: nothing to do
    scale = ch.scale[k];
  } else {
    float part[4] = {0.f, 0.f, 0.f, 0.f};
    for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) {
      uint32_t i0 = ins0(i, t0);
      float2 a0 = A.ld(i0), a1 = A.ld(i0 | bit);
      for (int j = 0; j < ch.nk; ++j) {
        const float2* K = kraus + (ch.kraus + j) * 4;
        float2 z = make_float2(0.f, 0.f);
        float2 v0 = cfma(K[1], a1, cfma(K[0], a0, z));
        float2 v1 = cfma(K[3], a1, cfma(K[2], a0, z));
        part[j] += v0.x * v0.x + v0.y * v0.y + v1.x * v1.x + v1.y * v1.y;
      }
    }
    warp_partials(red, 0, part, 4);
    __syncthreads();
    double p[4], tot = 0.0;
    for (int j = 0; j < ch.nk; ++j) { p[j] = red_total(red, 0, j); tot += p[j]; }
    double c = 0.0, target = u * tot;
    for (int j = 0; j < ch.nk; ++j) {
      c += p[j];
      if (target < c && p[j] > 0.0) { k = j; break; }
    }
    if (p[k] <= 0.0) {
      for (int j = ch.nk - 1; j >= 0; --j) if (p[j] > 0.0) { k = j; break; }
    }
    scale = p[k] > 0.0 ? float(1.0 / sqrt(p[k])) : 0.f;
    __syncthreads();  // everyone has read red before it is reused
  }
  const float2* K = kraus + (ch.kraus + k) * 4;
  float2 g[4];
  for (int j = 0; j < 4; ++j) g[j] = make_float2(K[j].x * scale, K[j].y * scale);
  for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) {
    uint32_t i0 = ins0(i, t0);
    float2 a0 = A.ld(i0), a1 = A.ld(i0 | bit);
    float2 z = make_float2(0.f, 0.f);
    A.st(i0, cfma(g[1], a1, cfma(g[0], a0, z)));
    A.st(i0 | bit, cfma(g[3], a1, cfma(g[2], a0, z)));
  }
}

__device__ void op_channel(float2* s, int T, int t0, const DevChannel& ch,
                           const float2* kraus, double u, double* red) {
  apply_channel(SharedAmps{s}, T, t0, ch, kraus, u, red);
}

struct RowCtx {
  int row;
  int traj;           // trajectory (noisy), else 0
  DevRow r;
  DevProgram p;
};

// Copies the sub-pass's descriptors and matrices into shared memory (st),
// and for the adjoint its list of derivative slots (rb slot list `slots`).
template <int MODE>
__device__ void stage_subpass(const BatchDevice& b, const RunArgs& a,
                              const RowCtx& rc, Stage* st, RedBuf* rb,
                              uint32_t first, int nops, int slots) {
  const float2* mats = a.mats + int64_t(rc.r.mat_offset) * 16;
  const float2* dmats = a.dmats + int64_t(rc.r.dmat_offset) * 16;
  const int per_op = MODE == kModeAdjoint ? 24 : 8;  // 16-byte chunks
  for (int w = threadIdx.x; w < nops * per_op; w += blockDim.x) {
    const int i = w / per_op, c = w % per_op;
    const DevOp op = b.ops[first + i];
    if (op.type == OP_MCH) {
      // draw the branch once for the whole sub-pass; the identity branch
      // becomes a no-op, any other branch a 2x2 matrix on the register bit
      if (c == 0 && MODE == kModeNoisy) {
        DevOp o2 = op;
        const DevChannel ch = b.channels[rc.p.channel_begin + op.gate];
        double u = uniform01(a.seed, uint32_t(rc.row), uint32_t(rc.traj), op.gate);
        int k = ch.nk - 1;
        for (int j = 0; j < ch.nk; ++j)
          if (u < ch.cum[j]) { k = j; break; }
        o2.cls = ((ch.ident_mask >> k) & 1) ? uint8_t(GC_SKIP) : uint8_t(GC_GENERAL);
        const float2* K = b.kraus + (ch.kraus + k) * 4;
        for (int j = 0; j < 4; ++j)
          st->mat[i][j] = make_float2(K[j].x * ch.scale[k], K[j].y * ch.scale[k]);
        st->code[i] = op_code(o2);
        st->lcmask[i] = 0; st->lcval[i] = 0; st->gcmask[i] = 0; st->gcval[i] = 0;
      }
      continue;
    }
    if (c == 0) {
      st->code[i] = op_code(op);
      st->lcmask[i] = op.lcmask; st->lcval[i] = op.lcval;
      st->gcmask[i] = op.gcmask; st->gcval[i] = op.gcval;
      if (MODE == kModeAdjoint && (op.type == OP_B1 || op.type == OP_B2))
        for (int g = 0; g < op.ngrad; ++g) rb->red_slot[slots][op.gi + g] = op.grad_slot + g;
    }
    if (c < 8) {
      reinterpret_cast<float4*>(st->mat[i])[c] =
          __ldg(reinterpret_cast<const float4*>(mats + int64_t(op.gate) * 16) + c);
    } else if (MODE == kModeAdjoint && op.grad_slot >= 0) {
      const int g = (c - 8) / 8, cc = (c - 8) % 8;
      if (g < op.ngrad)
        reinterpret_cast<float4*>(st->dmat[i][g])[cc] = __ldg(
            reinterpret_cast<const float4*>(dmats + int64_t(op.grad_slot + g) * 16) + cc);
    }
  }
  // entries of the sub-pass: counted by the planner into the header
  if (MODE == kModeAdjoint && threadIdx.x == 0) rb->nred[slots] = b.ops[first - 1].t1;
}

// Executes the instruction stream [ob, oe) on a tile: s (psi) and l
// (lambda) hold 2^T amplitudes; `base` are the tile's fixed global bits.
// `kc` counts the CTA's sub-passes across calls: sub-pass k uses staging
// buffer k & 1, partial buffer k & 1 and slot list k % 3.  While sub-pass
// k runs, sub-pass k + 1 of the same stream is staged into the other
// buffer, so one barrier separates consecutive sub-passes.
template <int MODE, class Exec>
__device__ void run_ops(const BatchDevice& b, const RunArgs& a, const Smem& sm,
                        const RowCtx& rc, uint32_t ob, uint32_t oe, float2* s,
                        float2* l, int T, uint32_t base, int& kc) {
  uint32_t o = ob;
  bool staged = false;  // ops[o] (a sub-pass) already staged in buffer kc & 1
  const uint32_t so = uint32_t(reinterpret_cast<unsigned char*>(s) - smem_raw);
  const uint32_t rbo = uint32_t(reinterpret_cast<unsigned char*>(sm.rb) - smem_raw);
  while (o < oe) {
    const DevOp h = b.ops[o];
    if (h.type == OP_CHAN) {
      if (MODE == kModeNoisy) {
        const DevChannel ch = b.channels[rc.p.channel_begin + h.gate];
        double u = uniform01(a.seed, uint32_t(rc.row), uint32_t(rc.traj), h.gate);
        op_channel(s, T, h.t0, ch, b.kraus, u, sm.red);
      }
      __syncthreads();
      ++o;
      staged = false;
      continue;
    }
    // sub-pass
    const int nops = int(h.gate);
    Stage* st = sm.st + (kc & 1);
    if (!staged) {
      stage_subpass<MODE>(b, a, rc, st, sm.rb, o + 1, nops, kc % 3);
      __syncthreads();
    }
    const uint32_t next = o + 1 + uint32_t(nops);
    staged = false;
    if (next < oe) {
      const DevOp hn = b.ops[next];
      if (hn.type != OP_CHAN) {
        stage_subpass<MODE>(b, a, rc, sm.st + ((kc + 1) & 1), sm.rb, next + 1,
                            int(hn.gate), (kc + 1) % 3);
        staged = true;
      }
    }
    const uint32_t sto = uint32_t(reinterpret_cast<unsigned char*>(st) - smem_raw);
    if (MODE == kModeAdjoint && h.t0 == kBwdRB) {
      const uint32_t lo = uint32_t(reinterpret_cast<unsigned char*>(l) - smem_raw);
      Exec::backward(so, lo, T, base, sto, rbo, nops, h.lcmask, kc & 1, h.grad_slot);
    } else {
      Exec::forward(so, T, base, sto, nops, h.lcmask, h.grad_slot);
    }
    __syncthreads();
    if (MODE == kModeAdjoint && int(threadIdx.x) < sm.rb->nred[kc % 3]) {
      double acc = 0.0;
      for (int w = 0; w < int(blockDim.x >> 5); ++w)
        acc += sm.rb->red[kc & 1][threadIdx.x][w];
      sm.grad[sm.rb->red_slot[kc % 3][threadIdx.x]] += acc;
    }
    ++kc;
    o = next;
  }
}

// Global offset of tile-local index i (bits 0..4 are global bits 0..4).
__device__ __forceinline__ uint32_t tile_global(const uint32_t* hi, uint32_t i) {
  return (i & 31u) | hi[i >> 5];
}

__device__ void build_hi_table(uint32_t* hi, uint32_t tile_mask) {
  // local bits 5.. map to the set bits of tile_mask above bit 4, in order
  for (uint32_t j = threadIdx.x; j < (1u << kHiBits); j += blockDim.x) {
    uint32_t g = 0, rest = tile_mask & ~31u;
    for (int k = 0; k < kHiBits; ++k) {
      uint32_t lowest = rest & (~rest + 1u);
      if ((j >> k) & 1) g |= lowest;
      rest &= rest - 1u;
    }
    hi[j] = g;
  }
}

// pdep of `t` into the bits of `mask` (tile index -> fixed global bits)
__device__ __forceinline__ uint32_t deposit(uint32_t t, uint32_t mask) {
  uint32_t r = 0;
  for (int k = 0; mask; ++k) {
    uint32_t lowest = mask & (~mask + 1u);
    if ((t >> k) & 1) r |= lowest;
    mask &= mask - 1u;
  }
  return r;
}

// Tile loads are asynchronous copies (cp.async) from global to shared
// memory: every load of a tile is in flight at once and none holds a
// register.  A pair of amplitudes (2k, 2k+1) lands in one aligned 16-byte
// slot, possibly swapped (swz(2k+1) == swz(2k) ^ 1), so each amplitude is an
// 8-byte copy.  tile_load_async issues; tile_load_wait (then a barrier)
// completes every copy this thread issued.
__device__ __forceinline__ void cp_async8(float2* smem_dst, const float2* gsrc) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gsrc)
               : "memory");
}

__device__ __forceinline__ void tile_load_wait() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

__device__ void tile_load_async(float2* dst, const float2* src, const uint32_t* hi,
                                uint32_t base) {
  const uint32_t n2 = 1u << (kTile - 1);
  for (uint32_t k = threadIdx.x; k < n2; k += blockDim.x) {
    const float2* g = src + (tile_global(hi, 2 * k) | base);
    cp_async8(dst + swz(2 * k), g);
    cp_async8(dst + swz(2 * k + 1), g + 1);
  }
}

__device__ void tile_store(float2* dst, const float2* src, const uint32_t* hi,
                           uint32_t base) {
  const uint32_t n2 = 1u << (kTile - 1);
  for (uint32_t k = threadIdx.x; k < n2; k += blockDim.x) {
    uint32_t g = tile_global(hi, 2 * k) | base;
    float2 a = src[swz(2 * k)], c = src[swz(2 * k + 1)];
    __stcg(reinterpret_cast<float4*>(dst + g), make_float4(a.x, a.y, c.x, c.y));
  }
}

__device__ void tile_zero(float2* dst, bool first_tile) {
  // swz(0) == 0 and swz permutes the tile, so plain order is fine here
  const uint32_t n = 1u << kTile;
  for (uint32_t k = threadIdx.x; k < n; k += blockDim.x)
    dst[k] = make_float2(k == 0 && first_tile ? 1.f : 0.f, 0.f);
}

// Runs passes [pb, pe) over a state.  Resident: `s_state` (and `s_lam`) hold
// the whole state in shared memory.  Streamed: `g_psi` (and `g_lam`) are the
// global states; tiles go through sm.psi / sm.lam.  `init` zero-initialises
// the state to |0...0> during the first pass instead of loading it.
template <int MODE, class Exec>
__device__ void run_passes(const BatchDevice& b, const RunArgs& a,
                           const Smem& sm, const RowCtx& rc, uint32_t pb,
                           uint32_t pe, float2* g_psi, float2* g_lam,
                           bool init, int& kc, uint32_t t0 = 0,
                           uint32_t tstride = 1) {
  const int n = rc.p.n;
  if (rc.p.resident) {
    const int T = n < kRB ? kRB : n;  // tiny states are padded to 4 bits
    for (uint32_t p = pb; p < pe; ++p) {
      const DevPass ps = b.passes[p];
      run_ops<MODE, Exec>(b, a, sm, rc, ps.op_begin, ps.op_end, sm.psi, sm.lam, T, 0u,
                    kc);
    }
    return;
  }
  const uint32_t all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
  for (uint32_t p = pb; p < pe; ++p) {
    const DevPass ps = b.passes[p];
    if (ps.global_channel) {
      if (init && p == pb) {
        for (uint32_t i = threadIdx.x; i <= all; i += blockDim.x)
          __stcg(g_psi + i, make_float2(i == 0 ? 1.f : 0.f, 0.f));
        __syncthreads();
      }
      if (MODE == kModeNoisy) {
        const DevOp h = b.ops[ps.op_begin];
        const DevChannel ch = b.channels[rc.p.channel_begin + h.gate];
        const double u = uniform01(a.seed, uint32_t(rc.row), uint32_t(rc.traj), h.gate);
        apply_channel(GlobalAmps{g_psi}, n, h.t0, ch, b.kraus, u, sm.red);
      }
      __syncthreads();
      continue;
    }
    build_hi_table(sm.hi, ps.tile_mask);
    __syncthreads();
    const uint32_t outside = all & ~ps.tile_mask;
    const uint32_t ntiles = 1u << (n - kTile);
    for (uint32_t t = t0; t < ntiles; t += tstride) {
      const uint32_t base = deposit(t, outside);
      if (init && p == pb) tile_zero(sm.psi, base == 0);
      else tile_load_async(sm.psi, g_psi, sm.hi, base);
      if (MODE == kModeAdjoint && g_lam) tile_load_async(sm.lam, g_lam, sm.hi, base);
      tile_load_wait();
      __syncthreads();
      run_ops<MODE, Exec>(b, a, sm, rc, ps.op_begin, ps.op_end, sm.psi, sm.lam, kTile,
                    base, kc);
      tile_store(g_psi, sm.psi, sm.hi, base);
      if (MODE == kModeAdjoint && g_lam) tile_store(g_lam, sm.lam, sm.hi, base);
      __syncthreads();
    }
  }
}

// Stages the terms of measurement pass M into shared memory; `w` is the
// coefficient (expectation) or the AccumulateOperators weight g_j * c_t with
// the reference's 1e-5 skip (lambda; util_qsim.h:378-383).
__device__ void stage_terms(const BatchDevice& b, const RunArgs& a, const Smem& sm,
                            const RowCtx& rc, const DevMeas& M, bool lambda) {
  const int nt = int(M.end - M.begin);
  for (int i = threadIdx.x; i < nt; i += blockDim.x) {
    const DevMeasTerm mt = b.meas_terms[M.begin + i];
    const DevTerm t = b.terms[mt.term];
    float w = t.coef;
    if (lambda) {
      w = a.dgrads[int64_t(rc.row) * b.num_ops + t.op] * t.coef;
      if (fabsf(w) < 1e-5f) w = 0.f;
    }
    sm.mterm[i].w = w;
    sm.mterm[i].lflip = mt.lflip;
    sm.mterm[i].zy = t.zy;
    sm.mterm[i].op = t.op;
    sm.mterm[i].ny = uint8_t((t.ny & 3) | ((__popc(t.flip & t.zy) & 1) << 2));
    sm.mterm[i].identity = t.identity;
  }
}

// Adds <psi| P_t |psi> over one tile in shared memory (N amplitudes, fixed
// global bits `base`) to the term sums sm.macc, for the nt staged terms.
// Each thread takes amplitudes x = x0 + threadIdx.x + k * blockDim.x in
// blocks of kMeasAmps and keeps them, their swizzled positions and global
// indices in registers across the terms.  For P = i^ny X^flip Z^zy:
// <psi|P|psi> = i^ny sum_x conj(psi_x) (-1)^popc((x ^ flip) & zy) psi_{x^flip},
// and (-1)^popc((x ^ flip) & zy) = (-1)^(popc(x & zy) + popc(flip & zy)).
// Only the component that Re(i^ny * sum) needs is accumulated: the real
// part for even ny (into macc[2i]), the imaginary part for odd ny (into
// macc[2i + 1]).
constexpr int kMeasAmps = 16;
__device__ void measure_tile(const Smem& sm, int nt, uint32_t N, uint32_t base,
                             bool resident) {
  const uint32_t stride = blockDim.x;
  for (uint32_t x0 = 0; x0 < N; x0 += kMeasAmps * stride) {
    float2 av[kMeasAmps];
    uint32_t sx[kMeasAmps], gx[kMeasAmps];
#pragma unroll
    for (int k = 0; k < kMeasAmps; ++k) {
      const uint32_t x = x0 + threadIdx.x + k * stride;
      const bool ok = x < N;
      sx[k] = swz(ok ? x : 0u);
      gx[k] = resident ? x : ((x & 31u) | sm.hi[(ok ? x : 0u) >> 5] | base);
      av[k] = ok ? sm.psi[sx[k]] : make_float2(0.f, 0.f);
    }
    for (int i = 0; i < nt; ++i) {
      const auto t = sm.mterm[i];
      if (t.identity) continue;
      const uint32_t zy = t.zy, c0 = (t.ny >> 2) & 1;
      float acc = 0.f;
      if (t.lflip == 0) {
        if (!(t.ny & 1)) {  // diagonal term: sum |psi_x|^2 (-1)^popc(x & zy)
#pragma unroll
          for (int k = 0; k < kMeasAmps; ++k) {
            const float p = fmaf(av[k].x, av[k].x, av[k].y * av[k].y);
            acc += ((__popc(gx[k] & zy) ^ c0) & 1) ? -p : p;
          }
        }
      } else {
        const uint32_t sl = swz(t.lflip);
        const bool odd = t.ny & 1;
#pragma unroll
        for (int k = 0; k < kMeasAmps; ++k) {
          const float2 bv = sm.psi[sx[k] ^ sl];
          const float v = odd ? fmaf(av[k].x, bv.y, -av[k].y * bv.x)
                              : fmaf(av[k].x, bv.x, av[k].y * bv.y);
          acc += ((__popc(gx[k] & zy) ^ c0) & 1) ? -v : v;
        }
      }
      acc = warp_sum(acc);
      if ((threadIdx.x & 31) == 0 && acc != 0.f)
        atomicAdd(&sm.macc[2 * i + (t.ny & 1)], double(acc));
    }
  }
}

// Pauli-sum expectation by measurement passes (util_qsim.h:142-188): each
// tile of the state is read once into shared memory and every term of the
// pass whose flip bits lie in the tile is summed there.  Resident rows use
// the state in shared memory as the single tile.  `sink(op, value)` is called
// by thread 0 once per term.
template <class Sink>
__device__ void measure_passes(const BatchDevice& b, const RunArgs& a,
                               const Smem& sm, const RowCtx& rc,
                               const float2* g_psi, Sink&& sink) {
  const int n = rc.p.n;
  const bool resident = rc.p.resident;
  const uint32_t all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
  for (uint32_t mp = rc.r.meas_begin; mp < rc.r.meas_end; ++mp) {
    const DevMeas M = b.meas[mp];
    const int nt = int(M.end - M.begin);
    stage_terms(b, a, sm, rc, M, false);
    for (int i = threadIdx.x; i < 2 * nt; i += blockDim.x) sm.macc[i] = 0.0;
    uint32_t ntiles = 1;
    int Tl = n;
    if (!resident) {
      build_hi_table(sm.hi, M.tile_mask);
      ntiles = 1u << (n - kTile);
      Tl = kTile;
    }
    __syncthreads();
    const uint32_t outside = all & ~M.tile_mask;
    const uint32_t N = 1u << Tl;
    for (uint32_t tile = 0; tile < ntiles; ++tile) {
      uint32_t base = 0;
      if (!resident) {
        base = deposit(tile, outside);
        tile_load_async(sm.psi, g_psi, sm.hi, base);
        tile_load_wait();
        __syncthreads();
      }
      measure_tile(sm, nt, N, base, resident);
      __syncthreads();  // before the next tile overwrites sm.psi
    }
    if (threadIdx.x == 0) {
      for (int i = 0; i < nt; ++i) {
        double v;
        if (sm.mterm[i].identity) {
          v = 1.0;
        } else {
          const double sre = sm.macc[2 * i], sim = sm.macc[2 * i + 1];
          switch (sm.mterm[i].ny & 3) {  // Re(i^ny * sum)
            case 0: v = sre; break;
            case 1: v = -sim; break;
            case 2: v = -sre; break;
            default: v = sim; break;
          }
        }
        if (a.sample_terms && !sm.mterm[i].identity) {
          // one measurement of the term: parity +1 with probability (1 + v)/2
          const double u = uniform01(a.seed, uint32_t(rc.row), uint32_t(rc.traj),
                                     0xB0000000u + M.begin + uint32_t(i));
          v = u < 0.5 + 0.5 * v ? 1.0 : -1.0;
        }
        sink(int(sm.mterm[i].op), double(sm.mterm[i].w) * v);
        if (a.term_vals)
          a.term_vals[int64_t(rc.row) * a.term_stride +
                      (b.meas_terms[M.begin + i].term - rc.r.term_begin)] = v;
      }
    }
    __syncthreads();
  }
}

// lambda[x] += sum_t w_t i^ny_t (-1)^popc((x ^ flip_t) & zy_t) psi[x ^ flip_t]
// over one tile for the nt staged terms (weights w = g_j c_t, zero for
// skipped terms).  Each thread keeps a block of kMeasAmps lambda entries,
// their swizzled positions and global indices in registers across the
// terms; `fresh` starts lambda at zero instead of loading it.
template <int NY>
__device__ __forceinline__ void lambda_term(float2 (&v)[kMeasAmps], const uint32_t (&sx)[kMeasAmps],
                                            const uint32_t (&gx)[kMeasAmps], const float2* psi,
                                            uint32_t sl, uint32_t zy, uint32_t c0, float w) {
#pragma unroll
  for (int k = 0; k < kMeasAmps; ++k) {
    float2 p = psi[sx[k] ^ sl];
    if (NY == 1) p = make_float2(-p.y, p.x);       // multiply by i^ny
    if (NY == 2) p = make_float2(-p.x, -p.y);
    if (NY == 3) p = make_float2(p.y, -p.x);
    const float ws = ((__popc(gx[k] & zy) ^ c0) & 1) ? -w : w;
    v[k].x = fmaf(ws, p.x, v[k].x);
    v[k].y = fmaf(ws, p.y, v[k].y);
  }
}

__device__ void lambda_tile(const Smem& sm, int nt, uint32_t N, uint32_t base,
                            bool resident, bool fresh) {
  const uint32_t stride = blockDim.x;
  for (uint32_t x0 = 0; x0 < N; x0 += kMeasAmps * stride) {
    float2 v[kMeasAmps];
    uint32_t sx[kMeasAmps], gx[kMeasAmps];
#pragma unroll
    for (int k = 0; k < kMeasAmps; ++k) {
      const uint32_t x = x0 + threadIdx.x + k * stride;
      const bool ok = x < N;
      sx[k] = swz(ok ? x : 0u);
      gx[k] = resident ? x : ((x & 31u) | sm.hi[(ok ? x : 0u) >> 5] | base);
      v[k] = (ok && !fresh) ? sm.lam[sx[k]] : make_float2(0.f, 0.f);
    }
    for (int i = 0; i < nt; ++i) {
      const auto t = sm.mterm[i];
      const float w = t.w;
      if (w == 0.f) continue;
      const uint32_t sl = t.identity ? 0u : swz(t.lflip);
      const uint32_t zy = t.identity ? 0u : t.zy, c0 = t.identity ? 0u : (t.ny >> 2) & 1;
      switch (t.identity ? 0 : (t.ny & 3)) {
        case 1: lambda_term<1>(v, sx, gx, sm.psi, sl, zy, c0, w); break;
        case 2: lambda_term<2>(v, sx, gx, sm.psi, sl, zy, c0, w); break;
        case 3: lambda_term<3>(v, sx, gx, sm.psi, sl, zy, c0, w); break;
        default: lambda_term<0>(v, sx, gx, sm.psi, sl, zy, c0, w); break;
      }
    }
#pragma unroll
    for (int k = 0; k < kMeasAmps; ++k)
      if (x0 + threadIdx.x + k * stride < N) sm.lam[sx[k]] = v[k];
  }
}

// lambda = sum_j g_j sum_t c_t P_t psi by measurement passes
// (AccumulateOperators, util_qsim.h:362-414).  Streamed rows read psi tiles
// and accumulate lambda tiles in their global slot.
__device__ void lambda_passes(const BatchDevice& b, const RunArgs& a,
                              const Smem& sm, const RowCtx& rc,
                              float2* g_psi, float2* g_lam) {
  const int n = rc.p.n;
  const bool resident = rc.p.resident;
  const uint32_t all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
  if (resident) {
    // zero lambda (including the padding of tiny states) before accumulating
    const uint32_t Np = 1u << (n < kRB ? kRB : n);
    for (uint32_t x = threadIdx.x; x < Np; x += blockDim.x)
      sm.lam[x] = make_float2(0.f, 0.f);
    __syncthreads();
  }
  for (uint32_t mp = rc.r.meas_begin; mp < rc.r.meas_end; ++mp) {
    const DevMeas M = b.meas[mp];
    const int nt = int(M.end - M.begin);
    const bool first = mp == rc.r.meas_begin;
    stage_terms(b, a, sm, rc, M, true);
    uint32_t ntiles = 1;
    int Tl = n;
    if (!resident) {
      build_hi_table(sm.hi, M.tile_mask);
      ntiles = 1u << (n - kTile);
      Tl = kTile;
    }
    __syncthreads();
    const uint32_t outside = all & ~M.tile_mask;
    const uint32_t N = 1u << Tl;
    for (uint32_t tile = 0; tile < ntiles; ++tile) {
      uint32_t base = 0;
      if (!resident) {
        base = deposit(tile, outside);
        tile_load_async(sm.psi, g_psi, sm.hi, base);
        if (!first) tile_load_async(sm.lam, g_lam, sm.hi, base);
        tile_load_wait();
        __syncthreads();
      }
      lambda_tile(sm, nt, N, base, resident, first && !resident);
      __syncthreads();
      if (!resident) {
        tile_store(g_lam, sm.lam, sm.hi, base);
        __syncthreads();
      }
    }
  }
  if (rc.r.meas_begin == rc.r.meas_end && !resident) {
    // no observable terms: lambda is zero
    for (uint32_t x = threadIdx.x; x < (1u << n); x += blockDim.x)
      g_lam[x] = make_float2(0.f, 0.f);
    __syncthreads();
  }
}

// lambda seeded from a.lambda_init (times i^lambda_rot) for row rc.row: into
// shared memory (resident, padding zeroed) or the row's global slot.
__device__ void lambda_from_buffer(const RunArgs& a, const Smem& sm, const RowCtx& rc,
                                   float2* g_lam) {
  const int n = rc.p.n;
  const uint32_t N = 1u << n;
  const float2* src = a.lambda_init + int64_t(rc.row) * a.lambda_stride;
  const int rot = a.lambda_rot & 3;
  auto turn = [rot](float2 v) {
    switch (rot) {
      case 1: return make_float2(-v.y, v.x);
      case 2: return make_float2(-v.x, -v.y);
      case 3: return make_float2(v.y, -v.x);
      default: return v;
    }
  };
  if (rc.p.resident) {
    const uint32_t Np = 1u << (n < kRB ? kRB : n);
    for (uint32_t x = threadIdx.x; x < Np; x += blockDim.x)
      sm.lam[swz(x)] = x < N ? turn(src[x]) : make_float2(0.f, 0.f);
  } else {
    for (uint32_t x = threadIdx.x; x < N; x += blockDim.x) g_lam[x] = turn(src[x]);
  }
  __syncthreads();
}

// Sampler: chunked |psi|^2 prefix sums in double, then per-sample search
// (StateSpace::Sample semantics: index x with probability |psi_x|^2).
// S samples into out (rows of max_n columns); sample s draws its uniform
// from the counter (row, s0 + s).
__device__ void sample_state(const BatchDevice& b, const RunArgs& a,
                             const Smem& sm, const RowCtx& rc,
                             const float2* psi, bool shared, int8_t* out, int S,
                             int s0) {
  const int n = rc.p.n, maxn = b.max_n;
  const uint32_t N = 1u << n;
  const uint32_t nch = N < kMaxChunks ? N : kMaxChunks;
  const uint32_t L = N / nch;
  for (uint32_t c = threadIdx.x; c < nch; c += blockDim.x) {
    double acc = 0.0;
    float f = 0.f;
    for (uint32_t j = 0; j < L; ++j) {
      float2 v = psi[sidx(c * L + j, shared)];
      f = fmaf(v.x, v.x, fmaf(v.y, v.y, f));
      if ((j & 31) == 31) { acc += f; f = 0.f; }
    }
    sm.csum[c] = acc + f;
  }
  __syncthreads();
  // inclusive scan (Hillis-Steele, nch <= 1024, 2 elements per thread)
  for (uint32_t off = 1; off < nch; off <<= 1) {
    double v0 = 0.0, v1 = 0.0;
    uint32_t i0 = threadIdx.x, i1 = threadIdx.x + blockDim.x;
    if (i0 < nch && i0 >= off) v0 = sm.csum[i0 - off];
    if (i1 < nch && i1 >= off) v1 = sm.csum[i1 - off];
    __syncthreads();
    if (i0 < nch) sm.csum[i0] += v0;
    if (i1 < nch) sm.csum[i1] += v1;
    __syncthreads();
  }
  const double total = sm.csum[nch - 1];
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    double u = uniform01(a.seed, uint32_t(rc.row), uint32_t(s0 + s), 0x5A3Fu) * total;
    uint32_t lo = 0, hi = nch - 1;
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (sm.csum[mid] > u) hi = mid; else lo = mid + 1;
    }
    double acc = lo ? sm.csum[lo - 1] : 0.0;
    uint32_t x = lo * L, last_nz = x;
    bool found = false;
    for (uint32_t j = 0; j < L; ++j) {
      float2 v = psi[sidx(lo * L + j, shared)];
      double p = double(v.x) * v.x + double(v.y) * v.y;
      if (p > 0.0) last_nz = lo * L + j;
      acc += p;
      if (acc > u && p > 0.0) { x = lo * L + j; found = true; break; }
    }
    if (!found) x = last_nz;
    int8_t* o = out + int64_t(s) * maxn;
    for (int c = 0; c < maxn; ++c) {
      int k = maxn - 1 - c;  // sample bit k -> column maxn-k-1
      o[c] = k >= n ? int8_t(-2) : int8_t((x >> k) & 1);
    }
  }
}

__device__ void init_resident(float2* s, int n) {
  const uint32_t N = 1u << (n < kRB ? kRB : n);
  for (uint32_t x = threadIdx.x; x < N; x += blockDim.x)
    s[x] = make_float2(x == 0 ? 1.f : 0.f, 0.f);  // swz(0) == 0
}

template <int MODE, class Exec>
__device__ void run_row(const BatchDevice& b, const RunArgs& a, const Smem& sm,
                        int row, int traj) {
  RowCtx rc;
  rc.row = row;
  rc.traj = traj;
  rc.r = b.rows[row];
  rc.p = b.programs[rc.r.program];
  const int n = rc.p.n;
  const bool empty = n == 0 || rc.p.fwd_pass_begin == rc.p.fwd_pass_end;
  int kc = 0;  // sub-pass counter

  if (MODE == kModeExpect || MODE == kModeNoisy) {
    if (empty) {
      if (MODE == kModeExpect)
        for (int j = threadIdx.x; j < b.num_ops; j += blockDim.x)
          a.out_f[int64_t(row) * b.num_ops + j] = -2.f;
      // noisy samples of an empty program: every column is padding
      if (MODE == kModeNoisy && a.out_samples) {
        int8_t* o = a.out_samples + (int64_t(row) * a.num_samples + traj) * b.max_n;
        for (int c = threadIdx.x; c < b.max_n; c += blockDim.x) o[c] = int8_t(-2);
      }
      return;  // noisy empty rows are finalised on the host side kernel
    }
  }
  if (MODE == kModeState && empty) {
    float2* o = a.out_state + (int64_t(row) << b.max_n);
    for (uint32_t x = threadIdx.x; x < (1u << b.max_n); x += blockDim.x)
      o[x] = x == 0 ? make_float2(1.f, 0.f) : make_float2(-2.f, 0.f);
    return;
  }
  if (MODE == kModeSample && empty) {
    int8_t* o = a.out_samples + int64_t(row) * a.num_samples * b.max_n;
    for (int64_t x = threadIdx.x; x < int64_t(a.num_samples) * b.max_n; x += blockDim.x)
      o[x] = -2;
    return;
  }
  if (MODE == kModeAdjoint && empty) return;

  // global slots of this CTA (streamed rows)
  float2* g_psi = a.work + int64_t(blockIdx.x) * a.slot_amps;
  float2* g_lam = MODE == kModeAdjoint ? g_psi + (int64_t(1) << n) : nullptr;
  if (MODE == kModeState && !rc.p.resident)
    g_psi = a.out_state + (int64_t(row) << b.max_n);

  // ---- forward ----
  if (rc.p.resident) {
    init_resident(sm.psi, n);
    __syncthreads();
    run_passes<MODE, Exec>(b, a, sm, rc, rc.p.fwd_pass_begin, rc.p.fwd_pass_end,
                     nullptr, nullptr, true, kc);
  } else {
    run_passes<MODE, Exec>(b, a, sm, rc, rc.p.fwd_pass_begin, rc.p.fwd_pass_end,
                     g_psi, nullptr, true, kc);
  }
  __syncthreads();
  const float2* psi = rc.p.resident ? sm.psi : g_psi;
  const bool shared = rc.p.resident;

  if (MODE == kModeExpect) {
    float* out = a.out_f + int64_t(row) * b.num_ops;
    const bool small = b.num_ops <= kMaxOpsSmem;
    for (int j = threadIdx.x; j < b.num_ops; j += blockDim.x) {
      if (small) sm.oacc[j] = 0.0;
      else out[j] = 0.f;
    }
    __syncthreads();
    measure_passes(b, a, sm, rc, g_psi, [&](int op, double v) {
      if (small) sm.oacc[op] += v;
      else out[op] += float(v);
    });
    if (small)
      for (int j = threadIdx.x; j < b.num_ops; j += blockDim.x) out[j] = float(sm.oacc[j]);
  } else if (MODE == kModeNoisy && a.out_samples) {
    // noisy samples: one measurement of every qubit per trajectory
    // (tfq_noisy_samples.cc:166-187)
    sample_state(b, a, sm, rc, psi, shared,
                 a.out_samples + (int64_t(row) * a.num_samples + traj) * b.max_n, 1, traj);
  } else if (MODE == kModeNoisy) {
    const int64_t base = int64_t(row) * b.num_ops;
    measure_passes(b, a, sm, rc, g_psi, [&](int op, double v) {
      if (rc.traj < a.reps[base + op]) atomicAdd(a.acc + base + op, v);
    });
  } else if (MODE == kModeState) {
    float2* o = a.out_state + (int64_t(row) << b.max_n);
    const uint32_t N = 1u << n, M = 1u << b.max_n;
    if (rc.p.resident)
      for (uint32_t x = threadIdx.x; x < N; x += blockDim.x) o[x] = sm.psi[swz(x)];
    for (uint32_t x = N + threadIdx.x; x < M; x += blockDim.x)
      o[x] = make_float2(-2.f, 0.f);
  } else if (MODE == kModeSample) {
    sample_state(b, a, sm, rc, psi, shared,
                 a.out_samples + int64_t(row) * a.num_samples * b.max_n, a.num_samples, 0);
  } else if (MODE == kModeAdjoint) {
    for (int k = threadIdx.x; k < rc.p.num_grads; k += blockDim.x) sm.grad[k] = 0.0;
    if (a.lambda_init) lambda_from_buffer(a, sm, rc, g_lam);
    else lambda_passes(b, a, sm, rc, g_psi, g_lam);
    __syncthreads();
    run_passes<MODE, Exec>(b, a, sm, rc, rc.p.bwd_pass_begin, rc.p.bwd_pass_end,
                     rc.p.resident ? nullptr : g_psi,
                     rc.p.resident ? nullptr : g_lam, false, kc);
    __syncthreads();
    if (threadIdx.x == 0) {
      float* out = a.out_f + int64_t(row) * b.num_symbols;
      for (int k = 0; k < rc.p.num_grads; ++k) {
        int col = b.grad_cols[rc.p.grad_col_begin + k];
        out[col] += float(double(a.grad_scale) * sm.grad[k]);
      }
    }
  }
  __syncthreads();
}

// Dynamic shared memory layout of a simulation CTA.  The state section holds
// at least kRA amplitudes (128 bytes), and every other section size is a
// multiple of 16 bytes, so each section starts 16-byte aligned.
static_assert(((1u << kHiBits) * sizeof(uint32_t)) % 16 == 0, "hi table");
static_assert((2 * 4 * kWarps * sizeof(double)) % 16 == 0, "reduction scratch");
static_assert((kMaxChunks * sizeof(double)) % 16 == 0, "sampler chunks");
static_assert((2 * kMaxMeasTermsDev * sizeof(double)) % 16 == 0, "term sums");
static_assert((kMaxOpsSmem * sizeof(double)) % 16 == 0, "per-op sums");
template <int MODE>
__device__ __forceinline__ Smem carve_smem(int state_amps, int nstates) {
  Smem sm;
  sm.psi = reinterpret_cast<float2*>(smem_raw);
  sm.lam = sm.psi + state_amps;
  unsigned char* p = smem_raw + size_t(state_amps) * nstates * sizeof(float2);
  sm.st = reinterpret_cast<Stage*>(p);
  p += 2 * sizeof(Stage);
  sm.rb = reinterpret_cast<RedBuf*>(p);
  p += sizeof(RedBuf);
  sm.hi = reinterpret_cast<uint32_t*>(p);
  p += (1u << kHiBits) * sizeof(uint32_t);
  sm.red = reinterpret_cast<double*>(p);
  p += 2 * 4 * kWarps * sizeof(double);
  sm.csum = reinterpret_cast<double*>(p);
  if (MODE == kModeSample || MODE == kModeNoisy) p += kMaxChunks * sizeof(double);
  sm.macc = reinterpret_cast<double*>(p);
  p += 2 * kMaxMeasTermsDev * sizeof(double);
  sm.mterm = reinterpret_cast<decltype(sm.mterm)>(p);
  p += kMaxMeasTermsDev * 16;
  sm.oacc = reinterpret_cast<double*>(p);
  if (MODE == kModeExpect) p += kMaxOpsSmem * sizeof(double);
  sm.grad = reinterpret_cast<double*>(p);
  return sm;
}

// Body of the persistent simulation kernel: lays out dynamic shared memory
// and pulls rows (or trajectories) from the work queue.  `Exec` executes
// sub-passes (the interpreter, or code specialized for one batch).
template <int MODE, class Exec>
__device__ __forceinline__ void simulate_body(BatchDevice b, RunArgs a,
                                              int state_amps, int nstates) {
  const Smem sm = carve_smem<MODE>(state_amps, nstates);

  __shared__ int s_item;
  const int64_t total = MODE == kModeNoisy ? a.total_traj : b.num_queue;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int64_t item = s_item;
    __syncthreads();
    if (item >= total) break;
    if (MODE == kModeNoisy) {
      int lo = 0, hi = b.num_rows - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (a.traj_prefix[mid] <= item) lo = mid; else hi = mid - 1;
      }
      run_row<MODE, Exec>(b, a, sm, lo, int(item - a.traj_prefix[lo]));
    } else {
      run_row<MODE, Exec>(b, a, sm, b.order[item], 0);
    }
  }
}


// ---------------------------------------------------------------------------
// wide rows: one large state, every CTA of the grid works on it
// ---------------------------------------------------------------------------
// A wide row's state lives in global memory and each forward pass is one
// launch: CTA c takes tiles c, c + gridDim.x, ... of the pass (tiles of one
// pass are independent; the launch boundary orders the passes).

// Forward pass `pass` of wide row `row` over the state `psi` (2^n amplitudes).
template <class Exec>
__device__ __forceinline__ void wide_pass_body(const BatchDevice& b, const RunArgs& a,
                                               int row, int pass, int init, float2* psi,
                                               int state_amps) {
  const Smem sm = carve_smem<kModeState>(state_amps, 1);
  RowCtx rc;
  rc.row = row;
  rc.traj = 0;
  rc.r = b.rows[row];
  rc.p = b.programs[rc.r.program];
  int kc = 0;  // sub-pass counter
  run_passes<kModeState, Exec>(b, a, sm, rc, uint32_t(pass), uint32_t(pass) + 1, psi,
                               nullptr, init != 0, kc, blockIdx.x, gridDim.x);
}

// Measurement pass `mp` of wide row `row`: this CTA's tiles add their term
// sums (re, im) to wacc[2 * (term - term0) + {0, 1}] (double atomics).
__device__ __forceinline__ void wide_measure_body(const BatchDevice& b, const RunArgs& a,
                                                  int row, int mp, const float2* psi,
                                                  double* wacc, int term0, int state_amps) {
  const Smem sm = carve_smem<kModeState>(state_amps, 1);
  RowCtx rc;
  rc.row = row;
  rc.traj = 0;
  rc.r = b.rows[row];
  rc.p = b.programs[rc.r.program];
  const int n = rc.p.n;
  const DevMeas M = b.meas[mp];
  const int nt = int(M.end - M.begin);
  stage_terms(b, a, sm, rc, M, false);
  for (int i = threadIdx.x; i < 2 * nt; i += blockDim.x) sm.macc[i] = 0.0;
  build_hi_table(sm.hi, M.tile_mask);
  __syncthreads();
  const uint32_t all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
  const uint32_t outside = all & ~M.tile_mask;
  const uint32_t ntiles = 1u << (n - kTile);
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint32_t base = deposit(t, outside);
    tile_load_async(sm.psi, psi, sm.hi, base);
    tile_load_wait();
    __syncthreads();
    measure_tile(sm, nt, 1u << kTile, base, false);
    __syncthreads();
  }
  double* dst = wacc + 2 * (int64_t(M.begin) - term0);
  for (int i = threadIdx.x; i < 2 * nt; i += blockDim.x)
    if (sm.macc[i] != 0.0) atomicAdd(dst + i, sm.macc[i]);
}

// Wide rows in the adjoint: psi and lambda (2^n amplitudes each) live in
// global memory and each pass is one launch over the whole grid, as in the
// forward wide path.

// lambda += sum_t w_t P_t psi over the terms of measurement pass `mp` of
// wide row `row` (lambda starts from zero when `first`); this CTA's tiles.
__device__ __forceinline__ void wide_lambda_body(const BatchDevice& b, const RunArgs& a,
                                                 int row, int mp, int first,
                                                 const float2* psi, float2* lam,
                                                 int state_amps) {
  const Smem sm = carve_smem<kModeAdjoint>(state_amps, 2);
  RowCtx rc;
  rc.row = row;
  rc.traj = 0;
  rc.r = b.rows[row];
  rc.p = b.programs[rc.r.program];
  const int n = rc.p.n;
  const DevMeas M = b.meas[mp];
  const int nt = int(M.end - M.begin);
  stage_terms(b, a, sm, rc, M, true);
  build_hi_table(sm.hi, M.tile_mask);
  __syncthreads();
  const uint32_t all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
  const uint32_t outside = all & ~M.tile_mask;
  const uint32_t ntiles = 1u << (n - kTile);
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint32_t base = deposit(t, outside);
    tile_load_async(sm.psi, psi, sm.hi, base);
    if (!first) tile_load_async(sm.lam, lam, sm.hi, base);
    tile_load_wait();
    __syncthreads();
    lambda_tile(sm, nt, 1u << kTile, base, false, first != 0);
    __syncthreads();
    tile_store(lam, sm.lam, sm.hi, base);
    __syncthreads();
  }
}

// Backward pass `pass` of wide row `row` over psi and lambda: this CTA's
// tiles.  Its gradient-slot sums (shared memory) are added to gacc[slot]
// with double atomics once, at the end.
template <class Exec>
__device__ __forceinline__ void wide_backward_body(const BatchDevice& b, const RunArgs& a,
                                                   int row, int pass, float2* psi,
                                                   float2* lam, double* gacc,
                                                   int state_amps) {
  const Smem sm = carve_smem<kModeAdjoint>(state_amps, 2);
  RowCtx rc;
  rc.row = row;
  rc.traj = 0;
  rc.r = b.rows[row];
  rc.p = b.programs[rc.r.program];
  for (int k = threadIdx.x; k < rc.p.num_grads; k += blockDim.x) sm.grad[k] = 0.0;
  __syncthreads();
  int kc = 0;
  run_passes<kModeAdjoint, Exec>(b, a, sm, rc, uint32_t(pass), uint32_t(pass) + 1, psi,
                                 lam, false, kc, blockIdx.x, gridDim.x);
  __syncthreads();
  for (int k = threadIdx.x; k < rc.p.num_grads; k += blockDim.x) {
    const double v = sm.grad[k];
    if (v != 0.0) atomicAdd(gacc + k, v);
  }
}

#ifndef TFQG_JIT
// Sub-passes run by the precompiled interpreter.
struct InterpExec {
  static __device__ __forceinline__ void forward(uint32_t so, int T, uint32_t base,
                                                 uint32_t sto, int nops,
                                                 uint32_t rbits, int sig) {
    exec_forward(so, T, base, sto, nops, rbits);
  }
  static __device__ __forceinline__ void backward(uint32_t so, uint32_t lo, int T,
                                                  uint32_t base, uint32_t sto,
                                                  uint32_t rbo, int nops,
                                                  uint32_t rbits, int rbuf, int sig) {
    exec_backward(so, lo, T, base, sto, rbo, nops, rbits, rbuf);
  }
};
#endif  // TFQG_JIT

}  // namespace
}  // namespace tfqg
