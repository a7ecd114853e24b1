// tcgen05 (5th-generation tensor core) building blocks for sm_103a, written
// as inline PTX: TMEM allocation, shared-memory operand descriptors, the
// kind::tf32 MMA with its completion on an mbarrier, and TMEM read-back.
//
// tc_gemm_tf32_kernel computes D[128 x 64] = A[128 x 32] * B[64 x 32]^T in
// one CTA: the operand tiles are staged in shared memory in the canonical
// K-major no-swizzle layout (core matrices of 8 rows x 16 bytes), one thread
// issues four K=8 MMAs into a TMEM accumulator, and the four warps read the
// accumulator back (warp w owns TMEM lanes 32w..32w+31).  It is the
// self-check of the descriptor and instruction encodings that the fused-gate
// tensor-core path builds on (a fused k-qubit gate is a real GEMM whose A
// operand is the state tile and whose B operand is the gate in real form).
//
// Every wait is bounded: on a timeout the kernel records an error code,
// waits (bounded) once more, frees its TMEM and returns.
#include <cuda_runtime.h>
#include <stdint.h>

namespace tfqg {
namespace {

constexpr int kTcM = 128, kTcN = 64, kTcK = 32;
constexpr uint32_t kTcCols = 64;         // TMEM columns (fp32 accumulators)
constexpr uint32_t kSpinLimit = 1u << 22;

// byte offset of element (row, k) of a K-major tile with `kdim` columns in
// the canonical no-swizzle layout: 8-row groups of 16-byte core matrices
__device__ __forceinline__ uint32_t kmajor_offset(int row, int k, int kdim) {
  const uint32_t sbo = uint32_t(kdim / 4) * 128u;  // between 8-row groups
  return uint32_t(row / 8) * sbo + uint32_t(k / 4) * 128u + uint32_t(row % 8) * 16u +
         uint32_t(k % 4) * 4u;
}

// Shared-memory matrix descriptor (sm_100 family): start address, leading
// byte offset (between core matrices along K), stride byte offset (between
// 8-row groups), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFFu);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;  // version
  return d;                // base offset 0, lbo mode 0, layout: no swizzle
}

// Instruction descriptor of kind::tf32: fp32 accumulator, tf32 A and B,
// both K-major, N >> 3 and M >> 4.
__device__ __forceinline__ uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(n >> 3) << 17) |
         (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__global__ void __launch_bounds__(128, 1)
tc_gemm_tf32_kernel(const float* A, const float* B, float* D, int* status) {
  __shared__ __align__(128) float sa[kTcM * kTcK];
  __shared__ __align__(128) float sb[kTcN * kTcK];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int timed_out;
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int i = tid; i < kTcM * kTcK; i += blockDim.x) {
    const int r = i / kTcK, k = i % kTcK;
    sa[kmajor_offset(r, k, kTcK) / 4] = A[i];
  }
  for (int i = tid; i < kTcN * kTcK; i += blockDim.x) {
    const int r = i / kTcK, k = i % kTcK;
    sb[kmajor_offset(r, k, kTcK) / 4] = B[i];
  }
  // operands written by the generic proxy are read by the tensor core
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  if (tid == 0) {
    timed_out = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (tid == 0) {
    const uint32_t idesc = idesc_tf32(kTcM, kTcN);
    const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
    const uint32_t sbo = uint32_t(kTcK / 4) * 128u;
    for (int s = 0; s < kTcK / 8; ++s) {  // K = 8 per MMA: two core matrices
      const uint64_t ad = smem_desc(a0 + uint32_t(s) * 256u, 128u, sbo);
      const uint64_t bd = smem_desc(b0 + uint32_t(s) * 256u, 128u, sbo);
      const uint32_t acc = s > 0 ? 1u : 0u;
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
          " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
          "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
          : "memory");
    }
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_u32(&bar))
        : "memory");
  }
  // every thread waits for the MMAs (bounded)
  bool done = false;
  for (uint32_t it = 0; it < kSpinLimit && !done; ++it) done = mbar_try_wait(smem_u32(&bar), 0);
  if (!done) {
    atomicExch(&timed_out, 1);
    for (uint32_t it = 0; it < kSpinLimit && !done; ++it)
      done = mbar_try_wait(smem_u32(&bar), 0);
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (!timed_out) {
    // warp w reads TMEM lanes 32w..32w+31 (rows of D), 16 columns at a time
    const int row = warp * 32 + (tid & 31);
    for (int c0 = 0; c0 < kTcN; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, "
          "%9, %10, %11, %12, %13, %14, %15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
            "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
            "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      for (int j = 0; j < 16; ++j) D[row * kTcN + c0 + j] = __uint_as_float(v[j]);
    }
  } else if (tid == 0) {
    *status = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(kTcCols)
                 : "memory");
}

// The same product with the A operand in tensor memory (the "TS" form of
// tcgen05.mma): each thread stores its row of A into its TMEM lane with
// tcgen05.st (columns kTcN.. kTcN + kTcK, one fp32/tf32 element per
// column), and the MMAs read A from there and B from shared memory.  This
// is the form that keeps state tiles out of shared memory on their way to
// the tensor core.
__global__ void __launch_bounds__(128, 1)
tc_gemm_tf32_ts_kernel(const float* A, const float* B, float* D, int* status) {
  __shared__ __align__(128) float sb[kTcN * kTcK];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int timed_out;
  constexpr uint32_t kCols = 128;  // D: columns 0..63, A: columns 64..95
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < kTcN * kTcK; i += blockDim.x) {
    const int r = i / kTcK, k = i % kTcK;
    sb[kmajor_offset(r, k, kTcK) / 4] = B[i];
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  if (tid == 0) {
    timed_out = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  {
    // row tid of A -> TMEM lane tid, columns kTcN .. kTcN + 31
    uint32_t v[32];
    for (int k = 0; k < kTcK; ++k) v[k] = __float_as_uint(A[tid * kTcK + k]);
    const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(kTcN);
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, "
        "%10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, "
        "%26, %27, %28, %29, %30, %31, %32};\n" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]),
        "r"(v[7]), "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]),
        "r"(v[14]), "r"(v[15]), "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]),
        "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]),
        "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (tid == 0) {
    const uint32_t idesc = idesc_tf32(kTcM, kTcN);
    const uint32_t b0 = smem_u32(sb);
    const uint32_t sbo = uint32_t(kTcK / 4) * 128u;
    for (int s = 0; s < kTcK / 8; ++s) {
      const uint64_t bd = smem_desc(b0 + uint32_t(s) * 256u, 128u, sbo);
      const uint32_t ta = tmem + uint32_t(kTcN + 8 * s);
      const uint32_t acc = s > 0 ? 1u : 0u;
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
          " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem),
          "r"(ta), "l"(bd), "r"(idesc), "r"(acc)
          : "memory");
    }
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_u32(&bar))
        : "memory");
  }
  bool done = false;
  for (uint32_t it = 0; it < kSpinLimit && !done; ++it) done = mbar_try_wait(smem_u32(&bar), 0);
  if (!done) {
    atomicExch(&timed_out, 1);
    for (uint32_t it = 0; it < kSpinLimit && !done; ++it)
      done = mbar_try_wait(smem_u32(&bar), 0);
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (!timed_out) {
    const int row = warp * 32 + (tid & 31);
    for (int c0 = 0; c0 < kTcN; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, "
          "%9, %10, %11, %12, %13, %14, %15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
            "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
            "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      for (int j = 0; j < 16; ++j) D[row * kTcN + c0 + j] = __uint_as_float(v[j]);
    }
  } else if (tid == 0) {
    *status = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(kCols)
                 : "memory");
}

}  // namespace
}  // namespace tfqg

extern "C" {

// As tfqg_internal_tc_gemm_tf32, with the A operand read from tensor memory.
int tfqg_internal_tc_gemm_tf32_ts(const float* A, const float* B, float* D, int* status,
                                  void* stream) {
  tfqg::tc_gemm_tf32_ts_kernel<<<1, 128, 0, static_cast<cudaStream_t>(stream)>>>(A, B, D,
                                                                                 status);
  return int(cudaGetLastError());
}

// D[128 x 64] = A[128 x 32] * B[64 x 32]^T on the tensor cores (kind::tf32),
// all pointers on the current device; *status (device int) is set to 1 when
// the MMA completion wait timed out.  Returns a cudaError_t.
int tfqg_internal_tc_gemm_tf32(const float* A, const float* B, float* D, int* status,
                               void* stream) {
  tfqg::tc_gemm_tf32_kernel<<<1, 128, 0, static_cast<cudaStream_t>(stream)>>>(A, B, D,
                                                                              status);
  return int(cudaGetLastError());
}

}  // extern "C"
