// Tensor-core forward path for wide rows: gates fused into 5-qubit blocks
// (plan_tc_blocks on the host), each block applied to the whole state in one
// launch as a real GEMM on the 5th-generation tensor cores.
//
// A block's 32 x 32 complex matrix U acts on the 32 amplitudes of every
// group (the index bits outside the block's 5 target bits fixed).  In real
// form, with amplitudes interleaved (re, im), U is a 64 x 64 real matrix R
// (R[2i][2j] = Re U_ij, R[2i][2j+1] = -Im U_ij, R[2i+1][2j] = Im U_ij,
// R[2i+1][2j+1] = Re U_ij), and a chunk of 128 groups is the GEMM
//   D[128 x 64] = A[128 x 64] * R^T,   A[g][2j + c] = component c of amplitude j of group g.
// The MMA is tcgen05.mma kind::tf32 with fp32 accumulation in TMEM.  Split
// 3xTF32 keeps fp32 accuracy: A = A_hi + A_lo and R = R_hi + R_lo with
// *_hi rounded to tf32, and D = A_lo R_hi + A_hi R_lo + A_hi R_hi (the
// A_lo R_lo term is below fp32 rounding).
//
// tc_fuse_kernel builds U for every block in complex128 (one thread per
// column) from the member gates' bound complex64 matrices; tc_apply5_kernel
// streams the state: each of 128 threads gathers its group's 32 amplitudes,
// splits them into the two A operands in shared memory (canonical K-major
// no-swizzle layout, core matrices of 8 rows x 16 bytes), one thread issues
// 24 MMAs (3 products x 8 K-steps of 8) and commits them to an mbarrier, and
// each warp reads its 32 TMEM lanes (its 32 groups) back and stores them in
// place.  The next chunk's gathers are in flight while the MMAs run.
//
// Every wait is bounded: on a timeout the kernel records status 1, waits
// (bounded) once more for its MMAs, frees its TMEM and returns.
//
// Blocks with a target among index bits 0-4 take the transposed variant.
// There a group's amplitudes lie within a few hundred bytes of each other
// and neighbouring groups are 2^(lowest row bit) apart, so per-thread
// gathers would touch every 32-byte sector several times.  Instead the CTA
// moves each chunk of 4096 amplitudes as whole 16-byte vectors in index
// order (every warp access a contiguous 512 bytes) through a staging buffer
// in shared memory, and each thread reads or writes its group's amplitudes
// there.  The chunk's 12 index bits always include bits 0-6 (they are either
// targets or among the 7 lowest non-target bits), so a chunk is made of
// 1 KiB runs.  The staging buffer is XOR-swizzled on its 8-byte slots: slot
// bits 0-3 of chunk position L are XORed with a linear function h of L's
// bits 4-11, chosen on the host so that the 32 groups of a warp fall on 16
// distinct bank pairs (2 per pair, the minimum for 8-byte accesses) while
// 16-byte accesses by consecutive lanes stay on distinct banks.
//
// Lockstep rows (many streamed states of 15-21 qubits) use the same chunk
// loop (tc_apply5_chunks) on units, runs of up to 16 chunks of one row's
// state under one block: tc_fuse_b_kernel writes every block's B operands
// to global memory once per call, and a unit brings them into shared memory
// with one bulk copy.  tc_lock_persistent_kernel runs all of a group's
// units in one launch (a unit waits for its row's earlier blocks);
// tc_apply5_units_kernel runs the units of one block index and variant.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gate_math.cuh"
#include "kernels.h"

namespace tfqg {
namespace {

constexpr int kTcRows = 128;            // groups per chunk (MMA M)
constexpr int kTcKdim = 64;             // real K: 32 complex amplitudes
constexpr int kTcNdim = 64;             // real N
constexpr uint32_t kTcTmemCols = 64;    // fp32 accumulator columns
constexpr uint32_t kTcSpin = 1u << 22;  // bounded mbarrier polls
constexpr uint32_t kTcSbo = (kTcKdim / 4) * 128u;  // bytes between 8-row groups
constexpr size_t kTcAbytes = size_t(kTcRows) * kTcKdim * 4;  // 32 KiB
constexpr size_t kTcBbytes = size_t(kTcNdim) * kTcKdim * 4;  // 16 KiB
constexpr size_t kTcSmem = 2 * kTcAbytes + 2 * kTcBbytes + 64;
constexpr int kTcBfloats = int(2 * kTcBbytes / 4);  // B hi and lo of one block

// byte offset of element (row, k) in the K-major no-swizzle layout with 64
// columns: 8-row groups kTcSbo apart, 16-byte core-matrix rows, 128-byte core
// matrices along K
__device__ __forceinline__ uint32_t kmaj(int row, int k) {
  return uint32_t(row >> 3) * kTcSbo + uint32_t(k >> 2) * 128u + uint32_t(row & 7) * 16u +
         uint32_t(k & 3) * 4u;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: start, leading byte offset (along K),
// stride byte offset (between 8-row groups), version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// kind::tf32 instruction descriptor: fp32 D, tf32 A and B, K-major, N>>3, M>>4
__device__ __forceinline__ uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(n >> 3) << 17) |
         (uint32_t(m >> 4) << 24);
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

// x rounded to the nearest tf32 value (10 mantissa bits), as an fp32
__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, "
      "%9, %10, %11, %12, %13, %14, %15}, [%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}

// index of group g: g's bits deposited into the bits that are not targets
// (targets ascending)
__device__ __forceinline__ int64_t group_base(int64_t g, const int* t) {
#pragma unroll
  for (int i = 0; i < kTcBits; ++i) {
    const int64_t low = (int64_t(1) << t[i]) - 1;
    g = ((g & ~low) << 1) | (g & low);
  }
  return g;
}

__global__ void tc_fuse_kernel(BatchDevice b, const float2* mats, int row,
                               const TcBlock* blocks, const int32_t* members, int nblocks,
                               float2* U) {
  const int blk = blockIdx.x, j = threadIdx.x;
  if (blk >= nblocks || j >= 32) return;
  const DevRow r = b.rows[row];
  const DevProgram p = b.programs[r.program];
  const GateTemplate* gates = b.gates + p.gate_begin;
  const float2* m0 = mats + int64_t(r.mat_offset) * 16;
  Cx<double> col[32];
  tc_block_column(gates, members, blocks[blk], j,
                  [&](int k, Cx<double>* m) {
                    const float2* src = m0 + int64_t(k) * 16;
                    for (int i = 0; i < 16; ++i) m[i] = Cx<double>(src[i].x, src[i].y);
                  },
                  col);
  float2* dst = U + int64_t(blk) * 1024;
  for (int i = 0; i < 32; ++i) dst[i * 32 + j] = make_float2(float(col[i].re), float(col[i].im));
}

// Lockstep rows: each block's matrix in complex64 (one thread per column;
// block blk belongs to batch row block_rows[blk]), written straight into
// the block kernel's B operands: R in real form split into tf32 hi and lo,
// K-major, kTcBbytes each, hi then lo (kTcBfloats floats per block).
__global__ void tc_fuse_b_kernel(BatchDevice b, const float2* mats, const int32_t* block_rows,
                                 const TcBlock* blocks, const int32_t* members, int nblocks,
                                 float* B) {
  const int blk = blockIdx.x, j = threadIdx.x;
  if (blk >= nblocks || j >= 32) return;
  const DevRow r = b.rows[block_rows[blk]];
  const DevProgram p = b.programs[r.program];
  const GateTemplate* gates = b.gates + p.gate_begin;
  const float2* m0 = mats + int64_t(r.mat_offset) * 16;
  Cx<float> col[32];
  tc_block_column(gates, members, blocks[blk], j,
                  [&](int k, Cx<float>* m) {
                    const float2* src = m0 + int64_t(k) * 16;
                    for (int i = 0; i < 16; ++i) m[i] = Cx<float>(src[i].x, src[i].y);
                  },
                  col);
  // thread j holds U[:, j]: the B entries of K columns 2j (re) and 2j + 1 (im)
  float* bh = B + int64_t(blk) * kTcBfloats;
  float* bl = bh + kTcBfloats / 2;
  for (int nr = 0; nr < kTcNdim; ++nr) {
    const Cx<float> u = col[nr >> 1];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const float v = (nr & 1) ? (c ? u.re : u.im) : (c ? -u.im : u.re);
      const float hi = tf32_hi(v);
      const uint32_t o = kmaj(nr, 2 * j + c) >> 2;
      bh[o] = hi;
      bl[o] = v - hi;
    }
  }
}

// physical offset of the chunk positions set in L
__device__ __forceinline__ int64_t tr_dep(uint32_t L, uint64_t cb) {
  int64_t o = 0;
#pragma unroll
  for (int p = 0; p < 12; ++p)
    if ((L >> p) & 1u) o |= int64_t(1) << int((cb >> (5 * p)) & 31u);
  return o;
}

// swizzle term of the positions >= 4 set in L
__device__ __forceinline__ uint32_t tr_h(uint32_t L, uint32_t c) {
  uint32_t h = 0;
#pragma unroll
  for (int p = 4; p < 12; ++p)
    if ((L >> p) & 1u) h ^= (c >> (4 * (p - 4))) & 15u;
  return h;
}

__device__ __forceinline__ uint32_t tr_deposit(uint32_t v, uint32_t pos, int bits) {
  uint32_t L = 0;
#pragma unroll
  for (int i = 0; i < 7; ++i)
    if (i < bits && ((v >> i) & 1u)) L |= 1u << ((pos >> (4 * i)) & 15u);
  return L;
}

// Shared memory of the block kernels: the A operands (hi, lo), the B
// operands (hi, lo), the MMA mbarrier, the TMEM base address and the
// timeout flag, at fixed offsets from the dynamic shared-memory base.
struct TcSmem {
  unsigned char* s;
  __device__ __forceinline__ float* a_hi() const { return reinterpret_cast<float*>(s); }
  __device__ __forceinline__ float* a_lo() const {
    return reinterpret_cast<float*>(s + kTcAbytes);
  }
  __device__ __forceinline__ float* b_hi() const {
    return reinterpret_cast<float*>(s + 2 * kTcAbytes);
  }
  __device__ __forceinline__ float* b_lo() const {
    return reinterpret_cast<float*>(s + 2 * kTcAbytes + kTcBbytes);
  }
  __device__ __forceinline__ uint64_t* bar() const {
    return reinterpret_cast<uint64_t*>(s + 2 * kTcAbytes + 2 * kTcBbytes);
  }
  __device__ __forceinline__ uint32_t* tmem_slot() const {
    return reinterpret_cast<uint32_t*>(bar() + 1);
  }
  __device__ __forceinline__ int* timed_out() const { return reinterpret_cast<int*>(bar() + 2); }
  // completion of the bulk copy of the B operands (units kernels)
  __device__ __forceinline__ uint64_t* bbar() const { return bar() + 3; }
  // the unit a CTA of the persistent kernel takes next
  __device__ __forceinline__ int* next_unit() const { return reinterpret_cast<int*>(bar() + 4); }
};

// mbarrier and timeout flag initialised, TMEM allocated; returns its base.
__device__ __forceinline__ uint32_t tc_begin(const TcSmem& m) {
  if (threadIdx.x == 0) {
    *m.timed_out() = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(m.bar())) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(m.bbar())) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(m.tmem_slot())),
                 "r"(kTcTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  return *m.tmem_slot();
}

// After a timed-out wait the MMAs may still be running: wait for them
// (bounded) and record status 1; then free the TMEM.
__device__ __forceinline__ void tc_end(const TcSmem& m, uint32_t tmem, bool failed,
                                       uint32_t parity, int* status) {
  if (failed) {
    bool done = false;
    for (uint32_t it = 0; it < kTcSpin && !done; ++it)
      done = mbar_try_wait(smem_u32(m.bar()), parity ^ 1u);
    if (threadIdx.x == 0) atomicExch(status, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(kTcTmemCols)
                 : "memory");
}

// Applies one block (matrix U, targets tpack, transposed geometry tr) to
// chunks chunk, chunk + step, ... below nchunk of the state psi.  `parity`
// is the MMA mbarrier's phase, carried from call to call.  kBulkB: the B
// operands arrive by a bulk copy that completes on m.bbar() in phase
// parity `bpar` (U unused); the MMA-issuing thread waits for it before its
// first MMAs.  kCg: state loads bypass L1 (other CTAs of the same launch
// wrote the state).  Returns false when a wait timed out (the same value in
// every thread of the CTA).
template <bool kTrans, bool kBulkB, bool kCg = false>
__device__ __forceinline__ bool tc_apply5_chunks(float2* __restrict__ psi,
                                                 const float2* __restrict__ U, uint32_t tpack,
                                                 const TcTrans& tr, int chunk, int nchunk,
                                                 int step, const TcSmem& m,
                                                 uint32_t tmem, uint32_t& parity,
                                                 uint32_t bpar = 0) {
  float* a_hi = m.a_hi();
  float* a_lo = m.a_lo();
  // staging buffers of the transposed variant: the A operands' space, free
  // whenever no MMA is in flight (loads stage in a_hi, results in a_lo)
  float2* stage_in = reinterpret_cast<float2*>(a_hi);
  float2* stage_out = reinterpret_cast<float2*>(a_lo);
  const int tid = threadIdx.x, warp = tid >> 5;

  int t[kTcBits];
#pragma unroll
  for (int i = 0; i < kTcBits; ++i) t[i] = int((tpack >> (5 * i)) & 31u);
  // gather offsets of a group's amplitudes (direct variant) or their
  // swizzled staging slots (transposed variant)
  uint32_t off[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    uint32_t o = 0;
    if (kTrans) {
      const uint32_t Lj = tr_deposit(uint32_t(j), tr.tpos, kTcBits);
      o = Lj ^ tr_h(Lj, tr.c);
    } else {
#pragma unroll
      for (int i = 0; i < kTcBits; ++i) o |= uint32_t((j >> i) & 1) << t[i];
    }
    off[j] = o;
  }
  // transposed variant: this thread's row slot base, and its part of the
  // linear 16-byte accesses (chunk positions 2 * (tid + 128 i))
  uint32_t swr = 0, h_t = 0;
  int64_t dep_t = 0;
  if (kTrans) {
    const uint32_t Lr = tr_deposit(uint32_t(tid), tr.rpos, 7);
    swr = Lr ^ tr_h(Lr, tr.c);
    dep_t = tr_dep(uint32_t(2 * tid), tr.cb);
    h_t = tr_h(uint32_t(2 * tid), tr.c);
  }

  // B operands: R in real form, split into tf32 hi and lo (no MMA is in
  // flight: the previous call's last completion was waited for)
  for (int idx = tid; !kBulkB && idx < kTcNdim * kTcKdim; idx += blockDim.x) {
    const int nr = idx / kTcKdim, k = idx % kTcKdim;
    const float2 u = U[(nr >> 1) * 32 + (k >> 1)];
    const float v = (nr & 1) ? ((k & 1) ? u.x : u.y) : ((k & 1) ? -u.y : u.x);
    const float hi = tf32_hi(v);
    const uint32_t o = kmaj(nr, k) >> 2;
    m.b_hi()[o] = hi;
    m.b_lo()[o] = v - hi;
  }

  float2 v[32];
  float4 raw[16];
  // chunk c starts at the index of its group 128 c (row and target bits 0)
  auto chunk_base = [&](int c) { return group_base(int64_t(c) * kTcRows, t); };
  // linear 16-byte loads of a chunk into registers (transposed variant)
  auto load_raw = [&](int c) {
    const float2* src = psi + chunk_base(c) + dep_t;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      raw[i] = kCg ? __ldcg(reinterpret_cast<const float4*>(src + tr_dep(uint32_t(256 * i), tr.cb)))
                   : __ldcs(reinterpret_cast<const float4*>(src + tr_dep(uint32_t(256 * i), tr.cb)));
  };
  // registers -> swizzled staging slots (transposed variant)
  auto stage_raw = [&]() {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint32_t L = uint32_t(2 * tid + 256 * i);
      const uint32_t h = h_t ^ tr_h(uint32_t(256 * i), tr.c);
      const uint32_t sw = L ^ h;
      float4 x = raw[i];
      if (h & 1u) x = make_float4(x.z, x.w, x.x, x.y);
      *reinterpret_cast<float4*>(stage_in + (sw & ~1u)) = x;
    }
  };
  if (chunk < nchunk) {
    if (kTrans) {
      load_raw(chunk);
    } else {
      const float2* src = psi + group_base(int64_t(chunk) * kTcRows + tid, t);
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] = kCg ? __ldcg(src + off[j]) : src[off[j]];
    }
  }
  bool failed = false, b_waited = !kBulkB;
  while (chunk < nchunk) {
    if (kTrans) {
      // staged chunk -> this thread's group (the staging space is the A
      // operands' space, free here: no MMA is in flight)
      stage_raw();
      __syncthreads();
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] = stage_in[swr ^ off[j]];
      __syncthreads();
    }
    // A operands of this chunk: row tid, 16-byte pieces of two amplitudes
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float x0 = v[2 * q].x, y0 = v[2 * q].y, x1 = v[2 * q + 1].x, y1 = v[2 * q + 1].y;
      const float4 hi = make_float4(tf32_hi(x0), tf32_hi(y0), tf32_hi(x1), tf32_hi(y1));
      const float4 lo = make_float4(x0 - hi.x, y0 - hi.y, x1 - hi.z, y1 - hi.w);
      const uint32_t o = kmaj(tid, 4 * q);
      *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(a_hi) + o) = hi;
      *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(a_lo) + o) = lo;
    }
    // operands written by the generic proxy are read by the tensor core
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    bool issue = tid == 0;
    if (!b_waited) {
      // the B operands' bulk copy (bounded wait; on a timeout no MMA is
      // issued, so the completion wait below times out as well)
      if (issue) {
        bool ok = false;
        for (uint32_t it = 0; it < kTcSpin && !ok; ++it) ok = mbar_try_wait(smem_u32(m.bbar()), bpar);
        if (!ok) {
          atomicExch(m.timed_out(), 1);
          issue = false;
        }
      }
      b_waited = true;
    }
    if (issue) {
      const uint32_t idesc = idesc_tf32(kTcRows, kTcNdim);
      const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo);
      const uint32_t bh = smem_u32(m.b_hi()), bl = smem_u32(m.b_lo());
      const uint32_t as[3] = {al, ah, ah}, bs[3] = {bh, bl, bh};
      uint32_t acc = 0;
      for (int pr = 0; pr < 3; ++pr)
        for (int s = 0; s < kTcKdim / 8; ++s) {
          const uint64_t ad = smem_desc(as[pr] + uint32_t(s) * 256u, 128u, kTcSbo);
          const uint64_t bd = smem_desc(bs[pr] + uint32_t(s) * 256u, 128u, kTcSbo);
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
              : "memory");
          acc = 1;
        }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              smem_u32(m.bar()))
          : "memory");
    }
    const int next = chunk + step;
    if (next < nchunk) {  // the next chunk's loads overlap the MMAs
      if (kTrans) {
        load_raw(next);
      } else {
        const float2* src = psi + group_base(int64_t(next) * kTcRows + tid, t);
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = kCg ? __ldcg(src + off[j]) : src[off[j]];
      }
    }
    bool done = false;
    for (uint32_t it = 0; it < kTcSpin && !done; ++it) done = mbar_try_wait(smem_u32(m.bar()), parity);
    if (!done) atomicExch(m.timed_out(), 1);
    parity ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (*m.timed_out()) {
      failed = true;
      break;
    }
    // D row tid (TMEM lane tid) back to the group's amplitudes
    {
      const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16);
      uint32_t d[64];
      tmem_ld16(taddr, d);
      tmem_ld16(taddr + 16u, d + 16);
      tmem_ld16(taddr + 32u, d + 32);
      tmem_ld16(taddr + 48u, d + 48);
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (kTrans) {
        // group -> swizzled staging slots, then linear 16-byte stores
#pragma unroll
        for (int i = 0; i < 32; ++i)
          stage_out[swr ^ off[i]] =
              make_float2(__uint_as_float(d[2 * i]), __uint_as_float(d[2 * i + 1]));
        __syncthreads();
        float2* dst = psi + chunk_base(chunk) + dep_t;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const uint32_t L = uint32_t(2 * tid + 256 * i);
          const uint32_t h = h_t ^ tr_h(uint32_t(256 * i), tr.c);
          float4 x = *reinterpret_cast<const float4*>(stage_out + ((L ^ h) & ~1u));
          if (h & 1u) x = make_float4(x.z, x.w, x.x, x.y);
          __stcs(reinterpret_cast<float4*>(dst + tr_dep(uint32_t(256 * i), tr.cb)), x);
        }
      } else {
        float2* dst = psi + group_base(int64_t(chunk) * kTcRows + tid, t);
#pragma unroll
        for (int i = 0; i < 32; ++i)
          dst[off[i]] = make_float2(__uint_as_float(d[2 * i]), __uint_as_float(d[2 * i + 1]));
      }
    }
    // TMEM and the A operands are free for the next chunk
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    chunk = next;
  }
  return !failed;
}

template <bool kTrans>
__global__ void __launch_bounds__(kTcRows, 2)
tc_apply5_kernel(float2* __restrict__ psi, int n, const float2* __restrict__ U,
                 uint32_t tpack, TcTrans tr, int* status) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  const TcSmem m{tc_smem};
  const uint32_t tmem = tc_begin(m);
  uint32_t parity = 0;
  const int nchunk = 1 << (n - kTcBits - 7);  // n <= 31: at most 2^19 chunks
  const bool ok = tc_apply5_chunks<kTrans, false>(psi, U, tpack, tr, int(blockIdx.x), nchunk,
                                                  int(gridDim.x), m, tmem, parity);
  tc_end(m, tmem, !ok, parity, status);
}

// Units of many rows' states (lockstep rows), taken grid-strided; each
// unit's chunks run in order, the next chunk's loads overlapping the MMAs.
// A unit's B operands (block `mat` of B, kTcBfloats floats) come in one
// bulk copy (cp.async.bulk, the TMA engine) issued when the unit starts;
// the previous unit's MMAs, which read the old ones, have completed then.
template <bool kTrans>
__global__ void __launch_bounds__(kTcRows, 2)
tc_apply5_units_kernel(float2* __restrict__ state, int row_shift, const float* __restrict__ B,
                       const TcUnit* __restrict__ units, int nunits, int* status) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  const TcSmem m{tc_smem};
  const uint32_t tmem = tc_begin(m);
  uint32_t parity = 0, copies = 0;
  bool ok = true;
  for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x, ++copies) {
    const TcUnit un = units[u];
    if (threadIdx.x == 0) {
      const uint32_t bar = smem_u32(m.bbar());
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                   "r"(uint32_t(kTcBfloats * 4))
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
          "[%3];\n" ::"r"(smem_u32(m.b_hi())),
          "l"(B + int64_t(un.mat) * kTcBfloats), "r"(uint32_t(kTcBfloats * 4)), "r"(bar)
          : "memory");
    }
    float2* psi = state + (row_shift >= 0 ? (int64_t(un.row) << row_shift) : un.off);
    ok = tc_apply5_chunks<kTrans, true>(psi, nullptr, un.tpack, un.tr, int(un.chunk0),
                                        int(un.chunk0) + un.nchunks, 1, m, tmem, parity,
                                        copies & 1u);
  }
  if (!ok) {
    // the failed unit's B copy may still be in flight (bounded wait)
    bool done = false;
    for (uint32_t it = 0; it < kTcSpin && !done; ++it)
      done = mbar_try_wait(smem_u32(m.bbar()), (copies - 1u) & 1u);
  }
  tc_end(m, tmem, !ok, parity, status);
}

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Persistent form: every unit of a lockstep group in one launch.  CTAs take
// units from a queue counter in order (block index, row, chunk), so the
// units a unit depends on (its row's earlier blocks) were taken before it
// by running CTAs and always finish: a unit waits (bounded) until its row's
// count of finished units reaches `need`, then runs, then publishes (every
// thread fences its state stores, the CTA synchronizes, one thread adds 1
// to the count).  State loads bypass L1, since other CTAs of the launch
// wrote the state.  A timed-out wait sets *status; a CTA that sees *status
// set takes no further units.
__global__ void __launch_bounds__(kTcRows, 2)
tc_lock_persistent_kernel(float2* __restrict__ state, int row_shift,
                          const float* __restrict__ B, const TcUnit* __restrict__ units,
                          int nunits, int* queue, int* done, int* status) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  const TcSmem m{tc_smem};
  const uint32_t tmem = tc_begin(m);
  uint32_t parity = 0, copies = 0;
  bool ok = true;
  for (;;) {
    if (threadIdx.x == 0)
      *m.next_unit() =
          *reinterpret_cast<volatile int*>(status) != 0 ? nunits : atomicAdd(queue, 1);
    __syncthreads();
    const int u = *m.next_unit();
    if (u >= nunits) break;
    const TcUnit un = units[u];
    if (threadIdx.x == 0 && un.need > 0) {
      bool ready = false;
      for (uint32_t it = 0; it < kTcSpin && !ready; ++it) {
        ready = ld_acquire_gpu(done + un.slot) >= un.need;
        if (!ready) {
          if (*reinterpret_cast<volatile int*>(status) != 0) break;
          __nanosleep(64);
        }
      }
      if (!ready) atomicExch(m.timed_out(), 1);
    }
    __syncthreads();
    if (*m.timed_out()) {
      ok = false;
      break;
    }
    if (threadIdx.x == 0) {
      const uint32_t bar = smem_u32(m.bbar());
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                   "r"(uint32_t(kTcBfloats * 4))
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
          "[%3];\n" ::"r"(smem_u32(m.b_hi())),
          "l"(B + int64_t(un.mat) * kTcBfloats), "r"(uint32_t(kTcBfloats * 4)), "r"(bar)
          : "memory");
    }
    float2* psi = state + (row_shift >= 0 ? (int64_t(un.row) << row_shift) : un.off);
    const uint32_t tpack = un.tpack & ~kTcUnitTrans;
    if (un.tpack & kTcUnitTrans)
      ok = tc_apply5_chunks<true, true, true>(psi, nullptr, tpack, un.tr, int(un.chunk0),
                                              int(un.chunk0) + un.nchunks, 1, m, tmem, parity,
                                              copies & 1u);
    else
      ok = tc_apply5_chunks<false, true, true>(psi, nullptr, tpack, un.tr, int(un.chunk0),
                                               int(un.chunk0) + un.nchunks, 1, m, tmem, parity,
                                               copies & 1u);
    ++copies;
    if (!ok) break;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(done + un.slot, 1);
    }
  }
  if (!ok && copies > 0) {
    // the failed unit's B copy may still be in flight (bounded wait)
    bool fin = false;
    for (uint32_t it = 0; it < kTcSpin && !fin; ++it)
      fin = mbar_try_wait(smem_u32(m.bbar()), (copies - 1u) & 1u);
  }
  tc_end(m, tmem, !ok, parity, status);
}

// ---- two blocks per sweep ------------------------------------------------------
// tc_sweep_kernel: 256 threads, one CTA per SM, tiles taken grid-strided.
// Per tile: bulk copies (cp.async.bulk, completing on an mbarrier) bring the
// tile's runs of 2^r0 contiguous amplitudes into one of two 64 KiB staging
// buffers while the other buffer's tile is processed; then for each block
// every thread gathers its group's 32 amplitudes from the tile, splits them
// into tf32 hi / lo and stores them into tensor memory (A operands of its
// 128-row chunk: warps 0-3 chunk 0, warps 4-7 chunk 1), one thread issues
// the 2 x 24 MMAs (A from TMEM, B from shared memory), and every thread
// writes its group's results back into the tile; finally bulk copies write
// the tile back.  TMEM: per chunk A_hi, A_lo and D, 64 columns each.
constexpr int kSwThreads = 256;
constexpr int kSwTileBits = 13;
constexpr size_t kSwTileBytes = size_t(8) << kSwTileBits;             // 64 KiB
constexpr size_t kSwBBytes = 2 * kTcBbytes;                           // hi + lo
// tables: tile bases (2 x 512 int64: low and high 9 bits of the tile index)
// and both blocks' target slot offsets (2 x 32 uint32)
constexpr size_t kSwTabBytes = 2 * 512 * 8 + 2 * 32 * 4;
constexpr size_t kSwSmem = 2 * kSwTileBytes + 2 * kSwBBytes + kSwTabBytes + 64;
constexpr uint32_t kSwTmemCols = 512;
constexpr uint32_t kSwChunkCols = 192;

__device__ __forceinline__ int sw_cb(const TcSweep& g, int p) {
  return p < 12 ? int((g.cb >> (5 * p)) & 31u) : int(g.cb12);
}

// physical offset of the tile positions set in L
__device__ __forceinline__ int64_t sw_dep(const TcSweep& g, uint32_t L) {
  int64_t o = 0;
#pragma unroll
  for (int p = 0; p < kSwTileBits; ++p)
    if ((L >> p) & 1u) o |= int64_t(1) << sw_cb(g, p);
  return o;
}

// staging slot of tile position L (an 8-byte slot; bit 3 flipped by the
// parity of L's bits in hmask)
__device__ __forceinline__ uint32_t sw_slot(const TcSweep& g, uint32_t L) {
  return L ^ ((uint32_t(__popc(L & g.hmask)) & 1u) << 3);
}

__device__ __forceinline__ uint32_t sw_deposit(uint32_t v, uint32_t pos, int bits) {
  uint32_t L = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i)
    if (i < bits && ((v >> i) & 1u)) L |= 1u << ((pos >> (4 * i)) & 15u);
  return L;
}

// the index bits outside the tile receive tile index t (ascending)
__device__ __forceinline__ int64_t sw_tile_base(uint32_t smask, int n, int64_t t) {
  int64_t o = 0;
  int k = 0;
  for (int b = 0; b < n; ++b)
    if (!((smask >> b) & 1u)) {
      if ((t >> k) & 1) o |= int64_t(1) << b;
      ++k;
    }
  return o;
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, "
      "%10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, "
      "%26, %27, %28, %29, %30, %31, %32};\n" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
      "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
      "r"(v[15]), "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]),
      "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]),
      "r"(v[29]), "r"(v[30]), "r"(v[31])
      : "memory");
}

__global__ void __launch_bounds__(kSwThreads, 1)
tc_sweep_kernel(float2* __restrict__ psi, int n, const float2* __restrict__ U0,
                const float2* __restrict__ U1, TcSweep g, int* status) {
  extern __shared__ __align__(1024) unsigned char sw_smem[];
  float2* tiles = reinterpret_cast<float2*>(sw_smem);
  float* bsm = reinterpret_cast<float*>(sw_smem + 2 * kSwTileBytes);
  int64_t* base_lo = reinterpret_cast<int64_t*>(sw_smem + 2 * kSwTileBytes + 2 * kSwBBytes);
  int64_t* base_hi = base_lo + 512;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(base_hi + 512);  // [block][j]
  uint64_t* lbar =
      reinterpret_cast<uint64_t*>(sw_smem + 2 * kSwTileBytes + 2 * kSwBBytes + kSwTabBytes);
  uint64_t* mbar = lbar + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(lbar + 3);
  int* timed_out = reinterpret_cast<int*>(lbar + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int chunk = warp >> 2;
  const uint32_t lane_field = uint32_t((warp & 3) * 32) << 16;

  // B operands of both blocks: R in real form, split into tf32 hi and lo
  for (int b = 0; b < 2; ++b) {
    const float2* U = b ? U1 : U0;
    float* bh = bsm + b * (kSwBBytes / 4);
    float* bl = bh + kTcBbytes / 4;
    for (int idx = tid; idx < kTcNdim * kTcKdim; idx += blockDim.x) {
      const int nr = idx / kTcKdim, k = idx % kTcKdim;
      const float2 u = U[(nr >> 1) * 32 + (k >> 1)];
      const float v = (nr & 1) ? ((k & 1) ? u.x : u.y) : ((k & 1) ? -u.y : u.x);
      const float hi = tf32_hi(v);
      const uint32_t o = kmaj(nr, k) >> 2;
      bh[o] = hi;
      bl[o] = v - hi;
    }
  }
  // tile bases: the tile index's low and high 9 bits deposited into the
  // index bits outside the tile; target slot offsets of both blocks (the
  // staging slot is XOR-linear in the tile position)
  for (int i = tid; i < 1024; i += blockDim.x) {
    const int half = i >> 9;
    base_lo[i] = sw_tile_base(g.smask, n, int64_t(i & 511) << (9 * half));
  }
  for (int i = tid; i < 64; i += blockDim.x)
    tslot[i] = sw_slot(g, sw_deposit(uint32_t(i & 31), g.tpos[i >> 5], 5));
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  if (tid == 0) {
    *timed_out = 0;
    for (int i = 0; i < 2; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(lbar + i)),
                   "r"(kSwThreads)
                   : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kSwTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const int64_t ntiles = int64_t(1) << (n - kSwTileBits);
  const int r0 = int(g.r0);
  const int runs = 1 << (kSwTileBits - r0);
  const uint32_t run_bytes = 8u << r0;

  // this thread's runs (at most 4): state offsets and staging slots
  int64_t run_off[4];
  uint32_t run_slot[4];
  int my_runs = 0;
  for (int q = tid; q < runs && my_runs < 4; q += kSwThreads, ++my_runs) {
    const uint32_t L0 = uint32_t(q) << r0;
    run_off[my_runs] = sw_dep(g, L0);
    run_slot[my_runs] = sw_slot(g, L0);
  }
  auto tile_base = [&](int64_t t) { return base_lo[t & 511] | base_hi[(t >> 9) & 511]; };
  auto issue_load = [&](int64_t t, int buf) {
    const int64_t base = tile_base(t);
    const uint32_t mine = uint32_t(my_runs) * run_bytes;
    const uint32_t bar = smem_u32(lbar + buf);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                 "r"(mine)
                 : "memory");
    float2* tile = tiles + (size_t(buf) << kSwTileBits);
    for (int i = 0; i < my_runs; ++i) {
      const float2* src = psi + base + run_off[i];
      const uint32_t dst = smem_u32(tile + run_slot[i]);
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
          "[%3];\n" ::"r"(dst),
          "l"(src), "r"(run_bytes), "r"(bar)
          : "memory");
    }
  };
  auto issue_store = [&](int64_t t, int buf) {
    const int64_t base = tile_base(t);
    const float2* tile = tiles + (size_t(buf) << kSwTileBits);
    for (int i = 0; i < my_runs; ++i) {
      float2* dst = psi + base + run_off[i];
      const uint32_t src = smem_u32(tile + run_slot[i]);
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst),
                   "r"(src), "r"(run_bytes)
                   : "memory");
    }
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
  };

  // this thread's group row slot in each block (constant over the tiles)
  const uint32_t grp = uint32_t(chunk * 128 + (warp & 3) * 32 + lane);
  const uint32_t srow0 = sw_slot(g, sw_deposit(grp, g.rpos[0], 8));
  const uint32_t srow1 = sw_slot(g, sw_deposit(grp, g.rpos[1], 8));
  uint32_t lpar[2] = {0u, 0u}, mpar = 0u;
  bool failed = false, load_pending[2] = {false, false};
  int64_t t = blockIdx.x;
  if (t < ntiles) {
    issue_load(t, 0);
    load_pending[0] = true;
  }
  for (int k = 0; t < ntiles && !failed; t += gridDim.x, ++k) {
    const int buf = k & 1;
    const int64_t next = t + gridDim.x;
    if (next < ntiles) {
      // the other buffer's store (tile k - 1) must have read shared memory
      asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
      __syncthreads();
      issue_load(next, buf ^ 1);
      load_pending[buf ^ 1] = true;
    }
    {
      bool done = false;
      for (uint32_t it = 0; it < kTcSpin && !done; ++it)
        done = mbar_try_wait(smem_u32(lbar + buf), lpar[buf]);
      if (!done) atomicExch(timed_out, 1);
      else load_pending[buf] = false;
      lpar[buf] ^= 1u;
    }
    __syncthreads();
    if (*timed_out) {
      failed = true;
      break;
    }
    float2* tile = tiles + (size_t(buf) << kSwTileBits);
    for (int b = 0; b < 2 && !failed; ++b) {
      const uint32_t sr = b ? srow1 : srow0;
      const uint32_t* ts = tslot + 32 * b;
      // A operands of this thread's row: amplitudes 16 h .. 16 h + 15
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t hi[32], lo[32];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float2 v = tile[sr ^ ts[16 * h + i]];
          const float hx = tf32_hi(v.x), hy = tf32_hi(v.y);
          hi[2 * i] = __float_as_uint(hx);
          hi[2 * i + 1] = __float_as_uint(hy);
          lo[2 * i] = __float_as_uint(v.x - hx);
          lo[2 * i + 1] = __float_as_uint(v.y - hy);
        }
        const uint32_t col = uint32_t(chunk) * kSwChunkCols + 32u * uint32_t(h);
        tmem_st32(tmem + lane_field + col, hi);
        tmem_st32(tmem + lane_field + col + 64u, lo);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      if (tid == 0) {
        const uint32_t idesc = idesc_tf32(kTcRows, kTcNdim);
        const float* bh = bsm + b * (kSwBBytes / 4);
        const uint32_t bhi = smem_u32(bh), blo = smem_u32(bh + kTcBbytes / 4);
        for (int c = 0; c < 2; ++c) {
          const uint32_t a_hi = tmem + uint32_t(c) * kSwChunkCols;
          const uint32_t a_lo = a_hi + 64u, d = a_hi + 128u;
          const uint32_t as[3] = {a_lo, a_hi, a_hi}, bs[3] = {bhi, blo, bhi};
          uint32_t acc = 0;
          for (int pr = 0; pr < 3; ++pr)
            for (int st = 0; st < kTcKdim / 8; ++st) {
              const uint64_t bd = smem_desc(bs[pr] + uint32_t(st) * 256u, 128u, kTcSbo);
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
                  "r"(as[pr] + uint32_t(8 * st)), "l"(bd), "r"(idesc), "r"(acc)
                  : "memory");
              acc = 1;
            }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(mbar))
            : "memory");
      }
      bool done = false;
      for (uint32_t it = 0; it < kTcSpin && !done; ++it)
        done = mbar_try_wait(smem_u32(mbar), mpar);
      if (!done) atomicExch(timed_out, 1);
      mpar ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      __syncthreads();
      if (*timed_out) {
        failed = true;
        break;
      }
      {
        uint32_t dv[64];
        const uint32_t taddr = tmem + lane_field + uint32_t(chunk) * kSwChunkCols + 128u;
        tmem_ld16(taddr, dv);
        tmem_ld16(taddr + 16u, dv + 16);
        tmem_ld16(taddr + 32u, dv + 32);
        tmem_ld16(taddr + 48u, dv + 48);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; ++j)
          tile[sr ^ ts[j]] =
              make_float2(__uint_as_float(dv[2 * j]), __uint_as_float(dv[2 * j + 1]));
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    }
    if (failed) break;
    // the tile's generic-proxy writes are read by the bulk copies
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    issue_store(t, buf);
  }
  // every bulk store has completed; a prefetched load still in flight after
  // a failure is waited for (bounded) before the CTA's shared memory goes
  asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
  if (failed) {
    for (int b = 0; b < 2; ++b)
      if (load_pending[b]) {
        bool done = false;
        for (uint32_t it = 0; it < kTcSpin && !done; ++it)
          done = mbar_try_wait(smem_u32(lbar + b), lpar[b]);
      }
    bool done = false;
    for (uint32_t it = 0; it < kTcSpin && !done; ++it)
      done = mbar_try_wait(smem_u32(mbar), mpar ^ 1u);
    if (tid == 0) atomicExch(status, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(kSwTmemCols)
                 : "memory");
}

}  // namespace

const void* tc_apply5_kernel_ptr() {
  return reinterpret_cast<const void*>(&tc_apply5_kernel<false>);
}
size_t tc_apply5_smem_bytes() { return kTcSmem; }

cudaError_t launch_tc_fuse(const BatchDevice& b, const float2* mats, int row,
                           const TcBlock* blocks, const int32_t* members, int nblocks,
                           float2* U, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  tc_fuse_kernel<<<nblocks, 32, 0, s>>>(b, mats, row, blocks, members, nblocks, U);
  return cudaGetLastError();
}

size_t tc_b_floats() { return size_t(kTcBfloats); }

cudaError_t launch_tc_fuse_b(const BatchDevice& b, const float2* mats,
                             const int32_t* block_rows, const TcBlock* blocks,
                             const int32_t* members, int nblocks, float* B, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  tc_fuse_b_kernel<<<nblocks, 32, 0, s>>>(b, mats, block_rows, blocks, members, nblocks, B);
  return cudaGetLastError();
}

// Chunk geometry of the transposed variant for a block, or false when the
// block's targets are all at bit 5 or above (the direct variant: the 32
// groups of a warp are then 32 consecutive amplitudes).
bool tc_transposed_geometry(const TcBlock& blk, int n, TcTrans* out) {
  if (blk.tgt[0] >= 5) return false;
  bool is_t[64] = {};
  for (int i = 0; i < kTcBits; ++i) is_t[blk.tgt[i]] = true;
  int rows[7], nr = 0;
  for (int b = 0; b < n && nr < 7; ++b)
    if (!is_t[b]) rows[nr++] = b;
  int cb[12], np = 0;
  int role[12];  // >= 0: target index; < 0: -1 - row index
  {
    int ti = 0, ri = 0;
    while (ti < kTcBits || ri < 7) {
      const bool take_t = ri == 7 || (ti < kTcBits && blk.tgt[ti] < rows[ri]);
      if (take_t) {
        cb[np] = blk.tgt[ti];
        role[np++] = ti++;
      } else {
        cb[np] = rows[ri];
        role[np++] = -1 - ri++;
      }
    }
  }
  TcTrans tr{};
  for (int p = 0; p < 12; ++p) {
    tr.cb |= uint64_t(cb[p]) << (5 * p);
    if (role[p] >= 0) tr.tpos |= uint32_t(p) << (4 * role[p]);
    else tr.rpos |= uint32_t(p) << (4 * (-1 - role[p]));
  }
  // swizzle: the 5 lowest row bits (a warp's lanes) must reach every slot
  // bit 0-3; positions below 4 contribute their own bit, positions above
  // take the slot bits still missing
  uint32_t covered = 0;
  for (int i = 0; i < 5; ++i) {
    const int p = int((tr.rpos >> (4 * i)) & 15u);
    if (p < 4) covered |= 1u << p;
  }
  for (int i = 0; i < 5; ++i) {
    const int p = int((tr.rpos >> (4 * i)) & 15u);
    if (p < 4) continue;
    for (int q = 0; q < 4; ++q)
      if (!(covered & (1u << q))) {
        covered |= 1u << q;
        tr.c |= (1u << q) << (4 * (p - 4));
        break;
      }
  }
  *out = tr;
  return true;
}

cudaError_t launch_tc_apply5(float2* psi, int n, const float2* U, const TcBlock& blk,
                             int* status, int grid, cudaStream_t s) {
  if (n < kTcBits + 7 || n > 31) return cudaErrorInvalidValue;
  uint32_t tpack = 0;
  for (int i = 0; i < kTcBits; ++i) {
    if (blk.tgt[i] >= n || (i > 0 && blk.tgt[i] <= blk.tgt[i - 1])) return cudaErrorInvalidValue;
    tpack |= uint32_t(blk.tgt[i]) << (5 * i);
  }
  const int64_t nchunk = int64_t(1) << (n - kTcBits - 7);
  if (grid > nchunk) grid = int(nchunk);
  TcTrans tr{};
  const bool trans = tc_transposed_geometry(blk, n, &tr);
  const void* k = trans ? reinterpret_cast<const void*>(&tc_apply5_kernel<true>)
                        : reinterpret_cast<const void*>(&tc_apply5_kernel<false>);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kTcSmem));
  if (e != cudaSuccess) return e;
  if (trans)
    tc_apply5_kernel<true><<<grid, kTcRows, kTcSmem, s>>>(psi, n, U, tpack, tr, status);
  else
    tc_apply5_kernel<false><<<grid, kTcRows, kTcSmem, s>>>(psi, n, U, tpack, tr, status);
  return cudaGetLastError();
}

int tc_unit_geometry(const TcBlock& blk, int n, uint32_t* tpack, TcTrans* tr) {
  if (n < kTcBits + 7 || n > 31) return -1;
  uint32_t tp = 0;
  for (int i = 0; i < kTcBits; ++i) {
    if (blk.tgt[i] >= n || (i > 0 && blk.tgt[i] <= blk.tgt[i - 1])) return -1;
    tp |= uint32_t(blk.tgt[i]) << (5 * i);
  }
  *tpack = tp;
  *tr = TcTrans{};
  return tc_transposed_geometry(blk, n, tr) ? 1 : 0;
}

cudaError_t launch_tc_apply5_units(float2* state, int row_shift, const float* B,
                                   const TcUnit* units, int nunits, bool trans, int* status,
                                   int grid, cudaStream_t s) {
  if (reinterpret_cast<uintptr_t>(B) % 16 != 0) return cudaErrorInvalidValue;
  if (nunits <= 0) return cudaSuccess;
  if (grid > nunits) grid = nunits;
  if (grid < 1) grid = 1;
  const void* k = trans ? reinterpret_cast<const void*>(&tc_apply5_units_kernel<true>)
                        : reinterpret_cast<const void*>(&tc_apply5_units_kernel<false>);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kTcSmem));
  if (e != cudaSuccess) return e;
  if (trans)
    tc_apply5_units_kernel<true><<<grid, kTcRows, kTcSmem, s>>>(state, row_shift, B, units,
                                                                nunits, status);
  else
    tc_apply5_units_kernel<false><<<grid, kTcRows, kTcSmem, s>>>(state, row_shift, B, units,
                                                                 nunits, status);
  return cudaGetLastError();
}

cudaError_t launch_tc_lock_persistent(float2* state, int row_shift, const float* B,
                                      const TcUnit* units, int nunits, int* queue, int* done,
                                      int* status, int grid, cudaStream_t s) {
  if (nunits <= 0) return cudaSuccess;
  if (reinterpret_cast<uintptr_t>(B) % 16 != 0) return cudaErrorInvalidValue;
  if (grid > nunits) grid = nunits;
  if (grid < 1) grid = 1;
  cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(&tc_lock_persistent_kernel),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kTcSmem));
  if (e != cudaSuccess) return e;
  tc_lock_persistent_kernel<<<grid, kTcRows, kTcSmem, s>>>(state, row_shift, B, units, nunits,
                                                           queue, done, status);
  return cudaGetLastError();
}

bool tc_sweep_geometry(const TcBlock& b0, const TcBlock& b1, int n, TcSweep* out) {
  if (n < kSwTileBits + 1 || n > 31) return false;
  const TcBlock* bl[2] = {&b0, &b1};
  uint32_t smask = 0x7u;  // bits 0-2
  for (int b = 0; b < 2; ++b)
    for (int i = 0; i < kTcBits; ++i) {
      if (bl[b]->tgt[i] < 4 || bl[b]->tgt[i] >= n) return false;
      smask |= 1u << bl[b]->tgt[i];
    }
  if (__builtin_popcount(smask) > kSwTileBits) return false;
  for (int bit = 3; bit < n && __builtin_popcount(smask) < kSwTileBits; ++bit)
    smask |= 1u << bit;
  if (__builtin_popcount(smask) != kSwTileBits) return false;
  TcSweep g{};
  g.smask = smask;
  int cb[kSwTileBits], np = 0;
  for (int bit = 0; bit < n; ++bit)
    if ((smask >> bit) & 1u) cb[np++] = bit;
  for (int p = 0; p < 12; ++p) g.cb |= uint64_t(cb[p]) << (5 * p);
  g.cb12 = uint32_t(cb[12]);
  int r0 = 0;
  while (r0 < kSwTileBits && cb[r0] == r0) ++r0;
  g.r0 = uint32_t(r0);
  for (int b = 0; b < 2; ++b) {
    int ti = 0, ri = 0;
    for (int p = 0; p < kSwTileBits; ++p) {
      bool is_t = false;
      for (int i = 0; i < kTcBits; ++i) is_t = is_t || bl[b]->tgt[i] == cb[p];
      if (is_t) g.tpos[b] |= uint32_t(p) << (4 * ti++);
      else g.rpos[b] |= uint32_t(p) << (4 * ri++);
    }
    if (ti != kTcBits || ri != 8) return false;
  }
  // swizzle: a warp's lanes are a block's 5 lowest row positions; slot bits
  // 0-2 are positions 0-2 (never targets); where position 3 is one of the
  // block's targets, one of its lane positions >= 4 must flip slot bit 3
  for (int b = 0; b < 2; ++b) {
    bool pos3_lane = false;
    uint32_t lanes_hi = 0;
    for (int i = 0; i < 5; ++i) {
      const int p = int((g.rpos[b] >> (4 * i)) & 15u);
      if (p == 3) pos3_lane = true;
      if (p >= 4) lanes_hi |= 1u << p;
    }
    if (pos3_lane || (g.hmask & lanes_hi)) continue;
    g.hmask |= lanes_hi & (~lanes_hi + 1u);  // its lowest lane position >= 4
  }
  // a flipped slot bit 3 must not split a run of contiguous amplitudes
  if (g.hmask && r0 > 3) return false;
  *out = g;
  return true;
}

size_t tc_sweep_smem_bytes() { return kSwSmem; }
const void* tc_sweep_kernel_ptr() { return reinterpret_cast<const void*>(&tc_sweep_kernel); }

cudaError_t launch_tc_sweep2(float2* psi, int n, const float2* U0, const float2* U1,
                             const TcBlock& b0, const TcBlock& b1, int* status, int grid,
                             cudaStream_t s) {
  TcSweep g{};
  if (!tc_sweep_geometry(b0, b1, n, &g)) return cudaErrorInvalidValue;
  const int64_t ntiles = int64_t(1) << (n - kSwTileBits);
  if (grid > ntiles) grid = int(ntiles);
  if (grid < 1) grid = 1;
  cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(&tc_sweep_kernel),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kSwSmem));
  if (e != cudaSuccess) return e;
  tc_sweep_kernel<<<grid, kSwThreads, kSwSmem, s>>>(psi, n, U0, U1, g, status);
  return cudaGetLastError();
}

}  // namespace tfqg
