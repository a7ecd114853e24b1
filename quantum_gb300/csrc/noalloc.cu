// Expectation entry point that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc.  A framework whose
// caching allocator has already reserved most of the device memory (as
// TensorFlow's GPU allocator does by default) can make a plugin's own
// cudaMalloc fail or fragment the pool; a serving process that sizes all
// device memory at start-up may forbid later allocations.  For them,
// tfqg_batch_expectation_noalloc runs the same expectation kernels as
// tfqg_batch_expectation, but every piece of scratch the kernels need (the
// compiled circuit tables, the bound gate matrices, the work-queue counter
// and the per-CTA state slots of states too large for shared memory) lives in
// one fixed device array declared below.  The caller passes the symbol
// values and the output buffer as device pointers.
//
// Limits and behaviour:
//  * the array holds kNoAllocScratchBytes (64 MiB); every GPU that loads the
//    library holds it until the process exits;
//  * a batch whose tables + matrices + one state slot do not fit is rejected
//    with RESOURCE_EXHAUSTED; when fewer state slots fit than the kernel would
//    normally use, the grid shrinks to the slots that fit;
//  * every call uses the same array and leaves the previous call's contents
//    in it; calls that overlap on the GPU (different streams, different host
//    threads) race on it and must be serialized by the caller;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture on the device.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "../../include/tfq_gb300.h"
#include "batch_internal.h"

namespace tfqg {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on the
// first call per device).
unsigned char* scratch_address(int dev) {
  if (dev < 0 || dev >= kMaxDevices)
    throw Error(kInternal, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      throw Error(kInternal, std::string("cudaGetSymbolAddress failed: ") +
                                 cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  return g_scratch_ptr[dev];
}

}  // namespace
}  // namespace tfqg

using namespace tfqg;

extern "C" int tfqg_batch_expectation_noalloc(tfqg_batch* b,
                                              const float* symbol_values,
                                              float* expectations,
                                              void* stream) {
  try {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    std::lock_guard<std::mutex> lk(b->mu);
    if (b->B == 0 || b->n_ops == 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev;
    TFQG_CUDA(cudaGetDevice(&dev));
    unsigned char* base = scratch_address(dev);

    // layout: [tables][matrices][counter][state slots]
    thread_local std::vector<unsigned char> blob;
    blob.clear();
    TableOffsets o = pack_tables(b, &blob);
    const size_t tables = align256(blob.size());
    const size_t mats = align256(size_t(b->total_gates) * 16 * sizeof(float2));
    const size_t counter = 256;
    const size_t fixed = tables + mats + counter;
    const int mode = kModeExpect;
    size_t smem = sim_smem_bytes(mode, b->max_resident_n, b->any_streamed, 0);
    int grid = sim_grid_size(mode, smem);
    if (b->B < grid) grid = int(b->B);
    int64_t slot_amps = 0;
    if (b->any_streamed) {
      slot_amps = int64_t(1) << b->max_streamed_n;
      const size_t slot_bytes = size_t(slot_amps) * sizeof(float2);
      if (fixed + slot_bytes > kNoAllocScratchBytes)
        throw Error(kResourceExhausted,
                    "tfqg_batch_expectation_noalloc: the batch needs " +
                        std::to_string(fixed + slot_bytes) +
                        " bytes of scratch; the fixed scratch array holds " +
                        std::to_string(kNoAllocScratchBytes));
      const int fit = int((kNoAllocScratchBytes - fixed) / slot_bytes);
      if (fit < grid) grid = fit;
    } else if (fixed > kNoAllocScratchBytes) {
      throw Error(kResourceExhausted,
                  "tfqg_batch_expectation_noalloc: the batch needs " +
                      std::to_string(fixed) +
                      " bytes of scratch; the fixed scratch array holds " +
                      std::to_string(kNoAllocScratchBytes));
    }

    TFQG_CUDA(cudaMemcpyAsync(base, blob.data(), blob.size(),
                              cudaMemcpyHostToDevice, s));
    BatchDevice bd = table_view(b, base, o);
    RunArgs a;
    a.values = symbol_values;
    a.mats = reinterpret_cast<float2*>(base + tables);
    a.counter = reinterpret_cast<int*>(base + tables + mats);
    a.work = reinterpret_cast<float2*>(base + fixed);
    a.slot_amps = slot_amps;
    a.out_f = expectations;
    TFQG_CUDA(cudaMemsetAsync(a.counter, 0, sizeof(int), s));
    TFQG_CUDA(launch_build_matrices(bd, a, false, s));
    const int state_amps = sim_state_amps(b->max_resident_n, b->any_streamed);
    TFQG_CUDA(launch_simulate(mode, bd, a, grid, smem, state_amps, s));
    // the pageable host blob is read before cudaMemcpyAsync returns; keep
    // the stream ordering for the caller
    return 0;
  } catch (const Error& e) {
    return set_last_error(e.code, e.what());
  } catch (const std::exception& e) {
    return set_last_error(kInternal, e.what());
  }
}
