// Internal batch representation shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"
#include "kernels.h"

namespace tfqg {

#define TFQG_CUDA(call)                                                    \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess)                                                 \
      throw ::tfqg::Error(::tfqg::kInternal,                               \
                          std::string("CUDA error: ") +                    \
                              cudaGetErrorString(e_) + " at " #call);      \
  } while (0)

// Process-wide pool of device blocks (capi.cc).  pool_take returns a cached
// block of at least `bytes` (and not much larger) or a new one; pool_give
// keeps a block for reuse.  A block is given back only when no work can
// still use it: `synced` says the caller has synchronized the device,
// otherwise pool_give does (as cudaFree would).  Cached bytes are capped
// (TFQG_POOL_MAX_BYTES, default 4 GiB; 0 disables the pool).
void* pool_take(size_t bytes, int dev, size_t* got);
void pool_give(void* p, size_t bytes, int dev, bool synced) noexcept;
void pool_trim(int dev) noexcept;  // dev < 0: every device

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int device = -1;
  void reserve(size_t need, int dev) {
    if (need <= bytes && dev == device) return;
    release();
    size_t got = 0;
    p = pool_take(std::max<size_t>(need, 256), dev, &got);
    bytes = got;
    device = dev;
  }
  void release(bool synced = false) noexcept {
    if (p) pool_give(p, bytes, device, synced);
    p = nullptr;
    bytes = 0;
  }
  ~DevBuf() { release(); }
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Offsets of the device tables inside one packed blob.
struct TableOffsets {
  size_t prog, rows, gates, pass, ops, terms, chan, kraus, gc, order, order_fwd, meas, mterms,
      order_lock, lock_items;
};

int set_last_error(int code, const std::string& msg);

}  // namespace tfqg

struct tfqg_batch {
  int kind = 0;
  int64_t B = 0, P = 0, n_ops = 0;
  int64_t value_rows = 0;          // rows that take symbol values
  int64_t inner_rows = 0, inner_others = 0;  // TFQG_KIND_INNER shape
  bool inner_grads = false;        // reference programs planned for the adjoint
  tfqg::DevBuf inner_tmp;
  int max_n = 0;
  int max_resident_n = -1;   // largest resident row (-1: none)
  bool any_streamed = false;
  int max_streamed_n = 0;
  // forward modes run wide rows (n >= kWideMinQubits) on the whole grid and
  // the other rows through the persistent kernel's queue (order_fwd)
  std::vector<int32_t> wide_rows;
  int max_wide_n = 0;
  bool any_streamed_fwd = false;
  int max_streamed_n_fwd = 0;
  // forward modes run lockstep rows (lock_min..21 qubits, not wide, in a
  // batch with many of them) group by group over the whole grid, one launch
  // per pass (kernels.h LockItem); the queue then takes order_lock
  struct LockLaunch {
    int32_t begin = 0, count = 0;  // items
    int64_t ntiles = 0;            // tiles (or chunks) the launch covers
  };
  // a launch of the tensor-core block kernel over lockstep rows: units
  // [begin, begin + count) of tcl_units, all of one variant
  struct TcLockLaunch {
    int32_t begin = 0, count = 0;
    bool trans = false;
  };
  struct LockGroup {
    int64_t arena_amps = 0;        // states of the group's rows
    int64_t acc_terms = 0;         // measurement terms of its rows (each row its own)
    LockLaunch rows;               // one item per row (chunk prefix, offset)
    std::vector<LockLaunch> fwd, meas;  // fwd: rows on tile passes only
    // rows whose gates run as tensor-core blocks: one tcl_items entry per
    // row (chunk prefix, offset), their blocks [tc_block_begin, +count) of
    // tcl_blocks, and per block index the direct then transposed launches
    LockLaunch tc_rows;
    int32_t tc_block_begin = 0, tc_block_count = 0;
    std::vector<TcLockLaunch> tc;
    // the same units for the persistent form: [tcp_begin, +tcp_count) of
    // tcl_punits, in queue order
    int32_t tcp_begin = 0, tcp_count = 0;
  };
  std::vector<int32_t> lock_rows;
  std::vector<int32_t> order_lock;
  std::vector<tfqg::LockItem> lock_items;
  std::vector<LockGroup> lock_groups;
  bool any_streamed_lock = false;
  int max_streamed_n_lock = 0;
  // lockstep rows on tensor-core blocks (their blocks' member gates and
  // batch rows, and the units of every launch), uploaded to tcl_tab
  std::vector<tfqg::LockItem> tcl_items;
  std::vector<tfqg::TcBlock> tcl_blocks;
  std::vector<int32_t> tcl_members, tcl_block_rows;
  std::vector<tfqg::TcUnit> tcl_units, tcl_punits;
  int max_grads = 0;
  int64_t total_gates = 0, total_grads = 0;
  bool any_fused = false;  // forward plans hold GK_FUSED gates

  // packed host copies of the device tables
  std::vector<tfqg::DevProgram> programs;
  std::vector<tfqg::DevRow> rows;
  std::vector<tfqg::GateTemplate> gates;
  std::vector<tfqg::DevPass> passes;
  std::vector<tfqg::DevOp> ops;
  std::vector<tfqg::DevTerm> terms;
  std::vector<tfqg::DevChannel> channels;
  std::vector<float2> kraus;
  std::vector<int32_t> grad_cols;
  std::vector<int32_t> order;
  std::vector<int32_t> order_fwd;
  std::vector<tfqg::DevMeas> meas;
  std::vector<tfqg::DevMeasTerm> meas_terms;

  // run-time specialization (jit.cc)
  std::vector<std::vector<uint32_t>> jit_signatures;
  int jit_mode = 0;            // -1 off, 0 automatic, 1 forced
  bool jit_loaded[6] = {};     // compile attempted, per SimMode and wide pass
  std::shared_ptr<void> jit_module[6];
  std::string jit_error;

  // device state
  std::mutex mu;
  int device = -1;
  tfqg::DevBuf tables, mats, dmats, work, counter, values, out, aux, aux2;
  tfqg::DevBuf wide_state, wide_acc;
  tfqg::DevBuf lock_state, lock_acc;
  // tensor-core forward path of wide rows (tc_gates.cu): per wide row its
  // first block and block count (count -1: the row has no 5-bit plan)
  bool tc_planned = false;
  std::vector<tfqg::TcBlock> tc_blocks;
  std::vector<int32_t> tc_members;
  std::vector<std::pair<int32_t, int32_t>> tc_rows;  // parallel to wide_rows
  std::vector<uint8_t> tc_ran;  // the row's last forward call ran the blocks
  std::vector<int32_t> tc_sweeps;  // state sweeps (launches) of that call
  tfqg::DevBuf tc_tab, tc_mats, tc_status;
  tfqg::DevBuf tcl_tab, tcl_mats, tcl_sync;
  const tfqg::LockItem* d_tcl_items = nullptr;
  const tfqg::TcBlock* d_tcl_blocks = nullptr;
  const int32_t* d_tcl_members = nullptr;
  const int32_t* d_tcl_block_rows = nullptr;
  const tfqg::TcUnit* d_tcl_units = nullptr;  // units of the uploaded form
  bool tcl_persistent = false;                 // the uploaded form
  // gives every device buffer back to the pool (the device is synchronized)
  void release_buffers() noexcept {
    tfqg::DevBuf* all[] = {&tables,     &mats,     &dmats,     &work,   &counter,
                           &values,     &out,      &aux,       &aux2,   &wide_state,
                           &wide_acc,   &inner_tmp, &tc_tab,   &tc_mats, &tc_status,
                           &lock_state, &lock_acc,  &tcl_tab,  &tcl_mats, &tcl_sync};
    for (tfqg::DevBuf* d : all) d->release(true);
  }
  tfqg::BatchDevice bd;
  const int32_t* d_order_fwd = nullptr;
  const int32_t* d_order_lock = nullptr;
  const tfqg::LockItem* d_lock_items = nullptr;
};

namespace tfqg {
// Packs the batch's tables into `blob` (256-byte aligned sections).
TableOffsets pack_tables(const tfqg_batch* b, std::vector<unsigned char>* blob);
// Device-table view of a blob copied to `base`.
BatchDevice table_view(const tfqg_batch* b, unsigned char* base,
                       const TableOffsets& o);
}  // namespace tfqg
