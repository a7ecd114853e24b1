// C ABI (include/tfq_gb300.h): batch compilation on the host, device upload,
// kernel launches.  See the header for the reference functions each entry
// point replaces.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tfq_gb300.h"
#include "batch_internal.h"
#include "gate_math.cuh"
#include "host.h"
#include "jit.h"
#include "kernels.h"
#include "plain.h"

using namespace tfqg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

}  // namespace

int tfqg::set_last_error(int code, const std::string& msg) { return fail(code, msg); }

// ---- device block pool -----------------------------------------------------
namespace {

struct DevicePool {
  std::multimap<size_t, void*> free;  // size -> block
  size_t bytes = 0;
};
std::mutex g_pool_mu;
DevicePool g_pool[64];

size_t pool_cap() {
  static const size_t cap = [] {
    const char* e = getenv("TFQG_POOL_MAX_BYTES");
    return e ? size_t(strtoull(e, nullptr, 10)) : size_t(4) << 30;
  }();
  return cap;
}

bool device_sync(int dev) noexcept {
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) return false;
  if (cur != dev && cudaSetDevice(dev) != cudaSuccess) return false;
  const bool ok = cudaDeviceSynchronize() == cudaSuccess;
  if (cur != dev) cudaSetDevice(cur);
  if (!ok) cudaGetLastError();
  return ok;
}

}  // namespace

void* tfqg::pool_take(size_t bytes, int dev, size_t* got) {
  if (dev >= 0 && dev < 64) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    DevicePool& pl = g_pool[dev];
    auto it = pl.free.lower_bound(bytes);
    // a cached block at most 1.5x (plus 1 MiB) the request
    if (it != pl.free.end() && it->first <= bytes + bytes / 2 + (size_t(1) << 20)) {
      void* p = it->second;
      *got = it->first;
      pl.bytes -= it->first;
      pl.free.erase(it);
      return p;
    }
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    pool_trim(dev);
    e = cudaMalloc(&p, bytes);
  }
  if (e != cudaSuccess)
    throw Error(kInternal, std::string("CUDA error: ") + cudaGetErrorString(e) +
                               " at cudaMalloc");
  *got = bytes;
  return p;
}

void tfqg::pool_give(void* p, size_t bytes, int dev, bool synced) noexcept {
  if (!p) return;
  if (dev < 0 || dev >= 64 || (!synced && !device_sync(dev))) {
    cudaFree(p);
    return;
  }
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    DevicePool& pl = g_pool[dev];
    if (pl.bytes + bytes <= pool_cap()) {
      pl.free.emplace(bytes, p);
      pl.bytes += bytes;
      return;
    }
  }
  cudaFree(p);
}

void tfqg::pool_trim(int dev) noexcept {
  std::vector<void*> blocks;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (int d = 0; d < 64; ++d) {
      if (dev >= 0 && d != dev) continue;
      for (auto& kv : g_pool[d].free) blocks.push_back(kv.second);
      g_pool[d].free.clear();
      g_pool[d].bytes = 0;
    }
  }
  for (void* p : blocks) cudaFree(p);
}

namespace {

std::atomic<int> g_wide_min_qubits{kWideMinQubits};
std::atomic<int> g_wide_few_rows{kWideFewRows};
// Streamed rows of at least this many qubits that do not run wide run in
// lockstep over the whole grid in the forward modes (kernels.h LockItem);
// a value above 21 turns lockstep rows off.
constexpr int kLockMinQubits = 17;
std::atomic<int> g_lock_min_qubits{kLockMinQubits};
// States of one lockstep group (amplitudes): 2^30 = 8 GiB of complex64.
constexpr int64_t kLockArenaAmps = int64_t(1) << 30;
std::atomic<int64_t> g_lock_arena_amps{kLockArenaAmps};

int wide_min_qubits() { return g_wide_min_qubits.load(); }

// Gate fusion of forward plans (on by default).
std::atomic<int> g_gate_fusion{1};
// Row policy per qubit count, set by an autotuner (quantum_gb300/autotune.py)
// for batches created from then on: gate fusion of the forward plans
// (-1: the global setting, 0 off, 1 on) and lockstep rows (-1: the
// lock_min rule, 0 never, 1 when the row is streamed and not wide, on tile
// passes, 2 the same on tensor-core blocks).  Each change starts a new
// epoch, which is part of the compiled-program cache key.
constexpr int kPolicyMaxQubits = 64;
std::atomic<int> g_fuse_by_n[kPolicyMaxQubits];
std::atomic<int> g_lock_by_n[kPolicyMaxQubits];
std::atomic<int> g_policy_epoch{0};
struct PolicyInit {
  PolicyInit() {
    for (int i = 0; i < kPolicyMaxQubits; ++i) {
      g_fuse_by_n[i].store(-1);
      g_lock_by_n[i].store(-1);
    }
  }
} g_policy_init;

bool fuse_for(int n, bool dflt) {
  const int v = (n >= 0 && n < kPolicyMaxQubits) ? g_fuse_by_n[n].load() : -1;
  return v < 0 ? dflt : v != 0;
}

// Lockstep rows run their gates as 5-qubit tensor-core blocks (one launch
// per block index over all the group's rows) or as tile passes, as their
// qubit count's policy says; without one, g_lock_tc decides: 0 tile
// passes, 1 blocks, 2 (default) blocks from kLockTcMinQubits qubits.  On
// GB300 an expectation call over 128 random rows (depth 5-40, random
// pairs) takes 1.20 / 3.35 / 26.1 ms on blocks (one persistent launch)
// against 1.40 / 4.7 / 43.5 ms on tile passes at 15 / 17 / 20 qubits.
std::atomic<int> g_lock_tc{2};
constexpr int kLockTcMinQubits = 15;
// Units of the lockstep tensor-core launches (kernels.h kTcUnitChunks,
// kTcUnitTarget), settable for measurements.
std::atomic<int64_t> g_tc_unit_chunks{kTcUnitChunks};
std::atomic<int64_t> g_tc_unit_target{kTcUnitTarget};
// Lockstep tensor-core rows run as one persistent launch per group (1) or
// one launch per block index and variant (0).
std::atomic<int> g_tc_lock_persistent{1};

// Forward passes of wide rows as 5-bit fused blocks on the tensor cores
// (tc_gates.cu) instead of tile passes on the FP32 pipe: 0 never, 1 always,
// 2 (default) for rows of at least kTcAutoMinQubits qubits, whose states
// (128 MiB and up) no longer fit in L2, so that every pass is an HBM sweep
// and fewer, fuller sweeps win.
std::atomic<int> g_tc_gates{2};
constexpr int kTcAutoMinQubits = 24;

// Whether a lockstep row of n qubits takes tensor-core blocks (decided when
// its batch is created; tensor cores switched off mean tile passes).
bool lock_tc_for(int n) {
  if (g_tc_gates.load() == 0 || n < kTcBits + 7) return false;
  const int pol = n < kPolicyMaxQubits ? g_lock_by_n[n].load() : -1;
  if (pol >= 0) return pol == 2;
  const int d = g_lock_tc.load();
  return d == 1 || (d == 2 && n >= kLockTcMinQubits);
}
// Test hook: a status value the host treats as read back from the block
// kernels of the next calls (0: read the real one).  It lets a test take
// the timeout branch without a timeout on the GPU.  Value 1 also makes a
// captured lockstep call write status 1 into the device word after its
// tensor-core launches (where a timed-out kernel would set it); value 2
// does only the latter, so that an ordinary call still succeeds.
std::atomic<int> g_tc_status_injected{0};
// Two consecutive blocks share one state sweep (tc_sweep_kernel) where
// their targets allow it (1), or every block has its own sweep (0, the
// default: on GB300 a two-block sweep takes 10.3 ms on the 30-qubit state
// against 2 x 3.3 ms for two single-block sweeps).
std::atomic<int> g_tc_sweep{0};

}  // namespace

namespace {

struct Str {
  const char* p;
  int64_t n;
};

std::string make_key(const char* p, int64_t n) { return std::string(p, size_t(n)); }

// Key of a serialized proto in the batch's dedup maps: a view of the
// caller's bytes (valid while the batch is built) and a tag (-1, or the
// reference program of a paired program).  Equality is exact (same
// pointer, or memcmp); the hash reads the length, the first and last 256
// bytes and 64 evenly spaced words, so that a batch of one circuit repeated
// thousands of times is not hashed in full per row.
struct ProtoKey {
  const char* p;
  size_t n;
  int tag;
  bool operator==(const ProtoKey& o) const {
    return n == o.n && tag == o.tag && (p == o.p || memcmp(p, o.p, n) == 0);
  }
};

struct ProtoKeyHash {
  size_t operator()(const ProtoKey& k) const {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ (uint64_t(k.n) * 0xBF58476D1CE4E5B9ull) ^
                 uint64_t(int64_t(k.tag));
    auto mix = [&h](const char* q, size_t m) {
      uint64_t w = 0;
      memcpy(&w, q, m < 8 ? m : 8);
      h ^= w;
      h *= 0xFF51AFD7ED558CCDull;
      h ^= h >> 33;
    };
    if (k.n <= 1024) {
      for (size_t i = 0; i < k.n; i += 8) mix(k.p + i, k.n - i);
    } else {
      for (size_t i = 0; i < 256; i += 8) mix(k.p + i, 8);
      for (size_t i = k.n - 256; i < k.n; i += 8) mix(k.p + i, k.n - i);
      const size_t step = (k.n - 8) / 64;
      for (size_t j = 0; j < 64; ++j) mix(k.p + j * step, 8);
    }
    return size_t(h);
  }
};

// Process-wide cache of compiled and planned programs (a training loop sends
// the same serialized circuits every step).  An entry is keyed exactly by
// the program bytes, the symbol names in column order, the job kind and the
// fusion setting: everything compile_program and plan_program read.  Only
// programs that compiled without error are stored, so a cached program
// raises no error and the order of the batch's errors is unchanged.
struct ProgramCacheEntry {
  std::string bytes;
  std::string names;  // length-prefixed symbol names, column order
  int job = 0;
  int plan_key = 0;    // fusion setting and row-policy epoch
  bool empty = false;  // no moments: expectation -2 (#679)
  CompiledProgram cp;
  std::unordered_map<std::string, int> index;
  size_t cost = 0;
  uint64_t stamp = 0;
  // the 5-qubit tensor-core block plan of the program's gates, made when a
  // batch first runs the program as a lockstep row on blocks
  mutable std::once_flag tc_once;
  mutable bool tc_ok = false;
  mutable std::vector<TcBlock> tc_blocks;
  mutable std::vector<int32_t> tc_members;
};

// Capacity: TFQG_PROGRAM_CACHE_BYTES (default 1 GiB; a batch of 4096 random
// 20-qubit circuits of depth up to 40 takes about 500 MB) and 65536
// entries.  A batch larger than the cache would miss on every call (its
// programs evict one another in order).
std::atomic<size_t> g_pc_cap{0};  // 0: not read from the environment yet
size_t program_cache_bytes() {
  size_t v = g_pc_cap.load();
  if (v == 0) {
    const char* e = getenv("TFQG_PROGRAM_CACHE_BYTES");
    v = e && strtoull(e, nullptr, 10) > 0 ? size_t(strtoull(e, nullptr, 10)) : size_t(1) << 30;
    g_pc_cap.store(v);
  }
  return v;
}
constexpr size_t kProgramCacheEntries = 65536;
std::mutex g_pc_mu;
std::unordered_multimap<uint64_t, std::shared_ptr<const ProgramCacheEntry>> g_pc;
uint64_t g_pc_clock = 0;
size_t g_pc_bytes = 0;
std::atomic<int> g_pc_on{1};
std::atomic<int64_t> g_pc_hits{0}, g_pc_misses{0};

uint64_t program_cache_hash(const char* p, size_t n, const std::string& names, int job,
                            int plan_key) {
  uint64_t h = ProtoKeyHash()(ProtoKey{p, n, -1});
  h ^= ProtoKeyHash()(ProtoKey{names.data(), names.size(), job * 4096 + plan_key}) +
       0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
  return h;
}

std::shared_ptr<const ProgramCacheEntry> program_cache_find(const char* p, size_t n,
                                                            const std::string& names,
                                                            int job, int plan_key) {
  if (!g_pc_on.load()) return nullptr;
  const uint64_t h = program_cache_hash(p, n, names, job, plan_key);
  std::lock_guard<std::mutex> lk(g_pc_mu);
  auto range = g_pc.equal_range(h);
  for (auto it = range.first; it != range.second; ++it) {
    const ProgramCacheEntry& e = *it->second;
    if (e.job == job && e.plan_key == plan_key && e.bytes.size() == n && e.names == names &&
        memcmp(e.bytes.data(), p, n) == 0) {
      const_cast<ProgramCacheEntry&>(e).stamp = ++g_pc_clock;
      g_pc_hits.fetch_add(1);
      return it->second;
    }
  }
  g_pc_misses.fetch_add(1);
  return nullptr;
}

void program_cache_insert(std::shared_ptr<ProgramCacheEntry> e) {
  if (!g_pc_on.load()) return;
  const CompiledProgram& cp = e->cp;
  e->cost = e->bytes.size() + e->names.size() + cp.gates.size() * sizeof(GateTemplate) +
            (cp.fwd_ops.size() + cp.bwd_ops.size()) * sizeof(DevOp) +
            (cp.fwd_passes.size() + cp.bwd_passes.size()) * sizeof(DevPass) +
            e->index.size() * 48 + 256;
  const size_t cap = program_cache_bytes();
  if (e->cost > cap / 4) return;
  const uint64_t h = program_cache_hash(e->bytes.data(), e->bytes.size(), e->names, e->job,
                                        e->plan_key);
  std::lock_guard<std::mutex> lk(g_pc_mu);
  if (!g_pc.empty() &&
      (g_pc_bytes + e->cost > cap || g_pc.size() >= kProgramCacheEntries)) {
    // evict the least recently used eighth of the entries (at least enough
    // for the new one) in one pass
    std::vector<std::pair<uint64_t, decltype(g_pc)::iterator>> by_age;
    by_age.reserve(g_pc.size());
    for (auto it = g_pc.begin(); it != g_pc.end(); ++it) by_age.emplace_back(it->second->stamp, it);
    std::sort(by_age.begin(), by_age.end(),
              [](const auto& a, const auto& b) { return a.first < b.first; });
    const size_t quota = std::max<size_t>(1, by_age.size() / 8);
    size_t k = 0;
    for (; k < by_age.size() &&
           (k < quota || g_pc_bytes + e->cost > cap || g_pc.size() >= kProgramCacheEntries);
         ++k) {
      g_pc_bytes -= by_age[k].second->second->cost;
      g_pc.erase(by_age[k].second);
    }
  }
  e->stamp = ++g_pc_clock;
  g_pc_bytes += e->cost;
  g_pc.emplace(h, std::move(e));
}

void program_cache_clear() {
  std::lock_guard<std::mutex> lk(g_pc_mu);
  g_pc.clear();
  g_pc_bytes = 0;
}

// Parses/compiles every row.  Throws Error on invalid input.
// TFQG_KIND_INNER: `others` holds batch x num_others paired programs
// (tfq_inner_product's other_programs); they become rows batch + i *
// num_others + j, resolved with the qubit map of their reference row i.
// Runs f(i) for i in [0, n) on the host's cores (serially for small n).  f
// must not throw: callers keep one exception slot per index and rethrow the
// first one in index order, so errors surface as a serial loop would raise
// them.
template <class F>
void parallel_for(size_t n, F&& f) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t workers = std::min<size_t>({size_t(hw), size_t(32), n});
  if (n < 32 || workers <= 1) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  auto run = [&]() {
    for (size_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) f(i);
  };
  std::vector<std::thread> pool;
  pool.reserve(workers - 1);
  for (size_t w = 1; w < workers; ++w) pool.emplace_back(run);
  run();
  for (std::thread& t : pool) t.join();
}

void rethrow_first(const std::vector<std::exception_ptr>& errs) {
  for (const std::exception_ptr& e : errs)
    if (e) std::rethrow_exception(e);
}

// Lockstep schedule of the batch's lock rows: groups of rows whose states
// fit g_lock_arena_amps together; per group one item per row (its chunk
// prefix and arena offset), then per launch k the items of forward pass k of
// every row on tile passes that has one, then per launch m those of
// measurement pass m.  Rows on tensor-core blocks get their own item list
// (tcl_items), their blocks and, per block index, the units of a direct and
// a transposed launch.
void build_lock_schedule(
    tfqg_batch* b, const std::vector<std::shared_ptr<const ProgramCacheEntry>>& entries) {
  const size_t nr = b->lock_rows.size();
  auto prog = [&](int32_t row) -> const DevProgram& {
    return b->programs[b->rows[size_t(row)].program];
  };
  // block plans of the rows that take the tensor cores (planned on the
  // host's cores, once per cached program; a row without a plan stays on
  // tile passes)
  std::vector<std::vector<TcBlock>> tcb(nr);
  std::vector<std::vector<int32_t>> tcm(nr);
  std::vector<std::vector<TcUnit>> tmpl(nr);  // per block: targets, variant, geometry
  std::vector<uint8_t> tc(nr, 0), bad(nr, 0);
  parallel_for(nr, [&](size_t k) {
    const int32_t pid = b->rows[size_t(b->lock_rows[k])].program;
    const DevProgram& p = b->programs[size_t(pid)];
    if (!lock_tc_for(p.n)) return;
    try {
      const ProgramCacheEntry* e = size_t(pid) < entries.size() ? entries[pid].get() : nullptr;
      if (e) {
        std::call_once(e->tc_once, [e]() {
          e->tc_ok = plan_tc_blocks(e->cp.gates.data(), int(e->cp.gates.size()), e->cp.n,
                                    &e->tc_blocks, &e->tc_members) &&
                     !e->tc_blocks.empty();
        });
        if (e->tc_ok) {
          tcb[k] = e->tc_blocks;
          tcm[k] = e->tc_members;
          tc[k] = 1;
        }
      } else {
        tc[k] = plan_tc_blocks(b->gates.data() + p.gate_begin, p.num_gates, p.n, &tcb[k],
                               &tcm[k]) &&
                !tcb[k].empty();
      }
      if (tc[k]) {
        tmpl[k].resize(tcb[k].size());
        for (size_t q = 0; q < tcb[k].size(); ++q) {
          TcUnit& u = tmpl[k][q];
          u = TcUnit{};
          const int v = tc_unit_geometry(tcb[k][q], p.n, &u.tpack, &u.tr);
          if (v < 0) bad[k] = 1;
          if (v > 0) u.tpack |= kTcUnitTrans;
        }
      }
    } catch (...) {
      tc[k] = 0;
      tcb[k].clear();
      tcm[k].clear();
      tmpl[k].clear();
    }
  });
  for (size_t k = 0; k < nr; ++k)
    if (bad[k]) throw Error(kInternal, "tensor-core block outside its row's qubits");
  size_t i = 0;
  while (i < nr) {
    tfqg_batch::LockGroup g;
    size_t j = i;
    while (j < nr) {
      const int64_t a = int64_t(1) << prog(b->lock_rows[j]).n;
      // (a group's rows are one grid dimension of its padding launch)
      if (j > i && (g.arena_amps + a > g_lock_arena_amps.load() || j - i >= 65535)) break;
      g.arena_amps += a;
      ++j;
    }
    std::vector<int64_t> off(j - i);
    std::vector<int32_t> accb(j - i);
    g.rows.begin = int32_t(b->lock_items.size());
    int64_t o = 0, chunks = 0;
    for (size_t k = i; k < j; ++k) {
      const int32_t row = b->lock_rows[k];
      const DevRow& r = b->rows[size_t(row)];
      const int n = prog(row).n;
      off[k - i] = o;
      accb[k - i] = int32_t(g.acc_terms);
      if (r.meas_begin < r.meas_end)
        g.acc_terms += b->meas[r.meas_end - 1].end - b->meas[r.meas_begin].begin;
      b->lock_items.push_back(LockItem{row, 0u, chunks, o, n, accb[k - i]});
      o += int64_t(1) << n;
      chunks += int64_t(1) << (n - kLockChunkBits);
    }
    if (g.acc_terms > INT32_MAX) throw Error(kResourceExhausted, "too many measurement terms");
    g.rows.count = int32_t(j - i);
    g.rows.ntiles = chunks;
    uint32_t max_fwd = 0, max_meas = 0;
    for (size_t k = i; k < j; ++k) {
      const DevProgram& p = prog(b->lock_rows[k]);
      const DevRow& r = b->rows[size_t(b->lock_rows[k])];
      if (!tc[k]) max_fwd = std::max(max_fwd, p.fwd_pass_end - p.fwd_pass_begin);
      max_meas = std::max(max_meas, r.meas_end - r.meas_begin);
    }
    for (int meas = 0; meas < 2; ++meas) {
      const uint32_t launches = meas ? max_meas : max_fwd;
      for (uint32_t q = 0; q < launches; ++q) {
        tfqg_batch::LockLaunch L;
        L.begin = int32_t(b->lock_items.size());
        for (size_t k = i; k < j; ++k) {
          if (!meas && tc[k]) continue;
          const int32_t row = b->lock_rows[k];
          const DevProgram& p = prog(row);
          const DevRow& r = b->rows[size_t(row)];
          const uint32_t first = meas ? r.meas_begin : p.fwd_pass_begin;
          const uint32_t count = meas ? r.meas_end - r.meas_begin
                                      : p.fwd_pass_end - p.fwd_pass_begin;
          if (q >= count) continue;
          b->lock_items.push_back(
              LockItem{row, first + q, L.ntiles, off[k - i], p.n, accb[k - i]});
          L.ntiles += int64_t(1) << (p.n - kStreamTileBits);
        }
        L.count = int32_t(b->lock_items.size()) - L.begin;
        (meas ? g.meas : g.fwd).push_back(L);
      }
    }
    // the group's tensor-core rows
    g.tc_rows.begin = int32_t(b->tcl_items.size());
    g.tc_block_begin = int32_t(b->tcl_blocks.size());
    std::vector<int32_t> first_block(j - i, -1);
    size_t max_blocks = 0;
    int64_t tchunks = 0;
    for (size_t k = i; k < j; ++k) {
      if (!tc[k]) continue;
      const int32_t row = b->lock_rows[k];
      const int n = prog(row).n;
      b->tcl_items.push_back(LockItem{row, 0u, tchunks, off[k - i], n, 0});
      tchunks += int64_t(1) << (n - kLockChunkBits);
      first_block[k - i] = int32_t(b->tcl_blocks.size());
      const uint32_t mbase = uint32_t(b->tcl_members.size());
      for (TcBlock t : tcb[k]) {
        t.member_begin += mbase;
        t.member_end += mbase;
        b->tcl_blocks.push_back(t);
        b->tcl_block_rows.push_back(row);
      }
      b->tcl_members.insert(b->tcl_members.end(), tcm[k].begin(), tcm[k].end());
      max_blocks = std::max(max_blocks, tcb[k].size());
    }
    g.tc_rows.count = int32_t(b->tcl_items.size()) - g.tc_rows.begin;
    g.tc_rows.ntiles = tchunks;
    g.tc_block_count = int32_t(b->tcl_blocks.size()) - g.tc_block_begin;
    for (size_t q = 0; q < max_blocks; ++q)
      for (int trans = 0; trans < 2; ++trans) {
        tfqg_batch::TcLockLaunch L;
        L.begin = int32_t(b->tcl_units.size());
        L.trans = trans != 0;
        std::vector<std::pair<TcUnit, int64_t>> rows_in;  // unit template, chunks
        int64_t total = 0;
        for (size_t k = i; k < j; ++k) {
          if (!tc[k] || q >= tcb[k].size()) continue;
          if (((tmpl[k][q].tpack & kTcUnitTrans) != 0) != (trans != 0)) continue;
          const int32_t row = b->lock_rows[k];
          const int n = prog(row).n;
          TcUnit u = tmpl[k][q];
          u.tpack &= ~kTcUnitTrans;
          u.off = off[k - i];
          u.row = row;
          u.mat = uint32_t(first_block[k - i] - g.tc_block_begin) + uint32_t(q);
          const int64_t nch = int64_t(1) << (n - kTcBits - 7);
          rows_in.emplace_back(u, nch);
          total += nch;
        }
        // units of up to kTcUnitChunks chunks, fewer when the launch would
        // otherwise have too few units to spread over the GPU
        int64_t per = g_tc_unit_chunks.load();
        while (per > 1 && total / per < g_tc_unit_target.load()) per >>= 1;
        for (auto& ru : rows_in)
          for (int64_t c = 0; c < ru.second; c += per) {
            ru.first.chunk0 = c;
            ru.first.nchunks = int32_t(std::min<int64_t>(per, ru.second - c));
            b->tcl_units.push_back(ru.first);
          }
        L.count = int32_t(b->tcl_units.size()) - L.begin;
        if (L.count) g.tc.push_back(L);
      }
    // the persistent form's queue: block index, then row, then chunk; each
    // unit waits for its row's units of the earlier blocks
    g.tcp_begin = int32_t(b->tcl_punits.size());
    {
      std::vector<int32_t> row_units(j - i, 0), slot(j - i, 0);
      for (size_t k = i, sl = size_t(g.tc_rows.begin); k < j; ++k)
        if (tc[k]) slot[k - i] = int32_t(sl++);
      for (size_t q = 0; q < max_blocks; ++q) {
        // units of up to kTcUnitChunks chunks, fewer where the block index
        // has too few chunks over all rows to keep the GPU busy
        int64_t level = 0;
        for (size_t k = i; k < j; ++k)
          if (tc[k] && q < tcb[k].size()) level += int64_t(1) << (prog(b->lock_rows[k]).n - kTcBits - 7);
        int64_t per = g_tc_unit_chunks.load();
        while (per > 1 && level / per < g_tc_unit_target.load()) per >>= 1;
        for (size_t k = i; k < j; ++k) {
          if (!tc[k] || q >= tcb[k].size()) continue;
          const int32_t row = b->lock_rows[k];
          const int n = prog(row).n;
          TcUnit u = tmpl[k][q];
          u.off = off[k - i];
          u.row = row;
          u.mat = uint32_t(first_block[k - i] - g.tc_block_begin) + uint32_t(q);
          u.slot = slot[k - i];
          u.need = row_units[k - i];
          const int64_t nch = int64_t(1) << (n - kTcBits - 7);
          for (int64_t c = 0; c < nch; c += per) {
            u.chunk0 = c;
            u.nchunks = int32_t(std::min<int64_t>(per, nch - c));
            b->tcl_punits.push_back(u);
          }
          row_units[k - i] += int32_t((nch + per - 1) / per);
        }
      }
    }
    g.tcp_count = int32_t(b->tcl_punits.size()) - g.tcp_begin;
    b->lock_groups.push_back(std::move(g));
    i = j;
  }
}

void build_batch(tfqg_batch* b, const char* const* programs,
                 const int64_t* program_lens, int64_t batch,
                 const char* const* symbol_names, const int64_t* name_lens,
                 int64_t num_symbols, const char* const* pauli_sums,
                 const int64_t* psum_lens, int64_t num_ops, int kind,
                 const char* const* others = nullptr,
                 const int64_t* other_lens = nullptr, int64_t num_others = 0,
                 bool inner_grads = false) {
  if (batch < 0 || num_symbols < 0 || num_ops < 0 || num_others < 0)
    throw Error(kInvalidArgument, "negative dimension");
  if (num_ops > 65535)
    throw Error(kInvalidArgument, "at most 65535 pauli_sums columns are supported");
  const bool inner = kind == TFQG_KIND_INNER;
  const int64_t main_rows = batch;
  if (inner) {
    b->inner_rows = batch;
    b->inner_others = num_others;
    batch = batch + batch * num_others;
  }
  b->value_rows = main_rows;
  b->kind = kind;
  b->B = batch;
  b->P = num_symbols;
  b->n_ops = num_ops;
  // reference programs of an inner-product batch plan the adjoint sweep
  // when the batch will compute gradients; paired programs only run forward
  const JobKind job = (kind == TFQG_KIND_ADJOINT || (inner && inner_grads)) ? kJobAdjoint
                      : kind == TFQG_KIND_NOISY                           ? kJobNoisy
                                                                          : kJobForward;
  b->inner_grads = inner && inner_grads;

  // symbol names in column order: part of the compiled-program cache key
  std::string names_key;
  for (int64_t j = 0; j < num_symbols; ++j) {
    const uint64_t ln = uint64_t(name_lens[j]);
    names_key.append(reinterpret_cast<const char*>(&ln), sizeof(ln));
    names_key.append(symbol_names[j], size_t(name_lens[j]));
  }
  const bool fuse = g_gate_fusion.load() != 0;
  // the cache key of a plan: the fusion setting and the row-policy epoch
  const int plan_key = (fuse ? 1 : 0) | ((g_policy_epoch.load() & 2047) << 1);

  // 1. parse programs (ParsePrograms, parse_context.cc:174-206), deduplicated;
  // programs found in the compiled-program cache are not decoded
  std::unordered_map<ProtoKey, int, ProtoKeyHash> prog_ids;
  std::vector<ProgramP> parsed;
  std::vector<std::shared_ptr<const ProgramCacheEntry>> cached;
  std::vector<ProtoKey> src;
  std::vector<int> row_prog(static_cast<size_t>(batch));
  std::vector<int> pair_of;  // paired program -> its reference program
  for (int64_t i = 0; i < batch; ++i) {
    const bool paired = i >= main_rows;
    const int64_t k = i - main_rows;  // paired row (main row k / num_others)
    const char* data = paired ? others[k] : programs[i];
    const int64_t len = paired ? other_lens[k] : program_lens[i];
    // a paired program resolves through its reference program's qubits
    const ProtoKey key{data, size_t(len), paired ? row_prog[k / num_others] : -1};
    auto it = prog_ids.find(key);
    if (it != prog_ids.end()) {
      row_prog[i] = it->second;
      continue;
    }
    int id = int(parsed.size());
    parsed.emplace_back();
    cached.emplace_back();
    src.push_back(key);
    pair_of.push_back(paired ? row_prog[k / num_others] : -1);
    prog_ids.emplace(key, id);
    row_prog[i] = id;
  }
  // the distinct programs: cache lookups and decoding on the host's cores;
  // the first failing program in row order raises its error
  {
    std::vector<std::exception_ptr> errs(parsed.size());
    parallel_for(parsed.size(), [&](size_t pid) {
      try {
        if (!inner)
          cached[pid] = program_cache_find(src[pid].p, src[pid].n, names_key, int(job),
                                           plan_key);
        if (!cached[pid]) decode_program(src[pid].p, src[pid].n, &parsed[pid]);
      } catch (...) {
        errs[pid] = std::current_exception();
      }
    });
    rethrow_first(errs);
  }
  // 2. parse pauli sums (GetPauliSums, parse_context.cc:367-403)
  std::unordered_map<ProtoKey, int, ProtoKeyHash> psum_ids;
  std::vector<PauliSumP> psums;
  std::vector<int> row_psum(static_cast<size_t>(batch * num_ops));
  for (int64_t k = 0; k < batch * num_ops; ++k) {
    const ProtoKey key{pauli_sums[k], size_t(psum_lens[k]), -1};
    auto it = psum_ids.find(key);
    if (it != psum_ids.end()) {
      row_psum[k] = it->second;
      continue;
    }
    PauliSumP ps;
    decode_paulisum(pauli_sums[k], size_t(psum_lens[k]), &ps);
    int id = int(psums.size());
    psums.push_back(std::move(ps));
    psum_ids.emplace(key, id);
    row_psum[k] = id;
  }
  // 3. symbol map (GetSymbolMaps): name -> column, last column wins
  SymbolTable names;
  names.num_symbols = num_symbols;
  for (int64_t j = 0; j < num_symbols; ++j)
    names.col[make_key(symbol_names[j], name_lens[j])] = int(j);

  // 4. resolve + compile each distinct program; check pauli-sum qubits
  std::vector<CompiledProgram> compiled(parsed.size());
  std::vector<std::unordered_map<std::string, int>> index(parsed.size());
  std::vector<char> resolved(parsed.size(), 0);
  // qubit resolution errors surface per row in batch order, before
  // circuit-construction errors, like GetProgramsAndNumQubits; a paired
  // program uses its reference's map (checked right after that reference,
  // as ResolveQubitIds(program, num_qubits, other_programs) does) and is
  // empty when its reference is
  auto resolve_paired = [&](int64_t i) {
    for (int64_t j = 0; j < num_others; ++j) {
      const int pid = row_prog[main_rows + i * num_others + j];
      if (resolved[pid]) continue;
      const int mpid = pair_of[pid];
      if (parsed[mpid].moments.empty()) {
        parsed[pid].moments.clear();
      } else {
        check_paired_qubits(parsed[pid], index[mpid]);
        index[pid] = index[mpid];
      }
      resolved[pid] = 1;
    }
  };
  // outside inner-product batches every distinct program resolves on its
  // own: on the host's cores, errors raised below in row order
  std::vector<std::exception_ptr> resolve_errs(parsed.size());
  if (!inner) {
    parallel_for(parsed.size(), [&](size_t pid) {
      try {
        if (cached[pid]) {
          index[pid] = cached[pid]->index;
        } else {
          resolve_qubits(parsed[pid], &index[pid]);
        }
        resolved[pid] = 1;
      } catch (...) {
        resolve_errs[pid] = std::current_exception();
      }
    });
  }
  for (int64_t i = 0; i < batch; ++i) {
    int pid = row_prog[i];
    if (i >= main_rows) break;  // paired rows: resolved with their reference
    if (resolve_errs[pid]) std::rethrow_exception(resolve_errs[pid]);
    if (!resolved[pid]) {
      if (cached[pid]) index[pid] = cached[pid]->index;
      else resolve_qubits(parsed[pid], &index[pid]);
      resolved[pid] = 1;
    }
    if (inner) resolve_paired(i);
    const bool empty = cached[pid] ? cached[pid]->empty : parsed[pid].moments.empty();
    if (empty) continue;  // (#679) empty program
    for (int64_t j = 0; j < num_ops; ++j) {
      const PauliSumP& ps = psums[row_psum[i * num_ops + j]];
      for (const TermP& t : ps)
        for (const auto& pq : t.paulis)
          if (!index[pid].count(pq.first))
            throw Error(kInvalidArgument,
                        "Found a Pauli sum operating on qubits not found in "
                        "circuit.");
    }
  }
  // reference programs first (their errors come first), then the paired
  // ones, which may not hold symbols (tfq_inner_product.cc: any construction
  // error of an other_program reports the symbols message)
  const SymbolTable no_symbols;
  // compile and plan the programs that were not cached (on the host's cores
  // outside inner-product batches; the first error in program order raises)
  std::vector<std::exception_ptr> compile_errs(parsed.size());
  if (!inner) {
    parallel_for(parsed.size(), [&](size_t pid) {
      if (cached[pid]) return;
      try {
        compile_program(parsed[pid], names, job, &compiled[pid], &index[pid]);
        plan_program(&compiled[pid], job, fuse_for(compiled[pid].n, fuse));
      } catch (...) {
        compile_errs[pid] = std::current_exception();
      }
    });
    rethrow_first(compile_errs);
  }
  // every program's cache entry (found, or made now), which also keeps the
  // program's tensor-core block plan once made
  std::vector<std::shared_ptr<const ProgramCacheEntry>> entries(cached);
  for (size_t pid = 0; pid < parsed.size(); ++pid) {
    if (inner && pair_of[pid] >= 0) continue;
    if (cached[pid]) continue;
    if (inner) {
      compile_program(parsed[pid], names, job, &compiled[pid], &index[pid]);
      plan_program(&compiled[pid], job, fuse_for(compiled[pid].n, fuse));
    }
    if (!inner) {
      auto e = std::make_shared<ProgramCacheEntry>();
      e->bytes.assign(src[pid].p, src[pid].n);
      e->names = names_key;
      e->job = int(job);
      e->plan_key = plan_key;
      e->empty = parsed[pid].moments.empty();
      e->cp = compiled[pid];
      e->index = index[pid];
      entries[pid] = e;
      program_cache_insert(std::move(e));
    }
  }
  for (size_t pid = 0; pid < parsed.size() && inner; ++pid) {
    if (pair_of[pid] < 0) continue;
    try {
      compile_program(parsed[pid], no_symbols, kJobForward, &compiled[pid], &index[pid]);
    } catch (const Error&) {
      throw Error(kInvalidArgument,
                  "Found symbols in other_programs.No symbols are allowed in these circuits.");
    }
    plan_program(&compiled[pid], kJobForward, fuse_for(compiled[pid].n, fuse));
  }

  // 5. pack programs
  // (a cached program is packed straight from its cache entry): every
  // program's table offsets first, then the copies on the host's cores
  b->programs.resize(compiled.size());
  auto cp_of = [&](size_t pid) -> const CompiledProgram& {
    return cached[pid] ? cached[pid]->cp : compiled[pid];
  };
  struct PackAt {
    size_t grads, gates, channels, kraus, passes, ops;
  };
  std::vector<PackAt> at(compiled.size() + 1);
  at[0] = PackAt{b->grad_cols.size(), b->gates.size(), b->channels.size(), b->kraus.size(),
                 b->passes.size(), b->ops.size()};
  for (size_t pid = 0; pid < compiled.size(); ++pid) {
    const CompiledProgram& cp = cp_of(pid);
    size_t kr = 0;
    for (const ChannelHost& ch : cp.channels) kr += ch.kraus.size() / 2;
    at[pid + 1] = PackAt{at[pid].grads + cp.grad_col.size(), at[pid].gates + cp.gates.size(),
                         at[pid].channels + cp.channels.size(), at[pid].kraus + kr,
                         at[pid].passes + cp.fwd_passes.size() + cp.bwd_passes.size(),
                         at[pid].ops + cp.fwd_ops.size() + cp.bwd_ops.size()};
  }
  const PackAt& total = at[compiled.size()];
  if (total.gates > UINT32_MAX || total.ops > UINT32_MAX || total.passes > UINT32_MAX)
    throw Error(kResourceExhausted, "the batch's gate tables exceed 2^32 entries");
  b->grad_cols.resize(total.grads);
  b->gates.resize(total.gates);
  b->channels.resize(total.channels);
  b->kraus.resize(total.kraus);
  b->passes.resize(total.passes);
  b->ops.resize(total.ops);
  parallel_for(compiled.size(), [&](size_t pid) {
    const CompiledProgram& cp = cp_of(pid);
    const PackAt& o = at[pid];
    DevProgram& dp = b->programs[pid];
    memset(&dp, 0, sizeof(dp));
    dp.n = cp.empty() ? 0 : cp.n;
    dp.num_gates = int32_t(cp.gates.size());
    dp.num_grads = int32_t(cp.grad_col.size());
    dp.grad_col_begin = uint32_t(o.grads);
    std::copy(cp.grad_col.begin(), cp.grad_col.end(), b->grad_cols.begin() + o.grads);
    dp.gate_begin = uint32_t(o.gates);
    std::copy(cp.gates.begin(), cp.gates.end(), b->gates.begin() + o.gates);
    dp.channel_begin = uint32_t(o.channels);
    dp.num_channels = int32_t(cp.channels.size());
    size_t kr = o.kraus;
    for (size_t c = 0; c < cp.channels.size(); ++c) {
      const ChannelHost& ch = cp.channels[c];
      DevChannel d = ch.dev;
      d.kraus = uint32_t(kr / 4);
      for (size_t k = 0; k < ch.kraus.size(); k += 2)
        b->kraus[kr++] = make_float2(float(ch.kraus[k]), float(ch.kraus[k + 1]));
      b->channels[o.channels + c] = d;
    }
    dp.resident = cp.resident ? 1 : 0;
    size_t pass = o.passes;
    const uint32_t op_base = uint32_t(o.ops);
    dp.fwd_pass_begin = uint32_t(pass);
    for (DevPass ps : cp.fwd_passes) {
      ps.op_begin += op_base;
      ps.op_end += op_base;
      b->passes[pass++] = ps;
    }
    dp.fwd_pass_end = uint32_t(pass);
    std::copy(cp.fwd_ops.begin(), cp.fwd_ops.end(), b->ops.begin() + o.ops);
    const uint32_t bop_base = uint32_t(o.ops + cp.fwd_ops.size());
    dp.bwd_pass_begin = uint32_t(pass);
    for (DevPass ps : cp.bwd_passes) {
      ps.op_begin += bop_base;
      ps.op_end += bop_base;
      b->passes[pass++] = ps;
    }
    dp.bwd_pass_end = uint32_t(pass);
    std::copy(cp.bwd_ops.begin(), cp.bwd_ops.end(), b->ops.begin() + bop_base);
  });
  for (size_t pid = 0; pid < compiled.size(); ++pid) {
    const CompiledProgram& cp = cp_of(pid);
    const DevProgram& dp = b->programs[pid];
    if (dp.n > 0) {
      b->max_n = std::max(b->max_n, dp.n);
      if (cp.resident) b->max_resident_n = std::max(b->max_resident_n, dp.n);
      else {
        b->any_streamed = true;
        b->max_streamed_n = std::max(b->max_streamed_n, dp.n);
      }
      b->max_grads = std::max(b->max_grads, dp.num_grads);
    } else {
      // the reference sizes outputs by the resolved qubit count even for
      // programs that hold no gates
      b->max_n = std::max(b->max_n, cp.n);
    }
  }

  // 6. rows: matrices, terms (deduplicated per distinct pauli-sum row)
  b->rows.resize(size_t(batch));
  std::unordered_map<std::string, std::pair<uint32_t, uint32_t>> term_rows, meas_rows;
  int64_t mat = 0, dmat = 0;
  for (int64_t i = 0; i < batch; ++i) {
    DevRow& r = b->rows[i];
    memset(&r, 0, sizeof(r));
    const int pid = row_prog[i];
    r.program = pid;
    r.n = b->programs[pid].n;
    r.mat_offset = uint64_t(mat);
    r.dmat_offset = uint64_t(dmat);
    mat += b->programs[pid].num_gates;
    dmat += b->programs[pid].num_grads;
    if (r.n == 0 || num_ops == 0) {
      r.term_begin = r.term_end = uint32_t(b->terms.size());
      r.meas_begin = r.meas_end = uint32_t(b->meas.size());
      continue;
    }
    std::string key = std::to_string(pid) + ":";
    for (int64_t j = 0; j < num_ops; ++j)
      key += std::to_string(row_psum[i * num_ops + j]) + ",";
    auto it = term_rows.find(key);
    if (it != term_rows.end()) {
      r.term_begin = it->second.first;
      r.term_end = it->second.second;
      r.meas_begin = meas_rows[key].first;
      r.meas_end = meas_rows[key].second;
      continue;
    }
    r.term_begin = uint32_t(b->terms.size());
    for (int64_t j = 0; j < num_ops; ++j)
      lower_paulisum(psums[row_psum[i * num_ops + j]], index[pid], r.n, int(j),
                     &b->terms);
    r.term_end = uint32_t(b->terms.size());
    r.meas_begin = uint32_t(b->meas.size());
    plan_measurement(b->terms, r.term_begin, r.term_end, r.n,
                     b->programs[pid].resident != 0, &b->meas, &b->meas_terms);
    r.meas_end = uint32_t(b->meas.size());
    term_rows.emplace(key, std::make_pair(r.term_begin, r.term_end));
    meas_rows.emplace(key, std::make_pair(r.meas_begin, r.meas_end));
  }
  b->total_gates = mat;
  b->total_grads = dmat;
  for (const GateTemplate& g : b->gates) b->any_fused |= g.kind == GK_FUSED;
  // most expensive rows first (approximate longest-processing-time order)
  b->order.resize(size_t(batch));
  for (int64_t i = 0; i < batch; ++i) b->order[i] = int32_t(i);
  auto cost = [&](int32_t i) {
    const DevProgram& p = b->programs[b->rows[i].program];
    return double(p.num_gates + 1) * double(int64_t(1) << std::min(p.n, 40));
  };
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int32_t x, int32_t y) { return cost(x) > cost(y); });
  if (inner)  // reference rows first: the gradient's adjoint runs only them
    std::stable_partition(b->order.begin(), b->order.end(),
                          [&](int32_t r) { return r < main_rows; });
  // wide rows: the whole grid simulates them one by one.  Rows of at least
  // wide_min qubits always.  A row of kWideFewQubits..wide_min-1 qubits
  // too when the batch streams few rows: in the queue R streamed rows run
  // side by side, one CTA each, while a wide pass keeps 2^(n-13) tiles
  // busy, and its adjoint passes run the interpreter (about 2x slower than
  // the queue's specialized module): the whole grid wins when
  // R <= 2^(n-14) (and R < kWideFewRows)
  const int wide_min = std::max(wide_min_qubits(), kStreamTileBits + 2);
  int64_t streamed_rows = 0;
  for (int64_t i = 0; i < batch; ++i) {
    const DevProgram& p = b->programs[b->rows[i].program];
    if (p.n > 0 && !p.resident && p.fwd_pass_begin != p.fwd_pass_end) ++streamed_rows;
  }
  const bool few = streamed_rows < g_wide_few_rows.load() && !inner;
  auto is_wide = [&](const DevProgram& p) {
    if (p.resident || p.fwd_pass_begin == p.fwd_pass_end) return false;
    if (p.n >= wide_min) return true;
    return few && p.n >= kWideFewQubits &&
           streamed_rows <= (int64_t(1) << std::min(p.n - kStreamTileBits - 1, 40));
  };
  for (const int32_t i : b->order) {
    const DevProgram& p = b->programs[b->rows[i].program];
    if (is_wide(p)) continue;
    b->order_fwd.push_back(i);
    if (p.n > 0 && !p.resident) {
      b->any_streamed_fwd = true;
      b->max_streamed_n_fwd = std::max(b->max_streamed_n_fwd, int(p.n));
    }
  }
  for (int64_t i = 0; i < batch; ++i) {
    const DevProgram& p = b->programs[b->rows[i].program];
    if (!is_wide(p)) continue;
    b->wide_rows.push_back(int32_t(i));
    b->max_wide_n = std::max(b->max_wide_n, int(p.n));
  }
  // lockstep rows: streamed rows of lock_min..21 qubits that are not wide.
  // In the queue each would stream through one CTA's slot (one SM for the
  // whole circuit); in lockstep every launch keeps the tiles of all of them
  // in flight over the whole grid.
  const int lock_min = std::max(g_lock_min_qubits.load(), kStreamTileBits + 1);
  auto is_lock = [&](const DevProgram& p) {
    if (inner || is_wide(p) || p.resident || p.num_channels != 0 ||
        p.fwd_pass_begin == p.fwd_pass_end || p.n < kStreamTileBits + 1)
      return false;
    const int pol = p.n < kPolicyMaxQubits ? g_lock_by_n[p.n].load() : -1;
    return pol < 0 ? p.n >= lock_min : pol != 0;
  };
  for (const int32_t i : b->order) {
    const DevProgram& p = b->programs[b->rows[i].program];
    if (is_wide(p)) continue;
    if (is_lock(p)) {
      b->lock_rows.push_back(i);
      continue;
    }
    b->order_lock.push_back(i);
    if (p.n > 0 && !p.resident) {
      b->any_streamed_lock = true;
      b->max_streamed_n_lock = std::max(b->max_streamed_n_lock, int(p.n));
    }
  }
  build_lock_schedule(b, entries);
  jit_assign_signatures(b);
  if (b->max_grads > 6144)
    throw Error(kResourceExhausted,
                "A circuit has more than 6144 symbolic gate parameters; the "
                "adjoint kernel keeps one accumulator per parameter in shared "
                "memory.");
}

template <class T>
size_t put(std::vector<unsigned char>* blob, const std::vector<T>& v) {
  size_t off = align256(blob->size());
  blob->resize(off + std::max<size_t>(v.size() * sizeof(T), 1));
  if (!v.empty()) memcpy(blob->data() + off, v.data(), v.size() * sizeof(T));
  return off;
}

void ensure_device(tfqg_batch* b, cudaStream_t s) {
  int dev;
  TFQG_CUDA(cudaGetDevice(&dev));
  if (b->device == dev && b->tables.p) return;
  std::vector<unsigned char> blob;
  TableOffsets o = pack_tables(b, &blob);
  b->tables.reserve(blob.size(), dev);
  TFQG_CUDA(cudaMemcpyAsync(b->tables.p, blob.data(), blob.size(),
                            cudaMemcpyHostToDevice, s));
  TFQG_CUDA(cudaStreamSynchronize(s));  // blob is a temporary
  b->bd = table_view(b, static_cast<unsigned char*>(b->tables.p), o);
  b->d_order_fwd = reinterpret_cast<const int32_t*>(
      static_cast<unsigned char*>(b->tables.p) + o.order_fwd);
  b->d_order_lock = reinterpret_cast<const int32_t*>(
      static_cast<unsigned char*>(b->tables.p) + o.order_lock);
  b->d_lock_items = reinterpret_cast<const LockItem*>(
      static_cast<unsigned char*>(b->tables.p) + o.lock_items);
  b->device = dev;
}

}  // namespace

TableOffsets tfqg::pack_tables(const tfqg_batch* b, std::vector<unsigned char>* blob) {
  TableOffsets o;
  o.prog = put(blob, b->programs);
  o.rows = put(blob, b->rows);
  o.gates = put(blob, b->gates);
  o.pass = put(blob, b->passes);
  o.ops = put(blob, b->ops);
  o.terms = put(blob, b->terms);
  o.chan = put(blob, b->channels);
  o.kraus = put(blob, b->kraus);
  o.gc = put(blob, b->grad_cols);
  o.order = put(blob, b->order);
  o.order_fwd = put(blob, b->order_fwd);
  o.order_lock = put(blob, b->order_lock);
  o.lock_items = put(blob, b->lock_items);
  o.meas = put(blob, b->meas);
  o.mterms = put(blob, b->meas_terms);
  blob->resize(align256(blob->size()));
  return o;
}

BatchDevice tfqg::table_view(const tfqg_batch* b, unsigned char* base,
                             const TableOffsets& o) {
  BatchDevice d;
  d.programs = reinterpret_cast<const DevProgram*>(base + o.prog);
  d.rows = reinterpret_cast<const DevRow*>(base + o.rows);
  d.gates = reinterpret_cast<const GateTemplate*>(base + o.gates);
  d.passes = reinterpret_cast<const DevPass*>(base + o.pass);
  d.ops = reinterpret_cast<const DevOp*>(base + o.ops);
  d.terms = reinterpret_cast<const DevTerm*>(base + o.terms);
  d.channels = reinterpret_cast<const DevChannel*>(base + o.chan);
  d.kraus = reinterpret_cast<const float2*>(base + o.kraus);
  d.grad_cols = reinterpret_cast<const int32_t*>(base + o.gc);
  d.order = reinterpret_cast<const int32_t*>(base + o.order);
  d.meas = reinterpret_cast<const DevMeas*>(base + o.meas);
  d.meas_terms = reinterpret_cast<const DevMeasTerm*>(base + o.mterms);
  d.num_rows = int32_t(b->B);
  d.num_queue = int32_t(b->B);
  d.num_ops = int32_t(b->n_ops);
  d.num_symbols = int32_t(b->P);
  d.max_n = b->max_n;
  d.total_gates = b->total_gates;
  d.total_grads = b->total_grads;
  d.any_fused = b->any_fused ? 1 : 0;
  return d;
}

namespace {

// Common preamble: device tables, symbol values on the device, matrices.
const float* prepare(tfqg_batch* b, const float* values, int device_buffers,
                     bool grads, int grad_rule, cudaStream_t s, RunArgs* a) {
  ensure_device(b, s);
  const float* dvals = values;
  size_t vbytes = size_t(b->value_rows * b->P) * sizeof(float);
  if (!device_buffers && vbytes) {
    b->values.reserve(vbytes, b->device);
    TFQG_CUDA(cudaMemcpyAsync(b->values.p, values, vbytes,
                              cudaMemcpyHostToDevice, s));
    dvals = static_cast<const float*>(b->values.p);
  }
  a->values = dvals;
  b->mats.reserve(size_t(b->total_gates) * 16 * sizeof(float2), b->device);
  a->mats = static_cast<float2*>(b->mats.p);
  if (grads) {
    b->dmats.reserve(size_t(b->total_grads) * 16 * sizeof(float2), b->device);
    a->dmats = static_cast<float2*>(b->dmats.p);
  }
  a->grad_rule = grad_rule;
  b->counter.reserve(sizeof(int), b->device);
  a->counter = static_cast<int*>(b->counter.p);
  TFQG_CUDA(launch_build_matrices(b->bd, *a, grads, s));
  return dvals;
}

// Grid of a kernel with `threads` per CTA: resident CTAs per SM x SMs.
int occupancy_grid(const void* k, int threads, size_t smem, int dev) {
  int sms = 0, per_sm = 0;
  TFQG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  TFQG_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  TFQG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem));
  return sms * std::max(per_sm, 1);
}

// Plans the tensor-core blocks of every wide row once per batch and uploads
// them (blocks, then members) into b->tc_tab.
void tc_prepare(tfqg_batch* b, cudaStream_t s) {
  if (b->tc_planned && b->tc_tab.device == b->device) return;
  b->tc_blocks.clear();
  b->tc_members.clear();
  b->tc_rows.clear();
  for (const int32_t row : b->wide_rows) {
    const DevProgram& p = b->programs[b->rows[size_t(row)].program];
    const int32_t first = int32_t(b->tc_blocks.size());
    // channels are not gates: a noisy program keeps its tile passes
    const bool ok = p.num_channels == 0 &&
                    plan_tc_blocks(b->gates.data() + p.gate_begin, p.num_gates, p.n,
                                   &b->tc_blocks, &b->tc_members);
    b->tc_rows.emplace_back(first, ok ? int32_t(b->tc_blocks.size()) - first : -1);
  }
  b->tc_ran.assign(b->wide_rows.size(), 0);
  b->tc_sweeps.assign(b->wide_rows.size(), 0);
  const size_t bb = b->tc_blocks.size() * sizeof(TcBlock);
  const size_t mb = b->tc_members.size() * sizeof(int32_t);
  b->tc_tab.reserve(align256(bb) + mb + 256, b->device);
  unsigned char* base = static_cast<unsigned char*>(b->tc_tab.p);
  if (bb) TFQG_CUDA(cudaMemcpyAsync(base, b->tc_blocks.data(), bb, cudaMemcpyHostToDevice, s));
  if (mb)
    TFQG_CUDA(cudaMemcpyAsync(base + align256(bb), b->tc_members.data(), mb,
                              cudaMemcpyHostToDevice, s));
  b->tc_mats.reserve(std::max<size_t>(b->tc_blocks.size(), 1) * 1024 * sizeof(float2),
                     b->device);
  b->tc_status.reserve(sizeof(int), b->device);
  TFQG_CUDA(cudaMemsetAsync(b->tc_status.p, 0, sizeof(int), s));
  b->tc_planned = true;
}

// Grid of the tensor-core block kernel: two CTAs per SM x SMs.  Two fit:
// 2 x (96 KiB of operands + 1 KiB reserved) of the 228 KiB of shared memory
// (carveout at its maximum), 2 x 128 threads x 208 registers of 64 Ki, and
// 2 x 64 TMEM columns of 512.  The occupancy query reports one on GB300
// (ncu reports the shared-memory and register limits as two), and with one
// CTA per SM the kernel stalls on its gathers.  Chunks are grid-strided, so
// a grid above the resident CTAs stays correct.
int tc_grid(int dev) {
  const void* k = tc_apply5_kernel_ptr();
  TFQG_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int sms = 0;
  TFQG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  return std::max(occupancy_grid(k, 128, tc_apply5_smem_bytes(), dev), 2 * sms);
}

// After the tensor-core rows of a call: a block kernel whose MMA completion
// wait timed out has left its row partly transformed, so the call fails
// (INTERNAL) instead of returning that row's results.  Reading the status
// word synchronizes the stream; calls with tensor-core rows (24 qubits and
// more, milliseconds of device work each) are synchronous for that reason.
void check_tc_status(tfqg_batch* b, cudaStream_t s) {
  int v = 0;
  TFQG_CUDA(cudaMemcpyAsync(&v, b->tc_status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  TFQG_CUDA(cudaStreamSynchronize(s));
  if (g_tc_status_injected.load() == 1) v = 1;
  if (v != 0)
    throw Error(kInternal,
                "tensor-core block kernel: an MMA completion wait timed out; the wide "
                "row's state is incomplete and the call's results were discarded");
}

// The forward passes of wide row `row` (the k-th wide row) as tensor-core
// blocks: fused matrices, |0...0>, one launch per block.  False when the row
// has no block plan (a gate on more than 5 bits).
bool run_wide_tc(tfqg_batch* b, const BatchDevice& bd, const RunArgs* a, size_t k, int row,
                 float2* psi, int sms, cudaStream_t s) {
  const std::pair<int32_t, int32_t> rp = b->tc_rows[k];
  b->tc_ran[k] = 0;
  if (rp.second < 0) return false;
  const int n = b->programs[b->rows[size_t(row)].program].n;
  if (g_tc_gates.load() == 2 && n < kTcAutoMinQubits) return false;
  b->tc_ran[k] = 1;
  unsigned char* base = static_cast<unsigned char*>(b->tc_tab.p);
  const TcBlock* dblocks = reinterpret_cast<const TcBlock*>(base) + rp.first;
  const int32_t* dmembers = reinterpret_cast<const int32_t*>(
      base + align256(b->tc_blocks.size() * sizeof(TcBlock)));
  float2* U = static_cast<float2*>(b->tc_mats.p) + int64_t(rp.first) * 1024;
  TFQG_CUDA(launch_tc_fuse(bd, a->mats, row, dblocks, dmembers, rp.second, U, s));
  TFQG_CUDA(launch_fill(psi, int64_t(1) << n, make_float2(1.f, 0.f), make_float2(0.f, 0.f),
                        sms * 4, s));
  const int grid = tc_grid(b->device);
  int* st = static_cast<int*>(b->tc_status.p);
  const bool pair = g_tc_sweep.load() != 0;
  int sweeps = 0;
  for (int i = 0; i < rp.second; ++sweeps) {
    const TcBlock& b0 = b->tc_blocks[size_t(rp.first + i)];
    TcSweep geo;
    if (pair && i + 1 < rp.second &&
        tc_sweep_geometry(b0, b->tc_blocks[size_t(rp.first + i + 1)], n, &geo)) {
      // two blocks in one sweep: one CTA per SM
      TFQG_CUDA(launch_tc_sweep2(psi, n, U + int64_t(i) * 1024, U + int64_t(i + 1) * 1024, b0,
                                 b->tc_blocks[size_t(rp.first + i + 1)], st, sms, s));
      i += 2;
    } else {
      TFQG_CUDA(launch_tc_apply5(psi, n, U + int64_t(i) * 1024, b0, st, grid, s));
      i += 1;
    }
  }
  b->tc_sweeps[k] = sweeps;
  return true;
}

// Forward-mode work of the wide rows, one row after another on stream s:
// every pass of a row is one launch over all SMs, then the row's
// measurement, state padding or sampling.
void run_wide(tfqg_batch* b, int mode, const BatchDevice& bd, RunArgs* a,
              cudaStream_t s) {
  const int dev = b->device;
  const int state_amps = 1 << kStreamTileBits;
  const size_t smem = sim_smem_bytes(kModeState, -1, true, 0);
  cudaKernel_t jk = jit_kernel(b, kJitWide, dev);
  int grid = jk ? jit_grid(jk, smem, dev, kWideThreads)
                : occupancy_grid(sim_kernel_wide(), kWideThreads, smem, dev);
  const int mgrid = occupancy_grid(wide_measure_kernel_ptr(), kWideThreads, smem, dev);
  int sms = 0;
  TFQG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const bool tc = g_tc_gates.load() != 0;
  if (tc) {
    tc_prepare(b, s);
    // each call starts with a clear status word
    TFQG_CUDA(cudaMemsetAsync(b->tc_status.p, 0, sizeof(int), s));
  } else if (b->tc_planned) {
    b->tc_ran.assign(b->wide_rows.size(), 0);
  }
  bool any_tc = false;
  for (size_t wk = 0; wk < b->wide_rows.size(); ++wk) {
    const int32_t row = b->wide_rows[wk];
    const DevRow& r = b->rows[size_t(row)];
    const DevProgram& p = b->programs[r.program];
    const int n = p.n;
    float2* psi;
    if (mode == kModeState) {
      psi = a->out_state + (int64_t(row) << b->max_n);
    } else {
      b->wide_state.reserve((size_t(1) << b->max_wide_n) * sizeof(float2), dev);
      psi = static_cast<float2*>(b->wide_state.p);
    }
    const bool tc_done = tc && run_wide_tc(b, bd, a, wk, row, psi, sms, s);
    any_tc = any_tc || tc_done;
    for (uint32_t q = p.fwd_pass_begin; q < p.fwd_pass_end && !tc_done; ++q) {
      const int init = q == p.fwd_pass_begin ? 1 : 0;
      if (jk) {
        cudaError_t e = jit_launch_wide(jk, bd, *a, row, int(q), init, psi, grid, smem,
                                        state_amps, s);
        if (e == cudaSuccess) continue;
        // a rejected launch (nothing ran): interpreter from here on
        cudaGetLastError();
        b->jit_error = std::string("specialized launch rejected: ") + cudaGetErrorString(e);
        b->jit_mode = -1;
        jk = nullptr;
        grid = occupancy_grid(sim_kernel_wide(), kWideThreads, smem, dev);
      }
      TFQG_CUDA(sim_launch_wide(bd, *a, row, int(q), init, psi, grid, smem, state_amps, s));
    }
    if (mode == kModeExpect) {
      int term0 = 0, term1 = 0;
      if (r.meas_begin != r.meas_end) {
        term0 = int(b->meas[r.meas_begin].begin);
        term1 = int(b->meas[r.meas_end - 1].end);
      }
      const size_t nacc = 2 * size_t(term1 - term0);
      b->wide_acc.reserve((nacc + size_t(b->n_ops)) * sizeof(double), dev);
      double* wacc = static_cast<double*>(b->wide_acc.p);
      if (nacc) TFQG_CUDA(cudaMemsetAsync(wacc, 0, nacc * sizeof(double), s));
      for (uint32_t mp = r.meas_begin; mp < r.meas_end; ++mp)
        TFQG_CUDA(launch_wide_measure(bd, *a, row, int(mp), psi, wacc, term0, mgrid, smem,
                                      state_amps, s));
      TFQG_CUDA(launch_wide_expect_finalize(bd, *a, row, wacc, term0, wacc + nacc, s));
    } else if (mode == kModeState) {
      const int64_t N = int64_t(1) << n, M = int64_t(1) << b->max_n;
      const float2 pad = make_float2(-2.f, 0.f);
      TFQG_CUDA(launch_fill(psi + N, M - N, pad, pad, sms * 4, s));
    } else {
      const size_t nch = size_t(1) << (n - kStreamTileBits);
      b->wide_acc.reserve(nch * sizeof(double), dev);
      double* csum = static_cast<double*>(b->wide_acc.p);
      TFQG_CUDA(launch_wide_chunk_sums(psi, n, csum, sms * 4, s));
      TFQG_CUDA(launch_wide_sample(bd, *a, row, psi, n, csum, s));
    }
  }
  if (any_tc) check_tc_status(b, s);
}

// Adjoint of the wide rows, one row after another on stream s: forward
// passes over the whole grid, lambda by measurement passes, backward passes
// whose CTAs add gradient-slot sums into a per-row double buffer, finalize.
void run_wide_adjoint(tfqg_batch* b, const BatchDevice& bd, RunArgs* a, cudaStream_t s) {
  const int dev = b->device;
  const int state_amps = 1 << kStreamTileBits;
  const size_t fsmem = sim_smem_bytes(kModeState, -1, true, 0);
  const size_t asmem = sim_smem_bytes(kModeAdjoint, -1, true, b->max_grads);
  if (asmem > 227 * 1024)
    throw Error(kResourceExhausted, "shared memory request too large");
  cudaKernel_t jk = jit_kernel(b, kJitWide, dev);
  int fgrid = jk ? jit_grid(jk, fsmem, dev, kWideThreads)
                 : occupancy_grid(sim_kernel_wide(), kWideThreads, fsmem, dev);
  const int lgrid = occupancy_grid(sim_kernel_wide_lambda(), kSimThreads, asmem, dev);
  const int bgrid = occupancy_grid(sim_kernel_wide_backward(), kSimThreads, asmem, dev);
  const size_t N = size_t(1) << b->max_wide_n;
  b->wide_state.reserve(2 * N * sizeof(float2), dev);
  float2* psi = static_cast<float2*>(b->wide_state.p);
  float2* lam = psi + N;
  b->wide_acc.reserve(size_t(std::max(b->max_grads, 1)) * sizeof(double), dev);
  double* gacc = static_cast<double*>(b->wide_acc.p);
  for (const int32_t row : b->wide_rows) {
    const DevRow& r = b->rows[size_t(row)];
    const DevProgram& p = b->programs[r.program];
    for (uint32_t q = p.fwd_pass_begin; q < p.fwd_pass_end; ++q) {
      const int init = q == p.fwd_pass_begin ? 1 : 0;
      if (jk) {
        cudaError_t e = jit_launch_wide(jk, bd, *a, row, int(q), init, psi, fgrid, fsmem,
                                        state_amps, s);
        if (e == cudaSuccess) continue;
        cudaGetLastError();
        b->jit_error = std::string("specialized launch rejected: ") + cudaGetErrorString(e);
        b->jit_mode = -1;
        jk = nullptr;
        fgrid = occupancy_grid(sim_kernel_wide(), kWideThreads, fsmem, dev);
      }
      TFQG_CUDA(sim_launch_wide(bd, *a, row, int(q), init, psi, fgrid, fsmem, state_amps, s));
    }
    if (r.meas_begin == r.meas_end)
      TFQG_CUDA(cudaMemsetAsync(lam, 0, (size_t(1) << p.n) * sizeof(float2), s));
    for (uint32_t mp = r.meas_begin; mp < r.meas_end; ++mp)
      TFQG_CUDA(sim_launch_wide_lambda(bd, *a, row, int(mp), mp == r.meas_begin ? 1 : 0,
                                       psi, lam, lgrid, asmem, state_amps, s));
    if (p.num_grads == 0) continue;
    TFQG_CUDA(cudaMemsetAsync(gacc, 0, size_t(p.num_grads) * sizeof(double), s));
    for (uint32_t q = p.bwd_pass_begin; q < p.bwd_pass_end; ++q)
      TFQG_CUDA(sim_launch_wide_backward(bd, *a, row, int(q), psi, lam, gacc, bgrid, asmem,
                                         state_amps, s));
    TFQG_CUDA(launch_wide_grad_finalize(bd, *a, row, gacc, s));
  }
}

// The tensor-core tables of the lockstep rows as one blob (items, blocks,
// members, block rows, then the units of the persistent form or of the
// per-block-index launches) and the sections' offsets.
struct TclOffsets {
  size_t items, blocks, members, rows, units;
};
TclOffsets tcl_blob(const tfqg_batch* b, bool persistent, std::vector<unsigned char>* blob) {
  TclOffsets o;
  o.items = put(blob, b->tcl_items);
  o.blocks = put(blob, b->tcl_blocks);
  o.members = put(blob, b->tcl_members);
  o.rows = put(blob, b->tcl_block_rows);
  o.units = put(blob, persistent ? b->tcl_punits : b->tcl_units);
  blob->resize(align256(blob->size()));
  return o;
}

// Uploads the tensor-core tables of the lockstep rows for the form in use,
// once per device and form, and sizes their fused-matrix buffer.
void tcl_prepare(tfqg_batch* b, bool persistent, cudaStream_t s) {
  if (b->tcl_tab.p && b->tcl_tab.device == b->device && b->tcl_persistent == persistent)
    return;
  std::vector<unsigned char> blob;
  const TclOffsets o = tcl_blob(b, persistent, &blob);
  b->tcl_tab.reserve(blob.size(), b->device);
  unsigned char* base = static_cast<unsigned char*>(b->tcl_tab.p);
  TFQG_CUDA(cudaMemcpyAsync(base, blob.data(), blob.size(), cudaMemcpyHostToDevice, s));
  TFQG_CUDA(cudaStreamSynchronize(s));  // blob is a temporary
  b->tcl_persistent = persistent;
  b->d_tcl_items = reinterpret_cast<const LockItem*>(base + o.items);
  b->d_tcl_blocks = reinterpret_cast<const TcBlock*>(base + o.blocks);
  b->d_tcl_members = reinterpret_cast<const int32_t*>(base + o.members);
  b->d_tcl_block_rows = reinterpret_cast<const int32_t*>(base + o.rows);
  b->d_tcl_units = reinterpret_cast<const TcUnit*>(base + o.units);
  // persistent form: a queue counter per group, then a count per row
  b->tcl_sync.reserve((b->lock_groups.size() + b->tcl_items.size()) * sizeof(int), b->device);
  // B operands of one group at a time (groups run one after another)
  size_t group_blocks = 1;
  for (const auto& g : b->lock_groups) group_blocks = std::max(group_blocks, size_t(g.tc_block_count));
  b->tcl_mats.reserve(group_blocks * tc_b_floats() * sizeof(float), b->device);
  b->tc_status.reserve(sizeof(int), b->device);
}

// Forward-mode work of the lockstep rows, group after group on stream s:
// the group's tensor-core rows (fused block matrices, |0...0>, one launch
// per block index and variant), one launch per forward pass index over its
// rows on tile passes, then the group's measurement, state padding or
// sampling.  A captured call cannot read the tensor-core status word back,
// so there the rows' results are replaced by markers on a timeout.
void run_lock(tfqg_batch* b, int mode, const BatchDevice& bd, RunArgs* a, cudaStream_t s) {
  const int dev = b->device;
  const int state_amps = 1 << kStreamTileBits;
  const size_t smem = sim_smem_bytes(kModeState, -1, true, 0);
  const int grid = occupancy_grid(sim_kernel_lock(), kWideThreads, smem, dev);
  const int mgrid = occupancy_grid(lock_measure_kernel_ptr(), kWideThreads, smem, dev);
  int sms = 0;
  TFQG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int64_t arena = 0, chunks = 0;
  int32_t rows = 0;
  for (const auto& g : b->lock_groups) {
    arena = std::max(arena, g.arena_amps);
    chunks = std::max(chunks, g.rows.ntiles);
    rows = std::max(rows, g.rows.count);
  }
  float2* state = nullptr;
  if (mode != kModeState) {
    b->lock_state.reserve(size_t(arena) * sizeof(float2), dev);
    state = static_cast<float2*>(b->lock_state.p);
  }
  double* acc = nullptr;
  size_t nwacc = 0;  // term accumulators of the largest group (2 per term and row)
  for (const auto& g : b->lock_groups) nwacc = std::max(nwacc, 2 * size_t(g.acc_terms));
  if (mode == kModeExpect) {
    b->lock_acc.reserve((nwacc + size_t(rows) * size_t(std::max<int64_t>(b->n_ops, 1))) *
                            sizeof(double),
                        dev);
    acc = static_cast<double*>(b->lock_acc.p);
  } else if (mode == kModeSample) {
    b->lock_acc.reserve(size_t(chunks) * sizeof(double), dev);
    acc = static_cast<double*>(b->lock_acc.p);
  }
  const LockItem* items = b->d_lock_items;
  const bool any_tc = !b->tcl_units.empty();
  bool capturing = false;
  int* st = nullptr;
  float* Bops = nullptr;
  int tgrid = 0;
  const bool persistent = any_tc && g_tc_lock_persistent.load() != 0;
  if (any_tc) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    TFQG_CUDA(cudaStreamIsCapturing(s, &cs));
    capturing = cs != cudaStreamCaptureStatusNone;
    tcl_prepare(b, persistent, s);
    st = static_cast<int*>(b->tc_status.p);
    TFQG_CUDA(cudaMemsetAsync(st, 0, sizeof(int), s));
    Bops = static_cast<float*>(b->tcl_mats.p);
    tgrid = tc_grid(dev);
  }
  int* queues = persistent ? static_cast<int*>(b->tcl_sync.p) : nullptr;
  int* done = persistent ? queues + b->lock_groups.size() : nullptr;
  if (persistent)
    TFQG_CUDA(cudaMemsetAsync(queues, 0,
                              (b->lock_groups.size() + b->tcl_items.size()) * sizeof(int), s));
  size_t gi = 0;
  // tensor-core rows write their states in place: the arena, or the output
  // rows of a state call
  float2* tc_state = mode == kModeState ? a->out_state : state;
  const int row_shift = mode == kModeState ? b->max_n : -1;
  for (const auto& g : b->lock_groups) {
    if (g.tc_rows.count) {
      TFQG_CUDA(launch_tc_fuse_b(bd, a->mats, b->d_tcl_block_rows + g.tc_block_begin,
                                 b->d_tcl_blocks + g.tc_block_begin, b->d_tcl_members,
                                 g.tc_block_count,
                                 Bops, s));
      TFQG_CUDA(launch_lock_zero(tc_state, row_shift, b->d_tcl_items + g.tc_rows.begin,
                                 g.tc_rows.count, g.tc_rows.ntiles, sms * 8, s));
      if (persistent)
        TFQG_CUDA(launch_tc_lock_persistent(tc_state, row_shift, Bops,
                                            b->d_tcl_units + g.tcp_begin, g.tcp_count,
                                            queues + gi, done, st, tgrid, s));
      else
        for (const auto& L : g.tc)
          TFQG_CUDA(launch_tc_apply5_units(tc_state, row_shift, Bops, b->d_tcl_units + L.begin,
                                           L.count, L.trans, st, tgrid, s));
      // test hook: a captured call records an injected status on the
      // device, where a timed-out kernel would have set it
      if (capturing && g_tc_status_injected.load() != 0)
        TFQG_CUDA(cudaMemsetAsync(st, 1, 1, s));
    }
    for (size_t k = 0; k < g.fwd.size(); ++k)
      TFQG_CUDA(sim_launch_lock(bd, *a, items + g.fwd[k].begin, g.fwd[k].count,
                                g.fwd[k].ntiles, state, k == 0 ? 1 : 0,
                                mode == kModeState ? 1 : 0, grid, smem, state_amps, s));
    const LockItem* rws = items + g.rows.begin;
    if (mode == kModeExpect) {
      if (g.acc_terms)
        TFQG_CUDA(cudaMemsetAsync(acc, 0, 2 * size_t(g.acc_terms) * sizeof(double), s));
      for (const auto& L : g.meas)
        TFQG_CUDA(launch_lock_measure(bd, *a, items + L.begin, L.count, L.ntiles, state, acc,
                                      mgrid, smem, state_amps, s));
      TFQG_CUDA(launch_lock_expect_finalize(bd, *a, rws, g.rows.count, acc, acc + nwacc, s));
    } else if (mode == kModeState) {
      TFQG_CUDA(launch_lock_pad(bd, *a, rws, g.rows.count, s));
    } else {
      TFQG_CUDA(launch_lock_chunk_sums(rws, g.rows.count, g.rows.ntiles, state, acc, sms * 4,
                                       s));
      TFQG_CUDA(launch_lock_sample(bd, *a, rws, g.rows.count, state, acc, s));
    }
    if (capturing && g.tc_rows.count)
      TFQG_CUDA(launch_lock_tc_poison(bd, *a, mode, b->d_tcl_items + g.tc_rows.begin,
                                      g.tc_rows.count, st, s));
    ++gi;
  }
  if (any_tc && !capturing) check_tc_status(b, s);
}

int simulate(tfqg_batch* b, int mode, RunArgs* a, cudaStream_t s) {
  // forward modes: wide rows run on the whole grid, the rest in the queue;
  // so does the adjoint of tfq_adj_grad (not the inner-product gradient,
  // whose lambda comes from a buffer)
  const bool fwd = mode == kModeExpect || mode == kModeState || mode == kModeSample;
  const bool wide_adj = mode == kModeAdjoint && b->kind != TFQG_KIND_INNER && !a->lambda_init;
  const bool lock = fwd && !b->lock_rows.empty();
  const bool split = (fwd || wide_adj) && (!b->wide_rows.empty() || lock);
  BatchDevice bd = b->bd;
  if (split) {
    bd.order = lock ? b->d_order_lock : b->d_order_fwd;
    bd.num_queue = int32_t(lock ? b->order_lock.size() : b->order_fwd.size());
  }
  // an inner-product gradient sweeps only the reference rows (first in order)
  if (b->kind == TFQG_KIND_INNER && mode == kModeAdjoint) bd.num_queue = int32_t(b->inner_rows);
  const bool any_streamed =
      lock ? b->any_streamed_lock : split ? b->any_streamed_fwd : b->any_streamed;
  const int max_streamed_n =
      lock ? b->max_streamed_n_lock : split ? b->max_streamed_n_fwd : b->max_streamed_n;
  int grid = 0;
  if (mode == kModeNoisy || bd.num_queue > 0) {
    const int max_grads = mode == kModeAdjoint ? b->max_grads : 0;
    size_t smem = sim_smem_bytes(mode, b->max_resident_n, any_streamed, max_grads);
    if (smem > 227 * 1024)
      throw Error(kResourceExhausted, "shared memory request too large");
    cudaKernel_t jk = jit_kernel(b, mode, b->device);
    grid = jk ? jit_grid(jk, smem, b->device, jit_threads(mode)) : sim_grid_size(mode, smem);
    int64_t units = mode == kModeNoisy ? a->total_traj : bd.num_queue;
    if (units < grid) grid = int(std::max<int64_t>(units, 1));
    if (any_streamed) {
      int64_t per = int64_t(1) << max_streamed_n;
      if (mode == kModeAdjoint) per *= 2;
      a->slot_amps = per;
      b->work.reserve(size_t(per) * grid * sizeof(float2), b->device);
      a->work = static_cast<float2*>(b->work.p);
    }
    TFQG_CUDA(cudaMemsetAsync(a->counter, 0, sizeof(int), s));
    int state_amps = sim_state_amps(b->max_resident_n, any_streamed);
    bool launched = false;
    if (jk) {
      cudaError_t e = jit_launch(jk, bd, *a, grid, smem, state_amps,
                                 mode == kModeAdjoint ? 2 : 1, s, jit_threads(mode));
      launched = e == cudaSuccess;
      if (!launched) {
        // a rejected launch (nothing ran): record why, stop specializing
        // this batch and run the interpreter instead
        cudaGetLastError();
        b->jit_error = std::string("specialized launch rejected: ") + cudaGetErrorString(e);
        b->jit_mode = -1;
      }
    }
    if (!launched) TFQG_CUDA(launch_simulate(mode, bd, *a, grid, smem, state_amps, s));
  }
  if (split && wide_adj) {
    run_wide_adjoint(b, bd, a, s);
  } else if (split) {
    if (!b->wide_rows.empty()) run_wide(b, mode, bd, a, s);
    if (lock) run_lock(b, mode, bd, a, s);
  }
  return grid;
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const Error& e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return fail(kResourceExhausted, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(kInternal, e.what());
  }
}

void finish(tfqg_batch* b, void* host_dst, const void* dev_src, size_t bytes,
            int device_buffers, cudaStream_t s) {
  if (!device_buffers && bytes)
    TFQG_CUDA(cudaMemcpyAsync(host_dst, dev_src, bytes, cudaMemcpyDeviceToHost, s));
  if (!device_buffers) TFQG_CUDA(cudaStreamSynchronize(s));
  TFQG_CUDA(cudaGetLastError());
  (void)b;
}

}  // namespace

extern "C" {

const char* tfqg_last_error(void) { return g_last_error.c_str(); }
const char* tfqg_version(void) { return "tfq_gb300 0.1.0 (sm_103a)"; }

int tfqg_batch_create(const char* const* programs, const int64_t* program_lens,
                      int64_t batch, const char* const* symbol_names,
                      const int64_t* symbol_name_lens, int64_t num_symbols,
                      const char* const* pauli_sums,
                      const int64_t* pauli_sum_lens, int64_t num_ops, int kind,
                      tfqg_batch** out) {
  return guarded([&]() {
    if (!out) throw Error(kInvalidArgument, "out is NULL");
    *out = nullptr;
    if (kind < TFQG_KIND_FORWARD || kind > TFQG_KIND_NOISY)
      throw Error(kInvalidArgument, "unknown batch kind");
    std::unique_ptr<tfqg_batch> b(new tfqg_batch());
    build_batch(b.get(), programs, program_lens, batch, symbol_names,
                symbol_name_lens, num_symbols, pauli_sums, pauli_sum_lens,
                pauli_sums ? num_ops : 0, kind);
    b->n_ops = num_ops;
    *out = b.release();
    return 0;
  });
}

int tfqg_batch_max_num_qubits(const tfqg_batch* b, int32_t* out) {
  if (!b || !out) return fail(kInvalidArgument, "NULL argument");
  *out = b->max_n;
  return 0;
}

void tfqg_batch_destroy(tfqg_batch* b) {
  if (!b) return;
  // one synchronize for all of the batch's buffers, which then return to
  // the device pool for the next batch
  if (b->device >= 0 && device_sync(b->device)) b->release_buffers();
  delete b;
}

void tfqg_release_cached_memory(void) {
  pool_trim(-1);
  program_cache_clear();
}

int tfqg_batch_expectation(tfqg_batch* b, const float* symbol_values,
                           float* expectations, int device_buffers,
                           void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    size_t obytes = size_t(b->B * b->n_ops) * sizeof(float);
    if (b->B == 0 || b->n_ops == 0) return 0;
    RunArgs a;
    prepare(b, symbol_values, device_buffers, false, 0, s, &a);
    float* dout = expectations;
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<float*>(b->out.p);
    }
    a.out_f = dout;
    simulate(b, kModeExpect, &a, s);
    finish(b, expectations, dout, obytes, device_buffers, s);
    return 0;
  });
}

int tfqg_batch_state(tfqg_batch* b, const float* symbol_values, void* states,
                     int device_buffers, void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    size_t obytes = size_t(b->B) * (size_t(1) << b->max_n) * sizeof(float2);
    if (b->B == 0) return 0;
    RunArgs a;
    prepare(b, symbol_values, device_buffers, false, 0, s, &a);
    float2* dout = static_cast<float2*>(states);
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<float2*>(b->out.p);
    }
    a.out_state = dout;
    simulate(b, kModeState, &a, s);
    finish(b, states, dout, obytes, device_buffers, s);
    return 0;
  });
}

int tfqg_batch_samples(tfqg_batch* b, const float* symbol_values,
                       int32_t num_samples, uint64_t seed, int8_t* samples,
                       int device_buffers, void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    if (num_samples < 0)
      throw Error(kInvalidArgument, "num_samples must be non-negative.");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    size_t obytes = size_t(b->B) * size_t(num_samples) * size_t(b->max_n);
    if (obytes == 0) return 0;
    RunArgs a;
    prepare(b, symbol_values, device_buffers, false, 0, s, &a);
    int8_t* dout = samples;
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<int8_t*>(b->out.p);
    }
    a.out_samples = dout;
    a.num_samples = num_samples;
    a.seed = seed;
    simulate(b, kModeSample, &a, s);
    finish(b, samples, dout, obytes, device_buffers, s);
    return 0;
  });
}

int tfqg_batch_adj_grad(tfqg_batch* b, const float* symbol_values,
                        const float* downstream_grads, int grad_rule,
                        float* grads, int device_buffers, void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    if (b->kind != TFQG_KIND_ADJOINT)
      throw Error(kInvalidArgument, "batch was not created for the adjoint");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    size_t obytes = size_t(b->B * b->P) * sizeof(float);
    if (b->B == 0 || b->P == 0) return 0;
    float* dout = grads;
    ensure_device(b, s);
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<float*>(b->out.p);
    }
    TFQG_CUDA(cudaMemsetAsync(dout, 0, obytes, s));
    if (b->n_ops == 0) {
      finish(b, grads, dout, obytes, device_buffers, s);
      return 0;
    }
    RunArgs a;
    prepare(b, symbol_values, device_buffers, true, grad_rule, s, &a);
    const float* dg = downstream_grads;
    size_t gbytes = size_t(b->B * b->n_ops) * sizeof(float);
    if (!device_buffers) {
      b->aux.reserve(gbytes, b->device);
      TFQG_CUDA(cudaMemcpyAsync(b->aux.p, downstream_grads, gbytes,
                                cudaMemcpyHostToDevice, s));
      dg = static_cast<const float*>(b->aux.p);
    }
    a.dgrads = dg;
    a.out_f = dout;
    simulate(b, kModeAdjoint, &a, s);
    finish(b, grads, dout, obytes, device_buffers, s);
    return 0;
  });
}

namespace {

// Trajectory expectations; with sample_terms each Pauli term is measured once
// per trajectory instead of evaluated exactly (noisy sampled expectation).
int noisy_expectation_impl(tfqg_batch* b, const float* symbol_values,
                           const int32_t* num_samples, uint64_t seed, float* expectations,
                           int device_buffers, void* stream, bool sample_terms) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    if (b->kind != TFQG_KIND_NOISY)
      throw Error(kInvalidArgument, "batch was not created for noisy simulation");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t cells = b->B * b->n_ops;
    size_t obytes = size_t(cells) * sizeof(float);
    if (cells == 0) return 0;
    // trajectories per row = max over its ops; the host needs the counts
    std::vector<int32_t> reps(static_cast<size_t>(cells));
    if (device_buffers) {
      TFQG_CUDA(cudaMemcpyAsync(reps.data(), num_samples, cells * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)));
      TFQG_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    } else {
      memcpy(reps.data(), num_samples, cells * sizeof(int32_t));
    }
    for (int32_t r : reps)
      if (r < 1)
        throw Error(kInvalidArgument,
                    "Each element of num_samples must be greater than 0.");
    std::vector<int64_t> prefix(static_cast<size_t>(b->B) + 1, 0);
    for (int64_t i = 0; i < b->B; ++i) {
      int32_t m = 0;
      const DevProgram& p = b->programs[b->rows[i].program];
      if (p.n > 0 && p.fwd_pass_begin != p.fwd_pass_end)
        for (int64_t j = 0; j < b->n_ops; ++j) m = std::max(m, reps[i * b->n_ops + j]);
      prefix[i + 1] = prefix[i] + m;
    }
    RunArgs a;
    prepare(b, symbol_values, device_buffers, false, 0, s, &a);
    // aux: reps (int32) ; aux2: prefix (int64) + accumulators (double)
    b->aux.reserve(cells * sizeof(int32_t), b->device);
    TFQG_CUDA(cudaMemcpyAsync(b->aux.p, reps.data(), cells * sizeof(int32_t),
                              cudaMemcpyHostToDevice, s));
    size_t pbytes = align256(prefix.size() * sizeof(int64_t));
    b->aux2.reserve(pbytes + cells * sizeof(double), b->device);
    TFQG_CUDA(cudaMemcpyAsync(b->aux2.p, prefix.data(), prefix.size() * sizeof(int64_t),
                              cudaMemcpyHostToDevice, s));
    double* acc = reinterpret_cast<double*>(static_cast<char*>(b->aux2.p) + pbytes);
    TFQG_CUDA(cudaMemsetAsync(acc, 0, cells * sizeof(double), s));
    float* dout = expectations;
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<float*>(b->out.p);
    }
    a.reps = static_cast<const int32_t*>(b->aux.p);
    a.traj_prefix = static_cast<const int64_t*>(b->aux2.p);
    a.total_traj = prefix.back();
    a.acc = acc;
    a.seed = seed;
    a.out_f = dout;
    a.sample_terms = sample_terms ? 1 : 0;
    if (a.total_traj > 0) simulate(b, kModeNoisy, &a, s);
    TFQG_CUDA(launch_noisy_finalize(b->bd, a, s));
    finish(b, expectations, dout, obytes, device_buffers, s);
    // the host vectors above are read by async copies: keep them alive
    TFQG_CUDA(cudaStreamSynchronize(s));
    return 0;
  });
}

}  // namespace

int tfqg_batch_noisy_expectation(tfqg_batch* b, const float* symbol_values,
                                 const int32_t* num_samples, uint64_t seed,
                                 float* expectations, int device_buffers,
                                 void* stream) {
  return noisy_expectation_impl(b, symbol_values, num_samples, seed, expectations,
                                device_buffers, stream, false);
}

int tfqg_batch_noisy_sampled_expectation(tfqg_batch* b, const float* symbol_values,
                                         const int32_t* num_samples, uint64_t seed,
                                         float* expectations, int device_buffers,
                                         void* stream) {
  return noisy_expectation_impl(b, symbol_values, num_samples, seed, expectations,
                                device_buffers, stream, true);
}

int tfqg_batch_noisy_samples(tfqg_batch* b, const float* symbol_values,
                             int32_t num_samples, uint64_t seed, int8_t* samples,
                             int device_buffers, void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    if (b->kind != TFQG_KIND_NOISY)
      throw Error(kInvalidArgument, "batch was not created for noisy simulation");
    if (num_samples < 0)
      throw Error(kInvalidArgument, "num_samples must be non-negative.");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t obytes = size_t(b->B) * size_t(num_samples) * size_t(b->max_n);
    if (obytes == 0) return 0;  // tfq_noisy_samples.cc:122-124
    // one trajectory per sample, rows in order
    std::vector<int64_t> prefix(static_cast<size_t>(b->B) + 1, 0);
    for (int64_t i = 0; i < b->B; ++i) prefix[i + 1] = prefix[i] + num_samples;
    RunArgs a;
    prepare(b, symbol_values, device_buffers, false, 0, s, &a);
    b->aux2.reserve(prefix.size() * sizeof(int64_t), b->device);
    TFQG_CUDA(cudaMemcpyAsync(b->aux2.p, prefix.data(), prefix.size() * sizeof(int64_t),
                              cudaMemcpyHostToDevice, s));
    int8_t* dout = samples;
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<int8_t*>(b->out.p);
    }
    a.traj_prefix = static_cast<const int64_t*>(b->aux2.p);
    a.total_traj = prefix.back();
    a.out_samples = dout;
    a.num_samples = num_samples;
    a.seed = seed;
    simulate(b, kModeNoisy, &a, s);
    finish(b, samples, dout, obytes, device_buffers, s);
    TFQG_CUDA(cudaStreamSynchronize(s));  // the host prefix is read asynchronously
    return 0;
  });
}

int tfqg_batch_sampled_expectation(tfqg_batch* b, const float* symbol_values,
                                   const int32_t* num_samples, uint64_t seed,
                                   float* expectations, int device_buffers,
                                   void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    if (b->kind == TFQG_KIND_NOISY)
      throw Error(kInvalidArgument, "batch was created for noisy simulation");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t cells = b->B * b->n_ops;
    const size_t obytes = size_t(cells) * sizeof(float);
    if (cells == 0) return 0;
    std::vector<int32_t> ns(static_cast<size_t>(cells));
    if (device_buffers) {
      TFQG_CUDA(cudaMemcpyAsync(ns.data(), num_samples, cells * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, s));
      TFQG_CUDA(cudaStreamSynchronize(s));
    } else {
      memcpy(ns.data(), num_samples, cells * sizeof(int32_t));
    }
    for (int32_t v : ns)  // GetNumSamples (parse_context.cc:349-381)
      if (v < 1)
        throw Error(kInvalidArgument, "Each element of num_samples must be greater than 0.");
    int64_t stride = 1;
    for (const DevRow& r : b->rows)
      stride = std::max<int64_t>(stride, int64_t(r.term_end) - int64_t(r.term_begin));
    RunArgs a;
    prepare(b, symbol_values, device_buffers, false, 0, s, &a);
    b->aux.reserve(cells * sizeof(int32_t), b->device);
    TFQG_CUDA(cudaMemcpyAsync(b->aux.p, ns.data(), cells * sizeof(int32_t),
                              cudaMemcpyHostToDevice, s));
    b->aux2.reserve(size_t(b->B * stride) * sizeof(double), b->device);
    a.term_vals = static_cast<double*>(b->aux2.p);
    a.term_stride = stride;
    float* dout = expectations;
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<float*>(b->out.p);
    }
    a.out_f = dout;
    a.seed = seed;
    simulate(b, kModeExpect, &a, s);
    TFQG_CUDA(launch_sampled_expectation(b->bd, a, static_cast<const int32_t*>(b->aux.p), s));
    finish(b, expectations, dout, obytes, device_buffers, s);
    // the host vector above is read by an async copy: keep it alive
    TFQG_CUDA(cudaStreamSynchronize(s));
    return 0;
  });
}

int tfqg_simulate_sampled_expectation(const char* const* programs,
                                      const int64_t* program_lens, int64_t batch,
                                      const char* const* symbol_names,
                                      const int64_t* symbol_name_lens, int64_t num_symbols,
                                      const float* symbol_values,
                                      const char* const* pauli_sums,
                                      const int64_t* pauli_sum_lens, int64_t num_ops,
                                      const int32_t* num_samples, uint64_t seed,
                                      float* expectations) {
  tfqg_batch* b = nullptr;
  int rc = tfqg_batch_create(programs, program_lens, batch, symbol_names,
                             symbol_name_lens, num_symbols, pauli_sums, pauli_sum_lens,
                             num_ops, TFQG_KIND_FORWARD, &b);
  if (rc) return rc;
  rc = tfqg_batch_sampled_expectation(b, symbol_values, num_samples, seed, expectations, 0,
                                      nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

int tfqg_batch_create_inner_product(const char* const* programs,
                                    const int64_t* program_lens, int64_t batch,
                                    const char* const* symbol_names,
                                    const int64_t* symbol_name_lens, int64_t num_symbols,
                                    const char* const* other_programs,
                                    const int64_t* other_program_lens, int64_t num_others,
                                    int with_grads, tfqg_batch** out) {
  return guarded([&]() {
    if (!out) throw Error(kInvalidArgument, "out is NULL");
    *out = nullptr;
    std::unique_ptr<tfqg_batch> b(new tfqg_batch());
    build_batch(b.get(), programs, program_lens, batch, symbol_names, symbol_name_lens,
                num_symbols, nullptr, nullptr, 0, TFQG_KIND_INNER, other_programs,
                other_program_lens, num_others, with_grads != 0);
    *out = b.release();
    return 0;
  });
}

int tfqg_batch_inner_product(tfqg_batch* b, const float* symbol_values,
                             void* inner_products, int device_buffers, void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    if (b->kind != TFQG_KIND_INNER)
      throw Error(kInvalidArgument, "batch was not created for inner products");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t pairs = b->inner_rows * b->inner_others;
    const size_t obytes = size_t(pairs) * sizeof(float2);
    if (pairs == 0) return 0;
    RunArgs a;
    prepare(b, symbol_values, device_buffers, false, 0, s, &a);
    const int64_t stride = int64_t(1) << b->max_n;
    b->aux.reserve(size_t(b->B * stride) * sizeof(float2), b->device);
    a.out_state = static_cast<float2*>(b->aux.p);
    simulate(b, kModeState, &a, s);
    b->aux2.reserve(size_t(pairs) * 2 * sizeof(double), b->device);
    double* acc = static_cast<double*>(b->aux2.p);
    TFQG_CUDA(cudaMemsetAsync(acc, 0, size_t(pairs) * 2 * sizeof(double), s));
    float2* dout = static_cast<float2*>(inner_products);
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<float2*>(b->out.p);
    }
    TFQG_CUDA(launch_inner_products(b->bd, a.out_state, stride, int(b->inner_rows),
                                    int(b->inner_others), acc, dout, s));
    finish(b, inner_products, dout, obytes, device_buffers, s);
    return 0;
  });
}

int tfqg_batch_inner_product_grad(tfqg_batch* b, const float* symbol_values,
                                  const float* downstream_grads, void* grads,
                                  int device_buffers, void* stream) {
  return guarded([&]() {
    if (!b) throw Error(kInvalidArgument, "NULL batch");
    if (b->kind != TFQG_KIND_INNER || !b->inner_grads)
      throw Error(kInvalidArgument,
                  "batch was not created for inner-product gradients");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t B = b->inner_rows, M = b->inner_others, P = b->P;
    const size_t obytes = size_t(B * P) * sizeof(float2);
    if (B == 0 || P == 0) return 0;
    float2* dout = static_cast<float2*>(grads);
    ensure_device(b, s);
    if (!device_buffers) {
      b->out.reserve(obytes, b->device);
      dout = static_cast<float2*>(b->out.p);
    }
    if (M == 0) {  // no paired circuits: chi = 0
      TFQG_CUDA(cudaMemsetAsync(dout, 0, obytes, s));
      finish(b, grads, dout, obytes, device_buffers, s);
      return 0;
    }
    RunArgs a;
    prepare(b, symbol_values, device_buffers, true, TFQG_GRAD_REFERENCE_FD, s, &a);
    // 1. every row's final state; 2. chi_i = sum_j g_ij phi_ij over the
    // reference rows' states (the adjoint recomputes psi_i itself)
    const int64_t stride = int64_t(1) << b->max_n;
    b->aux.reserve(size_t(b->B * stride) * sizeof(float2), b->device);
    float2* states = static_cast<float2*>(b->aux.p);
    a.out_state = states;
    simulate(b, kModeState, &a, s);
    const float* dg = downstream_grads;
    const size_t gbytes = size_t(B * M) * sizeof(float);
    b->aux2.reserve(gbytes, b->device);
    if (!device_buffers) {
      TFQG_CUDA(cudaMemcpyAsync(b->aux2.p, downstream_grads, gbytes,
                                cudaMemcpyHostToDevice, s));
      dg = static_cast<const float*>(b->aux2.p);
    }
    TFQG_CUDA(launch_paired_sum(b->bd, states, stride, int(B), int(M), dg, s));
    // 3. Re<chi|dU psi> and Im<chi|dU psi> = Re<i chi|dU psi> by two adjoint
    // sweeps seeded with chi and i chi; <dU psi|chi> = (Re, -Im)
    b->inner_tmp.reserve(size_t(2 * B * P) * sizeof(float), b->device);
    float* re = static_cast<float*>(b->inner_tmp.p);
    float* im = re + B * P;
    TFQG_CUDA(cudaMemsetAsync(re, 0, size_t(2 * B * P) * sizeof(float), s));
    a.lambda_init = states;
    a.lambda_stride = stride;
    a.grad_scale = 1.f;
    a.lambda_rot = 0;
    a.out_f = re;
    simulate(b, kModeAdjoint, &a, s);
    a.lambda_rot = 1;
    a.out_f = im;
    simulate(b, kModeAdjoint, &a, s);
    TFQG_CUDA(launch_conj_combine(re, im, dout, B * P, s));
    finish(b, grads, dout, obytes, device_buffers, s);
    return 0;
  });
}

int tfqg_inner_product(const char* const* programs, const int64_t* program_lens,
                       int64_t batch, const char* const* symbol_names,
                       const int64_t* symbol_name_lens, int64_t num_symbols,
                       const float* symbol_values, const char* const* other_programs,
                       const int64_t* other_program_lens, int64_t num_others,
                       void* inner_products) {
  tfqg_batch* b = nullptr;
  int rc = tfqg_batch_create_inner_product(programs, program_lens, batch, symbol_names,
                                           symbol_name_lens, num_symbols, other_programs,
                                           other_program_lens, num_others, 0, &b);
  if (rc) return rc;
  rc = tfqg_batch_inner_product(b, symbol_values, inner_products, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

int tfqg_noisy_sampled_expectation(const char* const* programs,
                                   const int64_t* program_lens, int64_t batch,
                                   const char* const* symbol_names,
                                   const int64_t* symbol_name_lens, int64_t num_symbols,
                                   const float* symbol_values,
                                   const char* const* pauli_sums,
                                   const int64_t* pauli_sum_lens, int64_t num_ops,
                                   const int32_t* num_samples, uint64_t seed,
                                   float* expectations) {
  tfqg_batch* b = nullptr;
  int rc = tfqg_batch_create(programs, program_lens, batch, symbol_names, symbol_name_lens,
                             num_symbols, pauli_sums, pauli_sum_lens, num_ops,
                             TFQG_KIND_NOISY, &b);
  if (rc) return rc;
  rc = tfqg_batch_noisy_sampled_expectation(b, symbol_values, num_samples, seed,
                                            expectations, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

int tfqg_noisy_samples(const char* const* programs, const int64_t* program_lens,
                       int64_t batch, const char* const* symbol_names,
                       const int64_t* symbol_name_lens, int64_t num_symbols,
                       const float* symbol_values, int32_t num_samples, uint64_t seed,
                       int8_t* samples) {
  tfqg_batch* b = nullptr;
  int rc = tfqg_batch_create(programs, program_lens, batch, symbol_names, symbol_name_lens,
                             num_symbols, nullptr, nullptr, 0, TFQG_KIND_NOISY, &b);
  if (rc) return rc;
  rc = tfqg_batch_noisy_samples(b, symbol_values, num_samples, seed, samples, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

int tfqg_simulate_expectation(const char* const* programs,
                              const int64_t* program_lens, int64_t batch,
                              const char* const* symbol_names,
                              const int64_t* symbol_name_lens,
                              int64_t num_symbols, const float* symbol_values,
                              const char* const* pauli_sums,
                              const int64_t* pauli_sum_lens, int64_t num_ops,
                              float* expectations) {
  tfqg_batch* b = nullptr;
  int rc = tfqg_batch_create(programs, program_lens, batch, symbol_names,
                             symbol_name_lens, num_symbols, pauli_sums,
                             pauli_sum_lens, num_ops, TFQG_KIND_FORWARD, &b);
  if (rc) return rc;
  rc = tfqg_batch_expectation(b, symbol_values, expectations, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

// ---- CUDA graphs of a batch's forward calls ----------------------------------

}  // extern "C"

struct tfqg_graph {
  tfqg_batch* batch = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> buffers;  // the batch's device buffers at capture
};

namespace {
// Device buffers a captured call may address; a graph replays only while
// every one of them is still the buffer it captured.
std::vector<void*> batch_buffers(tfqg_batch* b) {
  return {b->tables.p,     b->mats.p,      b->dmats.p,     b->work.p,     b->counter.p,
          b->values.p,     b->out.p,       b->aux.p,       b->aux2.p,     b->wide_state.p,
          b->wide_acc.p,   b->tc_tab.p,    b->tc_mats.p,   b->tc_status.p, b->lock_state.p,
          b->lock_acc.p,   b->tcl_tab.p,   b->tcl_mats.p,  b->tcl_sync.p};
}

int run_forward(tfqg_batch* b, int what, const float* values, int32_t num_samples,
                uint64_t seed, void* out, void* stream) {
  if (what == 0)
    return tfqg_batch_expectation(b, values, static_cast<float*>(out), 1, stream);
  if (what == 1) return tfqg_batch_state(b, values, out, 1, stream);
  return tfqg_batch_samples(b, values, num_samples, seed, static_cast<int8_t*>(out), 1, stream);
}
}  // namespace

extern "C" {

int tfqg_batch_graph_create(tfqg_batch* b, int what, const float* symbol_values,
                            int32_t num_samples, uint64_t seed, void* out, void* stream,
                            tfqg_graph** graph) {
  if (!b || !graph) return fail(kInvalidArgument, "NULL argument");
  if (what < 0 || what > 2) return fail(kInvalidArgument, "unknown call to capture");
  *graph = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!s) return fail(kInvalidArgument, "capture needs a stream other than the legacy default");
  // one ordinary call first: tables, buffers and compiled modules in place
  int rc = run_forward(b, what, symbol_values, num_samples, seed, out, stream);
  if (rc) return rc;
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return fail(kInternal, "stream synchronize failed before capture");
  std::unique_ptr<tfqg_graph> g(new tfqg_graph());
  g->batch = b;
  g->buffers = batch_buffers(b);
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess)
    return fail(kInternal, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
  rc = run_forward(b, what, symbol_values, num_samples, seed, out, stream);
  cudaGraph_t cg = nullptr;
  e = cudaStreamEndCapture(s, &cg);
  if (rc) {
    if (cg) cudaGraphDestroy(cg);
    return rc;
  }
  if (e != cudaSuccess || !cg) {
    cudaGetLastError();
    return fail(kInternal, std::string("this call cannot be captured: ") +
                               cudaGetErrorString(e));
  }
  if (batch_buffers(b) != g->buffers) {
    cudaGraphDestroy(cg);
    return fail(kInternal, "the captured call moved the batch's buffers");
  }
  g->graph = cg;
  e = cudaGraphInstantiate(&g->exec, cg, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(cg);
    g->graph = nullptr;
    return fail(kInternal, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  *graph = g.release();
  return 0;
}

int tfqg_graph_launch(tfqg_graph* g, void* stream) {
  if (!g || !g->exec) return fail(kInvalidArgument, "NULL graph");
  {
    std::lock_guard<std::mutex> lk(g->batch->mu);
    if (batch_buffers(g->batch) != g->buffers)
      return fail(kInvalidArgument,
                  "the batch's device buffers changed since the graph was captured "
                  "(another call on the batch needed larger ones); capture it again");
  }
  const cudaError_t e = cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess)
    return fail(kInternal, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
  return 0;
}

void tfqg_graph_destroy(tfqg_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

int tfqg_max_num_qubits(const char* const* programs, const int64_t* program_lens,
                        int64_t batch, int32_t* max_num_qubits) {
  return guarded([&]() {
    if (!max_num_qubits) throw Error(kInvalidArgument, "max_num_qubits is NULL");
    if (batch < 0 || (batch > 0 && (!programs || !program_lens)))
      throw Error(kInvalidArgument, "NULL programs");
    // decode and resolve qubits only: symbols are bound later, as in
    // GetProgramsAndNumQubits (parse_context.cc:268-320); on the host's
    // cores, the first error in row order raised
    std::vector<int> nq(size_t(batch), 0);
    std::vector<std::exception_ptr> errs(static_cast<size_t>(batch));
    parallel_for(size_t(batch), [&](size_t i) {
      try {
        ProgramP p;
        decode_program(programs[i], size_t(program_lens[i]), &p);
        std::unordered_map<std::string, int> index;
        nq[i] = resolve_qubits(p, &index);
      } catch (...) {
        errs[i] = std::current_exception();
      }
    });
    rethrow_first(errs);
    int mx = 0;
    for (const int n : nq) mx = std::max(mx, n);
    *max_num_qubits = mx;
    return 0;
  });
}

namespace {
// A transient forward batch whose widest program has `max_num_qubits`
// qubits (the caller sized its output from that), or an error code.
int forward_batch(const char* const* programs, const int64_t* program_lens, int64_t batch,
                  const char* const* symbol_names, const int64_t* symbol_name_lens,
                  int64_t num_symbols, int32_t max_num_qubits, tfqg_batch** out) {
  int rc = tfqg_batch_create(programs, program_lens, batch, symbol_names, symbol_name_lens,
                             num_symbols, nullptr, nullptr, 0, TFQG_KIND_FORWARD, out);
  if (rc) return rc;
  int32_t mq = 0;
  rc = tfqg_batch_max_num_qubits(*out, &mq);
  if (rc == 0 && mq != max_num_qubits)
    rc = fail(kInvalidArgument, "max_num_qubits is " + std::to_string(max_num_qubits) +
                                    " but the programs' largest qubit count is " +
                                    std::to_string(mq));
  if (rc) {
    tfqg_batch_destroy(*out);
    *out = nullptr;
  }
  return rc;
}
}  // namespace

int tfqg_simulate_state(const char* const* programs, const int64_t* program_lens,
                        int64_t batch, const char* const* symbol_names,
                        const int64_t* symbol_name_lens, int64_t num_symbols,
                        const float* symbol_values, int32_t max_num_qubits,
                        void* states) {
  tfqg_batch* b = nullptr;
  int rc = forward_batch(programs, program_lens, batch, symbol_names, symbol_name_lens,
                         num_symbols, max_num_qubits, &b);
  if (rc) return rc;
  rc = tfqg_batch_state(b, symbol_values, states, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

int tfqg_simulate_samples(const char* const* programs, const int64_t* program_lens,
                          int64_t batch, const char* const* symbol_names,
                          const int64_t* symbol_name_lens, int64_t num_symbols,
                          const float* symbol_values, int32_t num_samples, uint64_t seed,
                          int32_t max_num_qubits, int8_t* samples) {
  tfqg_batch* b = nullptr;
  int rc = forward_batch(programs, program_lens, batch, symbol_names, symbol_name_lens,
                         num_symbols, max_num_qubits, &b);
  if (rc) return rc;
  rc = tfqg_batch_samples(b, symbol_values, num_samples, seed, samples, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

int tfqg_adj_grad(const char* const* programs, const int64_t* program_lens,
                  int64_t batch, const char* const* symbol_names,
                  const int64_t* symbol_name_lens, int64_t num_symbols,
                  const float* symbol_values, const char* const* pauli_sums,
                  const int64_t* pauli_sum_lens, int64_t num_ops,
                  const float* downstream_grads, float* grads) {
  tfqg_batch* b = nullptr;
  int rc = tfqg_batch_create(programs, program_lens, batch, symbol_names,
                             symbol_name_lens, num_symbols, pauli_sums,
                             pauli_sum_lens, num_ops, TFQG_KIND_ADJOINT, &b);
  if (rc) return rc;
  rc = tfqg_batch_adj_grad(b, symbol_values, downstream_grads,
                           TFQG_GRAD_REFERENCE_FD, grads, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

int tfqg_noisy_expectation(const char* const* programs,
                           const int64_t* program_lens, int64_t batch,
                           const char* const* symbol_names,
                           const int64_t* symbol_name_lens,
                           int64_t num_symbols, const float* symbol_values,
                           const char* const* pauli_sums,
                           const int64_t* pauli_sum_lens, int64_t num_ops,
                           const int32_t* num_samples, uint64_t seed,
                           float* expectations) {
  tfqg_batch* b = nullptr;
  int rc = tfqg_batch_create(programs, program_lens, batch, symbol_names,
                             symbol_name_lens, num_symbols, pauli_sums,
                             pauli_sum_lens, num_ops, TFQG_KIND_NOISY, &b);
  if (rc) return rc;
  rc = tfqg_batch_noisy_expectation(b, symbol_values, num_samples, seed,
                                    expectations, 0, nullptr);
  tfqg_batch_destroy(b);
  return rc;
}

// Run-time specialization control: mode -1 off, 0 automatic, 1 forced, any
// other value leaves it unchanged.
// Returns the number of sub-pass signatures; bit m of `active` is set when
// the specialized module of SimMode m is loaded, `err` receives the last specialization error.
int tfqg_internal_batch_jit(void* batch, int mode, int32_t* nsig, int32_t* active,
                            char* err, int64_t err_size) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  if (!b) return kInvalidArgument;
  if (mode >= -1 && mode <= 1) b->jit_mode = mode;
  if (nsig) *nsig = int32_t(b->jit_signatures.size());
  if (active) {
    *active = 0;
    for (int m = 0; m < kJitModes; ++m)
      if (b->jit_module[m]) *active |= 1 << m;
  }
  if (err && err_size > 0) {
    strncpy(err, b->jit_error.c_str(), size_t(err_size - 1));
    err[err_size - 1] = 0;
  }
  return 0;
}

// Generated specialized source of `mode` for a batch; returns its length
// (the copy into buf is truncated to size - 1 bytes).
int64_t tfqg_internal_jit_source(void* batch, int mode, char* buf, int64_t size) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  if (!b || mode < 0 || mode >= kJitModes) return -1;
  const std::string src = jit_source(b, mode);
  if (buf && size > 0) {
    strncpy(buf, src.c_str(), size_t(size - 1));
    buf[size - 1] = 0;
  }
  return int64_t(src.size());
}

// Generates and compiles the batch's specialized module on the host only;
// `err` receives the compiler log (resource usage on success).
int tfqg_internal_jit_compile_check(void* batch, int mode, char* err, int64_t err_size) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  std::string log;
  int rc = jit_compile_check(b, mode, &log);
  if (err && err_size > 0) {
    strncpy(err, log.c_str(), size_t(err_size - 1));
    err[err_size - 1] = 0;
  }
  return rc;
}

// Bytes of compiled tables uploaded to the device per batch (benchmark
// accounting of host->device traffic).
// Qubit count from which forward-mode rows run as wide rows, for batches
// created after the call (clamped to at least the streamed tile + 2);
// returns the previous value.
int tfqg_internal_set_wide_min_qubits(int n) {
  return g_wide_min_qubits.exchange(n);
}

// Compiled-program cache on (1) or off (0); off also empties it.  Returns
// the previous setting; hits and misses since the process started go to
// *hits and *misses when not NULL.
int tfqg_internal_program_cache(int on, int64_t* hits, int64_t* misses) {
  if (hits) *hits = g_pc_hits.load();
  if (misses) *misses = g_pc_misses.load();
  if (on < 0) return g_pc_on.load();
  const int prev = g_pc_on.exchange(on ? 1 : 0);
  if (!on) program_cache_clear();
  return prev;
}

// Capacity of the compiled-program cache in bytes (0 keeps it); returns
// the previous capacity.  Entries beyond it are evicted on the next insert.
int64_t tfqg_internal_program_cache_bytes(int64_t bytes) {
  const size_t prev = program_cache_bytes();
  if (bytes > 0) g_pc_cap.store(size_t(bytes));
  return int64_t(prev);
}

// Entries and bytes held by the compiled-program cache.
int64_t tfqg_internal_program_cache_size(int64_t* bytes) {
  std::lock_guard<std::mutex> lk(g_pc_mu);
  if (bytes) *bytes = int64_t(g_pc_bytes);
  return int64_t(g_pc.size());
}

// Gate fusion of forward plans on (1) or off (0) for batches created after
// the call; returns the previous setting.
int tfqg_internal_set_gate_fusion(int on) {
  return g_gate_fusion.exchange(on ? 1 : 0);
}

// Forward passes of wide rows as 5-bit fused blocks on the tensor cores
// (tc_gates.cu): 0 never (tile passes), 1 always, 2 (default) for rows of
// 24 qubits and more; for calls made after this one.  Returns the previous
// setting.
int tfqg_internal_set_tensor_core_gates(int mode) {
  return g_tc_gates.exchange(mode < 0 || mode > 2 ? 2 : mode);
}

// One launch of the tensor-core block kernel on a caller's state: psi (2^n
// complex64, device), U (32 x 32 complex64 row-major, device), tgt (5
// ascending bits, host), status (device int).  grid <= 0 picks the
// occupancy grid.  Returns a cudaError_t.
int tfqg_internal_tc_apply(void* psi, int n, const void* U, const int32_t* tgt, int* status,
                           int grid, void* stream) {
  TcBlock blk{};
  for (int i = 0; i < kTcBits; ++i) {
    if (tgt[i] < 0 || tgt[i] > 31) return int(cudaErrorInvalidValue);
    blk.tgt[i] = uint8_t(tgt[i]);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return int(e);
  if (grid <= 0) {
    try {
      grid = tc_grid(dev);
    } catch (const Error&) {
      return int(cudaErrorInvalidValue);
    }
  }
  return int(launch_tc_apply5(static_cast<float2*>(psi), n, static_cast<const float2*>(U), blk,
                              status, grid, static_cast<cudaStream_t>(stream)));
}

// CTAs of a tensor-core block launch on the current device (-1 on error).
int tfqg_internal_tc_grid() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  try {
    return tc_grid(dev);
  } catch (const Error&) {
    return -1;
  }
}

// Tensor-core blocks that the k-th wide row of a batch ran in its last
// forward call (-1: it ran tile passes, or has not run), and the kernels'
// status word (nonzero: an MMA completion wait timed out); synchronizes the
// device when reading it.
int tfqg_internal_tc_blocks(void* batch, int64_t k) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  if (!b || !b->tc_planned || k < 0 || k >= int64_t(b->tc_rows.size())) return -1;
  return b->tc_ran[size_t(k)] ? b->tc_rows[size_t(k)].second : -1;
}

// State sweeps (kernel launches) of the tensor-core blocks of the k-th wide
// row in its last forward call (-1: it ran tile passes, or has not run).
int tfqg_internal_tc_sweeps(void* batch, int64_t k) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  if (!b || !b->tc_planned || k < 0 || k >= int64_t(b->tc_rows.size())) return -1;
  return b->tc_ran[size_t(k)] ? b->tc_sweeps[size_t(k)] : -1;
}

// Two blocks per sweep where their targets allow it (1) or one (0), for
// calls made from now on; returns the previous setting.
int tfqg_internal_set_tc_sweep(int on) { return g_tc_sweep.exchange(on ? 1 : 0); }
// Chunk geometry of the block kernel for targets tgt[0..4] (ascending) on an
// n-qubit state: 1 and the transposed variant's tables, or 0 for the direct
// variant (host only; lets tests check the kernel's index arithmetic).
int tfqg_internal_tc_geometry(int n, const int32_t* tgt, uint64_t* cb, uint32_t* rpos,
                              uint32_t* tpos, uint32_t* c) {
  TcBlock blk{};
  for (int i = 0; i < kTcBits; ++i) blk.tgt[i] = uint8_t(tgt[i]);
  TcTrans tr{};
  if (!tc_transposed_geometry(blk, n, &tr)) return 0;
  *cb = tr.cb;
  *rpos = tr.rpos;
  *tpos = tr.tpos;
  *c = tr.c;
  return 1;
}

// Geometry of a two-block sweep for targets tgt0 / tgt1 (5 each, ascending)
// on an n-qubit state: 1 and its tables (host only; lets tests check the
// sweep kernel's index arithmetic), or 0 when the blocks cannot share one.
// out[0..8]: cb (low 32 bits), cb (high 32 bits), cb12, smask, tpos0, tpos1,
// rpos0, rpos1, hmask; out[9]: r0.
int tfqg_internal_tc_sweep_geometry(int n, const int32_t* tgt0, const int32_t* tgt1,
                                    uint32_t* out) {
  TcBlock b0{}, b1{};
  for (int i = 0; i < kTcBits; ++i) {
    b0.tgt[i] = uint8_t(tgt0[i]);
    b1.tgt[i] = uint8_t(tgt1[i]);
  }
  TcSweep g{};
  if (!tc_sweep_geometry(b0, b1, n, &g)) return 0;
  const uint32_t v[10] = {uint32_t(g.cb), uint32_t(g.cb >> 32), g.cb12, g.smask, g.tpos[0],
                          g.tpos[1], g.rpos[0], g.rpos[1], g.hmask, g.r0};
  for (int i = 0; i < 10; ++i) out[i] = v[i];
  return 1;
}

// One two-block sweep (U0 on tgt0, then U1 on tgt1) on a device state psi
// of 2^n complex64 amplitudes; grid <= 0 picks one CTA per SM.  Returns a
// cudaError_t (cudaErrorInvalidValue when the blocks cannot share a sweep).
int tfqg_internal_tc_sweep(void* psi, int n, const void* U0, const void* U1,
                           const int32_t* tgt0, const int32_t* tgt1, int* status, int grid,
                           void* stream) {
  TcBlock b0{}, b1{};
  for (int i = 0; i < kTcBits; ++i) {
    if (tgt0[i] < 0 || tgt0[i] > 31 || tgt1[i] < 0 || tgt1[i] > 31)
      return int(cudaErrorInvalidValue);
    b0.tgt[i] = uint8_t(tgt0[i]);
    b1.tgt[i] = uint8_t(tgt1[i]);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return int(e);
  if (grid <= 0) {
    e = cudaDeviceGetAttribute(&grid, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return int(e);
  }
  return int(launch_tc_sweep2(static_cast<float2*>(psi), n, static_cast<const float2*>(U0),
                              static_cast<const float2*>(U1), b0, b1, status, grid,
                              static_cast<cudaStream_t>(stream)));
}

// Makes the next calls treat the tensor-core status word as `status`
// (0 restores the real read-back; 2: captured calls only, see
// g_tc_status_injected); returns the previous setting.
int tfqg_internal_tc_inject_status(int status) { return g_tc_status_injected.exchange(status); }

int tfqg_internal_tc_status(void* batch) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  if (!b || !b->tc_status.p) return 0;
  int v = 0;
  if (cudaMemcpy(&v, b->tc_status.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  return v;
}

// Host copy of the tensor-core block plan of row `row` with its matrices
// bound to `row_values` (complex128 products of the complex64 gate
// matrices, as tc_fuse_kernel computes them): per block 5 target bits in
// tgt[5 * i ...] and the 32 x 32 matrix, row-major, as (re, im) pairs in
// mats[2048 * i ...].  At most `max` blocks are written; *count gets the
// total, -1 when the row has no plan.
int tfqg_internal_tc_plan(void* batch, int64_t row, const float* row_values, int32_t* tgt,
                          double* mats, int64_t max, int64_t* count) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  if (!b || row < 0 || row >= int64_t(b->rows.size()) || !count) return kInvalidArgument;
  const DevProgram& p = b->programs[b->rows[size_t(row)].program];
  const GateTemplate* gates = b->gates.data() + p.gate_begin;
  std::vector<TcBlock> blocks;
  std::vector<int32_t> members;
  if (p.num_channels != 0 || !plan_tc_blocks(gates, p.num_gates, p.n, &blocks, &members)) {
    *count = -1;
    return 0;
  }
  *count = int64_t(blocks.size());
  for (size_t i = 0; i < blocks.size() && int64_t(i) < max; ++i) {
    for (int q = 0; q < kTcBits; ++q) tgt[i * kTcBits + q] = blocks[i].tgt[q];
    for (int j = 0; j < 32; ++j) {
      Cx<double> col[32];
      tc_block_column(gates, members.data(), blocks[i], j,
                      [&](int k, Cx<double>* m) {
                        Cx<double> md[16];
                        const int kq = bound_matrix(gates[k], row_values, md);
                        for (int e = 0; e < 16; ++e) {
                          const bool in = e < (kq == 1 ? 4 : 16);
                          // the device reads complex64 gate matrices
                          m[e] = in ? Cx<double>(double(float(md[e].re)),
                                                 double(float(md[e].im)))
                                    : Cx<double>(0.0, 0.0);
                        }
                      },
                      col);
      for (int r = 0; r < 32; ++r) {
        mats[i * 2048 + (r * 32 + j) * 2] = col[r].re;
        mats[i * 2048 + (r * 32 + j) * 2 + 1] = col[r].im;
      }
    }
  }
  return 0;
}

// Streamed-row count below which rows of 17+ qubits run as wide rows, for
// batches created after the call (0: never); returns the previous value.
int tfqg_internal_set_wide_few_rows(int rows) { return g_wide_few_rows.exchange(rows); }

// Row policy for rows of n qubits in batches created from now on (see
// g_fuse_by_n): fuse -1 default, 0 off, 1 on; lock -1 default, 0 off, 1
// lockstep on tile passes, 2 lockstep on tensor-core blocks; n < 0 resets
// every qubit count.  Returns the new policy epoch.
int tfqg_internal_set_row_policy(int n, int fuse, int lock) {
  if (n < 0) {
    for (int i = 0; i < kPolicyMaxQubits; ++i) {
      g_fuse_by_n[i].store(-1);
      g_lock_by_n[i].store(-1);
    }
  } else if (n < kPolicyMaxQubits) {
    g_fuse_by_n[n].store(fuse < 0 ? -1 : fuse != 0);
    g_lock_by_n[n].store(lock < 0 ? -1 : std::min(lock, 2));
  }
  return g_policy_epoch.fetch_add(1) + 1;
}

// Lockstep rows of batches created from now on default to tile passes (0),
// tensor-core blocks (1) or blocks from kLockTcMinQubits qubits (2);
// returns the previous value.
int tfqg_internal_set_lock_tc(int mode) {
  return g_lock_tc.exchange(mode < 0 || mode > 2 ? 2 : mode);
}

// Lockstep tensor-core rows of later calls run as one persistent launch per
// group (1) or one launch per block index and variant (0); returns the
// previous setting.
int tfqg_internal_set_tc_lock_persistent(int on) {
  return g_tc_lock_persistent.exchange(on ? 1 : 0);
}

// Largest unit (chunks) and the units a lockstep tensor-core launch aims
// for, for batches created from now on (<= 0 keeps the value).
void tfqg_internal_set_tc_units(int64_t max_chunks, int64_t target) {
  if (max_chunks > 0) g_tc_unit_chunks.store(max_chunks);
  if (target > 0) g_tc_unit_target.store(target);
}

// Tensor-core blocks and units of a batch's lockstep rows (for tests).
int64_t tfqg_internal_batch_lock_tc(const tfqg_batch* b, int64_t* units) {
  if (!b) return -1;
  if (units) *units = int64_t(b->tcl_units.size());
  return int64_t(b->tcl_blocks.size());
}

// The persistent form's units in queue order, 6 values each (group, row
// slot, batch row, need, first chunk, chunks), at most `max` of them;
// returns their number.
int64_t tfqg_internal_batch_lock_punits(const tfqg_batch* b, int64_t* out, int64_t max) {
  if (!b) return -1;
  int64_t k = 0;
  for (size_t gi = 0; gi < b->lock_groups.size(); ++gi) {
    const auto& g = b->lock_groups[gi];
    for (int32_t u = g.tcp_begin; u < g.tcp_begin + g.tcp_count; ++u, ++k) {
      if (k >= max || !out) continue;
      const TcUnit& t = b->tcl_punits[size_t(u)];
      const int64_t v[6] = {int64_t(gi), t.slot, t.row, t.need, t.chunk0, t.nchunks};
      for (int i = 0; i < 6; ++i) out[6 * k + i] = v[i];
    }
  }
  return k;
}

// Qubit count from which streamed rows of batches created from now on run in
// lockstep in the forward modes (above 21: never); returns the previous value.
int tfqg_internal_set_lock_min_qubits(int n) { return g_lock_min_qubits.exchange(n); }

// Largest lockstep group (amplitudes of its rows' states) for batches created
// from now on; returns the previous value.
int64_t tfqg_internal_set_lock_arena_amps(int64_t amps) {
  return g_lock_arena_amps.exchange(amps);
}

// Lockstep groups of a batch.
int tfqg_internal_batch_lock_groups(void* batch) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  return b ? int(b->lock_groups.size()) : -1;
}

// Lockstep rows of a batch (forward modes).
int tfqg_internal_batch_lock_rows(void* batch) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  return b ? int(b->lock_rows.size()) : -1;
}

// Number of wide rows of a batch (forward modes).
int tfqg_internal_batch_wide_rows(void* batch) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  return b ? int(b->wide_rows.size()) : -1;
}

// FNV-1a hash of the batch's packed host tables: equal for batches that
// compile to the same programs, terms and plans.
uint64_t tfqg_internal_batch_fingerprint(void* batch) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  if (!b) return 0;
  std::vector<unsigned char> blob;
  pack_tables(b, &blob);
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : blob) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

int tfqg_internal_batch_row_costs(void* batch, double* costs) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  if (!b || (b->B > 0 && !costs)) return kInvalidArgument;
  for (int64_t i = 0; i < b->B; ++i) {
    const DevRow& r = b->rows[size_t(i)];
    const DevProgram& p = b->programs[r.program];
    costs[i] = r.n > 0 ? double(p.num_gates + 1) * std::ldexp(1.0, r.n) : 0.0;
  }
  return 0;
}

// The gates of row `row`'s forward plan in execution order, with their
// matrices bound to `row_values` on the host (the product the device builds
// for a fused gate).  Per gate, meta holds (nq, b0, b1, cmask, cval, kind)
// and mats 16 complex entries (row-major 2x2 or 4x4, b0 the MSB).  Returns
// the count in *count; at most `max` gates are written.
int tfqg_internal_forward_plan_gates(void* batch, int64_t row,
                                     const float* row_values, int32_t* meta,
                                     float* mats, int64_t max, int64_t* count) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  if (!b || row < 0 || row >= int64_t(b->rows.size()) || !count)
    return kInvalidArgument;
  const DevProgram& p = b->programs[b->rows[size_t(row)].program];
  const GateTemplate* gates = b->gates.data() + p.gate_begin;
  int64_t k = 0;
  for (uint32_t ps = p.fwd_pass_begin; ps < p.fwd_pass_end; ++ps)
    for (uint32_t o = b->passes[ps].op_begin; o < b->passes[ps].op_end; ++o) {
      const DevOp& op = b->ops[o];
      if (op.type != OP_F1 && op.type != OP_F2) continue;
      if (k < max) {
        const GateTemplate& g = gates[op.gate];
        Cx<double> m[16];
        int nq = g.nq;
        if (g.kind == GK_FUSED) {
          Cx<float> f[16];
          fused_product(gates, g,
                        [&](int k, Cx<float>* mf) {
                          Cx<double> md[16];
                          const int kq = bound_matrix(gates[k], row_values, md);
                          for (int i = 0; i < 16; ++i)
                            mf[i] = i < (kq == 1 ? 4 : 16)
                                        ? Cx<float>(float(md[i].re), float(md[i].im))
                                        : Cx<float>(0.f, 0.f);
                        },
                        f);
          for (int i = 0; i < 16; ++i) m[i] = Cx<double>(f[i].re, f[i].im);
        } else {
          nq = bound_matrix(g, row_values, m);
        }
        const int32_t mt[6] = {nq, g.b0, g.b1, int32_t(g.cmask), int32_t(g.cval),
                               g.kind};
        for (int i = 0; i < 6; ++i) meta[k * 6 + i] = mt[i];
        for (int i = 0; i < 16; ++i) {
          const bool in = i < (nq == 1 ? 4 : 16);
          mats[k * 32 + 2 * i] = in ? float(m[i].re) : 0.f;
          mats[k * 32 + 2 * i + 1] = in ? float(m[i].im) : 0.f;
        }
      }
      ++k;
    }
  *count = k;
  return 0;
}

int64_t tfqg_internal_batch_table_bytes(void* batch) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  // every table a forward call uploads: the packed batch tables, the
  // lockstep rows' tensor-core tables (the form in use) and the wide rows'
  // tensor-core plans
  std::vector<unsigned char> blob;
  pack_tables(b, &blob);
  size_t bytes = blob.size();
  if (!b->tcl_units.empty()) {
    blob.clear();
    tcl_blob(b, g_tc_lock_persistent.load() != 0, &blob);
    bytes += blob.size();
  }
  if (b->tc_planned)
    bytes += align256(b->tc_blocks.size() * sizeof(TcBlock)) + b->tc_members.size() * 4;
  return int64_t(bytes);
}

// Forward / backward pass counts and residency of program 0 (benchmark
// accounting of the state traffic the pass schedule moves).
int tfqg_internal_batch_passes(void* batch, int32_t* fwd, int32_t* bwd,
                               int32_t* resident) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  if (!b || b->programs.empty()) return kInvalidArgument;
  const DevProgram& p = b->programs[0];
  *fwd = int32_t(p.fwd_pass_end - p.fwd_pass_begin);
  *bwd = int32_t(p.bwd_pass_end - p.bwd_pass_begin);
  *resident = p.resident;
  return 0;
}

// State sweeps of row `row`: forward passes (each reads and writes the
// state once) and measurement passes (each reads it once).
int tfqg_internal_row_sweeps(void* batch, int64_t row, int32_t* fwd, int32_t* meas) {
  const tfqg_batch* b = static_cast<const tfqg_batch*>(batch);
  if (!b || row < 0 || row >= int64_t(b->rows.size()) || !fwd || !meas)
    return kInvalidArgument;
  const DevRow& r = b->rows[size_t(row)];
  const DevProgram& p = b->programs[r.program];
  *fwd = int32_t(p.fwd_pass_end - p.fwd_pass_begin);
  *meas = int32_t(r.meas_end - r.meas_begin);
  return 0;
}

// Sub-pass statistics of program 0: number of sub-pass headers and ops in
// the forward and backward instruction streams (planner diagnostics).
int tfqg_internal_batch_subpasses(void* batch, int32_t* fwd_subs,
                                  int32_t* fwd_ops, int32_t* bwd_subs,
                                  int32_t* bwd_ops) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  if (!b || b->programs.empty()) return kInvalidArgument;
  const DevProgram& p = b->programs[0];
  auto count = [&](uint32_t pb, uint32_t pe, int32_t* subs, int32_t* ops) {
    *subs = 0;
    *ops = 0;
    for (uint32_t q = pb; q < pe; ++q)
      for (uint32_t o = b->passes[q].op_begin; o < b->passes[q].op_end; ++o) {
        if (b->ops[o].type == OP_SUB) ++*subs; else ++*ops;
      }
  };
  count(p.fwd_pass_begin, p.fwd_pass_end, fwd_subs, fwd_ops);
  count(p.bwd_pass_begin, p.bwd_pass_end, bwd_subs, bwd_ops);
  return 0;
}

int tfqg_internal_plain_expect_adj(void* batch, const float* symbol_values,
                                   const float* downstream_grads,
                                   float* expectations, float* grads,
                                   void* stream, int64_t* launches) {
  tfqg_batch* b = static_cast<tfqg_batch*>(batch);
  return guarded([&]() {
    if (!b || b->kind != TFQG_KIND_ADJOINT)
      throw Error(kInvalidArgument, "needs an adjoint batch");
    if (b->programs.size() != 1 || b->B == 0)
      throw Error(kUnimplemented, "the plain path needs one shared program");
    for (const DevRow& r : b->rows)
      if (r.term_begin != b->rows[0].term_begin || r.term_end != b->rows[0].term_end)
        throw Error(kUnimplemented, "the plain path needs shared observables");
    const DevProgram& p = b->programs[0];
    if (p.n < 7) throw Error(kUnimplemented, "the plain path needs n >= 7");
    std::lock_guard<std::mutex> lk(b->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    RunArgs a;
    prepare(b, symbol_values, 1, true, 0, s, &a);
    const size_t sv = size_t(b->B) << p.n;
    b->work.reserve(2 * sv * sizeof(float2), b->device);
    size_t eb = align256(size_t(b->B * b->n_ops) * sizeof(double));
    size_t gb = size_t(b->B * b->P) * sizeof(double);
    b->aux2.reserve(eb + gb, b->device);
    TFQG_CUDA(cudaMemsetAsync(b->aux2.p, 0, eb + gb, s));
    PlainJob j;
    j.rows = int(b->B);
    j.n = p.n;
    j.num_gates = p.num_gates;
    j.num_grads = p.num_grads;
    j.num_terms = int(b->rows[0].term_end - b->rows[0].term_begin);
    j.n_ops = int(b->n_ops);
    j.num_symbols = int(b->P);
    j.gates = b->gates.data() + p.gate_begin;
    j.terms = b->terms.data() + b->rows[0].term_begin;
    j.grad_cols = b->grad_cols.data() + p.grad_col_begin;
    j.mats = a.mats;
    j.dmats = a.dmats;
    j.psi = static_cast<float2*>(b->work.p);
    j.lam = j.psi + sv;
    j.dgrads = downstream_grads;
    j.acc_exp = static_cast<double*>(b->aux2.p);
    j.acc_grad = reinterpret_cast<double*>(static_cast<char*>(b->aux2.p) + eb);
    j.out_exp = expectations;
    j.out_grad = grads;
    int64_t n0 = 0;
    TFQG_CUDA(plain_expect_adjoint(j, s, &n0));
    if (launches) *launches = n0 + 1;  // + the matrix build
    return 0;
  });
}

}  // extern "C"
