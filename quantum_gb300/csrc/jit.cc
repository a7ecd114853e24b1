// Batch-specialized sub-pass code, compiled at run time with NVRTC.
//
// The interpreter (kernels.cu) decodes every gate of a sub-pass at run time;
// that dispatch costs about as much as the arithmetic itself.  For a batch
// whose sub-passes fall into few distinct *signatures* (the sequence of packed
// op codes: gate class, register bits, register controls, gradient count),
// this file generates one straight-line device function per signature, with
// all of those as compile-time constants, plus executors that switch on the
// signature id recorded in each sub-pass header.  Matrices and non-register
// controls stay run-time data (staged in shared memory as before), so one
// compiled module serves every set of symbol values.  The module is cached
// per generated source, in process and on disk.
#include "jit.h"

#include <dlfcn.h>
#include <nvrtc.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <map>
#include <unordered_map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "batch_internal.h"

namespace tfqg {

// Embedded copies of the device headers (generated by the build).
extern const char* const kJitHeaderNames[];
extern const char* const kJitHeaderSources[];
extern const int kJitHeaderCount;

namespace {

constexpr int kMaxSignatures = 512;

// kernel names per SimMode, then the wide-row forward pass
const char* kModeNames[kJitModes] = {"tfqg_jit_expect", "tfqg_jit_state",
                                     "tfqg_jit_sample", "tfqg_jit_adjoint",
                                     "tfqg_jit_noisy", "tfqg_jit_wide"};
const char* kModeEnums[5] = {"kModeExpect", "kModeState", "kModeSample",
                             "kModeAdjoint", "kModeNoisy"};

// One compiled module: the kernel of one mode, loaded per device on demand.
struct Loaded {
  std::vector<char> cubin;
  int mode = 0;
  cudaLibrary_t lib[64] = {};
  cudaKernel_t kernel[64] = {};
};

// NVRTC is loaded at run time so that the library works (interpreter only)
// where it is absent.
struct Nvrtc {
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcVersion) version = nullptr;
  bool ok = false;
};

const Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", TFQG_CUDA_LIB_DIR "/libnvrtc.so.13",
                           TFQG_CUDA_LIB_DIR "/libnvrtc.so"};
    void* h = nullptr;
    for (const char* nm : names)
      if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return;
    n.create = reinterpret_cast<decltype(n.create)>(dlsym(h, "nvrtcCreateProgram"));
    n.compile = reinterpret_cast<decltype(n.compile)>(dlsym(h, "nvrtcCompileProgram"));
    n.log_size = reinterpret_cast<decltype(n.log_size)>(dlsym(h, "nvrtcGetProgramLogSize"));
    n.log = reinterpret_cast<decltype(n.log)>(dlsym(h, "nvrtcGetProgramLog"));
    n.cubin_size = reinterpret_cast<decltype(n.cubin_size)>(dlsym(h, "nvrtcGetCUBINSize"));
    n.cubin = reinterpret_cast<decltype(n.cubin)>(dlsym(h, "nvrtcGetCUBIN"));
    n.destroy = reinterpret_cast<decltype(n.destroy)>(dlsym(h, "nvrtcDestroyProgram"));
    n.version = reinterpret_cast<decltype(n.version)>(dlsym(h, "nvrtcVersion"));
    n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy;
  });
  return n;
}

std::mutex g_mu;
std::map<std::string, std::shared_ptr<Loaded>> g_cache;  // source -> module

// Compile options of every specialized module (sm_103a only).
const char* const kNvrtcOptions[] = {"--gpu-architecture=sm_103a", "-std=c++17",
                                     "-DTFQG_JIT=1", "--ptxas-options=-v"};

uint64_t fnv1a(const std::string& s) {
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

// Hash of everything besides the generated source that determines a
// module: the embedded device headers, the compile options and the NVRTC
// version.  It keys the disk cache together with the source, so a library
// built from changed headers never loads a module compiled from old ones.
uint64_t toolchain_hash() {
  static uint64_t h = [] {
    std::string all;
    for (int i = 0; i < kJitHeaderCount; ++i) {
      all += kJitHeaderNames[i];
      all += kJitHeaderSources[i];
    }
    for (const char* o : kNvrtcOptions) all += o;
    int major = 0, minor = 0;
    const Nvrtc& nv = nvrtc();
    if (nv.version) nv.version(&major, &minor);
    all += std::to_string(major) + "." + std::to_string(minor);
    return fnv1a(all);
  }();
  return h;
}

const char* cls_name(int cls) {
  switch (cls) {
    case GC_REAL: return "real";
    case GC_DIAG: return "diag";
    case GC_X: return "x";
    default: return "general";
  }
}

// One forward op of a signature: reads array `in`, writes `out`.
void emit_forward_op(std::ostringstream& o, int i, uint32_t code,
                     const char* in, const char* out) {
  const int type = code & 7, cls = (code >> 3) & 7, j0 = (code >> 6) & 3,
            j1 = (code >> 8) & 3, km = (code >> 10) & 15, kv = (code >> 14) & 15;
  const bool ctrl = (code >> 20) & 1, single = (code >> 21) & 1;
  const int jc = (code >> 22) & 3, cv = (code >> 24) & 1;
  std::ostringstream call;
  if (type == OP_MCH) {
    // the branch (identity or a Kraus matrix) is drawn at staging time
    call << "if (((st->code[" << i << "] >> 3) & 7) == GC_SKIP) copy_regs(" << in
         << ", " << out << "); else f1_general<" << j0 << ", NA>(" << in << ", "
         << out << ", st->mat[" << i << "], 0, 0);";
  } else if (type == OP_F1) {
    if (cls == GC_SKIP) {
      call << "copy_regs(" << in << ", " << out << ");";
    } else if (cls == GC_X && km && single) {
      call << "f1_cx<" << j0 << ", " << jc << ", " << cv << ", NA>(" << in << ", "
           << out << ");";
    } else if (cls == GC_X) {
      call << "f1_x<" << j0 << ", NA>(" << in << ", " << out << ", " << km << ", "
           << kv << ");";
    } else {
      call << "f1_" << cls_name(cls) << "<" << j0 << ", NA>(" << in << ", " << out
           << ", st->mat[" << i << "], " << km << ", " << kv << ");";
    }
  } else {
    call << "f2_" << (cls == GC_DIAG ? "diag" : "general") << "<" << j0 << ", "
         << j1 << ", NA>(" << in << ", " << out << ", st->mat[" << i << "], " << km
         << ", " << kv << ");";
  }
  if (ctrl) {
    o << "    if (op_active(st, " << i << ", " << code << "u, gb, base)) { "
      << call.str() << " } else { copy_regs(" << in << ", " << out << "); }\n";
  } else {
    o << "    " << call.str() << "\n";
  }
}

void emit_forward(std::ostringstream& o, int id, const std::vector<uint32_t>& codes) {
  o << "__device__ __noinline__ void jit_sub_" << id
    << "(uint32_t s_off, int T, uint32_t base, uint32_t st_off, uint32_t rbits) {\n"
       "  constexpr int RB = kFwdRB, NA = 1 << RB;\n"
       "  float2* s = reinterpret_cast<float2*>(smem_raw + s_off);\n"
       "  const Stage* st = reinterpret_cast<const Stage*>(smem_raw + st_off);\n"
       "  // swz is XOR-linear: the offset of amplitude k is the XOR of the\n"
       "  // offsets of its register bits\n"
       "  const uint32_t o0 = swz(1u << (rbits & 0xFF)), o1 = swz(1u << ((rbits >> 8) & 0xFF));\n"
       "  const uint32_t o2 = swz(1u << ((rbits >> 16) & 0xFF)), o3 = swz(1u << (rbits >> 24));\n"
       "  const uint32_t ngroups = 1u << (T - RB);\n"
       "  for (uint32_t g = threadIdx.x; g < ngroups; g += blockDim.x) {\n"
       "    const uint32_t gb = group_base(g, rbits, RB);\n"
       "    const uint32_t sgb = swz(gb);\n"
       "    float2 A[NA], B[NA];\n"
       "#pragma unroll\n"
       "    for (int k = 0; k < NA; ++k)\n"
       "      A[k] = s[sgb ^ (k & 1 ? o0 : 0u) ^ (k & 2 ? o1 : 0u) ^ (k & 4 ? o2 : 0u) ^ (k & 8 ? o3 : 0u)];\n"
       "    (void)base;\n";
  for (size_t i = 0; i < codes.size(); ++i)
    emit_forward_op(o, int(i), codes[i], i % 2 ? "B" : "A", i % 2 ? "A" : "B");
  const char* fin = codes.size() % 2 ? "B" : "A";
  o << "#pragma unroll\n"
       "    for (int k = 0; k < NA; ++k)\n"
       "      s[sgb ^ (k & 1 ? o0 : 0u) ^ (k & 2 ? o1 : 0u) ^ (k & 4 ? o2 : 0u) ^ (k & 8 ? o3 : 0u)] = "
    << fin << "[k];\n  }\n}\n\n";
}

void emit_backward(std::ostringstream& o, int id, const std::vector<uint32_t>& codes) {
  // gradient entries of the sub-pass; up to kRegGradEntries of them are
  // accumulated in registers over the group iterations and warp-reduced once
  constexpr int kRegGradEntries = 16;
  int entries = 0;
  for (uint32_t code : codes)
    if ((code & 7) == OP_B1 || (code & 7) == OP_B2) entries += (code >> 18) & 3;
  const bool in_regs = entries <= kRegGradEntries;
  o << "__device__ __noinline__ void jit_sub_" << id
    << "(uint32_t s_off, uint32_t l_off, int T, uint32_t base, uint32_t st_off,"
       " uint32_t rb_off, uint32_t rbits, int rbuf) {\n"
       "  constexpr int RB = kBwdRB, NA = 1 << RB;\n"
       "  float2* s = reinterpret_cast<float2*>(smem_raw + s_off);\n"
       "  float2* l = reinterpret_cast<float2*>(smem_raw + l_off);\n"
       "  const Stage* st = reinterpret_cast<const Stage*>(smem_raw + st_off);\n"
       "  RedBuf* rb = reinterpret_cast<RedBuf*>(smem_raw + rb_off);\n"
       "  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;\n"
       "  uint32_t soff[NA];\n"
       "#pragma unroll\n"
       "  for (int k = 0; k < NA; ++k) {\n"
       "    uint32_t o = 0;\n"
       "#pragma unroll\n"
       "    for (int j = 0; j < RB; ++j) if (k >> j & 1) o |= 1u << ((rbits >> (8 * j)) & 0xFF);\n"
       "    soff[k] = swz(o);\n"
       "  }\n"
       "  const uint32_t ngroups = 1u << (T - RB);\n"
       "  const uint32_t iters = (ngroups + blockDim.x - 1) / blockDim.x;\n";
  // accumulator count padded to a power of two for warp_sum_many
  int padded = 1, lg = 0;
  while (padded < entries) { padded <<= 1; ++lg; }
  if (in_regs && entries) {
    o << "  float gp[" << padded << "];\n#pragma unroll\n  for (int e = 0; e < " << padded
      << "; ++e) gp[e] = 0.f;\n";
  }
  o << "  for (uint32_t it = 0; it < iters; ++it) {\n"
       "    const uint32_t g = it * blockDim.x + threadIdx.x;\n"
       "    const bool active = g < ngroups;\n"
       "    const uint32_t gb = group_base(active ? g : 0u, rbits, RB);\n"
       "    const uint32_t sgb = swz(gb);\n"
       "    float2 A[NA], LA[NA], B[NA], LB[NA];\n"
       "    if (active) {\n"
       "#pragma unroll\n"
       "      for (int k = 0; k < NA; ++k) { A[k] = s[sgb ^ soff[k]]; LA[k] = l[sgb ^ soff[k]]; }\n"
       "    } else {\n"
       "#pragma unroll\n"
       "      for (int k = 0; k < NA; ++k) { A[k] = make_float2(0.f, 0.f); LA[k] = A[k]; }\n"
       "    }\n"
       "    (void)base; (void)lane; (void)warp;\n";
  int gi = 0;
  for (size_t i = 0; i < codes.size(); ++i) {
    const uint32_t code = codes[i];
    const char *a = i % 2 ? "B" : "A", *la = i % 2 ? "LB" : "LA";
    const char *b = i % 2 ? "A" : "B", *lb = i % 2 ? "LA" : "LB";
    const int cls = (code >> 3) & 7, j0 = (code >> 6) & 3, j1 = (code >> 8) & 3,
              km = (code >> 10) & 15, kv = (code >> 14) & 15,
              ng = (code >> 18) & 3;
    const bool ctrl = (code >> 20) & 1, single = (code >> 21) & 1;
    const int jc = (code >> 22) & 3, cv = (code >> 24) & 1;
    const bool one = (code & 7) == OP_B1;
    std::ostringstream call;
    if (one && cls == GC_X && km && single) {
      call << "f1_cx<" << j0 << ", " << jc << ", " << cv << ", NA>(" << a << ", " << b
           << "); f1_cx<" << j0 << ", " << jc << ", " << cv << ", NA>(" << la << ", "
           << lb << ");";
    } else if (one) {
      call << "b1_" << cls_name(cls) << "<" << j0 << ", NA, " << ng << ">(" << a << ", "
           << la << ", " << b << ", " << lb << ", st->mat[" << i << "], &st->dmat[" << i
           << "][0][0], " << km << ", " << kv << ", part);";
    } else {
      call << "b2_" << (cls == GC_DIAG ? "diag" : "general") << "<" << j0 << ", " << j1
           << ", NA, " << ng << ">(" << a << ", " << la << ", " << b << ", " << lb
           << ", st->mat[" << i << "], &st->dmat[" << i << "][0][0], " << km << ", "
           << kv << ", part);";
    }
    o << "    {\n      float part[2] = {0.f, 0.f};\n      (void)part;\n";
    std::string cond = "active";
    if (ctrl)
      cond += " && op_active(st, " + std::to_string(i) + ", " + std::to_string(code) +
              "u, gb, base)";
    o << "      if (" << cond << ") { " << call.str() << " } else { copy_regs(" << a << ", " << b
      << "); copy_regs(" << la << ", " << lb << "); }\n";
    for (int q = 0; q < ng; ++q) {
      if (in_regs)
        o << "      gp[" << gi + q << "] += part[" << q << "];\n";
      else
        o << "      { float v = warp_sum(part[" << q << "]); if (lane == 0) { if (it == 0) rb->red[rbuf]["
          << gi + q << "][warp] = v; else rb->red[rbuf][" << gi + q << "][warp] += v; } }\n";
    }
    o << "    }\n";
    gi += ng;
  }
  const char* fin = codes.size() % 2 ? "B" : "A";
  const char* lfin = codes.size() % 2 ? "LB" : "LA";
  o << "    if (active) {\n#pragma unroll\n"
       "      for (int k = 0; k < NA; ++k) { s[sgb ^ soff[k]] = "
    << fin << "[k]; l[sgb ^ soff[k]] = " << lfin << "[k]; }\n    }\n  }\n";
  if (in_regs && entries) {
    // value j of the warp sums ends in lanes whose bits 4 .. 5 - lg spell j
    const int low = 5 - lg;
    o << "  {\n    const float v = warp_sum_many<" << padded << ">(gp, lane);\n"
      << "    const int j = lane >> " << low << ";\n"
      << "    if (j < " << entries << " && (lane & " << ((1 << low) - 1)
      << ") == 0) rb->red[rbuf][j][warp] = v;\n  }\n";
  }
  o << "}\n\n";
}

std::string cache_dir() {
  const char* x = getenv("TFQG_CACHE_DIR");
  std::string d;
  if (x && *x) {
    d = x;
  } else {
    const char* xdg = getenv("XDG_CACHE_HOME");
    const char* home = getenv("HOME");
    if (xdg && *xdg) d = std::string(xdg) + "/tfq_gb300";
    else if (home && *home) d = std::string(home) + "/.cache/tfq_gb300";
    else return "";
  }
  return d;
}

void mkdirs(const std::string& d) {
  std::string cur;
  for (size_t i = 0; i < d.size(); ++i) {
    cur += d[i];
    if (d[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(d.c_str(), 0755);
}

bool read_file(const std::string& path, std::vector<char>* out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  out->resize(size_t(n));
  bool ok = n > 0 && fread(out->data(), 1, size_t(n), f) == size_t(n);
  fclose(f);
  return ok;
}

void write_file(const std::string& path, const std::vector<char>& data) {
  std::string tmp = path + ".tmp" + std::to_string(getpid());
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return;
  bool ok = fwrite(data.data(), 1, data.size(), f) == data.size();
  fclose(f);
  if (ok) rename(tmp.c_str(), path.c_str());
  else remove(tmp.c_str());
}

// Compiles `src` for sm_103a; returns the CUBIN.  With `info`, ptxas also
// reports resource usage (registers, spills, shared memory) into *info.
std::vector<char> nvrtc_compile(const std::string& src, std::string* info = nullptr) {
  const Nvrtc& nv = nvrtc();
  if (!nv.ok) throw Error(kUnimplemented, "NVRTC is not available");
  nvrtcProgram prog;
  if (nv.create(&prog, src.c_str(), "tfqg_jit.cu", kJitHeaderCount,
                kJitHeaderSources, kJitHeaderNames) != NVRTC_SUCCESS)
    throw Error(kInternal, "nvrtcCreateProgram failed");
  nvrtcResult r = nv.compile(prog, info ? 4 : 3, kNvrtcOptions);
  size_t n = 0;
  nv.log_size(prog, &n);
  std::string log(n, '\0');
  if (n) nv.log(prog, &log[0]);
  if (r != NVRTC_SUCCESS) {
    nv.destroy(&prog);
    throw Error(kInternal, "NVRTC compile failed: " + log.substr(0, 2000));
  }
  if (info) *info = log;
  size_t bytes = 0;
  nv.cubin_size(prog, &bytes);
  std::vector<char> cubin(bytes);
  nv.cubin(prog, cubin.data());
  nv.destroy(&prog);
  return cubin;
}

}  // namespace

struct SignatureHash {
  size_t operator()(const std::vector<uint32_t>& v) const {
    uint64_t h = 0xcbf29ce484222325ull;
    for (const uint32_t x : v) h = (h ^ x) * 0x100000001b3ull;
    return size_t(h ^ (h >> 29));
  }
};

void jit_assign_signatures(tfqg_batch* b) {
  std::unordered_map<std::vector<uint32_t>, int, SignatureHash> ids;
  b->jit_signatures.clear();
  for (size_t o = 0; o < b->ops.size(); ++o) {
    DevOp& h = b->ops[o];
    if (h.type != OP_SUB) continue;
    std::vector<uint32_t> key;
    key.push_back(h.t0);  // register bits (4 forward, 3 adjoint)
    for (uint32_t i = 0; i < h.gate; ++i) key.push_back(op_code(b->ops[o + 1 + i]));
    auto it = ids.find(key);
    int id;
    if (it == ids.end()) {
      id = int(b->jit_signatures.size());
      ids.emplace(key, id);
      b->jit_signatures.push_back(key);
    } else {
      id = it->second;
    }
    h.grad_slot = id;
  }
}

std::string jit_source(const tfqg_batch* b, int mode) {
  // backward signatures (3 register bits) run only in the adjoint sweep
  const bool adj = mode == kModeAdjoint;
  auto used = [&](size_t id) { return adj || b->jit_signatures[id][0] != 3; };
  std::ostringstream o;
  o << "// generated: " << kModeNames[mode] << ", " << b->jit_signatures.size()
    << " sub-pass signatures\n"
       "#include \"sim_device.cuh\"\nnamespace tfqg {\nnamespace {\n\n";
  for (size_t id = 0; id < b->jit_signatures.size(); ++id) {
    if (!used(id)) continue;
    const auto& key = b->jit_signatures[id];
    std::vector<uint32_t> codes(key.begin() + 1, key.end());
    if (key[0] == 3) emit_backward(o, int(id), codes);
    else emit_forward(o, int(id), codes);
  }
  o << "struct JitExec {\n"
       "  static __device__ __forceinline__ void forward(uint32_t so, int T, uint32_t base,"
       " uint32_t sto, int nops, uint32_t rbits, int sig) {\n    switch (sig) {\n";
  for (size_t id = 0; id < b->jit_signatures.size(); ++id)
    if (b->jit_signatures[id][0] != 3)
      o << "      case " << id << ": jit_sub_" << id << "(so, T, base, sto, rbits); break;\n";
  o << "      default: break;\n    }\n    (void)nops;\n  }\n"
       "  static __device__ __forceinline__ void backward(uint32_t so, uint32_t lo, int T,"
       " uint32_t base, uint32_t sto, uint32_t rbo, int nops, uint32_t rbits, int rbuf,"
       " int sig) {\n"
       "    switch (sig) {\n";
  for (size_t id = 0; id < b->jit_signatures.size(); ++id)
    if (adj && b->jit_signatures[id][0] == 3)
      o << "      case " << id << ": jit_sub_" << id
        << "(so, lo, T, base, sto, rbo, rbits, rbuf); break;\n";
  o << "      default: break;\n    }\n    (void)nops;\n  }\n};\n\n}  // namespace\n\n";
  if (mode == kJitWide)
    o << "extern \"C\" __global__ void __launch_bounds__(kWideThreads, 2) " << kModeNames[mode]
      << "(BatchDevice b, RunArgs a, int row, int pass, int init, float2* psi,"
         " int state_amps) {\n"
         "  wide_pass_body<JitExec>(b, a, row, pass, init, psi, state_amps);\n}\n";
  else
    o << "extern \"C\" __global__ void __launch_bounds__(" << jit_threads(mode) << ", 1) "
      << kModeNames[mode]
      << "(BatchDevice b, RunArgs a, int state_amps, int nstates) {\n"
         "  simulate_body<"
      << kModeEnums[mode] << ", JitExec>(b, a, state_amps, nstates);\n}\n";
  o << "}  // namespace tfqg\n";
  return o.str();
}

bool jit_enabled_for(const tfqg_batch* b) {
  const char* env = getenv("TFQG_JIT");
  if (b->jit_mode < 0 || (env && strcmp(env, "0") == 0)) return false;
  if (b->jit_signatures.empty() || b->jit_signatures.size() > size_t(kMaxSignatures))
    return false;
  if (b->jit_mode > 0 || (env && strcmp(env, "1") == 0)) return true;
  // enough work to amortize a compile: amplitude-gate updates per call
  double work = 0;
  for (const DevRow& r : b->rows)
    work += double(b->programs[r.program].num_gates) * double(uint64_t(1) << r.n);
  return work >= 2e8;
}

// Returns the specialized kernel for `mode`, compiling and loading the
// batch's module on first use; nullptr when specialization is off or fails
// (the caller then uses the interpreter).
cudaKernel_t jit_kernel(tfqg_batch* b, int mode, int dev) {
  if (!jit_enabled_for(b) || dev < 0 || dev >= 64 || mode < 0 || mode >= kJitModes)
    return nullptr;
  if (!b->jit_loaded[mode]) {
    b->jit_loaded[mode] = true;  // one attempt per batch and mode
    try {
      std::string src = jit_source(b, mode);
      std::shared_ptr<Loaded> mod;
      {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_cache.find(src);
        if (it != g_cache.end()) mod = it->second;
      }
      if (!mod) {
        mod = std::make_shared<Loaded>();
        mod->mode = mode;
        std::string dir = cache_dir();
        char name[64];
        snprintf(name, sizeof(name), "/jit_%016llx_%016llx_%zu.cubin",
                 (unsigned long long)toolchain_hash(), (unsigned long long)fnv1a(src),
                 src.size());
        std::string path = dir.empty() ? "" : dir + name;
        if (path.empty() || !read_file(path, &mod->cubin)) {
          mod->cubin = nvrtc_compile(src);
          if (!path.empty()) {
            mkdirs(dir);
            write_file(path, mod->cubin);
          }
        }
        std::lock_guard<std::mutex> lk(g_mu);
        g_cache[src] = mod;
      }
      b->jit_module[mode] = mod;
    } catch (const Error& e) {
      b->jit_error = e.what();
      b->jit_module[mode].reset();
      return nullptr;
    }
  }
  if (!b->jit_module[mode]) return nullptr;
  Loaded* mod = static_cast<Loaded*>(b->jit_module[mode].get());
  std::lock_guard<std::mutex> lk(g_mu);
  if (!mod->lib[dev]) {
    if (cudaLibraryLoadData(&mod->lib[dev], mod->cubin.data(), nullptr, nullptr,
                            0, nullptr, nullptr, 0) != cudaSuccess) {
      cudaGetLastError();
      mod->lib[dev] = nullptr;
      b->jit_error = "cudaLibraryLoadData failed";
      return nullptr;
    }
  }
  if (!mod->kernel[dev]) {
    if (cudaLibraryGetKernel(&mod->kernel[dev], mod->lib[dev], kModeNames[mode]) !=
        cudaSuccess) {
      cudaGetLastError();
      mod->kernel[dev] = nullptr;
      b->jit_error = std::string("kernel not in module: ") + kModeNames[mode];
      return nullptr;
    }
  }
  return mod->kernel[dev];
}

// Generates and compiles the batch's specialized source without loading it
// (no GPU needed).  Returns 0 on success; `log` receives the error text.
int jit_compile_check(tfqg_batch* b, int mode, std::string* log) {
  if (mode < 0 || mode >= kJitModes) return kInvalidArgument;
  try {
    std::vector<char> cubin = nvrtc_compile(jit_source(b, mode), log);
    return cubin.empty() ? kInternal : 0;
  } catch (const Error& e) {
    *log = e.what();
    return e.code;
  }
}

int jit_grid(cudaKernel_t k, size_t smem, int dev, int threads) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(smem), dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, reinterpret_cast<const void*>(k), threads, smem) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

// Threads per CTA of the specialized persistent kernel of `mode`.  (1024
// threads for the adjoint, whose backward sub-passes fit the 64 registers a
// thread then has, measured no faster than 512.)
int jit_threads(int mode) {
  (void)mode;
  return kSimThreads;
}

cudaError_t jit_launch(cudaKernel_t k, const BatchDevice& bd, const RunArgs& a,
                       int grid, size_t smem, int state_amps, int nstates,
                       cudaStream_t s, int threads) {
  BatchDevice b = bd;
  RunArgs ra = a;
  void* args[] = {&b, &ra, &state_amps, &nstates};
  return cudaLaunchKernel(reinterpret_cast<const void*>(k), dim3(grid),
                          dim3(threads), args, smem, s);
}

cudaError_t jit_launch_wide(cudaKernel_t k, const BatchDevice& bd, const RunArgs& a,
                            int row, int pass, int init, float2* psi, int grid,
                            size_t smem, int state_amps, cudaStream_t s) {
  BatchDevice b = bd;
  RunArgs ra = a;
  void* args[] = {&b, &ra, &row, &pass, &init, &psi, &state_amps};
  return cudaLaunchKernel(reinterpret_cast<const void*>(k), dim3(grid),
                          dim3(kWideThreads), args, smem, s);
}

}  // namespace tfqg
