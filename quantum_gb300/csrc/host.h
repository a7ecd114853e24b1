// Host side of the path: decode serialized programs / Pauli sums, resolve
// qubits and symbols, build gate templates and plan tile passes.
#pragma once
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "tfqg_types.h"

namespace tfqg {

// Status codes follow tensorflow::error::Code numbering.
enum StatusCode {
  kOk = 0,
  kInvalidArgument = 3,
  kResourceExhausted = 8,
  kUnimplemented = 12,
  kInternal = 13,
};

struct Error : public std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ---- decoded wire messages (tensorflow_quantum/core/proto/*.proto) ----
struct ArgP {
  float f = 0.f;        // arg_value.float_value
  std::string symbol;   // symbol
  std::string str;      // arg_value.string_value
};

struct OpP {
  std::string gate;
  std::vector<std::pair<std::string, ArgP>> args;  // map entries, last wins
  std::vector<std::string> qubits;
  const ArgP* find(const std::string& key) const;
};

struct ProgramP {
  std::vector<std::vector<OpP>> moments;
};

struct TermP {
  float re = 0.f, im = 0.f;
  std::vector<std::pair<std::string, std::string>> paulis;  // (qubit id, type)
};
using PauliSumP = std::vector<TermP>;

void decode_program(const char* data, size_t len, ProgramP* out);
// Protobuf text format of a Program (pauli_sum = false) or PauliSum,
// re-encoded in the binary wire format; false if it does not parse.
bool text_proto_to_wire(const char* data, size_t len, bool pauli_sum, std::string* wire);
void decode_paulisum(const char* data, size_t len, PauliSumP* out);

// absl::SimpleAtoi semantics: optional surrounding whitespace and sign.
bool simple_atoi(const std::string& s, int64_t* out);

// ---- compiled programs ----
enum JobKind { kJobForward = 0, kJobAdjoint = 1, kJobNoisy = 2 };

// Largest qubit count kept resident in shared memory (one CTA per circuit).
constexpr int kResidentMaxSingle = 14;   // one state: 2^14 * 8 B = 128 KiB
constexpr int kResidentMaxAdjoint = 13;  // psi and lambda: 2 * 64 KiB
constexpr int kStreamTileBits = 13;      // tile of a streamed pass: 64 KiB
constexpr int kLaneBits = 5;             // low bits every streamed tile holds
constexpr int kRegBits = 4;              // register bits of a sub-pass (16 amps)
constexpr int kRegBitsAdjoint = 3;       // adjoint sub-passes (psi + lambda)
constexpr int kMaxSubOps = 32;           // ops per sub-pass (staging limit)

struct ChannelHost {
  DevChannel dev;
  int bit = 0;                // target bit
  std::vector<double> kraus;  // nk * 8 doubles (2x2 complex)
};

struct CompiledProgram {
  int n = 0;
  bool resident = true;
  std::vector<GateTemplate> gates;
  std::vector<int32_t> grad_col;      // derivative slot -> symbol column
  std::vector<ChannelHost> channels;  // noisy programs
  // op list in program order: gate index, or ~channel index (< 0)
  std::vector<int32_t> sequence;
  std::vector<DevPass> fwd_passes, bwd_passes;
  std::vector<DevOp> fwd_ops, bwd_ops;
  bool empty() const { return n == 0 || sequence.empty(); }
};

struct SymbolTable {
  std::unordered_map<std::string, int> col;  // name -> column (last wins)
  int64_t num_symbols = 0;
};

// Builds the gate templates of `prog` (circuit_parser_qsim.cc:828-861 /
// 773-826 for noisy programs).  `names` resolves symbols; errors mirror the
// reference messages.  `index` maps qubit id -> resolved index.
void compile_program(const ProgramP& prog, const SymbolTable& names,
                     JobKind kind, CompiledProgram* out,
                     std::unordered_map<std::string, int>* index);

// Resolves qubit ids (program_resolution.cc:90-186).
int resolve_qubits(const ProgramP& prog,
                   std::unordered_map<std::string, int>* index);

// A paired circuit of tfq_inner_product must use exactly the reference
// circuit's qubits (program_resolution.cc:188-310); `index` is the reference
// circuit's map.  Throws with the reference's messages.
void check_paired_qubits(const ProgramP& other,
                         const std::unordered_map<std::string, int>& index);

// Structure class (GateClass) of a gate template.
uint8_t classify_gate(const GateTemplate& g);

// Plans forward (and, for the adjoint, backward) passes.
void plan_program(CompiledProgram* prog, JobKind kind, bool fuse = false);

// Tensor-core blocks of a forward program (tc_gates.cu): its gates
// (gates[0, num_gates) in program order, GK_FUSED products and identities
// skipped) grouped into blocks of at most 5 bits each, appended to `blocks`
// and `members` (member ranges index `members`).  A gate depends on the
// previous gate on each of its bits (targets and controls); the "front" is
// the gates whose dependencies are all placed.  A block grows from a front
// gate by taking, again and again, the front gate that adds the fewest new
// bits while the block stays within 5 bits; of all front gates as seeds,
// the one whose block takes the most gates wins.  Members are in the order
// taken, which respects every dependency.  Blocks are padded to 5 bits with
// the highest free bits, which keeps the low index bits for coalesced group
// addressing.  Returns false (appending nothing) when a gate spans more than
// 5 bits or n is outside [12, 31].
bool plan_tc_blocks(const GateTemplate* gates, int num_gates, int n,
                    std::vector<TcBlock>* blocks, std::vector<int32_t>* members);

// Groups terms [tb, te) into measurement passes: each pass's tile holds the
// flip bits of all its terms (resident rows: one pass over the whole state).
constexpr int kMaxMeasTerms = 128;  // terms per measurement pass
void plan_measurement(const std::vector<DevTerm>& terms, uint32_t tb,
                      uint32_t te, int n, bool resident,
                      std::vector<DevMeas>* passes,
                      std::vector<DevMeasTerm>* list);

// Pauli sum -> device terms for column `op` (bits relative to n qubits).
void lower_paulisum(const PauliSumP& ps,
                    const std::unordered_map<std::string, int>& index, int n,
                    int op, std::vector<DevTerm>* out);

}  // namespace tfqg
