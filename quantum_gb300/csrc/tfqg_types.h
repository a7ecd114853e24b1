// Data structures shared by the host compiler and the sm_103a kernels.
//
// State layout: one complex64 vector per circuit (or trajectory), float2
// interleaved, amplitude index x whose bit b is qubit (n-1-b) in TFQ's
// resolved qubit order (program_resolution.cc:120-131 sorts qubits; the
// first qubit is the most significant bit, circuit_parser_qsim.cc:161 maps
// qubit q to simulator index n-q-1).  Bit positions below are these "bits".
#pragma once
#ifdef __CUDACC_RTC__
#include "rtc_types.h"
#else
#include <stdint.h>
#endif

namespace tfqg {

// Gate kinds: the 16 gate ids of circuit_parser_qsim.cc:577-584.
enum GateKind : uint8_t {
  GK_I1 = 0, GK_I2, GK_XP, GK_YP, GK_ZP, GK_HP, GK_XXP, GK_YYP, GK_ZZP,
  GK_CZP, GK_CNP, GK_SP, GK_ISP, GK_PXP, GK_FSIM, GK_PISP, GK_COUNT,
  // Product of several gates of one program on one or two bits, made by the
  // host's gate fuser for forward plans; its matrix is built on the device
  // from the members' matrices (GateTemplate::link).
  GK_FUSED = 32
};

// Placement of a fused gate's member inside the fused matrix.
enum FusePos : uint8_t {
  FP_HIGH = 0,     // 1-qubit member on the fused gate's b0 (matrix MSB)
  FP_LOW = 1,      // 1-qubit member on b1
  FP_SAME = 2,     // 2-qubit member with the fused gate's (b0, b1)
  FP_SWAPPED = 3   // 2-qubit member on (b1, b0)
};

// Upper bound on the members of one fused gate.
constexpr int kMaxFuseMembers = 64;

// Channel kinds: the 8 channel ids of circuit_parser_qsim.cc:757-761.
enum ChannelKind : uint8_t {
  CK_DP = 0, CK_ADP, CK_GAD, CK_AD, CK_RST, CK_PD, CK_PF, CK_BF
};

// One gate of a distinct program, with its parameters still unbound.
// a[i] is the constant from the proto, replaced per batch row by
// symbol_values[row, src[i]] when src[i] >= 0 (ParseProtoArg,
// circuit_parser_qsim.cc:53-82).  Parameter k (0 or 1) of the gate is the
// raw value a[2k] times the scalar a[2k+1]; eigen gates use a[0]*a[1] as
// exponent and a[2] as global shift, PhasedX uses a[4] as global shift.
struct GateTemplate {
  uint8_t kind;
  uint8_t nq;          // 1 or 2 targets
  uint8_t b0, b1;      // target bits; b0 is the first listed qubit (matrix MSB)
  uint32_t cmask;      // control bits
  uint32_t cval;       // required control values on those bits
  float a[5];
  int16_t src[5];      // symbol column of a[i], or -1
  uint8_t ngrad;       // symbolic parameters = derivative slots
  uint8_t gparam[2];   // parameter (0 or 1) differentiated by each slot
  uint8_t cls;         // GateClass
  int32_t grad_slot;   // first derivative slot of this gate, or -1
  // Fusion links: a GK_FUSED gate names its first member here, and each
  // member names the next one (-1 ends the list; members are in time order).
  int32_t link;
  uint8_t fpos;        // FusePos of a member
};

// Structure class of a gate matrix, chosen on the host; the kernels use the
// cheapest arithmetic the class allows.
enum GateClass : uint8_t {
  GC_GENERAL = 0,  // dense complex matrix
  GC_REAL,         // real entries (e.g. Ry: YPow with global shift -1/2)
  GC_DIAG,         // diagonal (ZPow, ZZPow, CZPow, ...)
  GC_X,            // exact Pauli X on one target (X, CNOT: control folded in)
  GC_SKIP          // identity: no work
};

// Instruction stream of a pass.  Gates are grouped into sub-passes: an
// OP_SUB header names 4 tile-local "register" bits and the number of ops that
// follow; every thread loads the 16 amplitudes spanning those bits into
// registers, applies the ops, and stores once.
enum OpType : uint8_t {
  OP_SUB = 0,   // header: gate = #ops, lcmask = r0 | r1<<8 | r2<<16 | r3<<24
  OP_F1,        // 1-qubit gate on register bit t0 (class cls)
  OP_F2,        // 2-qubit gate on register bits t0 (matrix MSB), t1
  OP_B1,        // adjoint step on a 1-qubit gate (psi and lambda)
  OP_B2,        // adjoint step on a 2-qubit gate
  OP_MCH,       // mixed-unitary channel on register bit t0
  OP_CHAN,      // any channel on tile-local bit t0 (outside sub-passes)
};

struct DevOp {
  uint8_t type;
  uint8_t t0, t1;
  uint8_t ngrad;
  uint32_t gate;     // gate (matrix slot) or channel index within the program
  uint32_t lcmask, lcval;  // controls on tile-local bits outside the registers
  uint32_t gcmask, gcval;  // controls on bits outside the tile (global bits)
  int32_t grad_slot;       // first derivative slot (OP_B*)
  uint8_t cls;             // GateClass
  uint8_t kmask, kval;     // controls on register bits
  uint8_t gi;              // first gradient entry of the op in its sub-pass
                           // (sub-pass header: t1 = entries of the sub-pass)
};
static_assert(sizeof(DevOp) == 32, "DevOp layout");

// A pass streams every tile of the state once: the tile holds the 2^T
// amplitudes whose index bits outside `tile_mask` are fixed.  A
// global-channel pass (streamed noisy rows) instead applies its one OP_CHAN,
// whose t0 is a global bit, to the whole state in global memory: its Kraus
// branch probabilities are norms over the whole state, not over a tile.
struct DevPass {
  uint32_t tile_mask;
  uint32_t op_begin, op_end;
  uint32_t global_channel;  // 1 for a global-channel pass
};

// A Pauli term: P|y> = i^ny (-1)^popc(y & zy) |y ^ flip>  (bits).
struct DevTerm {
  uint32_t flip;
  uint32_t zy;
  float coef;          // coefficient_real (util_qsim.h:184-185)
  uint16_t op;         // which pauli_sums column this term belongs to
  uint8_t ny;          // number of Y factors mod 4
  uint8_t identity;    // no Pauli factors: contributes coef directly
};

// A channel: up to 4 Kraus operators on one qubit.  Mixed-unitary channels
// (every K_k proportional to a unitary) select their branch from fixed
// probabilities; the others from |K_k psi|^2.
struct DevChannel {
  uint8_t kind;
  uint8_t nk;
  uint8_t mixed_unitary;
  uint8_t ident_mask;  // bit k set when K_k is proportional to identity
  uint32_t kraus;      // index of the first Kraus matrix (2x2 float2 x4)
  double cum[4];       // cumulative branch probabilities (mixed unitary)
  float scale[4];      // 1/sqrt(p_k) restoring unit norm (mixed unitary)
};

// Per distinct program: where its passes/ops/gates live in the packed arrays.
struct DevProgram {
  int32_t n;            // qubits (0 = empty program)
  int32_t num_gates;    // gate templates (matrix slots)
  int32_t num_grads;    // derivative slots
  uint32_t grad_col_begin;                 // derivative slot -> symbol column
  uint32_t fwd_pass_begin, fwd_pass_end;   // forward passes
  uint32_t bwd_pass_begin, bwd_pass_end;   // adjoint backward passes
  uint32_t gate_begin;                     // first GateTemplate
  uint32_t channel_begin;                  // first DevChannel
  int32_t resident;                        // state kept in shared memory
  int32_t num_channels;
};

// A measurement pass: the terms [begin, end) of the measurement list are
// evaluated on tiles holding the index bits of tile_mask (each term's flip
// bits lie inside the tile).
struct DevMeas {
  uint32_t tile_mask;
  uint32_t begin, end;
  uint32_t pad;
};

// Entry of the measurement list: a term and its flip mask in tile-local bits.
struct DevMeasTerm {
  uint32_t term;
  uint32_t lflip;
};

// Per batch row.
struct DevRow {
  int32_t program;       // index into DevProgram[]
  int32_t n;
  uint32_t term_begin, term_end;   // DevTerm range for this row's pauli_sums
  uint32_t meas_begin, meas_end;   // DevMeas range (measurement passes)
  uint64_t mat_offset;   // first matrix slot (float2[16] each) of this row
  uint64_t dmat_offset;  // first derivative matrix slot of this row
};

// A fused block of the tensor-core forward path: the gates
// members[member_begin, member_end) of one program (template indices, time
// order) act only on the 5 bits tgt[0] < ... < tgt[4]; their product is a
// 32 x 32 complex matrix whose index bit i is tgt[i].  Bits beyond the
// members' own are padding (the product is the identity on them).
constexpr int kTcBits = 5;
struct TcBlock {
  uint32_t member_begin, member_end;
  uint8_t tgt[kTcBits];
  uint8_t used;        // bits that some member touches (<= 5)
  uint8_t pad_[2];
};
static_assert(sizeof(TcBlock) == 16, "TcBlock layout");

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define TFQG_TYPES_HD __host__ __device__ __forceinline__
#else
#define TFQG_TYPES_HD inline
#endif

// Packed op code (one 32-bit word per staged op):
//   bits 0-2 type, 3-5 class, 6-7 j0, 8-9 j1, 10-13 kmask, 14-17 kval,
//   18-19 ngrad, 20 has non-register controls, 21 single register control,
//   22-23 that control's register bit, 24 its value.
TFQG_TYPES_HD uint32_t op_code(const DevOp& op) {
  uint32_t km = op.kmask & 15u, kv = op.kval & 15u;
  uint32_t single = km && !(km & (km - 1u));
  uint32_t jc = 0;
  if (single) { while (!((km >> jc) & 1u)) ++jc; }
  uint32_t cv = single ? ((kv >> jc) & 1u) : 0u;
  return uint32_t(op.type & 7) | uint32_t(op.cls & 7) << 3 | uint32_t(op.t0 & 3) << 6 |
         uint32_t(op.t1 & 3) << 8 | km << 10 | kv << 14 | uint32_t(op.ngrad & 3) << 18 |
         uint32_t((op.lcmask | op.gcmask) != 0) << 20 | single << 21 | jc << 22 | cv << 24;
}

}  // namespace tfqg
