// Host compiler: wire decoding, qubit/symbol resolution, gate templates and
// tile-pass planning.  Follows the reference's parse path:
//   ParseProto ............ tensorflow_quantum/core/ops/parse_context.cc:155-170
//   ResolveQubitIds ....... tensorflow_quantum/core/src/program_resolution.cc:49-186
//   ParseAppendGate ....... tensorflow_quantum/core/src/circuit_parser_qsim.cc:53-596
//   channels .............. circuit_parser_qsim.cc:598-769
#include "host.h"

#include "gate_math.cuh"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <set>
#include <tuple>

namespace tfqg {

// ---------------------------------------------------------------------------
// protobuf wire decoding
// ---------------------------------------------------------------------------
namespace {

struct Reader {
  const uint8_t* p;
  const uint8_t* end;
  bool ok = true;

  bool done() const { return p >= end; }

  uint64_t varint() {
    uint64_t v = 0;
    for (int shift = 0; shift < 64; shift += 7) {
      if (p >= end) { ok = false; return 0; }
      uint8_t c = *p++;
      v |= uint64_t(c & 0x7F) << shift;
      if (!(c & 0x80)) return v;
    }
    ok = false;
    return 0;
  }

  // Reads one field; returns false at end or on malformed input.
  bool field(uint32_t* num, uint32_t* wt, const uint8_t** data, size_t* len,
             uint64_t* ival) {
    if (p >= end) return false;
    uint64_t key = varint();
    if (!ok) return false;
    *num = uint32_t(key >> 3);
    *wt = uint32_t(key & 7);
    if (*num == 0) { ok = false; return false; }
    switch (*wt) {
      case 0:
        *ival = varint();
        return ok;
      case 1:
        if (end - p < 8) { ok = false; return false; }
        *data = p; *len = 8; p += 8;
        return true;
      case 2: {
        uint64_t l = varint();
        if (!ok || uint64_t(end - p) < l) { ok = false; return false; }
        *data = p; *len = size_t(l); p += l;
        return true;
      }
      case 5:
        if (end - p < 4) { ok = false; return false; }
        *data = p; *len = 4; p += 4;
        return true;
      default:
        ok = false;
        return false;
    }
  }
};

// Calls f(field, wire_type, data, len) for each field; false on bad input.
template <class F>
bool for_fields(const uint8_t* b, size_t n, F&& f) {
  Reader rd{b, b + n};
  uint32_t fn, wt;
  const uint8_t* fd = nullptr;
  size_t fl = 0;
  uint64_t iv = 0;
  while (rd.field(&fn, &wt, &fd, &fl, &iv))
    if (!f(fn, wt, fd, fl)) return false;
  return rd.ok;
}

float read_f32(const uint8_t* d) {
  float f;
  memcpy(&f, d, 4);
  return f;
}

bool parse_arg(const uint8_t* b, size_t n, ArgP* a) {
  return for_fields(b, n, [&](uint32_t fn, uint32_t wt, const uint8_t* fd,
                              size_t fl) {
    if (fn == 1 && wt == 2) {
      return for_fields(fd, fl, [&](uint32_t fn2, uint32_t wt2,
                                    const uint8_t* d2, size_t l2) {
        if (fn2 == 1 && wt2 == 5) a->f = read_f32(d2);
        else if (fn2 == 3 && wt2 == 2) a->str.assign((const char*)d2, l2);
        return true;
      });
    }
    if (fn == 2 && wt == 2) a->symbol.assign((const char*)fd, fl);
    return true;
  });
}

bool parse_op(const uint8_t* b, size_t n, OpP* op) {
  return for_fields(b, n, [&](uint32_t fn, uint32_t wt, const uint8_t* fd,
                              size_t fl) {
    if (fn == 1 && wt == 2) {
      return for_fields(fd, fl, [&](uint32_t f2, uint32_t w2,
                                    const uint8_t* d2, size_t l2) {
        if (f2 == 1 && w2 == 2) op->gate.assign((const char*)d2, l2);
        return true;
      });
    }
    if (fn == 2 && wt == 2) {
      std::string key;
      ArgP val;
      bool ok = for_fields(fd, fl, [&](uint32_t f2, uint32_t w2,
                                       const uint8_t* d2, size_t l2) {
        if (f2 == 1 && w2 == 2) {
          key.assign((const char*)d2, l2);
        } else if (f2 == 2 && w2 == 2) {
          val = ArgP();
          return parse_arg(d2, l2, &val);
        }
        return true;
      });
      if (!ok) return false;
      op->args.emplace_back(std::move(key), std::move(val));
      return true;
    }
    if (fn == 3 && wt == 2) {
      std::string id;
      bool ok = for_fields(fd, fl, [&](uint32_t f2, uint32_t w2,
                                       const uint8_t* d2, size_t l2) {
        if (f2 == 2 && w2 == 2) id.assign((const char*)d2, l2);
        return true;
      });
      if (!ok) return false;
      op->qubits.push_back(std::move(id));
    }
    return true;
  });
}

bool parse_program(const uint8_t* b, size_t n, ProgramP* prog) {
  return for_fields(b, n, [&](uint32_t fn, uint32_t wt, const uint8_t* fd,
                              size_t fl) {
    if (!(fn == 2 && wt == 2)) return true;  // circuit (messages merge)
    return for_fields(fd, fl, [&](uint32_t f2, uint32_t w2, const uint8_t* d2,
                                  size_t l2) {
      if (!(f2 == 2 && w2 == 2)) return true;  // moment
      std::vector<OpP> ops;
      bool ok = for_fields(d2, l2, [&](uint32_t f3, uint32_t w3,
                                       const uint8_t* d3, size_t l3) {
        if (f3 == 1 && w3 == 2) {
          OpP op;
          if (!parse_op(d3, l3, &op)) return false;
          ops.push_back(std::move(op));
        }
        return true;
      });
      if (!ok) return false;
      prog->moments.push_back(std::move(ops));
      return true;
    });
  });
}

bool parse_paulisum(const uint8_t* b, size_t n, PauliSumP* ps) {
  return for_fields(b, n, [&](uint32_t fn, uint32_t wt, const uint8_t* fd,
                              size_t fl) {
    if (!(fn == 1 && wt == 2)) return true;
    TermP t;
    bool ok = for_fields(fd, fl, [&](uint32_t f2, uint32_t w2,
                                     const uint8_t* d2, size_t l2) {
      if (f2 == 1 && w2 == 5) {
        t.re = read_f32(d2);
      } else if (f2 == 2 && w2 == 5) {
        t.im = read_f32(d2);
      } else if (f2 == 3 && w2 == 2) {
        std::string q, ty;
        bool ok2 = for_fields(d2, l2, [&](uint32_t f3, uint32_t w3,
                                          const uint8_t* d3, size_t l3) {
          if (f3 == 1 && w3 == 2) q.assign((const char*)d3, l3);
          else if (f3 == 2 && w3 == 2) ty.assign((const char*)d3, l3);
          return true;
        });
        if (!ok2) return false;
        t.paulis.emplace_back(std::move(q), std::move(ty));
      }
      return true;
    });
    if (!ok) return false;
    ps->push_back(std::move(t));
    return true;
  });
}

}  // namespace

const ArgP* OpP::find(const std::string& key) const {
  for (auto it = args.rbegin(); it != args.rend(); ++it)
    if (it->first == key) return &it->second;
  return nullptr;
}

// Binary first, then text format (ParseProto, parse_context.cc:155-170).
void decode_program(const char* data, size_t len, ProgramP* out) {
  *out = ProgramP();
  if (parse_program(reinterpret_cast<const uint8_t*>(data), len, out)) return;
  std::string wire;
  *out = ProgramP();
  if (text_proto_to_wire(data, len, false, &wire) &&
      parse_program(reinterpret_cast<const uint8_t*>(wire.data()), wire.size(), out))
    return;
  throw Error(kInvalidArgument, "Unparseable proto: " + std::string(data, len));
}

void decode_paulisum(const char* data, size_t len, PauliSumP* out) {
  out->clear();
  if (parse_paulisum(reinterpret_cast<const uint8_t*>(data), len, out)) return;
  std::string wire;
  out->clear();
  if (text_proto_to_wire(data, len, true, &wire) &&
      parse_paulisum(reinterpret_cast<const uint8_t*>(wire.data()), wire.size(), out))
    return;
  throw Error(kInvalidArgument, "Unparseable proto: " + std::string(data, len));
}

bool simple_atoi(const std::string& s, int64_t* out) {
  size_t i = 0, j = s.size();
  while (i < j && isspace((unsigned char)s[i])) ++i;
  while (j > i && isspace((unsigned char)s[j - 1])) --j;
  if (i == j) return false;
  bool neg = false;
  if (s[i] == '+' || s[i] == '-') {
    neg = s[i] == '-';
    ++i;
  }
  if (i == j) return false;
  int64_t v = 0;
  for (; i < j; ++i) {
    if (s[i] < '0' || s[i] > '9') return false;
    v = v * 10 + (s[i] - '0');
    if (v > int64_t(2147483648LL)) return false;
  }
  v = neg ? -v : v;
  if (v > 2147483647LL || v < -2147483648LL) return false;
  *out = v;
  return true;
}

// ---------------------------------------------------------------------------
// qubit resolution (program_resolution.cc:49-186)
// ---------------------------------------------------------------------------
namespace {

std::vector<std::string> split(const std::string& s, char sep) {
  std::vector<std::string> out;
  size_t start = 0;
  while (true) {
    size_t k = s.find(sep, start);
    if (k == std::string::npos) {
      out.push_back(s.substr(start));
      return out;
    }
    out.push_back(s.substr(start, k - start));
    start = k + 1;
  }
}

using QubitKey = std::tuple<int64_t, int64_t, std::string>;

void register_qubits(const std::string& qb_string, std::set<QubitKey>* ids) {
  if (qb_string.empty()) return;
  for (const std::string& qb : split(qb_string, ',')) {
    std::vector<std::string> parts = split(qb, '_');
    if (parts.size() == 1) parts.insert(parts.begin(), "2147483647");
    int64_t r, c;
    if (parts.size() != 2 || !simple_atoi(parts[0], &r) ||
        !simple_atoi(parts[1], &c))
      throw Error(kInvalidArgument, "Unable to parse qubit: " + qb);
    ids->insert(QubitKey(r, c, qb));
  }
}

const std::string& control_string(const OpP& op, const char* key) {
  static const std::string empty;
  const ArgP* a = op.find(key);
  return a ? a->str : empty;
}

}  // namespace

int resolve_qubits(const ProgramP& prog,
                   std::unordered_map<std::string, int>* index) {
  index->clear();
  if (prog.moments.empty()) return 0;  // (#679) empty program
  std::set<QubitKey> ids;
  for (const auto& m : prog.moments)
    for (const auto& op : m) {
      for (const auto& q : op.qubits) register_qubits(q, &ids);
      register_qubits(control_string(op, "control_qubits"), &ids);
    }
  int i = 0;
  for (const auto& k : ids) (*index)[std::get<2>(k)] = i++;
  return i;
}

void check_paired_qubits(const ProgramP& other,
                         const std::unordered_map<std::string, int>& index) {
  std::set<std::string> visited;
  for (const auto& m : other.moments)
    for (const auto& op : m) {
      for (const auto& q : op.qubits) {
        if (!index.count(q))
          throw Error(kInvalidArgument,
                      "A paired circuit contains qubits not found in reference circuit.");
        visited.insert(q);
      }
      const std::string& cs = control_string(op, "control_qubits");
      if (cs.empty()) continue;
      for (const std::string& q : split(cs, ',')) {
        if (!index.count(q))
          throw Error(kInvalidArgument,
                      "A paired circuit contains qubits not found in reference circuit.");
        visited.insert(q);
      }
    }
  if (visited.size() != index.size())
    throw Error(kInvalidArgument,
                "A reference circuit contains qubits not found in paired circuit.");
}

// ---------------------------------------------------------------------------
// gate templates (circuit_parser_qsim.cc:53-596)
// ---------------------------------------------------------------------------
namespace {

struct GateInfo {
  GateKind kind;
  int nq;
};

bool lookup_gate(const std::string& id, GateInfo* g) {
  static const std::unordered_map<std::string, GateInfo> table = {
      {"I", {GK_I1, 1}},    {"HP", {GK_HP, 1}},    {"XP", {GK_XP, 1}},
      {"XXP", {GK_XXP, 2}}, {"YP", {GK_YP, 1}},    {"YYP", {GK_YYP, 2}},
      {"ZP", {GK_ZP, 1}},   {"ZZP", {GK_ZZP, 2}},  {"CZP", {GK_CZP, 2}},
      {"I2", {GK_I2, 2}},   {"CNP", {GK_CNP, 2}},  {"SP", {GK_SP, 2}},
      {"ISP", {GK_ISP, 2}}, {"PXP", {GK_PXP, 1}},  {"FSIM", {GK_FSIM, 2}},
      {"PISP", {GK_PISP, 2}}};
  auto it = table.find(id);
  if (it == table.end()) return false;
  *g = it->second;
  return true;
}

bool lookup_channel(const std::string& id, ChannelKind* k) {
  static const std::unordered_map<std::string, ChannelKind> table = {
      {"DP", CK_DP}, {"ADP", CK_ADP}, {"GAD", CK_GAD}, {"AD", CK_AD},
      {"RST", CK_RST}, {"PD", CK_PD}, {"PF", CK_PF}, {"BF", CK_BF}};
  auto it = table.find(id);
  if (it == table.end()) return false;
  *k = it->second;
  return true;
}

// ParseProtoArg: constant value, or the symbol's column.
void parse_arg(const OpP& op, const char* name, const SymbolTable& names,
               float* value, int16_t* src) {
  const ArgP* a = op.find(name);
  if (!a)
    throw Error(kInvalidArgument,
                std::string("Could not find arg: ") + name + " in op.");
  *value = a->f;
  *src = -1;
  if (!a->symbol.empty()) {
    auto it = names.col.find(a->symbol);
    if (it == names.col.end())
      throw Error(kInvalidArgument,
                  "Could not find symbol in parameter map: " + a->symbol);
    *src = int16_t(it->second);
  }
}

int qubit_bit(const OpP& op, int i, int n,
              const std::unordered_map<std::string, int>& index) {
  if (int(op.qubits.size()) <= i)
    throw Error(kInvalidArgument,
                "Operation " + op.gate + " has too few qubits.");
  auto it = index.find(op.qubits[i]);
  if (it == index.end())
    throw Error(kInvalidArgument, "Unable to parse qubit: " + op.qubits[i]);
  return n - it->second - 1;
}

// ParseProtoControls (circuit_parser_qsim.cc:84-129).
void parse_controls(const OpP& op, int n,
                    const std::unordered_map<std::string, int>& index,
                    uint32_t* cmask, uint32_t* cval) {
  *cmask = 0;
  *cval = 0;
  const std::string& cq = control_string(op, "control_qubits");
  const std::string& cv = control_string(op, "control_values");
  if (cq.empty() && cv.empty()) return;
  std::vector<std::string> qt = split(cq, ','), vt = split(cv, ',');
  if (qt.size() != vt.size())
    throw Error(kInvalidArgument,
                "Mistmatched number of control qubits and control values.");
  std::vector<int> bits;
  for (const auto& t : qt) {
    auto it = index.find(t);
    if (it == index.end())
      throw Error(kInvalidArgument, "Unable to parse qubit: " + t);
    bits.push_back(n - it->second - 1);
  }
  for (size_t k = 0; k < vt.size(); ++k) {
    int64_t v;
    if (!simple_atoi(vt[k], &v))
      throw Error(kInvalidArgument, "Unparseable control value: " + vt[k]);
    *cmask |= 1u << bits[k];
    if (v & 1) *cval |= 1u << bits[k];
  }
}

void build_gate(const OpP& op, const GateInfo& info, int n,
                const SymbolTable& names,
                const std::unordered_map<std::string, int>& index,
                GateTemplate* g) {
  memset(g, 0, sizeof(*g));
  g->kind = info.kind;
  g->nq = uint8_t(info.nq);
  for (int i = 0; i < 5; ++i) g->src[i] = -1;
  g->grad_slot = -1;
  g->link = -1;
  g->b0 = uint8_t(qubit_bit(op, 0, n, index));
  if (info.nq == 2) g->b1 = uint8_t(qubit_bit(op, 1, n, index));
  switch (info.kind) {
    case GK_I1: case GK_I2:
      break;
    case GK_PXP:
      // argument order of PhasedXGate (circuit_parser_qsim.cc:393-421)
      parse_arg(op, "exponent", names, &g->a[2], &g->src[2]);
      parse_arg(op, "exponent_scalar", names, &g->a[3], &g->src[3]);
      parse_arg(op, "phase_exponent", names, &g->a[0], &g->src[0]);
      parse_arg(op, "phase_exponent_scalar", names, &g->a[1], &g->src[1]);
      parse_arg(op, "global_shift", names, &g->a[4], &g->src[4]);
      break;
    case GK_FSIM:
      parse_arg(op, "theta", names, &g->a[0], &g->src[0]);
      parse_arg(op, "theta_scalar", names, &g->a[1], &g->src[1]);
      parse_arg(op, "phi", names, &g->a[2], &g->src[2]);
      parse_arg(op, "phi_scalar", names, &g->a[3], &g->src[3]);
      break;
    case GK_PISP:
      parse_arg(op, "exponent", names, &g->a[2], &g->src[2]);
      parse_arg(op, "exponent_scalar", names, &g->a[3], &g->src[3]);
      parse_arg(op, "phase_exponent", names, &g->a[0], &g->src[0]);
      parse_arg(op, "phase_exponent_scalar", names, &g->a[1], &g->src[1]);
      break;
    default:  // eigen gates (SingleEigenGate / TwoEigenGate)
      parse_arg(op, "exponent", names, &g->a[0], &g->src[0]);
      parse_arg(op, "exponent_scalar", names, &g->a[1], &g->src[1]);
      parse_arg(op, "global_shift", names, &g->a[2], &g->src[2]);
      break;
  }
  parse_controls(op, n, index, &g->cmask, &g->cval);
  const uint32_t tmask = (1u << g->b0) | (info.nq == 2 ? (1u << g->b1) : 0u);
  if (info.nq == 2 && g->b0 == g->b1)
    throw Error(kInvalidArgument,
                "Operation " + op.gate + " acts twice on qubit " + op.qubits[0] + ".");
  if (g->cmask & tmask)
    throw Error(kInvalidArgument,
                "A control qubit of operation " + op.gate + " is also a target.");
  // Symbolic parameters get gradients, in the reference's metadata order:
  // phase exponent / theta first, then exponent / phi (adj_util.cc:37-150).
  bool two_param =
      info.kind == GK_PXP || info.kind == GK_FSIM || info.kind == GK_PISP;
  if (g->src[0] >= 0) g->gparam[g->ngrad++] = 0;
  if (two_param && g->src[2] >= 0) g->gparam[g->ngrad++] = 1;
}

float channel_arg(const OpP& op, const char* name) {
  const ArgP* a = op.find(name);
  if (!a)
    throw Error(kInvalidArgument,
                std::string("Could not find arg: ") + name + " in op.");
  if (!a->symbol.empty())
    throw Error(kInvalidArgument,
                "Could not find symbol in parameter map: " + a->symbol);
  return a->f;
}

// Kraus operators of the supported channels: the published definitions of
// cirq.depolarize, asymmetric_depolarize, generalized_amplitude_damp,
// amplitude_damp, reset, phase_damp, phase_flip and bit_flip, which the
// reference builds through qsim (circuit_parser_qsim.cc:598-747).
void build_channel(const OpP& op, ChannelKind kind, ChannelHost* ch) {
  std::vector<std::vector<double>> K;  // each 8 doubles: re,im row-major
  auto mat = [](double a, double b, double c, double d) {
    return std::vector<double>{a, 0, b, 0, c, 0, d, 0};
  };
  auto paulis = [&](double p0, double px, double py, double pz) {
    K.push_back(mat(sqrt(p0), 0, 0, sqrt(p0)));
    K.push_back(mat(0, sqrt(px), sqrt(px), 0));
    K.push_back({0, 0, 0, -sqrt(py), 0, sqrt(py), 0, 0});
    K.push_back(mat(sqrt(pz), 0, 0, -sqrt(pz)));
  };
  bool mixed = false;
  std::vector<double> probs;
  switch (kind) {
    case CK_DP: {
      double p = channel_arg(op, "p");
      paulis(1 - p, p / 3, p / 3, p / 3);
      probs = {1 - p, p / 3, p / 3, p / 3};
      mixed = true;
      break;
    }
    case CK_ADP: {
      double px = channel_arg(op, "p_x"), py = channel_arg(op, "p_y"),
             pz = channel_arg(op, "p_z");
      paulis(1 - px - py - pz, px, py, pz);
      probs = {1 - px - py - pz, px, py, pz};
      mixed = true;
      break;
    }
    case CK_PF: {
      double p = channel_arg(op, "p");
      K.push_back(mat(sqrt(1 - p), 0, 0, sqrt(1 - p)));
      K.push_back(mat(sqrt(p), 0, 0, -sqrt(p)));
      probs = {1 - p, p};
      mixed = true;
      break;
    }
    case CK_BF: {
      double p = channel_arg(op, "p");
      K.push_back(mat(sqrt(1 - p), 0, 0, sqrt(1 - p)));
      K.push_back(mat(0, sqrt(p), sqrt(p), 0));
      probs = {1 - p, p};
      mixed = true;
      break;
    }
    case CK_GAD: {
      double p = channel_arg(op, "p"), g = channel_arg(op, "gamma");
      K.push_back(mat(sqrt(p), 0, 0, sqrt(p) * sqrt(1 - g)));
      K.push_back(mat(0, sqrt(p) * sqrt(g), 0, 0));
      K.push_back(mat(sqrt(1 - p) * sqrt(1 - g), 0, 0, sqrt(1 - p)));
      K.push_back(mat(0, 0, sqrt(1 - p) * sqrt(g), 0));
      break;
    }
    case CK_AD: {
      double g = channel_arg(op, "gamma");
      K.push_back(mat(1, 0, 0, sqrt(1 - g)));
      K.push_back(mat(0, sqrt(g), 0, 0));
      break;
    }
    case CK_RST:
      K.push_back(mat(1, 0, 0, 0));
      K.push_back(mat(0, 1, 0, 0));
      break;
    case CK_PD: {
      double g = channel_arg(op, "gamma");
      K.push_back(mat(1, 0, 0, sqrt(1 - g)));
      K.push_back(mat(0, 0, 0, sqrt(g)));
      break;
    }
  }
  memset(&ch->dev, 0, sizeof(ch->dev));
  ch->dev.kind = kind;
  ch->dev.nk = uint8_t(K.size());
  ch->dev.mixed_unitary = mixed;
  ch->kraus.clear();
  double cum = 0;
  for (size_t k = 0; k < K.size(); ++k) {
    ch->kraus.insert(ch->kraus.end(), K[k].begin(), K[k].end());
    if (mixed) {
      cum += probs[k];
      ch->dev.cum[k] = cum;
      ch->dev.scale[k] = probs[k] > 0 ? float(1.0 / sqrt(probs[k])) : 0.f;
      bool ident = K[k][2] == 0 && K[k][3] == 0 && K[k][4] == 0 &&
                   K[k][5] == 0 && K[k][0] == K[k][6] && K[k][1] == K[k][7];
      if (ident) ch->dev.ident_mask |= uint8_t(1u << k);
    }
  }
}

}  // namespace

void compile_program(const ProgramP& prog, const SymbolTable& names,
                     JobKind kind, CompiledProgram* out,
                     std::unordered_map<std::string, int>* index) {
  *out = CompiledProgram();
  int n = resolve_qubits(prog, index);
  if (n > 30)
    throw Error(kResourceExhausted,
                "Circuit acts on " + std::to_string(n) +
                    " qubits; at most 30 fit this simulator's state layout.");
  out->n = n;
  if (n <= 0) return;
  int grad_slots = 0;
  for (const auto& m : prog.moments) {
    for (const auto& op : m) {
      GateInfo info;
      if (lookup_gate(op.gate, &info)) {
        GateTemplate g;
        build_gate(op, info, n, names, *index, &g);
        g.cls = classify_gate(g);
        if (kind == kJobAdjoint && g.ngrad > 0) {
          g.grad_slot = grad_slots;
          for (int k = 0; k < g.ngrad; ++k)
            out->grad_col.push_back(g.src[2 * g.gparam[k]]);
          grad_slots += g.ngrad;
        }
        out->sequence.push_back(int32_t(out->gates.size()));
        out->gates.push_back(g);
        continue;
      }
      ChannelKind ck;
      if (kind == kJobNoisy && lookup_channel(op.gate, &ck)) {
        ChannelHost ch;
        ch.bit = qubit_bit(op, 0, n, *index);
        build_channel(op, ck, &ch);
        out->sequence.push_back(~int32_t(out->channels.size()));
        out->channels.push_back(std::move(ch));
        continue;
      }
      if (kind == kJobNoisy)
        throw Error(kInvalidArgument, "Could not parse channel id: " + op.gate);
      throw Error(kInvalidArgument,
                  "Could not parse gate id: " + op.gate +
                      ". This is likely because a cirq.Channel was used in an "
                      "op that does not support them.");
    }
  }
}

// ---------------------------------------------------------------------------
// gate structure classes
// ---------------------------------------------------------------------------
namespace {

bool near(double a, double b) { return fabs(a - b) < 1e-9; }

}  // namespace

static uint32_t low_mask_bits(int k) { return k >= 32 ? 0xFFFFFFFFu : ((1u << k) - 1u); }

// Chooses the cheapest exact arithmetic for a gate.  Constant gates are
// classified from their matrix (fp32 parameter products, as the device
// computes them); symbolic gates from their kind.
uint8_t classify_gate(const GateTemplate& g) {
  bool symbolic = false;
  for (int i = 0; i < 5; ++i) symbolic |= g.src[i] >= 0;
  if (!symbolic) {
    float e0, e1, e2;
    effective_params(g, g.a[0], g.a[2], &e0, &e1, &e2);
    Cx<double> m[16];
    int nq = gate_matrix<double>(g.kind, e0, e1, e2, m);
    int D = nq == 1 ? 2 : 4;
    bool diag = true, ident = true, real = true;
    for (int r = 0; r < D; ++r)
      for (int c = 0; c < D; ++c) {
        const Cx<double>& v = m[r * D + c];
        if (r != c && (fabs(v.re) > 1e-9 || fabs(v.im) > 1e-9)) diag = false;
        if (r == c && (!near(v.re, 1.0) || fabs(v.im) > 1e-9)) ident = false;
        if (fabs(v.im) > 1e-9) real = false;
      }
    if (diag && ident) return GC_SKIP;
    if (diag) return GC_DIAG;
    if (nq == 1 && fabs(m[0].re) < 1e-9 && fabs(m[0].im) < 1e-9 &&
        fabs(m[3].re) < 1e-9 && fabs(m[3].im) < 1e-9 && near(m[1].re, 1.0) &&
        near(m[2].re, 1.0) && fabs(m[1].im) < 1e-9 && fabs(m[2].im) < 1e-9)
      return GC_X;
    if (nq == 2 && g.kind == GK_CNP) {
      // exactly CNOT: identity on control 0, X on the target for control 1
      bool cx = near(m[0].re, 1) && near(m[5].re, 1) && near(m[11].re, 1) &&
                near(m[14].re, 1);
      for (int i = 0; i < 16; ++i) {
        if (i == 0 || i == 5 || i == 11 || i == 14) {
          if (fabs(m[i].im) > 1e-9) cx = false;
        } else if (fabs(m[i].re) > 1e-9 || fabs(m[i].im) > 1e-9) {
          cx = false;
        }
      }
      if (cx) return GC_X;
    }
    if (nq == 1 && real) return GC_REAL;
    return GC_GENERAL;
  }
  if (g.kind == GK_ZP || g.kind == GK_ZZP || g.kind == GK_CZP) return GC_DIAG;
  if (g.kind == GK_YP && g.src[2] < 0 && g.a[2] == -0.5f) return GC_REAL;
  return GC_GENERAL;
}

// ---------------------------------------------------------------------------
// pass planning
// ---------------------------------------------------------------------------
namespace {

struct PlanItem {
  int32_t seq;       // gate index, or ~channel
  uint32_t targets;  // target bits
  uint32_t deps;     // targets | controls
};

uint32_t low_mask(int k) { return k >= 32 ? 0xFFFFFFFFu : ((1u << k) - 1u); }

int local_pos(uint32_t tile_mask, int bit) {
  return __builtin_popcount(tile_mask & low_mask(bit));
}

// Targets and controls of a gate as executed (CNOT runs as X on its target
// controlled by its first qubit).
void gate_bits(const GateTemplate& g, uint32_t* targets, uint32_t* cmask,
               uint32_t* cval) {
  *cmask = g.cmask;
  *cval = g.cval;
  if (g.cls == GC_X && g.nq == 2) {
    *targets = 1u << g.b1;
    *cmask |= 1u << g.b0;
    *cval |= 1u << g.b0;
    return;
  }
  *targets = (1u << g.b0) | (g.nq == 2 ? 1u << g.b1 : 0u);
}

// One op on tile-local bits; register fields are filled by the sub-pass
// planner.
DevOp make_op(const CompiledProgram& p, const PlanItem& it, uint32_t tile,
              bool backward, const std::vector<int>& chan_bits) {
  DevOp op;
  memset(&op, 0, sizeof(op));
  op.grad_slot = -1;
  if (it.seq < 0) {
    int c = ~it.seq;
    op.type = p.channels[c].dev.mixed_unitary ? OP_MCH : OP_CHAN;
    op.t0 = uint8_t(local_pos(tile, chan_bits[c]));
    op.gate = uint32_t(c);
    op.cls = GC_GENERAL;
    return op;
  }
  const GateTemplate& g = p.gates[it.seq];
  uint32_t targets, cmask, cval;
  gate_bits(g, &targets, &cmask, &cval);
  op.gate = uint32_t(it.seq);
  op.cls = g.cls;
  bool one = g.nq == 1 || g.cls == GC_X;
  if (g.cls == GC_X && g.nq == 2) {
    op.t0 = uint8_t(local_pos(tile, g.b1));
  } else {
    op.t0 = uint8_t(local_pos(tile, g.b0));
    op.t1 = g.nq == 2 ? uint8_t(local_pos(tile, g.b1)) : 0;
  }
  for (int b = 0; b < 32; ++b) {
    if (!(cmask >> b & 1)) continue;
    uint32_t v = cval >> b & 1;
    if (tile >> b & 1) {
      int lp = local_pos(tile, b);
      op.lcmask |= 1u << lp;
      op.lcval |= v << lp;
    } else {
      op.gcmask |= 1u << b;
      op.gcval |= v << b;
    }
  }
  if (backward) {
    op.type = one ? OP_B1 : OP_B2;
    op.ngrad = g.ngrad;
    op.grad_slot = g.grad_slot;
  } else {
    op.type = one ? OP_F1 : OP_F2;
  }
  return op;
}

uint32_t op_local_targets(const DevOp& op) {
  if (op.type == OP_F2 || op.type == OP_B2) return (1u << op.t0) | (1u << op.t1);
  return 1u << op.t0;
}

// Groups the ops of one pass (tile of T local bits) into sub-passes of
// kRegBits register bits, reordering only ops that commute (disjoint bits).
void plan_subpasses(const std::vector<DevOp>& in, int T, int regbits,
                    std::vector<DevOp>* out) {
  std::vector<DevOp> remaining = in;
  const uint32_t all = low_mask(T);
  while (!remaining.empty()) {
    const DevOp& first = remaining.front();
    if (first.type == OP_CHAN) {  // needs block-wide norms: stands alone
      out->push_back(first);
      remaining.erase(remaining.begin());
      continue;
    }
    uint32_t R = 0, blocked = 0;
    std::vector<DevOp> taken, rest;
    for (const DevOp& op : remaining) {
      uint32_t tg = op_local_targets(op);
      uint32_t deps = tg | op.lcmask;
      bool fits = op.type != OP_CHAN &&
                  __builtin_popcount(R | tg) <= regbits &&
                  taken.size() < size_t(kMaxSubOps) && !(deps & blocked);
      if (fits) {
        R |= tg;
        taken.push_back(op);
      } else {
        rest.push_back(op);
        blocked |= deps;
      }
    }
    // pad the register set, preferring bits above the 5 lane bits so the
    // warp's lanes keep walking consecutive amplitudes
    for (int b = T - 1; b >= kLaneBits && __builtin_popcount(R) < regbits; --b)
      if (!(R >> b & 1)) R |= 1u << b;
    for (int b = 0; b < T && __builtin_popcount(R) < regbits; ++b)
      if (!(R >> b & 1)) R |= 1u << b;
    int rb[kRegBits] = {0, 0, 0, 0}, nr = 0, regidx[32];
    for (int b = 0; b < 32; ++b) regidx[b] = -1;
    for (int b = 0; b < T; ++b)
      if (R >> b & 1) { regidx[b] = nr; rb[nr++] = b; }
    DevOp h;
    memset(&h, 0, sizeof(h));
    h.type = OP_SUB;
    h.t0 = uint8_t(regbits);
    h.gate = uint32_t(taken.size());
    h.lcmask = uint32_t(rb[0]) | uint32_t(rb[1]) << 8 | uint32_t(rb[2]) << 16 |
               uint32_t(rb[3]) << 24;
    h.grad_slot = -1;
    int entries = 0;
    for (const DevOp& op : taken)
      if (op.type == OP_B1 || op.type == OP_B2) entries += op.ngrad;
    h.t1 = uint8_t(entries);  // <= 2 * kMaxSubOps
    out->push_back(h);
    int gi = 0;
    for (DevOp op : taken) {
      op.gi = uint8_t(gi);
      if (op.type == OP_B1 || op.type == OP_B2) gi += op.ngrad;
      uint32_t lm = op.lcmask, lv = op.lcval;
      op.lcmask = 0;
      op.lcval = 0;
      for (int b = 0; b < T; ++b) {
        if (!(lm >> b & 1)) continue;
        uint32_t v = lv >> b & 1;
        if (regidx[b] >= 0) {
          op.kmask |= uint8_t(1u << regidx[b]);
          op.kval |= uint8_t(v << regidx[b]);
        } else {
          op.lcmask |= 1u << b;
          op.lcval |= v << b;
        }
      }
      op.t0 = uint8_t(regidx[op.t0]);
      if (op.type == OP_F2 || op.type == OP_B2) op.t1 = uint8_t(regidx[op.t1]);
      out->push_back(op);
    }
    (void)all;
    remaining.swap(rest);
  }
}

void plan_sequence(const CompiledProgram& p, const std::vector<PlanItem>& items,
                   int tile_bits, bool backward,
                   const std::vector<int>& chan_bits,
                   std::vector<DevPass>* passes, std::vector<DevOp>* ops) {
  const int n = p.n;
  if (n <= tile_bits) {
    // resident: the tile is the state, padded to at least kRegBits bits
    const int T = n < kRegBits ? kRegBits : n;
    const uint32_t all = low_mask(T);
    std::vector<DevOp> flat;
    for (const auto& it : items) flat.push_back(make_op(p, it, all, backward, chan_bits));
    DevPass ps{all, uint32_t(ops->size()), 0, 0};
    plan_subpasses(flat, T, backward ? kRegBitsAdjoint : kRegBits, ops);
    ps.op_end = uint32_t(ops->size());
    passes->push_back(ps);
    return;
  }
  std::vector<PlanItem> remaining = items;
  const uint32_t lanes = low_mask(kLaneBits);
  if (remaining.empty()) {
    // gates that do nothing (identities) still make a non-empty program, as
    // in the reference, whose fused circuit keeps them: one pass, no ops
    passes->push_back(DevPass{low_mask(tile_bits), uint32_t(ops->size()),
                              uint32_t(ops->size()), 0});
    return;
  }
  // a channel whose branch probabilities are state norms (not mixed-unitary)
  // needs the whole state: it gets a global-channel pass of its own, and
  // blocks only its own bit for the passes around it
  auto global_channel = [&](const PlanItem& it) {
    return it.seq < 0 && !p.channels[~it.seq].dev.mixed_unitary;
  };
  while (!remaining.empty()) {
    if (global_channel(remaining.front())) {
      const DevOp op = make_op(p, remaining.front(), low_mask(n), backward, chan_bits);
      passes->push_back(DevPass{0u, uint32_t(ops->size()), uint32_t(ops->size() + 1), 1u});
      ops->push_back(op);
      remaining.erase(remaining.begin());
      continue;
    }
    uint32_t S = lanes, blocked = 0;
    std::vector<PlanItem> taken, rest;
    for (const auto& it : remaining) {
      if (global_channel(it)) {
        rest.push_back(it);
        blocked |= it.deps;
        continue;
      }
      if (it.deps & blocked) {
        rest.push_back(it);
        blocked |= it.deps;
        continue;
      }
      uint32_t U = S | it.targets;
      if (__builtin_popcount(U) <= tile_bits) {
        S = U;
        taken.push_back(it);
      } else {
        rest.push_back(it);
        blocked |= it.deps;
      }
    }
    for (int b = 0; b < n && __builtin_popcount(S) < tile_bits; ++b) S |= 1u << b;
    std::vector<DevOp> flat;
    for (const auto& it : taken) flat.push_back(make_op(p, it, S, backward, chan_bits));
    DevPass ps{S, uint32_t(ops->size()), 0, 0};
    plan_subpasses(flat, tile_bits, backward ? kRegBitsAdjoint : kRegBits, ops);
    ps.op_end = uint32_t(ops->size());
    passes->push_back(ps);
    if (taken.empty()) throw Error(kInternal, "pass planner made no progress");
    remaining.swap(rest);
  }
}

// ---------------------------------------------------------------------------
// gate fusion (forward plans)
// ---------------------------------------------------------------------------
// The analog of qsim's basic fuser, which the reference runs on every
// parsed circuit (circuit_parser_qsim.cc:857, qsim::BasicGateFuser into
// 2-qubit gates; applied by tfq_simulate_expectation_op.cc:164-165): runs of
// uncontrolled 1-qubit
// gates ("chains") are folded into a neighbouring uncontrolled 2-qubit gate
// ("anchor") on their qubit, or merged into one 1-qubit gate.  Unlike qsim,
// a fold is taken only where a cost model over the device's arithmetic per
// amplitude says the fused gate is cheaper: a diagonal CZ stays diagonal
// unless enough dense 1-qubit work is folded into it.

// FP32 operations per amplitude of the device's gate arithmetic, plus one
// for the op itself.
int fuse_cost(int nq, uint8_t cls) {
  switch (cls) {
    case GC_SKIP: return 0;
    case GC_X: return 1;
    case GC_DIAG: return 5;
    case GC_REAL: return nq == 1 ? 5 : 17;
    default: return nq == 1 ? 9 : 17;
  }
}

// Structure class of a product of gates of the given classes.
uint8_t fold_class(uint8_t acc, uint8_t cls, int nq) {
  if (cls == GC_SKIP) return acc;
  if (acc == GC_SKIP) return (nq == 2 && cls == GC_X) ? uint8_t(GC_GENERAL) : cls;
  if (acc == GC_DIAG && cls == GC_DIAG) return GC_DIAG;
  if (nq == 1 && (acc == GC_REAL || acc == GC_X) && (cls == GC_REAL || cls == GC_X))
    return GC_REAL;
  return GC_GENERAL;
}

struct FuseChain {
  int bit = 0;
  std::vector<int> pos;  // sequence positions of the chain's gates
  int owner = -1;        // anchor that absorbs it, -1 none
  uint8_t cls = GC_SKIP;
  int separate = 0;      // cost of its gates run one by one
};

struct FuseAnchor {
  int pos = 0;
  int chain[4] = {-1, -1, -1, -1};  // before on b0, b1; after on b0, b1
  uint8_t cls = GC_GENERAL;
};

constexpr int kMaxChainGates = 15;  // 4 chains + anchor <= kMaxFuseMembers

// Chain cost where it is not folded into an anchor: merged when that is not
// more expensive than its gates one by one.
int chain_cost(const FuseChain& c) {
  if (c.pos.size() < 2) return c.separate;
  return std::min(c.separate, fuse_cost(1, c.cls));
}

// Rewrites p->sequence into `out`, appending GK_FUSED templates to p->gates.
void fuse_forward(CompiledProgram* p, std::vector<int32_t>* out) {
  const std::vector<int32_t>& seq = p->sequence;
  std::vector<FuseChain> chains;
  std::vector<FuseAnchor> anchors;
  int cur[32], last[32];
  for (int q = 0; q < 32; ++q) cur[q] = last[q] = -1;
  auto barrier = [&](uint32_t bits) {
    for (int q = 0; q < 32; ++q)
      if (bits >> q & 1) cur[q] = last[q] = -1;
  };
  for (size_t i = 0; i < seq.size(); ++i) {
    const int32_t s = seq[i];
    if (s < 0) {
      barrier(1u << p->channels[~s].bit);
      continue;
    }
    const GateTemplate& g = p->gates[s];
    if (g.cls == GC_SKIP) continue;  // identities commute with everything
    if (g.cmask != 0 || g.nq > 2) {
      barrier(g.cmask | 1u << g.b0 | (g.nq == 2 ? 1u << g.b1 : 0u));
      continue;
    }
    if (g.nq == 1) {
      const int q = g.b0;
      if (cur[q] >= 0 && int(chains[cur[q]].pos.size()) >= kMaxChainGates)
        cur[q] = last[q] = -1;  // full: the next chain starts unattached
      if (cur[q] < 0) {
        cur[q] = int(chains.size());
        chains.emplace_back();
        chains.back().bit = q;
        if (last[q] >= 0) {
          FuseAnchor& a = anchors[last[q]];
          a.chain[q == p->gates[seq[a.pos]].b0 ? 2 : 3] = cur[q];
        }
      }
      FuseChain& c = chains[cur[q]];
      c.pos.push_back(int(i));
      c.cls = fold_class(c.cls, g.cls, 1);
      c.separate += fuse_cost(1, g.cls);
      continue;
    }
    FuseAnchor a;
    a.pos = int(i);
    a.cls = g.cls;
    const int bits[2] = {g.b0, g.b1};
    for (int j = 0; j < 2; ++j) {
      const int q = bits[j];
      a.chain[j] = cur[q];
      cur[q] = -1;
      last[q] = int(anchors.size());
    }
    anchors.push_back(a);
  }

  // dense anchors take every chain beside them for free
  for (FuseAnchor& a : anchors) {
    if (a.cls != GC_GENERAL) continue;
    for (int c : a.chain)
      if (c >= 0 && chains[c].owner < 0) chains[c].owner = int(&a - anchors.data());
  }
  // other anchors: diagonal chains into a diagonal anchor keep it diagonal;
  // the rest are taken together when the dense product is cheaper
  for (FuseAnchor& a : anchors) {
    if (a.cls == GC_GENERAL) continue;
    const int id = int(&a - anchors.data());
    uint8_t cls = a.cls;
    if (cls == GC_DIAG)
      for (int c : a.chain)
        if (c >= 0 && chains[c].owner < 0 && chains[c].cls == GC_DIAG)
          chains[c].owner = id;
    int separate = fuse_cost(2, cls);
    std::vector<int> rest;
    for (int c : a.chain)
      if (c >= 0 && chains[c].owner < 0) {
        rest.push_back(c);
        separate += chain_cost(chains[c]);
      }
    if (!rest.empty() && fuse_cost(2, GC_GENERAL) <= separate)
      for (int c : rest) chains[c].owner = id;
  }

  // emit
  std::vector<int32_t> at(seq.begin(), seq.end());  // per position, or drop
  const int32_t kDrop = INT32_MIN;
  auto new_fused = [&](int nq, int b0, int b1, uint8_t cls) {
    GateTemplate f;
    memset(&f, 0, sizeof(f));
    f.kind = GK_FUSED;
    f.nq = uint8_t(nq);
    f.b0 = uint8_t(b0);
    f.b1 = uint8_t(b1);
    for (int i = 0; i < 5; ++i) f.src[i] = -1;
    f.grad_slot = -1;
    f.link = -1;
    f.cls = cls;
    p->gates.push_back(f);
    return int32_t(p->gates.size() - 1);
  };
  for (size_t ai = 0; ai < anchors.size(); ++ai) {
    const FuseAnchor& a = anchors[ai];
    std::vector<int> members;  // sequence positions, time order
    uint8_t cls = GC_SKIP;
    const GateTemplate anchor = p->gates[seq[a.pos]];
    for (int j = 0; j < 4; ++j) {
      if (j == 2) {
        members.push_back(a.pos);
        cls = fold_class(cls, anchor.cls, 2);
      }
      const int c = a.chain[j];
      if (c < 0 || chains[c].owner != int(ai)) continue;
      for (int ps : chains[c].pos) members.push_back(ps);
      cls = fold_class(cls, chains[c].cls, 2);
    }
    if (members.size() < 2) continue;
    const int32_t f = new_fused(2, anchor.b0, anchor.b1, cls);
    int32_t prev = -1;
    for (int ps : members) {
      const int32_t gi = seq[ps];
      GateTemplate& m = p->gates[gi];
      m.fpos = ps == a.pos ? uint8_t(FP_SAME)
                           : (m.b0 == anchor.b0 ? uint8_t(FP_HIGH) : uint8_t(FP_LOW));
      m.link = -1;
      if (prev < 0) p->gates[f].link = gi; else p->gates[prev].link = gi;
      prev = gi;
      at[ps] = kDrop;
    }
    at[a.pos] = f;
  }
  for (const FuseChain& c : chains) {
    if (c.owner >= 0 || c.pos.size() < 2 || fuse_cost(1, c.cls) > c.separate)
      continue;
    const int32_t f = new_fused(1, c.bit, 0, c.cls);
    int32_t prev = -1;
    for (int ps : c.pos) {
      const int32_t gi = seq[ps];
      p->gates[gi].fpos = FP_HIGH;
      p->gates[gi].link = -1;
      if (prev < 0) p->gates[f].link = gi; else p->gates[prev].link = gi;
      prev = gi;
      at[ps] = kDrop;
    }
    at[c.pos.back()] = f;
  }
  out->clear();
  for (int32_t s : at)
    if (s != kDrop) out->push_back(s);
}

}  // namespace

void plan_program(CompiledProgram* p, JobKind kind, bool fuse) {
  p->fwd_passes.clear();
  p->bwd_passes.clear();
  p->fwd_ops.clear();
  p->bwd_ops.clear();
  if (p->empty()) return;
  const int res_max = kind == kJobAdjoint ? kResidentMaxAdjoint : kResidentMaxSingle;
  p->resident = p->n <= res_max;
  const int tile_bits = p->resident ? p->n : kStreamTileBits;
  std::vector<int> chan_bits(p->channels.size(), 0);
  // a re-plan starts again from the program's own gates
  while (!p->gates.empty() && p->gates.back().kind == GK_FUSED) p->gates.pop_back();
  // the forward passes run the fused gates (also the adjoint's forward
  // recompute of psi, as the reference's full_fuse does); the adjoint's
  // backward passes keep one step per gate, since every symbolic gate needs
  // its own lambda step
  std::vector<int32_t> fused;
  const bool fusing = fuse && (kind == kJobForward || kind == kJobAdjoint);
  if (fusing) fuse_forward(p, &fused);
  auto make_items = [&](const std::vector<int32_t>& sequence) {
    std::vector<PlanItem> items;
    items.reserve(sequence.size());
    for (int32_t s : sequence) {
      PlanItem it;
      it.seq = s;
      if (s >= 0) {
        const GateTemplate& g = p->gates[s];
        // identity gates do nothing, also in the adjoint (no parameters)
        if (g.cls == GC_SKIP) continue;
        uint32_t targets, cmask, cval;
        gate_bits(g, &targets, &cmask, &cval);
        it.targets = targets;
        it.deps = targets | cmask;
      } else {
        int bit = p->channels[~s].bit;
        chan_bits[~s] = bit;
        it.targets = 1u << bit;
        it.deps = it.targets;
      }
      items.push_back(it);
    }
    return items;
  };
  const std::vector<PlanItem> items = make_items(fusing ? fused : p->sequence);
  plan_sequence(*p, items, tile_bits, false, chan_bits, &p->fwd_passes, &p->fwd_ops);
  if (kind == kJobAdjoint) {
    const std::vector<PlanItem> per_gate = fusing ? make_items(p->sequence) : items;
    std::vector<PlanItem> rev(per_gate.rbegin(), per_gate.rend());
    plan_sequence(*p, rev, tile_bits, true, chan_bits, &p->bwd_passes, &p->bwd_ops);
  }
}

// ---------------------------------------------------------------------------
// measurement passes
// ---------------------------------------------------------------------------
bool plan_tc_blocks(const GateTemplate* gates, int num_gates, int n,
                    std::vector<TcBlock>* blocks, std::vector<int32_t>* members) {
  if (n < kTcBits + 7 || n > 31) return false;
  // the gates and their bit masks; dependencies: the previous gate on each bit
  std::vector<int32_t> gi;
  std::vector<uint32_t> mask;
  for (int k = 0; k < num_gates; ++k) {
    const GateTemplate& g = gates[k];
    if (g.kind == GK_FUSED || g.cls == GC_SKIP) continue;
    uint32_t q = g.cmask | (1u << g.b0);
    if (g.nq == 2) q |= 1u << g.b1;
    if (__builtin_popcount(q) > kTcBits) return false;
    gi.push_back(k);
    mask.push_back(q);
  }
  const int G = int(gi.size());
  std::vector<std::vector<int32_t>> users(static_cast<size_t>(G));
  std::vector<int32_t> indeg(size_t(G), 0);
  {
    int lastg[32];
    for (int b = 0; b < 32; ++b) lastg[b] = -1;
    for (int i = 0; i < G; ++i) {
      int prev[kTcBits], np = 0;
      for (int b = 0; b < n; ++b) {
        if (!((mask[size_t(i)] >> b) & 1u)) continue;
        const int d = lastg[b];
        bool seen = d < 0;
        for (int t = 0; t < np && !seen; ++t) seen = prev[t] == d;
        if (!seen) {
          prev[np++] = d;
          users[size_t(d)].push_back(i);
          ++indeg[size_t(i)];
        }
        lastg[b] = i;
      }
    }
  }
  std::vector<int32_t> front;
  for (int i = 0; i < G; ++i)
    if (indeg[size_t(i)] == 0) front.push_back(i);
  // Grows a block from `seed`: repeatedly takes the front gate that adds the
  // fewest new bits (the earliest on ties) while the block stays within 5 bits.
  auto grow = [&](int seed, std::vector<int32_t>* fr, std::vector<int32_t>* deg,
                  std::vector<int32_t>* taken, uint32_t* bits) {
    uint32_t S = 0;
    int pick = seed;
    while (pick >= 0) {
      S |= mask[size_t(pick)];
      taken->push_back(pick);
      fr->erase(std::find(fr->begin(), fr->end(), pick));
      for (const int32_t u : users[size_t(pick)])
        if (--(*deg)[size_t(u)] == 0) fr->insert(std::upper_bound(fr->begin(), fr->end(), u), u);
      pick = -1;
      int best_add = kTcBits + 1;
      for (const int32_t f : *fr) {
        const int tot = __builtin_popcount(S | mask[size_t(f)]);
        const int add = tot - __builtin_popcount(S);
        if (tot <= kTcBits && add < best_add) {
          best_add = add;
          pick = f;
        }
      }
    }
    *bits = S;
  };
  // Each block takes the seed (a front gate) whose block absorbs the most gates.
  int done = 0;
  std::vector<int32_t> fr, deg, taken, best_fr, best_deg, best_taken;
  while (done < G) {
    uint32_t best_bits = 0;
    best_taken.clear();
    for (const int32_t seed : front) {
      fr = front;
      deg = indeg;
      taken.clear();
      uint32_t bits = 0;
      grow(seed, &fr, &deg, &taken, &bits);
      if (taken.size() > best_taken.size()) {
        best_taken.swap(taken);
        best_fr.swap(fr);
        best_deg.swap(deg);
        best_bits = bits;
      }
    }
    if (best_taken.empty()) return false;  // unreachable: any seed takes itself
    front.swap(best_fr);
    indeg.swap(best_deg);
    done += int(best_taken.size());
    TcBlock t{};
    t.used = uint8_t(__builtin_popcount(best_bits));
    uint32_t m = best_bits;
    for (int b = n - 1; b >= 0 && __builtin_popcount(m) < kTcBits; --b) m |= 1u << b;
    int k = 0;
    for (int b = 0; b < n; ++b)
      if ((m >> b) & 1u) t.tgt[k++] = uint8_t(b);
    t.member_begin = uint32_t(members->size());
    for (const int32_t x : best_taken) members->push_back(gi[size_t(x)]);
    t.member_end = uint32_t(members->size());
    blocks->push_back(t);
  }
  return true;
}

void plan_measurement(const std::vector<DevTerm>& terms, uint32_t tb,
                      uint32_t te, int n, bool resident,
                      std::vector<DevMeas>* passes,
                      std::vector<DevMeasTerm>* list) {
  if (tb == te) return;
  if (resident) {
    // the tile is the whole state: local bits are global bits
    for (uint32_t base = tb; base < te; base += kMaxMeasTerms) {
      DevMeas m{low_mask_bits(n), uint32_t(list->size()), 0, 0};
      for (uint32_t t = base; t < te && t < base + kMaxMeasTerms; ++t)
        list->push_back(DevMeasTerm{t, terms[t].flip});
      m.end = uint32_t(list->size());
      passes->push_back(m);
    }
    return;
  }
  const uint32_t lanes = low_mask_bits(kLaneBits);
  std::vector<uint32_t> remaining;
  for (uint32_t t = tb; t < te; ++t) remaining.push_back(t);
  while (!remaining.empty()) {
    uint32_t S = lanes;
    std::vector<uint32_t> taken, rest;
    for (uint32_t t : remaining) {
      uint32_t U = S | terms[t].flip;
      if (__builtin_popcount(U) <= kStreamTileBits &&
          taken.size() < size_t(kMaxMeasTerms)) {
        S = U;
        taken.push_back(t);
      } else {
        rest.push_back(t);
      }
    }
    for (int b = 0; b < n && __builtin_popcount(S) < kStreamTileBits; ++b)
      S |= 1u << b;
    DevMeas m{S, uint32_t(list->size()), 0, 0};
    for (uint32_t t : taken) {
      // flip mask in tile-local bit positions
      uint32_t lf = 0;
      int j = 0;
      for (int b = 0; b < 32; ++b)
        if (S >> b & 1) {
          if (terms[t].flip >> b & 1) lf |= 1u << j;
          ++j;
        }
      list->push_back(DevMeasTerm{t, lf});
    }
    m.end = uint32_t(list->size());
    passes->push_back(m);
    if (taken.empty()) throw Error(kInternal, "measurement planner made no progress");
    remaining.swap(rest);
  }
}

// ---------------------------------------------------------------------------
// Pauli sums -> device terms (util_qsim.h:142-188)
// ---------------------------------------------------------------------------
void lower_paulisum(const PauliSumP& ps,
                    const std::unordered_map<std::string, int>& index, int n,
                    int op, std::vector<DevTerm>* out) {
  for (const TermP& t : ps) {
    DevTerm d;
    memset(&d, 0, sizeof(d));
    d.coef = t.re;
    d.op = uint16_t(op);
    if (t.paulis.empty()) {
      d.identity = 1;
      out->push_back(d);
      continue;
    }
    for (const auto& pq : t.paulis) {
      auto it = index.find(pq.first);
      if (it == index.end())
        throw Error(kInvalidArgument,
                    "Found a Pauli sum operating on qubits not found in "
                    "circuit.");
      int bit = n - it->second - 1;
      uint32_t m = 1u << bit;
      // Products on one qubit are applied in order, as the reference applies
      // one gate per factor (circuit_parser_qsim.cc:863-895).
      const std::string& ty = pq.second;
      if (ty == "X") {
        d.flip ^= m;
      } else if (ty == "Z") {
        // Z after the preceding factors: sign from the current bit value
        d.zy ^= m;
      } else if (ty == "Y") {
        d.flip ^= m;
        d.zy ^= m;
        d.ny = uint8_t((d.ny + 1) & 3);
      } else {
        throw Error(kInvalidArgument,
                    "Could not parse gate id: " + ty +
                        "P. This is likely because a cirq.Channel was used in "
                        "an op that does not support them.");
      }
    }
    out->push_back(d);
  }
}

}  // namespace tfqg
