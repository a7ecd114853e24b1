// Protobuf text format for tfq.proto.Program and tfq.proto.PauliSum.
//
// The reference parses each program and pauli sum as binary first and falls
// back to text format when that fails (ParseProto, parse_context.cc:155-170;
// the reference's own benchmark feeds text protos).  This file reads the text
// form and re-encodes it in the binary wire format, so the binary decoder
// (host.cc) and all of its validation apply unchanged.  It covers the syntax
// of the text format (comments, quoted strings with escapes and adjacent
// concatenation, numbers with exponents / f suffixes / inf / nan, enum and
// bool identifiers, `{}` and `<>` message bodies, `[...]` lists, optional
// `:` before a message and `,` / `;` separators) over the fields of
// program.proto and pauli_sum.proto.  An unknown field name fails the parse,
// as it does for TextFormat.
#include <ctype.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "host.h"

namespace tfqg {
namespace {

enum FieldType { kMsg, kString, kFloat, kDouble, kInt64, kBool, kEnum };

struct FieldDef {
  const char* name;
  int number;
  FieldType type;
  int sub;  // message index (kMsg) or enum index (kEnum)
};

// Messages of program.proto and pauli_sum.proto (field numbers and types as
// declared there).
enum MsgId {
  mProgram, mCircuit, mMoment, mSchedule, mScheduledOp, mLanguage, mOperation,
  mGate, mQubit, mArgsEntry, mArg, mArgValue, mRepeatedBool, mArgFunction,
  mPauliSum, mPauliTerm, mPauliPair, kNumMsgs
};

const FieldDef kProgram[] = {{"language", 1, kMsg, mLanguage},
                             {"circuit", 2, kMsg, mCircuit},
                             {"schedule", 3, kMsg, mSchedule}};
const FieldDef kCircuit[] = {{"scheduling_strategy", 1, kEnum, 0},
                             {"moments", 2, kMsg, mMoment}};
const FieldDef kMoment[] = {{"operations", 1, kMsg, mOperation}};
const FieldDef kSchedule[] = {{"scheduled_operations", 3, kMsg, mScheduledOp}};
const FieldDef kScheduledOp[] = {{"operation", 1, kMsg, mOperation},
                                 {"start_time_picos", 2, kInt64, 0}};
const FieldDef kLanguage[] = {{"gate_set", 1, kString, 0},
                              {"arg_function_language", 2, kString, 0}};
const FieldDef kOperation[] = {{"gate", 1, kMsg, mGate},
                               {"args", 2, kMsg, mArgsEntry},
                               {"qubits", 3, kMsg, mQubit}};
const FieldDef kGate[] = {{"id", 1, kString, 0}};
const FieldDef kQubit[] = {{"id", 2, kString, 0}};
const FieldDef kArgsEntry[] = {{"key", 1, kString, 0}, {"value", 2, kMsg, mArg}};
const FieldDef kArg[] = {{"arg_value", 1, kMsg, mArgValue},
                         {"symbol", 2, kString, 0},
                         {"func", 3, kMsg, mArgFunction}};
const FieldDef kArgValue[] = {{"float_value", 1, kFloat, 0},
                              {"bool_values", 2, kMsg, mRepeatedBool},
                              {"string_value", 3, kString, 0},
                              {"double_value", 4, kDouble, 0}};
const FieldDef kRepeatedBool[] = {{"values", 1, kBool, 0}};
const FieldDef kArgFunction[] = {{"type", 1, kString, 0}, {"args", 2, kMsg, mArg}};
const FieldDef kPauliSum[] = {{"terms", 1, kMsg, mPauliTerm}};
const FieldDef kPauliTerm[] = {{"coefficient_real", 1, kFloat, 0},
                               {"coefficient_imag", 2, kFloat, 0},
                               {"paulis", 3, kMsg, mPauliPair}};
const FieldDef kPauliPair[] = {{"qubit_id", 1, kString, 0},
                               {"pauli_type", 2, kString, 0}};

struct MsgDef {
  const FieldDef* fields;
  int n;
};
#define TFQG_MSG(a) {a, int(sizeof(a) / sizeof(a[0]))}
const MsgDef kMsgs[kNumMsgs] = {
    TFQG_MSG(kProgram), TFQG_MSG(kCircuit), TFQG_MSG(kMoment),
    TFQG_MSG(kSchedule), TFQG_MSG(kScheduledOp), TFQG_MSG(kLanguage),
    TFQG_MSG(kOperation), TFQG_MSG(kGate), TFQG_MSG(kQubit),
    TFQG_MSG(kArgsEntry), TFQG_MSG(kArg), TFQG_MSG(kArgValue),
    TFQG_MSG(kRepeatedBool), TFQG_MSG(kArgFunction), TFQG_MSG(kPauliSum),
    TFQG_MSG(kPauliTerm), TFQG_MSG(kPauliPair)};
#undef TFQG_MSG

// Circuit.SchedulingStrategy
struct EnumValue {
  const char* name;
  int value;
};
const EnumValue kStrategy[] = {{"SCHEDULING_STRATEGY_UNSPECIFIED", 0},
                               {"MOMENT_BY_MOMENT", 1}};

// ---- tokens ----------------------------------------------------------------
struct Tok {
  enum Kind { kEnd, kIdent, kNumber, kString, kSymbol, kBad } kind = kEnd;
  std::string s;  // identifier / number text / unescaped string / symbol
};

struct Lexer {
  const char* p;
  const char* e;

  void skip() {
    for (;;) {
      while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r' ||
                       *p == '\f' || *p == '\v'))
        ++p;
      if (p < e && *p == '#') {
        while (p < e && *p != '\n') ++p;
        continue;
      }
      return;
    }
  }

  static bool ident_start(char c) {
    return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || c == '_';
  }
  static bool ident_char(char c) { return ident_start(c) || (c >= '0' && c <= '9'); }

  bool string_body(char q, std::string* out) {
    ++p;  // opening quote
    while (p < e && *p != q) {
      char c = *p++;
      if (c == '\n') return false;
      if (c != '\\') {
        out->push_back(c);
        continue;
      }
      if (p >= e) return false;
      char x = *p++;
      switch (x) {
        case 'n': out->push_back('\n'); break;
        case 't': out->push_back('\t'); break;
        case 'r': out->push_back('\r'); break;
        case 'a': out->push_back('\a'); break;
        case 'b': out->push_back('\b'); break;
        case 'f': out->push_back('\f'); break;
        case 'v': out->push_back('\v'); break;
        case '?': out->push_back('?'); break;
        case '\\': case '\'': case '"': out->push_back(x); break;
        case 'x': case 'X': {
          int v = 0, k = 0;
          while (k < 2 && p < e && isxdigit(static_cast<unsigned char>(*p))) {
            const char h = *p++;
            v = v * 16 + (h <= '9' ? h - '0' : (h | 32) - 'a' + 10);
            ++k;
          }
          if (!k) return false;
          out->push_back(char(v));
          break;
        }
        default:
          if (x >= '0' && x <= '7') {
            int v = x - '0', k = 1;
            while (k < 3 && p < e && *p >= '0' && *p <= '7') v = v * 8 + (*p++ - '0'), ++k;
            out->push_back(char(v));
          } else {
            return false;
          }
      }
    }
    if (p >= e) return false;
    ++p;  // closing quote
    return true;
  }

  Tok next() {
    skip();
    Tok t;
    if (p >= e) return t;
    const char c = *p;
    if (c == '"' || c == '\'') {
      t.kind = Tok::kString;
      // adjacent string literals concatenate
      while (p < e && (*p == '"' || *p == '\'')) {
        if (!string_body(*p, &t.s)) {
          t.kind = Tok::kBad;
          return t;
        }
        skip();
      }
      return t;
    }
    if (ident_start(c)) {
      t.kind = Tok::kIdent;
      while (p < e && ident_char(*p)) t.s.push_back(*p++);
      return t;
    }
    if ((c >= '0' && c <= '9') || c == '.' || c == '-' || c == '+') {
      t.kind = Tok::kNumber;
      if (c == '-' || c == '+') {
        t.s.push_back(*p++);
        skip();
        if (p < e && ident_start(*p)) {  // -inf, -nan
          while (p < e && ident_char(*p)) t.s.push_back(*p++);
          return t;
        }
      }
      while (p < e && (ident_char(*p) || *p == '.' ||
                       ((*p == '-' || *p == '+') && (t.s.back() == 'e' || t.s.back() == 'E'))))
        t.s.push_back(*p++);
      return t;
    }
    if (strchr("{}<>:,;[]", c)) {
      t.kind = Tok::kSymbol;
      t.s.assign(1, c);
      ++p;
      return t;
    }
    t.kind = Tok::kBad;
    return t;
  }

  Tok peek() {
    const char* save = p;
    Tok t = next();
    p = save;
    return t;
  }
};

// ---- wire encoding ---------------------------------------------------------
void put_varint(std::string* w, uint64_t v) {
  while (v >= 0x80) {
    w->push_back(char(uint8_t(v) | 0x80));
    v >>= 7;
  }
  w->push_back(char(v));
}
void put_tag(std::string* w, int number, int wire) {
  put_varint(w, (uint64_t(number) << 3) | uint64_t(wire));
}

bool parse_double(const std::string& s0, double* out) {
  std::string s = s0;
  bool neg = false;
  if (!s.empty() && (s[0] == '-' || s[0] == '+')) {
    neg = s[0] == '-';
    s.erase(0, 1);
  }
  std::string low;
  for (char c : s) low.push_back(char(c | 32));
  if (low == "inf" || low == "infinity") {
    *out = neg ? -INFINITY : INFINITY;
    return true;
  }
  if (low == "nan") {
    *out = NAN;
    return true;
  }
  if (!s.empty() && (s.back() == 'f' || s.back() == 'F') &&
      !(s.size() > 1 && (s[0] == '0') && (s[1] == 'x' || s[1] == 'X')))
    s.pop_back();
  if (s.empty()) return false;
  char* end = nullptr;
  const double v = strtod(s.c_str(), &end);
  if (!end || *end != '\0') return false;
  *out = neg ? -v : v;
  return true;
}

bool parse_int(const std::string& s, int64_t* out) {
  if (s.empty()) return false;
  char* end = nullptr;
  const long long v = strtoll(s.c_str(), &end, 0);
  if (!end || *end != '\0') return false;
  *out = v;
  return true;
}

bool encode_scalar(const FieldDef& f, const Tok& t, std::string* w) {
  switch (f.type) {
    case kString:
      if (t.kind != Tok::kString) return false;
      put_tag(w, f.number, 2);
      put_varint(w, t.s.size());
      w->append(t.s);
      return true;
    case kFloat:
    case kDouble: {
      double v;
      if (!((t.kind == Tok::kNumber || t.kind == Tok::kIdent) && parse_double(t.s, &v)))
        return false;
      if (f.type == kFloat) {
        const float fv = float(v);
        put_tag(w, f.number, 5);
        w->append(reinterpret_cast<const char*>(&fv), 4);
      } else {
        put_tag(w, f.number, 1);
        w->append(reinterpret_cast<const char*>(&v), 8);
      }
      return true;
    }
    case kInt64: {
      int64_t v;
      if (t.kind != Tok::kNumber || !parse_int(t.s, &v)) return false;
      put_tag(w, f.number, 0);
      put_varint(w, uint64_t(v));
      return true;
    }
    case kBool: {
      int v = -1;
      if (t.s == "true" || t.s == "True" || t.s == "t" || t.s == "1") v = 1;
      if (t.s == "false" || t.s == "False" || t.s == "f" || t.s == "0") v = 0;
      if (v < 0) return false;
      put_tag(w, f.number, 0);
      put_varint(w, uint64_t(v));
      return true;
    }
    case kEnum: {
      int64_t v = -1;
      if (t.kind == Tok::kIdent) {
        for (const EnumValue& ev : kStrategy)
          if (t.s == ev.name) v = ev.value;
        if (v < 0) return false;
      } else if (t.kind != Tok::kNumber || !parse_int(t.s, &v)) {
        return false;
      }
      put_tag(w, f.number, 0);
      put_varint(w, uint64_t(v));
      return true;
    }
    default:
      return false;
  }
}

bool parse_message(Lexer* lx, int msg, const char* close, std::string* w, int depth);

bool parse_sub(Lexer* lx, const FieldDef& f, std::string* w, int depth) {
  Tok open = lx->next();
  if (open.kind != Tok::kSymbol || (open.s != "{" && open.s != "<")) return false;
  std::string body;
  if (!parse_message(lx, f.sub, open.s == "{" ? "}" : ">", &body, depth + 1)) return false;
  put_tag(w, f.number, 2);
  put_varint(w, body.size());
  w->append(body);
  return true;
}

bool parse_message(Lexer* lx, int msg, const char* close, std::string* w, int depth) {
  if (depth > 64) return false;
  const MsgDef& md = kMsgs[msg];
  for (;;) {
    Tok t = lx->next();
    if (t.kind == Tok::kEnd) return close == nullptr;
    if (t.kind == Tok::kSymbol && close && t.s == close) return true;
    if (t.kind != Tok::kIdent) return false;
    const FieldDef* f = nullptr;
    for (int i = 0; i < md.n; ++i)
      if (t.s == md.fields[i].name) f = &md.fields[i];
    if (!f) return false;  // unknown field
    Tok sep = lx->peek();
    const bool colon = sep.kind == Tok::kSymbol && sep.s == ":";
    if (colon) lx->next();
    Tok v = lx->peek();
    const bool list = v.kind == Tok::kSymbol && v.s == "[";
    if (f->type == kMsg) {
      if (list) {
        lx->next();
        if (lx->peek().s == "]" && lx->peek().kind == Tok::kSymbol) {
          lx->next();
        } else {
          for (;;) {
            if (!parse_sub(lx, *f, w, depth)) return false;
            Tok d = lx->next();
            if (d.kind == Tok::kSymbol && d.s == "]") break;
            if (!(d.kind == Tok::kSymbol && d.s == ",")) return false;
          }
        }
      } else if (!parse_sub(lx, *f, w, depth)) {
        return false;
      }
    } else {
      if (!colon) return false;
      if (list) {
        lx->next();
        if (lx->peek().kind == Tok::kSymbol && lx->peek().s == "]") {
          lx->next();
        } else {
          for (;;) {
            if (!encode_scalar(*f, lx->next(), w)) return false;
            Tok d = lx->next();
            if (d.kind == Tok::kSymbol && d.s == "]") break;
            if (!(d.kind == Tok::kSymbol && d.s == ",")) return false;
          }
        }
      } else if (!encode_scalar(*f, lx->next(), w)) {
        return false;
      }
    }
    Tok s = lx->peek();
    if (s.kind == Tok::kSymbol && (s.s == "," || s.s == ";")) lx->next();
  }
}

}  // namespace

bool text_proto_to_wire(const char* data, size_t len, bool pauli_sum, std::string* wire) {
  Lexer lx{data, data + len};
  wire->clear();
  return parse_message(&lx, pauli_sum ? mPauliSum : mProgram, nullptr, wire, 0);
}

}  // namespace tfqg
