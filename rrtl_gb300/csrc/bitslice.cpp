// Bit-slice lowering (see bitslice.h).
//
// Plane semantics follow the packed two-state rules
// (crates/rrtl-sim-ir/src/lib.rs:9796-9907, 12942-13196) as the reference's
// bit-slice engine evaluates them (crates/rrtl-sim-ir/src/bitslice.rs:121-389):
// operand planes past an operand's width are 0; add/sub wrap at the result
// width (sub as a + ~b + 1); eq/ne compare every plane of the operands;
// lt is the borrow out of a - b at the left operand's width (signed: with
// both sign planes inverted); mux selects on plane 0 of the condition; sext
// repeats the operand's top plane; concat is MSB-first.
#include "bitslice.h"

#include <cstdio>

namespace rrtl {

namespace {

struct Blaster {
  const PackedProgram& P;
  Module m;
  std::vector<std::vector<uint32_t>> planes;  // packed signal -> plane signal ids
  uint32_t clk = 0;
  uint32_t n_tmp = 0;

  explicit Blaster(const PackedProgram& p) : P(p) {}

  static std::string strip(const std::string& name, const std::string& top) {
    const std::string pre = top + ".";
    return name.compare(0, pre.size(), pre) == 0 ? name.substr(pre.size()) : name;
  }

  uint32_t add_signal(const std::string& name, SigKind kind) {
    SignalInfo s;
    s.handle = SigRef{0, (uint32_t)m.signals.size()};
    s.name = name;
    s.width = 1;
    s.ty = uint_t(1);
    s.kind = kind;
    m.signals.push_back(s);
    return s.handle.id;
  }

  // ---- 1-bit atoms: literal 0/1 or a plane signal
  static Expr lit(bool v) {
    Expr e;
    e.kind = EK::Lit;
    e.value = v ? 1 : 0;
    e.ty = uint_t(1);
    return e;
  }
  static Expr sig(uint32_t id) {
    Expr e;
    e.kind = EK::Signal;
    e.sig = SigRef{0, id};
    return e;
  }
  static bool is_lit(const Expr& e, bool* v) {
    if (e.kind != EK::Lit) return false;
    *v = e.value != 0;
    return true;
  }
  static bool same(const Expr& a, const Expr& b) {
    return a.kind == b.kind && (a.kind == EK::Lit ? a.value == b.value : a.sig == b.sig);
  }
  static Expr node(EK k, std::vector<Expr> args) {
    Expr e;
    e.kind = k;
    e.args = std::move(args);
    return e;
  }
  // a new wire holding a 1-bit expression of atoms
  Expr wire(Expr e) {
    const uint32_t id = add_signal("__bs" + std::to_string(n_tmp++), SigKind::Wire);
    m.assignments.push_back(Assignment{SigRef{0, id}, std::move(e)});
    return sig(id);
  }

  Expr NOT(const Expr& a) {
    bool v;
    if (is_lit(a, &v)) return lit(!v);
    return wire(node(EK::Not, {a}));
  }
  Expr AND(const Expr& a, const Expr& b) {
    bool v;
    if (is_lit(a, &v)) return v ? b : lit(false);
    if (is_lit(b, &v)) return v ? a : lit(false);
    if (same(a, b)) return a;
    return wire(node(EK::And, {a, b}));
  }
  Expr OR(const Expr& a, const Expr& b) {
    bool v;
    if (is_lit(a, &v)) return v ? lit(true) : b;
    if (is_lit(b, &v)) return v ? lit(true) : a;
    if (same(a, b)) return a;
    return wire(node(EK::Or, {a, b}));
  }
  Expr XOR(const Expr& a, const Expr& b) {
    bool v;
    if (is_lit(a, &v)) return v ? NOT(b) : b;
    if (is_lit(b, &v)) return v ? NOT(a) : a;
    if (same(a, b)) return lit(false);
    return wire(node(EK::Xor, {a, b}));
  }
  Expr MUX(const Expr& c, const Expr& t, const Expr& f) {
    bool v;
    if (is_lit(c, &v)) return v ? t : f;
    if (same(t, f)) return t;
    if (is_lit(t, &v) && is_lit(f, &v)) {
      bool tv, fv;
      is_lit(t, &tv);
      is_lit(f, &fv);
      return tv ? c : NOT(c);  // (1, 0) -> c; (0, 1) -> ~c
    }
    Expr e;
    e.kind = EK::Mux;
    e.args = {c, t, f};
    return wire(std::move(e));
  }
  // full adder: sum and carry out of a + b + c
  void add3(const Expr& a, const Expr& b, const Expr& c, Expr* sum, Expr* carry) {
    *sum = XOR(XOR(a, b), c);
    *carry = OR(AND(a, b), AND(c, XOR(a, b)));
  }

  static Expr at(const std::vector<Expr>& v, size_t i) { return i < v.size() ? v[i] : lit(false); }

  // OR of all planes (0 for none)
  Expr any(std::vector<Expr> v) {
    if (v.empty()) return lit(false);
    while (v.size() > 1) {
      std::vector<Expr> nx;
      for (size_t i = 0; i + 1 < v.size(); i += 2) nx.push_back(OR(v[i], v[i + 1]));
      if (v.size() & 1) nx.push_back(v.back());
      v.swap(nx);
    }
    return v[0];
  }

  // unsigned a < b over w planes: the borrow out of a - b
  Expr less(const std::vector<Expr>& a, const std::vector<Expr>& b, uint32_t w) {
    Expr borrow = lit(false);
    for (uint32_t i = 0; i < w; ++i) {
      // borrow' = (~a & b) | (~(a ^ b) & borrow)
      const Expr ai = at(a, i), bi = at(b, i);
      borrow = OR(AND(NOT(ai), bi), AND(NOT(XOR(ai, bi)), borrow));
    }
    return borrow;
  }

  [[noreturn]] static void scope(const std::string& what) { throw RrtlError("E_BITSLICE", what); }

  std::vector<Expr> blast(const PackedExpr& e) {
    const uint32_t w = e.ty.width;
    std::vector<Expr> out;
    switch (e.kind) {
      case PK::Lit:
        for (uint32_t i = 0; i < w; ++i) {
          const uint32_t limb = i / 32;
          out.push_back(lit(limb < e.lit.size() && ((e.lit[limb] >> (i % 32)) & 1u)));
        }
        return out;
      case PK::Signal: {
        const auto& pl = planes.at(e.index);
        for (uint32_t i = 0; i < w; ++i) out.push_back(i < pl.size() ? sig(pl[i]) : lit(false));
        return out;
      }
      case PK::Not: {
        auto a = blast(e.args[0]);
        for (uint32_t i = 0; i < w; ++i) out.push_back(NOT(at(a, i)));
        return out;
      }
      case PK::And:
      case PK::Or:
      case PK::Xor: {
        auto a = blast(e.args[0]), b = blast(e.args[1]);
        for (uint32_t i = 0; i < w; ++i)
          out.push_back(e.kind == PK::And ? AND(at(a, i), at(b, i))
                                          : e.kind == PK::Or ? OR(at(a, i), at(b, i)) : XOR(at(a, i), at(b, i)));
        return out;
      }
      case PK::Add:
      case PK::Sub: {
        auto a = blast(e.args[0]), b = blast(e.args[1]);
        const bool sub = e.kind == PK::Sub;
        Expr carry = lit(sub);
        for (uint32_t i = 0; i < w; ++i) {
          Expr bi = at(b, i);
          if (sub) bi = NOT(bi);
          Expr s, c;
          add3(at(a, i), bi, carry, &s, &c);
          out.push_back(s);
          carry = c;
        }
        return out;
      }
      case PK::Eq:
      case PK::Ne: {
        auto a = blast(e.args[0]), b = blast(e.args[1]);
        std::vector<Expr> d;
        for (size_t i = 0; i < std::max(a.size(), b.size()); ++i) d.push_back(XOR(at(a, i), at(b, i)));
        Expr ne = any(d);
        out.push_back(e.kind == PK::Ne ? ne : NOT(ne));
        for (uint32_t i = 1; i < w; ++i) out.push_back(lit(false));
        return out;
      }
      case PK::Lt: {
        auto a = blast(e.args[0]), b = blast(e.args[1]);
        const uint32_t wl = e.args[0].ty.width;
        if (e.is_signed && wl > 0) {
          a.resize(std::max<size_t>(a.size(), wl), lit(false));
          b.resize(std::max<size_t>(b.size(), wl), lit(false));
          a[wl - 1] = NOT(a[wl - 1]);
          b[wl - 1] = NOT(b[wl - 1]);
        }
        out.push_back(less(a, b, wl));
        for (uint32_t i = 1; i < w; ++i) out.push_back(lit(false));
        return out;
      }
      case PK::Mux: {
        auto c = blast(e.args[0]), t = blast(e.args[1]), f = blast(e.args[2]);
        const Expr c0 = at(c, 0);
        for (uint32_t i = 0; i < w; ++i) out.push_back(MUX(c0, at(t, i), at(f, i)));
        return out;
      }
      case PK::Slice: {
        auto a = blast(e.args[0]);
        for (uint32_t i = 0; i < w; ++i) out.push_back(at(a, (size_t)e.lsb + i));
        return out;
      }
      case PK::Zext:
      case PK::Trunc:
      case PK::Cast: {
        auto a = blast(e.args[0]);
        for (uint32_t i = 0; i < w; ++i) out.push_back(at(a, i));
        return out;
      }
      case PK::Sext: {
        auto a = blast(e.args[0]);
        const uint32_t wo = e.args[0].ty.width;
        for (uint32_t i = 0; i < w; ++i) out.push_back(i < wo ? at(a, i) : (wo ? at(a, wo - 1) : lit(false)));
        return out;
      }
      case PK::Concat: {
        // MSB-first: the last operand supplies the lowest planes
        for (size_t k = e.args.size(); k-- > 0;) {
          auto a = blast(e.args[k]);
          for (uint32_t i = 0; i < e.args[k].ty.width; ++i) out.push_back(at(a, i));
        }
        out.resize(w, lit(false));
        return out;
      }
      case PK::Mul: scope("multiply is outside the bit-slice engine");
      case PK::MemRead: scope("memories are outside the bit-slice engine");
    }
    scope("unknown expression");
  }

  Design run() {
    m.id = 0;
    m.name = P.top;
    if (!P.memories.empty()) scope("memories are outside the bit-slice engine");
    if (!P.async_reset_comb.empty())
      for (auto& pk : P.async_reset_comb)
        if (!pk.empty()) scope("asynchronous resets are outside the bit-slice engine");
    // planes of every packed signal
    planes.resize(P.signals.size());
    for (size_t s = 0; s < P.signals.size(); ++s) {
      const PackedSignal& ps = P.signals[s];
      // ports of flattened instances are driven by their connections: wires
      const SigKind k = ps.kind == PSK::Reg ? SigKind::Reg
                        : !ps.top ? SigKind::Wire
                        : ps.kind == PSK::Input ? SigKind::Input
                        : ps.kind == PSK::Output ? SigKind::Output : SigKind::Wire;
      const std::string base = strip(ps.name, P.top);
      for (uint32_t b = 0; b < ps.layout.width; ++b) planes[s].push_back(add_signal(base + "[" + std::to_string(b) + "]", k));
    }
    clk = add_signal("__bitslice_clk", SigKind::Input);
    for (auto& pk : P.comb)
      for (const PackedOp& op : pk) {
        if (op.kind != POK::Assign) scope("unexpected effect in the comb stream");
        auto bits = blast(op.expr);
        const auto& pl = planes.at(op.dst);
        for (size_t b = 0; b < pl.size(); ++b) m.assignments.push_back(Assignment{SigRef{0, pl[b]}, at(bits, b)});
      }
    for (auto& pk : P.tick_next)
      for (const PackedOp& op : pk) {
        if (op.kind != POK::CaptureReg) scope("unexpected effect in the register stream");
        if (op.has_reset && op.reset.async) scope("asynchronous resets are outside the bit-slice engine");
        auto bits = blast(op.expr);
        const auto& pl = planes.at(op.dst);
        for (size_t b = 0; b < pl.size(); ++b) {
          SignalInfo& s = m.signals[pl[b]];
          s.kind = SigKind::Reg;
          s.clock = SigRef{0, clk};
          s.next = at(bits, b);
          if (op.has_reset) {
            Reset r;
            r.signal = SigRef{0, planes.at(op.reset.signal).at(0)};
            const uint32_t limb = (uint32_t)(b / 32);
            r.value = (limb < op.reset.value.size() && ((op.reset.value[limb] >> (b % 32)) & 1u)) ? 1 : 0;
            r.async = false;
            r.active_low = op.reset.active_low;
            s.reset = r;
          }
        }
      }
    for (auto& pk : P.tick_commit)
      if (!pk.empty()) scope("memories are outside the bit-slice engine");
    Design d;
    d.modules.push_back(std::move(m));
    return d;
  }
};

// ---- JSON writer
std::string jsig(SigRef s) { return "{\"module\": " + std::to_string(s.module) + ", \"id\": " + std::to_string(s.id) + "}"; }
std::string jty(BitType t) {
  return "{\"width\": " + std::to_string(t.width) + ", \"signedness\": \"" + (t.is_signed ? "Signed" : "Unsigned") + "\"}";
}
std::string jint(i128 v) {
  if (v == 0) return "0";
  bool neg = v < 0;
  u128 u = neg ? (u128)(-v) : (u128)v;
  std::string s;
  while (u) {
    s.insert(s.begin(), (char)('0' + (int)(u % 10)));
    u /= 10;
  }
  return neg ? "-" + s : s;
}
std::string jstr(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
  }
  return o + "\"";
}
std::string jexpr(const Expr& e) {
  auto two = [&](const char* tag) { return std::string("{\"") + tag + "\": [" + jexpr(e.args[0]) + ", " + jexpr(e.args[1]) + "]}"; };
  switch (e.kind) {
    case EK::Lit: return "{\"Lit\": {\"value\": " + jint(e.value) + ", \"ty\": " + jty(e.ty) + "}}";
    case EK::Signal: return "{\"Signal\": " + jsig(e.sig) + "}";
    case EK::Not: return "{\"Not\": " + jexpr(e.args[0]) + "}";
    case EK::And: return two("And");
    case EK::Or: return two("Or");
    case EK::Xor: return two("Xor");
    case EK::Add: return two("Add");
    case EK::Sub: return two("Sub");
    case EK::Mul: return two("Mul");
    case EK::Eq: return two("Eq");
    case EK::Ne: return two("Ne");
    case EK::Lt: return two("Lt");
    case EK::Mux:
      return "{\"Mux\": {\"cond\": " + jexpr(e.args[0]) + ", \"then_expr\": " + jexpr(e.args[1]) +
             ", \"else_expr\": " + jexpr(e.args[2]) + "}}";
    case EK::Slice:
      return "{\"Slice\": {\"expr\": " + jexpr(e.args[0]) + ", \"lsb\": " + std::to_string(e.lsb) +
             ", \"width\": " + std::to_string(e.width) + "}}";
    case EK::Zext:
    case EK::Sext:
    case EK::Trunc: {
      const char* tag = e.kind == EK::Zext ? "Zext" : e.kind == EK::Sext ? "Sext" : "Trunc";
      return std::string("{\"") + tag + "\": {\"expr\": " + jexpr(e.args[0]) + ", \"width\": " + std::to_string(e.width) + "}}";
    }
    case EK::Cast:
      return "{\"Cast\": {\"expr\": " + jexpr(e.args[0]) + ", \"signedness\": \"" + (e.cast_signed ? "Signed" : "Unsigned") + "\"}}";
    case EK::Concat: {
      std::string o = "{\"Concat\": [";
      for (size_t i = 0; i < e.args.size(); ++i) o += (i ? ", " : "") + jexpr(e.args[i]);
      return o + "]}";
    }
    case EK::MemRead: return "{\"MemRead\": {\"mem\": " + jsig(e.sig) + ", \"addr\": " + jexpr(e.args[0]) + "}}";
  }
  return "null";
}

}  // namespace

Design bitslice_design(const PackedProgram& P) { return Blaster(P).run(); }

std::string design_to_json(const Design& d) {
  std::string o = "{\"modules\": [";
  for (size_t mi = 0; mi < d.modules.size(); ++mi) {
    const Module& m = d.modules[mi];
    o += mi ? ", " : "";
    o += "{\"id\": " + std::to_string(m.id) + ", \"name\": " + jstr(m.name) + ", \"is_external\": " +
         (m.is_external ? "true" : "false") + ", \"signals\": [";
    for (size_t i = 0; i < m.signals.size(); ++i) {
      const SignalInfo& s = m.signals[i];
      o += i ? ", " : "";
      o += "{\"handle\": " + jsig(s.handle) + ", \"name\": " + jstr(s.name) + ", \"width\": " + std::to_string(s.width) +
           ", \"ty\": " + jty(s.ty) + ", \"kind\": ";
      switch (s.kind) {
        case SigKind::Input: o += "\"Input\""; break;
        case SigKind::Output: o += "\"Output\""; break;
        case SigKind::Inout: o += "\"Inout\""; break;
        case SigKind::Wire: o += "\"Wire\""; break;
        case SigKind::Reg: {
          o += "{\"Reg\": {\"clock\": " + (s.clock ? jsig(*s.clock) : std::string("null")) + ", \"reset\": ";
          if (s.reset)
            o += "{\"signal\": " + jsig(s.reset->signal) + ", \"value\": " + jint(s.reset->value) + ", \"kind\": \"" +
                 (s.reset->async ? "Async" : "Sync") + "\", \"polarity\": \"" +
                 (s.reset->active_low ? "ActiveLow" : "ActiveHigh") + "\"}";
          else
            o += "null";
          o += ", \"next\": " + (s.next ? jexpr(*s.next) : std::string("null")) + "}}";
          break;
        }
        case SigKind::Mem:
          o += "{\"Mem\": {\"addr_width\": " + std::to_string(s.addr_width) + ", \"data_width\": " +
               std::to_string(s.data_width) + ", \"depth\": " + std::to_string(s.depth) + "}}";
          break;
      }
      o += "}";
    }
    o += "], \"assignments\": [";
    for (size_t i = 0; i < m.assignments.size(); ++i)
      o += (i ? ", " : "") + std::string("{\"dst\": ") + jsig(m.assignments[i].dst) + ", \"expr\": " +
           jexpr(m.assignments[i].expr) + "}";
    o += "], \"memory_writes\": [], \"instances\": []}";
  }
  return o + "]}";
}

}  // namespace rrtl
