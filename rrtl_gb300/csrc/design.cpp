// Design IR loader and type rules. See design.h for the reference mapping.
#include "design.h"

#include <functional>

namespace rrtl {

uint32_t limbs_for(uint32_t width) {
  // crates/rrtl-sim-ir/src/lib.rs:12942-12944: width.div_ceil(32).max(1)
  uint32_t l = (width + 31) / 32;
  return l == 0 ? 1 : l;
}

uint32_t final_limb_mask(uint32_t width) {
  // crates/rrtl-sim-ir/src/lib.rs:12946-12953
  uint32_t rem = width % 32;
  return rem == 0 ? 0xFFFFFFFFu : ((1u << rem) - 1u);
}

std::vector<uint32_t> encode_limbs(i128 value, BitType ty) {
  // crates/rrtl-sim-ir/src/lib.rs:12955-12968: two's complement, limb-wise,
  // top limb masked; limbs beyond 128 bits carry the sign extension of the
  // u128 cast (which is zero after the shift-out in the reference).
  u128 enc = (u128)value;
  uint32_t n = limbs_for(ty.width);
  std::vector<uint32_t> out(n, 0);
  for (uint32_t i = 0; i < n; ++i) {
    out[i] = (uint32_t)enc;
    enc = (i < 3) ? (enc >> 32) : 0;
  }
  out[n - 1] &= final_limb_mask(ty.width);
  return out;
}

// ---------------------------------------------------------------- JSON load --

static SigRef sigref(const json::Value& v) {
  SigRef s;
  s.module = v.at("module").u32();
  s.id = v.at("id").u32();
  return s;
}

static BitType bittype(const json::Value& v) {
  BitType t;
  t.width = v.at("width").u32();
  const std::string& sg = v.at("signedness").str();
  t.is_signed = (sg == "Signed");
  return t;
}

static Expr expr_of(const json::Value& v);

static void two(const json::Value& arr, Expr& e) {
  if (!arr.is_arr() || arr.arr.size() != 2) throw RrtlError("E_DESIGN_JSON", "binary expression needs two operands");
  e.args.push_back(expr_of(arr.arr[0]));
  e.args.push_back(expr_of(arr.arr[1]));
}

static Expr expr_of(const json::Value& v) {
  if (!v.is_obj() || v.obj.size() != 1) throw RrtlError("E_DESIGN_JSON", "expression must be an externally tagged object");
  const std::string& tag = v.obj[0].first;
  const json::Value& b = v.obj[0].second;
  Expr e;
  if (tag == "Lit") {
    e.kind = EK::Lit;
    e.value = b.at("value").i128();
    e.ty = bittype(b.at("ty"));
  } else if (tag == "Signal") {
    e.kind = EK::Signal;
    e.sig = sigref(b);
  } else if (tag == "Not") {
    e.kind = EK::Not;
    e.args.push_back(expr_of(b));
  } else if (tag == "And") { e.kind = EK::And; two(b, e); }
  else if (tag == "Or") { e.kind = EK::Or; two(b, e); }
  else if (tag == "Xor") { e.kind = EK::Xor; two(b, e); }
  else if (tag == "Add") { e.kind = EK::Add; two(b, e); }
  else if (tag == "Sub") { e.kind = EK::Sub; two(b, e); }
  else if (tag == "Mul") { e.kind = EK::Mul; two(b, e); }
  else if (tag == "Eq") { e.kind = EK::Eq; two(b, e); }
  else if (tag == "Ne") { e.kind = EK::Ne; two(b, e); }
  else if (tag == "Lt") { e.kind = EK::Lt; two(b, e); }
  else if (tag == "Mux") {
    e.kind = EK::Mux;
    e.args.push_back(expr_of(b.at("cond")));
    e.args.push_back(expr_of(b.at("then_expr")));
    e.args.push_back(expr_of(b.at("else_expr")));
  } else if (tag == "Slice") {
    e.kind = EK::Slice;
    e.args.push_back(expr_of(b.at("expr")));
    e.lsb = b.at("lsb").u32();
    e.width = b.at("width").u32();
  } else if (tag == "Zext" || tag == "Sext" || tag == "Trunc") {
    e.kind = tag == "Zext" ? EK::Zext : tag == "Sext" ? EK::Sext : EK::Trunc;
    e.args.push_back(expr_of(b.at("expr")));
    e.width = b.at("width").u32();
  } else if (tag == "Cast") {
    e.kind = EK::Cast;
    e.args.push_back(expr_of(b.at("expr")));
    e.cast_signed = b.at("signedness").str() == "Signed";
  } else if (tag == "Concat") {
    e.kind = EK::Concat;
    if (!b.is_arr()) throw RrtlError("E_DESIGN_JSON", "Concat needs an array");
    for (auto& p : b.arr) e.args.push_back(expr_of(p));
  } else if (tag == "MemRead") {
    e.kind = EK::MemRead;
    e.sig = sigref(b.at("mem"));
    e.args.push_back(expr_of(b.at("addr")));
  } else {
    throw RrtlError("E_DESIGN_JSON", "unknown expression variant `" + tag + "`");
  }
  return e;
}

static Reset reset_of(const json::Value& v) {
  Reset r;
  r.signal = sigref(v.at("signal"));
  r.value = v.at("value").i128();
  r.async = v.at("kind").str() == "Async";
  r.active_low = v.at("polarity").str() == "ActiveLow";
  return r;
}

Design design_from_json(const char* text, size_t len) {
  json::Value root;
  try {
    root = json::parse(text, len);
  } catch (const std::exception& ex) {
    throw RrtlError("E_DESIGN_JSON", ex.what());
  }
  // Accept both `rrtl_ir::Design` ({"modules": [...]}) and the
  // `rrtl_core::Design` wrapper ({"ir": {"modules": [...]}}).
  const json::Value* mods = root.find("modules");
  if (!mods) {
    const json::Value* ir = root.find("ir");
    if (ir) mods = ir->find("modules");
  }
  if (!mods || !mods->is_arr()) throw RrtlError("E_DESIGN_JSON", "missing `modules` array");
  Design d;
  try {
    for (auto& mv : mods->arr) {
      Module m;
      m.id = mv.at("id").u32();
      m.name = mv.at("name").str();
      if (auto* ext = mv.find("is_external")) m.is_external = ext->boolean();
      for (auto& sv : mv.at("signals").arr) {
        SignalInfo s;
        s.handle = sigref(sv.at("handle"));
        s.name = sv.at("name").str();
        s.width = sv.at("width").u32();
        s.ty = bittype(sv.at("ty"));
        const json::Value& k = sv.at("kind");
        if (k.is_str()) {
          const std::string& ks = k.str();
          if (ks == "Input") s.kind = SigKind::Input;
          else if (ks == "Output") s.kind = SigKind::Output;
          else if (ks == "Inout") s.kind = SigKind::Inout;
          else if (ks == "Wire") s.kind = SigKind::Wire;
          else throw RrtlError("E_DESIGN_JSON", "unknown signal kind `" + ks + "`");
        } else if (k.is_obj() && k.obj.size() == 1) {
          const std::string& tag = k.obj[0].first;
          const json::Value& b = k.obj[0].second;
          if (tag == "Reg") {
            s.kind = SigKind::Reg;
            if (auto* c = b.find("clock"); c && !c->is_null()) s.clock = sigref(*c);
            if (auto* r = b.find("reset"); r && !r->is_null()) s.reset = reset_of(*r);
            if (auto* n = b.find("next"); n && !n->is_null()) s.next = expr_of(*n);
          } else if (tag == "Mem") {
            s.kind = SigKind::Mem;
            s.addr_width = b.at("addr_width").u32();
            s.data_width = b.at("data_width").u32();
            s.depth = b.at("depth").u64();
          } else {
            throw RrtlError("E_DESIGN_JSON", "unknown signal kind `" + tag + "`");
          }
        } else {
          throw RrtlError("E_DESIGN_JSON", "bad signal kind");
        }
        m.signals.push_back(std::move(s));
      }
      if (auto* a = mv.find("assignments"))
        for (auto& av : a->arr) m.assignments.push_back(Assignment{sigref(av.at("dst")), expr_of(av.at("expr"))});
      if (auto* w = mv.find("memory_writes"))
        for (auto& wv : w->arr) {
          MemoryWrite mw;
          mw.mem = sigref(wv.at("mem"));
          mw.clock = sigref(wv.at("clock"));
          mw.enable = expr_of(wv.at("enable"));
          mw.addr = expr_of(wv.at("addr"));
          mw.data = expr_of(wv.at("data"));
          m.memory_writes.push_back(std::move(mw));
        }
      if (auto* r = mv.find("initial_register_values"))
        for (auto& rv : r->arr) m.initial_register_values.push_back({sigref(rv.at("signal")), rv.at("value").i128()});
      if (auto* r = mv.find("initial_memory_values"))
        for (auto& rv : r->arr) m.initial_memory_values.push_back({sigref(rv.at("mem")), rv.at("addr").u64(), rv.at("value").i128()});
      if (auto* ins = mv.find("instances"))
        for (auto& iv : ins->arr) {
          Instance inst;
          inst.name = iv.at("name").str();
          inst.module = iv.at("module").str();
          for (auto& c : iv.at("connections").arr) {
            if (!c.is_arr() || c.arr.size() != 2) throw RrtlError("E_DESIGN_JSON", "bad instance connection");
            inst.connections.emplace_back(c.arr[0].str(), sigref(c.arr[1]));
          }
          m.instances.push_back(std::move(inst));
        }
      if (auto* as = mv.find("assertions")) m.n_assertions = as->arr.size();
      if (auto* cv = mv.find("cover_points")) m.n_cover_points = cv->arr.size();
      d.modules.push_back(std::move(m));
    }
  } catch (const RrtlError&) {
    throw;
  } catch (const std::exception& ex) {
    throw RrtlError("E_DESIGN_JSON", ex.what());
  }
  return d;
}

// -------------------------------------------------------------- type rules --

static std::string where(const Module& m) { return " [module: " + m.name + "]"; }

BitType expr_type(const Module& m, const Expr& e) {
  switch (e.kind) {
    case EK::Lit:
      if (e.ty.width == 0) throw RrtlError("E_LIT_WIDTH_ZERO", "literal width must be greater than zero" + where(m));
      return e.ty;
    case EK::Signal: {
      const SignalInfo* s = m.signal(e.sig);
      if (!s) throw RrtlError("E_SIGNAL_SCOPE", "signal does not belong to this module" + where(m));
      return s->ty;
    }
    case EK::Not:
      return expr_type(m, e.args[0]);
    case EK::And: case EK::Or: case EK::Xor: {
      BitType l = expr_type(m, e.args[0]), r = expr_type(m, e.args[1]);
      if (l != r) throw RrtlError("E_EXPR_TYPE", "expression type mismatch" + where(m));
      return l;
    }
    case EK::Add: case EK::Sub: case EK::Mul: {
      BitType l = expr_type(m, e.args[0]), r = expr_type(m, e.args[1]);
      if (l != r) {
        if (l.width == r.width) throw RrtlError("E_SIGNED_MIX", "mixed signedness requires an explicit cast" + where(m));
        throw RrtlError("E_EXPR_TYPE", "expression type mismatch" + where(m));
      }
      return l;
    }
    case EK::Eq: case EK::Ne: case EK::Lt: {
      BitType l = expr_type(m, e.args[0]), r = expr_type(m, e.args[1]);
      if (l != r) {
        if (l.width == r.width) throw RrtlError("E_SIGNED_MIX", "mixed signedness requires an explicit cast" + where(m));
        throw RrtlError("E_EXPR_TYPE", "expression type mismatch" + where(m));
      }
      return uint_t(1);
    }
    case EK::Mux: {
      BitType c = expr_type(m, e.args[0]);
      if (c != uint_t(1)) throw RrtlError("E_MUX_COND_WIDTH", "mux condition must be unsigned 1 bit" + where(m));
      BitType t = expr_type(m, e.args[1]), f = expr_type(m, e.args[2]);
      if (t != f) throw RrtlError("E_EXPR_TYPE", "expression type mismatch" + where(m));
      return t;
    }
    case EK::Slice: {
      if (e.width == 0) throw RrtlError("E_SLICE_WIDTH_ZERO", "slice width must be greater than zero" + where(m));
      BitType in = expr_type(m, e.args[0]);
      if (e.lsb + e.width > in.width) throw RrtlError("E_SLICE_RANGE", "slice exceeds expression width" + where(m));
      return uint_t(e.width);
    }
    case EK::Zext: case EK::Sext: {
      if (e.width == 0) throw RrtlError(e.kind == EK::Zext ? "E_ZEXT_WIDTH_ZERO" : "E_SEXT_WIDTH_ZERO", "extension width must be greater than zero" + where(m));
      BitType in = expr_type(m, e.args[0]);
      if (e.width < in.width) throw RrtlError(e.kind == EK::Zext ? "E_ZEXT_WIDTH" : "E_SEXT_WIDTH", "extension target narrower than source" + where(m));
      return e.kind == EK::Zext ? uint_t(e.width) : sint_t(e.width);
    }
    case EK::Trunc: {
      if (e.width == 0) throw RrtlError("E_TRUNC_WIDTH_ZERO", "trunc width must be greater than zero" + where(m));
      BitType in = expr_type(m, e.args[0]);
      if (e.width > in.width) throw RrtlError("E_TRUNC_WIDTH", "trunc target wider than source" + where(m));
      return BitType{e.width, in.is_signed};
    }
    case EK::Cast: {
      BitType in = expr_type(m, e.args[0]);
      return BitType{in.width, e.cast_signed};
    }
    case EK::Concat: {
      if (e.args.empty()) throw RrtlError("E_CONCAT_EMPTY", "concat needs at least one part" + where(m));
      uint32_t w = 0;
      for (auto& p : e.args) w += expr_type(m, p).width;
      return uint_t(w);
    }
    case EK::MemRead: {
      const SignalInfo* s = m.signal(e.sig);
      if (!s || s->kind != SigKind::Mem) throw RrtlError("E_MEM_READ_TARGET", "memory read target is not a memory" + where(m));
      BitType a = expr_type(m, e.args[0]);
      if (a != uint_t(s->addr_width)) throw RrtlError("E_MEM_ADDR_WIDTH", "memory read address type mismatch" + where(m));
      return s->ty;
    }
  }
  throw RrtlError("E_DESIGN_JSON", "bad expression kind");
}

void validate(const Design& d) {
  for (const Module& m : d.modules) {
    for (size_t i = 0; i < m.signals.size(); ++i) {
      const SignalInfo& s = m.signals[i];
      if (s.handle.module != m.id || s.handle.id != i)
        throw RrtlError("E_DESIGN_JSON", "signal handle does not match its position" + where(m));
      if (s.width == 0 || s.ty.width != s.width) throw RrtlError("E_SIGNAL_WIDTH", "signal `" + s.name + "` has a bad width" + where(m));
      if (s.kind == SigKind::Reg) {
        if (!s.clock) throw RrtlError("E_REG_CLOCK", "register `" + s.name + "` has no clock" + where(m));
        if (!s.next) throw RrtlError("E_REG_NEXT", "register `" + s.name + "` has no next-state expression" + where(m));
        BitType nt = expr_type(m, *s.next);
        if (nt.width != s.width) throw RrtlError("E_REG_NEXT_WIDTH", "register `" + s.name + "` next width mismatch" + where(m));
        if (s.reset && !m.signal(s.reset->signal)) throw RrtlError("E_RESET_SIGNAL", "reset signal out of scope" + where(m));
      }
      if (s.kind == SigKind::Mem && (s.depth == 0 || s.addr_width == 0 || s.addr_width > 64))
        throw RrtlError("E_MEM_SHAPE", "memory `" + s.name + "` has a bad shape" + where(m));
    }
    for (auto& a : m.assignments) {
      const SignalInfo* dst = m.signal(a.dst);
      if (!dst) throw RrtlError("E_SIGNAL_SCOPE", "assignment target out of scope" + where(m));
      BitType t = expr_type(m, a.expr);
      if (t.width != dst->width) throw RrtlError("E_ASSIGN_WIDTH", "assignment to `" + dst->name + "` width mismatch" + where(m));
    }
    for (auto& w : m.memory_writes) {
      const SignalInfo* mem = m.signal(w.mem);
      if (!mem || mem->kind != SigKind::Mem) throw RrtlError("E_MEM_WRITE_TARGET", "memory write target is not a memory" + where(m));
      if (expr_type(m, w.enable) != uint_t(1)) throw RrtlError("E_MEM_WRITE_ENABLE", "memory write enable must be uint(1)" + where(m));
      if (expr_type(m, w.addr) != uint_t(mem->addr_width)) throw RrtlError("E_MEM_ADDR_WIDTH", "memory write address type mismatch" + where(m));
      if (expr_type(m, w.data).width != mem->width) throw RrtlError("E_MEM_DATA_WIDTH", "memory write data width mismatch" + where(m));
    }
  }
}

}  // namespace rrtl
