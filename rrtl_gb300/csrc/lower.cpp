// Packed and machine lowering. Each step cites the reference function it
// restates; identical inputs give identical signal/memory layouts, stream
// contents and packet structure.
#include "lower.h"

#include <functional>
#include <unordered_set>

namespace rrtl {

// ----------------------------------------------------------- PackedExpr ---

static inline size_t mix(size_t h, size_t v) {
  return h ^ (v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2));
}

void PackedExpr::finish() {
  size_t h = (size_t)kind * 0x100000001b3ull;
  h = mix(h, ty.width * 2 + (ty.is_signed ? 1 : 0));
  for (uint32_t l : lit) h = mix(h, l);
  h = mix(h, index);
  h = mix(h, lsb);
  h = mix(h, is_signed);
  for (auto& a : args) h = mix(h, a.hash);
  hash = h;
}

bool PackedExpr::operator==(const PackedExpr& o) const {
  if (hash != o.hash || kind != o.kind || ty != o.ty || index != o.index || lsb != o.lsb ||
      is_signed != o.is_signed || lit != o.lit || args.size() != o.args.size())
    return false;
  for (size_t i = 0; i < args.size(); ++i)
    if (!(args[i] == o.args[i])) return false;
  return true;
}

struct PEHash {
  size_t operator()(const PackedExpr& e) const { return e.hash; }
};

// ------------------------------------------------------- packed lowering ---

namespace {

// `expr_type` used by the packed lowering (crates/rrtl-sim-ir/src/lib.rs:12902-12940):
// Not/And/Or/Xor/Add/Sub/Mul take their left operand's type, Mux its then arm.
std::optional<BitType> lower_expr_type(const Module& m, const Expr& e) {
  switch (e.kind) {
    case EK::Lit: return e.ty;
    case EK::Signal: {
      const SignalInfo* s = m.signal(e.sig);
      if (!s) return std::nullopt;
      return s->ty;
    }
    case EK::Not: case EK::And: case EK::Or: case EK::Xor: case EK::Add: case EK::Sub: case EK::Mul:
      return lower_expr_type(m, e.args[0]);
    case EK::Eq: case EK::Ne: case EK::Lt: return uint_t(1);
    case EK::Mux: return lower_expr_type(m, e.args[1]);
    case EK::Slice: return uint_t(e.width);
    case EK::Zext: return uint_t(e.width);
    case EK::Sext: return sint_t(e.width);
    case EK::Trunc: {
      auto in = lower_expr_type(m, e.args[0]);
      if (!in) return std::nullopt;
      return BitType{e.width, in->is_signed};
    }
    case EK::Cast: {
      auto in = lower_expr_type(m, e.args[0]);
      if (!in) return std::nullopt;
      return BitType{in->width, e.cast_signed};
    }
    case EK::Concat: {
      uint32_t w = 0;
      for (auto& p : e.args) {
        auto t = lower_expr_type(m, p);
        if (!t) return std::nullopt;
        w += t->width;
      }
      return uint_t(w);
    }
    case EK::MemRead: {
      const SignalInfo* s = m.signal(e.sig);
      if (!s) return std::nullopt;
      return s->ty;
    }
  }
  return std::nullopt;
}

struct Ctx {
  std::string path;
  const Module* module;
};

struct RegRef {
  uint32_t signal;
  PackedExpr next;
  bool has_reset = false;
  PackedReset reset;
};

struct Lowering {
  const Design& d;
  std::vector<Ctx> contexts;
  std::vector<PackedSignal> signals;
  std::vector<PackedMemory> memories;
  std::unordered_map<uint64_t, uint32_t> signal_map, memory_map;  // (instance<<32|signal id)
  std::unordered_map<uint32_t, uint32_t> top_signal_index, top_memory_index;
  std::vector<std::pair<uint32_t, PackedExpr>> assignments;
  std::vector<RegRef> registers;
  std::vector<PackedOp> memory_writes;
  uint64_t next_signal_offset = 0, next_memory_offset = 0;

  explicit Lowering(const Design& design) : d(design) {}

  // Lowering::add_context (crates/rrtl-sim-ir/src/lib.rs:12307-12338): pre-order.
  void add_context(const Module* module, const std::string& path) {
    size_t index = contexts.size();
    for (auto& inst : module->instances) {
      const Module* target = d.find_module(inst.module);
      if (!target) throw RrtlError("E_SIM_IR_INSTANCE", "instance target `" + inst.module + "` does not exist");
      if (target->is_external) throw RrtlError("E_SIM_IR_EXTERN", "instance `" + inst.name + "` targets external module `" + target->name + "`");
      add_context(target, path + "." + inst.name);
    }
    contexts.insert(contexts.begin() + index, Ctx{path, module});
  }

  static uint64_t key(size_t inst, uint32_t sig) { return ((uint64_t)inst << 32) | sig; }

  // Lowering::allocate_contexts (crates/rrtl-sim-ir/src/lib.rs:12340-12414).
  void allocate_contexts() {
    for (size_t inst = 0; inst < contexts.size(); ++inst) {
      const Module& m = *contexts[inst].module;
      if (m.n_assertions || m.n_cover_points)
        throw RrtlError("E_SIM_IR_ASSERT_COVER", "packed simulation IR does not support assertions or cover points");
      for (auto& s : m.signals) {
        if (s.kind == SigKind::Inout) throw RrtlError("E_SIM_IR_INOUT", "packed simulation IR does not support inout");
        if (s.kind == SigKind::Mem) {
          PackedMemory pm;
          pm.name = contexts[inst].path + "." + s.name;
          pm.src_id = s.handle.id;
          pm.top = inst == 0;
          pm.owner_path = contexts[inst].path;
          pm.addr_width = s.addr_width;
          pm.depth = s.depth;
          pm.data_layout = ValueLayout{s.ty.width, s.ty, 0, limbs_for(s.ty.width)};
          pm.offset = next_memory_offset;
          memory_map[key(inst, s.handle.id)] = (uint32_t)memories.size();
          if (inst == 0) top_memory_index[s.handle.id] = (uint32_t)memories.size();
          memories.push_back(pm);
          next_memory_offset += s.depth * pm.data_layout.limbs;
        } else {
          PackedSignal ps;
          ps.name = contexts[inst].path + "." + s.name;
          ps.top = inst == 0;
          ps.src_id = s.handle.id;
          ps.owner_path = contexts[inst].path;
          ps.layout = ValueLayout{s.ty.width, s.ty, (uint32_t)next_signal_offset, limbs_for(s.ty.width)};
          next_signal_offset += ps.layout.limbs;
          ps.kind = s.kind == SigKind::Input ? PSK::Input : s.kind == SigKind::Output ? PSK::Output
                    : s.kind == SigKind::Reg ? PSK::Reg : PSK::Wire;
          signal_map[key(inst, s.handle.id)] = (uint32_t)signals.size();
          if (inst == 0) top_signal_index[s.handle.id] = (uint32_t)signals.size();
          signals.push_back(std::move(ps));
        }
      }
    }
  }

  uint32_t signal_index(size_t inst, SigRef s, bool* ok) {
    auto it = signal_map.find(key(inst, s.id));
    if (it == signal_map.end() || s.module != contexts[inst].module->id) {
      *ok = false;
      return 0;
    }
    *ok = true;
    return it->second;
  }

  PackedExpr signal_expr(uint32_t index) {
    PackedExpr e;
    e.kind = PK::Signal;
    e.index = index;
    e.ty = signals[index].layout.ty;
    e.finish();
    return e;
  }

  // Lowering::lower_raw_expr (crates/rrtl-sim-ir/src/lib.rs:12505-12620).
  PackedExpr lower_raw(size_t inst, const Module& m, const Expr& e, BitType ty) {
    PackedExpr out;
    out.ty = ty;
    auto bin = [&](PK k) {
      BitType lt = lower_expr_type(m, e.args[0]).value_or(ty);
      out.kind = k;
      out.args.push_back(lower_raw(inst, m, e.args[0], lt));
      out.args.push_back(lower_raw(inst, m, e.args[1], lt));
    };
    switch (e.kind) {
      case EK::Lit:
        out.kind = PK::Lit;
        out.lit = encode_limbs(e.value, e.ty);
        break;
      case EK::Signal: {
        bool ok;
        uint32_t idx = signal_index(inst, e.sig, &ok);
        if (!ok) throw RrtlError("E_SIM_IR_SIGNAL", "signal is not a packed scalar signal [module: " + m.name + "]");
        out.kind = PK::Signal;
        out.index = idx;
        break;
      }
      case EK::Not:
        out.kind = PK::Not;
        out.args.push_back(lower_raw(inst, m, e.args[0], ty));
        break;
      case EK::And: bin(PK::And); break;
      case EK::Or: bin(PK::Or); break;
      case EK::Xor: bin(PK::Xor); break;
      case EK::Add: bin(PK::Add); break;
      case EK::Sub: bin(PK::Sub); break;
      case EK::Mul: bin(PK::Mul); break;
      case EK::Eq: bin(PK::Eq); break;
      case EK::Ne: bin(PK::Ne); break;
      case EK::Lt: {
        BitType lt = lower_expr_type(m, e.args[0]).value_or(ty);
        out.kind = PK::Lt;
        out.args.push_back(lower_raw(inst, m, e.args[0], lt));
        out.args.push_back(lower_raw(inst, m, e.args[1], lt));
        out.is_signed = lt.is_signed;
        break;
      }
      case EK::Mux:
        out.kind = PK::Mux;
        out.args.push_back(lower_raw(inst, m, e.args[0], uint_t(1)));
        out.args.push_back(lower_raw(inst, m, e.args[1], ty));
        out.args.push_back(lower_raw(inst, m, e.args[2], ty));
        break;
      case EK::Slice: {
        BitType it = lower_expr_type(m, e.args[0]).value_or(ty);
        out.kind = PK::Slice;
        out.args.push_back(lower_raw(inst, m, e.args[0], it));
        out.lsb = e.lsb;
        break;
      }
      case EK::Zext: case EK::Sext: case EK::Trunc: case EK::Cast: {
        BitType it = lower_expr_type(m, e.args[0]).value_or(ty);
        out.kind = e.kind == EK::Zext ? PK::Zext : e.kind == EK::Sext ? PK::Sext : e.kind == EK::Trunc ? PK::Trunc : PK::Cast;
        out.args.push_back(lower_raw(inst, m, e.args[0], it));
        break;
      }
      case EK::Concat:
        out.kind = PK::Concat;
        for (auto& p : e.args) out.args.push_back(lower_raw(inst, m, p, lower_expr_type(m, p).value_or(uint_t(1))));
        break;
      case EK::MemRead: {
        auto it = memory_map.find(key(inst, e.sig.id));
        if (it == memory_map.end()) throw RrtlError("E_SIM_IR_MEMORY", "signal is not a packed memory [module: " + m.name + "]");
        out.kind = PK::MemRead;
        out.index = it->second;
        out.args.push_back(lower_raw(inst, m, e.args[0], lower_expr_type(m, e.args[0]).value_or(uint_t(32))));
        break;
      }
    }
    out.finish();
    return out;
  }

  PackedExpr lower_compiled(size_t inst, const Module& m, const Expr& e) {
    // CompiledExpr carries `expr_type` from the compiler (crates/rrtl-core/src/lib.rs:3592-3602).
    return lower_raw(inst, m, e, expr_type(m, e));
  }

  int find_child_context(size_t parent, const std::string& name) {
    std::string want = contexts[parent].path + "." + name;
    for (size_t i = 0; i < contexts.size(); ++i)
      if (contexts[i].path == want) return (int)i;
    return -1;
  }

  // Lowering::lower_contexts (crates/rrtl-sim-ir/src/lib.rs:12416-12503).
  void lower_contexts() {
    for (size_t inst = 0; inst < contexts.size(); ++inst) {
      const Module& m = *contexts[inst].module;
      for (auto& a : m.assignments) {
        bool ok;
        uint32_t dst = signal_index(inst, a.dst, &ok);
        if (!ok) throw RrtlError("E_SIM_IR_SIGNAL", "assignment target is not a packed scalar signal [module: " + m.name + "]");
        assignments.emplace_back(dst, lower_compiled(inst, m, a.expr));
      }
      for (auto& child : m.instances) {
        int ci = find_child_context(inst, child.name);
        if (ci < 0) continue;
        const Module* cm = d.find_module(child.module);
        if (!cm) continue;
        for (auto& conn : child.connections) {
          const SignalInfo* port = nullptr;
          for (auto& s : cm->signals)
            if (s.name == conn.first && (s.kind == SigKind::Input || s.kind == SigKind::Output || s.kind == SigKind::Inout)) {
              port = &s;
              break;
            }
          if (!port) continue;
          bool ok1, ok2;
          if (port->kind == SigKind::Input) {
            uint32_t dst = signal_index(ci, port->handle, &ok1);
            uint32_t src = signal_index(inst, conn.second, &ok2);
            if (ok1 && ok2) assignments.emplace_back(dst, signal_expr(src));
          } else if (port->kind == SigKind::Output) {
            uint32_t dst = signal_index(inst, conn.second, &ok1);
            uint32_t src = signal_index(ci, port->handle, &ok2);
            if (ok1 && ok2) assignments.emplace_back(dst, signal_expr(src));
          }
        }
      }
      for (auto& s : m.signals) {
        if (s.kind != SigKind::Reg) continue;
        bool ok;
        uint32_t sig = signal_index(inst, s.handle, &ok);
        RegRef r;
        r.signal = sig;
        r.next = lower_compiled(inst, m, *s.next);
        if (s.reset) {
          bool rok;
          uint32_t rs = signal_index(inst, s.reset->signal, &rok);
          if (rok) {
            r.has_reset = true;
            r.reset.signal = rs;
            r.reset.value = encode_limbs(s.reset->value, r.next.ty);
            r.reset.async = s.reset->async;
            r.reset.active_low = s.reset->active_low;
          }
        }
        registers.push_back(std::move(r));
      }
      for (auto& w : m.memory_writes) {
        auto it = memory_map.find(key(inst, w.mem.id));
        if (it == memory_map.end()) throw RrtlError("E_SIM_IR_MEMORY", "memory write target is not a packed memory");
        PackedOp op;
        op.kind = POK::MemoryWrite;
        op.dst = it->second;
        op.expr = lower_compiled(inst, m, w.enable);
        op.addr = lower_compiled(inst, m, w.addr);
        op.data = lower_compiled(inst, m, w.data);
        memory_writes.push_back(std::move(op));
      }
    }
  }
};

void collect_signal_deps(const PackedExpr& e, std::unordered_set<uint32_t>& deps) {
  if (e.kind == PK::Signal) deps.insert(e.index);
  for (auto& a : e.args) collect_signal_deps(a, deps);
}

// schedule_assignments / assignment_level (crates/rrtl-sim-ir/src/lib.rs:12734-12789).
std::vector<std::vector<PackedOp>> schedule_assignments(const std::vector<std::pair<uint32_t, PackedExpr>>& as) {
  std::unordered_map<uint32_t, size_t> dst_to;
  for (size_t i = 0; i < as.size(); ++i) dst_to[as[i].first] = i;
  std::vector<std::vector<uint32_t>> deps(as.size());
  for (size_t i = 0; i < as.size(); ++i) {
    std::unordered_set<uint32_t> sd;
    collect_signal_deps(as[i].second, sd);
    for (uint32_t s : sd) {
      auto it = dst_to.find(s);
      if (it != dst_to.end() && it->second != i) deps[i].push_back((uint32_t)it->second);
    }
  }
  std::vector<int64_t> memo(as.size(), -1);
  std::vector<char> visiting(as.size(), 0);
  // The reference's recursive assignment_level restated as a DFS over an
  // explicit stack (a 100k-deep chain of wires must not recurse 100k frames
  // deep on the host stack). Same visiting order and cycle rule: a node
  // re-entered while on the stack contributes level 0, and every node is
  // memoised when its own visit ends.
  struct Frame {
    size_t node;
    size_t next_dep;
    int64_t lv;
  };
  std::vector<Frame> stack;
  auto level = [&](size_t root) -> int64_t {
    if (memo[root] >= 0) return memo[root];
    int64_t result = 0;
    visiting[root] = 1;
    stack.push_back(Frame{root, 0, 0});
    while (!stack.empty()) {
      const size_t top = stack.size() - 1;
      const size_t node = stack[top].node;
      if (stack[top].next_dep < deps[node].size()) {
        const uint32_t d = deps[node][stack[top].next_dep++];
        int64_t child;
        if (memo[d] >= 0) {
          child = memo[d];
        } else if (visiting[d]) {
          child = 0;
        } else {
          visiting[d] = 1;
          stack.push_back(Frame{d, 0, 0});
          continue;
        }
        stack[top].lv = std::max(stack[top].lv, child + 1);
        continue;
      }
      const int64_t lv = stack[top].lv;
      visiting[node] = 0;
      memo[node] = lv;
      stack.pop_back();
      if (stack.empty()) result = lv;
      else stack.back().lv = std::max(stack.back().lv, lv + 1);
    }
    return result;
  };
  std::vector<std::vector<PackedOp>> levels;
  for (size_t i = 0; i < as.size(); ++i) {
    int64_t lv = level(i);
    if ((int64_t)levels.size() <= lv) levels.resize(lv + 1);
    PackedOp op;
    op.kind = POK::Assign;
    op.dst = as[i].first;
    op.expr = as[i].second;
    levels[lv].push_back(std::move(op));
  }
  std::vector<std::vector<PackedOp>> out;
  for (auto& l : levels)
    if (!l.empty()) out.push_back(std::move(l));
  return out;
}

}  // namespace

PackedProgram lower_to_packed_program(const Design& d, const std::string& top) {
  const Module* tm = d.find_module(top);
  if (!tm) throw RrtlError("E_SIM_IR_MODULE", "module `" + top + "` does not exist");
  if (tm->is_external) throw RrtlError("E_SIM_IR_EXTERN", "packed simulation IR does not support external top modules");
  validate(d);
  Lowering L(d);
  L.add_context(tm, top);
  L.allocate_contexts();
  L.lower_contexts();

  PackedProgram p;
  p.top = top;
  p.comb = schedule_assignments(L.assignments);
  // schedule_async_resets (crates/rrtl-sim-ir/src/lib.rs:12791-12814)
  std::vector<PackedOp> async_ops;
  for (auto& r : L.registers) {
    if (!r.has_reset || !r.reset.async) continue;
    PackedOp op;
    op.kind = POK::CaptureReg;
    op.dst = r.signal;
    op.expr.kind = PK::Lit;
    op.expr.lit = r.reset.value;
    op.expr.ty = r.next.ty;
    op.expr.finish();
    op.has_reset = true;
    op.reset = r.reset;
    async_ops.push_back(std::move(op));
  }
  if (!async_ops.empty()) p.async_reset_comb.push_back(std::move(async_ops));
  // schedule_tick_next (crates/rrtl-sim-ir/src/lib.rs:12816-12830)
  std::vector<PackedOp> tn;
  for (auto& r : L.registers) {
    PackedOp op;
    op.kind = POK::CaptureReg;
    op.dst = r.signal;
    op.expr = r.next;
    op.has_reset = r.has_reset;
    op.reset = r.reset;
    tn.push_back(std::move(op));
  }
  if (!tn.empty()) p.tick_next.push_back(std::move(tn));
  // schedule_memory_writes (crates/rrtl-sim-ir/src/lib.rs:12832-12840)
  if (!L.memory_writes.empty()) p.tick_commit.push_back(std::move(L.memory_writes));

  p.signals = std::move(L.signals);
  p.memories = std::move(L.memories);
  p.top_signal_index = std::move(L.top_signal_index);
  p.top_memory_index = std::move(L.top_memory_index);
  p.total_signal_words = L.next_signal_offset;
  p.total_memory_words_per_lane = L.next_memory_offset;
  return p;
}

// ------------------------------------------------------ machine lowering ---

static const std::vector<uint32_t> kNoDeps;

const std::vector<uint32_t>& instr_deps(const Instr& i) {
  if (i.kind == IK::Lit || i.kind == IK::Signal) return kNoDeps;
  return i.ops;
}

namespace {

// MachinePacketLowerer (crates/rrtl-sim-ir/src/lib.rs:3051-3138): post-order
// SSA with a per-packet structural CSE memo; value ids are block-global.
struct PacketLowerer {
  uint32_t next_value;
  std::unordered_map<PackedExpr, uint32_t, PEHash> memo;
  std::vector<Instr> instrs;
  std::vector<uint32_t>* widths;

  uint32_t lower(const PackedExpr& e) {
    auto it = memo.find(e);
    if (it != memo.end()) return it->second;
    Instr in;
    in.kind = e.kind;
    in.ty = e.ty;
    in.lit = e.lit;
    in.index = e.index;
    in.lsb = e.lsb;
    in.is_signed = e.is_signed;
    for (auto& a : e.args) in.ops.push_back(lower(a));
    in.dst = next_value++;
    if (widths->size() <= in.dst) widths->resize(in.dst + 1, 0);
    (*widths)[in.dst] = e.ty.width;
    instrs.push_back(std::move(in));
    memo.emplace(e, instrs.back().dst);
    return instrs.back().dst;
  }
};

// schedule_machine_instrs (crates/rrtl-sim-ir/src/lib.rs:3140-3178).
std::vector<MPacket> schedule_machine_instrs(std::vector<Instr>& instrs) {
  std::unordered_map<uint32_t, size_t> by_value;
  for (size_t i = 0; i < instrs.size(); ++i) by_value[instrs[i].dst] = i;
  std::vector<size_t> level(instrs.size(), 0);
  // Instructions are in post-order, so every dependency precedes its user.
  std::vector<MPacket> packets;
  for (size_t i = 0; i < instrs.size(); ++i) {
    size_t lv = 0;
    bool any = false;
    for (uint32_t d : instr_deps(instrs[i])) {
      auto it = by_value.find(d);
      if (it == by_value.end()) continue;
      lv = std::max(lv, level[it->second] + 1);
      any = true;
    }
    (void)any;
    level[i] = lv;
    if (packets.size() <= lv) packets.resize(lv + 1);
    packets[lv].instrs.push_back(instrs[i]);
  }
  std::vector<MPacket> out;
  for (auto& p : packets)
    if (!p.instrs.empty() || !p.effects.empty()) out.push_back(std::move(p));
  return out;
}

// lower_packets_to_block (crates/rrtl-sim-ir/src/lib.rs:2997-3048).
Block lower_block(const std::vector<std::vector<PackedOp>>& packets) {
  Block b;
  uint32_t next_value = 0;
  for (auto& pkt : packets) {
    PacketLowerer L{next_value, {}, {}, &b.value_width};
    std::vector<Effect> effects;
    for (auto& op : pkt) {
      Effect ef;
      switch (op.kind) {
        case POK::Assign:
          ef.kind = EffK::StoreSignal;
          ef.dst = op.dst;
          ef.value = L.lower(op.expr);
          break;
        case POK::CaptureReg:
          ef.kind = EffK::CaptureReg;
          ef.dst = op.dst;
          ef.value = L.lower(op.expr);
          ef.has_reset = op.has_reset;
          ef.reset = op.reset;
          break;
        case POK::MemoryWrite:
          ef.kind = EffK::MemoryWrite;
          ef.dst = op.dst;
          ef.enable = L.lower(op.expr);
          ef.addr = L.lower(op.addr);
          ef.value = L.lower(op.data);
          break;
      }
      effects.push_back(std::move(ef));
    }
    next_value = L.next_value;
    std::vector<MPacket> lowered = schedule_machine_instrs(L.instrs);
    if (lowered.empty()) lowered.emplace_back();
    for (auto& e : effects) lowered.back().effects.push_back(std::move(e));
    for (auto& p : lowered) b.packets.push_back(std::move(p));
  }
  b.num_values = next_value;
  b.value_width.resize(next_value, 0);
  return b;
}

}  // namespace

MachineProgram lower_to_machine_program(const PackedProgram& p) {
  MachineProgram m;
  m.source = p;
  m.async_reset_comb = lower_block(p.async_reset_comb);
  m.comb = lower_block(p.comb);
  m.tick_next = lower_block(p.tick_next);
  m.tick_commit = lower_block(p.tick_commit);
  return m;
}

}  // namespace rrtl
