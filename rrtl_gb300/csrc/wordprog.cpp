// Word-program lowering (see wordprog.h).
#include "wordprog.h"

#include <algorithm>
#include <map>
#include <unordered_map>
#include <unordered_set>

namespace rrtl {

namespace {

// One scheduled item: a value definition (instr) or an effect.
struct Item {
  const Instr* instr = nullptr;
  const Effect* effect = nullptr;
};

struct Emitter {
  const MachineProgram& mp;
  WordProgram& wp;
  std::map<unsigned long long, uint32_t> lit_index;
  uint32_t cap_words = 0;

  // per block
  std::unordered_map<uint32_t, uint32_t> slot_of;  // value -> slot
  std::unordered_map<uint32_t, size_t> last_use;   // value -> item index of last use
  std::vector<uint32_t> free_slots;
  uint32_t next_slot = 0;
  uint32_t temp_base = 0x80000000u;  // synthetic value ids for concat temporaries

  Emitter(const MachineProgram& m, WordProgram& w) : mp(m), wp(w) {}

  uint32_t lit(unsigned long long v) {
    auto it = lit_index.find(v);
    if (it != lit_index.end()) return it->second;
    uint32_t i = (uint32_t)wp.lits.size();
    wp.lits.push_back(v);
    lit_index[v] = i;
    return i;
  }

  static unsigned long long limbs_to_u64(const std::vector<uint32_t>& l) {
    unsigned long long v = 0;
    if (l.size() > 0) v |= l[0];
    if (l.size() > 1) v |= (unsigned long long)l[1] << 32;
    return v;
  }

  uint32_t alloc() {
    if (!free_slots.empty()) {
      uint32_t s = free_slots.back();
      free_slots.pop_back();
      return s;
    }
    uint32_t s = next_slot++;
    if (next_slot > 0xFFFF) throw RrtlError("E_WORD_SCOPE", "too many live values");
    return s;
  }
  void release_if_last(uint32_t v, size_t at) {
    auto it = last_use.find(v);
    if (it != last_use.end() && it->second == at) {
      free_slots.push_back(slot_of.at(v));
      last_use.erase(it);
    }
  }

  void check_width(uint32_t w) {
    if (w > 64) throw RrtlError("E_WORD_SCOPE", "values wider than 64 bits are outside the word engine");
  }

  // Emit a block's items (already ordered) with slot allocation.
  void emit_items(const std::vector<Item>& items, const Block& blk) {
    slot_of.clear();
    last_use.clear();
    free_slots.clear();
    next_slot = 0;
    // last uses
    for (size_t i = 0; i < items.size(); ++i) {
      if (items[i].instr) {
        for (uint32_t v : instr_deps(*items[i].instr)) last_use[v] = i;
        last_use.emplace(items[i].instr->dst, i);  // a value nobody reads dies where it is defined
      } else {
        const Effect& e = *items[i].effect;
        if (e.kind == EffK::MemoryWrite) {
          last_use[e.enable] = i;
          last_use[e.addr] = i;
        }
        last_use[e.value] = i;
      }
    }
    for (size_t i = 0; i < items.size(); ++i) {
      if (items[i].instr) emit_instr(*items[i].instr, blk, i);
      else emit_effect(*items[i].effect, i);
    }
    wp.n_vslots = std::max(wp.n_vslots, next_slot);
  }

  WInstr base(uint8_t op, uint32_t width) {
    WInstr w{};
    w.op = op;
    w.width = (uint16_t)width;
    return w;
  }

  void emit_instr(const Instr& in, const Block& blk, size_t at) {
    check_width(in.ty.width);
    auto S = [&](uint32_t v) { return (uint16_t)slot_of.at(v); };
    WInstr w = base(0, in.ty.width);
    std::vector<uint16_t> ops;
    for (uint32_t v : instr_deps(in)) ops.push_back(S(v));
    auto finish = [&](WInstr x) {
      for (uint32_t v : instr_deps(in)) release_if_last(v, at);
      x.dst = (uint16_t)alloc();
      slot_of[in.dst] = x.dst;
      wp.code.push_back(x);
      release_if_last(in.dst, at);
    };
    switch (in.kind) {
      case IK::Lit: w.op = W_LIT; w.aux = lit(limbs_to_u64(in.lit)); break;
      case IK::Signal: {
        const ValueLayout& L = mp.source.signals[in.index].layout;
        check_width(L.width);
        w.op = W_SIG;
        w.aux = L.offset;
        w.flags = L.limbs == 2 ? 1 : 0;
        w.width = (uint16_t)std::min(in.ty.width, L.width);
        break;
      }
      case IK::Not: w.op = W_NOT; w.a = ops[0]; break;
      case IK::And: w.op = W_AND; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Or: w.op = W_OR; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Xor: w.op = W_XOR; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Add: w.op = W_ADD; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Sub: w.op = W_SUB; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Mul: w.op = W_MUL; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Eq: w.op = W_EQ; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Ne: w.op = W_NE; w.a = ops[0]; w.b = ops[1]; break;
      case IK::Lt:
        w.op = in.is_signed ? W_LTS : W_LT;
        w.a = ops[0];
        w.b = ops[1];
        w.aux = blk.value_width[in.ops[0]];
        check_width(w.aux);
        break;
      case IK::Mux: w.op = W_MUX; w.a = ops[0]; w.b = ops[1]; w.c = ops[2]; break;
      case IK::Slice: w.op = W_SLICE; w.a = ops[0]; w.aux = in.lsb; check_width(blk.value_width[in.ops[0]]); break;
      case IK::Zext: case IK::Trunc: case IK::Cast: w.op = W_MASK; w.a = ops[0]; break;
      case IK::Sext: w.op = W_SEXT; w.a = ops[0]; w.aux = blk.value_width[in.ops[0]]; break;
      case IK::MemRead: w.op = W_MEMRD; w.a = ops[0]; w.aux = in.index; break;
      case IK::Concat: {
        // t0 = p0; t_i = (t_{i-1} << w_i) | p_i
        uint32_t acc_w = blk.value_width[in.ops[0]];
        check_width(acc_w);
        WInstr m = base(W_MASK, std::min<uint32_t>(acc_w, in.ty.width));
        m.a = ops[0];
        if (in.ops.size() == 1) {
          finish(m);
          return;
        }
        // the accumulator gets its own slot, kept until the last part is merged
        uint32_t acc_slot = alloc();
        m.dst = (uint16_t)acc_slot;
        wp.code.push_back(m);
        for (size_t k = 1; k < in.ops.size(); ++k) {
          uint32_t pw = blk.value_width[in.ops[k]];
          acc_w += pw;
          WInstr c = base(W_CAT, std::min<uint32_t>(acc_w, in.ty.width));
          c.a = (uint16_t)acc_slot;
          c.b = ops[k];
          c.aux = pw;
          c.dst = (uint16_t)acc_slot;
          if (k + 1 == in.ops.size()) {
            c.width = (uint16_t)in.ty.width;
            for (uint32_t v : instr_deps(in)) release_if_last(v, at);
            slot_of[in.dst] = acc_slot;
            wp.code.push_back(c);
            release_if_last(in.dst, at);
            return;
          }
          wp.code.push_back(c);
        }
        return;
      }
    }
    finish(w);
  }

  void emit_effect(const Effect& e, size_t at) {
    const PackedProgram& P = mp.source;
    auto S = [&](uint32_t v) { return (uint16_t)slot_of.at(v); };
    if (e.kind == EffK::StoreSignal) {
      const ValueLayout& L = P.signals[e.dst].layout;
      check_width(L.width);
      WInstr w = base(W_STORE, L.width);
      w.a = S(e.value);
      w.aux = L.offset;
      w.flags = L.limbs == 2 ? 1 : 0;
      wp.code.push_back(w);
      release_if_last(e.value, at);
    } else if (e.kind == EffK::CaptureReg) {
      const ValueLayout& L = P.signals[e.dst].layout;
      check_width(L.width);
      bool async_block = cur_block_async;
      if (async_block) {
        if (e.has_reset && e.reset.async) {
          WInstr w = base(W_ASTORE, L.width);
          w.a = S(e.value);
          w.aux = L.offset;
          w.aux2 = P.signals[e.reset.signal].layout.offset;
          w.flags = (uint8_t)((L.limbs == 2 ? 1 : 0) | 2 | (e.reset.active_low ? 4 : 0));
          wp.code.push_back(w);
        }
      } else {
        WInstr w = base(W_CAPTURE, L.width);
        w.a = S(e.value);
        w.aux = cap_words;
        w.flags = (uint8_t)(L.limbs == 2 ? 1 : 0);
        if (e.has_reset) {
          w.flags |= 2;
          if (e.reset.active_low) w.flags |= 4;
          w.aux2 = P.signals[e.reset.signal].layout.offset;
          std::vector<uint32_t> rv = e.reset.value;
          rv.resize(L.limbs, 0);
          rv.back() &= final_limb_mask(L.width);
          w.aux3 = lit(limbs_to_u64(rv));
        }
        wp.code.push_back(w);
        wp.commits.push_back(WCommitDev{cap_words, L.offset, L.limbs, 0});
        cap_words += L.limbs;
      }
      release_if_last(e.value, at);
    } else {
      const PackedMemory& M = P.memories[e.dst];
      WInstr w = base(W_MEMWR, M.data_layout.width);
      w.a = S(e.enable);
      w.b = S(e.addr);
      w.c = S(e.value);
      w.aux = e.dst;
      wp.code.push_back(w);
      release_if_last(e.enable, at);
      release_if_last(e.addr, at);
      release_if_last(e.value, at);
    }
  }

  bool cur_block_async = false;

  // Reference order: every instruction of each machine packet, then its effects.
  std::vector<Item> reference_order(const Block& b) {
    std::vector<Item> items;
    for (auto& p : b.packets) {
      for (auto& in : p.instrs) items.push_back(Item{&in, nullptr});
      for (auto& e : p.effects) items.push_back(Item{nullptr, &e});
    }
    return items;
  }

  // Comb order: per level, depth-first per store when the level never reads its own stores.
  std::vector<Item> comb_order(const Block& b) {
    std::vector<Item> items;
    size_t p = 0;
    while (p < b.packets.size()) {
      size_t q = p;
      while (q < b.packets.size() && b.packets[q].effects.empty()) ++q;
      if (q == b.packets.size()) q = b.packets.size() - 1;
      // level = packets [p, q]
      std::unordered_map<uint32_t, const Instr*> def;
      std::unordered_set<uint32_t> stored;
      for (size_t k = p; k <= q; ++k) {
        for (auto& in : b.packets[k].instrs) def[in.dst] = &in;
        for (auto& e : b.packets[k].effects)
          if (e.kind == EffK::StoreSignal) stored.insert(e.dst);
      }
      bool self_read = false;
      for (auto& kv : def)
        if (kv.second->kind == IK::Signal && stored.count(kv.second->index)) self_read = true;
      if (self_read) {
        for (size_t k = p; k <= q; ++k) {
          for (auto& in : b.packets[k].instrs) items.push_back(Item{&in, nullptr});
          for (auto& e : b.packets[k].effects) items.push_back(Item{nullptr, &e});
        }
      } else {
        std::unordered_set<uint32_t> done;
        std::vector<std::pair<uint32_t, int>> stack;
        for (size_t k = p; k <= q; ++k)
          for (auto& e : b.packets[k].effects) {
            // post-order DFS of e.value
            stack.push_back({e.value, 0});
            while (!stack.empty()) {
              auto& top = stack.back();
              if (done.count(top.first)) {
                stack.pop_back();
                continue;
              }
              const Instr* in = def.at(top.first);
              const auto& deps = instr_deps(*in);
              if (top.second < (int)deps.size()) {
                uint32_t d = deps[top.second++];
                if (!done.count(d)) stack.push_back({d, 0});
              } else {
                done.insert(top.first);
                items.push_back(Item{in, nullptr});
                stack.pop_back();
              }
            }
            items.push_back(Item{nullptr, &e});
          }
        // instructions no store reaches (none in lowered programs) still run, for exactness
        for (size_t k = p; k <= q; ++k)
          for (auto& in : b.packets[k].instrs)
            if (!done.count(in.dst)) items.insert(items.end() - 0, Item{&in, nullptr});
      }
      p = q + 1;
    }
    return items;
  }
};

}  // namespace

WordProgram build_word_program(const MachineProgram& mp) {
  WordProgram wp;
  const PackedProgram& P = mp.source;
  for (auto& s : P.signals)
    if (s.layout.width > 64) throw RrtlError("E_WORD_SCOPE", "signal `" + s.name + "` is wider than 64 bits");
  for (auto& m : P.memories) {
    if (m.data_layout.width > 64) throw RrtlError("E_WORD_SCOPE", "memory `" + m.name + "` is wider than 64 bits");
    if (m.depth > 0xFFFFFFFFull || m.offset + m.depth * m.data_layout.limbs > 0xFFFFFFFFull)
      throw RrtlError("E_WORD_SCOPE", "memory `" + m.name + "` is too deep");
    wp.mems.push_back(WMemDev{(uint32_t)m.offset, (uint32_t)m.depth, m.data_layout.limbs, m.data_layout.width});
  }
  if (P.total_signal_words > 0xFFFFFFFFull) throw RrtlError("E_WORD_SCOPE", "too many signal words");
  for (const Block* b : {&mp.async_reset_comb, &mp.comb, &mp.tick_next, &mp.tick_commit})
    for (auto& p : b->packets) wp.source_instrs += p.instrs.size();

  Emitter E(mp, wp);
  wp.comb_b = (uint32_t)wp.code.size();
  if (!mp.comb.packets.empty()) E.emit_items(E.comb_order(mp.comb), mp.comb);
  wp.comb_e = (uint32_t)wp.code.size();
  wp.async_b = wp.comb_e;
  E.cur_block_async = true;
  E.emit_items(E.reference_order(mp.async_reset_comb), mp.async_reset_comb);
  E.cur_block_async = false;
  wp.async_e = (uint32_t)wp.code.size();
  wp.next_b = wp.async_e;
  E.emit_items(E.reference_order(mp.tick_next), mp.tick_next);
  wp.next_e = (uint32_t)wp.code.size();
  wp.commit_b = wp.next_e;
  E.emit_items(E.reference_order(mp.tick_commit), mp.tick_commit);
  wp.commit_e = (uint32_t)wp.code.size();
  wp.total_capture_words = E.cap_words;
  wp.n_sig_words = (uint32_t)P.total_signal_words;
  if (wp.lits.empty()) wp.lits.push_back(0);
  return wp;
}

}  // namespace rrtl
