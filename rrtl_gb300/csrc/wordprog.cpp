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
  const Block* blk_ = nullptr;
  std::unordered_map<uint32_t, uint32_t> slot_of;  // value -> slot (the first of a pair)
  std::unordered_map<uint32_t, size_t> last_use;   // value -> item index of last use
  std::unordered_set<uint32_t> pair_val;           // values held in a slot pair (wider than 64 bits)
  std::vector<uint32_t> free_slots, free_pairs;
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

  static unsigned long long limbs_to_u64(const std::vector<uint32_t>& l, size_t first = 0) {
    unsigned long long v = 0;
    if (l.size() > first) v |= l[first];
    if (l.size() > first + 1) v |= (unsigned long long)l[first + 1] << 32;
    return v;
  }
  // two consecutive literal entries (bits 0-63, 64-127) of a wide value
  uint32_t lit_pair(const std::vector<uint32_t>& l) {
    uint32_t i = (uint32_t)wp.lits.size();
    wp.lits.push_back(limbs_to_u64(l, 0));
    wp.lits.push_back(limbs_to_u64(l, 2));
    return i;
  }

  uint32_t alloc(bool pair = false) {
    std::vector<uint32_t>& fl = pair ? free_pairs : free_slots;
    if (!fl.empty()) {
      uint32_t s = fl.back();
      fl.pop_back();
      return s;
    }
    uint32_t s = next_slot;
    next_slot += pair ? 2 : 1;
    if (next_slot > 0xFFFF) throw RrtlError("E_WORD_SCOPE", "too many live values");
    return s;
  }
  void release_if_last(uint32_t v, size_t at) {
    auto it = last_use.find(v);
    if (it != last_use.end() && it->second == at) {
      (pair_val.count(v) ? free_pairs : free_slots).push_back(slot_of.at(v));
      last_use.erase(it);
    }
  }
  // Slot of value v as an operand; sets `pair_flag` in *flags when v is a pair.
  uint16_t opnd(uint32_t v, uint8_t pair_flag, uint8_t* flags) {
    if (pair_val.count(v)) *flags |= pair_flag;
    return (uint16_t)slot_of.at(v);
  }
  uint32_t vwidth(uint32_t v) const { return blk_->value_width[v]; }

  void check_width(uint32_t w) {
    if (w > 128) throw RrtlError("E_WORD_SCOPE", "values wider than 128 bits are outside the word engine");
  }

  // Emit a block's items (already ordered) with slot allocation.
  void emit_items(const std::vector<Item>& items, const Block& blk) {
    blk_ = &blk;
    slot_of.clear();
    last_use.clear();
    pair_val.clear();
    free_slots.clear();
    free_pairs.clear();
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
    WInstr w = base(0, in.ty.width);
    // a value wider than 64 bits, or any operand that is, makes the instruction wide
    bool wide = in.ty.width > 64;
    for (uint32_t v : instr_deps(in)) wide = wide || blk.value_width[v] > 64;
    std::vector<uint16_t> ops;
    const uint8_t pair_bits[3] = {kWPairA, kWPairB, kWPairC};
    size_t k = 0;
    for (uint32_t v : instr_deps(in)) {
      ops.push_back(opnd(v, k < 3 ? pair_bits[k] : 0, &w.flags));
      ++k;
    }
    auto finish = [&](WInstr x) {
      for (uint32_t v : instr_deps(in)) release_if_last(v, at);
      const bool pair = in.ty.width > 64;
      if (wide) x.flags |= kWWide;
      if (pair) {
        x.flags |= kWPairD;
        pair_val.insert(in.dst);
      }
      x.dst = (uint16_t)alloc(pair);
      slot_of[in.dst] = x.dst;
      wp.code.push_back(x);
      release_if_last(in.dst, at);
    };
    switch (in.kind) {
      case IK::Lit:
        w.op = W_LIT;
        w.aux = wide ? lit_pair(in.lit) : lit(limbs_to_u64(in.lit));
        break;
      case IK::Signal: {
        const ValueLayout& L = mp.source.signals[in.index].layout;
        check_width(L.width);
        w.op = W_SIG;
        w.aux = L.offset;
        w.width = (uint16_t)std::min(in.ty.width, L.width);
        if (wide || L.width > 64) {
          wide = true;
          w.c = (uint16_t)L.limbs;
        } else {
          w.flags = L.limbs == 2 ? 1 : 0;
        }
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
      case IK::MemRead: {
        w.op = W_MEMRD;
        w.a = ops[0];
        w.aux = in.index;
        wide = wide || mp.source.memories[in.index].data_layout.width > 64;
        break;
      }
      case IK::Concat: {
        // t0 = p0; t_i = (t_{i-1} << w_i) | p_i, in one accumulator (a pair
        // when the result is wider than 64 bits)
        const bool pair = in.ty.width > 64;
        uint32_t acc_w = blk.value_width[in.ops[0]];
        check_width(acc_w);
        WInstr m = base(W_MASK, std::min<uint32_t>(acc_w, in.ty.width));
        m.flags = w.flags & kWPairA;
        m.a = ops[0];
        if (in.ops.size() == 1) {
          finish(m);
          return;
        }
        // the accumulator gets its own slot, kept until the last part is merged
        const uint32_t acc_slot = alloc(pair);
        m.dst = (uint16_t)acc_slot;
        if (wide) m.flags |= kWWide | (pair ? kWPairD : 0);
        wp.code.push_back(m);
        for (size_t k2 = 1; k2 < in.ops.size(); ++k2) {
          uint32_t pw = blk.value_width[in.ops[k2]];
          acc_w += pw;
          WInstr c = base(W_CAT, std::min<uint32_t>(acc_w, in.ty.width));
          c.a = (uint16_t)acc_slot;
          c.b = ops[k2];
          c.aux = pw;
          c.dst = (uint16_t)acc_slot;
          if (wide) {
            c.flags = kWWide | (pair ? kWPairA | kWPairD : 0);
            if (pair_val.count(in.ops[k2])) c.flags |= kWPairB;
          }
          if (k2 + 1 == in.ops.size()) {
            c.width = (uint16_t)in.ty.width;
            for (uint32_t v : instr_deps(in)) release_if_last(v, at);
            slot_of[in.dst] = acc_slot;
            if (pair) pair_val.insert(in.dst);
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
    if (e.kind == EffK::StoreSignal) {
      const ValueLayout& L = P.signals[e.dst].layout;
      check_width(L.width);
      WInstr w = base(W_STORE, L.width);
      w.a = opnd(e.value, kWPairA, &w.flags);
      w.aux = L.offset;
      if (L.width > 64 || vwidth(e.value) > 64) {
        w.flags |= kWWide;
        w.c = (uint16_t)L.limbs;
      } else {
        w.flags = L.limbs == 2 ? 1 : 0;
      }
      wp.code.push_back(w);
      release_if_last(e.value, at);
    } else if (e.kind == EffK::CaptureReg) {
      const ValueLayout& L = P.signals[e.dst].layout;
      check_width(L.width);
      const bool wide = L.width > 64 || vwidth(e.value) > 64;
      bool async_block = cur_block_async;
      if (async_block) {
        if (e.has_reset && e.reset.async) {
          WInstr w = base(W_ASTORE, L.width);
          w.a = opnd(e.value, kWPairA, &w.flags);
          w.aux = L.offset;
          w.aux2 = P.signals[e.reset.signal].layout.offset;
          w.flags |= (uint8_t)(2 | (e.reset.active_low ? 4 : 0));
          if (wide) {
            w.flags |= kWWide;
            w.c = (uint16_t)L.limbs;
          } else if (L.limbs == 2) {
            w.flags |= 1;
          }
          wp.code.push_back(w);
        }
      } else {
        WInstr w = base(W_CAPTURE, L.width);
        w.a = opnd(e.value, kWPairA, &w.flags);
        w.aux = cap_words;
        if (wide) {
          w.flags |= kWWide;
          w.c = (uint16_t)L.limbs;
        } else if (L.limbs == 2) {
          w.flags |= 1;
        }
        if (e.has_reset) {
          w.flags |= 2;
          if (e.reset.active_low) w.flags |= 4;
          w.aux2 = P.signals[e.reset.signal].layout.offset;
          std::vector<uint32_t> rv = e.reset.value;
          rv.resize(L.limbs, 0);
          rv.back() &= final_limb_mask(L.width);
          w.aux3 = wide ? lit_pair(rv) : lit(limbs_to_u64(rv));
        }
        wp.code.push_back(w);
        wp.commits.push_back(WCommitDev{cap_words, L.offset, L.limbs, 0});
        cap_words += L.limbs;
      }
      release_if_last(e.value, at);
    } else {
      const PackedMemory& M = P.memories[e.dst];
      WInstr w = base(W_MEMWR, M.data_layout.width);
      w.a = opnd(e.enable, kWPairA, &w.flags);
      w.b = opnd(e.addr, kWPairB, &w.flags);
      w.c = opnd(e.value, kWPairC, &w.flags);
      w.aux = e.dst;
      if (M.data_layout.width > 64 || w.flags) w.flags |= kWWide;
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
    if (s.layout.width > 128) throw RrtlError("E_WORD_SCOPE", "signal `" + s.name + "` is wider than 128 bits");
  for (auto& m : P.memories) {
    if (m.data_layout.width > 128) throw RrtlError("E_WORD_SCOPE", "memory `" + m.name + "` is wider than 128 bits");
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
