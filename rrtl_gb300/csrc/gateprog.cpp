// Gate-program lowering (see gateprog.h).
#include "gateprog.h"

#include <algorithm>
#include <array>
#include <map>
#include <tuple>
#include <unordered_map>

namespace rrtl {

// Truth table of a LUT3 with its inputs permuted: input k of the new cell is
// input p[k] of the old one (table bit index = a<<2 | b<<1 | c).
static uint8_t permute_lut(uint8_t lut, const int p[3]) {
  uint8_t out = 0;
  for (int idx = 0; idx < 8; ++idx) {
    const int nv[3] = {(idx >> 2) & 1, (idx >> 1) & 1, idx & 1};  // values of the new inputs a, b, c
    int ov[3] = {0, 0, 0};
    for (int k = 0; k < 3; ++k) ov[p[k]] = nv[k];
    const int oidx = (ov[0] << 2) | (ov[1] << 1) | ov[2];
    if ((lut >> oidx) & 1) out |= (uint8_t)(1u << idx);
  }
  return out;
}

// Reorder a cell's inputs so its truth table is the smallest over the six
// input orders: every table maps to one of 80 permutation classes, so the
// fused kernel needs one specialised loop per class instead of per table.
void canonicalize_inputs(GateCell& c) {
  static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  uint8_t best = c.lut;
  int bi = 0;
  for (int k = 1; k < 6; ++k) {
    const uint8_t t = permute_lut(c.lut, perms[k]);
    if (t < best) {
      best = t;
      bi = k;
    }
  }
  const uint32_t in[3] = {c.in[0], c.in[1], c.in[2]};
  for (int k = 0; k < 3; ++k) c.in[k] = in[perms[bi][k]];
  c.lut = best;
}

bool lut_is_canonical(uint8_t lut) {
  GateCell c;
  c.lut = lut;
  canonicalize_inputs(c);
  return c.lut == lut;
}


namespace {

const uint8_t kVarMask[3] = {0xF0, 0xCC, 0xAA};

// Evaluate an 8-bit LOP3 table on three 8-bit variable masks.
uint8_t apply_tt(uint8_t tt, uint8_t x, uint8_t y, uint8_t z) {
  uint8_t r = 0;
  for (int p = 0; p < 8; ++p) {
    int idx = (((x >> p) & 1) << 2) | (((y >> p) & 1) << 1) | ((z >> p) & 1);
    if ((tt >> idx) & 1) r |= (uint8_t)(1u << p);
  }
  return r;
}

// A boolean function over at most three leaf nets.
struct Fn {
  uint8_t n = 0;
  uint32_t leaf[3] = {0, 0, 0};
  uint8_t tt = 0;
};

Fn fn_const(bool b) {
  Fn f;
  f.tt = b ? 0xFF : 0x00;
  return f;
}

Fn fn_leaf(uint32_t net) {
  if (net == kNetConst0) return fn_const(false);
  if (net == kNetConst1) return fn_const(true);
  Fn f;
  f.n = 1;
  f.leaf[0] = net;
  f.tt = kVarMask[0];
  return f;
}

// Re-express f over the leaf list `u` (which contains all of f's leaves).
uint8_t remap(const Fn& f, const uint32_t* u, int un) {
  uint8_t m[3] = {0, 0, 0};
  for (int i = 0; i < f.n; ++i)
    for (int j = 0; j < un; ++j)
      if (u[j] == f.leaf[i]) m[i] = kVarMask[j];
  return apply_tt(f.tt, m[0], m[1], m[2]);
}

// Drop leaves the table does not depend on and renumber.
Fn simplify(Fn f) {
  for (int i = 0; i < f.n;) {
    uint8_t v = kVarMask[i];
    // f depends on var i iff cofactors differ
    uint8_t hi = f.tt & v, lo = f.tt & (uint8_t)~v;
    int sh = i == 0 ? 4 : i == 1 ? 2 : 1;
    bool depends = (uint8_t)(hi >> sh) != lo;
    if (depends) {
      ++i;
      continue;
    }
    // remove leaf i: rebuild the table over the remaining leaves
    Fn g;
    g.n = f.n - 1;
    int k = 0;
    for (int j = 0; j < f.n; ++j)
      if (j != i) g.leaf[k++] = f.leaf[j];
    // evaluate f with var i fixed to 0 over the new variable positions
    uint8_t m[3] = {0, 0, 0};
    k = 0;
    for (int j = 0; j < f.n; ++j) m[j] = (j == i) ? 0 : kVarMask[k++];
    g.tt = apply_tt(f.tt, m[0], m[1], m[2]);
    f = g;
  }
  if (f.n == 0) f.tt = (f.tt & 1) ? 0xFF : 0x00;
  return f;
}

bool merge(const Fn* parts, int np, uint32_t* u, int* un) {
  *un = 0;
  for (int p = 0; p < np; ++p)
    for (int i = 0; i < parts[p].n; ++i) {
      bool seen = false;
      for (int j = 0; j < *un; ++j) seen |= u[j] == parts[p].leaf[i];
      if (!seen) {
        if (*un == 3) return false;
        u[(*un)++] = parts[p].leaf[i];
      }
    }
  return true;
}

struct Builder {
  const MachineProgram& mp;
  GateProgram& gp;
  // per-block state
  const Block* blk = nullptr;
  std::unordered_map<uint32_t, const Instr*> instr_of;
  std::unordered_map<uint32_t, Fn> fn_memo;
  std::unordered_map<uint32_t, uint32_t> net_memo;
  std::vector<uint32_t> sig_cur_net;  // current net holding each signal's value
  std::map<std::tuple<uint8_t, uint8_t, uint32_t, uint32_t, uint32_t>, uint32_t> cell_cse;  // internal-cell dedup
  int cur_packet = 0;
  std::vector<int> store_packet;  // comb packet storing each signal, -1 if none

  Builder(const MachineProgram& m, GateProgram& g) : mp(m), gp(g) {}

  uint32_t new_net() {
    gp.net_signal.push_back(-1);
    gp.net_is_source.push_back(0);
    return gp.n_nets++;
  }

  void add_cell(const Fn& f0, uint32_t out) {
    Fn f = simplify(f0);
    GateCell c;
    c.lut = f.tt;
    for (int i = 0; i < 3; ++i) c.in[i] = i < f.n ? f.leaf[i] : kNetConst0;
    canonicalize_inputs(c);
    c.out = out;
    gp.cells.push_back(c);
  }

  uint32_t signal_net_for_read(uint32_t s) {
    if (blk == &mp.comb && store_packet[s] >= 0 && store_packet[s] >= cur_packet)
      throw RrtlError("E_GATE_SCOPE", "signal read before its combinational store (combinational loop)");
    return sig_cur_net[s];
  }

  Fn fn_of(uint32_t v) {
    auto it = fn_memo.find(v);
    if (it != fn_memo.end()) return it->second;
    const Instr& in = *instr_of.at(v);
    Fn r;
    switch (in.kind) {
      case IK::Signal: r = fn_leaf(signal_net_for_read(in.index)); break;
      case IK::Lit: r = fn_const(!in.lit.empty() && (in.lit[0] & 1)); break;
      case IK::Not: r = fn_of(in.ops[0]); r.tt = (uint8_t)~r.tt; break;
      case IK::And: case IK::Or: case IK::Xor: case IK::Mux: {
        int np = in.kind == IK::Mux ? 3 : 2;
        Fn parts[3];
        for (int i = 0; i < np; ++i) parts[i] = simplify(fn_of(in.ops[i]));
        uint32_t u[3];
        int un;
        while (!merge(parts, np, u, &un)) {
          // materialise the operand with the widest support
          int best = -1;
          for (int i = 0; i < np; ++i)
            if (parts[i].n >= 2 && (best < 0 || parts[i].n > parts[best].n)) best = i;
          if (best < 0) throw RrtlError("E_GATE_SCOPE", "internal: cannot cover expression");
          parts[best] = fn_leaf(realize(in.ops[best]));
        }
        uint8_t t[3];
        for (int i = 0; i < np; ++i) t[i] = remap(parts[i], u, un);
        r.n = (uint8_t)un;
        for (int i = 0; i < un; ++i) r.leaf[i] = u[i];
        if (in.kind == IK::And) r.tt = t[0] & t[1];
        else if (in.kind == IK::Or) r.tt = t[0] | t[1];
        else if (in.kind == IK::Xor) r.tt = t[0] ^ t[1];
        else r.tt = (uint8_t)((t[0] & t[1]) | (~t[0] & t[2]));
        r = simplify(r);
        break;
      }
      default:
        throw RrtlError("E_GATE_SCOPE", "op is not a gate-level bitwise op");
    }
    fn_memo[v] = r;
    return r;
  }

  // A net holding value v (creates an internal cell if needed).
  uint32_t realize(uint32_t v) {
    auto it = net_memo.find(v);
    if (it != net_memo.end()) return it->second;
    Fn f = simplify(fn_of(v));
    uint32_t net;
    if (f.n == 0) net = (f.tt & 1) ? kNetConst1 : kNetConst0;
    else if (f.n == 1 && f.tt == kVarMask[0]) net = f.leaf[0];
    else {
      auto key = std::make_tuple(f.tt, f.n, f.leaf[0], f.leaf[1], f.leaf[2]);
      auto c = cell_cse.find(key);
      if (c != cell_cse.end()) {
        net = c->second;
      } else {
        net = new_net();
        add_cell(f, net);
        cell_cse[key] = net;
      }
    }
    net_memo[v] = net;
    fn_memo[v] = fn_leaf(net);
    return net;
  }

  void start_block(const Block& b) {
    blk = &b;
    instr_of.clear();
    fn_memo.clear();
    net_memo.clear();
    for (auto& p : b.packets)
      for (auto& in : p.instrs) instr_of[in.dst] = &in;
  }
};

}  // namespace

// Input symmetries of a truth table: the input orders that map it to itself
// (a cell may read its inputs in any of them without changing its table).
struct LutSymmetry {
  std::vector<std::array<int, 3>> perms;  // automorphisms, identity first
};

const LutSymmetry& lut_symmetry(uint8_t lut) {
  static const std::vector<LutSymmetry> table = [] {
    static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    std::vector<LutSymmetry> t(256);
    for (int l = 0; l < 256; ++l)
      for (int k = 0; k < 6; ++k)
        if (permute_lut((uint8_t)l, perms[k]) == (uint8_t)l) t[l].perms.push_back({perms[k][0], perms[k][1], perms[k][2]});
    return t;
  }();
  return table[lut];
}

// Shared-memory wavefronts of a group's operand reads with the given input
// orders: per position, the largest number of distinct rows that share a
// bank residue (rows read twice are one broadcast).
uint32_t group_wavefronts(const GateProgram& gp, const std::vector<uint32_t>& grp, const bool use[3], uint32_t G,
                          const int* choice, const LutSymmetry& sym) {
  uint32_t total = 0;
  const size_t n = grp.size();
  uint32_t rows[32];
  for (int p = 0; p < 3; ++p) {
    if (!use[p]) continue;
    uint32_t per[32] = {0}, mx = 0;
    for (size_t k = 0; k < n; ++k) {
      const GateCell& c = gp.cells[grp[k]];
      const uint32_t r = (uint32_t)gp.net_slot[c.in[sym.perms[choice ? choice[k] : 0][p]]];
      bool seen = false;
      for (size_t q = 0; q < k && !seen; ++q) seen = rows[q] == r;
      rows[k] = r;
      if (!seen) mx = std::max(mx, ++per[r % G]);
    }
    total += mx;
  }
  return total;
}

// The fewest wavefronts a group reaches over its cells' input orders, and
// the orders that reach it: every combination for small groups of tables
// with two orders, else a local search from the identity.
uint32_t best_orientation(const GateProgram& gp, const std::vector<uint32_t>& grp, const LutSymmetry& sym,
                          const bool use[3], uint32_t G, std::vector<int>* out) {
  std::vector<int> choice(grp.size(), 0);
  uint32_t best = group_wavefronts(gp, grp, use, G, choice.data(), sym);
  if (sym.perms.size() >= 2) {
    if (sym.perms.size() == 2 && grp.size() <= 4) {
      std::vector<int> c(grp.size(), 0), bc = choice;
      for (uint32_t m = 1; m < (1u << grp.size()) && best > 0; ++m) {
        for (size_t k = 0; k < grp.size(); ++k) c[k] = (m >> k) & 1;
        const uint32_t w = group_wavefronts(gp, grp, use, G, c.data(), sym);
        if (w < best) {
          best = w;
          bc = c;
        }
      }
      choice = bc;
    } else {
      for (int pass = 0; pass < 2; ++pass) {
        bool improved = false;
        for (size_t k = 0; k < grp.size(); ++k) {
          const int keep = choice[k];
          for (int q = 0; q < (int)sym.perms.size(); ++q) {
            if (q == keep) continue;
            choice[k] = q;
            const uint32_t w = group_wavefronts(gp, grp, use, G, choice.data(), sym);
            if (w < best) {
              best = w;
              improved = true;
              break;
            }
            choice[k] = keep;
          }
        }
        if (!improved) break;
      }
    }
  }
  if (out) *out = choice;
  return best;
}

// Apply the best input orders to a group's cells.
void orient_group(GateProgram& gp, const std::vector<uint32_t>& grp, const LutSymmetry& sym, const bool use[3],
                  uint32_t G) {
  if (sym.perms.size() < 2) return;
  std::vector<int> choice;
  best_orientation(gp, grp, sym, use, G, &choice);
  for (size_t k = 0; k < grp.size(); ++k) {
    if (!choice[k]) continue;
    GateCell& c = gp.cells[grp[k]];
    const uint32_t in[3] = {c.in[0], c.in[1], c.in[2]};
    for (int p = 0; p < 3; ++p) c.in[p] = in[sym.perms[choice[k]][p]];
  }
}

// Move cells between the groups of one truth-table run to cut bank
// conflicts: random swaps of two cells of two groups, kept when the pair's
// wavefronts (each at its best input orders) do not grow. The greedy
// grouping fills groups from a bounded look-ahead, so later groups take what
// is left; swapping evens them out.
void refine_groups(const GateProgram& gp, std::vector<std::vector<uint32_t>>& groups, const LutSymmetry& sym,
                   const bool use[3], uint32_t G, uint64_t& rng) {
  const size_t ng = groups.size();
  if (ng < 2) return;
  std::vector<uint32_t> cost(ng);
  size_t cells = 0;
  for (size_t g = 0; g < ng; ++g) {
    cost[g] = best_orientation(gp, groups[g], sym, use, G, nullptr);
    cells += groups[g].size();
  }
  uint32_t floor = 0;  // a group reads each used position at least once
  for (int p = 0; p < 3; ++p) floor += use[p] ? 1 : 0;
  auto next = [&]() {
    rng ^= rng << 13;
    rng ^= rng >> 7;
    rng ^= rng << 17;
    return rng;
  };
  const size_t tries = cells * (G <= 4 ? 40 : G <= 8 ? 4 : 0);
  for (size_t t = 0; t < tries; ++t) {
    const size_t a = next() % ng, b = next() % ng;
    if (a == b || (cost[a] <= floor && cost[b] <= floor)) continue;
    const size_t i = next() % groups[a].size(), j = next() % groups[b].size();
    std::swap(groups[a][i], groups[b][j]);
    const uint32_t ca = best_orientation(gp, groups[a], sym, use, G, nullptr);
    const uint32_t cb = best_orientation(gp, groups[b], sym, use, G, nullptr);
    if (ca + cb <= cost[a] + cost[b]) {
      cost[a] = ca;
      cost[b] = cb;
    } else {
      std::swap(groups[a][i], groups[b][j]);
    }
  }
}

// Residue bookkeeping for placing rows: per consumer bucket (level, truth
// table, operand position) the number of operand rows placed at each bank
// residue so far. A net's cost at residue r is the count at r summed over its
// consumers' buckets.
struct ResidueBalance {
  uint32_t G;
  std::vector<uint32_t> cons_off, cons_bucket;  // per net: buckets of its consumer inputs
  std::vector<uint32_t> cnt;                    // bucket * G + residue
  std::vector<uint32_t> placed;                 // rows placed per residue (tie-break: even packing)

  ResidueBalance(const GateProgram& gp, uint32_t g) : G(g), placed(g, 0) {
    std::vector<uint64_t> keys;
    std::vector<std::pair<uint32_t, uint64_t>> uses;  // (net, key)
    for (const GateCell& c : gp.cells) {
      const bool use[3] = {(c.lut & 0x0F) != ((c.lut >> 4) & 0x0F), (c.lut & 0x33) != ((c.lut >> 2) & 0x33),
                           (c.lut & 0x55) != ((c.lut >> 1) & 0x55)};
      for (int p = 0; p < 3; ++p) {
        if (!use[p]) continue;
        const uint64_t key = ((uint64_t)(uint32_t)c.level << 10) | ((uint64_t)c.lut << 2) | (uint64_t)p;
        uses.push_back({c.in[p], key});
        keys.push_back(key);
      }
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    cons_off.assign(gp.n_nets + 1, 0);
    for (auto& u : uses) ++cons_off[u.first + 1];
    for (size_t n = 0; n < gp.n_nets; ++n) cons_off[n + 1] += cons_off[n];
    cons_bucket.resize(uses.size());
    std::vector<uint32_t> fill(cons_off.begin(), cons_off.end() - 1);
    for (auto& u : uses)
      cons_bucket[fill[u.first]++] =
          (uint32_t)(std::lower_bound(keys.begin(), keys.end(), u.second) - keys.begin());
    cnt.assign(keys.size() * G, 0);
  }
  uint64_t cost(uint32_t n, uint32_t r) const {
    uint64_t c = 0;
    for (uint32_t i = cons_off[n]; i < cons_off[n + 1]; ++i) c += cnt[(size_t)cons_bucket[i] * G + r];
    return c;
  }
  void place(uint32_t n, uint32_t r) {
    for (uint32_t i = cons_off[n]; i < cons_off[n + 1]; ++i) ++cnt[(size_t)cons_bucket[i] * G + r];
    ++placed[r];
  }
  // One net, any residue.
  uint32_t pick(uint32_t n) {
    uint32_t best = 0;
    uint64_t bc = ~0ull;
    for (uint32_t r = 0; r < G; ++r) {
      const uint64_t c = cost(n, r) * 65536u + placed[r];
      if (c < bc) {
        bc = c;
        best = r;
      }
    }
    place(n, best);
    return best;
  }
  // The outputs of one group: distinct residues (not 0 when `padded`), the
  // cheapest assignment (every permutation for four cells, greedy beyond).
  std::vector<uint32_t> assign(const std::vector<uint32_t>& outs, bool padded) {
    const size_t k = outs.size();
    std::vector<uint32_t> res(k);
    const uint32_t r0 = padded ? 1u : 0u;
    std::vector<std::vector<uint64_t>> c(k, std::vector<uint64_t>(G));
    for (size_t i = 0; i < k; ++i)
      for (uint32_t r = r0; r < G; ++r) c[i][r] = cost(outs[i], r);
    if (G <= 4) {
      std::vector<uint32_t> perm;
      for (uint32_t r = r0; r < G; ++r) perm.push_back(r);
      uint64_t best = ~0ull;
      do {
        uint64_t t = 0;
        for (size_t i = 0; i < k; ++i) t += c[i][perm[i]];
        if (t < best) {
          best = t;
          std::copy(perm.begin(), perm.begin() + (long)k, res.begin());
        }
      } while (std::next_permutation(perm.begin(), perm.end()));
    } else {
      std::vector<uint8_t> used_r(G, 0), done(k, 0);
      for (size_t step = 0; step < k; ++step) {
        uint64_t best = ~0ull;
        size_t bi = 0;
        uint32_t br = r0;
        for (size_t i = 0; i < k; ++i) {
          if (done[i]) continue;
          for (uint32_t r = r0; r < G; ++r)
            if (!used_r[r] && c[i][r] < best) {
              best = c[i][r];
              bi = i;
              br = r;
            }
        }
        done[bi] = 1;
        used_r[br] = 1;
        res[bi] = br;
      }
    }
    for (size_t i = 0; i < k; ++i) place(outs[i], res[i]);
    return res;
  }
};

GateProgram build_gate_program(const MachineProgram& mp, uint32_t tile_words) {
  const PackedProgram& P = mp.source;
  GateProgram gp;
  if (tile_words != 8 && tile_words != 4 && tile_words != 2 && tile_words != 1)
    throw RrtlError("E_GATE_SCOPE", "tile width must be 1, 2, 4 or 8 words");
  gp.tile_words = tile_words;
  gp.group = 32 / tile_words;
  const uint32_t G = gp.group;
  for (auto& s : P.signals)
    if (s.layout.width != 1) throw RrtlError("E_GATE_SCOPE", "signal `" + s.name + "` is wider than 1 bit");
  if (!P.memories.empty()) throw RrtlError("E_GATE_SCOPE", "memories are outside the gate engine");
  if (!mp.async_reset_comb.packets.empty()) throw RrtlError("E_GATE_SCOPE", "asynchronous resets are outside the gate engine");
  for (const Block* b : {&mp.comb, &mp.tick_next, &mp.tick_commit})
    for (auto& p : b->packets) {
      gp.source_instrs += p.instrs.size();
      for (auto& e : p.effects)
        if (e.kind == EffK::MemoryWrite) throw RrtlError("E_GATE_SCOPE", "memory writes are outside the gate engine");
    }

  uint32_t ns = (uint32_t)P.signals.size();
  gp.n_signals = ns;
  gp.n_nets = 2 + ns;
  gp.net_signal.assign(gp.n_nets, -1);
  gp.net_is_source.assign(gp.n_nets, 0);
  gp.net_is_source[kNetConst0] = gp.net_is_source[kNetConst1] = 1;
  gp.signal_net.resize(ns);
  for (uint32_t s = 0; s < ns; ++s) {
    gp.signal_net[s] = 2 + s;
    gp.net_signal[2 + s] = (int32_t)s;
  }

  Builder B(mp, gp);
  B.store_packet.assign(ns, -1);
  for (size_t p = 0; p < mp.comb.packets.size(); ++p)
    for (auto& e : mp.comb.packets[p].effects)
      if (e.kind == EffK::StoreSignal) {
        if (B.store_packet[e.dst] >= 0) throw RrtlError("E_GATE_SCOPE", "signal assigned more than once");
        B.store_packet[e.dst] = (int)p;
      }
  for (uint32_t s = 0; s < ns; ++s)
    if (B.store_packet[s] < 0) gp.net_is_source[2 + s] = 1;
  B.sig_cur_net.resize(ns);
  for (uint32_t s = 0; s < ns; ++s) B.sig_cur_net[s] = 2 + s;

  // comb block: one cell per stored signal
  B.start_block(mp.comb);
  for (size_t p = 0; p < mp.comb.packets.size(); ++p) {
    B.cur_packet = (int)p;
    for (auto& e : mp.comb.packets[p].effects) {
      if (e.kind != EffK::StoreSignal) continue;
      Fn f = B.fn_of(e.value);
      B.add_cell(f, 2 + e.dst);
    }
  }
  // tick_next block: D nets
  B.start_block(mp.tick_next);
  B.cur_packet = 1 << 30;
  for (auto& p : mp.tick_next.packets)
    for (auto& e : p.effects) {
      if (e.kind != EffK::CaptureReg) continue;
      if (gp.net_is_source[2 + e.dst] == 0)
        throw RrtlError("E_GATE_SCOPE", "captured signal is also combinationally assigned");
      GateReg r;
      r.signal = e.dst;
      r.q_net = 2 + e.dst;
      uint32_t d = B.realize(e.value);
      bool d_is_reg = d >= 2 && d < 2 + ns && P.signals[d - 2].kind == PSK::Reg;
      if (d_is_reg) {  // keep D distinct from every Q so the commit is one pass
        uint32_t nd = B.new_net();
        B.add_cell(fn_leaf(d), nd);
        d = nd;
      }
      r.d_net = d;
      r.has_reset = e.has_reset;
      r.rst_net = e.has_reset ? 2 + e.reset.signal : kNetConst0;
      if (e.has_reset && P.signals[e.reset.signal].kind == PSK::Reg) {  // same one-pass rule for resets
        uint32_t nr = B.new_net();
        B.add_cell(fn_leaf(r.rst_net), nr);
        r.rst_net = nr;
      }
      r.active_low = e.has_reset && e.reset.active_low;
      r.reset_value = e.has_reset && !e.reset.value.empty() && (e.reset.value[0] & 1);
      gp.regs.push_back(r);
    }

  // ---- levelize
  // cells were created in dependency order except for signal reads of later
  // stores (rejected above), so one forward pass suffices; iterate to a fixpoint
  // to be robust to creation order.
  auto levelize = [&]() {
    gp.net_level.assign(gp.n_nets, -1);
    std::vector<int32_t> cell_of_net(gp.n_nets, -1);
    for (size_t i = 0; i < gp.cells.size(); ++i) cell_of_net[gp.cells[i].out] = (int32_t)i;
    bool changed = true;
    for (auto& c : gp.cells) c.level = 0;
    while (changed) {
      changed = false;
      for (auto& c : gp.cells) {
        int32_t lv = 0;
        for (int k = 0; k < 3; ++k) {
          int32_t pc = cell_of_net[c.in[k]];
          if (pc >= 0) lv = std::max(lv, gp.cells[pc].level + 1);
        }
        if (lv != c.level) {
          if (lv > (int32_t)gp.cells.size()) throw RrtlError("E_GATE_SCOPE", "combinational cycle between cells");
          c.level = lv;
          changed = true;
        }
      }
    }
    int32_t max_level = -1;
    for (auto& c : gp.cells) {
      max_level = std::max(max_level, c.level);
      gp.net_level[c.out] = c.level;
    }
    gp.n_levels = (uint32_t)(max_level + 1);
  };
  levelize();
  gp.n_real_cells = (uint32_t)gp.cells.size();

  // ---- liveness: consumer level; D nets, reset nets and output-port nets live to the end
  const int32_t kEnd = (int32_t)gp.n_levels;
  std::vector<int32_t> last_use(gp.n_nets, -1);
  for (auto& c : gp.cells)
    for (int k = 0; k < 3; ++k) last_use[c.in[k]] = std::max(last_use[c.in[k]], c.level);
  for (auto& r : gp.regs) {
    last_use[r.d_net] = kEnd;
    last_use[r.rst_net] = kEnd;
  }
  for (uint32_t s = 0; s < ns; ++s)
    if (P.signals[s].kind == PSK::Output) last_use[2 + s] = kEnd;
  auto end_live = [&](uint32_t n) { return std::max(last_use[n], gp.net_level[n]) >= kEnd; };

  // ---- on-chip slots
  // With W words per slot, slot s occupies banks W*(s%G) .. W*(s%G)+W-1 of the
  // 32 banks (G = 32/W), so the G cells of a group conflict only when two of
  // their operand rows share s%G. Cells are grouped to spread operand rows
  // over the residues and each group's outputs get distinct residues.
  //
  // Registers are rewritten by every commit, so between a register's last
  // read in the settle and the commit its slot can host nets that die before
  // the end of the cycle. End-live nets (D, reset, outputs) never take such a
  // slot, so every register slot is free again when the commit writes it.
  //
  // A group's cells read their operand rows in one access per position, so
  // what decides the conflicts of a truth-table run is how evenly the
  // residues of its operand rows spread: with c cells per residue among n
  // groups, max(c) - n groups must take a residue twice. Each net's residue is
  // chosen where its row is placed (sources up front, cell outputs as their
  // group is placed) to even out the residues seen by the (level, table,
  // position) buckets of its consumers.
  ResidueBalance bal(gp, G);
  gp.net_slot.assign(gp.n_nets, -1);
  std::vector<uint8_t> is_reg_q(gp.n_nets, 0);
  for (auto& r : gp.regs) is_reg_q[r.q_net] = 1;
  uint32_t next_slot = 1;  // slot 0 is the scratch slot for padding cells
  std::vector<std::vector<uint32_t>> q_free_after(gp.n_levels + 1);  // register slots released before level L
  std::vector<uint8_t> slot_is_q;
  std::vector<uint32_t> src_next(G);  // next unused source slot of each residue
  for (uint32_t r = 0; r < G; ++r) src_next[r] = r == 0 ? G : r;
  for (uint32_t n = 0; n < gp.n_nets; ++n)
    if (gp.net_is_source[n]) {
      const uint32_t r = bal.pick(n);
      gp.net_slot[n] = (int32_t)src_next[r];
      src_next[r] += G;
      next_slot = std::max(next_slot, (uint32_t)gp.net_slot[n] + 1);
      if (n != kNetConst0 && n != kNetConst1) gp.source_nets.push_back(n);
    }
  slot_is_q.assign(next_slot, 0);
  std::vector<uint8_t> src_used(next_slot, 0);
  for (uint32_t n = 0; n < gp.n_nets; ++n)
    if (gp.net_is_source[n]) {
      src_used[gp.net_slot[n]] = 1;
      if (is_reg_q[n]) {
        slot_is_q[gp.net_slot[n]] = 1;
        if (last_use[n] < kEnd) q_free_after[std::max<int32_t>(last_use[n], -1) + 1].push_back((uint32_t)gp.net_slot[n]);
      }
    }
  std::vector<std::vector<uint32_t>> dying(gp.n_levels + 1);
  for (uint32_t n = 0; n < gp.n_nets; ++n) {
    if (gp.net_is_source[n] || gp.net_level[n] < 0) continue;
    int32_t lu = std::max(last_use[n], gp.net_level[n]);
    if (lu < kEnd) dying[lu].push_back(n);
  }
  std::vector<std::vector<uint32_t>> free_general(G), free_q(G);
  auto release = [&](uint32_t s) {
    bool q = s < slot_is_q.size() && slot_is_q[s];
    (q ? free_q : free_general)[s % G].push_back(s);
  };
  // source slots skipped by the residue choice are free from the start
  for (uint32_t s2 = next_slot; s2-- > 1;)
    if (!src_used[s2]) free_general[s2 % G].push_back(s2);
  auto take = [&](bool live_to_end, uint32_t res) -> uint32_t {
    if (!live_to_end && !free_q[res].empty()) {
      uint32_t s = free_q[res].back();
      free_q[res].pop_back();
      return s;
    }
    if (!free_general[res].empty()) {
      uint32_t s = free_general[res].back();
      free_general[res].pop_back();
      return s;
    }
    while (next_slot % G != res) {
      const uint32_t skipped = next_slot++;
      free_general[skipped % G].push_back(skipped);
    }
    return next_slot++;
  };

  std::vector<std::vector<uint32_t>> cells_at(gp.n_levels);
  for (uint32_t i = 0; i < gp.cells.size(); ++i) cells_at[gp.cells[i].level].push_back(i);
  std::vector<GateCell> grouped;
  gp.level_group_begin.assign(gp.n_levels + 1, 0);
  const int kLook = 200;
  // per operand position: distinct rows per residue in the group being built
  std::vector<uint32_t> cnt(3 * G);
  std::vector<uint32_t> stamp(3 * (size_t)65536, 0);
  uint32_t group_id = 0;
  uint64_t refine_rng = 0x243F6A8885A308D3ull;  // fixed seed: the lowering is deterministic
  for (uint32_t L = 0; L < gp.n_levels; ++L) {
    for (uint32_t s : q_free_after[L]) release(s);
    if (L > 0)
      for (uint32_t n : dying[L - 1]) release((uint32_t)gp.net_slot[n]);
    gp.level_group_begin[L] = (uint32_t)(grouped.size() / G);
    std::vector<uint32_t>& cs = cells_at[L];
    std::stable_sort(cs.begin(), cs.end(), [&](uint32_t x, uint32_t y) { return gp.cells[x].lut < gp.cells[y].lut; });
    for (size_t i = 0; i < cs.size();) {
      size_t j = i;
      const uint8_t lut = gp.cells[cs[i]].lut;
      while (j < cs.size() && gp.cells[cs[j]].lut == lut) ++j;
      const bool use[3] = {(lut & 0x0F) != ((lut >> 4) & 0x0F), (lut & 0x33) != ((lut >> 2) & 0x33),
                           (lut & 0x55) != ((lut >> 1) & 0x55)};
      std::vector<uint32_t> rem(cs.begin() + i, cs.begin() + j);
      std::vector<std::vector<uint32_t>> run_groups;
      size_t head = 0;
      std::vector<uint8_t> taken(rem.size(), 0);
      auto slot_in = [&](uint32_t cell, int p) { return (uint32_t)gp.net_slot[gp.cells[cell].in[p]]; };
      while (head < rem.size()) {
        while (head < rem.size() && taken[head]) ++head;
        if (head == rem.size()) break;
        ++group_id;
        std::fill(cnt.begin(), cnt.end(), 0u);
        auto add = [&](uint32_t cell) {
          for (int p = 0; p < 3; ++p) {
            if (!use[p]) continue;
            uint32_t sl = slot_in(cell, p);
            uint32_t& st = stamp[(size_t)p * 65536 + (sl & 0xFFFF)];
            if (st == group_id) continue;  // row already read by this group: broadcast
            st = group_id;
            cnt[p * G + sl % G]++;
          }
        };
        std::vector<uint32_t> grp{rem[head]};
        taken[head] = 1;
        add(rem[head]);
        // greedy: add the candidate that adds the fewest operand-row conflicts
        for (uint32_t pick = 1; pick < G; ++pick) {
          int best = -1;
          uint32_t best_cost = ~0u;
          int seen = 0;
          for (size_t k = head + 1; k < rem.size() && seen < kLook; ++k) {
            if (taken[k]) continue;
            ++seen;
            uint32_t cost = 0;
            for (int p = 0; p < 3; ++p) {
              if (!use[p]) continue;
              uint32_t sl = slot_in(rem[k], p);
              if (stamp[(size_t)p * 65536 + (sl & 0xFFFF)] == group_id) continue;
              cost += cnt[p * G + sl % G];
            }
            if (cost < best_cost) {
              best_cost = cost;
              best = (int)k;
              if (cost == 0) break;
            }
          }
          if (best < 0) break;
          grp.push_back(rem[best]);
          taken[best] = 1;
          add(rem[best]);
        }
        run_groups.push_back(std::move(grp));
      }
      const LutSymmetry& sym = lut_symmetry(lut);
      refine_groups(gp, run_groups, sym, use, G, refine_rng);
      for (std::vector<uint32_t>& grp : run_groups) {
        orient_group(gp, grp, sym, use, G);
        // outputs: distinct residues, residue 0 left to the padding (scratch
        // slot 0) when the group is short, assigned to even out the consumers
        const bool padded = grp.size() < G;
        std::vector<uint32_t> outs(grp.size());
        for (size_t k = 0; k < grp.size(); ++k) outs[k] = gp.cells[grp[k]].out;
        const std::vector<uint32_t> res_of = bal.assign(outs, padded);
        for (size_t k = 0; k < grp.size(); ++k) {
          GateCell c = gp.cells[grp[k]];
          gp.net_slot[c.out] = (int32_t)take(end_live(c.out), res_of[k]);
          if (slot_is_q.size() <= (size_t)gp.net_slot[c.out]) slot_is_q.resize(gp.net_slot[c.out] + 1, 0);
          grouped.push_back(c);
        }
        while (grouped.size() % G) {
          GateCell pad;
          pad.lut = lut;
          pad.level = (int32_t)L;
          pad.pad = true;
          pad.out = kNetConst0;  // redirected to the scratch slot / row
          grouped.push_back(pad);
        }
      }
      i = j;
    }
  }
  gp.level_group_begin[gp.n_levels] = (uint32_t)(grouped.size() / G);
  gp.cells = std::move(grouped);
  for (uint32_t n = 0; n < gp.n_nets; ++n) gp.net_end_live.push_back(end_live(n) ? 1 : 0);
  for (uint32_t n = 0; n < gp.n_nets; ++n)
    if (gp.net_is_source[n] && !is_reg_q[n]) gp.net_end_live[n] = 1;
  gp.n_slots = next_slot;
  return gp;
}

void build_pieces(GateProgram& gp, uint32_t piece_groups) {
  gp.piece_groups = piece_groups;
  gp.pieces.clear();
  gp.segments.clear();
  for (uint32_t L = 0; L < gp.n_levels; ++L) {
    uint32_t g0 = gp.level_group_begin[L], g1 = gp.level_group_begin[L + 1];
    uint32_t n = g1 - g0;
    if (n == 0) continue;
    uint32_t np = (n + piece_groups - 1) / piece_groups;
    for (uint32_t k = 0; k < np; ++k) {
      GatePiece pc;
      pc.level = L;
      pc.group_begin = g0 + (uint32_t)((uint64_t)n * k / np);
      uint32_t end = g0 + (uint32_t)((uint64_t)n * (k + 1) / np);
      pc.n_groups = end - pc.group_begin;
      pc.last_of_level = k + 1 == np;
      pc.seg_begin = (uint32_t)gp.segments.size();
      for (uint32_t g = pc.group_begin; g < end;) {
        uint32_t h = g;
        uint8_t lut = gp.cells[(size_t)g * gp.group].lut;
        while (h < end && gp.cells[(size_t)h * gp.group].lut == lut) ++h;
        gp.segments.push_back(GateSegment{lut, g - pc.group_begin, h - pc.group_begin});
        g = h;
      }
      pc.seg_end = (uint32_t)gp.segments.size();
      gp.pieces.push_back(pc);
    }
  }
}

// Split one piece's truth-table runs over `warps` warps. A warp step covers
// `steps_per` groups of one run, and every run a warp takes costs about
// `run_cost` steps of dispatch. The split fills warps in order, cutting runs
// at multiples of `steps_per` groups, with the smallest per-warp cost cap
// (found by bisection) that lets `warps` warps take every group; warp 0,
// which also keeps the ring full, gets `lead_weight` of the cap.
static std::vector<std::vector<uint32_t>> split_piece(const GateProgram& gp, const GatePiece& pc, uint32_t warps,
                                                      double lead_weight, uint32_t steps_per, double run_cost) {
  // greedy fill under cap `cap`; returns warps used (warps + 1 when it does not fit)
  auto fill = [&](double cap, std::vector<std::vector<uint32_t>>* out) -> uint32_t {
    uint32_t k = 0;
    double used = 0;
    for (uint32_t s = pc.seg_begin; s < pc.seg_end; ++s) {
      const GateSegment& sg = gp.segments[s];
      uint32_t b = sg.begin;
      while (b < sg.end) {
        if (k >= warps) return warps + 1;
        const double c = (k == 0 ? lead_weight : 1.0) * cap;
        const double room = c - used - run_cost;
        const uint32_t left = sg.end - b;
        uint32_t take = room >= 1.0 ? (uint32_t)room * steps_per : 0u;
        if (take >= left) take = left;
        if (take > 0) {
          if (out) (*out)[k].push_back(pack_run(sg.lut, b, b + take));
          used += run_cost + (double)((take + steps_per - 1) / steps_per);
          b += take;
        }
        if (b < sg.end) {
          ++k;
          used = 0;
        }
      }
    }
    return k + 1;
  };
  double lo = 0, hi = run_cost;
  for (uint32_t s = pc.seg_begin; s < pc.seg_end; ++s)
    hi += (double)((gp.segments[s].end - gp.segments[s].begin + steps_per - 1) / steps_per) + run_cost;
  hi = hi / std::min(lead_weight, 1.0) + 1.0;
  for (int it = 0; it < 40 && hi - lo > 0.25; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (fill(mid, nullptr) <= warps) hi = mid;
    else lo = mid;
  }
  std::vector<std::vector<uint32_t>> out(warps);
  if (fill(hi, &out) > warps) throw RrtlError("E_INTERNAL", "piece split failed");
  return out;
}

std::vector<uint32_t> commit_order(const GateProgram& gp) {
  const uint32_t G = gp.group;
  const size_t n = gp.regs.size();
  std::vector<uint32_t> out;
  out.reserve(n);
  std::vector<uint8_t> taken(n, 0);
  const size_t kLook = 256;
  size_t head = 0;
  std::vector<uint8_t> used_d(G), used_q(G);
  auto res = [&](uint32_t net) { return (uint32_t)gp.net_slot[net] % G; };
  while (out.size() < n) {
    while (taken[head]) ++head;
    std::fill(used_d.begin(), used_d.end(), 0);
    std::fill(used_q.begin(), used_q.end(), 0);
    auto add = [&](size_t k) {
      taken[k] = 1;
      out.push_back((uint32_t)k);
      used_d[res(gp.regs[k].d_net)] = 1;
      used_q[res(gp.regs[k].q_net)] = 1;
    };
    add(head);
    for (uint32_t pick = 1; pick < G && out.size() < n; ++pick) {
      size_t best = n, seen = 0;
      uint32_t best_cost = ~0u;
      for (size_t k = head + 1; k < n && seen < kLook; ++k) {
        if (taken[k]) continue;
        ++seen;
        const uint32_t cost = used_d[res(gp.regs[k].d_net)] + used_q[res(gp.regs[k].q_net)];
        if (cost < best_cost) {
          best_cost = cost;
          best = k;
          if (cost == 0) break;
        }
      }
      if (best == n) break;
      add(best);
    }
  }
  return out;
}

PieceBlob build_piece_blob(const GateProgram& gp, uint32_t warps, double lead_weight, uint32_t steps_per,
                           double run_cost) {
  PieceBlob pb;
  const uint32_t G = gp.group;
  const int32_t c0 = gp.net_slot[kNetConst0];
  // per piece: the header words (2 per warp + extra runs), built first to size the common header
  std::vector<std::vector<uint32_t>> heads;
  uint32_t max_extra = 0;
  for (const GatePiece& pc : gp.pieces) {
    if (pc.n_groups >= 4096) throw RrtlError("E_GATE_SCOPE", "piece too large for its header");
    std::vector<std::vector<uint32_t>> split = split_piece(gp, pc, warps, lead_weight, steps_per, run_cost);
    std::vector<uint32_t> head(2 * warps, 0), extra;
    for (uint32_t k = 0; k < warps; ++k) {
      const std::vector<uint32_t>& mine = split[k];
      head[2 * k] = mine.empty() ? 0u : mine[0];
      const uint32_t first = (uint32_t)extra.size();
      for (size_t i = 1; i < mine.size(); ++i) extra.push_back(mine[i]);
      head[2 * k + 1] = first | ((uint32_t)extra.size() << 16);
    }
    if (extra.size() >= 65536) throw RrtlError("E_GATE_SCOPE", "piece too large for its header");
    max_extra = std::max(max_extra, (uint32_t)extra.size());
    head.insert(head.end(), extra.begin(), extra.end());
    heads.push_back(std::move(head));
  }
  const uint32_t hdr_words = (2 * warps + max_extra + 3) & ~3u;
  pb.hdr_bytes = hdr_words * 4;
  for (size_t i = 0; i < gp.pieces.size(); ++i) {
    const GatePiece& pc = gp.pieces[i];
    const uint32_t start = (uint32_t)pb.words.size();
    std::vector<uint32_t>& head = heads[i];
    // extra-run indices are relative to the extra list, which starts after the 2*warps words
    pb.words.insert(pb.words.end(), head.begin(), head.end());
    pb.words.resize(start + hdr_words, 0);
    for (uint32_t g = pc.group_begin; g < pc.group_begin + pc.n_groups; ++g)
      for (uint32_t k = 0; k < G; ++k) {
        const GateCell& c = gp.cells[(size_t)g * G + k];
        const uint32_t a = c.pad ? c0 : gp.net_slot[c.in[0]], b = c.pad ? c0 : gp.net_slot[c.in[1]];
        const uint32_t cc = c.pad ? c0 : gp.net_slot[c.in[2]], o = c.pad ? 0 : gp.net_slot[c.out];
        const uint64_t x = pack_smem_record(a, b, cc, o);
        pb.words.push_back((uint32_t)x);
        pb.words.push_back((uint32_t)(x >> 32));
      }
    while (pb.words.size() % 4) pb.words.push_back(0);
    pb.off_words.push_back(start);
    pb.bytes.push_back((uint32_t)(pb.words.size() - start) * 4);
    pb.max_bytes = std::max(pb.max_bytes, pb.bytes.back());
  }
  return pb;
}

}  // namespace rrtl
