// CPU oracle for the batched cycle-simulation path. TEST INFRASTRUCTURE ONLY:
// tests, the smoke check and the CPU-baseline leg of the benchmark call it as
// the checker; the product never links or calls it.
//
// It restates the reference's CPU engines:
//   PackedSim    <- PackedSimulator   crates/rrtl-sim-ir/src/lib.rs:9033-9307, 9573-10252,
//                                      limb helpers :12942-13196
//   BitParallel  <- BitParallelSimulator crates/rrtl-sim-ir/src/bitparallel.rs:32-347
//   ScalarSim    <- rrtl_core::Simulator crates/rrtl-core/src/lib.rs:5820-6470
//   BitSlice     <- BitSliceSimulator crates/rrtl-sim-ir/src/bitslice.rs:26-402
// The packed/machine programs come from the lowering in rrtl_gb300/csrc
// (itself a restatement of lower_to_packed_program / lower_to_machine_program);
// ScalarSim works on the unlowered design, so it checks that lowering.
//
// Parity pins (tests/test_oracle_golden.py): the reference's Counter known
// answer [1,0,2,2] (crates/rrtl-gpu-sim/src/lib.rs:5763-5787), the crc32 gate
// netlist against the CRC-32 algorithm (crates/rrtl-sim-ir/examples/netlist_crc32.rs)
// and the stuck-at fault-sim coverage 64/64 with latency 1/6/2.1
// (crates/rrtl-sim-ir/examples/fault_sim.rs; docs/rrtl-optimizations.md:1411-1416),
// the ATPG answers confirmed concretely (crc_5 stuck-at-0: golden 0x690ce0ee,
// faulty 0x690ce0ce; the reconvergent cone's testable and untestable faults;
// crates/rrtl-sim-ir/examples/symbolic_exec.rs:76-212). BitSlice is pinned by
// the reference's own bit-slice test (tests/test_bitslice.py,
// crates/rrtl-sim-ir/src/bitslice.rs:727-778).
#include <algorithm>
#include <functional>
#include <cstring>
#include <map>
#include <stdexcept>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../include/rrtl_cuda.h"
#include "../rrtl_gb300/csrc/design.h"
#include "../rrtl_gb300/csrc/lower.h"

using namespace rrtl;

namespace {

thread_local std::string g_err;

// ------------------------------------------------ stimulus / hash (restated) --
// Independent restatement of the stimulus convention (counter hash built on the
// SplitMix64 finaliser); tests pin both copies to the same known answers.
uint64_t o_smix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint32_t o_stim_word(uint64_t seed, uint64_t stream, uint64_t cycle, uint64_t idx) {
  uint64_t k = o_smix(seed ^ (stream * 0xD6E8FEB86659FD93ull));
  return (uint32_t)o_smix(k ^ (cycle * 0xA0761D6478BD642Full) ^ (idx * 0xE7037ED1A0B428DBull));
}
uint32_t o_stim_lane_limb(uint64_t seed, uint64_t stream, uint64_t cycle, uint64_t lane, uint32_t width, uint32_t limb) {
  if (width == 1) return (o_stim_word(seed, stream, cycle, lane / 32) >> (uint32_t)(lane % 32)) & 1u;
  uint32_t v = o_stim_word(seed, stream ^ ((uint64_t)limb << 40), cycle, lane);
  uint32_t nl = (width + 31) / 32;
  if (limb + 1 == nl && width % 32) v &= (1u << (width % 32)) - 1u;
  return v;
}
uint64_t o_hash_term(uint64_t cycle, uint32_t rec, uint64_t idx, uint32_t value) {
  uint64_t salt = o_smix((cycle << 20) ^ (uint64_t)rec ^ 0x5851F42D4C957F2Dull);
  return o_smix((uint64_t)value ^ (idx << 32) ^ salt);
}

// ------------------------------------------------------------ limb helpers --
// crates/rrtl-sim-ir/src/lib.rs:12942-13196, one function each.
typedef std::vector<uint32_t> Limbs;

uint32_t nlimbs(uint32_t w) { uint32_t l = (w + 31) / 32; return l ? l : 1; }
uint32_t top_mask(uint32_t w) { uint32_t r = w % 32; return r ? ((1u << r) - 1u) : 0xFFFFFFFFu; }
void mask_to_width(Limbs& v, uint32_t w) {
  v.resize(nlimbs(w), 0);
  v.back() &= top_mask(w);
}
Limbs fit_limbs(Limbs v, BitType ty) { mask_to_width(v, ty.width); return v; }
bool get_bit(const Limbs& v, uint32_t bit) {
  size_t l = bit / 32;
  return l < v.size() && ((v[l] >> (bit % 32)) & 1u);
}
void set_bit(Limbs& v, uint32_t bit) {
  size_t l = bit / 32;
  if (v.size() <= l) v.resize(l + 1, 0);
  v[l] |= 1u << (bit % 32);
}
Limbs bit_not(Limbs v, BitType ty) {
  v.resize(nlimbs(ty.width), 0);
  for (auto& x : v) x = ~x;
  return fit_limbs(v, ty);
}
template <class F>
Limbs bit_binop(Limbs a, Limbs b, BitType ty, F f) {
  uint32_t n = nlimbs(ty.width);
  a.resize(n, 0); b.resize(n, 0);
  Limbs o(n);
  for (uint32_t i = 0; i < n; ++i) o[i] = f(a[i], b[i]);
  mask_to_width(o, ty.width);
  return o;
}
Limbs add_limbs(Limbs a, Limbs b, BitType ty) {
  uint32_t n = nlimbs(ty.width);
  a.resize(n, 0); b.resize(n, 0);
  Limbs o(n);
  uint64_t c = 0;
  for (uint32_t i = 0; i < n; ++i) { uint64_t s = (uint64_t)a[i] + b[i] + c; o[i] = (uint32_t)s; c = s >> 32; }
  mask_to_width(o, ty.width);
  return o;
}
Limbs sub_limbs(Limbs a, Limbs b, BitType ty) {
  uint32_t n = nlimbs(ty.width);
  a.resize(n, 0); b.resize(n, 0);
  Limbs o(n);
  uint64_t br = 0;
  for (uint32_t i = 0; i < n; ++i) {
    uint64_t sub = (uint64_t)b[i] + br, lw = a[i];
    o[i] = (uint32_t)(lw - sub);
    br = lw < sub;
  }
  mask_to_width(o, ty.width);
  return o;
}
Limbs mul_limbs(Limbs a, Limbs b, BitType ty) {
  uint32_t n = nlimbs(ty.width);
  a.resize(n, 0); b.resize(n, 0);
  std::vector<u128> acc(2 * n, 0);
  for (uint32_t i = 0; i < n; ++i)
    for (uint32_t j = 0; j < n; ++j) acc[i + j] += (u128)a[i] * b[j];
  Limbs o(n);
  u128 c = 0;
  for (uint32_t i = 0; i < n; ++i) { u128 w = acc[i] + c; o[i] = (uint32_t)w; c = w >> 32; }
  mask_to_width(o, ty.width);
  return o;
}
bool eq_values(Limbs a, Limbs b, uint32_t w) {
  uint32_t n = nlimbs(w);
  a.resize(n, 0); b.resize(n, 0);
  mask_to_width(a, w); mask_to_width(b, w);
  return a == b;
}
bool lt_values(Limbs a, Limbs b, uint32_t w, bool sgn) {
  uint32_t n = nlimbs(w);
  a.resize(n, 0); b.resize(n, 0);
  mask_to_width(a, w); mask_to_width(b, w);
  if (sgn) {
    bool ls = get_bit(a, w - 1), rs = get_bit(b, w - 1);
    if (ls != rs) return ls;
  }
  for (int i = (int)n - 1; i >= 0; --i)
    if (a[i] != b[i]) return a[i] < b[i];
  return false;
}
Limbs slice_limbs(const Limbs& v, uint32_t lsb, BitType ty) {
  Limbs o(nlimbs(ty.width), 0);
  for (uint32_t bit = 0; bit < ty.width; ++bit)
    if (get_bit(v, lsb + bit)) set_bit(o, bit);
  mask_to_width(o, ty.width);
  return o;
}
Limbs sext_limbs(Limbs v, uint32_t in_w, BitType ty) {
  bool sign = get_bit(v, in_w - 1);
  Limbs o = fit_limbs(v, BitType{in_w, false});
  o.resize(nlimbs(ty.width), sign ? 0xFFFFFFFFu : 0u);
  if (sign)
    for (uint32_t bit = in_w; bit < ty.width; ++bit) set_bit(o, bit);
  mask_to_width(o, ty.width);
  return o;
}
Limbs concat_limbs(const std::vector<std::pair<Limbs, uint32_t>>& parts, BitType ty) {
  Limbs o(nlimbs(ty.width), 0);
  uint32_t off = 0;
  for (auto it = parts.rbegin(); it != parts.rend(); ++it) {
    for (uint32_t bit = 0; bit < it->second; ++bit)
      if (get_bit(it->first, bit)) set_bit(o, off + bit);
    off += it->second;
  }
  mask_to_width(o, ty.width);
  return o;
}
uint64_t decode_usize(const Limbs& v) {
  uint64_t out = 0;
  for (size_t i = 0; i < v.size() && i < 2; ++i) out |= (uint64_t)v[i] << (32 * i);
  for (size_t i = 2; i < v.size(); ++i)
    if (v[i]) return UINT64_MAX;
  return out;
}
bool decode_bool(const Limbs& v) { return !v.empty() && (v[0] & 1u); }

// ------------------------------------------------------------ design holder --
struct OracleDesign {
  Design design;
  std::string top;
  PackedProgram packed;
  MachineProgram machine;
};

// ---------------------------------------------------------------- PackedSim --
struct PackedSim {
  const OracleDesign* d;
  const PackedProgram* P;
  const MachineProgram* M;
  uint32_t lanes;
  std::vector<uint32_t> values;    // [(offset+limb)*lanes + lane]
  std::vector<uint32_t> memories;  // [lane*mem_words + offset + addr*limbs + limb]
  struct Capture { uint32_t signal; std::vector<uint32_t> vals; };
  std::vector<Capture> captures;
  size_t capture_count = 0;
  std::vector<std::vector<uint32_t>> ws;  // block value workspace [value] -> [limb][lane]

  PackedSim(const OracleDesign* od, uint32_t n) : d(od), P(&od->packed), M(&od->machine), lanes(n) {
    values.assign(P->total_signal_words * lanes, 0);
    memories.assign(P->total_memory_words_per_lane * lanes, 0);
    PackedSim::eval_combinational();  // PackedSimulator::new settles once (lib.rs:3058)
  }
  virtual ~PackedSim() = default;

  size_t vidx(uint32_t off, uint32_t limb, uint32_t lane) const { return ((size_t)off + limb) * lanes + lane; }
  size_t midx(const PackedMemory& m, uint32_t lane, uint64_t addr, uint32_t limb) const {
    return (size_t)lane * P->total_memory_words_per_lane + m.offset + addr * m.data_layout.limbs + limb;
  }
  Limbs load_layout(const ValueLayout& L, uint32_t lane) const {
    Limbs o(L.limbs);
    for (uint32_t i = 0; i < L.limbs; ++i) o[i] = values[vidx(L.offset, i, lane)];
    mask_to_width(o, L.width);
    return o;
  }
  void store_layout(const ValueLayout& L, uint32_t lane, const Limbs& v) {
    Limbs s = fit_limbs(v, L.ty);
    for (uint32_t i = 0; i < L.limbs; ++i) values[vidx(L.offset, i, lane)] = s[i];
  }
  Limbs load_memory(const PackedMemory& m, uint32_t lane, uint64_t addr) const {
    Limbs o(m.data_layout.limbs);
    for (uint32_t i = 0; i < m.data_layout.limbs; ++i) o[i] = memories[midx(m, lane, addr, i)];
    mask_to_width(o, m.data_layout.width);
    return o;
  }
  void store_memory(uint32_t mi, uint32_t lane, uint64_t addr, const Limbs& v) {
    const PackedMemory& m = P->memories[mi];
    Limbs s = fit_limbs(v, m.data_layout.ty);
    for (uint32_t i = 0; i < m.data_layout.limbs; ++i) memories[midx(m, lane, addr, i)] = s[i];
  }

  Limbs val(uint32_t v, uint32_t lane, const Block& b) const {
    uint32_t n = nlimbs(b.value_width[v]);
    Limbs o(n);
    for (uint32_t i = 0; i < n; ++i) o[i] = ws[v][(size_t)i * lanes + lane];
    return o;
  }
  void set_val(uint32_t v, uint32_t lane, const Limbs& x, const Block& b) {
    uint32_t n = nlimbs(b.value_width[v]);
    for (uint32_t i = 0; i < n; ++i) ws[v][(size_t)i * lanes + lane] = i < x.size() ? x[i] : 0;
  }

  // eval_machine_instr_lane (crates/rrtl-sim-ir/src/lib.rs:9796-9907).
  Limbs eval_lane(const Instr& in, uint32_t lane, const Block& b) const {
    auto V = [&](uint32_t k) { return val(in.ops[k], lane, b); };
    auto W = [&](uint32_t k) { return b.value_width[in.ops[k]]; };
    Limbs r;
    switch (in.kind) {
      case IK::Lit: r = in.lit; break;
      case IK::Signal: r = load_layout(P->signals[in.index].layout, lane); break;
      case IK::Not: r = bit_not(V(0), in.ty); break;
      case IK::And: r = bit_binop(V(0), V(1), in.ty, [](uint32_t x, uint32_t y) { return x & y; }); break;
      case IK::Or: r = bit_binop(V(0), V(1), in.ty, [](uint32_t x, uint32_t y) { return x | y; }); break;
      case IK::Xor: r = bit_binop(V(0), V(1), in.ty, [](uint32_t x, uint32_t y) { return x ^ y; }); break;
      case IK::Add: r = add_limbs(V(0), V(1), in.ty); break;
      case IK::Sub: r = sub_limbs(V(0), V(1), in.ty); break;
      case IK::Mul: r = mul_limbs(V(0), V(1), in.ty); break;
      case IK::Eq: r = Limbs{(uint32_t)eq_values(V(0), V(1), std::max(W(0), W(1)))}; break;
      case IK::Ne: r = Limbs{(uint32_t)!eq_values(V(0), V(1), std::max(W(0), W(1)))}; break;
      case IK::Lt: r = Limbs{(uint32_t)lt_values(V(0), V(1), W(0), in.is_signed)}; break;
      case IK::Mux: r = decode_bool(V(0)) ? V(1) : V(2); break;
      case IK::Slice: r = slice_limbs(V(0), in.lsb, in.ty); break;
      case IK::Zext: case IK::Trunc: case IK::Cast: r = fit_limbs(V(0), in.ty); break;
      case IK::Sext: r = sext_limbs(V(0), W(0), in.ty); break;
      case IK::Concat: {
        std::vector<std::pair<Limbs, uint32_t>> parts;
        for (uint32_t k = 0; k < in.ops.size(); ++k) parts.emplace_back(V(k), W(k));
        r = concat_limbs(parts, in.ty);
        break;
      }
      case IK::MemRead: {
        uint64_t a = decode_usize(V(0));
        const PackedMemory& m = P->memories[in.index];
        r = a < m.depth ? load_memory(m, lane, a) : Limbs(nlimbs(in.ty.width), 0);
        break;
      }
    }
    return fit_limbs(r, in.ty);
  }

  void prepare(const Block& b) {
    if (ws.size() < b.num_values) ws.resize(b.num_values);
    for (uint32_t v = 0; v < b.num_values; ++v) ws[v].assign((size_t)nlimbs(b.value_width[v]) * lanes, 0);
  }
  void eval_instr(const Instr& in, const Block& b) {
    for (uint32_t lane = 0; lane < lanes; ++lane) set_val(in.dst, lane, eval_lane(in, lane, b), b);
  }
  bool reset_asserted(const PackedReset& r, uint32_t lane) const {
    bool v = decode_bool(load_layout(P->signals[r.signal].layout, lane));
    return r.active_low ? !v : v;
  }

  // execute_machine_block + execute_machine_effect (lib.rs:9700-9777).
  void execute_block(const Block& b) {
    if (b.packets.empty()) return;
    prepare(b);
    for (auto& pkt : b.packets) {
      for (auto& in : pkt.instrs) eval_instr(in, b);
      for (auto& ef : pkt.effects) {
        if (ef.kind == EffK::StoreSignal) {
          const ValueLayout& L = P->signals[ef.dst].layout;
          for (uint32_t lane = 0; lane < lanes; ++lane) store_layout(L, lane, val(ef.value, lane, b));
        } else if (ef.kind == EffK::CaptureReg) {
          if (!ef.has_reset || !ef.reset.async) continue;
          for (uint32_t lane = 0; lane < lanes; ++lane)
            if (reset_asserted(ef.reset, lane)) store_layout(P->signals[ef.dst].layout, lane, val(ef.value, lane, b));
        } else {
          const PackedMemory& m = P->memories[ef.dst];
          for (uint32_t lane = 0; lane < lanes; ++lane) {
            if (!decode_bool(val(ef.enable, lane, b))) continue;
            uint64_t a = decode_usize(val(ef.addr, lane, b));
            if (a < m.depth) store_memory(ef.dst, lane, a, val(ef.value, lane, b));
          }
        }
      }
    }
  }

  virtual void eval_combinational() {  // lib.rs:9278-9281: comb, then async-reset comb
    execute_block(M->comb);
    execute_block(M->async_reset_comb);
  }
  // capture_register_stream / capture_register_value (lib.rs:9614-9686).
  void capture_registers() {
    capture_count = 0;
    const Block& b = M->tick_next;
    if (b.packets.empty()) return;
    prepare(b);
    for (auto& pkt : b.packets) {
      for (auto& in : pkt.instrs) eval_instr(in, b);
      for (auto& ef : pkt.effects) {
        if (ef.kind != EffK::CaptureReg) continue;
        const ValueLayout& L = P->signals[ef.dst].layout;
        if (capture_count == captures.size()) captures.emplace_back();
        Capture& c = captures[capture_count++];
        c.signal = ef.dst;
        c.vals.assign((size_t)L.limbs * lanes, 0);
        for (uint32_t lane = 0; lane < lanes; ++lane) {
          Limbs v = (ef.has_reset && reset_asserted(ef.reset, lane)) ? fit_limbs(ef.reset.value, L.ty) : val(ef.value, lane, b);
          for (uint32_t i = 0; i < L.limbs; ++i) c.vals[(size_t)i * lanes + lane] = i < v.size() ? v[i] : 0;
        }
      }
    }
  }
  void commit_registers() {  // lib.rs:9688-9699
    for (size_t k = 0; k < capture_count; ++k) {
      const Capture& c = captures[k];
      const ValueLayout& L = P->signals[c.signal].layout;
      for (uint32_t i = 0; i < L.limbs; ++i)
        std::copy(c.vals.begin() + (size_t)i * lanes, c.vals.begin() + (size_t)(i + 1) * lanes, values.begin() + vidx(L.offset, i, 0));
    }
  }
  virtual void tick_from_evaluated_no_post_eval() {  // lib.rs:9289-9293
    capture_registers();
    execute_block(M->tick_commit);
    commit_registers();
  }
  void tick() { eval_combinational(); tick_from_evaluated_no_post_eval(); eval_combinational(); }
  void tick_many(uint64_t n) {  // lib.rs:9295-9307 (comb-fused)
    if (!n) return;
    eval_combinational();
    for (uint64_t i = 0; i < n; ++i) { tick_from_evaluated_no_post_eval(); eval_combinational(); }
  }
};

// ---------------------------------------------------------------- SimdSim --
// SimdCpuSimulator restated (crates/rrtl-sim-ir/src/lib.rs:5375-7457, its
// tick_many at :5784): the packed simulator's cycle, evaluated instruction by
// instruction across every lane of the batch (eval_simd_instr_into, :6109),
// with the reference's one- and two-limb fast paths as one u64 per lane: it
// takes designs whose values, signals and memory words are all at most 64
// bits wide. Storage, streams and effects are PackedSim's, so every
// PackedSim entry point (signals, memories, snapshots, the run protocol)
// works on it unchanged. The lane loops are plain arrays the host compiler
// vectorises; a caller runs disjoint lane ranges on several threads (lanes
// never interact), as the reference's parallel engines do.
struct SimdSim : PackedSim {
  std::vector<uint64_t> wv;    // [value][lane] of the current block
  std::vector<uint64_t> caps;  // [capture][lane]
  std::vector<uint32_t> cap_sig;

  static uint64_t m64(uint32_t w) { return w >= 64 ? ~0ull : ((1ull << w) - 1ull); }
  static uint64_t lit64(const std::vector<uint32_t>& l) {
    return (l.empty() ? 0ull : l[0]) | (l.size() > 1 ? (uint64_t)l[1] << 32 : 0ull);
  }
  static void check_block(const Block& b) {
    for (uint32_t w : b.value_width)
      if (w > 64) throw std::runtime_error("E_UNSUPPORTED: the SIMD engine takes values of at most 64 bits");
  }

  SimdSim(const OracleDesign* od, uint32_t n) : PackedSim(od, n) {
    for (const PackedSignal& sg : P->signals)
      if (sg.layout.width > 64) throw std::runtime_error("E_UNSUPPORTED: the SIMD engine takes signals of at most 64 bits");
    for (const PackedMemory& m : P->memories)
      if (m.data_layout.width > 64) throw std::runtime_error("E_UNSUPPORTED: the SIMD engine takes memory words of at most 64 bits");
    check_block(M->comb);
    check_block(M->async_reset_comb);
    check_block(M->tick_next);
    check_block(M->tick_commit);
  }

  uint64_t* V(uint32_t v) { return wv.data() + (size_t)v * lanes; }
  void load_signal(const ValueLayout& L, uint64_t m, uint64_t* o) const {
    const uint32_t* lo = values.data() + (size_t)L.offset * lanes;
    if (L.limbs == 1) {
      for (uint32_t l = 0; l < lanes; ++l) o[l] = lo[l] & m;
    } else {
      const uint32_t* hi = lo + lanes;
      for (uint32_t l = 0; l < lanes; ++l) o[l] = ((uint64_t)lo[l] | ((uint64_t)hi[l] << 32)) & m;
    }
  }
  void store_signal(const ValueLayout& L, const uint64_t* v) {
    const uint64_t m = m64(L.width);
    uint32_t* lo = values.data() + (size_t)L.offset * lanes;
    if (L.limbs == 1) {
      for (uint32_t l = 0; l < lanes; ++l) lo[l] = (uint32_t)(v[l] & m);
    } else {
      uint32_t* hi = lo + lanes;
      for (uint32_t l = 0; l < lanes; ++l) {
        const uint64_t x = v[l] & m;
        lo[l] = (uint32_t)x;
        hi[l] = (uint32_t)(x >> 32);
      }
    }
  }
  bool reset_on(const PackedReset& r, uint32_t lane) const {
    const bool v = values[(size_t)P->signals[r.signal].layout.offset * lanes + lane] & 1u;
    return r.active_low ? !v : v;
  }
  uint64_t mem_load(const PackedMemory& m, uint32_t lane, uint64_t a) const {
    const uint32_t* p = memories.data() + (size_t)lane * P->total_memory_words_per_lane + m.offset +
                        a * m.data_layout.limbs;
    const uint64_t x = m.data_layout.limbs == 1 ? p[0] : ((uint64_t)p[0] | ((uint64_t)p[1] << 32));
    return x & m64(m.data_layout.width);
  }

  // eval_machine_instr_lane's semantics (lib.rs:9796-9907) on u64 lanes; every
  // result is masked to its width as fit_limbs does.
  void eval(const Instr& in, const Block& b) {
    uint64_t* o = V(in.dst);
    const uint64_t m = m64(in.ty.width);
    const uint32_t n = lanes;
    auto A = [&](uint32_t k) { return (const uint64_t*)V(in.ops[k]); };
    auto Wd = [&](uint32_t k) { return b.value_width[in.ops[k]]; };
    switch (in.kind) {
      case IK::Lit: {
        const uint64_t v = lit64(in.lit) & m;
        for (uint32_t l = 0; l < n; ++l) o[l] = v;
        break;
      }
      case IK::Signal: load_signal(P->signals[in.index].layout, m, o); break;
      case IK::Not: { const uint64_t* a = A(0); for (uint32_t l = 0; l < n; ++l) o[l] = ~a[l] & m; break; }
      case IK::And: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] & c[l]) & m; break; }
      case IK::Or: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] | c[l]) & m; break; }
      case IK::Xor: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] ^ c[l]) & m; break; }
      case IK::Add: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] + c[l]) & m; break; }
      case IK::Sub: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] - c[l]) & m; break; }
      case IK::Mul: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] * c[l]) & m; break; }
      case IK::Eq: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = a[l] == c[l]; break; }
      case IK::Ne: { const uint64_t *a = A(0), *c = A(1); for (uint32_t l = 0; l < n; ++l) o[l] = a[l] != c[l]; break; }
      case IK::Lt: {
        // at the left operand's width (lt_values): the right operand's higher bits are dropped
        const uint64_t *a = A(0), *c = A(1);
        const uint32_t w = Wd(0);
        const uint64_t mw = m64(w);
        if (in.is_signed) {
          const uint32_t sh = 64 - w;
          for (uint32_t l = 0; l < n; ++l)
            o[l] = (int64_t)((a[l] & mw) << sh) < (int64_t)((c[l] & mw) << sh);
        } else {
          for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] & mw) < (c[l] & mw);
        }
        break;
      }
      case IK::Mux: {
        const uint64_t *c = A(0), *t = A(1), *e = A(2);
        for (uint32_t l = 0; l < n; ++l) o[l] = ((c[l] & 1u) ? t[l] : e[l]) & m;
        break;
      }
      case IK::Slice: {
        const uint64_t* a = A(0);
        if (in.lsb >= 64) { for (uint32_t l = 0; l < n; ++l) o[l] = 0; break; }
        for (uint32_t l = 0; l < n; ++l) o[l] = (a[l] >> in.lsb) & m;
        break;
      }
      case IK::Zext: case IK::Trunc: case IK::Cast: { const uint64_t* a = A(0); for (uint32_t l = 0; l < n; ++l) o[l] = a[l] & m; break; }
      case IK::Sext: {
        const uint64_t* a = A(0);
        const uint32_t w = Wd(0);
        const uint64_t mw = m64(w);
        for (uint32_t l = 0; l < n; ++l) {
          const uint64_t x = a[l] & mw;
          o[l] = (((x >> (w - 1)) & 1u) ? (x | ~mw) : x) & m;
        }
        break;
      }
      case IK::Concat: {
        // MSB-first parts (concat_limbs): the last part takes the low bits
        for (uint32_t l = 0; l < n; ++l) o[l] = 0;
        uint32_t off = 0;
        for (size_t k = in.ops.size(); k-- > 0;) {
          const uint64_t* a = A((uint32_t)k);
          const uint32_t w = Wd((uint32_t)k);
          if (off < 64) {
            const uint64_t mw = m64(w);
            for (uint32_t l = 0; l < n; ++l) o[l] |= (a[l] & mw) << off;
          }
          off += w;
        }
        for (uint32_t l = 0; l < n; ++l) o[l] &= m;
        break;
      }
      case IK::MemRead: {
        const PackedMemory& mem = P->memories[in.index];
        const uint64_t* a = A(0);
        for (uint32_t l = 0; l < n; ++l) o[l] = a[l] < mem.depth ? mem_load(mem, l, a[l]) & m : 0ull;
        break;
      }
    }
  }

  // execute_machine_block + execute_machine_effect (lib.rs:9700-9777).
  void exec(const Block& b) {
    if (b.packets.empty()) return;
    wv.resize((size_t)b.num_values * lanes);
    for (auto& pkt : b.packets) {
      for (auto& in : pkt.instrs) eval(in, b);
      for (auto& ef : pkt.effects) {
        const uint64_t* v = V(ef.value);
        if (ef.kind == EffK::StoreSignal) {
          store_signal(P->signals[ef.dst].layout, v);
        } else if (ef.kind == EffK::CaptureReg) {
          if (!ef.has_reset || !ef.reset.async) continue;
          const ValueLayout& L = P->signals[ef.dst].layout;
          for (uint32_t lane = 0; lane < lanes; ++lane)
            if (reset_on(ef.reset, lane)) {
              Limbs x{(uint32_t)v[lane], (uint32_t)(v[lane] >> 32)};
              store_layout(L, lane, x);
            }
        } else {
          const PackedMemory& mem = P->memories[ef.dst];
          const uint64_t *en = V(ef.enable), *ad = V(ef.addr);
          const uint64_t dm = m64(mem.data_layout.width);
          for (uint32_t lane = 0; lane < lanes; ++lane) {
            if (!(en[lane] & 1u) || ad[lane] >= mem.depth) continue;
            uint32_t* p = memories.data() + (size_t)lane * P->total_memory_words_per_lane + mem.offset +
                          ad[lane] * mem.data_layout.limbs;
            const uint64_t x = v[lane] & dm;
            p[0] = (uint32_t)x;
            if (mem.data_layout.limbs > 1) p[1] = (uint32_t)(x >> 32);
          }
        }
      }
    }
  }

  void eval_combinational() override {
    exec(M->comb);
    exec(M->async_reset_comb);
  }
  // capture_register_stream / capture_register_value (lib.rs:9614-9686),
  // memory writes, then the commit of every capture (:9688-9699).
  void tick_from_evaluated_no_post_eval() override {
    const Block& b = M->tick_next;
    size_t k = 0;
    if (!b.packets.empty()) {
      wv.resize((size_t)b.num_values * lanes);
      for (auto& pkt : b.packets) {
        for (auto& in : pkt.instrs) eval(in, b);
        for (auto& ef : pkt.effects) {
          if (ef.kind != EffK::CaptureReg) continue;
          const ValueLayout& L = P->signals[ef.dst].layout;
          if (caps.size() < (k + 1) * lanes) caps.resize((k + 1) * lanes);
          if (cap_sig.size() <= k) cap_sig.resize(k + 1);
          cap_sig[k] = ef.dst;
          uint64_t* c = caps.data() + k * lanes;
          const uint64_t* v = V(ef.value);
          const uint64_t rv = lit64(ef.reset.value) & m64(L.width);
          for (uint32_t lane = 0; lane < lanes; ++lane)
            c[lane] = (ef.has_reset && reset_on(ef.reset, lane)) ? rv : v[lane];
          ++k;
        }
      }
    }
    exec(M->tick_commit);
    for (size_t i = 0; i < k; ++i) store_signal(P->signals[cap_sig[i]].layout, caps.data() + i * lanes);
  }
};

// -------------------------------------------------------------- BitParallel --
// 64 lanes per u64 word, gates as bitwise ops, per-lane stuck-at forces.
struct BitParallel {
  const OracleDesign* d;
  const MachineProgram* M;
  uint32_t lanes, words;
  size_t nsig;
  std::vector<uint64_t> state;  // [sig*words + w]
  std::vector<std::tuple<uint32_t, uint32_t, bool>> forces;

  BitParallel(const OracleDesign* od, uint32_t n) : d(od), M(&od->machine), lanes(n) {
    for (auto& s : M->source.signals)
      if (s.layout.width != 1) throw RrtlError("E_BITPARALLEL", "signal `" + s.name + "` is not 1 bit");
    if (!M->source.memories.empty()) throw RrtlError("E_BITPARALLEL", "memories are not supported by the bit-parallel engine");
    for (const Block* b : {&M->async_reset_comb, &M->comb, &M->tick_next, &M->tick_commit})
      for (auto& p : b->packets) {
        for (auto& in : p.instrs)
          if (!(in.kind == IK::And || in.kind == IK::Or || in.kind == IK::Xor || in.kind == IK::Not ||
                in.kind == IK::Mux || in.kind == IK::Signal || in.kind == IK::Lit))
            throw RrtlError("E_BITPARALLEL", "op is not a gate-level bitwise op");
        for (auto& e : p.effects)
          if (e.kind == EffK::MemoryWrite) throw RrtlError("E_BITPARALLEL", "memory writes are not supported");
      }
    words = std::max<uint32_t>(1, (lanes + 63) / 64);
    nsig = M->source.signals.size();
    state.assign(nsig * words, 0);
  }
  void set_force_bit(uint32_t sig, uint32_t lane, bool v) {
    uint64_t& w = state[(size_t)sig * words + lane / 64];
    if (v) w |= 1ull << (lane % 64); else w &= ~(1ull << (lane % 64));
  }
  void apply_forces() { for (auto& f : forces) set_force_bit(std::get<0>(f), std::get<1>(f), std::get<2>(f)); }
  void clamp_signal(uint32_t sig) {
    for (auto& f : forces)
      if (std::get<0>(f) == sig) set_force_bit(sig, std::get<1>(f), std::get<2>(f));
  }
  void eval_packet(const MPacket& p, std::vector<uint64_t>& work) const {
    for (auto& in : p.instrs) {
      uint64_t* D = &work[(size_t)in.dst * words];
      switch (in.kind) {
        case IK::Signal: std::copy(&state[(size_t)in.index * words], &state[(size_t)in.index * words] + words, D); break;
        case IK::Lit: { uint64_t f = (!in.lit.empty() && (in.lit[0] & 1)) ? ~0ull : 0ull; for (uint32_t k = 0; k < words; ++k) D[k] = f; break; }
        case IK::Not: { const uint64_t* A = &work[(size_t)in.ops[0] * words]; for (uint32_t k = 0; k < words; ++k) D[k] = ~A[k]; break; }
        case IK::And: case IK::Or: case IK::Xor: {
          const uint64_t* A = &work[(size_t)in.ops[0] * words];
          const uint64_t* B = &work[(size_t)in.ops[1] * words];
          for (uint32_t k = 0; k < words; ++k)
            D[k] = in.kind == IK::And ? (A[k] & B[k]) : in.kind == IK::Or ? (A[k] | B[k]) : (A[k] ^ B[k]);
          break;
        }
        case IK::Mux: {
          const uint64_t* C = &work[(size_t)in.ops[0] * words];
          const uint64_t* T = &work[(size_t)in.ops[1] * words];
          const uint64_t* E = &work[(size_t)in.ops[2] * words];
          for (uint32_t k = 0; k < words; ++k) D[k] = (C[k] & T[k]) | (~C[k] & E[k]);
          break;
        }
        default: break;
      }
    }
  }
  void asserted(const PackedReset& r, uint64_t* out) const {
    const uint64_t* s = &state[(size_t)r.signal * words];
    for (uint32_t k = 0; k < words; ++k) out[k] = r.active_low ? ~s[k] : s[k];
  }
  // settle (bitparallel.rs:256-300): async-reset-comb then comb, stores per packet.
  void settle() {
    std::vector<uint64_t> as(words);
    for (const Block* b : {&M->async_reset_comb, &M->comb}) {
      std::vector<uint64_t> work((size_t)b->num_values * words, 0);
      for (auto& p : b->packets) {
        eval_packet(p, work);
        for (auto& e : p.effects) {
          if (e.kind == EffK::StoreSignal) {
            std::copy(&work[(size_t)e.value * words], &work[(size_t)e.value * words] + words, &state[(size_t)e.dst * words]);
            if (!forces.empty()) clamp_signal(e.dst);
          } else if (e.kind == EffK::CaptureReg && e.has_reset) {
            asserted(e.reset, as.data());
            uint64_t rv = (!e.reset.value.empty() && (e.reset.value[0] & 1)) ? ~0ull : 0ull;
            for (uint32_t k = 0; k < words; ++k)
              state[(size_t)e.dst * words + k] = (as[k] & rv) | (~as[k] & work[(size_t)e.value * words + k]);
            if (!forces.empty()) clamp_signal(e.dst);
          }
        }
      }
    }
  }
  // The capture + commit + force part of tick (bitparallel.rs:303-336).
  void capture_commit() {
    const Block& b = M->tick_next;
    std::vector<uint64_t> work((size_t)b.num_values * words, 0);
    for (auto& p : b.packets) eval_packet(p, work);
    std::vector<std::pair<uint32_t, std::vector<uint64_t>>> next;
    std::vector<uint64_t> as(words);
    for (auto& p : b.packets)
      for (auto& e : p.effects) {
        if (e.kind != EffK::CaptureReg) continue;
        std::vector<uint64_t> nv(&work[(size_t)e.value * words], &work[(size_t)e.value * words] + words);
        if (e.has_reset) {
          asserted(e.reset, as.data());
          uint64_t rv = (!e.reset.value.empty() && (e.reset.value[0] & 1)) ? ~0ull : 0ull;
          for (uint32_t k = 0; k < words; ++k) nv[k] = (as[k] & rv) | (~as[k] & nv[k]);
        }
        next.emplace_back(e.dst, std::move(nv));
      }
    for (auto& n : next) std::copy(n.second.begin(), n.second.end(), &state[(size_t)n.first * words]);
    apply_forces();
  }
  void tick() { settle(); capture_commit(); settle(); }
  bool get(uint32_t sig, uint32_t lane) const { return (state[(size_t)sig * words + lane / 64] >> (lane % 64)) & 1; }
  void set(uint32_t sig, uint32_t lane, bool v) {
    uint64_t& w = state[(size_t)sig * words + lane / 64];
    if (v) w |= 1ull << (lane % 64); else w &= ~(1ull << (lane % 64));
  }
};

// ---------------------------------------------------------------- BitSlice --
// BitSliceSimulator (crates/rrtl-sim-ir/src/bitslice.rs:26-402): a W-bit signal is
// W bit-planes of 64 lanes per u64. Bitwise ops and muxes per plane (the mux on
// plane 0 of the condition), add/sub as a ripple carry (sub as a + ~b + 1),
// eq/ne as xor planes OR-reduced over the wider operand, slice / zext / trunc /
// cast / sext (repeating the top plane) / MSB-first concat as plane
// reindexing; operand planes past an operand's width read 0. Settle runs the
// async-reset stream, then comb, storing per packet; tick settles, captures
// every register (reset select per plane) and commits, then settles.
// Scope as the reference's (:37-80): no memories, no multiply, no compare.
struct BitSlice {
  const MachineProgram* M;
  uint32_t lanes, words;
  std::vector<size_t> sig_base;
  std::vector<uint32_t> widths;
  std::vector<uint64_t> state;  // [(sig_base[s] + p) * words + k]

  BitSlice(const OracleDesign* od, uint32_t n) : M(&od->machine), lanes(n) {
    if (!M->source.memories.empty()) throw RrtlError("E_BITSLICE", "bit-slice does not support memories");
    for (const Block* b : {&M->async_reset_comb, &M->comb, &M->tick_next, &M->tick_commit})
      for (auto& p : b->packets)
        for (auto& in : p.instrs)
          if (in.kind == IK::Mul || in.kind == IK::Lt || in.kind == IK::MemRead)
            throw RrtlError("E_BITSLICE", "op outside the bit-slice scope");
    words = std::max<uint32_t>(1, (lanes + 63) / 64);
    size_t total = 0;
    for (auto& s : M->source.signals) {
      sig_base.push_back(total);
      widths.push_back(s.layout.width);
      total += s.layout.width;
    }
    state.assign(total * words, 0);
  }

  struct Work {
    std::vector<size_t> base;
    std::vector<uint32_t> width;
    std::vector<uint64_t> ws;
  };
  uint64_t rd(const Work& W, uint32_t v, size_t p, uint32_t k) const {
    return p < W.width[v] ? W.ws[(W.base[v] + p) * words + k] : 0ull;
  }
  Work eval(const Block& b) const {
    Work W;
    W.width.assign(b.num_values, 0);
    for (uint32_t v = 0; v < b.num_values && v < b.value_width.size(); ++v) W.width[v] = b.value_width[v];
    W.base.assign(b.num_values, 0);
    size_t total = 0;
    for (uint32_t v = 0; v < b.num_values; ++v) {
      W.base[v] = total;
      total += W.width[v];
    }
    W.ws.assign(total * words, 0);
    for (auto& pk : b.packets)
      for (auto& in : pk.instrs) {
        const size_t db = W.base[in.dst];
        const uint32_t dw = W.width[in.dst];
        uint64_t* D = &W.ws[db * words];
        auto put = [&](size_t p, uint32_t k, uint64_t v) { D[p * words + k] = v; };
        switch (in.kind) {
          case IK::Signal:
            for (size_t p = 0; p < dw; ++p)
              for (uint32_t k = 0; k < words; ++k)
                put(p, k, p < widths[in.index] ? state[(sig_base[in.index] + p) * words + k] : 0ull);
            break;
          case IK::Lit:
            for (size_t p = 0; p < dw; ++p) {
              const uint32_t limb = (uint32_t)(p / 32);
              const bool bit = limb < in.lit.size() && ((in.lit[limb] >> (p % 32)) & 1u);
              for (uint32_t k = 0; k < words; ++k) put(p, k, bit ? ~0ull : 0ull);
            }
            break;
          case IK::Not:
            for (size_t p = 0; p < dw; ++p)
              for (uint32_t k = 0; k < words; ++k) put(p, k, ~rd(W, in.ops[0], p, k));
            break;
          case IK::And: case IK::Or: case IK::Xor:
            for (size_t p = 0; p < dw; ++p)
              for (uint32_t k = 0; k < words; ++k) {
                const uint64_t a = rd(W, in.ops[0], p, k), c = rd(W, in.ops[1], p, k);
                put(p, k, in.kind == IK::And ? (a & c) : in.kind == IK::Or ? (a | c) : (a ^ c));
              }
            break;
          case IK::Mux:
            for (uint32_t k = 0; k < words; ++k) {
              const uint64_t c = rd(W, in.ops[0], 0, k);
              for (size_t p = 0; p < dw; ++p) put(p, k, (c & rd(W, in.ops[1], p, k)) | (~c & rd(W, in.ops[2], p, k)));
            }
            break;
          case IK::Eq: case IK::Ne: {
            const size_t wmax = std::max(W.width[in.ops[0]], W.width[in.ops[1]]);
            for (uint32_t k = 0; k < words; ++k) {
              uint64_t diff = 0;
              for (size_t p = 0; p < wmax; ++p) diff |= rd(W, in.ops[0], p, k) ^ rd(W, in.ops[1], p, k);
              put(0, k, in.kind == IK::Eq ? ~diff : diff);
              for (size_t p = 1; p < dw; ++p) put(p, k, 0ull);
            }
            break;
          }
          case IK::Add: case IK::Sub: {
            const bool sub = in.kind == IK::Sub;
            for (uint32_t k = 0; k < words; ++k) {
              uint64_t carry = sub ? ~0ull : 0ull;
              for (size_t p = 0; p < dw; ++p) {
                const uint64_t a = rd(W, in.ops[0], p, k);
                const uint64_t c = sub ? ~rd(W, in.ops[1], p, k) : rd(W, in.ops[1], p, k);
                const uint64_t x = a ^ c;
                put(p, k, x ^ carry);
                carry = (a & c) | (carry & x);
              }
            }
            break;
          }
          case IK::Slice:
            for (size_t p = 0; p < dw; ++p)
              for (uint32_t k = 0; k < words; ++k) put(p, k, rd(W, in.ops[0], p + in.lsb, k));
            break;
          case IK::Zext: case IK::Trunc: case IK::Cast:
            for (size_t p = 0; p < dw; ++p)
              for (uint32_t k = 0; k < words; ++k) put(p, k, rd(W, in.ops[0], p, k));
            break;
          case IK::Sext: {
            const size_t sw = W.width[in.ops[0]];
            for (size_t p = 0; p < dw; ++p)
              for (uint32_t k = 0; k < words; ++k) put(p, k, sw ? rd(W, in.ops[0], p < sw ? p : sw - 1, k) : 0ull);
            break;
          }
          case IK::Concat: {
            size_t off = 0;
            for (size_t q = in.ops.size(); q-- > 0;) {
              const uint32_t pw = W.width[in.ops[q]];
              for (size_t p = 0; p < pw && off + p < dw; ++p)
                for (uint32_t k = 0; k < words; ++k) put(off + p, k, rd(W, in.ops[q], p, k));
              off += pw;
            }
            break;
          }
          default: break;
        }
      }
    return W;
  }
  void asserted(const PackedReset& r, std::vector<uint64_t>& out) const {
    for (uint32_t k = 0; k < words; ++k) {
      const uint64_t b = state[sig_base[r.signal] * words + k];  // plane 0 of the reset signal
      out[k] = r.active_low ? ~b : b;
    }
  }
  void store(uint32_t dst, const Work& W, uint32_t v, const PackedReset* r) {
    std::vector<uint64_t> as(words, 0);
    if (r) asserted(*r, as);
    for (size_t p = 0; p < widths[dst]; ++p) {
      const uint32_t limb = (uint32_t)(p / 32);
      const bool rb = r && limb < r->value.size() && ((r->value[limb] >> (p % 32)) & 1u);
      for (uint32_t k = 0; k < words; ++k) {
        const uint64_t nv = rd(W, v, p, k);
        state[(sig_base[dst] + p) * words + k] = r ? ((as[k] & (rb ? ~0ull : 0ull)) | (~as[k] & nv)) : nv;
      }
    }
  }
  void settle() {
    for (const Block* b : {&M->async_reset_comb, &M->comb}) {
      const Work W = eval(*b);
      for (auto& pk : b->packets)
        for (auto& e : pk.effects) {
          if (e.kind == EffK::StoreSignal) store(e.dst, W, e.value, nullptr);
          else if (e.kind == EffK::CaptureReg && e.has_reset) store(e.dst, W, e.value, &e.reset);
        }
    }
  }
  void tick() {
    settle();
    const Work W = eval(M->tick_next);
    // every capture reads the pre-commit state; all commit together
    std::vector<std::pair<uint32_t, std::vector<uint64_t>>> next;
    std::vector<uint64_t> as(words, 0);
    for (auto& pk : M->tick_next.packets)
      for (auto& e : pk.effects) {
        if (e.kind != EffK::CaptureReg) continue;
        if (e.has_reset) asserted(e.reset, as);
        std::vector<uint64_t> planes((size_t)widths[e.dst] * words);
        for (size_t p = 0; p < widths[e.dst]; ++p) {
          const uint32_t limb = (uint32_t)(p / 32);
          const bool rb = e.has_reset && limb < e.reset.value.size() && ((e.reset.value[limb] >> (p % 32)) & 1u);
          for (uint32_t k = 0; k < words; ++k) {
            const uint64_t nv = rd(W, e.value, p, k);
            planes[p * words + k] = e.has_reset ? ((as[k] & (rb ? ~0ull : 0ull)) | (~as[k] & nv)) : nv;
          }
        }
        next.emplace_back(e.dst, std::move(planes));
      }
    for (auto& n : next) std::copy(n.second.begin(), n.second.end(), &state[sig_base[n.first] * words]);
    settle();
  }
  void set_lanes(uint32_t sig, const uint32_t* data) {  // [limbs][lanes]
    const uint32_t limbs = std::max<uint32_t>(1, (widths[sig] + 31) / 32);
    for (size_t p = 0; p < widths[sig]; ++p)
      for (uint32_t k = 0; k < words; ++k) state[(sig_base[sig] + p) * words + k] = 0;
    for (uint32_t l = 0; l < lanes; ++l)
      for (size_t p = 0; p < widths[sig]; ++p)
        if ((p / 32) < limbs && ((data[(p / 32) * lanes + l] >> (p % 32)) & 1u))
          state[(sig_base[sig] + p) * words + l / 64] |= 1ull << (l % 64);
  }
  void get_lanes(uint32_t sig, uint32_t* out) const {  // [limbs][lanes]
    const uint32_t limbs = std::max<uint32_t>(1, (widths[sig] + 31) / 32);
    std::fill(out, out + (size_t)limbs * lanes, 0u);
    for (uint32_t l = 0; l < lanes; ++l)
      for (size_t p = 0; p < widths[sig]; ++p)
        if ((state[(sig_base[sig] + p) * words + l / 64] >> (l % 64)) & 1ull) out[(p / 32) * lanes + l] |= 1u << (p % 32);
  }
};

// ---------------------------------------------------------------- ScalarSim --
// rrtl_core::Simulator: hierarchical, unmasked u128 intermediates, fixpoint settle.
u128 mask128(uint32_t w) { return w >= 128 ? ~(u128)0 : (((u128)1 << w) - 1); }
u128 encode_value(i128 v, BitType ty) { return (u128)v & mask128(ty.width); }
i128 signed_value(u128 v, uint32_t w) {
  if (w == 0) return 0;
  if (w >= 128) return (i128)v;
  u128 sb = (u128)1 << (w - 1);
  v &= mask128(w);
  return (v & sb) ? (i128)v - ((i128)1 << w) : (i128)v;
}

struct ScalarSim {
  const Design* d;
  const Module* m;
  std::unordered_map<uint32_t, u128> values;
  std::unordered_map<uint32_t, std::vector<u128>> mems;
  struct Child { const Instance* inst; std::unique_ptr<ScalarSim> sim; };
  std::vector<Child> children;

  ScalarSim(const Design* dd, const Module* mm) : d(dd), m(mm) {
    for (auto& s : m->signals) {
      u128 iv = 0;
      for (auto& ir : m->initial_register_values)
        if (ir.signal.id == s.handle.id) { iv = encode_value(ir.value, s.ty) & mask128(s.width); break; }
      values[s.handle.id] = iv & mask128(s.width);
      if (s.kind == SigKind::Mem) {
        std::vector<u128> mem(s.depth, 0);
        for (auto& im : m->initial_memory_values)
          if (im.mem.id == s.handle.id && im.addr < mem.size()) mem[im.addr] = encode_value(im.value, s.ty);
        mems[s.handle.id] = std::move(mem);
      }
    }
    for (auto& inst : m->instances) {
      const Module* cm = d->find_module(inst.module);
      if (!cm) throw RrtlError("E_SIM_INSTANCE", "instance target `" + inst.module + "` does not exist");
      children.push_back(Child{&inst, std::make_unique<ScalarSim>(d, cm)});
    }
  }
  static ScalarSim* create(const Design* d, const std::string& top) {
    const Module* m = d->find_module(top);
    if (!m) throw RrtlError("E_SIM_MODULE", "module `" + top + "` does not exist");
    auto* s = new ScalarSim(d, m);
    s->eval_combinational();
    return s;
  }
  u128 get(uint32_t id) const { auto it = values.find(id); return it == values.end() ? 0 : it->second; }
  void set(uint32_t id, u128 v) { values[id] = v & mask128(m->signals[id].width); eval_combinational(); }
  void set_raw(uint32_t id, u128 v) { values[id] = v & mask128(m->signals[id].width); }

  std::optional<BitType> type_of(const Expr& e) const {  // expr_type_no_diag
    try { return expr_type(*m, e); } catch (...) { return std::nullopt; }
  }
  u128 eval(const Expr& e) const {  // Simulator::eval_expr (lib.rs:6401-6469)
    switch (e.kind) {
      case EK::Lit: return encode_value(e.value, e.ty);
      case EK::Signal: return get(e.sig.id);
      case EK::Not: return ~eval(e.args[0]);
      case EK::And: return eval(e.args[0]) & eval(e.args[1]);
      case EK::Or: return eval(e.args[0]) | eval(e.args[1]);
      case EK::Xor: return eval(e.args[0]) ^ eval(e.args[1]);
      case EK::Add: return eval(e.args[0]) + eval(e.args[1]);
      case EK::Sub: return eval(e.args[0]) - eval(e.args[1]);
      case EK::Mul: return eval(e.args[0]) * eval(e.args[1]);
      case EK::Eq: return eval(e.args[0]) == eval(e.args[1]);
      case EK::Ne: return eval(e.args[0]) != eval(e.args[1]);
      case EK::Lt: {
        BitType lt = type_of(e.args[0]).value_or(uint_t(128));
        if (lt.is_signed) return signed_value(eval(e.args[0]), lt.width) < signed_value(eval(e.args[1]), lt.width);
        return eval(e.args[0]) < eval(e.args[1]);
      }
      case EK::Mux: return eval(e.args[0]) != 0 ? eval(e.args[1]) : eval(e.args[2]);
      case EK::Slice: {
        u128 v = eval(e.args[0]);
        return (e.lsb >= 128 ? 0 : (v >> e.lsb)) & mask128(e.width);
      }
      case EK::Zext: case EK::Trunc: return eval(e.args[0]) & mask128(e.width);
      case EK::Sext: {
        BitType it = type_of(e.args[0]).value_or(uint_t(e.width));
        return encode_value(signed_value(eval(e.args[0]), it.width), sint_t(e.width));
      }
      case EK::Cast: return eval(e.args[0]);
      case EK::Concat: {
        u128 v = 0;
        uint32_t sh = 0;
        for (auto it = e.args.rbegin(); it != e.args.rend(); ++it) {
          uint32_t w = type_of(*it) ? type_of(*it)->width : 0;
          if (sh < 128) v |= eval(*it) << sh;
          sh += w;
        }
        return v;
      }
      case EK::MemRead: {
        u128 a = eval(e.args[0]);
        auto it = mems.find(e.sig.id);
        if (it == mems.end() || a >= it->second.size()) return 0;
        return it->second[(size_t)a];
      }
    }
    return 0;
  }
  bool reset_asserted(const Reset& r) const { return r.active_low ? get(r.signal.id) == 0 : get(r.signal.id) != 0; }
  bool apply_async_resets() {
    bool changed = false;
    for (auto& s : m->signals)
      if (s.kind == SigKind::Reg && s.reset && s.reset->async && reset_asserted(*s.reset)) {
        u128 v = encode_value(s.reset->value, s.ty);
        if (get(s.handle.id) != v) changed = true;
        values[s.handle.id] = v;
      }
    return changed;
  }
  void drive_child_inputs() {
    for (auto& c : children) {
      const Module* cm = c.sim->m;
      for (auto& conn : c.inst->connections)
        for (auto& s : cm->signals)
          if (s.name == conn.first && s.kind == SigKind::Input) {
            c.sim->values[s.handle.id] = get(conn.second.id) & mask128(s.width);
            break;
          }
    }
  }
  bool eval_instances() {
    drive_child_inputs();
    bool changed = false;
    std::vector<std::pair<uint32_t, u128>> writes;
    for (auto& c : children) {
      c.sim->eval_combinational();
      for (auto& conn : c.inst->connections)
        for (auto& s : c.sim->m->signals)
          if (s.name == conn.first && s.kind == SigKind::Output) {
            writes.emplace_back(conn.second.id, c.sim->get(s.handle.id) & mask128(s.width));
            break;
          }
    }
    for (auto& w : writes) {
      if (get(w.first) != w.second) changed = true;
      values[w.first] = w.second;
    }
    return changed;
  }
  void eval_combinational() {  // lib.rs:6286-6311
    size_t limit = std::max<size_t>(1, m->assignments.size() + m->instances.size());
    for (size_t it = 0; it < limit; ++it) {
      bool changed = apply_async_resets();
      for (auto& a : m->assignments) {
        const SignalInfo* dst = m->signal(a.dst);
        if (!dst) continue;
        u128 v = eval(a.expr) & mask128(dst->width);
        if (get(a.dst.id) != v) changed = true;
        values[a.dst.id] = v;
      }
      if (eval_instances()) changed = true;
      if (apply_async_resets()) changed = true;
      if (!changed) break;
    }
  }
  struct TickState {
    std::vector<std::pair<uint32_t, u128>> vals;
    std::vector<std::tuple<uint32_t, u128, u128>> mem;
    std::vector<TickState> kids;
  };
  TickState capture_tick() {  // lib.rs:6140-6186
    drive_child_inputs();
    for (auto& c : children) c.sim->eval_combinational();
    TickState t;
    for (auto& s : m->signals) {
      if (s.kind != SigKind::Reg) continue;
      u128 v = (s.reset && reset_asserted(*s.reset)) ? encode_value(s.reset->value, s.ty) : eval(*s.next);
      t.vals.emplace_back(s.handle.id, v & mask128(s.width));
    }
    for (auto& w : m->memory_writes)
      if (eval(w.enable) != 0) {
        const SignalInfo* mem = m->signal(w.mem);
        if (!mem) continue;
        t.mem.emplace_back(w.mem.id, eval(w.addr), eval(w.data) & mask128(mem->width));
      }
    for (auto& c : children) t.kids.push_back(c.sim->capture_tick());
    return t;
  }
  void apply_tick(TickState& t) {
    for (auto& v : t.vals) values[v.first] = v.second;
    for (auto& w : t.mem) {
      auto& mem = mems[std::get<0>(w)];
      if (std::get<1>(w) < mem.size()) mem[(size_t)std::get<1>(w)] = std::get<2>(w);
    }
    for (size_t i = 0; i < children.size(); ++i) children[i].sim->apply_tick(t.kids[i]);
  }
  void tick() {  // tick_checked without assertions/covers (lib.rs:6036-6044)
    eval_combinational();
    TickState t = capture_tick();
    apply_tick(t);
    eval_combinational();
  }
};

}  // namespace

// ------------------------------------------------------------------- C ABI --
extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_design_load(const char* json, size_t len, const char* top) {
  try {
    auto* d = new OracleDesign;
    d->design = design_from_json(json, len);
    d->top = top;
    d->packed = lower_to_packed_program(d->design, top);
    d->machine = lower_to_machine_program(d->packed);
    return d;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void orc_design_free(void* d) { delete (OracleDesign*)d; }

int orc_signal_index(void* dp, const char* name) {
  auto* d = (OracleDesign*)dp;
  std::string full = std::string(d->top) + "." + name;
  for (size_t i = 0; i < d->packed.signals.size(); ++i)
    if (d->packed.signals[i].name == name || d->packed.signals[i].name == full) return (int)i;
  return -1;
}
int orc_memory_index(void* dp, const char* name) {
  auto* d = (OracleDesign*)dp;
  std::string full = std::string(d->top) + "." + name;
  for (size_t i = 0; i < d->packed.memories.size(); ++i)
    if (d->packed.memories[i].name == name || d->packed.memories[i].name == full) return (int)i;
  return -1;
}
uint32_t orc_signal_width(void* dp, uint32_t i) { return ((OracleDesign*)dp)->packed.signals[i].layout.width; }
uint32_t orc_signal_kind(void* dp, uint32_t i) { return (uint32_t)((OracleDesign*)dp)->packed.signals[i].kind; }
uint32_t orc_num_signals(void* dp) { return (uint32_t)((OracleDesign*)dp)->packed.signals.size(); }
uint64_t orc_total_signal_words(void* dp) { return ((OracleDesign*)dp)->packed.total_signal_words; }
uint64_t orc_total_memory_words(void* dp) { return ((OracleDesign*)dp)->packed.total_memory_words_per_lane; }
uint64_t orc_num_instrs(void* dp) {
  auto* d = (OracleDesign*)dp;
  uint64_t n = 0;
  for (const Block* b : {&d->machine.async_reset_comb, &d->machine.comb, &d->machine.tick_next, &d->machine.tick_commit})
    for (auto& p : b->packets) n += p.instrs.size();
  return n;
}
uint32_t orc_num_comb_packets(void* dp) { return (uint32_t)((OracleDesign*)dp)->machine.comb.packets.size(); }
uint32_t orc_num_levels(void* dp) { return (uint32_t)((OracleDesign*)dp)->packed.comb.size(); }
int orc_signal_top_id(void* dp, uint32_t i) {
  auto* d = (OracleDesign*)dp;
  return d->packed.signals[i].top ? (int)d->packed.signals[i].src_id : -1;
}

// ---- stimulus / hash known answers
uint32_t orc_stim_word(uint64_t seed, uint64_t stream, uint64_t cycle, uint64_t idx) { return o_stim_word(seed, stream, cycle, idx); }
uint64_t orc_hash_term(uint64_t cycle, uint32_t rec, uint64_t idx, uint32_t value) { return o_hash_term(cycle, rec, idx, value); }

// ---- PackedSim
void* orc_packed_new(void* dp, uint32_t lanes) {
  if (!lanes) { g_err = "E_SIM_IR_LANES: packed simulator requires at least one lane"; return nullptr; }
  try { return new PackedSim((OracleDesign*)dp, lanes); } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_packed_free(void* s) { delete (PackedSim*)s; }
// SimdSim: a PackedSim whose cycle runs on u64 lanes (every orc_packed_* call applies).
void* orc_simd_new(void* dp, uint32_t lanes) {
  if (!lanes) { g_err = "E_SIM_IR_LANES: packed simulator requires at least one lane"; return nullptr; }
  try { return static_cast<PackedSim*>(new SimdSim((OracleDesign*)dp, lanes)); } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}
// set_signal_limbs re-settles (lib.rs:9911-9944); `settle`=0 gives the raw store.
void orc_packed_set_signal(void* sp, uint32_t sig, const uint32_t* data, int settle) {
  auto* s = (PackedSim*)sp;
  const ValueLayout& L = s->P->signals[sig].layout;
  for (uint32_t lane = 0; lane < s->lanes; ++lane) {
    Limbs v(L.limbs);
    for (uint32_t i = 0; i < L.limbs; ++i) v[i] = data[(size_t)i * s->lanes + lane];
    s->store_layout(L, lane, v);
  }
  if (settle) s->eval_combinational();
}
void orc_packed_get_signal(void* sp, uint32_t sig, uint32_t* out) {
  auto* s = (PackedSim*)sp;
  const ValueLayout& L = s->P->signals[sig].layout;
  for (uint32_t lane = 0; lane < s->lanes; ++lane) {
    Limbs v = s->load_layout(L, lane);
    for (uint32_t i = 0; i < L.limbs; ++i) out[(size_t)i * s->lanes + lane] = v[i];
  }
}
// data layout [addr][limb][lane]
void orc_packed_set_memory(void* sp, uint32_t mi, const uint32_t* data, int settle) {
  auto* s = (PackedSim*)sp;
  const PackedMemory& m = s->P->memories[mi];
  uint32_t nl = m.data_layout.limbs;
  for (uint64_t a = 0; a < m.depth; ++a)
    for (uint32_t lane = 0; lane < s->lanes; ++lane) {
      Limbs v(nl);
      for (uint32_t i = 0; i < nl; ++i) v[i] = data[(a * nl + i) * s->lanes + lane];
      s->store_memory(mi, lane, a, v);
    }
  if (settle) s->eval_combinational();
}
void orc_packed_get_memory(void* sp, uint32_t mi, uint32_t* out) {
  auto* s = (PackedSim*)sp;
  const PackedMemory& m = s->P->memories[mi];
  uint32_t nl = m.data_layout.limbs;
  for (uint64_t a = 0; a < m.depth; ++a)
    for (uint32_t lane = 0; lane < s->lanes; ++lane) {
      Limbs v = s->load_memory(m, lane, a);
      for (uint32_t i = 0; i < nl; ++i) out[(a * nl + i) * s->lanes + lane] = v[i];
    }
}
void orc_packed_eval(void* s) { ((PackedSim*)s)->eval_combinational(); }
void orc_packed_tick(void* s) { ((PackedSim*)s)->tick(); }
void orc_packed_tick_many(void* s, uint64_t n) { ((PackedSim*)s)->tick_many(n); }
void orc_packed_tick_from_evaluated(void* s) { ((PackedSim*)s)->tick_from_evaluated_no_post_eval(); }
void orc_packed_snapshot(void* sp, uint32_t* values, uint32_t* mems) {
  auto* s = (PackedSim*)sp;
  if (values) std::copy(s->values.begin(), s->values.end(), values);
  if (mems) std::copy(s->memories.begin(), s->memories.end(), mems);
}

// Run protocol on PackedSim (per cycle: inputs, settle, record, tick_from_evaluated).
int orc_packed_run(void* sp, const rrtl_run* r) {
  auto* s = (PackedSim*)sp;
  const PackedProgram& P = *s->P;
  uint32_t lanes = s->lanes;
  if (r->record_mode & RRTL_REC_DETECT) { g_err = "E_UNSUPPORTED: detection needs the bit-parallel engine"; return RRTL_E_UNSUPPORTED; }
  uint32_t words = (lanes + 31) / 32;
  for (uint64_t c = 0; c < r->cycles; ++c) {
    for (uint32_t k = 0; k < r->n_stim; ++k) {
      const rrtl_stim& st = r->stim[k];
      const ValueLayout& L = P.signals[st.signal].layout;
      if (st.kind == RRTL_STIM_HOLD) continue;
      // limb i of every lane, masked to the width like store_layout (fit_limbs)
      for (uint32_t i = 0; i < L.limbs; ++i) {
        const uint32_t m = i + 1 == L.limbs ? top_mask(L.width) : 0xFFFFFFFFu;
        uint32_t* dst = s->values.data() + s->vidx(L.offset, i, 0);
        if (st.kind == RRTL_STIM_RANDOM) {
          for (uint32_t lane = 0; lane < lanes; ++lane)
            dst[lane] = o_stim_lane_limb(r->seed, st.param, c, r->lane_base + lane, L.width, i) & m;
        } else if (st.kind == RRTL_STIM_TRACE) {
          for (uint32_t lane = 0; lane < lanes; ++lane)
            dst[lane] = r->input_trace[(c * r->n_trace_cols + st.param + i) * lanes + lane] & m;
        } else {
          uint32_t v = 0;  // lane-uniform kinds
          if (st.kind == RRTL_STIM_RANDOM_UNIFORM) v = o_stim_lane_limb(r->seed, st.param, c, 0, L.width, i);
          else if (st.kind == RRTL_STIM_PULSE) v = (i == 0 && c < st.param) ? 1u : 0u;
          else if (st.kind == RRTL_STIM_CONST) v = i < 2 ? (uint32_t)(st.param >> (32 * i)) : 0u;
          for (uint32_t lane = 0; lane < lanes; ++lane) dst[lane] = v & m;
        }
      }
    }
    s->eval_combinational();
    uint64_t h = 0;
    for (uint32_t q = 0; q < r->n_record; ++q) {
      const ValueLayout& L = P.signals[r->record[q]].layout;
      if (L.width == 1) {
        // hash terms of 1-bit signals cover 32-lane packed words
        for (uint32_t w = 0; w < words; ++w) {
          uint32_t packed = 0;
          for (uint32_t b = 0; b < 32 && w * 32 + b < lanes; ++b) packed |= (s->values[s->vidx(L.offset, 0, w * 32 + b)] & 1u) << b;
          if (r->record_mode & RRTL_REC_HASH) h += o_hash_term(c, q, r->lane_base / 32 + w, packed);
        }
      }
      {
        for (uint32_t i = 0; i < L.limbs; ++i)
          for (uint32_t lane = 0; lane < lanes; ++lane) {
            uint32_t v = s->values[s->vidx(L.offset, i, lane)];
            if (i + 1 == L.limbs) v &= top_mask(L.width);
            if (r->record_mode & RRTL_REC_TRACE) {
              // word engine trace layout: [cycle][rec][limb][lane] with the per-record limb prefix
              size_t base = 0;
              for (uint32_t q2 = 0; q2 < q; ++q2) base += (size_t)P.signals[r->record[q2]].layout.limbs;
              size_t total = 0;
              for (uint32_t q2 = 0; q2 < r->n_record; ++q2) total += (size_t)P.signals[r->record[q2]].layout.limbs;
              r->out_trace[(c * total + base + i) * lanes + lane] = v;
            }
            if ((r->record_mode & RRTL_REC_HASH) && L.width != 1)
              h += o_hash_term(c, q, (r->lane_base + lane) * L.limbs + i, v);
          }
      }
    }
    if (r->record_mode & RRTL_REC_HASH) r->out_hash[c] = h;
    s->tick_from_evaluated_no_post_eval();
  }
  s->eval_combinational();
  return 0;
}

// ---- BitSlice
void* orc_bs_new(void* dp, uint32_t lanes) {
  try { return new BitSlice((OracleDesign*)dp, lanes); } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_bs_free(void* s) { delete (BitSlice*)s; }
void orc_bs_set_signal(void* s, uint32_t sig, const uint32_t* data) { ((BitSlice*)s)->set_lanes(sig, data); }
void orc_bs_get_signal(void* s, uint32_t sig, uint32_t* out) { ((BitSlice*)s)->get_lanes(sig, out); }
void orc_bs_tick(void* s) { ((BitSlice*)s)->tick(); }

// ---- BitParallel
void* orc_bp_new(void* dp, uint32_t lanes) {
  try { return new BitParallel((OracleDesign*)dp, lanes); } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_bp_free(void* s) { delete (BitParallel*)s; }
void orc_bp_set_force(void* sp, uint32_t sig, uint32_t lane, int v) { ((BitParallel*)sp)->forces.emplace_back(sig, lane, v != 0); }
void orc_bp_set(void* sp, uint32_t sig, uint32_t lane, int v) { ((BitParallel*)sp)->set(sig, lane, v != 0); }
void orc_bp_set_all(void* sp, uint32_t sig, int v) {
  auto* s = (BitParallel*)sp;
  for (uint32_t w = 0; w < s->words; ++w) s->state[(size_t)sig * s->words + w] = v ? ~0ull : 0ull;
}
int orc_bp_get(void* sp, uint32_t sig, uint32_t lane) { return ((BitParallel*)sp)->get(sig, lane); }
void orc_bp_tick(void* s) { ((BitParallel*)s)->tick(); }
void orc_bp_settle(void* s) { ((BitParallel*)s)->settle(); }
// 32-lane words of one signal (bit k of word w = lane 32w+k)
void orc_bp_get_bits(void* sp, uint32_t sig, uint32_t* out) {
  auto* s = (BitParallel*)sp;
  uint32_t nw = (s->lanes + 31) / 32;
  for (uint32_t w = 0; w < nw; ++w) {
    uint64_t x = s->state[(size_t)sig * s->words + w / 2];
    uint32_t v = (uint32_t)(w % 2 ? x >> 32 : x);
    uint32_t valid = s->lanes - w * 32;
    if (valid < 32) v &= (1u << valid) - 1u;
    out[w] = v;
  }
}
void orc_bp_set_bits(void* sp, uint32_t sig, const uint32_t* in) {
  auto* s = (BitParallel*)sp;
  uint32_t nw = (s->lanes + 31) / 32;
  for (uint32_t w = 0; w < nw; ++w) {
    uint64_t& x = s->state[(size_t)sig * s->words + w / 2];
    uint32_t valid = s->lanes - w * 32;
    uint32_t v = in[w];
    if (valid < 32) v &= (1u << valid) - 1u;
    if (w % 2) x = (x & 0xFFFFFFFFull) | ((uint64_t)v << 32);
    else x = (x & ~0xFFFFFFFFull) | v;
  }
}

// Run protocol on BitParallel (inputs, settle, record, capture/commit/forces).
// `threads` > 1 splits 64-lane groups across host threads (tick_many_parallel,
// bitparallel.rs:513-523); each thread runs an independent engine on its lanes.
int orc_bp_run(void* sp, const rrtl_run* r) {
  auto* s = (BitParallel*)sp;
  const PackedProgram& P = s->M->source;
  uint32_t lanes = s->lanes, words32 = (lanes + 31) / 32;
  for (uint32_t k = 0; k < r->n_stim; ++k)
    if (s->M->source.signals[r->stim[k].signal].layout.width != 1) { g_err = "E_ARG: stimulus on a wide signal"; return RRTL_E_ARG; }
  std::vector<uint32_t> col(words32);
  if (r->record_mode & RRTL_REC_DETECT)
    for (uint32_t l = 0; l < lanes; ++l) r->detect[l] = 0xFFFFFFFFu;
  for (uint64_t c = 0; c < r->cycles; ++c) {
    for (uint32_t k = 0; k < r->n_stim; ++k) {
      const rrtl_stim& st = r->stim[k];
      if (st.kind == RRTL_STIM_HOLD) continue;
      for (uint32_t w = 0; w < words32; ++w) {
        uint32_t v = 0;
        if (st.kind == RRTL_STIM_RANDOM) v = o_stim_word(r->seed, st.param, c, r->lane_base / 32 + w);
        else if (st.kind == RRTL_STIM_RANDOM_UNIFORM) v = (o_stim_word(r->seed, st.param, c, 0) & 1u) ? 0xFFFFFFFFu : 0u;
        else if (st.kind == RRTL_STIM_PULSE) v = c < st.param ? 0xFFFFFFFFu : 0u;
        else if (st.kind == RRTL_STIM_CONST) v = (st.param & 1) ? 0xFFFFFFFFu : 0u;
        else if (st.kind == RRTL_STIM_TRACE) v = r->input_trace[(c * r->n_trace_cols + st.param) * words32 + w];
        col[w] = v;
      }
      orc_bp_set_bits(s, st.signal, col.data());
    }
    s->settle();
    uint64_t h = 0;
    std::vector<uint32_t> diff(words32, 0);
    for (uint32_t q = 0; q < r->n_record; ++q) {
      orc_bp_get_bits(s, r->record[q], col.data());
      for (uint32_t w = 0; w < words32; ++w) {
        if (r->record_mode & RRTL_REC_TRACE) r->out_trace[(c * r->n_record + q) * words32 + w] = col[w];
        if (r->record_mode & RRTL_REC_HASH) h += o_hash_term(c, q, r->lane_base / 32 + w, col[w]);
        if (r->record_mode & RRTL_REC_DETECT) diff[w] |= col[w] ^ ((col[w] & 1u) ? 0xFFFFFFFFu : 0u);
      }
    }
    if (r->record_mode & RRTL_REC_HASH) r->out_hash[c] = h;
    if (r->record_mode & RRTL_REC_DETECT)
      for (uint32_t l = 0; l < lanes; ++l)
        if (r->detect[l] == 0xFFFFFFFFu && ((diff[l / 32] >> (l % 32)) & 1u)) r->detect[l] = (uint32_t)c;
    s->capture_commit();
  }
  s->settle();
  (void)P;
  return 0;
}

// Lane-parallel CPU baseline: `threads` independent BitParallel engines over
// disjoint 64-lane groups, each running the same protocol on its lanes. Only
// RANDOM / RANDOM_UNIFORM / PULSE / CONST stimuli (functions of the global lane).
// Returns the per-cycle hash (sum over all engines) in r->out_hash.
int orc_bp_run_parallel(void* dp, uint32_t lanes, const rrtl_run* r, uint32_t threads) {
  auto* d = (OracleDesign*)dp;
  if (lanes % 64) { g_err = "E_ARG: lanes must be a multiple of 64"; return RRTL_E_ARG; }
  uint32_t groups = lanes / 64;
  threads = std::max<uint32_t>(1, std::min(threads, groups));
  std::vector<std::vector<uint64_t>> hashes(threads, std::vector<uint64_t>(r->cycles, 0));
  std::vector<int> rc(threads, 0);
  std::vector<std::thread> pool;
  for (uint32_t t = 0; t < threads; ++t) {
    pool.emplace_back([&, t]() {
      uint32_t g0 = (uint32_t)((uint64_t)groups * t / threads), g1 = (uint32_t)((uint64_t)groups * (t + 1) / threads);
      uint32_t my = (g1 - g0) * 64;
      if (!my) return;
      BitParallel bp(d, my);
      const uint64_t w32 = my / 32, wbase = r->lane_base / 32 + (uint64_t)g0 * 2;
      std::vector<uint32_t> col(w32);
      for (uint64_t c = 0; c < r->cycles; ++c) {
        for (uint32_t k = 0; k < r->n_stim; ++k) {
          const rrtl_stim& st = r->stim[k];
          if (st.kind == RRTL_STIM_HOLD) continue;
          for (uint32_t w = 0; w < w32; ++w) {
            uint32_t v = 0;
            if (st.kind == RRTL_STIM_RANDOM) v = o_stim_word(r->seed, st.param, c, wbase + w);
            else if (st.kind == RRTL_STIM_RANDOM_UNIFORM) v = (o_stim_word(r->seed, st.param, c, 0) & 1u) ? 0xFFFFFFFFu : 0u;
            else if (st.kind == RRTL_STIM_PULSE) v = c < st.param ? 0xFFFFFFFFu : 0u;
            else if (st.kind == RRTL_STIM_CONST) v = (st.param & 1) ? 0xFFFFFFFFu : 0u;
            col[w] = v;
          }
          orc_bp_set_bits(&bp, st.signal, col.data());
        }
        bp.settle();
        uint64_t h = 0;
        for (uint32_t q = 0; q < r->n_record; ++q) {
          orc_bp_get_bits(&bp, r->record[q], col.data());
          for (uint32_t w = 0; w < w32; ++w) h += o_hash_term(c, q, wbase + w, col[w]);
        }
        hashes[t][c] = h;
        bp.capture_commit();
      }
    });
  }
  for (auto& th : pool) th.join();
  if (r->out_hash)
    for (uint64_t c = 0; c < r->cycles; ++c) {
      uint64_t h = 0;
      for (uint32_t t = 0; t < threads; ++t) h += hashes[t][c];
      r->out_hash[c] = h;
    }
  for (int x : rc)
    if (x) return x;
  return 0;
}

// ---- ScalarSim (top-module signal ids, values as two u64 halves)
// Bit-parallel AOT source (BitParallelAot, crates/rrtl-sim-ir/src/bitparallel.rs:348-528:
// `aot::emit_block_c` / `generate_c`): the design's comb and tick_next blocks
// as straight-line u64 C over one 64-lane group, inside a group loop and a
// cycle loop. Unlike the reference's single function, the straight-line code
// is cut into functions of about kAotChunk instructions (see AotEmitter),
// which keeps the C compiler's time linear in the design size. To be comparable with the other engines it also runs this
// library's run protocol per cycle: stimulus from the counter hash
// (RANDOM / RANDOM_UNIFORM / PULSE / CONST), settle, per-cycle output hash, capture/commit.
// Entry: run_bp(st, groups, g_base, c0, cycles, seed, hash) with st the
// [group][signal] state of `groups` groups starting at global group g_base.
// The source comes as translation units separated by "//@@PART@@" lines.
static const size_t kAotChunk = 400;

struct AotEmitter {
  std::vector<std::string> fns;    // emitted functions
  std::vector<std::string> calls;  // call statements, in order
  std::vector<uint32_t> caps;      // tick_next capture destinations (index = nx slot)
  int nfn = 0;

  // Emit a block level by level (a level = sub-packets up to the one that
  // carries the effects; values never cross levels). Inside a level every
  // effect's expression tree is emitted depth first right before the effect,
  // sharing the values already emitted in the current function; functions
  // are cut at effect boundaries after about kAotChunk instructions, and a
  // value from an earlier function of the level is recomputed (a signal
  // reloaded) rather than passed on. The C compiler's time stays linear in
  // the design size.
  void block(const Block& b, const char* p, bool capture) {
    std::string body;
    size_t n = 0;
    std::unordered_map<uint32_t, const Instr*> def;  // value id -> instruction (current level)
    std::unordered_map<uint32_t, int> emitted;       // value id -> function index it was emitted in
    auto flush = [&]() {
      if (body.empty()) return;
      const std::string name = std::string("blk_") + p + std::to_string(nfn);
      fns.push_back("void " + name + "(u64* restrict s, u64* restrict nx) {\n" + body + "  (void)nx;\n}\n");
      calls.push_back(name + "(s, nx);");
      body.clear();
      n = 0;
      ++nfn;
    };
    auto op = [&](uint32_t v) { return std::string(p) + std::to_string(v); };
    std::function<void(uint32_t)> emit = [&](uint32_t v) {
      auto e = emitted.find(v);
      if (e != emitted.end() && e->second == nfn) return;
      const Instr& in = *def.at(v);
      for (uint32_t o : in.ops) emit(o);
      std::string rhs;
      switch (in.kind) {
        case IK::Signal: rhs = "s[" + std::to_string(in.index) + "]"; break;
        case IK::Lit: rhs = (!in.lit.empty() && (in.lit[0] & 1)) ? "~0ull" : "0ull"; break;
        case IK::Not: rhs = "~" + op(in.ops[0]); break;
        case IK::And: rhs = "(" + op(in.ops[0]) + " & " + op(in.ops[1]) + ")"; break;
        case IK::Or: rhs = "(" + op(in.ops[0]) + " | " + op(in.ops[1]) + ")"; break;
        case IK::Xor: rhs = "(" + op(in.ops[0]) + " ^ " + op(in.ops[1]) + ")"; break;
        case IK::Mux:
          rhs = "((" + op(in.ops[0]) + " & " + op(in.ops[1]) + ") | (~" + op(in.ops[0]) + " & " + op(in.ops[2]) + "))";
          break;
        default: rhs = "0ull"; break;
      }
      body += "  u64 " + op(v) + " = " + rhs + ";\n";
      emitted[v] = nfn;
      ++n;
    };
    for (auto& pk : b.packets) {
      for (auto& in : pk.instrs) def[in.dst] = &in;
      if (pk.effects.empty()) continue;
      for (auto& e : pk.effects) {
        if (e.kind == EffK::StoreSignal && !capture) {
          emit(e.value);
          body += "  s[" + std::to_string(e.dst) + "] = " + op(e.value) + ";\n";
        } else if (e.kind == EffK::CaptureReg && (capture || e.has_reset)) {
          emit(e.value);
          std::string v = op(e.value), nv = v;
          if (e.has_reset) {
            std::string a = "s[" + std::to_string(e.reset.signal) + "]";
            if (e.reset.active_low) a = "(~" + a + ")";
            const char* rv = (!e.reset.value.empty() && (e.reset.value[0] & 1)) ? "~0ull" : "0ull";
            nv = "((" + a + " & " + rv + ") | (~" + a + " & " + v + "))";
          }
          if (capture) {
            body += "  nx[" + std::to_string(caps.size()) + "] = " + nv + ";\n";
            caps.push_back(e.dst);
          } else {
            body += "  s[" + std::to_string(e.dst) + "] = " + nv + ";\n";  // asynchronous reset in a settle
          }
        } else {
          continue;
        }
        if (n >= kAotChunk) flush();
      }
      // next level: its values are new
      def.clear();
      emitted.clear();
    }
    flush();
  }
};

int orc_bp_emit_c(void* dp, const rrtl_stim* stim, uint32_t n_stim, const uint32_t* rec, uint32_t n_rec, char* out,
                  size_t cap, size_t* need) {
  auto* d = (OracleDesign*)dp;
  try {
    BitParallel probe(d, 64);  // scope check (1-bit gate-level, no memories)
    const MachineProgram& M = d->machine;
    const size_t ns = M.source.signals.size();
    AotEmitter em;
    em.block(M.async_reset_comb, "a", false);
    em.block(M.comb, "c", false);
    const size_t n_settle = em.calls.size();
    em.block(M.tick_next, "n", true);
    // several translation units (separated by a marker line) so the level
    // functions compile in parallel: the first holds run_bp, the others the
    // level functions
    const std::string head = "typedef unsigned long long u64;\ntypedef unsigned int u32;\n";
    std::string c = head;
    c += "static inline u64 sm(u64 z) { z += 0x9E3779B97F4A7C15ull; z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;\n"
         "  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull; return z ^ (z >> 31); }\n";
    c += "static inline u32 sw(u64 seed, u64 stream, u64 cycle, u64 idx) {\n"
         "  u64 k = sm(seed ^ (stream * 0xD6E8FEB86659FD93ull));\n"
         "  return (u32)sm(k ^ (cycle * 0xA0761D6478BD642Full) ^ (idx * 0xE7037ED1A0B428DBull)); }\n";
    c += "static inline u64 ht(u64 cycle, u32 rec, u64 idx, u32 v) {\n"
         "  u64 salt = sm((cycle << 20) ^ (u64)rec ^ 0x5851F42D4C957F2Dull); return sm((u64)v ^ (idx << 32) ^ salt); }\n";
    for (const std::string& call : em.calls)
      c += "void " + call.substr(0, call.find('(')) + "(u64* restrict s, u64* restrict nx);\n";
    c += "void run_bp(u64* restrict st, long groups, long g_base, long c0, long nc, u64 seed, u64* restrict hash) {\n";
    c += " u64 nx[" + std::to_string(std::max<size_t>(1, em.caps.size())) + "];\n";
    c += " for (long c = c0; c < c0 + nc; ++c) {\n  u64 h = 0;\n  for (long gi = 0; gi < groups; ++gi) {\n";
    c += "   u64* restrict s = st + gi * " + std::to_string(ns) + "L;\n   const u64 w0 = 2 * (u64)(g_base + gi);\n";
    for (uint32_t k = 0; k < n_stim; ++k) {
      const rrtl_stim& t = stim[k];
      std::string v;
      if (t.kind == RRTL_STIM_RANDOM)
        v = "((u64)sw(seed, " + std::to_string(t.param) + "ull, c, w0) | ((u64)sw(seed, " + std::to_string(t.param) +
            "ull, c, w0 + 1) << 32))";
      else if (t.kind == RRTL_STIM_RANDOM_UNIFORM)
        v = "((sw(seed, " + std::to_string(t.param) + "ull, c, 0) & 1u) ? ~0ull : 0ull)";
      else if (t.kind == RRTL_STIM_PULSE) v = "((u64)c < " + std::to_string(t.param) + "ull ? ~0ull : 0ull)";
      else if (t.kind == RRTL_STIM_CONST) v = (t.param & 1) ? "~0ull" : "0ull";
      else continue;
      c += "   s[" + std::to_string(t.signal) + "] = " + v + ";\n";
    }
    for (size_t i = 0; i < n_settle; ++i) c += "   " + em.calls[i] + "\n";
    for (uint32_t q = 0; q < n_rec; ++q) {
      const std::string sv = "s[" + std::to_string(rec[q]) + "]";
      c += "   h += ht(c, " + std::to_string(q) + "u, w0, (u32)" + sv + ") + ht(c, " + std::to_string(q) + "u, w0 + 1, (u32)(" +
           sv + " >> 32));\n";
    }
    for (size_t i = n_settle; i < em.calls.size(); ++i) c += "   " + em.calls[i] + "\n";
    for (size_t i = 0; i < em.caps.size(); ++i)
      c += "   s[" + std::to_string(em.caps[i]) + "] = nx[" + std::to_string(i) + "];\n";
    c += "  }\n  hash[c - c0] += h;\n }\n}\n";
    const size_t parts = std::min<size_t>(em.fns.size(), 32);
    for (size_t k = 0; k < parts; ++k) {
      c += "\n//@@PART@@\n" + head;
      for (size_t i = em.fns.size() * k / parts; i < em.fns.size() * (k + 1) / parts; ++i) c += em.fns[i];
    }
    if (need) *need = c.size() + 1;
    if (out && cap > c.size()) memcpy(out, c.c_str(), c.size() + 1);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return RRTL_E_DESIGN;
  }
}

void* orc_scalar_new(void* dp) {
  auto* d = (OracleDesign*)dp;
  try { return ScalarSim::create(&d->design, d->top); } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_scalar_free(void* s) { delete (ScalarSim*)s; }
int orc_scalar_id(void* sp, const char* name) {
  auto* s = (ScalarSim*)sp;
  for (auto& sig : s->m->signals)
    if (sig.name == name) return (int)sig.handle.id;
  return -1;
}
void orc_scalar_set(void* sp, uint32_t id, uint64_t lo, uint64_t hi, int settle) {
  auto* s = (ScalarSim*)sp;
  u128 v = ((u128)hi << 64) | lo;
  if (settle) s->set(id, v); else s->set_raw(id, v);
}
uint64_t orc_scalar_get(void* sp, uint32_t id, uint64_t* hi) {
  u128 v = ((ScalarSim*)sp)->get(id);
  if (hi) *hi = (uint64_t)(v >> 64);
  return (uint64_t)v;
}
void orc_scalar_tick(void* s) { ((ScalarSim*)s)->tick(); }
void orc_scalar_eval(void* s) { ((ScalarSim*)s)->eval_combinational(); }
uint64_t orc_scalar_peek_mem(void* sp, uint32_t id, uint64_t addr) {
  auto* s = (ScalarSim*)sp;
  auto it = s->mems.find(id);
  if (it == s->mems.end() || addr >= it->second.size()) return 0;
  return (uint64_t)it->second[addr];
}
void orc_scalar_poke_mem(void* sp, uint32_t id, uint64_t addr, uint64_t v) {
  auto* s = (ScalarSim*)sp;
  auto it = s->mems.find(id);
  if (it != s->mems.end() && addr < it->second.size()) it->second[addr] = v;
}

}  // extern "C"
