// Per-design compiled word kernels: emitter, NVRTC compile, load and launch.
//
// Each word instruction becomes one C++ statement on 64-bit locals (the value
// slots), in program order, with the interpreter's semantics
// (word_kernels.cu WordLane::run, which follows eval_machine_instr_lane,
// crates/rrtl-sim-ir/src/lib.rs:9796-9907): every result masked to its
// width, shifts of 64 or more giving 0, out-of-range memory reads giving 0
// and out-of-range writes dropped (:12989-13008, 9759-9775). Widths, shift
// amounts, literals and memory geometry are folded into the source as
// constants. Streams keep their own locals (the word lowering allocates
// slots per stream); register captures go to locals c<k> that the clock edge
// commits after the memory writes, as the interpreter's capture buffer does.
#include "word_jit.h"

#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <mutex>
#include <set>
#include <unordered_map>
#include <unordered_set>

// kJitHeaderCount, kJitHeaderNames, kJitHeaderTexts: the headers the
// generated source includes, embedded at build time.
#include "word_jit_headers.inc"

#ifndef RRTL_CUDA_LIB_DIR
#define RRTL_CUDA_LIB_DIR "/usr/local/cuda/lib64"
#endif

namespace rrtl {

namespace {

std::string hex(unsigned long long v) {
  char b[32];
  snprintf(b, sizeof b, "0x%llxull", v);
  return b;
}

unsigned long long wmask(uint32_t w) { return w >= 64u ? ~0ull : ((1ull << w) - 1ull); }

std::string u(uint64_t v) { return std::to_string(v) + "u"; }

struct Emitter {
  const WordProgram& wp;
  const WordRunTables* run = nullptr;
  const WordSplitPlan* split = nullptr;
  std::string o;

  const bool regs;  // signal words as register members s<k>

  explicit Emitter(const WordProgram& w) : wp(w), regs(w.n_sig_words <= kJitRegSignals) {}

  std::string sig(uint32_t off) const { return regs ? "s" + std::to_string(off) : "SV(" + u(off) + ")"; }

  static std::string V(uint32_t s) { return "v" + std::to_string(s); }

  std::string mem(uint32_t k, const std::string& w) const {
    if (k < kJitPlacedMems) return "MK(" + u(k) + ", " + w + ")";
    return "MG((size_t)" + u(wp.mems[k].offset) + " + " + w + ")";
  }
  std::string reset(uint32_t off, bool low) const {
    return "(((" + sig(off) + " & 1u) != 0u) != " + (low ? "true" : "false") + ")";
  }
  std::string store(uint32_t off, bool two, const std::string& t) const {
    std::string s = sig(off) + " = (uint32_t)" + t + ";";
    if (two) s += " " + sig(off + 1) + " = (uint32_t)(" + t + " >> 32);";
    return s;
  }

  void line(const std::string& s) {
    o += "    ";
    o += s;
    o += '\n';
  }

  // Bit width bound of each slot's current value within the block being
  // emitted (every result is masked to its width, compares give 1 bit).
  std::vector<uint32_t> vw;

  uint32_t W(uint32_t s) const { return s < vw.size() ? vw[s] : 64u; }

  void define(const WInstr& I) {
    uint32_t w = 0;
    switch (I.op) {
      case W_STORE:
      case W_ASTORE:
      case W_CAPTURE:
      case W_MEMWR: return;
      case W_EQ:
      case W_NE:
      case W_LT:
      case W_LTS: w = 1; break;
      case W_MEMRD: w = std::min<uint32_t>(I.width, wp.mems[I.aux].width); break;
      default: w = I.width; break;
    }
    if (I.dst + 1u >= vw.size()) vw.resize(I.dst + 2u, 64u);
    vw[I.dst] = std::min<uint32_t>(w, 64u);
    if (I.flags & kWPairD) vw[I.dst + 1u] = 64u;
  }

  // 32-bit form of an instruction whose result (and every operand bit it
  // depends on) fits 32 bits: the low k bits of a sum, difference, product or
  // bitwise result depend only on the operands' low k bits. Empty when the
  // 64-bit form is needed.
  std::string narrow(const WInstr& I) const {
    if (I.width > 32) return "";
    const std::string M = hex(wmask(I.width)).substr(0, hex(wmask(I.width)).size() - 3) + "u";
    auto n = [](uint32_t s) { return "(uint32_t)" + V(s); };
    const std::string d = V(I.dst) + " = (u64)(uint32_t)(";
    switch (I.op) {
      case W_NOT: return d + "~" + n(I.a) + " & " + M + ");";
      case W_AND: return d + "(" + n(I.a) + " & " + n(I.b) + ") & " + M + ");";
      case W_OR: return d + "(" + n(I.a) + " | " + n(I.b) + ") & " + M + ");";
      case W_XOR: return d + "(" + n(I.a) + " ^ " + n(I.b) + ") & " + M + ");";
      case W_ADD: return d + "(" + n(I.a) + " + " + n(I.b) + ") & " + M + ");";
      case W_SUB: return d + "(" + n(I.a) + " - " + n(I.b) + ") & " + M + ");";
      case W_MUL: return d + "(" + n(I.a) + " * " + n(I.b) + ") & " + M + ");";
      case W_MUX: return d + "((" + n(I.a) + " & 1u) ? " + n(I.b) + " : " + n(I.c) + ") & " + M + ");";
      case W_MASK: return d + n(I.a) + " & " + M + ");";
      case W_EQ:
      case W_NE:
        if (W(I.a) > 32 || W(I.b) > 32) return "";
        return d + n(I.a) + (I.op == W_EQ ? " == " : " != ") + n(I.b) + ");";
      case W_LT: {
        if (I.aux > 32) return "";
        const std::string om = hex(wmask(I.aux)).substr(0, hex(wmask(I.aux)).size() - 3) + "u";
        return d + "(" + n(I.a) + " & " + om + ") < (" + n(I.b) + " & " + om + "));";
      }
      case W_LTS: {
        if (I.aux == 0 || I.aux > 32) return "";
        const std::string om = hex(wmask(I.aux)).substr(0, hex(wmask(I.aux)).size() - 3) + "u";
        const std::string sb = u(1u << (I.aux - 1u));
        return "{ const uint32_t x = " + n(I.a) + " & " + om + ", y = " + n(I.b) + " & " + om +
               "; const bool xs = (x & " + sb + ") != 0u, ys = (y & " + sb + ") != 0u; " + V(I.dst) +
               " = (xs != ys) ? (u64)xs : (u64)(x < y); }";
      }
      case W_SLICE:
        if (I.aux >= 64u || I.aux + I.width > 32) return "";
        return d + "(" + n(I.a) + " >> " + u(I.aux) + ") & " + M + ");";
      case W_SEXT: {
        if (I.aux == 0 || I.aux > 32) return "";
        const unsigned long long wm = wmask(I.aux);
        const std::string wms = u((uint32_t)wm), nwm = u((uint32_t)~wm);
        return "{ const uint32_t x = " + n(I.a) + " & " + wms + "; " + V(I.dst) + " = (u64)(uint32_t)((((x >> " +
               u(I.aux - 1u) + ") & 1u) ? (x | " + nwm + ") : x) & " + M + "); }";
      }
      case W_CAT:
        if (I.aux >= 32u) return d + n(I.b) + " & " + M + ");";
        return d + "((" + n(I.a) + " << " + u(I.aux) + ") | " + n(I.b) + ") & " + M + ");";
      default: return "";
    }
  }

  // Statement for one wide instruction (kWWide): the same semantics on
  // 128-bit integers; a pair slot s holds bits 0-63 and s+1 bits 64-127.
  std::string wide_stmt(const WInstr& I) const {
    auto P = [&](uint32_t s, uint8_t bit) {
      return (I.flags & bit) ? "(((u128)" + V(s + 1) + " << 64) | (u128)" + V(s) + ")" : "(u128)" + V(s);
    };
    auto M2 = [](uint32_t w) {
      return w >= 128u ? std::string("(~(u128)0)") : "((((u128)1) << " + u(w) + ") - (u128)1)";
    };
    const std::string a = P(I.a, kWPairA), b = P(I.b, kWPairB), c = P(I.c, kWPairC), m = M2(I.width);
    auto set = [&](const std::string& e) {
      if (I.flags & kWPairD)
        return "{ const u128 t = " + e + "; " + V(I.dst) + " = (u64)t; " + V(I.dst + 1) + " = (u64)(t >> 64); }";
      return V(I.dst) + " = (u64)(" + e + ");";
    };
    auto load_sig = [&](uint32_t off, uint32_t limbs) {
      std::string s = "((u128)0";
      for (uint32_t l = 0; l < limbs; ++l) s += " | ((u128)" + sig(off + l) + " << " + u(32 * l) + ")";
      return s + ")";
    };
    auto store_sig = [&](uint32_t off, uint32_t limbs, const std::string& t) {
      std::string s;
      for (uint32_t l = 0; l < limbs; ++l) s += sig(off + l) + " = (uint32_t)(" + t + " >> " + u(32 * l) + "); ";
      return s;
    };
    // decode_usize: an address past 64 bits saturates
    auto addr = [](const std::string& x) { return "(((" + x + ") >> 64) != 0 ? ~0ull : (u64)(" + x + "))"; };
    switch (I.op) {
      case W_LIT: {
        char buf[96];
        snprintf(buf, sizeof buf, "((((u128)0x%llxull) << 64) | (u128)0x%llxull)", wp.lits[I.aux + 1], wp.lits[I.aux]);
        return set(std::string(buf) + " & " + m);
      }
      case W_SIG: return set(load_sig(I.aux, I.c) + " & " + m);
      case W_NOT: return set("~" + a + " & " + m);
      case W_AND: return set("(" + a + " & " + b + ") & " + m);
      case W_OR: return set("(" + a + " | " + b + ") & " + m);
      case W_XOR: return set("(" + a + " ^ " + b + ") & " + m);
      case W_ADD: return set("(" + a + " + " + b + ") & " + m);
      case W_SUB: return set("(" + a + " - " + b + ") & " + m);
      case W_MUL: return set("(" + a + " * " + b + ") & " + m);
      case W_EQ: return set("(u128)(" + a + " == " + b + ")");
      case W_NE: return set("(u128)(" + a + " != " + b + ")");
      case W_LT: return set("(u128)((" + a + " & " + M2(I.aux) + ") < (" + b + " & " + M2(I.aux) + "))");
      case W_LTS: {
        if (I.aux == 0) return set("(u128)0");
        const std::string om = M2(I.aux), sb = "(((u128)1) << " + u(I.aux - 1u) + ")";
        return "{ const u128 x = " + a + " & " + om + ", y = " + b + " & " + om + "; const bool xs = (x & " + sb +
               ") != 0, ys = (y & " + sb + ") != 0; " + set("(xs != ys) ? (u128)xs : (u128)(x < y)") + " }";
      }
      case W_MUX: return set("(((u64)" + a + " & 1ull) ? " + b + " : " + c + ") & " + m);
      case W_SLICE:
        if (I.aux >= 128u) return set("(u128)0");
        return set("(" + a + " >> " + u(I.aux) + ") & " + m);
      case W_MASK: return set(a + " & " + m);
      case W_SEXT: {
        if (I.aux == 0) return set("(u128)0");
        const std::string wm = M2(I.aux);
        return "{ const u128 x = " + a + " & " + wm + "; " +
               set("((((x >> " + u(I.aux - 1u) + ") & (u128)1) != 0) ? (x | ~" + wm + ") : x) & " + m) + " }";
      }
      case W_CAT:
        if (I.aux >= 128u) return set(b + " & " + m);
        return set("((" + a + " << " + u(I.aux) + ") | " + b + ") & " + m);
      case W_MEMRD: {
        const WMemDev& Md = wp.mems[I.aux];
        std::string s = "{ const u64 ad = " + addr(a) + "; u128 r = 0; if (ad < " + hex(Md.depth) +
                        ") { const size_t w0 = (size_t)ad * " + u(Md.limbs) + ";";
        for (uint32_t l = 0; l < Md.limbs; ++l)
          s += " r |= (u128)" + mem(I.aux, "w0 + " + u(l)) + " << " + u(32 * l) + ";";
        s += " r &= " + M2(Md.width) + " & " + m + "; } " + set("r") + " }";
        return s;
      }
      case W_STORE: return "{ const u128 t = " + a + " & " + m + "; " + store_sig(I.aux, I.c, "t") + "}";
      case W_ASTORE:
        return "if (" + reset(I.aux2, I.flags & 4) + ") { const u128 t = " + a + " & " + m + "; " +
               store_sig(I.aux, I.c, "t") + "}";
      case W_CAPTURE: {
        std::string t = a;
        if (I.flags & 2) {
          char buf[96];
          snprintf(buf, sizeof buf, "((((u128)0x%llxull) << 64) | (u128)0x%llxull)", wp.lits[I.aux3 + 1],
                   wp.lits[I.aux3]);
          t = "(" + reset(I.aux2, I.flags & 4) + " ? " + std::string(buf) + " : " + a + ")";
        }
        std::string s = "{ const u128 t = " + t + " & " + m + ";";
        for (uint32_t l = 0; l < I.c; ++l)
          s += " c" + std::to_string(I.aux + l) + " = (uint32_t)(t >> " + u(32 * l) + ");";
        return s + " }";
      }
      case W_MEMWR: {
        const WMemDev& Md = wp.mems[I.aux];
        std::string s = "if ((u64)" + a + " & 1ull) { const u64 ad = " + addr(b) + "; if (ad < " + hex(Md.depth) +
                        ") { const u128 t = " + c + " & " + M2(Md.width) + "; const size_t w0 = (size_t)ad * " +
                        u(Md.limbs) + ";";
        for (uint32_t l = 0; l < Md.limbs; ++l)
          s += " " + mem(I.aux, "w0 + " + u(l)) + " = (uint32_t)(t >> " + u(32 * l) + ");";
        return s + " } }";
      }
      default: return "";
    }
  }

  // Statement for one instruction (empty for opcodes the interpreter skips).
  std::string stmt(const WInstr& I) const {
    if (I.flags & kWWide) return wide_stmt(I);
    {
      std::string s = narrow(I);
      if (!s.empty()) return s;
    }
    const unsigned long long m = wmask(I.width);
    const std::string M = hex(m);
    const std::string d = V(I.dst), a = V(I.a), b = V(I.b), c = V(I.c);
    const bool two = I.flags & 1;
    switch (I.op) {
      case W_LIT: return d + " = " + hex(wp.lits[I.aux] & m) + ";";
      case W_SIG: {
        std::string s = "(u64)" + sig(I.aux);
        if (two) s = "(" + s + " | ((u64)" + sig(I.aux + 1) + " << 32))";
        return d + " = " + s + " & " + M + ";";
      }
      case W_NOT: return d + " = ~" + a + " & " + M + ";";
      case W_AND: return d + " = (" + a + " & " + b + ") & " + M + ";";
      case W_OR: return d + " = (" + a + " | " + b + ") & " + M + ";";
      case W_XOR: return d + " = (" + a + " ^ " + b + ") & " + M + ";";
      case W_ADD: return d + " = (" + a + " + " + b + ") & " + M + ";";
      case W_SUB: return d + " = (" + a + " - " + b + ") & " + M + ";";
      case W_MUL: return d + " = (" + a + " * " + b + ") & " + M + ";";
      case W_EQ: return d + " = (u64)(" + a + " == " + b + ");";
      case W_NE: return d + " = (u64)(" + a + " != " + b + ");";
      case W_LT: {
        const std::string om = hex(wmask(I.aux));
        return d + " = (u64)((" + a + " & " + om + ") < (" + b + " & " + om + "));";
      }
      case W_LTS: {
        // operand width 0 compares zeros; past 64 bits there is no sign bit
        if (I.aux == 0) return d + " = 0ull;";
        const std::string om = hex(wmask(I.aux));
        if (I.aux > 64) return d + " = (u64)((" + a + " & " + om + ") < (" + b + " & " + om + "));";
        const std::string sb = hex(1ull << (I.aux - 1u));
        return "{ const u64 x = " + a + " & " + om + ", y = " + b + " & " + om + "; const bool xs = (x & " + sb +
               ") != 0ull, ys = (y & " + sb + ") != 0ull; " + d + " = (xs != ys) ? (u64)xs : (u64)(x < y); }";
      }
      case W_MUX: return d + " = ((" + a + " & 1ull) ? " + b + " : " + c + ") & " + M + ";";
      case W_SLICE:
        if (I.aux >= 64u) return d + " = 0ull;";
        return d + " = (" + a + " >> " + u(I.aux) + ") & " + M + ";";
      case W_MASK: return d + " = " + a + " & " + M + ";";
      case W_SEXT: {
        if (I.aux == 0) return d + " = 0ull;";
        if (I.aux >= 64) return d + " = " + a + " & " + M + ";";
        const std::string wm = hex(wmask(I.aux)), nwm = hex(~wmask(I.aux));
        return "{ const u64 x = " + a + " & " + wm + "; " + d + " = (((x >> " + u(I.aux - 1u) + ") & 1ull) ? (x | " + nwm +
               ") : x) & " + M + "; }";
      }
      case W_CAT:
        if (I.aux >= 64u) return d + " = " + b + " & " + M + ";";
        return d + " = ((" + a + " << " + u(I.aux) + ") | " + b + ") & " + M + ";";
      case W_MEMRD: {
        const WMemDev& Md = wp.mems[I.aux];
        std::string s = "{ const u64 ad = " + a + "; u64 r = 0ull; if (ad < " + hex(Md.depth) +
                        ") { const size_t w0 = (size_t)ad * " + u(Md.limbs) + "; r = (u64)" + mem(I.aux, "w0") + ";";
        if (Md.limbs == 2) s += " r |= (u64)" + mem(I.aux, "w0 + 1u") + " << 32;";
        s += " r &= " + hex(wmask(Md.width) & m) + "; } " + d + " = r; }";
        return s;
      }
      case W_STORE: return "{ const u64 t = " + a + " & " + M + "; " + store(I.aux, two, "t") + " }";
      case W_ASTORE:
        return "if (" + reset(I.aux2, I.flags & 4) + ") { const u64 t = " + a + " & " + M + "; " + store(I.aux, two, "t") +
               " }";
      case W_CAPTURE: {
        std::string t = a;
        if (I.flags & 2) t = "(" + reset(I.aux2, I.flags & 4) + " ? " + hex(wp.lits[I.aux3]) + " : " + a + ")";
        std::string s = "{ const u64 t = " + t + " & " + M + "; c" + std::to_string(I.aux) + " = (uint32_t)t;";
        if (two) s += " c" + std::to_string(I.aux + 1) + " = (uint32_t)(t >> 32);";
        return s + " }";
      }
      case W_MEMWR: {
        const WMemDev& Md = wp.mems[I.aux];
        std::string s = "if (" + a + " & 1ull) { const u64 ad = " + b + "; if (ad < " + hex(Md.depth) + ") { const u64 t = " +
                        c + " & " + hex(wmask(Md.width)) + "; const size_t w0 = (size_t)ad * " + u(Md.limbs) + "; " +
                        mem(I.aux, "w0") + " = (uint32_t)t;";
        if (Md.limbs == 2) s += " " + mem(I.aux, "w0 + 1u") + " = (uint32_t)(t >> 32);";
        return s + " } }";
      }
      default: return "";
    }
  }

  static void uses(const WInstr& I, std::set<uint32_t>& s) {
    if (I.flags & kWWide) {
      // wide instructions: the slots the opcode uses, and the second slot of every pair
      switch (I.op) {
        case W_LIT: case W_SIG: break;
        case W_NOT: case W_SLICE: case W_MASK: case W_SEXT: case W_MEMRD: s.insert(I.a); break;
        case W_MUX: case W_MEMWR: s.insert(I.a); s.insert(I.b); s.insert(I.c); break;
        case W_STORE: case W_ASTORE: case W_CAPTURE: s.insert(I.a); break;
        default: s.insert(I.a); s.insert(I.b); break;
      }
      if (I.op != W_STORE && I.op != W_ASTORE && I.op != W_CAPTURE && I.op != W_MEMWR) s.insert(I.dst);
      if (I.flags & kWPairA) s.insert(I.a + 1u);
      if (I.flags & kWPairB) s.insert(I.b + 1u);
      if (I.flags & kWPairC) s.insert(I.c + 1u);
      if (I.flags & kWPairD) s.insert(I.dst + 1u);
      return;
    }
    switch (I.op) {
      case W_LIT:
      case W_SIG: s.insert(I.dst); break;
      case W_NOT:
      case W_SLICE:
      case W_MASK:
      case W_SEXT:
      case W_MEMRD: s.insert(I.dst); s.insert(I.a); break;
      case W_MUX: s.insert(I.dst); s.insert(I.a); s.insert(I.b); s.insert(I.c); break;
      case W_STORE:
      case W_ASTORE:
      case W_CAPTURE: s.insert(I.a); break;
      case W_MEMWR: s.insert(I.a); s.insert(I.b); s.insert(I.c); break;
      default: s.insert(I.dst); s.insert(I.a); s.insert(I.b); break;
    }
  }

  // One stream in its own scope with its own slot locals.
  void block(uint32_t b, uint32_t e, const char* what, const std::vector<uint8_t>* mask = nullptr) {
    if (b == e) return;
    std::set<uint32_t> slots;
    for (uint32_t pc = b; pc < e; ++pc)
      if (!mask || (*mask)[pc]) uses(wp.code[pc], slots);
    o += "  {  // ";
    o += what;
    o += '\n';
    if (!slots.empty()) {
      std::string decl = "u64";
      bool first = true;
      for (uint32_t s : slots) {
        decl += (first ? " " : ", ") + V(s) + " = 0ull";
        first = false;
      }
      line(decl + ";");
    }
    vw.assign(slots.empty() ? 0 : *slots.rbegin() + 1, 64u);
    for (uint32_t pc = b; pc < e; ++pc) {
      if (mask && !(*mask)[pc]) continue;
      std::string s = stmt(wp.code[pc]);
      if (!s.empty()) line(s);
      define(wp.code[pc]);
    }
    o += "  }\n";
  }

  std::string source() {
    const bool big = wp.code.size() > 4000;  // keep one copy of large settle bodies
    o += "// Compiled word kernel (generated from the design's word program).\n";
    o += "#include \"word_lane.h\"\n";
    o += "namespace rrtl {\n";
    o += "typedef unsigned long long u64;\n";
    o += "typedef unsigned __int128 u128;\n";
    o += "struct JitLane : JitLaneBase {\n";
    if (regs && wp.n_sig_words) {
      const uint32_t n = wp.n_sig_words;
      o += "  static constexpr bool kRegSignals = true;\n";
      std::string decl = "  uint32_t";
      for (uint32_t k = 0; k < n; ++k) decl += (k ? ", s" : " s") + std::to_string(k);
      o += decl + ";\n";
      o += "  __device__ __forceinline__ uint32_t get(uint32_t off) const {\n    switch (off) {\n";
      for (uint32_t k = 0; k < n; ++k) o += "      case " + u(k) + ": return s" + std::to_string(k) + ";\n";
      o += "      default: return 0u;\n    }\n  }\n";
      o += "  __device__ __forceinline__ void set(uint32_t off, uint32_t v) {\n    switch (off) {\n";
      for (uint32_t k = 0; k < n; ++k) o += "      case " + u(k) + ": s" + std::to_string(k) + " = v; break;\n";
      o += "      default: break;\n    }\n  }\n";
      o += "  __device__ __forceinline__ void load(const uint32_t* g, size_t lp) {\n";
      for (uint32_t k = 0; k < n; ++k) o += "    s" + std::to_string(k) + " = g[" + u(k) + " * lp];\n";
      o += "  }\n";
      o += "  __device__ __forceinline__ void store(uint32_t* g, size_t lp) const {\n";
      for (uint32_t k = 0; k < n; ++k) o += "    g[" + u(k) + " * lp] = s" + std::to_string(k) + ";\n";
      o += "  }\n";
    }
    o += "  __device__ void settle();\n";
    o += "  __device__ void edge();\n";
    if (split) {
      o += "  __device__ void settle_part(uint32_t p);\n";
      o += "  __device__ void edge_part(uint32_t p);\n";
      for (const char* fn : {"xout", "xin"}) {
        o += std::string("  __device__ __forceinline__ void ") + fn + "(uint32_t p, uint32_t* X, uint32_t lid) {\n";
        for (int q = 0; q < 2; ++q) {
          o += std::string(q ? "    else {\n" : "    if (p == 0u) {\n");
          for (size_t x = 0; x < split->xwords.size(); ++x) {
            const std::string cell = "X[" + u(x) + " * 32u + lid]";
            const std::string sv = "s" + std::to_string(split->xwords[x]);
            if (fn[1] == 'o' && split->owner[x] == q) o += "      " + cell + " = " + sv + ";\n";
            if (fn[1] == 'i' && split->need[q][x]) o += "      " + sv + " = " + cell + ";\n";
          }
          o += "    }\n";
        }
        o += "  }\n";
      }
      o += "  __device__ __forceinline__ void xin_all(uint32_t* X, uint32_t lid) {\n";
      for (size_t x = 0; x < split->xwords.size(); ++x)
        if (split->owner[x] != 0) o += "    s" + std::to_string(split->xwords[x]) + " = X[" + u(x) + " * 32u + lid];\n";
      o += "  }\n";
    }
    o += "};\n";
    o += std::string(big ? "__device__ __noinline__" : "__device__ __forceinline__") + " void JitLane::settle() {\n";
    block(wp.comb_b, wp.comb_e, "comb");
    block(wp.async_b, wp.async_e, "async reset");
    o += "}\n";
    o += "__device__ __forceinline__ void JitLane::edge() {\n";
    if (wp.total_capture_words) {
      std::string decl = "  uint32_t";
      for (uint32_t k = 0; k < wp.total_capture_words; ++k) decl += (k ? ", c" : " c") + std::to_string(k) + " = 0u";
      o += decl + ";\n";
    }
    block(wp.next_b, wp.next_e, "tick_next: register captures");
    block(wp.commit_b, wp.commit_e, "tick_commit: memory writes");
    for (const WCommitDev& cm : wp.commits)
      for (uint32_t l = 0; l < cm.limbs; ++l)
        o += "  " + sig(cm.sig_off + l) + " = c" + std::to_string(cm.cap_off + l) + ";\n";
    o += "}\n";
    if (split) {
      o += "__device__ __forceinline__ void JitLane::settle_part(uint32_t p) {\n";
      for (int q = 0; q < 2; ++q) {
        o += std::string(q ? "  else {\n" : "  if (p == 0u) {\n");
        block(wp.comb_b, wp.comb_e, "comb, this warp's cones", &split->in[q]);
        o += "  }\n";
      }
      o += "}\n";
      o += "__device__ __forceinline__ void JitLane::edge_part(uint32_t p) {\n";
      for (int q = 0; q < 2; ++q) {
        o += std::string(q ? "  else {\n" : "  if (p == 0u) {\n");
        if (wp.total_capture_words) {
          std::string decl = "  uint32_t";
          for (uint32_t k = 0; k < wp.total_capture_words; ++k) decl += (k ? ", c" : " c") + std::to_string(k) + " = 0u";
          o += decl + ";\n";
        }
        block(wp.next_b, wp.next_e, "tick_next: this warp's captures", &split->in[q]);
        block(wp.commit_b, wp.commit_e, "tick_commit: this warp's memory writes", &split->in[q]);
        for (size_t k = 0; k < wp.commits.size(); ++k) {
          if (split->commit_owner[k] != q) continue;
          const WCommitDev& cm = wp.commits[k];
          for (uint32_t l = 0; l < cm.limbs; ++l)
            o += "  " + sig(cm.sig_off + l) + " = c" + std::to_string(cm.cap_off + l) + ";\n";
        }
        o += "  }\n";
      }
      o += "}\n";
    }
    o += "}  // namespace rrtl\n";
    if (run) {
      // this run's tables as compile-time constants
      o += "namespace rrtl {\n";
      o += "struct RunSpec {\n";
      o += "  __device__ __forceinline__ static constexpr uint32_t n_stim() { return " + u(run->stim.size()) + "; }\n";
      o += "  __device__ __forceinline__ static constexpr WordStimDev stim(uint32_t k) {\n    switch (k) {\n";
      for (size_t k = 0; k < run->stim.size(); ++k) {
        const WordStimDev& t = run->stim[k];
        o += "      case " + u(k) + ": return WordStimDev{" + u(t.sig_off) + ", " + u(t.limbs) + ", " + u(t.width) + ", " +
             u(t.kind) + ", " + hex(t.param) + "};\n";
      }
      o += "      default: return WordStimDev{0u, 0u, 0u, 0u, 0ull};\n    }\n  }\n";
      o += "  __device__ __forceinline__ static constexpr uint32_t n_rec() { return " + u(run->rec.size()) + "; }\n";
      o += "  __device__ __forceinline__ static constexpr WordRecDev rec(uint32_t k) {\n    switch (k) {\n";
      for (size_t k = 0; k < run->rec.size(); ++k) {
        const WordRecDev& t = run->rec[k];
        o += "      case " + u(k) + ": return WordRecDev{" + u(t.sig_off) + ", " + u(t.limbs) + ", " + u(t.width) + ", " +
             u(t.base) + "};\n";
      }
      o += "      default: return WordRecDev{0u, 0u, 0u, 0u};\n    }\n  }\n";
      o += "  __device__ __forceinline__ static constexpr uint32_t mode() { return " + u(run->mode) + "; }\n";
      o += "};\n}  // namespace rrtl\n";
    }
    o += std::string("extern \"C\" __global__ void __launch_bounds__(") + (split ? "64" : "128") +
         ") rrtl_word_jit(const rrtl::WordRunDev R, "
         "const rrtl::WordJitPlace Pl) {\n";
    o += "  extern __shared__ uint32_t rrtl_jsm[];\n";
    if (run && split) {
      o += "  rrtl::word_jit_run_split<rrtl::JitLane>(R, Pl, rrtl_jsm, rrtl::RunSpec{});\n";
    } else if (run) {
      o += "  rrtl::word_jit_run<rrtl::JitLane>(R, Pl, rrtl_jsm, rrtl::RunSpec{});\n";
    } else {
      o += "  __shared__ rrtl::JitDynamicRun tables;\n";
      o += "  const rrtl::WordRunSpec spec = tables.load(R);\n";
      o += "  rrtl::word_jit_run<rrtl::JitLane>(R, Pl, rrtl_jsm, spec);\n";
    }
    o += "}\n";
    return o;
  }
};

// ---- NVRTC, opened at run time so the library loads without it
struct Nvrtc {
  bool ok = false;
  std::string error;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) get_log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) get_cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcGetErrorString) err_str = nullptr;

  Nvrtc() {
    void* h = nullptr;
    for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", RRTL_CUDA_LIB_DIR "/libnvrtc.so.13",
                             RRTL_CUDA_LIB_DIR "/libnvrtc.so"}) {
      h = dlopen(name, RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) {
      const char* e = dlerror();
      error = std::string("NVRTC not found: ") + (e ? e : "dlopen failed");
      return;
    }
    create = reinterpret_cast<decltype(create)>(dlsym(h, "nvrtcCreateProgram"));
    compile = reinterpret_cast<decltype(compile)>(dlsym(h, "nvrtcCompileProgram"));
    log_size = reinterpret_cast<decltype(log_size)>(dlsym(h, "nvrtcGetProgramLogSize"));
    get_log = reinterpret_cast<decltype(get_log)>(dlsym(h, "nvrtcGetProgramLog"));
    cubin_size = reinterpret_cast<decltype(cubin_size)>(dlsym(h, "nvrtcGetCUBINSize"));
    get_cubin = reinterpret_cast<decltype(get_cubin)>(dlsym(h, "nvrtcGetCUBIN"));
    destroy = reinterpret_cast<decltype(destroy)>(dlsym(h, "nvrtcDestroyProgram"));
    err_str = reinterpret_cast<decltype(err_str)>(dlsym(h, "nvrtcGetErrorString"));
    ok = create && compile && log_size && get_log && cubin_size && get_cubin && destroy && err_str;
    if (!ok) error = "NVRTC library lacks an entry point";
  }
};

Nvrtc& nvrtc() {
  static Nvrtc n;
  return n;
}

}  // namespace

JitKernel::~JitKernel() {
  if (lib) cudaLibraryUnload(lib);
}

std::string word_jit_source(const WordProgram& wp, const WordRunTables* run, const WordSplitPlan* split) {
  Emitter e(wp);
  e.run = run;
  e.split = run ? split : nullptr;
  return e.source();
}

bool word_split_plan(const WordProgram& wp, const WordRunTables& run, WordSplitPlan* sp, std::string* why) {
  auto no = [&](const char* w) {
    if (why) *why = w;
    return false;
  };
  if (wp.async_b != wp.async_e) return no("asynchronous resets");
  if (wp.n_sig_words > kJitRegSignals || wp.code.size() > kJitMaxInstrs) return no("too large");
  for (const WInstr& I : wp.code)
    if (I.flags & kWWide) return no("values wider than 64 bits");
  const size_t N = wp.code.size();
  std::vector<std::vector<uint32_t>> dep(N);
  std::unordered_map<uint32_t, uint32_t> sig_def;  // signal word -> the comb store that defines it this cycle
  std::unordered_set<uint32_t> read_before_store;
  auto walk = [&](uint32_t b, uint32_t e, bool comb) {
    std::unordered_map<uint32_t, uint32_t> slot_def;
    for (uint32_t pc = b; pc < e; ++pc) {
      const WInstr& I = wp.code[pc];
      auto use = [&](uint32_t sl) {
        auto it = slot_def.find(sl);
        if (it != slot_def.end()) dep[pc].push_back(it->second);
      };
      auto usesig = [&](uint32_t off) {
        auto it = sig_def.find(off);
        if (it != sig_def.end()) dep[pc].push_back(it->second);
        else if (comb) read_before_store.insert(off);
      };
      switch (I.op) {
        case W_LIT: break;
        case W_SIG: usesig(I.aux); if (I.flags & 1) usesig(I.aux + 1); break;
        case W_NOT: case W_SLICE: case W_MASK: case W_SEXT: case W_MEMRD: use(I.a); break;
        case W_MUX: use(I.a); use(I.b); use(I.c); break;
        case W_STORE: use(I.a); break;
        case W_ASTORE: use(I.a); usesig(I.aux2); break;
        case W_CAPTURE: use(I.a); if (I.flags & 2) usesig(I.aux2); break;
        case W_MEMWR: use(I.a); use(I.b); use(I.c); break;
        default: use(I.a); use(I.b); break;
      }
      if (I.op == W_STORE) {
        // a word the cycle reads before it stores it feeds back: not split
        if (read_before_store.count(I.aux) || ((I.flags & 1) && read_before_store.count(I.aux + 1))) {
          sig_def.clear();
          read_before_store.insert(0xFFFFFFFFu);
        }
        sig_def[I.aux] = pc;
        if (I.flags & 1) sig_def[I.aux + 1] = pc;
      } else if (I.op != W_CAPTURE && I.op != W_MEMWR && I.op != W_ASTORE) {
        slot_def[I.dst] = pc;
      }
    }
  };
  walk(wp.comb_b, wp.comb_e, true);
  if (read_before_store.count(0xFFFFFFFFu)) return no("combinational feedback");
  walk(wp.next_b, wp.next_e, false);
  walk(wp.commit_b, wp.commit_e, false);
  auto cone = [&](uint32_t root) {
    std::vector<uint32_t> out, st{root};
    std::vector<uint8_t> seen(N, 0);
    while (!st.empty()) {
      const uint32_t x = st.back();
      st.pop_back();
      if (seen[x]) continue;
      seen[x] = 1;
      out.push_back(x);
      for (uint32_t y : dep[x]) st.push_back(y);
    }
    return out;
  };
  sp->in[0].assign(N, 0);
  sp->in[1].assign(N, 0);
  size_t size[2] = {0, 0};
  auto add = [&](int p, const std::vector<uint32_t>& c) {
    for (uint32_t x : c)
      if (!sp->in[p][x]) {
        sp->in[p][x] = 1;
        ++size[p];
      }
  };
  // what the record stage reads is computed by warp 0
  for (const WordRecDev& r : run.rec)
    for (uint32_t l = 0; l < r.limbs; ++l) {
      auto it = sig_def.find(r.sig_off + l);
      if (it != sig_def.end()) add(0, cone(it->second));
    }
  std::vector<std::pair<size_t, uint32_t>> sinks;
  std::vector<std::vector<uint32_t>> cones(N);
  for (uint32_t pc = wp.next_b; pc < wp.commit_e; ++pc)
    if (wp.code[pc].op == W_CAPTURE || wp.code[pc].op == W_MEMWR) {
      cones[pc] = cone(pc);
      sinks.push_back({cones[pc].size(), pc});
    }
  std::sort(sinks.begin(), sinks.end(), [](const std::pair<size_t, uint32_t>& a, const std::pair<size_t, uint32_t>& b) {
    return a.first != b.first ? a.first > b.first : a.second < b.second;
  });
  std::vector<int8_t> sink_part(N, -1);
  for (auto& sk : sinks) {
    size_t grow[2] = {0, 0};
    for (int p = 0; p < 2; ++p)
      for (uint32_t x : cones[sk.second]) grow[p] += !sp->in[p][x];
    const int p = size[0] + grow[0] <= size[1] + grow[1] ? 0 : 1;
    add(p, cones[sk.second]);
    sink_part[sk.second] = (int8_t)p;
  }
  const size_t total = (wp.comb_e - wp.comb_b) + (wp.commit_e - wp.next_b);
  sp->sizes[0] = size[0];
  sp->sizes[1] = size[1];
  if (size[1] == 0 || (double)std::max(size[0], size[1]) > 0.75 * (double)total) return no("unbalanced");
  // memory reads in the register or commit stream run after the first
  // barrier, beside the other warp's memory writes: a memory read there by
  // one warp must not be written by the other (the single warp reads first)
  std::vector<uint8_t> writer(wp.mems.size(), 0);  // bit p: warp p writes memory k
  for (uint32_t pc = wp.commit_b; pc < wp.commit_e; ++pc)
    if (wp.code[pc].op == W_MEMWR && wp.code[pc].aux < writer.size())
      for (int p = 0; p < 2; ++p)
        if (sp->in[p][pc]) writer[wp.code[pc].aux] |= (uint8_t)(1u << p);
  for (uint32_t pc = wp.next_b; pc < wp.commit_e; ++pc) {
    const WInstr& I = wp.code[pc];
    if (I.op != W_MEMRD || I.aux >= writer.size()) continue;
    for (int p = 0; p < 2; ++p)
      if (sp->in[p][pc] && (writer[I.aux] & (1u << (1 - p)))) return no("a register-stream memory read races the other warp's write");
  }
  // register words: owned by the warp that captures them
  std::unordered_map<uint32_t, uint32_t> cap_instr;
  for (uint32_t pc = wp.next_b; pc < wp.next_e; ++pc)
    if (wp.code[pc].op == W_CAPTURE) {
      cap_instr[wp.code[pc].aux] = pc;
      if (wp.code[pc].flags & 1) cap_instr[wp.code[pc].aux + 1] = pc;
    }
  std::unordered_map<uint32_t, uint32_t> xindex;
  sp->commit_owner.clear();
  for (const WCommitDev& cm : wp.commits) {
    auto it = cap_instr.find(cm.cap_off);
    if (it == cap_instr.end() || sink_part[it->second] < 0) return no("register without a capture");
    const uint8_t own = (uint8_t)sink_part[it->second];
    sp->commit_owner.push_back(own);
    for (uint32_t l = 0; l < cm.limbs; ++l) {
      xindex[cm.sig_off + l] = (uint32_t)sp->xwords.size();
      sp->xwords.push_back(cm.sig_off + l);
      sp->owner.push_back(own);
    }
  }
  sp->need[0].assign(sp->xwords.size(), 0);
  sp->need[1].assign(sp->xwords.size(), 0);
  auto needs = [&](int p, uint32_t word) {
    auto it = xindex.find(word);
    if (it != xindex.end() && sp->owner[it->second] != p) sp->need[p][it->second] = 1;
  };
  for (int p = 0; p < 2; ++p)
    for (uint32_t pc = 0; pc < N; ++pc) {
      if (!sp->in[p][pc]) continue;
      const WInstr& I = wp.code[pc];
      if (I.op == W_SIG) {
        needs(p, I.aux);
        if (I.flags & 1) needs(p, I.aux + 1);
      }
      if ((I.op == W_CAPTURE && (I.flags & 2)) || I.op == W_ASTORE) needs(p, I.aux2);
    }
  for (const WordRecDev& r : run.rec)
    for (uint32_t l = 0; l < r.limbs; ++l) needs(0, r.sig_off + l);
  return true;
}

std::string WordRunTables::key() const {
  std::string k = std::to_string(mode) + "|";
  for (const WordStimDev& t : stim)
    k += std::to_string(t.sig_off) + "," + std::to_string(t.limbs) + "," + std::to_string(t.width) + "," +
         std::to_string(t.kind) + "," + std::to_string(t.param) + ";";
  k += "|";
  for (const WordRecDev& t : rec)
    k += std::to_string(t.sig_off) + "," + std::to_string(t.limbs) + "," + std::to_string(t.width) + "," +
         std::to_string(t.base) + ";";
  return k;
}

std::vector<char> word_jit_compile(const std::string& src, const std::string& arch, std::string* log) {
  Nvrtc& N = nvrtc();
  if (!N.ok) {
    *log = N.error;
    return {};
  }
  nvrtcProgram prog = nullptr;
  nvrtcResult r = N.create(&prog, src.c_str(), "rrtl_word_jit.cu", kJitHeaderCount, kJitHeaderTexts, kJitHeaderNames);
  if (r != NVRTC_SUCCESS) {
    *log = std::string("nvrtcCreateProgram: ") + N.err_str(r);
    return {};
  }
  const std::string arch_opt = "--gpu-architecture=" + arch;
  // -default-device: the C ABI header's host prototypes become inert device declarations
  // --device-int128: values of 65 to 128 bits compute on unsigned __int128
  const char* opts[] = {arch_opt.c_str(), "-std=c++17", "-default-device", "--device-int128"};
  r = N.compile(prog, 4, opts);
  size_t ls = 0;
  N.log_size(prog, &ls);
  std::string lg(ls, '\0');
  if (ls) N.get_log(prog, &lg[0]);
  *log = lg;
  std::vector<char> cubin;
  if (r == NVRTC_SUCCESS) {
    size_t n = 0;
    if (N.cubin_size(prog, &n) == NVRTC_SUCCESS && n) {
      cubin.resize(n);
      if (N.get_cubin(prog, cubin.data()) != NVRTC_SUCCESS) cubin.clear();
    }
  } else {
    *log = std::string("nvrtcCompileProgram: ") + N.err_str(r) + "\n" + lg;
  }
  N.destroy(&prog);
  return cubin;
}

void jit_warm() {
  static std::once_flag once;
  std::call_once(once, [] {
    std::string log;
    word_jit_compile("extern \"C\" __global__ void rrtl_warm() {}\n", "sm_103a", &log);
  });
}

void jit_build_kernel(const std::string& src, int device, const char* name, JitKernel* J) {
  const auto t0 = std::chrono::steady_clock::now();
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    J->error = "cudaGetDeviceProperties failed";
    return;
  }
  const std::string arch = "sm_" + std::to_string(prop.major) + std::to_string(prop.minor) + "a";
  J->source_bytes = src.size();
  std::string log;
  std::vector<char> cubin = word_jit_compile(src, arch, &log);
  if (cubin.empty()) {
    J->error = log.size() > 2000 ? log.substr(0, 2000) : log;
    return;
  }
  cudaError_t e = cudaLibraryLoadData(&J->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&J->fn, J->lib, name);
  cudaFuncAttributes fa{};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(J->fn));
  if (e == cudaSuccess) {
    J->static_smem = fa.sharedSizeBytes;
    e = cudaFuncSetAttribute(reinterpret_cast<const void*>(J->fn), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(prop.sharedMemPerBlockOptin - fa.sharedSizeBytes));
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    J->error = std::string("loading the compiled kernel: ") + cudaGetErrorString(e);
    return;
  }
  J->ok = true;
  J->compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void word_jit_build(const WordProgram& wp, int device, JitKernel* J, const WordRunTables* run,
                    const WordSplitPlan* split) {
  J->written.assign(wp.mems.size(), 0);
  J->reg_signals = wp.n_sig_words <= kJitRegSignals;
  for (const WInstr& I : wp.code)
    if (I.op == W_MEMWR && I.aux < J->written.size()) J->written[I.aux] = 1;
  if (wp.code.size() > kJitMaxInstrs) {
    J->error = "word program of " + std::to_string(wp.code.size()) + " instructions runs interpreted";
    return;
  }
  if (split) {
    J->split = true;
    J->n_xwords = (uint32_t)split->xwords.size();
  }
  jit_build_kernel(word_jit_source(wp, run, split), device, "rrtl_word_jit", J);
}

size_t word_jit_place(const WordProgram& wp, const JitKernel& J, uint32_t n_sig_words, uint32_t lanes_pad, uint64_t cycles,
                      uint32_t sm_count, size_t max_smem_block, size_t max_smem_sm, WordJitPlace* out) {
  // a row holds one word of every lane of a block: 128 lanes, 32 for a split kernel
  const uint32_t kThreads = J.split ? 32u : 128u;
  const size_t kRowBytes = (size_t)kThreads * 4u;
  WordJitPlace P{};
  P.n_sig_words = n_sig_words;
  P.n_mems = (uint32_t)std::min<size_t>(wp.mems.size(), kJitPlacedMems);
  // several blocks per SM when there are lanes for them: split the SM's
  // shared memory between them (one block's rows sit idle otherwise)
  const uint32_t blocks = lanes_pad / kThreads;
  const uint32_t per_sm = std::max<uint32_t>(
      1, std::min<uint32_t>(J.split ? 16u : 4u, (blocks + sm_count - 1) / std::max<uint32_t>(sm_count, 1)));
  const size_t share = std::min(max_smem_block, max_smem_sm / per_sm);
  const size_t reserve = 1024 + J.static_smem + (size_t)J.n_xwords * kRowBytes;
  const size_t budget = share > reserve ? share - reserve : 0;
  // staging costs one pass over the rows at each end of the launch: worth it
  // when the launch runs a few cycles per staged row
  auto worth = [&](uint64_t rows) { return rows <= 64 || rows <= 4 * cycles; };
  size_t used = 0;
  if (!J.reg_signals && n_sig_words && (size_t)n_sig_words * kRowBytes <= budget && worth(n_sig_words)) {
    P.sig_smem = 1;
    used = (size_t)n_sig_words * kRowBytes;
  }
  std::vector<uint32_t> order;
  for (uint32_t k = 0; k < P.n_mems; ++k) {
    P.mem_off[k] = wp.mems[k].offset;
    P.mem_words[k] = wp.mems[k].depth * wp.mems[k].limbs;
    P.smem_row[k] = 0xFFFFFFFFu;
    P.written[k] = k < J.written.size() ? J.written[k] : 1;
    order.push_back(k);
  }
  std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return P.mem_words[a] < P.mem_words[b]; });
  for (uint32_t k : order) {
    const size_t bytes = (size_t)P.mem_words[k] * kRowBytes;
    if (used + bytes <= budget && worth(P.mem_words[k])) {
      P.smem_row[k] = (uint32_t)(used / kRowBytes);
      used += bytes;
    }
  }
  // the split kernel's register exchange rows follow the staged rows
  P.x_row = (uint32_t)(used / kRowBytes);
  used += (size_t)J.n_xwords * kRowBytes;
  *out = P;
  return used;
}

cudaError_t launch_word_jit(const JitKernel& J, const WordRunDev& R, const WordJitPlace& Pl, size_t smem, cudaStream_t st) {
  WordRunDev r = R;
  WordJitPlace p = Pl;
  void* args[] = {&r, &p};
  if (J.split)  // 32 lanes per block on two warps
    return cudaLaunchKernel(reinterpret_cast<const void*>(J.fn), dim3(R.lanes_pad / 32u), dim3(64), args, smem, st);
  return cudaLaunchKernel(reinterpret_cast<const void*>(J.fn), dim3(R.lanes_pad / 128u), dim3(128), args, smem, st);
}

}  // namespace rrtl
