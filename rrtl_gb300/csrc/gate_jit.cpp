// Per-design compiled gate kernels: emitter (see gate_jit.h).
//
// The emitted kernel follows the gate engine's cycle exactly as the fused and
// plain kernels do (gate_kernels.cu): stimulus into the source nets, every
// cell in level order, record (trace word, hash term, detection against lane
// 0 of the word, trace checks), then the register commit with synchronous
// reset select; the closing settle re-evaluates the cells and the launch
// writes back the sources and every signal net.
#include "gate_jit.h"

#include <cstdio>

#include "../../include/rrtl_cuda.h"

namespace rrtl {

namespace {

std::string u(uint64_t v) { return std::to_string(v) + "u"; }
std::string n(uint32_t net) {
  if (net == kNetConst0) return "0u";
  if (net == kNetConst1) return "0xFFFFFFFFu";
  return "n" + std::to_string(net);
}

void cells(std::string& o, const GateProgram& gp) {
  for (const GateCell& c : gp.cells) {
    if (c.pad) continue;
    char lut[8];
    snprintf(lut, sizeof lut, "0x%02x", c.lut);
    o += "    " + n(c.out) + " = lop3<" + lut + ">(" + n(c.in[0]) + ", " + n(c.in[1]) + ", " + n(c.in[2]) + ");\n";
  }
}

}  // namespace

std::string GateRunTables::key() const {
  std::string k = std::to_string(mode) + "|";
  for (const GateStimDev& t : stim)
    k += std::to_string(t.net) + "," + std::to_string(t.kind) + "," + std::to_string(t.param) + ";";
  k += "|";
  for (const GateRecDev& t : rec) k += std::to_string(t.net) + ";";
  return k;
}

std::string gate_jit_source(const GateProgram& gp, const GateRunTables& run) {
  std::string o;
  o += "// Compiled gate kernel (generated from the design's gate program and one run's tables).\n";
  o += "#include \"gate_common.h\"\n";
  o += "extern \"C\" __global__ void __launch_bounds__(" + std::to_string(kGateJitThreads) +
       ") rrtl_gate_jit(const rrtl::GateRunDev R) {\n";
  o += "  using namespace rrtl;\n";
  o += "  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;  // 32-lane word\n";
  o += "  const bool own = w < R.words_pad;\n";
  o += "  const uint32_t vm = valid_mask(w, R.lanes);\n";
  o += "  uint32_t* G = R.nets + w;\n";
  o += "  const size_t wp = R.words_pad;\n";
  // every net a register: sources loaded, cell outputs declared
  std::vector<uint8_t> produced(gp.n_nets, 0);
  for (const GateCell& c : gp.cells)
    if (!c.pad) produced[c.out] = 1;
  std::vector<uint32_t> sources;
  for (uint32_t k = 2; k < gp.n_nets; ++k)
    if (gp.net_is_source[k] && !produced[k]) sources.push_back(k);
  for (uint32_t k : sources) o += "  uint32_t " + n(k) + " = own ? G[(size_t)" + u(k) + " * wp] : 0u;\n";
  {
    std::string decl;
    for (uint32_t k = 2; k < gp.n_nets; ++k)
      if (produced[k]) decl += (decl.empty() ? "  uint32_t " : ", ") + n(k) + " = 0u";
    if (!decl.empty()) o += decl + ";\n";
  }
  const uint32_t mode = run.mode;
  const bool trace = mode & RRTL_REC_TRACE, hash = mode & RRTL_REC_HASH, detect = mode & RRTL_REC_DETECT,
             check = mode & RRTL_REC_CHECK;
  const bool any_rec = !run.rec.empty() && (trace || hash || detect || check);
  if (detect) {
    o += "  uint32_t det = 0u;  // lanes detected by an earlier launch of the run stay detected\n";
    o += "  if (w < R.words)\n    for (uint32_t b = 0; b < 32u; ++b)\n";
    o += "      if (R.detect[w * 32u + b] != 0xFFFFFFFFu) det |= 1u << b;\n";
  }
  o += "  for (unsigned long long i = 0; i < R.cycles; ++i) {\n";
  o += "    const unsigned long long c = R.cycle_base + i;\n";
  for (const GateStimDev& s : run.stim) {
    if (s.kind == RRTL_STIM_HOLD) continue;
    char buf[160];
    snprintf(buf, sizeof buf, "GateStimDev{0u, %uu, %uu, 0u, 0x%llxull}", s.net, s.kind, (unsigned long long)s.param);
    o += "    " + n(s.net) + " = stim_value(" + buf + ", R, c, w, " + n(s.net) + ");\n";
  }
  cells(o, gp);
  if (any_rec) {
    o += "    {\n";
    if (hash) o += "      unsigned long long h = 0ull;\n";
    if (detect) o += "      uint32_t diff = 0u;\n";
    for (size_t k = 0; k < run.rec.size(); ++k) {
      const std::string kk = u(k);
      if (hash && k % 32 == 0)  // the cycle's hash salts, one per lane of the warp, shared by shuffles
        o += "      const unsigned long long salt" + std::to_string(k / 32) + " = hash_salt(c, " + u(k) +
             " + (threadIdx.x & 31u));\n";
      if (hash)
        o += "      const unsigned long long sk" + kk + " = __shfl_sync(0xFFFFFFFFu, salt" + std::to_string(k / 32) +
             ", " + u(k % 32) + ");\n";
      o += "      { const uint32_t v = " + n(run.rec[k].net) + " & vm; if (w < R.words) {";
      if (trace) o += " R.out_trace[((size_t)c * " + u(run.rec.size()) + " + " + kk + ") * R.words + w] = v;";
      if (hash) o += " h += hash_term_salted(sk" + kk + ", R.word_base + w, v);";
      if (detect) o += " diff |= v ^ (0u - (v & 1u));";
      if (check) o += " check_word(R, c, " + kk + ", w, v);";
      o += " } }\n";
    }
    if (hash) {
      o += "      for (int s = 16; s > 0; s >>= 1) h += __shfl_xor_sync(0xFFFFFFFFu, h, s);\n";
      o += "      if ((threadIdx.x & 31u) == 0 && h) atomicAdd(R.out_hash + c, h);\n";
    }
    if (detect) {
      o += "      uint32_t nb = diff & ~det & vm;\n      det |= nb;\n";
      o += "      while (nb) { const uint32_t b = __ffs(nb) - 1u; R.detect[w * 32u + b] = (uint32_t)c; nb &= nb - 1u; }\n";
    }
    o += "    }\n";
  }
  // commit: every register's next value from the pre-commit nets, then all at once
  if (!gp.regs.empty()) {
    o += "    {\n";
    for (size_t k = 0; k < gp.regs.size(); ++k) {
      const GateReg& r = gp.regs[k];
      std::string e = n(r.d_net);
      if (r.has_reset) {
        // m = reset asserted per lane; next = (m & reset value) | (~m & d)
        const std::string m = r.active_low ? "(~" + n(r.rst_net) + ")" : n(r.rst_net);
        const std::string rv = r.reset_value ? "0xFFFFFFFFu" : "0u";
        e = "((" + m + " & " + rv + ") | (~" + m + " & " + n(r.d_net) + "))";
      }
      o += "      const uint32_t q" + std::to_string(k) + " = " + e + ";\n";
    }
    for (size_t k = 0; k < gp.regs.size(); ++k) o += "      " + n(gp.regs[k].q_net) + " = q" + std::to_string(k) + ";\n";
    o += "    }\n";
  }
  o += "  }\n";
  o += "  if (R.final_settle) {\n";
  cells(o, gp);
  o += "  }\n";
  o += "  if (!own) return;\n";
  for (uint32_t k : sources) o += "  G[(size_t)" + u(k) + " * wp] = " + n(k) + ";\n";
  o += "  if (R.final_settle) {\n";
  for (uint32_t k = 2; k < gp.n_nets; ++k)
    if (produced[k] && gp.net_signal[k] >= 0) o += "    G[(size_t)" + u(k) + " * wp] = " + n(k) + ";\n";
  o += "  }\n";
  o += "}\n";
  return o;
}

void gate_jit_build(const GateProgram& gp, const GateRunTables& run, int device, JitKernel* J) {
  if (gp.n_real_cells > kGateJitMaxCells) {
    J->error = "gate program of " + std::to_string(gp.n_real_cells) + " cells runs on the fused kernel";
    return;
  }
  jit_build_kernel(gate_jit_source(gp, run), device, "rrtl_gate_jit", J);
}

cudaError_t launch_gate_jit(const JitKernel& J, const GateRunDev& R, cudaStream_t st) {
  GateRunDev r = R;
  void* args[] = {&r};
  const uint32_t grid = (R.words_pad + kGateJitThreads - 1) / kGateJitThreads;
  return cudaLaunchKernel(reinterpret_cast<const void*>(J.fn), dim3(grid), dim3(kGateJitThreads), args, 0, st);
}

std::string gate_fused_jit_source(const GateProgram& gp) {
  std::vector<uint8_t> used(256, 0);
  used[0] = 1;  // an empty run (header word 0) dispatches to class 0
  for (const GateCell& c : gp.cells) used[c.lut] = 1;
  // the kernel's shape as the host library was built with it (launch size, shares)
  std::string o = "// rrtl_gate_fused_jit: gate_fused_kernel<" + std::to_string(gp.tile_words) +
                  "> for one design's truth-table classes\n#define RRTL_FUSED_WARPS " +
                  std::to_string(kGateFusedWarps) + "\n#define RRTL_FUSED_CTAS_PER_SM " +
                  std::to_string(kGateFusedCtasPerSm) + "\n#define RRTL_FUSED_V " + std::to_string(RRTL_FUSED_V) +
                  "\n#define RRTL_LUT_CLASSES(X)";
  for (int l = 0; l < 256; ++l)
    if (used[l]) o += " X(" + std::to_string(l) + ")";
  o += "\n#include \"gate_fused.h\"\n";
  o += "extern \"C\" __global__ void __launch_bounds__(rrtl::kFusedThreads, rrtl::kGateFusedCtasPerSm)\n";
  o += "rrtl_gate_fused_jit(rrtl::GateProgDev P, rrtl::GateRunDev R) {\n";
  o += "  rrtl::fused_kernel_body<" + std::to_string(gp.tile_words) + ", true>(P, R);\n}\n";
  return o;
}

void gate_fused_jit_build(const GateProgram& gp, int device, JitKernel* J) {
  for (const GateCell& c : gp.cells)
    if (!lut_is_canonical(c.lut)) {
      J->error = "a cell's truth table is not a class representative";
      return;
    }
  jit_build_kernel(gate_fused_jit_source(gp), device, "rrtl_gate_fused_jit", J);
}

cudaError_t launch_gate_fused_jit(const JitKernel& J, const GateProgDev& P, const GateRunDev& R, uint32_t grid,
                                  size_t smem, cudaStream_t st) {
  GateProgDev p = P;
  GateRunDev r = R;
  void* args[] = {&p, &r};
  return cudaLaunchKernel(reinterpret_cast<const void*>(J.fn), dim3(grid), dim3(kGateFusedWarps * 32u), args, smem, st);
}

}  // namespace rrtl
