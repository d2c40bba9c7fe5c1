// CPU emulation of the fused gate kernel's program (test infrastructure).
//
// Runs the gate lowering's output exactly as the fused kernels consume it —
// the staged piece blob (per-warp run headers and slot records), the slot
// array, the register commit list in commit order — over `lanes` lanes on
// the CPU, and checks the invariants the kernels rely on without checking
// them: every group of a piece is evaluated exactly once through the warp
// headers, each run's table is its groups' table, a cell reads each input
// from a slot that still holds that net (slot reuse never clobbers a live
// net), no cell reads a slot written earlier in its own piece, records and
// commit rows hold the nets they name. Stimulus and the per-cycle output hash
// follow stim.h, so the hashes compare with the bit-parallel oracle's and
// the GPU's. No stuck-at forces, no input traces.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>  // vector types of the device descriptors (host compile)

#include "../../rrtl_gb300/csrc/design.h"
#include "../../rrtl_gb300/csrc/gate_dev.h"
#include "../../rrtl_gb300/csrc/gateprog.h"
#include "../../rrtl_gb300/csrc/stim.h"
#include "../../include/rrtl_cuda.h"

using namespace rrtl;

namespace {

uint32_t lut_word(uint32_t t, uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r = 0;
  for (uint32_t i = 0; i < 8; ++i) {
    if (!((t >> i) & 1u)) continue;
    const uint32_t ma = (i & 4u) ? a : ~a, mb = (i & 2u) ? b : ~b, mc = (i & 1u) ? c : ~c;
    r |= ma & mb & mc;
  }
  return r;
}

uint32_t valid_mask_host(uint32_t gw, uint32_t lanes) {
  const uint64_t base = (uint64_t)gw * 32u;
  if (base >= lanes) return 0u;
  const uint64_t n = lanes - base;
  return n >= 32u ? 0xFFFFFFFFu : ((1u << n) - 1u);
}

struct Fail {
  std::string msg;
};

}  // namespace

extern "C" int emu_gate_run(const char* json, size_t len, const char* top, uint32_t tile_words, uint32_t piece_groups,
                            uint32_t warps, double lead_weight, double run_cost, uint32_t lanes, uint64_t cycles,
                            uint64_t seed, uint64_t lane_base, uint32_t n_stim, const uint32_t* stim_sig,
                            const uint32_t* stim_kind, const uint64_t* stim_param, uint32_t n_rec,
                            const uint32_t* rec_sig, uint64_t* out_hash, char* err, size_t errcap) {
  try {
    Design d = design_from_json(json, len);
    MachineProgram mp = lower_to_machine_program(lower_to_packed_program(d, top));
    GateProgram gp = build_gate_program(mp, tile_words);
    build_pieces(gp, piece_groups);
    const uint32_t V = gate_fused_vec(tile_words);
    PieceBlob blob = build_piece_blob(gp, warps, lead_weight, V, run_cost);
    const uint32_t G = gp.group;
    const uint32_t words = (lanes + 31) / 32;
    const uint64_t word_base = lane_base / 32;
    const uint32_t kScratch = 0xFFFFFFFEu, kNone = 0xFFFFFFFFu;
    std::vector<uint32_t> S((size_t)gp.n_slots * words, 0u);
    std::vector<uint32_t> occ(gp.n_slots, kNone), wrote(gp.n_slots, kNone);
    auto row = [&](uint32_t slot) { return &S[(size_t)slot * words]; };
    auto fail = [&](const std::string& m) { throw Fail{m}; };
    // sources in their permanent slots, constants set, register state 0
    occ[0] = kScratch;
    for (uint32_t n = 0; n < gp.n_nets; ++n)
      if (gp.net_is_source[n] && gp.net_slot[n] >= 0) occ[gp.net_slot[n]] = n;
    std::fill(row(gp.net_slot[kNetConst1]), row(gp.net_slot[kNetConst1]) + words, 0xFFFFFFFFu);
    std::vector<uint32_t> rec_net(n_rec), stim_net(n_stim);
    for (uint32_t i = 0; i < n_rec; ++i) rec_net[i] = gp.signal_net.at(rec_sig[i]);
    for (uint32_t i = 0; i < n_stim; ++i) {
      stim_net[i] = gp.signal_net.at(stim_sig[i]);
      if (!gp.net_is_source[stim_net[i]]) fail("stimulus on a driven signal");
    }
    const std::vector<uint32_t> order = commit_order(gp);
    if (order.size() != gp.regs.size()) fail("commit order does not list every register once");
    {
      std::vector<uint8_t> seen(gp.regs.size(), 0);
      for (uint32_t k : order) {
        if (k >= gp.regs.size() || seen[k]) fail("commit order repeats or skips a register");
        seen[k] = 1;
      }
    }
    const uint32_t hdr_words = blob.hdr_bytes / 4;
    for (uint64_t c = 0; c < cycles; ++c) {
      // stimulus
      for (uint32_t i = 0; i < n_stim; ++i) {
        const uint32_t slot = (uint32_t)gp.net_slot[stim_net[i]];
        if (occ[slot] != stim_net[i]) fail("an input's slot holds another net");
        for (uint32_t w = 0; w < words; ++w) {
          uint32_t& v = row(slot)[w];
          switch (stim_kind[i]) {
            case RRTL_STIM_RANDOM: v = stim_word(seed, stim_param[i], c, word_base + w); break;
            case RRTL_STIM_RANDOM_UNIFORM: v = stim_uniform_word(seed, stim_param[i], c); break;
            case RRTL_STIM_PULSE: v = c < stim_param[i] ? 0xFFFFFFFFu : 0u; break;
            case RRTL_STIM_CONST: v = (stim_param[i] & 1u) ? 0xFFFFFFFFu : 0u; break;
            case RRTL_STIM_HOLD: break;
            default: fail("stimulus kind outside the emulator");
          }
        }
      }
      // pieces, through the staged blob as the warps read it
      for (size_t p = 0; p < gp.pieces.size(); ++p) {
        const GatePiece& pc = gp.pieces[p];
        const uint32_t* pw = blob.words.data() + blob.off_words[p];
        const uint32_t* recs = pw + hdr_words;
        std::vector<uint8_t> done(pc.n_groups, 0);
        for (uint32_t k = 0; k < warps; ++k) {
          std::vector<uint32_t> runs;
          if (pw[2 * k]) runs.push_back(pw[2 * k]);
          for (uint32_t x = pw[2 * k + 1] & 0xFFFFu; x < (pw[2 * k + 1] >> 16); ++x) runs.push_back(pw[2 * warps + x]);
          for (uint32_t run : runs) {
            const uint32_t lut = run & 0xFFu, b = (run >> 8) & 0xFFFu, e = run >> 20;
            if (e > pc.n_groups || b > e) fail("a run outside its piece");
            for (uint32_t h = 0; h < V; ++h)
              for (uint32_t g = b + h; g < e; g += V) {
                if (done[g]) fail("a group evaluated twice in one piece");
                done[g] = 1;
                for (uint32_t cc = 0; cc < G; ++cc) {
                  const GateCell& cell = gp.cells[(size_t)(pc.group_begin + g) * G + cc];
                  if (cell.lut != lut) fail("a run's table differs from its group's");
                  const uint32_t r0 = recs[2 * (g * G + cc)], r1 = recs[2 * (g * G + cc) + 1];
                  const uint32_t sa = r0 & 0xFFFFu, sb = r0 >> 16, sc = r1 & 0xFFFFu, so = r1 >> 16;
                  const uint32_t sl[3] = {sa, sb, sc};
                  const bool use[3] = {(lut & 0x0F) != ((lut >> 4) & 0x0F), (lut & 0x33) != ((lut >> 2) & 0x33),
                                       (lut & 0x55) != ((lut >> 1) & 0x55)};
                  for (int q = 0; q < 3; ++q) {
                    if (!use[q]) continue;
                    const uint32_t want = cell.pad ? (uint32_t)kNetConst0 : cell.in[q];
                    if (!cell.pad && (int32_t)sl[q] != gp.net_slot[want]) fail("a record's slot is not its net's");
                    if (occ[sl[q]] != want) fail("a cell reads a slot that no longer holds its net");
                    if (wrote[sl[q]] == (uint32_t)p) fail("a cell reads a slot written in its own piece");
                  }
                  const uint32_t* A = row(sa);
                  const uint32_t* B = row(sb);
                  const uint32_t* C = row(sc);
                  std::vector<uint32_t> outv(words);
                  for (uint32_t w = 0; w < words; ++w) outv[w] = lut_word(lut, A[w], B[w], C[w]);
                  std::memcpy(row(so), outv.data(), words * 4);
                  occ[so] = cell.pad ? kScratch : cell.out;
                  wrote[so] = (uint32_t)p;
                }
              }
          }
        }
        for (uint32_t g = 0; g < pc.n_groups; ++g)
          if (!done[g]) fail("a group of a piece is left out of every warp's share");
      }
      // record
      unsigned long long hs = 0ull;
      for (uint32_t k = 0; k < n_rec; ++k) {
        const uint32_t slot = (uint32_t)gp.net_slot[rec_net[k]];
        if (gp.net_slot[rec_net[k]] < 0 || occ[slot] != rec_net[k]) fail("a recorded net is not in its slot");
        for (uint32_t w = 0; w < words; ++w)
          hs += hash_term(c, k, word_base + w, row(slot)[w] & valid_mask_host(w, lanes));
      }
      if (out_hash) out_hash[c] = hs;
      // commit, in commit order (D and reset rows are never register rows)
      for (uint32_t k : order) {
        const GateReg& r = gp.regs[k];
        const uint32_t sq = (uint32_t)gp.net_slot[r.q_net], sd = (uint32_t)gp.net_slot[r.d_net];
        const uint32_t sr = (uint32_t)gp.net_slot[r.rst_net];
        if (occ[sd] != r.d_net || (r.has_reset && occ[sr] != r.rst_net)) fail("a commit row does not hold its net");
        for (uint32_t w = 0; w < words; ++w) {
          uint32_t v = row(sd)[w];
          if (r.has_reset) {
            uint32_t m = row(sr)[w];
            if (r.active_low) m = ~m;
            const uint32_t rv = r.reset_value ? 0xFFFFFFFFu : 0u;
            v = (m & rv) | (~m & v);
          }
          row(sq)[w] = v;
        }
        occ[sq] = r.q_net;
      }
      std::fill(wrote.begin(), wrote.end(), kNone);
    }
    return 0;
  } catch (const Fail& f) {
    if (err && errcap) snprintf(err, errcap, "%s", f.msg.c_str());
    return 1;
  } catch (const std::exception& e) {
    if (err && errcap) snprintf(err, errcap, "error: %s", e.what());
    return 2;
  }
}
