// Device code of the fused gate kernel: the per-tile body shared by
// gate_fused_kernel and gate_queue_kernel (gate_kernels.cu) and the
// per-design compiled fused kernel (gate_jit.cpp, compiled at run time by
// NVRTC), which is why this header includes only headers handed to NVRTC
// with it. A compiled kernel defines RRTL_LUT_CLASSES before the include, so
// its run dispatch lists only the truth-table classes its design uses.
#pragma once

#include <stdint.h>

#include "../../include/rrtl_cuda.h"
#include "gate_common.h"
#include "gate_dev.h"
#include "lut_classes.h"

namespace rrtl {

constexpr int kFusedWarps = (int)kGateFusedWarps;
constexpr int kFusedThreads = kFusedWarps * 32;
constexpr int kRing = 4;                  // record ring buffers
constexpr uint32_t kSpinLimit = 1u << 22;  // bounded mbarrier wait
constexpr uint32_t kFusedHeader = 128;     // bytes between the ring and the slot array
#ifndef RRTL_FUSED_UNROLL
#define RRTL_FUSED_UNROLL 1  // warp steps per unrolled iteration (unpaired loop)
#endif
#ifndef RRTL_PAIR_STEPS
#define RRTL_PAIR_STEPS 0  // 1: two warp steps per loop iteration, loads ahead of stores
#endif
#if !RRTL_PAIR_STEPS
constexpr int kUnroll = RRTL_FUSED_UNROLL;
#endif
static_assert(kRing * 8 + 8 + 16 * 4 + 8 <= kFusedHeader, "fused kernel header overflows");
static_assert(kRing == 4, "ring parity arithmetic assumes four buffers");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait for the mbarrier phase with the given parity; false after
// `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kSpinLimit) {
  uint32_t addr = smem_u32(bar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Runtime truth table: Shannon expansion on a, then b, then c.
__device__ __forceinline__ uint32_t lut_eval(uint32_t t, uint32_t a, uint32_t b, uint32_t c) {
  uint32_t m0 = 0u - (t & 1u), m1 = 0u - ((t >> 1) & 1u), m2 = 0u - ((t >> 2) & 1u), m3 = 0u - ((t >> 3) & 1u);
  uint32_t m4 = 0u - ((t >> 4) & 1u), m5 = 0u - ((t >> 5) & 1u), m6 = 0u - ((t >> 6) & 1u), m7 = 0u - ((t >> 7) & 1u);
  uint32_t u0 = (c & m1) | (~c & m0), u1 = (c & m3) | (~c & m2);
  uint32_t u2 = (c & m5) | (~c & m4), u3 = (c & m7) | (~c & m6);
  uint32_t f0 = (b & u1) | (~b & u0), f1 = (b & u3) | (~b & u2);
  return (a & f1) | (~a & f0);
}

// Bytes of the fused kernel's slot array, rounded so the tables behind it
// stay 16-byte aligned.
__host__ __device__ __forceinline__ size_t fused_slot_bytes(uint32_t n_slots, uint32_t words) {
  return ((size_t)n_slots * words * 4u + 15u) & ~(size_t)15u;
}

// ------------------------------------------------------------ fused path --
//
// A thread owns V consecutive words (gate_fused_vec: one 64- or 128-bit
// shared access moves them). The warp splits into V sub-warps of 32/V lanes;
// sub-warp h covers one group (G cells x W words), so a warp step evaluates
// groups g .. g+V-1 of one truth-table run. Cells of a group sit in G
// distinct bank residues, so each sub-warp access is one shared-memory
// wavefront.

template <int W>
struct FusedShape {
  static constexpr int V = (int)gate_fused_vec(W);  // words per thread
  static constexpr int G = 32 / W;                  // cells per group
  static constexpr int kSteps = V;                  // groups per warp step
  static constexpr int kSub = 32 / V;               // lanes per sub-warp (one group)
};

template <int V>
struct WordVec;
template <>
struct WordVec<1> {
  using T = uint32_t;
};
template <>
struct WordVec<2> {
  using T = uint2;
};
template <>
struct WordVec<4> {
  using T = uint4;
};

template <int L>
__device__ __forceinline__ uint32_t lopv(uint32_t a, uint32_t b, uint32_t c) {
  return lop3<L>(a, b, c);
}
template <int L>
__device__ __forceinline__ uint2 lopv(uint2 a, uint2 b, uint2 c) {
  return make_uint2(lop3<L>(a.x, b.x, c.x), lop3<L>(a.y, b.y, c.y));
}
template <int L>
__device__ __forceinline__ uint4 lopv(uint4 a, uint4 b, uint4 c) {
  return make_uint4(lop3<L>(a.x, b.x, c.x), lop3<L>(a.y, b.y, c.y), lop3<L>(a.z, b.z, c.z), lop3<L>(a.w, b.w, c.w));
}

// Evaluate this thread's cell in groups g, g+V, ... < e of one truth-table
// run (g already offset by the sub-warp). `rb` is this thread's record in
// group 0 of the staged piece and `Sv` its word column of the slot array (row
// stride W/V vectors); both are shared memory, so every access below is an
// LDS/STS.
template <int W, int L>
__device__ __forceinline__ void run_seg(const uint2* __restrict__ rb, typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv,
                                        int g, int e) {
  using Sh = FusedShape<W>;
  using T = typename WordVec<Sh::V>::T;
  constexpr int R = W / Sh::V;
  constexpr bool kUseA = (L & 0x0F) != ((L >> 4) & 0x0F);
  constexpr bool kUseB = (L & 0x33) != ((L >> 2) & 0x33);
  constexpr bool kUseC = (L & 0x55) != ((L >> 1) & 0x55);
  const T zero{};
#if RRTL_PAIR_STEPS
  // two steps per iteration with every load before either store: cells of one
  // piece never read each other's outputs, so the second step's loads may
  // overtake the first step's store (the compiler cannot know that)
  for (; g + Sh::kSteps < e; g += 2 * Sh::kSteps) {
    const uint2 r0 = rb[g * Sh::G];
    const uint2 r1 = rb[(g + Sh::kSteps) * Sh::G];
    const T a0 = kUseA ? Sv[(r0.x & 0xFFFFu) * R] : zero;
    const T a1 = kUseA ? Sv[(r1.x & 0xFFFFu) * R] : zero;
    const T b0 = kUseB ? Sv[(r0.x >> 16) * R] : zero;
    const T b1 = kUseB ? Sv[(r1.x >> 16) * R] : zero;
    const T c0 = kUseC ? Sv[(r0.y & 0xFFFFu) * R] : zero;
    const T c1 = kUseC ? Sv[(r1.y & 0xFFFFu) * R] : zero;
    Sv[(r0.y >> 16) * R] = lopv<L>(a0, b0, c0);
    Sv[(r1.y >> 16) * R] = lopv<L>(a1, b1, c1);
  }
  if (g < e) {
    const uint2 r = rb[g * Sh::G];
    const T va = kUseA ? Sv[(r.x & 0xFFFFu) * R] : zero;
    const T vb = kUseB ? Sv[(r.x >> 16) * R] : zero;
    const T vc = kUseC ? Sv[(r.y & 0xFFFFu) * R] : zero;
    Sv[(r.y >> 16) * R] = lopv<L>(va, vb, vc);
  }
#else
#pragma unroll kUnroll
  for (; g < e; g += Sh::kSteps) {
    const uint2 r = rb[g * Sh::G];
    const T va = kUseA ? Sv[(r.x & 0xFFFFu) * R] : zero;
    const T vb = kUseB ? Sv[(r.x >> 16) * R] : zero;
    const T vc = kUseC ? Sv[(r.y & 0xFFFFu) * R] : zero;
    Sv[(r.y >> 16) * R] = lopv<L>(va, vb, vc);
  }
#endif
}

// One warp step of a run: the cells of record r.
template <int W, int L>
__device__ __forceinline__ void cell_step(typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv, uint2 r) {
  using Sh = FusedShape<W>;
  using T = typename WordVec<Sh::V>::T;
  constexpr int R = W / Sh::V;
  constexpr bool kUseA = (L & 0x0F) != ((L >> 4) & 0x0F);
  constexpr bool kUseB = (L & 0x33) != ((L >> 2) & 0x33);
  constexpr bool kUseC = (L & 0x55) != ((L >> 1) & 0x55);
  const T zero{};
  const T va = kUseA ? Sv[(r.x & 0xFFFFu) * R] : zero;
  const T vb = kUseB ? Sv[(r.x >> 16) * R] : zero;
  const T vc = kUseC ? Sv[(r.y & 0xFFFFu) * R] : zero;
  Sv[(r.y >> 16) * R] = lopv<L>(va, vb, vc);
}

// A warp's first run of a piece under the split barrier: wait until every
// warp finished the previous piece (its outputs are this piece's operands),
// then the first step from the record read before the wait, then the rest.
template <int W, int L>
__device__ __forceinline__ void run_seg_first(const uint2* __restrict__ rb,
                                              typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv, int g, int e,
                                              uint2 rf, uint64_t* pbar, uint32_t parity, int& abort_flag) {
  if (!mbar_wait(pbar, parity)) abort_flag = 1;
  if (g < e) {
    cell_step<W, L>(Sv, rf);
    g += FusedShape<W>::kSteps;
  }
  run_seg<W, L>(rb, Sv, g, e);
}

#define RRTL_CASE_FIRST(n) \
  case n: run_seg_first<W, n>(rb, Sv, b + h, e, rf, pbar, parity, abort_flag); break;

template <int W>
__device__ __forceinline__ void eval_run_first(const uint2* __restrict__ rb,
                                               typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv, uint32_t run, int h,
                                               uint2 rf, uint64_t* pbar, uint32_t parity, int& abort_flag) {
  const int b = (int)((run >> 8) & 0xFFFu), e = (int)(run >> 20);
  switch (run & 0xFFu) {
    RRTL_LUT_CLASSES(RRTL_CASE_FIRST)
    default:
      if (!mbar_wait(pbar, parity)) abort_flag = 1;
      break;
  }
}

#define RRTL_CASE(n) \
  case n: run_seg<W, n>(rb, Sv, b + h, e); break;

// One truth-table run (pack_run) of this warp's share.
template <int W>
__device__ __forceinline__ void eval_run(const uint2* __restrict__ rb, typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv,
                                         uint32_t run, int h) {
  const int b = (int)((run >> 8) & 0xFFFu), e = (int)(run >> 20);
  switch (run & 0xFFu) {
    RRTL_LUT_CLASSES(RRTL_CASE)
    default: break;  // not a class representative: the lowering never emits it
  }
}

// This warp's share of a staged piece: its first run (from its header word)
// and its further runs extra[k0, k1).
template <int W>
__device__ __forceinline__ void eval_piece(const uint2* __restrict__ rb, typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv,
                                           uint32_t run0, const uint32_t* __restrict__ extra, uint32_t k0, uint32_t k1,
                                           int h) {
  eval_run<W>(rb, Sv, run0, h);
  for (uint32_t k = k0; k < k1; ++k) eval_run<W>(rb, Sv, extra[k], h);
}

__device__ __forceinline__ uint32_t lut_v(uint32_t t, uint32_t a, uint32_t b, uint32_t c) { return lut_eval(t, a, b, c); }
__device__ __forceinline__ uint2 lut_v(uint32_t t, uint2 a, uint2 b, uint2 c) {
  return make_uint2(lut_eval(t, a.x, b.x, c.x), lut_eval(t, a.y, b.y, c.y));
}
__device__ __forceinline__ uint4 lut_v(uint32_t t, uint4 a, uint4 b, uint4 c) {
  return make_uint4(lut_eval(t, a.x, b.x, c.x), lut_eval(t, a.y, b.y, c.y), lut_eval(t, a.z, b.z, c.z),
                    lut_eval(t, a.w, b.w, c.w));
}
// Synchronous reset on commit: where the reset net is active (flags: 2
// active low), the register takes its reset value (flags: 4 one) instead of D.
__device__ __forceinline__ uint32_t reset_select(uint32_t d, uint32_t m, uint32_t flags) {
  if (flags & 2u) m = ~m;
  const uint32_t rv = (flags & 4u) ? 0xFFFFFFFFu : 0u;
  return (m & rv) | (~m & d);
}
__device__ __forceinline__ uint2 reset_select(uint2 d, uint2 m, uint32_t flags) {
  return make_uint2(reset_select(d.x, m.x, flags), reset_select(d.y, m.y, flags));
}
__device__ __forceinline__ uint4 reset_select(uint4 d, uint4 m, uint32_t flags) {
  return make_uint4(reset_select(d.x, m.x, flags), reset_select(d.y, m.y, flags), reset_select(d.z, m.z, flags),
                    reset_select(d.w, m.w, flags));
}
__device__ __forceinline__ void store_net(uint32_t* p, uint32_t v) { p[0] = v; }
__device__ __forceinline__ void store_net(uint32_t* p, uint2 v) {
  p[0] = v.x;
  p[1] = v.y;
}
__device__ __forceinline__ void store_net(uint32_t* p, uint4 v) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
  p[3] = v.w;
}

// Final settle: same evaluation with a runtime truth table, plus a copy of
// every signal net to the global state (`col` = this thread's first word).
template <int W>
__device__ __forceinline__ void writeback_run(const uint2* __restrict__ rb,
                                              typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv, uint32_t run, int h,
                                              const uint32_t* __restrict__ wb, uint32_t* nets, size_t words_pad,
                                              uint32_t col) {
  using Sh = FusedShape<W>;
  constexpr int R = W / Sh::V;
  const uint32_t lut = run & 0xFFu;
  const int b = (int)((run >> 8) & 0xFFFu), e = (int)(run >> 20);
  for (int g = b + h; g < e; g += Sh::kSteps) {
    const uint2 r = rb[g * Sh::G];
    const auto v = lut_v(lut, Sv[(r.x & 0xFFFFu) * R], Sv[(r.x >> 16) * R], Sv[(r.y & 0xFFFFu) * R]);
    Sv[(r.y >> 16) * R] = v;
    const uint32_t net = __ldg(wb + g * Sh::G);
    if (net != 0xFFFFFFFFu) store_net(nets + (size_t)net * words_pad + col, v);
  }
}

template <int W>
__device__ __forceinline__ void eval_piece_writeback(const uint2* __restrict__ rb,
                                                     typename WordVec<FusedShape<W>::V>::T* __restrict__ Sv, uint32_t run0,
                                                     const uint32_t* __restrict__ extra, uint32_t k0, uint32_t k1, int h,
                                                     const uint32_t* __restrict__ wb, uint32_t* nets, size_t words_pad,
                                                     uint32_t col) {
  writeback_run<W>(rb, Sv, run0, h, wb, nets, words_pad, col);
  for (uint32_t k = k0; k < k1; ++k) writeback_run<W>(rb, Sv, extra[k], h, wb, nets, words_pad, col);
}

template <int W>
__device__ __forceinline__ void apply_forces(const GateRunDev& R, uint32_t* S, uint32_t tile, uint32_t stage,
                                             uint32_t stages) {
  const uint32_t* off = R.force_off + (size_t)tile * (stages + 1);
  uint32_t b = __ldg(off + stage), e = __ldg(off + stage + 1);
  for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    GateForceDev f = R.forces[i];
    uint32_t& v = S[f.slot * W + f.word];
    v = (v & ~f.mask) | (f.val & f.mask);
  }
}

// Per-CTA state of the fused kernels that outlives one tile. The 128-byte
// header at the start of shared memory holds the ring's mbarriers, the hash
// accumulator and the detect state; everything after it is laid out per tile
// from the tile's program: [piece ring][slots][piece table], each region on
// a 16-byte boundary (ring buffers are bulk-copy destinations).
struct FusedCta {
  uint64_t* bars;
  uint64_t* pbar;    // split piece barrier: one arrival per warp
  uint32_t pphase;   // its phases started (every thread)
  unsigned long long* hacc;
  uint32_t* dstate;  // diff[8], detected[8]
  uint8_t* dyn;
  uint64_t q;       // pieces consumed (every thread)
  uint64_t issued;  // copies issued (thread 0)
  bool aborted;
};

__device__ __forceinline__ void fused_cta_init(FusedCta& cta, uint8_t* smem) {
  cta.bars = reinterpret_cast<uint64_t*>(smem);
  cta.hacc = reinterpret_cast<unsigned long long*>(smem + kRing * 8);
  cta.dstate = reinterpret_cast<uint32_t*>(smem + kRing * 8 + 8);
  cta.dyn = smem + kFusedHeader;
  cta.pbar = reinterpret_cast<uint64_t*>(smem + kRing * 8 + 8 + 16 * 4);
  cta.pphase = 0;
  cta.q = 0;
  cta.issued = 0;
  cta.aborted = false;
  if (threadIdx.x == 0) {
    *cta.hacc = 0ull;
    for (int i = 0; i < kRing; ++i) mbar_init(&cta.bars[i], 1);
    mbar_init(cta.pbar, (uint32_t)kFusedWarps);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
}

// After an abort, let every copy still in flight land before the CTA's shared
// memory is released. A drain wait that gives up leaves a copy in flight into
// shared memory the next CTA on this SM may reuse, possibly for another job:
// it is recorded in `err`, which covers every run the launch serves.
__device__ __forceinline__ void fused_cta_drain(const FusedCta& cta, uint32_t* err) {
  if (cta.aborted && threadIdx.x == 0)
    for (uint64_t k = cta.q; k < cta.issued; ++k)
      if (!mbar_wait(&cta.bars[(uint32_t)k & (kRing - 1u)], ((uint32_t)k >> 2) & 1u))
        atomicExch(err, (uint32_t)RRTL_E_TIMEOUT);
}

// Cycles [c0, c0 + ncyc) of one tile (W words) of a run, then the closing
// settle if `final_settle`. Net state is read from and written back to the
// run's global net rows, so a run may be split into consecutive calls.
// kSplit: cycles without forces separate pieces by the split piece barrier
// (the fused kernel compiled for a design's few truth-table classes);
// without it every piece ends at a CTA barrier (the generic fused kernel and
// the job queue, whose loops cover all 80 classes: with the split form's
// second copy of each, the generic kernel measured 3x slower on the 50k-gate
// netlist and the job queue 1.8x).
template <int W, bool kSplit>
__device__ __forceinline__ void fused_tile(const GateProgDev& P, const GateRunDev& R, uint32_t tile, uint64_t c0,
                                           uint64_t ncyc, bool final_settle, FusedCta& cta) {
  constexpr uint32_t G = 32 / W;
  using Sh = FusedShape<W>;
  using T = typename WordVec<Sh::V>::T;
  const size_t ring_bytes = P.ring_bytes;  // one ring buffer: a staged piece
  uint8_t* ring = cta.dyn;
  uint32_t* S = reinterpret_cast<uint32_t*>(cta.dyn + (size_t)kRing * ring_bytes);
  GatePieceDev* pieces = reinterpret_cast<GatePieceDev*>(cta.dyn + (size_t)kRing * ring_bytes + fused_slot_bytes(P.n_slots, W));
  uint64_t* bars = cta.bars;
  uint32_t* dstate = cta.dstate;
  unsigned long long* hacc = cta.hacc;

  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  // lane -> (sub-warp h, cell c of the group, first word w of this thread)
  const uint32_t h = lane / Sh::kSub;
  const uint32_t hl = lane % Sh::kSub;
  const uint32_t cidx = hl / (W / Sh::V), w = (hl % (W / Sh::V)) * Sh::V;
  const bool resident = P.n_pieces <= (uint32_t)kRing;
  const uint32_t stages = P.n_levels + 1;
  const uint64_t passes = ncyc + (final_settle ? 1u : 0u);
  const uint64_t q0 = cta.q;
  const uint64_t q_end = q0 + (resident ? (uint64_t)P.n_pieces : passes * P.n_pieces);
  const uint32_t col0 = tile * W;
  T* const Sv = reinterpret_cast<T*>(S + w);
  const uint32_t hdr_bytes = P.hdr_bytes;

  // piece table, constants, scratch, sources, detect state
  for (uint32_t i = tid; i < P.n_pieces; i += blockDim.x) pieces[i] = P.pieces[i];
  for (uint32_t i = tid; i < W; i += blockDim.x) {
    S[0 * W + i] = 0u;
    S[P.const0_slot * W + i] = 0u;
    S[P.const1_slot * W + i] = 0xFFFFFFFFu;
  }
  if (tid < 8u) {
    // lanes already detected by an earlier part of this run stay detected
    uint32_t det = 0u;
    if ((R.mode & RRTL_REC_DETECT) && tid < W && col0 + tid < R.words)
      for (uint32_t b = 0; b < 32u; ++b)
        if (R.detect[(col0 + tid) * 32u + b] != 0xFFFFFFFFu) det |= 1u << b;
    dstate[tid] = 0u;
    dstate[8 + tid] = det;
  }
  for (uint32_t i = tid; i < P.n_src * W; i += blockDim.x) {
    uint32_t k = i / W, ww = i % W;
    S[__ldg(P.src_slot + k) * W + ww] = R.nets[(size_t)__ldg(P.src_net + k) * R.words_pad + col0 + ww];
  }
  __syncthreads();

  // Ring bookkeeping. Piece q of this CTA's stream lands in buffer q % kRing;
  // its copy completes phase (q / kRing) & 1 of that buffer's mbarrier.
  // Thread 0 keeps the ring full: at the start of piece q it refills the
  // buffer that piece q-1 released (the CTA barrier ending q-1 guarantees no
  // warp still reads it); after its share of piece q it waits for piece q+1
  // to land, and the barrier that ends piece q publishes that piece to every
  // thread. A program of at most kRing pieces is loaded once per tile and
  // stays resident. A wait that runs out sets the error word, and the
  // barrier's OR ends the CTA's work.
  //
  // Cycles without stuck-at forces separate pieces by the split piece
  // barrier instead (cta.pbar, one arrival per warp): thread 0 refills the
  // buffer of piece q-1 once its own wait has seen every warp finish piece
  // q-1, and every thread waits for piece q+1 to land itself before it reads
  // that piece's header and first record. A thread whose wait runs out reads
  // nothing more, and the CTA barrier that ends the cycle ORs the error.
  uint32_t next_piece = 0;                // piece index of the next copy (thread 0)
  uint32_t next_off = 0, next_bytes = 0;  // its blob offset and size, loaded one copy ahead
  int abort_flag = 0;                     // this thread: a bounded wait ran out
  auto load_next = [&]() {
    next_off = pieces[next_piece].off_words;
    next_bytes = pieces[next_piece].bytes;
  };
  auto issue_next = [&]() {
    const uint32_t b = (uint32_t)cta.issued & (kRing - 1u);
    bulk_load(ring + b * ring_bytes, P.blob + next_off, next_bytes, &bars[b]);
    ++cta.issued;
    if (++next_piece == P.n_pieces) next_piece = 0;
    load_next();
  };
  auto timed_out = [&]() {
    abort_flag = 1;
    atomicExch(R.err, (uint32_t)RRTL_E_TIMEOUT);
  };
  if (tid == 0 && q_end > q0) {
    load_next();
    const uint64_t n0 = q_end - q0 < (uint64_t)kRing ? q_end : q0 + kRing;
    while (cta.issued < n0) issue_next();
    const uint64_t first = resident ? q_end : q0 + 1;
    for (uint64_t k = q0; k < first; ++k)
      if (!mbar_wait(&bars[(uint32_t)k & (kRing - 1u)], ((uint32_t)k >> 2) & 1u)) timed_out();
  }
  if (__syncthreads_or(abort_flag)) {
    cta.aborted = true;
    return;
  }
  uint64_t q = q0;

  for (uint64_t pass = 0; pass < passes; ++pass) {
    const bool final_pass = pass == ncyc;
    const uint64_t c = c0 + pass;
    if (final_pass) {
      // register slots may host other nets during a settle: write the
      // sources back before the final settle recomputes every signal
      for (uint32_t i = tid; i < P.n_src * W; i += blockDim.x) {
        uint32_t k = i / W, ww = i % W;
        R.nets[(size_t)__ldg(P.src_net + k) * R.words_pad + col0 + ww] = S[__ldg(P.src_slot + k) * W + ww];
      }
    } else {
      for (uint32_t i = tid; i < R.n_stim * W; i += blockDim.x) {
        const GateStimDev& st = R.stim[i / W];
        if (st.kind == RRTL_STIM_HOLD) continue;
        uint32_t ww = i % W;
        uint32_t& slot = S[st.slot * W + ww];
        slot = stim_value(st, R, c, col0 + ww, slot);
      }
    }
    __syncthreads();
    if (kSplit && !final_pass && !R.has_forces && P.n_pieces > 1) {
      // Split piece barrier: a warp that finished piece p arrives, reads the
      // next piece's header word and its first record, and waits for the
      // other warps only right before its first operand load of piece p+1,
      // so a piece's start latency overlaps the slowest warp's tail. The
      // last piece of a cycle ends at the CTA barrier below.
      uint2 hw_n = make_uint2(0u, 0u), rf_n = make_uint2(0u, 0u);
      for (uint32_t p = 0; p < P.n_pieces; ++p) {
        const uint32_t buf = (uint32_t)(resident ? q0 + p : q) & (kRing - 1u);
        const uint8_t* pb = ring + buf * ring_bytes;
        const uint2* rb = reinterpret_cast<const uint2*>(pb + hdr_bytes) + cidx;
        const uint32_t* extra = reinterpret_cast<const uint32_t*>(pb) + 2 * kFusedWarps;
        if (p == 0) {
          if (!resident && tid == 0 && q > q0 && cta.issued < q_end) issue_next();
          const uint2 hw = reinterpret_cast<const uint2*>(pb)[warp];
          eval_piece<W>(rb, Sv, hw.x, extra, hw.y & 0xFFFFu, hw.y >> 16, (int)h);
        } else {
          eval_run_first<W>(rb, Sv, hw_n.x, (int)h, rf_n, cta.pbar, (cta.pphase - 1u) & 1u, abort_flag);
          for (uint32_t k = hw_n.y & 0xFFFFu; k < (hw_n.y >> 16); ++k) eval_run<W>(rb, Sv, extra[k], (int)h);
          // every warp finished piece p-1: the ring buffer it used is free
          if (!resident && tid == 0 && cta.issued < q_end) issue_next();
        }
        if (p + 1 < P.n_pieces) {
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(cta.pbar)) : "memory");
          ++cta.pphase;
          const uint64_t qn = resident ? q0 + p + 1 : q + 1;
          bool landed = true;
          if (!resident && !mbar_wait(&bars[(uint32_t)qn & (kRing - 1u)], ((uint32_t)qn >> 2) & 1u)) {
            timed_out();
            landed = false;
          }
          hw_n = make_uint2(0u, 0u);
          if (landed) {
            const uint8_t* pbn = ring + ((uint32_t)qn & (kRing - 1u)) * ring_bytes;
            hw_n = reinterpret_cast<const uint2*>(pbn)[warp];
            const int bn = (int)((hw_n.x >> 8) & 0xFFFu) + (int)h, en = (int)(hw_n.x >> 20);
            if (bn < en) rf_n = (reinterpret_cast<const uint2*>(pbn + hdr_bytes) + cidx)[bn * Sh::G];
          }
        }
        if (!resident) ++q;
      }
      if (!resident && tid == 0) {
        const uint64_t qn = q;
        if (qn < q_end && !mbar_wait(&bars[(uint32_t)qn & (kRing - 1u)], ((uint32_t)qn >> 2) & 1u)) timed_out();
      }
      if (__syncthreads_or(abort_flag)) {
        cta.q = q;
        cta.aborted = true;
        return;
      }
    } else
    for (uint32_t p = 0; p < P.n_pieces; ++p) {
      const uint32_t buf = (uint32_t)(resident ? q0 + p : q) & (kRing - 1u);
      if (!resident && tid == 0 && q > q0 && cta.issued < q_end) issue_next();
      {
        // the staged piece: two header words per warp, the further runs, then the records
        const uint8_t* pb = ring + buf * ring_bytes;
        const uint2 hw = reinterpret_cast<const uint2*>(pb)[warp];
        const uint32_t* extra = reinterpret_cast<const uint32_t*>(pb) + 2 * kFusedWarps;
        const uint2* rb = reinterpret_cast<const uint2*>(pb + hdr_bytes) + cidx;
        if (final_pass)
          eval_piece_writeback<W>(rb, Sv, hw.x, extra, hw.y & 0xFFFFu, hw.y >> 16, (int)h,
                                  P.wb_net + (size_t)pieces[p].group_begin * G + cidx, R.nets, R.words_pad, col0 + w);
        else
          eval_piece<W>(rb, Sv, hw.x, extra, hw.y & 0xFFFFu, hw.y >> 16, (int)h);
      }
      if (!resident && tid == 0) {
        // warp 0 has a lighter share: wait for the next piece while the others finish
        const uint64_t qn = q + 1;
        if (qn < q_end && !mbar_wait(&bars[(uint32_t)qn & (kRing - 1u)], ((uint32_t)qn >> 2) & 1u)) timed_out();
      }
      if (R.has_forces && pieces[p].last_of_level) {
        __syncthreads();
        apply_forces<W>(R, S, tile, pieces[p].level + 1, stages);
      }
      if (!resident) ++q;
      if (__syncthreads_or(abort_flag)) {
        cta.q = q;
        cta.aborted = true;
        return;
      }
    }
    if (final_pass) break;
    // record
    if (R.n_rec) {
      unsigned long long hs = 0ull;
      for (uint32_t i = tid; i < R.n_rec * W; i += blockDim.x) {
        uint32_t k = i / W, ww = i % W, gw = col0 + ww;
        uint32_t v = S[R.rec[k].slot * W + ww] & valid_mask(gw, R.lanes);
        if (gw < R.words) {
          if (R.mode & RRTL_REC_TRACE) R.out_trace[((size_t)c * R.n_rec + k) * R.words + gw] = v;
          if (R.mode & RRTL_REC_HASH) hs += hash_term(c, k, R.word_base + gw, v);
          if (R.mode & RRTL_REC_DETECT) atomicOr(&dstate[ww], v ^ (0u - (v & 1u)));
          if (R.mode & RRTL_REC_CHECK) check_word(R, c, k, gw, v);
        }
      }
      if (R.mode & RRTL_REC_HASH) {
        for (int o = 16; o > 0; o >>= 1) hs += __shfl_xor_sync(0xFFFFFFFFu, hs, o);
        if (lane == 0 && hs) atomicAdd(hacc, hs);
      }
      __syncthreads();
      if (tid == 0 && (R.mode & RRTL_REC_HASH)) {
        unsigned long long t = *hacc;
        if (t) atomicAdd(R.out_hash + c, t);
        *hacc = 0ull;
      }
      if ((R.mode & RRTL_REC_DETECT) && tid < W) {
        uint32_t gw = col0 + tid;
        uint32_t nb = dstate[tid] & ~dstate[8 + tid] & valid_mask(gw, R.lanes);
        dstate[8 + tid] |= nb;
        dstate[tid] = 0u;
        while (nb) {
          uint32_t b = __ffs(nb) - 1u;
          R.detect[gw * 32u + b] = (uint32_t)c;
          nb &= nb - 1u;
        }
      }
    }
    // commit (D and reset nets are never register nets, so one pass is
    // safe): a thread moves V words of one register with one vector access
    // per row; the list is ordered so the registers of one wavefront have
    // distinct D and Q residues
    {
      constexpr uint32_t RV = W / Sh::V;
      T* const Sb = reinterpret_cast<T*>(S);
#pragma unroll 4
      for (uint32_t j = tid; j < P.n_regs * RV; j += blockDim.x) {
        const uint4 rr = __ldg(reinterpret_cast<const uint4*>(P.sregs) + j / RV);
        const uint32_t part = j % RV;
        T d = Sb[rr.y * RV + part];
        if (rr.w & 1u) d = reset_select(d, Sb[rr.z * RV + part], rr.w);
        Sb[rr.x * RV + part] = d;
      }
    }
    __syncthreads();
    if (R.has_forces) {
      apply_forces<W>(R, S, tile, 0, stages);
      __syncthreads();
    }
  }
  cta.q = q_end;
  if (!final_settle) {
    for (uint32_t i = tid; i < P.n_src * W; i += blockDim.x) {
      uint32_t k = i / W, ww = i % W;
      R.nets[(size_t)__ldg(P.src_net + k) * R.words_pad + col0 + ww] = S[__ldg(P.src_slot + k) * W + ww];
    }
  }
  __syncthreads();
}

// The whole fused kernel: tiles blockIdx.x, blockIdx.x + gridDim.x, ...
template <int W, bool kSplit>
__device__ __forceinline__ void fused_kernel_body(const GateProgDev& P, const GateRunDev& R) {
  extern __shared__ __align__(128) uint8_t smem[];
  FusedCta cta;
  fused_cta_init(cta, smem);
  for (uint32_t tile = blockIdx.x; tile < R.n_tiles && !cta.aborted; tile += gridDim.x)
    fused_tile<W, kSplit>(P, R, tile, R.cycle_base, R.cycles, R.final_settle != 0, cta);
  fused_cta_drain(cta, R.err);
}

}  // namespace rrtl
