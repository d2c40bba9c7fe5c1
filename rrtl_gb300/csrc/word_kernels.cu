// Lane-per-thread word kernel for sm_103a (general designs: multi-bit values,
// memories, asynchronous resets). One thread simulates one lane through the
// whole run; lanes never communicate, so the kernel has no barriers. Signals
// and memories are word-major [word][lane] in HBM, so the 32 lanes of a warp
// touch one contiguous 128-byte line per access. Value slots of the current
// block live in shared memory ([slot][thread], conflict-free) or, when a
// design needs more slots than fit, in a spill array in HBM.
//
// Operation semantics follow eval_machine_instr_lane and its limb helpers
// (crates/rrtl-sim-ir/src/lib.rs:9796-9907, 12942-13196) for values of at
// most 128 bits (those past 64 bits in slot pairs, computed on 128-bit
// integers): every result is masked to its width.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "../../include/rrtl_cuda.h"
#include "runtime.h"
#include "word_dev.h"
#include "word_lane.h"

namespace rrtl {

__device__ __forceinline__ unsigned long long wmask(uint32_t w) { return w >= 64u ? ~0ull : ((1ull << w) - 1ull); }

struct WordLane {
  const WordProgDev& P;
  const WordRunDev& R;
  unsigned long long* vbase;
  uint32_t vstride;
  uint32_t lane;
  size_t LP;
  uint32_t* sv;   // this lane's signal values: shared memory [word][block] or HBM [word][lanes_pad]
  size_t svs;     // their word stride

  __device__ unsigned long long& V(uint32_t s) const { return vbase[(size_t)s * vstride]; }
  __device__ uint32_t& SV(uint32_t off) const { return sv[(size_t)off * svs]; }
  __device__ uint32_t get(uint32_t off) const { return SV(off); }
  __device__ void set(uint32_t off, uint32_t v) const { SV(off) = v; }

  __device__ unsigned long long load_sig(uint32_t off, bool two) const {
    unsigned long long v = SV(off);
    if (two) v |= (unsigned long long)SV(off + 1) << 32;
    return v;
  }
  __device__ void store_sig(uint32_t off, bool two, unsigned long long v) const {
    SV(off) = (uint32_t)v;
    if (two) SV(off + 1) = (uint32_t)(v >> 32);
  }
  __device__ bool reset_asserted(uint32_t off, bool active_low) const {
    bool b = SV(off) & 1u;
    return active_low ? !b : b;
  }

  // ---- values of 65 to 128 bits (slot pairs, see kWWide)
  typedef unsigned __int128 u128;
  __device__ static u128 wmask2(uint32_t w) { return w >= 128u ? ~(u128)0 : (((u128)1 << w) - 1u); }
  __device__ u128 W2(uint16_t s, bool pair) const {
    return pair ? (((u128)V(s + 1u) << 64) | (u128)V(s)) : (u128)V(s);
  }
  __device__ void set2(uint16_t s, bool pair, u128 x) const {
    V(s) = (unsigned long long)x;
    if (pair) V(s + 1u) = (unsigned long long)(x >> 64);
  }
  __device__ u128 load_limbs(uint32_t off, uint32_t limbs) const {
    u128 v = 0;
    for (uint32_t l = 0; l < limbs; ++l) v |= (u128)SV(off + l) << (32u * l);
    return v;
  }
  __device__ void store_limbs(uint32_t off, uint32_t limbs, u128 v) const {
    for (uint32_t l = 0; l < limbs; ++l) SV(off + l) = (uint32_t)(v >> (32u * l));
  }
  // decode_usize (crates/rrtl-sim-ir/src/lib.rs:12989-13008): an address past 64 bits saturates
  __device__ static unsigned long long addr_of(u128 a) { return (a >> 64) ? ~0ull : (unsigned long long)a; }
  __device__ u128 mem_load(const WMemDev& M, unsigned long long addr) const {
    u128 r = 0;
    const size_t w0 = (size_t)M.offset + (size_t)addr * M.limbs;
    for (uint32_t l = 0; l < M.limbs; ++l) r |= (u128)R.mems[(w0 + l) * LP + lane] << (32u * l);
    return r & wmask2(M.width);
  }

  // One wide instruction: the narrow semantics below on 128-bit values.
  __device__ void run_wide(const WInstr& I) const {
    const u128 m = wmask2(I.width);
    const u128 a = W2(I.a, I.flags & kWPairA), b = W2(I.b, I.flags & kWPairB);
    u128 r = 0;
    switch (I.op) {
      case W_LIT: r = (((u128)__ldg(P.lits + I.aux + 1u) << 64) | __ldg(P.lits + I.aux)) & m; break;
      case W_SIG: r = load_limbs(I.aux, I.c) & m; break;
      case W_NOT: r = ~a & m; break;
      case W_AND: r = (a & b) & m; break;
      case W_OR: r = (a | b) & m; break;
      case W_XOR: r = (a ^ b) & m; break;
      case W_ADD: r = (a + b) & m; break;
      case W_SUB: r = (a - b) & m; break;
      case W_MUL: r = (a * b) & m; break;
      case W_EQ: r = a == b; break;
      case W_NE: r = a != b; break;
      case W_LT: {
        const u128 om = wmask2(I.aux);
        r = (a & om) < (b & om);
        break;
      }
      case W_LTS: {
        if (I.aux == 0u) break;
        const u128 om = wmask2(I.aux), sb = (u128)1 << (I.aux - 1u);
        const u128 x = a & om, y = b & om;
        const bool xs = (x & sb) != 0, ys = (y & sb) != 0;
        r = (xs != ys) ? (u128)xs : (u128)(x < y);
        break;
      }
      case W_MUX: r = (((unsigned long long)a & 1ull) ? b : W2(I.c, I.flags & kWPairC)) & m; break;
      case W_SLICE: r = I.aux >= 128u ? (u128)0 : ((a >> I.aux) & m); break;
      case W_MASK: r = a & m; break;
      case W_SEXT: {
        if (I.aux == 0u) break;
        const u128 x = a & wmask2(I.aux);
        r = ((((x >> (I.aux - 1u)) & 1u) != 0) ? (x | ~wmask2(I.aux)) : x) & m;
        break;
      }
      case W_CAT: r = ((I.aux >= 128u ? (u128)0 : (a << I.aux)) | b) & m; break;
      case W_MEMRD: {
        const WMemDev M = P.mems[I.aux];
        const unsigned long long addr = addr_of(a);
        if (addr < M.depth) r = mem_load(M, addr) & m;
        break;
      }
      case W_STORE: store_limbs(I.aux, I.c, a & m); return;
      case W_ASTORE:
        if (reset_asserted(I.aux2, I.flags & 4)) store_limbs(I.aux, I.c, a & m);
        return;
      case W_CAPTURE: {
        u128 v = a;
        if ((I.flags & 2) && reset_asserted(I.aux2, I.flags & 4))
          v = ((u128)__ldg(P.lits + I.aux3 + 1u) << 64) | __ldg(P.lits + I.aux3);
        v &= m;
        for (uint32_t l = 0; l < I.c; ++l) R.caps[(size_t)(I.aux + l) * LP + lane] = (uint32_t)(v >> (32u * l));
        return;
      }
      case W_MEMWR: {
        if ((unsigned long long)a & 1ull) {
          const WMemDev M = P.mems[I.aux];
          const unsigned long long addr = addr_of(b);
          if (addr < M.depth) {
            const u128 v = W2(I.c, I.flags & kWPairC) & wmask2(M.width);
            const size_t w0 = (size_t)M.offset + (size_t)addr * M.limbs;
            for (uint32_t l = 0; l < M.limbs; ++l) R.mems[(w0 + l) * LP + lane] = (uint32_t)(v >> (32u * l));
          }
        }
        return;
      }
      default: return;
    }
    set2(I.dst, I.flags & kWPairD, r);
  }

  __device__ void run(uint32_t b, uint32_t e) const {
    for (uint32_t pc = b; pc < e; ++pc) {
      const WInstr I = P.code[pc];
      if (I.flags & kWWide) {
        run_wide(I);
        continue;
      }
      const unsigned long long m = wmask(I.width);
      unsigned long long r = 0;
      switch (I.op) {
        case W_LIT: r = __ldg(P.lits + I.aux) & m; break;
        case W_SIG: r = load_sig(I.aux, I.flags & 1) & m; break;
        case W_NOT: r = ~V(I.a) & m; break;
        case W_AND: r = (V(I.a) & V(I.b)) & m; break;
        case W_OR: r = (V(I.a) | V(I.b)) & m; break;
        case W_XOR: r = (V(I.a) ^ V(I.b)) & m; break;
        case W_ADD: r = (V(I.a) + V(I.b)) & m; break;
        case W_SUB: r = (V(I.a) - V(I.b)) & m; break;
        case W_MUL: r = (V(I.a) * V(I.b)) & m; break;
        case W_EQ: r = V(I.a) == V(I.b); break;
        case W_NE: r = V(I.a) != V(I.b); break;
        case W_LT: {
          unsigned long long om = wmask(I.aux);
          r = (V(I.a) & om) < (V(I.b) & om);
          break;
        }
        case W_LTS: {
          unsigned long long om = wmask(I.aux);
          unsigned long long x = V(I.a) & om, y = V(I.b) & om;
          unsigned long long sb = 1ull << (I.aux - 1u);
          bool xs = x & sb, ys = y & sb;
          r = (xs != ys) ? (unsigned long long)xs : (unsigned long long)(x < y);
          break;
        }
        case W_MUX: r = ((V(I.a) & 1ull) ? V(I.b) : V(I.c)) & m; break;
        case W_SLICE: r = I.aux >= 64u ? 0ull : ((V(I.a) >> I.aux) & m); break;
        case W_MASK: r = V(I.a) & m; break;
        case W_SEXT: {
          unsigned long long x = V(I.a) & wmask(I.aux);
          bool s = (x >> (I.aux - 1u)) & 1ull;
          r = (s ? (x | ~wmask(I.aux)) : x) & m;
          break;
        }
        case W_CAT: r = ((I.aux >= 64u ? 0ull : (V(I.a) << I.aux)) | V(I.b)) & m; break;
        case W_MEMRD: {
          const WMemDev M = P.mems[I.aux];
          unsigned long long addr = V(I.a);
          if (addr < M.depth) {
            size_t w0 = (size_t)M.offset + (size_t)addr * M.limbs;
            r = R.mems[w0 * LP + lane];
            if (M.limbs == 2) r |= (unsigned long long)R.mems[(w0 + 1) * LP + lane] << 32;
            r &= wmask(M.width) & m;
          }
          break;
        }
        case W_STORE: store_sig(I.aux, I.flags & 1, V(I.a) & m); continue;
        case W_ASTORE:
          if (reset_asserted(I.aux2, I.flags & 4)) store_sig(I.aux, I.flags & 1, V(I.a) & m);
          continue;
        case W_CAPTURE: {
          unsigned long long v = ((I.flags & 2) && reset_asserted(I.aux2, I.flags & 4)) ? __ldg(P.lits + I.aux3) : V(I.a);
          v &= m;
          R.caps[(size_t)I.aux * LP + lane] = (uint32_t)v;
          if (I.flags & 1) R.caps[(size_t)(I.aux + 1) * LP + lane] = (uint32_t)(v >> 32);
          continue;
        }
        case W_MEMWR: {
          if (V(I.a) & 1ull) {
            const WMemDev M = P.mems[I.aux];
            unsigned long long addr = V(I.b);
            if (addr < M.depth) {
              unsigned long long v = V(I.c) & wmask(M.width);
              size_t w0 = (size_t)M.offset + (size_t)addr * M.limbs;
              R.mems[w0 * LP + lane] = (uint32_t)v;
              if (M.limbs == 2) R.mems[(w0 + 1) * LP + lane] = (uint32_t)(v >> 32);
            }
          }
          continue;
        }
        default: continue;
      }
      V(I.dst) = r;
    }
  }

  __device__ void commit() const {
    for (uint32_t k = 0; k < P.n_commits; ++k) {
      const WCommitDev cm = P.commits[k];
      for (uint32_t l = 0; l < cm.limbs; ++l)
        SV(cm.sig_off + l) = R.caps[(size_t)(cm.cap_off + l) * LP + lane];
    }
  }

  __device__ void settle() const {
    run(P.comb_b, P.comb_e);
    run(P.async_b, P.async_e);
  }
  __device__ void edge() const {
    run(P.next_b, P.next_e);
    run(P.commit_b, P.commit_e);
    commit();
  }
};

// One lane through one launch's cycles (the body shared by the single-run
// and the multi-job kernels).
// Shared memory of a word block: [value slots: n_vslots][block] (u64) then,
// with sig_smem, [signal words: n_sig_words][block] (u32).
template <bool kSmem>
__device__ __forceinline__ void word_lane_run(const WordProgDev& P, const WordRunDev& R, uint32_t lane,
                                              unsigned long long* vsm) {
  uint32_t* ssm = reinterpret_cast<uint32_t*>(vsm + (size_t)P.n_vslots * blockDim.x) + threadIdx.x;
  const bool sig_smem = kSmem && P.sig_smem;
  WordLane W{P, R, kSmem ? vsm + threadIdx.x : R.vspill + lane, kSmem ? blockDim.x : R.lanes_pad, lane, R.lanes_pad,
             sig_smem ? ssm : R.values + lane, sig_smem ? (size_t)blockDim.x : (size_t)R.lanes_pad};
  if (sig_smem)
    for (uint32_t w = 0; w < P.n_sig_words; ++w) ssm[(size_t)w * blockDim.x] = R.values[(size_t)w * R.lanes_pad + lane];
  word_lane_cycles(R, lane, W, WordRunSpec{R.stim, R.rec, R.n_stim, R.n_rec, R.mode});
  if (sig_smem)
    for (uint32_t w = 0; w < P.n_sig_words; ++w) R.values[(size_t)w * R.lanes_pad + lane] = ssm[(size_t)w * blockDim.x];
}

// Dynamic shared memory a word block needs (value slots, staged signals).
__host__ __device__ inline size_t word_block_smem(const WordProgDev& P, uint32_t threads) {
  return (size_t)P.n_vslots * threads * 8u + (P.sig_smem ? (size_t)P.n_sig_words * threads * 4u : 0u);
}

template <bool kSmem>
__global__ void __launch_bounds__(128) word_kernel(WordProgDev P, WordRunDev R) {
  extern __shared__ unsigned long long vsm[];
  word_lane_run<kSmem>(P, R, blockIdx.x * blockDim.x + threadIdx.x, vsm);
}

// Many word-engine runs in one launch: block b belongs to the job whose block
// range holds it (jobs sorted by block_begin). Used by the serving loop so the
// word-engine requests of a round run side by side.
__global__ void __launch_bounds__(128) word_multi_kernel(const WordJobDev* __restrict__ jobs, uint32_t n_jobs) {
  extern __shared__ unsigned long long vsm[];
  __shared__ WordJobDev s_job;
  __shared__ uint32_t s_j;
  if (threadIdx.x == 0) {
    uint32_t lo = 0, hi = n_jobs;  // last job with block_begin <= blockIdx.x
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (jobs[mid].block_begin <= blockIdx.x) lo = mid;
      else hi = mid;
    }
    s_j = lo;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < sizeof(WordJobDev) / 4; i += blockDim.x)
    reinterpret_cast<uint32_t*>(&s_job)[i] = reinterpret_cast<const uint32_t*>(jobs + s_j)[i];
  __syncthreads();
  word_lane_run<true>(s_job.P, s_job.R, (blockIdx.x - s_job.block_begin) * blockDim.x + threadIdx.x, vsm);
}

cudaError_t launch_word_multi(const WordJobDev* jobs, uint32_t n_jobs, uint32_t blocks, size_t smem, cudaStream_t st) {
  word_multi_kernel<<<blocks, 128, smem, st>>>(jobs, n_jobs);
  return cudaGetLastError();
}

cudaError_t word_multi_prepare(size_t smem) {
  return cudaFuncSetAttribute(word_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_word(const WordProgDev& P, const WordRunDev& R, bool smem_slots, cudaStream_t st) {
  const uint32_t threads = 128;
  uint32_t grid = R.lanes_pad / threads;
  if (smem_slots) {
    word_kernel<true><<<grid, threads, word_block_smem(P, threads), st>>>(P, R);
  } else {
    word_kernel<false><<<grid, threads, 0, st>>>(P, R);
  }
  return cudaGetLastError();
}

cudaError_t word_prepare(size_t smem) {
  return cudaFuncSetAttribute(word_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// ---------------------------------------------------------------------------
// Allocation-free tick_many.
//
// Some callers cannot call cudaMalloc or cudaFree: a serving process that has
// divided device memory among tenants up front and forbids any further
// allocation, or a latency-critical loop that must not risk the implicit
// device-wide synchronisation cudaFree (and at times cudaMalloc) performs.
// rrtl_word_tick_many_noalloc serves them: the caller owns the lane state, and
// the only scratch the kernel needs, the register capture buffer plus a status
// word, lives in the fixed device array below.
//
// The array is file-scope device memory of fixed size, loaded with the
// library and held by every GPU that loads it until the process exits. All
// calls share it and it keeps the last call's contents; captures are written
// before they are read every cycle and the status word is cleared at the
// start of each call, so nothing else needs clearing. Two calls whose work
// overlaps on the GPU (different streams, threads or contexts of the same
// device) race on this array and corrupt each other's results.

constexpr size_t kNoAllocScratchWords = (size_t)1 << 20;  // 4 MiB of capture words
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords + 64];

void set_last_error(const std::string& msg);

// Host code cannot use the array's name as a device address: the name is a
// host-side stand-in. rrtl_ctx_create calls this once per context, with the
// context's device current, and keeps the address in the context, so the
// address is never used past the context (and the device context) it was
// looked up in.
cudaError_t noalloc_scratch_lookup(uint32_t** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<uint32_t*>(p);
  return cudaSuccess;
}

namespace {
// Whether p is memory the design's device can dereference as ordinary device
// memory (a cudaMalloc or managed allocation of that device).
bool device_pointer_of(const void* p, int device) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();  // clear the (non-sticky) error an unknown pointer leaves
    return false;
  }
  if (a.type == cudaMemoryTypeDevice) return a.device == device;
  if (a.type == cudaMemoryTypeManaged) return true;
  return false;
}
}  // namespace

}  // namespace rrtl

extern "C" rrtl_status rrtl_word_tick_many_noalloc(rrtl_design* d, uint32_t* values, uint32_t* memories,
                                                   uint32_t lanes, uint64_t steps) {
  using namespace rrtl;
  auto fail_with = [](rrtl_status st, const std::string& msg) {
    set_last_error(msg);
    return st;
  };
  if (!d || !values) return fail_with(RRTL_E_ARG, "E_ARG: null argument");
  if (d->engine != RRTL_ENGINE_WORD) return fail_with(RRTL_E_UNSUPPORTED, "E_NOALLOC: the design runs on the gate engine");
  if (lanes == 0) return fail_with(RRTL_E_LANES, "E_GPU_LANES: GPU simulator requires at least one lane");
  if (steps >= (1ull << 32)) return fail_with(RRTL_E_ARG, "E_GPU_STEPS: tick_many step count exceeds 2^32");
  if (d->mp.source.total_memory_words_per_lane > 0 && !memories) return fail_with(RRTL_E_ARG, "E_ARG: memories is null");
  if ((size_t)d->wdev.n_vslots * 128u * 8u > 96u * 1024u)
    return fail_with(RRTL_E_UNSUPPORTED, "E_WORD_SCOPE: design needs more live value slots than shared memory holds");
  // padded in 64 bits: lanes near 2^32 must not wrap to a zero-sized request
  const uint64_t lanes_pad = ((uint64_t)lanes + 127u) / 128u * 128u;
  if (lanes_pad > 0xFFFFFF80ull)
    return fail_with(RRTL_E_LANES, "E_GPU_LANES: " + std::to_string(lanes) + " lanes exceed the padded-lane limit");
  const uint64_t cap_words = (uint64_t)d->wp.total_capture_words * lanes_pad;
  if (cap_words > kNoAllocScratchWords)
    return fail_with(RRTL_E_ARG, "E_NOALLOC_SIZE: " + std::to_string(d->wp.total_capture_words) + " capture words x " +
                                     std::to_string(lanes_pad) + " padded lanes exceed the fixed scratch of " +
                                     std::to_string(kNoAllocScratchWords) + " words");
  cudaError_t e = cudaSetDevice(d->ctx->device);
  if (e != cudaSuccess) return fail_with(RRTL_E_DEVICE, std::string("E_DEVICE: ") + cudaGetErrorString(e));
  // the kernel dereferences these: host memory or another device's memory is
  // refused before anything is launched
  if (!device_pointer_of(values, d->ctx->device))
    return fail_with(RRTL_E_ARG, "E_ARG: values is not device memory of the design's device");
  if (memories && !device_pointer_of(memories, d->ctx->device))
    return fail_with(RRTL_E_ARG, "E_ARG: memories is not device memory of the design's device");
  uint32_t* scratch = d->ctx->noalloc_scratch;
  if (!scratch) return fail_with(RRTL_E_DEVICE, "E_DEVICE: the context has no scratch address");
  uint32_t* status = scratch + kNoAllocScratchWords;
  cudaStream_t st = d->ctx->stream;
  e = cudaMemsetAsync(status, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return fail_with(RRTL_E_DEVICE, std::string("E_DEVICE: ") + cudaGetErrorString(e));
  WordRunDev R{};
  R.cycles = steps;
  R.lanes = lanes;
  R.lanes_pad = (uint32_t)lanes_pad;
  R.values = values;
  R.mems = memories;
  R.caps = scratch;
  R.start_settle = 1;
  R.final_settle = 1;
  R.err = status;
  if (steps > 0) {
    e = launch_word(d->wdev, R, true, st);
    if (e != cudaSuccess) return fail_with(RRTL_E_DEVICE, std::string("E_DEVICE: word_kernel: ") + cudaGetErrorString(e));
  }
  uint32_t err = 0;
  e = cudaMemcpyAsync(&err, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail_with(RRTL_E_DEVICE, std::string("E_DEVICE: ") + cudaGetErrorString(e));
  if (err) return fail_with((rrtl_status)err, "E_TIMEOUT: a bounded device wait gave up");
  set_last_error("");
  return RRTL_OK;
}
