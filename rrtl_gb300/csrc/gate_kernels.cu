// Bit-sliced gate kernels for sm_103a.
//
// Evaluates a GateProgram (see gateprog.h) over many 32-lane words. Each
// cycle follows the run order documented in include/rrtl_cuda.h: stimulus,
// settle (levels), record, register commit, register forces.
//
//  gate_fused_kernel<W>  persistent: one CTA per SM walks tiles of W words; a
//                        tile's nets live in shared memory for all cycles, and
//                        the cell records are streamed level piece by level
//                        piece from HBM/L2 into a shared-memory ring by
//                        cp.async.bulk (TMA bulk copy) with mbarrier completion.
//                        W = 8, 4, 2 or 1: a design with more live nets runs
//                        narrower tiles so that its slots still fit on chip.
//  gate_plain_kernel     one launch per cycle; nets live in HBM, read and
//                        written once per cell per cycle (the baseline path).
//
// Fused warp layout: a group is G = 32/W cells that share one truth table, so
// the table is warp-uniform and evaluates as one LOP3 with an immediate
// table. A thread owns V words of one cell (see FusedShape).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rrtl_cuda.h"
#include "check_log.h"
#include "gate_common.h"
#include "gate_dev.h"
#include "gate_fused.h"
#include "stim.h"

namespace rrtl {

constexpr int kPlainThreads = 256;

template <int W>
__global__ void __launch_bounds__(kFusedThreads, kGateFusedCtasPerSm) gate_fused_kernel(GateProgDev P, GateRunDev R) {
  fused_kernel_body<W, false>(P, R);
}

// Persistent job-queue kernel: CTAs take (job, tile, cycle range) items from
// a device-side list with an atomic counter until the list is empty. Every
// job carries its own program (any tile width), run descriptor and state, so
// uneven jobs share one launch; items are listed longest first.
__global__ void __launch_bounds__(kFusedThreads, kGateFusedCtasPerSm) gate_queue_kernel(GateQueueDev Q) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ uint32_t s_item;
  __shared__ GateJobDev s_job;
  FusedCta cta;
  fused_cta_init(cta, smem);
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(Q.next, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    if (it >= Q.n_items) break;
    const GateItemDev item = Q.items[it];
    // stage the job descriptor; the barrier also orders the s_item read before its next write
    for (uint32_t i = threadIdx.x; i < sizeof(GateJobDev) / 4; i += blockDim.x)
      reinterpret_cast<uint32_t*>(&s_job)[i] = reinterpret_cast<const uint32_t*>(Q.jobs + item.job)[i];
    __syncthreads();
    const uint64_t c0 = item.c0;
    const bool fin = (item.flags & 1u) != 0;
    switch (s_job.P.group) {
      case 4: fused_tile<8, false>(s_job.P, s_job.R, item.tile, c0, item.ncyc, fin, cta); break;
      case 8: fused_tile<4, false>(s_job.P, s_job.R, item.tile, c0, item.ncyc, fin, cta); break;
      case 16: fused_tile<2, false>(s_job.P, s_job.R, item.tile, c0, item.ncyc, fin, cta); break;
      default: fused_tile<1, false>(s_job.P, s_job.R, item.tile, c0, item.ncyc, fin, cta); break;
    }
    if (cta.aborted) break;
  }
  fused_cta_drain(cta, Q.next + 1);
}

// ------------------------------------------------------------ plain path --

// One launch = one cycle (phase 0) or one settle with no stimulus/commit
// (phase 1). Tiles are 8 words; a warp evaluates 4 consecutive cells x 8
// words (a group of G >= 4 cells is G/4 such quads).
__global__ void __launch_bounds__(kPlainThreads) gate_plain_kernel(GateProgDev P, GateRunDev R, uint64_t c,
                                                                    int phase) {
  __shared__ unsigned long long hacc;
  __shared__ uint32_t diff[8];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const uint32_t w = lane & 7u, gsub = lane >> 3;
  const uint32_t tile = blockIdx.x, col0 = tile * 8u, col = col0 + w;
  uint32_t* G = R.nets;
  const size_t wp = R.words_pad;
  const uint32_t stages = P.n_levels + 1;
  const uint32_t quads_per_group = P.group / 4u;
  if (tid == 0) hacc = 0ull;
  if (tid < 8) diff[tid] = 0u;
  if (phase == 0) {
    for (uint32_t i = tid; i < R.n_stim * 8u; i += blockDim.x) {
      const GateStimDev& s = R.stim[i >> 3];
      if (s.kind == RRTL_STIM_HOLD) continue;
      uint32_t ww = i & 7u;
      uint32_t* p = G + (size_t)s.net * wp + col0 + ww;
      *p = stim_value(s, R, c, col0 + ww, *p);
    }
  }
  __syncthreads();
  for (uint32_t L = 0; L < P.n_levels; ++L) {
    uint32_t q0 = P.level_group_begin[L] * quads_per_group, q1 = P.level_group_begin[L + 1] * quads_per_group;
    for (uint32_t qd = q0 + warp; qd < q1; qd += nwarps) {
      uint4 r = P.grecs[(size_t)qd * 4 + gsub];
      uint32_t va = G[(size_t)r.x * wp + col], vb = G[(size_t)r.y * wp + col], vc = G[(size_t)r.z * wp + col];
      G[(size_t)(r.w & 0xFFFFFFu) * wp + col] = lut_eval(r.w >> 24, va, vb, vc);
    }
    __syncthreads();
    if (R.has_forces) {
      const uint32_t* off = R.force_off + (size_t)tile * (stages + 1);
      for (uint32_t i = off[L + 1] + tid; i < off[L + 2]; i += blockDim.x) {
        GateForceDev f = R.forces[i];
        uint32_t& v = G[(size_t)f.net * wp + col0 + f.word];
        v = (v & ~f.mask) | (f.val & f.mask);
      }
      __syncthreads();
    }
  }
  if (phase != 0) return;
  if (R.n_rec) {
    unsigned long long h = 0ull;
    for (uint32_t i = tid; i < R.n_rec * 8u; i += blockDim.x) {
      uint32_t k = i >> 3, ww = i & 7u, gw = col0 + ww;
      uint32_t v = G[(size_t)R.rec[k].net * wp + gw] & valid_mask(gw, R.lanes);
      if (gw < R.words) {
        if (R.mode & RRTL_REC_TRACE) R.out_trace[((size_t)c * R.n_rec + k) * R.words + gw] = v;
        if (R.mode & RRTL_REC_HASH) h += hash_term(c, k, R.word_base + gw, v);
        if (R.mode & RRTL_REC_DETECT) atomicOr(&diff[ww], v ^ (0u - (v & 1u)));
        if (R.mode & RRTL_REC_CHECK) check_word(R, c, k, gw, v);
      }
    }
    if (R.mode & RRTL_REC_HASH) {
      for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xFFFFFFFFu, h, o);
      if (lane == 0 && h) atomicAdd(&hacc, h);
    }
    __syncthreads();
    if (tid == 0 && (R.mode & RRTL_REC_HASH) && hacc) atomicAdd(R.out_hash + c, hacc);
    if ((R.mode & RRTL_REC_DETECT) && tid < 8u) {
      uint32_t gw = col0 + tid;
      uint32_t nb = diff[tid] & valid_mask(gw, R.lanes);
      while (nb) {
        uint32_t b = __ffs(nb) - 1u;
        uint32_t* d = R.detect + gw * 32u + b;
        if (*d == 0xFFFFFFFFu) *d = (uint32_t)c;
        nb &= nb - 1u;
      }
    }
    __syncthreads();
  }
  for (uint32_t i = tid; i < P.n_regs * 8u; i += blockDim.x) {
    GateRegDev r = P.gregs[i >> 3];
    uint32_t ww = i & 7u;
    uint32_t d = G[(size_t)r.d * wp + col0 + ww];
    if (r.flags & 1u) {
      uint32_t m = G[(size_t)r.rst * wp + col0 + ww];
      if (r.flags & 2u) m = ~m;
      uint32_t rv = (r.flags & 4u) ? 0xFFFFFFFFu : 0u;
      d = (m & rv) | (~m & d);
    }
    G[(size_t)r.q * wp + col0 + ww] = d;
  }
  if (R.has_forces) {
    __syncthreads();
    const uint32_t* off = R.force_off + (size_t)tile * (stages + 1);
    for (uint32_t i = off[0] + tid; i < off[1]; i += blockDim.x) {
      GateForceDev f = R.forces[i];
      uint32_t& v = G[(size_t)f.net * wp + col0 + f.word];
      v = (v & ~f.mask) | (f.val & f.mask);
    }
  }
}

// ------------------------------------------------------------- launchers --

size_t gate_fused_smem_bytes(const GateProgDev& P) {
  const uint32_t W = 32u / P.group;
  return kFusedHeader + (size_t)kRing * P.ring_bytes + fused_slot_bytes(P.n_slots, W) +
         (size_t)P.n_pieces * sizeof(GatePieceDev);
}
static_assert(sizeof(GatePieceDev) == 32, "piece descriptor layout");

template <int W>
static cudaError_t fused_prepare_w(size_t smem) {
  return cudaFuncSetAttribute(gate_fused_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t gate_fused_prepare(const GateProgDev& P, size_t smem) {
  switch (P.group) {
    case 4: return fused_prepare_w<8>(smem);
    case 8: return fused_prepare_w<4>(smem);
    case 16: return fused_prepare_w<2>(smem);
    case 32: return fused_prepare_w<1>(smem);
    default: return cudaErrorInvalidValue;
  }
}

// Resident CTAs of the fused kernel per SM at `smem` bytes of shared memory.
template <int W>
static int fused_ctas_w(size_t smem) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gate_fused_kernel<W>, kFusedThreads, smem) != cudaSuccess) n = 1;
  return n > 0 ? n : 1;
}

int gate_fused_ctas_per_sm(const GateProgDev& P, size_t smem) {
  switch (P.group) {
    case 4: return fused_ctas_w<8>(smem);
    case 8: return fused_ctas_w<4>(smem);
    case 16: return fused_ctas_w<2>(smem);
    default: return fused_ctas_w<1>(smem);
  }
}

cudaError_t launch_gate_fused(const GateProgDev& P, const GateRunDev& R, uint32_t grid, size_t smem,
                              cudaStream_t st) {
  switch (P.group) {
    case 4: gate_fused_kernel<8><<<grid, kFusedThreads, smem, st>>>(P, R); break;
    case 8: gate_fused_kernel<4><<<grid, kFusedThreads, smem, st>>>(P, R); break;
    case 16: gate_fused_kernel<2><<<grid, kFusedThreads, smem, st>>>(P, R); break;
    case 32: gate_fused_kernel<1><<<grid, kFusedThreads, smem, st>>>(P, R); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

size_t gate_queue_static_smem() {
  cudaFuncAttributes a{};
  if (cudaFuncGetAttributes(&a, gate_queue_kernel) != cudaSuccess) return 1024;
  return a.sharedSizeBytes;
}

cudaError_t gate_queue_prepare(size_t smem) {
  return cudaFuncSetAttribute(gate_queue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_gate_queue(const GateQueueDev& Q, uint32_t grid, size_t smem, cudaStream_t st) {
  gate_queue_kernel<<<grid, kFusedThreads, smem, st>>>(Q);
  return cudaGetLastError();
}

cudaError_t launch_gate_plain(const GateProgDev& P, const GateRunDev& R, uint64_t c, int phase, cudaStream_t st) {
  gate_plain_kernel<<<R.n_tiles, kPlainThreads, 0, st>>>(P, R, c, phase);
  return cudaGetLastError();
}

// Self-check of the bounded wait the fused and queue kernels use: one thread
// waits `limit` polls on an mbarrier that nothing arrives on, so the wait
// must give up; then it arrives once and waits again with the kernels' own
// limit, which must complete at once. out[0]: RRTL_E_TIMEOUT when the first
// wait gave up (RRTL_OK if it did not); out[1]: 1 when the second wait
// completed. No copy is ever in flight.
__global__ void mbar_wait_check_kernel(uint32_t limit, uint32_t* out) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  out[0] = mbar_wait(&bar, 0, limit) ? (uint32_t)RRTL_OK : (uint32_t)RRTL_E_TIMEOUT;
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
  out[1] = mbar_wait(&bar, 0) ? 1u : 0u;
}

cudaError_t launch_mbar_wait_check(uint32_t limit, uint32_t* out, cudaStream_t st) {
  mbar_wait_check_kernel<<<1, 32, 0, st>>>(limit, out);
  return cudaGetLastError();
}

}  // namespace rrtl
