// day_phase.cu — the per-tick Day Phase kernels for sm_103a.
//
// One tick (reference order: genesis-compute/src/cuda/physics.cu:441-495):
//
//   k_incoming  network spike ids -> per-axon push counts      (physics.cu:114-132)
//   k_axons     input-bitmask pushes + network pushes + propagation of all
//               eight heads, and the tick's segment-hit mask    (physics.cu:88-108,137-154)
//   k_update    burst reset + GLIF soma update + dendrite gather/sum, spike
//               compaction into the shard's spiker list        (physics.cu:25-30,159-276)
//   k_push      the spikers' own-axon pushes, readout           (physics.cu:257-261,378-395)
//   k_gsop      GSOP plasticity, one warp per spiker           (physics.cu:281-373)
//
// Snapshot semantics: k_update reads the heads as left by k_axons; the soma
// pushes are applied by k_push, after every neuron was updated and before
// GSOP (the reference pushes inside its update kernel and so races with the
// reads of other neurons, physics.cu:194 vs :257-261).
//
// The segment-hit mask (one u32 per axon) lets the dendrite gather read 4
// bytes per slot instead of a 32-byte BurstHeads8.  Bit s (s < 31) is set
// when some head h satisfies (u32)(h - s) < Pmax, bit 31 when some segment
// s >= 31 could be hit; Pmax is the largest signal_propagation_length in
// the LUT.  A clear bit proves "no hit" for every variant; a set bit is a
// hit for variants whose length equals Pmax, and any other case re-tests
// the eight heads exactly.
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace axc {

__constant__ VariantParameters VARIANT_LUT[16];

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

__device__ __forceinline__ uint32_t lut_pmax() {
  uint32_t m = 0;
#pragma unroll
  for (int v = 0; v < 16; v++) m = max(m, (uint32_t)VARIANT_LUT[v].signal_propagation_length);
  return m;
}

__device__ __forceinline__ void lut_to_smem(VariantParameters* dst) {
  const uint32_t* s = reinterpret_cast<const uint32_t*>(VARIANT_LUT);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  for (int i = threadIdx.x; i < 256; i += blockDim.x) d[i] = s[i];
}

// push_burst_head applied c times (physics.cu:32-41): shift by c, zeros in.
__device__ __forceinline__ void push_n(uint32_t h[8], uint32_t c) {
#pragma unroll
  for (uint32_t r = 0; r < 8; r++) {
    if (r < c) {
      h[7] = h[6]; h[6] = h[5]; h[5] = h[4]; h[4] = h[3];
      h[3] = h[2]; h[2] = h[1]; h[1] = h[0]; h[0] = 0u;
    }
  }
}

__device__ __forceinline__ void load_heads(const BurstHeads8* heads, uint32_t a, uint32_t h[8]) {
  const uint4* p = reinterpret_cast<const uint4*>(heads + a);
  uint4 x = __ldg(p), y = __ldg(p + 1);
  h[0] = x.x; h[1] = x.y; h[2] = x.z; h[3] = x.w; h[4] = y.x; h[5] = y.y; h[6] = y.z; h[7] = y.w;
}

// physics.cu:198-201
__device__ __forceinline__ bool heads_hit(const BurstHeads8* heads, uint32_t a, uint32_t s, uint32_t prop) {
  uint32_t h[8];
  load_heads(heads, a, h);
  bool hit = false;
#pragma unroll
  for (int k = 0; k < 8; k++) hit |= (h[k] - s) < prop;
  return hit;
}

__device__ __forceinline__ uint32_t seg_mask_of(const uint32_t h[8], uint32_t P) {
  uint32_t m = 0;
  if (P == 0) return 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    uint32_t x = h[k];
    if (x < 255u + P) {
      uint32_t lo = (x + 1u > P) ? x + 1u - P : 0u;
      if (lo <= 30u) {
        uint32_t top = min(x, 30u);
        m |= ((2u << top) - 1u) & ~((1u << lo) - 1u);
      }
      if (x >= 31u) m |= 0x80000000u;
    }
  }
  return m;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
  return v;
}

// Sums up to three per-thread counters over the block into ctl->ctr[i0..].
__device__ __forceinline__ void block_count(unsigned long long a, unsigned long long b,
                                            unsigned long long c, unsigned long long* dst) {
  __shared__ unsigned long long red[3][32];
  a = warp_sum(a); b = warp_sum(b); c = warp_sum(c);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();  // a previous call's reader is done with red[]
  if (lane == 0) { red[0][w] = a; red[1][w] = b; red[2][w] = c; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s0 = 0, s1 = 0, s2 = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) { s0 += red[0][i]; s1 += red[1][i]; s2 += red[2][i]; }
    if (s0) atomicAdd(dst + 0, s0);
    if (s1) atomicAdd(dst + 1, s1);
    if (s2) atomicAdd(dst + 2, s2);
  }
}

// ---------------------------------------------------------------------------
// k_incoming — physics.cu:114-132.  Ids >= A are ignored (physics.cu:127);
// duplicates count once per occurrence.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_incoming(const uint32_t* __restrict__ ids, uint32_t count_arg,
                                                  const uint32_t* __restrict__ batch_counts, uint32_t k,
                                                  uint32_t cap, uint32_t A, uint32_t* __restrict__ incoming) {
  uint32_t count = batch_counts ? min(batch_counts[k], cap) : count_arg;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    uint32_t id = ids[i];
    if (id < A) atomicAdd(&incoming[id], 1u);
  }
}

// ---------------------------------------------------------------------------
// k_axons — physics.cu:88-108 (inject), :114-132 (network pushes), :137-154
// (propagate), and the segment-hit mask of the propagated heads.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_axons(BurstHeads8* __restrict__ heads, uint32_t A, uint32_t v_seg,
                                               const uint32_t* __restrict__ bitmask, uint32_t voff, uint32_t nv,
                                               uint32_t* __restrict__ incoming, int use_incoming,
                                               const uint32_t* __restrict__ batch_counts, uint32_t k,
                                               uint32_t* __restrict__ seg_mask, ShardCtl* __restrict__ ctl,
                                               uint32_t raise_err) {
  __shared__ uint32_t s_pmax;
  __shared__ int s_inc;
  if (threadIdx.x == 0) {
    s_pmax = lut_pmax();
    s_inc = use_incoming || (batch_counts && batch_counts[k] > 0);
    if (blockIdx.x == 0) {
      ctl->spike_count = 0;
      ctl->ctr[0] += 1;
      if (raise_err) atomicOr(&ctl->err, raise_err);
    }
  }
  __syncthreads();
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A) return;
  uint4* p = reinterpret_cast<uint4*>(heads + a);
  uint4 x = p[0], y = p[1];
  uint32_t h[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
  uint32_t npush = 0;
  if (bitmask) {
    uint32_t v = a - voff;
    if (v < nv) npush += (__ldg(bitmask + (v >> 5)) >> (v & 31u)) & 1u;
  }
  if (s_inc) {
    uint32_t c = incoming[a];
    if (c) { npush += c; incoming[a] = 0; }
  }
  push_n(h, npush);
#pragma unroll
  for (int j = 0; j < 8; j++)
    if (h[j] != AXC_AXON_SENTINEL) h[j] += v_seg;
  p[0] = make_uint4(h[0], h[1], h[2], h[3]);
  p[1] = make_uint4(h[4], h[5], h[6], h[7]);
  seg_mask[a] = seg_mask_of(h, s_pmax);
}

// ---------------------------------------------------------------------------
// k_update — physics.cu:25-30 (burst reset, folded: every neuron's flags are
// rewritten) and physics.cu:159-276 (GLIF + dendrite gather/sum).
// ---------------------------------------------------------------------------
template <int U>
__global__ void __launch_bounds__(256) k_update(ShardVramPtrs P, uint32_t N, uint32_t A, uint32_t tick_arg,
                                                const uint32_t* __restrict__ seg_mask, uint32_t* __restrict__ pend,
                                                uint32_t* __restrict__ spikers, ShardCtl* __restrict__ ctl,
                                                int batch, uint32_t k) {
  __shared__ VariantParameters lut[16];
  __shared__ uint32_t s_pmax;
  lut_to_smem(lut);
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  const uint32_t tick = batch ? ctl->tick_base + k : tick_arg;
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  int spike = 0;
  uint32_t ev = 0, hits = 0, err = 0, nev = 0;
  if (n < N) {
    const uint8_t flags = P.soma_flags[n];
    const uint8_t timer = P.timers[n];
    const uint8_t ftype = flags & 0xF0;  // burst bits reset (:25-30), spike bit cleared (:168)
    if (timer > 0) {                     // :170-174
      P.timers[n] = (uint8_t)(timer - 1);
      P.soma_flags[n] = ftype;
    } else {
      nev = 1;
      const VariantParameters& p = lut[flags >> 4];
      const uint32_t prop = p.signal_propagation_length;
      const bool mask_exact = prop == s_pmax;
      const uint32_t* tg = P.dendrite_targets + n;
      const int16_t* wt = P.dendrite_weights + n;
      int32_t i_in = 0;
      bool live = true;
      for (uint32_t i = 0; live && i < AXC_MAX_DENDRITES; i += U) {   // :182-206
        uint32_t t[U], m[U], ax[U];
        bool ok[U];
#pragma unroll
        for (int j = 0; j < U; j++) t[j] = __ldg(tg + (size_t)(i + j) * N);
#pragma unroll
        for (int j = 0; j < U; j++) {
          live = live && t[j] != 0;
          ax[j] = (t[j] & AXC_TARGET_AXON_MASK) - 1u;
          ok[j] = live && ax[j] < A;
          ev += live;
          err |= (live && !ok[j]) ? AXC_ERR_TARGET_RANGE : 0u;
          m[j] = ok[j] ? __ldg(seg_mask + ax[j]) : 0u;
        }
#pragma unroll
        for (int j = 0; j < U; j++) {
          if (!ok[j]) continue;
          const uint32_t s = t[j] >> AXC_TARGET_SEG_SHIFT;
          bool hit;
          if (s < 31u) {
            hit = (m[j] >> s) & 1u;
            if (hit && !mask_exact) hit = heads_hit(P.axon_heads, ax[j], s, prop);
          } else {
            hit = (m[j] >> 31) && heads_hit(P.axon_heads, ax[j], s, prop);
          }
          if (hit) {
            i_in = wadd(i_in, (int32_t)__ldg(wt + (size_t)(i + j) * N));
            hits++;
          }
        }
      }
      int32_t thr = P.threshold_offset[n];                           // :209-213
      const int32_t decayed = wsub(thr, (int32_t)p.homeostasis_decay);
      thr = decayed & ~(decayed >> 31);
      int32_t leak = p.leak_rate;                                    // :216-223
      if (p.adaptive_mode == 1) {
        leak = wadd(leak, wmul(thr, (int32_t)p.adaptive_leak_gain) >> 8);
        const int32_t over = wsub(leak, p.adaptive_leak_max);
        leak = wsub(leak, over & ~(over >> 31));
      }
      int32_t v = wadd(P.soma_voltage[n], i_in);                     // :225-235
      const int32_t diff = wsub(v, p.rest_potential);
      const int32_t sign = (diff > 0) - (diff < 0);
      int32_t leaked = wsub(wmul(diff, sign), leak);
      leaked = leaked & ~(leaked >> 31);
      v = wadd(p.rest_potential, wmul(sign, leaked));
      const int32_t glif = v >= wadd(p.threshold, thr) ? 1 : 0;     // :237-245
      const uint32_t period = p.spontaneous_firing_period_ticks;
      const int32_t hb = (period > 0 && ((tick + n * 104729u) % period) == 0) ? 1 : 0;
      spike = glif | hb;
      if (glif) {                                                    // :248-250
        v = p.rest_potential;
        thr = wadd(thr, p.homeostasis_penalty);
      }
      P.soma_voltage[n] = v;                                         // :269-275
      // burst count after the reset is 0; a spike sets bit 1 (:255) and then
      // increments (:271-273), so a spiker's flags are type | 0b101.
      P.soma_flags[n] = (uint8_t)(ftype | (spike ? 0x05 : 0x00));
      P.threshold_offset[n] = thr;
      P.timers[n] = glif ? p.refractory_period : timer;
      if (spike) {                                                   // :257-261 (deferred)
        const uint32_t my_axon = P.soma_to_axon[n];
        if (my_axon != AXC_NO_AXON) {
          if (my_axon < A) atomicAdd(&pend[my_axon], 1u);
          else err |= AXC_ERR_SOMA_AXON;
        }
      }
    }
  }
  // warp-aggregated append to the spiker list (physics.cu:400-434 pattern)
  const uint32_t ballot = __ballot_sync(kFull, spike);
  if (ballot) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&ctl->spike_count, (uint32_t)__popc(ballot));
    base = __shfl_sync(kFull, base, leader);
    if (spike) spikers[base + __popc(ballot & ((1u << lane) - 1u))] = n;
  }
  const uint32_t err_any = __reduce_or_sync(kFull, err);
  if (err_any && (threadIdx.x & 31) == 0) atomicOr(&ctl->err, err_any);
  block_count(ev, hits, (unsigned long long)spike, &ctl->ctr[1]);
  block_count(0, nev, 0, &ctl->ctr[4]);
}

// ---------------------------------------------------------------------------
// k_push — the spikers' own-axon pushes (physics.cu:257-261), once per axon
// with the pushes counted by k_update; readout (physics.cu:378-395).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_push(BurstHeads8* __restrict__ heads, const uint32_t* __restrict__ s2a,
                                              uint32_t A, uint32_t* __restrict__ pend,
                                              const uint32_t* __restrict__ spikers, ShardCtl* __restrict__ ctl,
                                              const uint8_t* __restrict__ flags, uint32_t N,
                                              const uint32_t* __restrict__ ids, uint8_t* __restrict__ out,
                                              uint32_t num_outputs) {
  const uint32_t cnt = ctl->spike_count;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t i = tid; i < cnt; i += stride) {
    const uint32_t ax = s2a[spikers[i]];
    if (ax >= A) continue;
    const uint32_t c = atomicExch(&pend[ax], 0u);
    if (!c) continue;
    uint4* p = reinterpret_cast<uint4*>(heads + ax);
    uint4 x = p[0], y = p[1];
    uint32_t h[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
    push_n(h, c);
    p[0] = make_uint4(h[0], h[1], h[2], h[3]);
    p[1] = make_uint4(h[4], h[5], h[6], h[7]);
  }
  uint32_t err = 0;
  for (uint32_t j = tid; j < num_outputs; j += stride) {
    const uint32_t id = ids[j];
    uint8_t v = 0;
    if (id != AXC_NO_AXON) {
      if (id < N) v = flags[id] & 0x01;
      else err = AXC_ERR_READOUT_RANGE;
    }
    out[j] = v;
  }
  if (err) atomicOr(&ctl->err, err);
}

// ---------------------------------------------------------------------------
// k_gsop — physics.cu:281-373, one warp per spiker; lane L handles slots
// L, L+32, L+64, L+96 up to the first empty target.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gsop(ShardVramPtrs P, uint32_t N, uint32_t A, int16_t dopa_arg,
                                              const uint32_t* __restrict__ spikers, ShardCtl* __restrict__ ctl,
                                              int batch) {
  __shared__ VariantParameters lut[16];
  lut_to_smem(lut);
  __syncthreads();
  const int32_t dopamine = batch ? (int32_t)(int16_t)ctl->dopamine : (int32_t)dopa_arg;
  const uint32_t cnt = ctl->spike_count;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  uint32_t done = 0, err = 0;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < cnt; w += nwarps) {
    const uint32_t n = spikers[w];
    const uint8_t flags = P.soma_flags[n];
    const uint32_t burst = (flags >> 1) & 0x07;                       // :290-291
    const int32_t burst_mult = burst > 0 ? (int32_t)burst : 1;
    const VariantParameters& p = lut[flags >> 4];
    const uint32_t len = p.signal_propagation_length;
    const int32_t pot_mod = wmul(dopamine, (int32_t)p.d1_affinity) >> 7;   // :336-345
    const int32_t dep_mod = wmul(dopamine, (int32_t)p.d2_affinity) >> 7;
    const int32_t raw_pot = wadd((int32_t)p.gsop_potentiation, pot_mod);
    const int32_t raw_dep = wsub((int32_t)p.gsop_depression, dep_mod);
    const int32_t final_dep = raw_dep & ~(raw_dep >> 31);
    for (uint32_t c = 0; c < AXC_MAX_DENDRITES / 32; c++) {
      const size_t col = (size_t)(c * 32 + lane) * N + n;
      const uint32_t t = P.dendrite_targets[col];
      const uint32_t zb = __ballot_sync(kFull, t == 0);
      const uint32_t first = zb ? (uint32_t)(__ffs(zb) - 1) : 32u;
      if (lane < first) {
        const uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
        if (a >= A) {
          err |= AXC_ERR_TARGET_RANGE;
        } else {
          const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
          uint32_t h[8];
          load_heads(P.axon_heads, a, h);
          uint32_t md = 0xFFFFFFFFu;                                 // :311-318
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const uint32_t d = h[q] - s;
            md = min(md, d < len ? d : 0xFFFFFFFFu);
          }
          const bool active = md != 0xFFFFFFFFu;
          const int16_t w16 = P.dendrite_weights[col];               // :322-332
          const int32_t sign = w16 >= 0 ? 1 : -1;
          int32_t abs_w = (int32_t)w16;
          if (abs_w < 0) abs_w = -abs_w;
          uint32_t rank = (uint32_t)abs_w >> 11;
          if (rank > 15) rank = 15;
          const int32_t inertia = p.inertia_curve[rank];
          const int32_t delta_pot = wmul(wmul(raw_pot, inertia), burst_mult) >> 7;   // :348-358
          const int32_t delta_dep = wmul(wmul(final_dep, inertia), burst_mult) >> 7;
          const uint32_t cs = active ? (md >> 4) : 0u;
          int32_t delta = active ? (delta_pot >> cs) : wsub(0, delta_dep);
          delta = wmul(delta, 128) >> (7u + cs);
          int32_t new_abs = wadd(abs_w, delta);                      // :361-371
          new_abs = new_abs & ~(new_abs >> 31);
          if (new_abs > 32767) new_abs = 32767;
          P.dendrite_weights[col] = (int16_t)wmul(new_abs, sign);
          done++;
        }
      }
      if (zb) break;
    }
  }
  if (err) atomicOr(&ctl->err, err);
  block_count(done, 0, 0, &ctl->ctr[4]);
}

// physics.cu:25-30
__global__ void __launch_bounds__(256) k_reset_burst(uint8_t* __restrict__ flags, uint32_t N) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) flags[i] &= 0xF1;
}

// Segment-hit mask of the current heads without moving them (used by the
// stand-alone update stage of the legacy launchers).
__global__ void __launch_bounds__(256) k_mask_only(const BurstHeads8* __restrict__ heads, uint32_t A,
                                                   uint32_t* __restrict__ seg_mask) {
  __shared__ uint32_t s_pmax;
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A) return;
  uint32_t h[8];
  load_heads(heads, a, h);
  seg_mask[a] = seg_mask_of(h, s_pmax);
}

// Pending network pushes applied without propagation (physics.cu:114-132).
__global__ void __launch_bounds__(256) k_apply_incoming(BurstHeads8* __restrict__ heads, uint32_t A,
                                                        uint32_t* __restrict__ incoming) {
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A) return;
  const uint32_t c = incoming[a];
  if (!c) return;
  incoming[a] = 0;
  uint4* p = reinterpret_cast<uint4*>(heads + a);
  uint4 x = p[0], y = p[1];
  uint32_t h[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
  push_n(h, c);
  p[0] = make_uint4(h[0], h[1], h[2], h[3]);
  p[1] = make_uint4(h[4], h[5], h[6], h[7]);
}

// physics.cu:137-154 alone.
__global__ void __launch_bounds__(256) k_propagate_only(BurstHeads8* __restrict__ heads, uint32_t A,
                                                        uint32_t v_seg) {
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A) return;
  uint4* p = reinterpret_cast<uint4*>(heads + a);
  uint4 x = p[0], y = p[1];
  uint32_t h[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
#pragma unroll
  for (int j = 0; j < 8; j++)
    if (h[j] != AXC_AXON_SENTINEL) h[j] += v_seg;
  p[0] = make_uint4(h[0], h[1], h[2], h[3]);
  p[1] = make_uint4(h[4], h[5], h[6], h[7]);
}

// Ascending spike list: per-block counts, one-block scan, per-block writes.
constexpr uint32_t kListBlock = 1024;

__global__ void __launch_bounds__(kListBlock) k_list_count(const uint8_t* __restrict__ flags, uint32_t N,
                                                           uint32_t* __restrict__ block_counts) {
  const uint32_t i = blockIdx.x * kListBlock + threadIdx.x;
  const int s = i < N ? (flags[i] & 1) : 0;
  const int c = __syncthreads_count(s);
  if (threadIdx.x == 0) block_counts[blockIdx.x] = (uint32_t)c;
}

__global__ void __launch_bounds__(1024) k_list_scan(uint32_t* __restrict__ block_counts, uint32_t nblocks,
                                                    uint32_t* __restrict__ out_count) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (nblocks + 1023) / 1024;
  const uint32_t b0 = threadIdx.x * per;
  uint32_t s = 0;
  for (uint32_t b = b0; b < min(b0 + per, nblocks); b++) s += block_counts[b];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = *out_count;
    for (int i = 0; i < 1024; i++) { uint32_t v = part[i]; part[i] = acc; acc += v; }
    *out_count = acc;
  }
  __syncthreads();
  uint32_t acc = part[threadIdx.x];
  for (uint32_t b = b0; b < min(b0 + per, nblocks); b++) {
    uint32_t v = block_counts[b];
    block_counts[b] = acc;
    acc += v;
  }
}

__global__ void __launch_bounds__(kListBlock) k_list_write(const uint8_t* __restrict__ flags, uint32_t N,
                                                           const uint32_t* __restrict__ block_offsets,
                                                           uint32_t* __restrict__ out_ids) {
  __shared__ uint32_t warp_base[kListBlock / 32];
  const uint32_t i = blockIdx.x * kListBlock + threadIdx.x;
  const int s = i < N ? (flags[i] & 1) : 0;
  const uint32_t ballot = __ballot_sync(kFull, s);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warp_base[w] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = block_offsets[blockIdx.x];
    for (int q = 0; q < (int)(kListBlock / 32); q++) { uint32_t v = warp_base[q]; warp_base[q] = acc; acc += v; }
  }
  __syncthreads();
  if (s) out_ids[warp_base[w] + __popc(ballot & ((1u << lane) - 1u))] = i;
}

}  // namespace
}  // namespace axc

#include "row_engine.cuh"

namespace axc {

int sm_count() {
  static int cached = 0;
  if (!cached) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached = v > 0 ? v : 1;
  }
  return cached;
}

static std::atomic<uint64_t> g_lut_gen{1};

uint64_t lut_generation() { return g_lut_gen.load(); }

cudaError_t lut_upload(const VariantParameters* lut, cudaStream_t stream, bool async) {
  g_lut_gen.fetch_add(1);   // row caches built from the previous LUT (frozen ranks, Pmax) are stale
  if (async)
    return cudaMemcpyToSymbolAsync(VARIANT_LUT, lut, sizeof(VariantParameters) * 16, 0,
                                   cudaMemcpyHostToDevice, stream);
  return cudaMemcpyToSymbol(VARIANT_LUT, lut, sizeof(VariantParameters) * 16);
}

cudaError_t launch_reset_burst(const ShardVramPtrs& v, uint32_t padded_n, cudaStream_t stream) {
  if (padded_n == 0) return cudaSuccess;
  k_reset_burst<<<(padded_n + 255) / 256, 256, 0, stream>>>(v.soma_flags, padded_n);
  return cudaGetLastError();
}

cudaError_t launch_tick(const ShardVramPtrs& v, ShardScratch& s, const TickArgs& a, cudaStream_t stream,
                        cudaEvent_t* ev) {
  const uint32_t N = a.padded_n, A = a.total_axons;
  const int sms = sm_count();
  const uint32_t* batch_counts = a.batch ? s.batch_counts : nullptr;
  const bool have_incoming = a.incoming_spikes != nullptr && (a.batch || a.num_incoming > 0);
  if (ev) cudaEventRecord(ev[0], stream);
  if (have_incoming)
    k_incoming<<<sms, 256, 0, stream>>>(a.incoming_spikes, a.num_incoming, batch_counts, a.k,
                                        a.max_incoming, A, s.incoming);
  if (ev) cudaEventRecord(ev[1], stream);
  if (a.rows) return launch_tick_rows(v, s, a, stream, ev, have_incoming);
  const uint32_t* bitmask = (a.num_virtual > 0) ? a.input_bitmask : nullptr;
  uint32_t raise = 0;
  if (bitmask && ((uint64_t)a.virtual_offset + a.num_virtual > A)) raise |= AXC_ERR_VIRTUAL_RANGE;
  if (A > 0)
    k_axons<<<(A + 255) / 256, 256, 0, stream>>>(v.axon_heads, A, a.v_seg, bitmask, a.virtual_offset,
                                                 a.num_virtual, s.incoming,
                                                 (!a.batch && have_incoming) ? 1 : 0,
                                                 have_incoming ? batch_counts : nullptr, a.k, s.seg_mask,
                                                 s.ctl, raise);
  if (ev) cudaEventRecord(ev[2], stream);
  if (N > 0)
    k_update<4><<<(N + 255) / 256, 256, 0, stream>>>(v, N, A, a.tick, s.seg_mask, s.pend, s.spikers, s.ctl,
                                                     a.batch ? 1 : 0, a.k);
  if (ev) cudaEventRecord(ev[3], stream);
  const bool readout = a.num_outputs > 0 && a.mapped_soma_ids && a.output_history;
  k_push<<<2 * sms, 256, 0, stream>>>(v.axon_heads, v.soma_to_axon, A, s.pend, s.spikers, s.ctl, v.soma_flags,
                                      N, a.mapped_soma_ids, a.output_history, readout ? a.num_outputs : 0);
  if (ev) cudaEventRecord(ev[4], stream);
  k_gsop<<<8 * sms, 256, 0, stream>>>(v, N, A, a.dopamine, s.spikers, s.ctl, a.batch ? 1 : 0);
  if (ev) cudaEventRecord(ev[5], stream);
  return cudaGetLastError();
}

cudaError_t launch_push_incoming(BurstHeads8* heads, ShardScratch& s, uint32_t A, const uint32_t* ids,
                                 uint32_t count, cudaStream_t stream) {
  if (count == 0 || !ids || A == 0) return cudaSuccess;
  k_incoming<<<sm_count(), 256, 0, stream>>>(ids, count, nullptr, 0, count, A, s.incoming);
  k_apply_incoming<<<(A + 255) / 256, 256, 0, stream>>>(heads, A, s.incoming);
  return cudaGetLastError();
}

cudaError_t launch_propagate_only(BurstHeads8* heads, uint32_t A, uint32_t v_seg, cudaStream_t stream) {
  if (A == 0) return cudaSuccess;
  k_propagate_only<<<(A + 255) / 256, 256, 0, stream>>>(heads, A, v_seg);
  return cudaGetLastError();
}

cudaError_t launch_update_stage(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, uint32_t A, uint32_t tick,
                                cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(&s.ctl->spike_count, 0, 4, stream);
  if (e != cudaSuccess) return e;
  if (A) k_mask_only<<<(A + 255) / 256, 256, 0, stream>>>(v.axon_heads, A, s.seg_mask);
  if (N)
    k_update<4><<<(N + 255) / 256, 256, 0, stream>>>(v, N, A, tick, s.seg_mask, s.pend, s.spikers, s.ctl, 0, 0);
  k_push<<<2 * sm_count(), 256, 0, stream>>>(v.axon_heads, v.soma_to_axon, A, s.pend, s.spikers, s.ctl,
                                             v.soma_flags, N, nullptr, nullptr, 0);
  return cudaGetLastError();
}

cudaError_t launch_gsop_stage(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, uint32_t A, int16_t dopamine,
                              cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(&s.ctl->spike_count, 0, 4, stream);
  if (e != cudaSuccess) return e;
  e = launch_spike_list_sorted(v, N, s.spikers, &s.ctl->spike_count, stream);
  if (e != cudaSuccess) return e;
  k_gsop<<<8 * sm_count(), 256, 0, stream>>>(v, N, A, dopamine, s.spikers, s.ctl, 0);
  return cudaGetLastError();
}

cudaError_t launch_spike_list_sorted(const ShardVramPtrs& v, uint32_t padded_n, uint32_t* out_ids,
                                     uint32_t* out_count, cudaStream_t stream) {
  if (padded_n == 0) return cudaSuccess;
  const uint32_t nb = (padded_n + kListBlock - 1) / kListBlock;
  uint32_t* tmp = nullptr;
  cudaError_t e = cudaMallocAsync(&tmp, nb * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  k_list_count<<<nb, kListBlock, 0, stream>>>(v.soma_flags, padded_n, tmp);
  k_list_scan<<<1, 1024, 0, stream>>>(tmp, nb, out_count);
  k_list_write<<<nb, kListBlock, 0, stream>>>(v.soma_flags, padded_n, tmp, out_ids);
  cudaFreeAsync(tmp, stream);
  return cudaGetLastError();
}

}  // namespace axc

#include "population.cuh"
#include "learned.cuh"
