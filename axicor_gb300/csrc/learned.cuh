// learned.cuh — the learned-schedule engine (compiled as part of day_phase.cu,
// after row_engine.cuh, whose kernels it shares).
//
// A small MLP (64 -> 128 -> 1, BF16 weights, FP32 accumulation) predicts, per
// tile of 1024 axons, how many synapses will be active on the next tick (the
// fan-out of the tile's axons whose heads cover at least one segment).  Before
// each tick the plan kernel turns the predictions into a schedule:
//
//   dense   the row engine's update pass (every evaluated neuron reads its
//           whole dendrite row);
//   sparse  an axon-driven gather: the prologue compacts the active axons into
//           per-tile segments sized from the prediction, k_learn_scatter walks
//           an inverted index (axon -> dendrite slots) and adds the weights of
//           hit slots into the evaluated neurons' input current, k_learn_update
//           runs GLIF from that current and lists the spikers for the row
//           engine's GSOP passes (the same passes as the dense form).
//
// A tile whose actual activity exceeds its pre-sized segment sets the overflow
// flag in the prologue; the dense kernels then run the tick and the sparse
// ones return at once, so a misprediction costs time and never changes a
// result.  The dendrite input current is a wrapping int32 sum, so the order in
// which the scatter adds weights does not matter: both schedules give the
// plain path's state bit for bit.
//
// Training data come from the simulator: while collecting, the features
// kernel records (features of tick t-1, active-synapse fraction of tick t)
// per tile.  Training runs on the GPU with the kernels at the end of this
// file: forward + backward per block over a slice of the minibatch, a
// fixed-order reduction of the block partials and an Adam step that also
// refreshes the BF16 copy of the weights.

#include <cuda_bf16.h>

namespace axc {
namespace {

constexpr uint32_t kTileN = 1024;
constexpr uint32_t kFeat = 64, kHid = 128;
constexpr uint32_t kOffB1 = kHid * kFeat, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid;
constexpr uint32_t kParams = kOffB2 + 1;   // W1[128][64], b1[128], w2[128], b2
constexpr uint32_t kHistCh = 4;            // spikes, active synapses, heads in flight, evaluated
constexpr uint32_t kHistLen = 8;
constexpr uint32_t kHistF = kHistCh * kHistLen + 1;   // + the tile's next-tick evaluated count
constexpr uint32_t kGradPer = 16;          // samples per block of the gradient kernel
constexpr uint32_t kResidF = 8;            // the tile's active-synapse fraction of the tick just run

// LearnCtl.stat[]
enum : int {
  kStTicks = 0,        // ticks run by the learned engine
  kStSparse = 1,       // ticks that ran sparse
  kStOverflow = 2,     // sparse ticks re-run dense (a tile outgrew its segment)
  kStMismatch = 3,     // ticks whose schedule differs from the one exact counts pick
  kStAbsErr = 4,       // sum over tiles of |predicted - actual| active synapses
  kStActual = 5,       // sum over tiles of actual active synapses
  kStJudged = 6,       // ticks counted in kStMismatch / kStAbsErr
  kStSparsePicked = 7, // ticks planned sparse
  kStStale = 8,        // ticks forced dense because the targets changed
};

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// D = A x B + D on the tensor cores: A 16x16 BF16 (row-major), B 16x8 BF16
// (column-major), D 16x8 FP32 (PTX mma.sync.aligned.m16n8k16.row.col, BF16
// inputs, FP32 accumulation).  Fragments of lane l, g = l / 4, q = l % 4:
// a[0] row g cols 2q, 2q+1; a[1] row g + 8; a[2] row g cols 2q + 8, 2q + 9;
// a[3] row g + 8 cols 2q + 8, 2q + 9; b[0] rows (k) 2q, 2q+1 of column g;
// b[1] rows 2q + 8, 2q + 9; d[0], d[1] row g cols 2q, 2q+1; d[2], d[3] row g + 8.
// The lower-indexed element of a pair sits in the low half of its register.
__device__ __forceinline__ void mma_bf16_16816(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t ld_bf16x2(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// The MLP on 16 input rows by one warp (all 32 lanes): the hidden layer as 64
// tensor-core MMAs (16 tiles of 8 units x 4 steps of 16 features, BF16 inputs
// and weights, FP32 accumulators starting at b1), ReLU, BF16 rounding of the
// activations, then the output layer in FP32 in a fixed order: the units are
// taken in 4 groups of 32 (32p .. 32p + 31); in each, a lane sums w2[u] * h
// over its units (tile by tile, unit 2q before 2q + 1) and the four lanes of a
// quad are added pairwise (xor 1, then xor 2); the groups are combined as
// (G0 + G1) + (G2 + G3).  That is the order of the training kernel, whose
// warp p holds group p, so training and inference give the same outputs.
// *yg / *yg8: rows g and g + 8, on every lane of the quad, without b2 and the
// residual (mlp_out).
__device__ __forceinline__ float mlp_group_sum(const __nv_bfloat16* __restrict__ wb, const uint32_t (&a_frag)[4][4],
                                               uint32_t grp, float* s8, float (*keep)[4] = nullptr) {
  const uint32_t lane = threadIdx.x & 31u, g = lane >> 2, q = lane & 3u;
  float sg = 0.f, sg8 = 0.f;
#pragma unroll
  for (int nt = 0; nt < 4; nt++) {
    const uint32_t u0 = 32u * grp + 8u * nt + 2u * q;
    const float b1a = __bfloat162float(wb[kOffB1 + u0]), b1b = __bfloat162float(wb[kOffB1 + u0 + 1]);
    float d[4] = {b1a, b1b, b1a, b1b};
    const __nv_bfloat16* wrow = wb + (size_t)(32u * grp + 8u * nt + g) * kFeat + 2u * q;
#pragma unroll
    for (int ks = 0; ks < 4; ks++) mma_bf16_16816(d, a_frag[ks], ld_bf16x2(wrow + 16 * ks), ld_bf16x2(wrow + 16 * ks + 8));
    if (keep) {
#pragma unroll
      for (int e = 0; e < 4; e++) keep[nt][e] = d[e];
    }
    const float w2a = __bfloat162float(wb[kOffW2 + u0]), w2b = __bfloat162float(wb[kOffW2 + u0 + 1]);
    sg = __fadd_rn(sg, __fmul_rn(w2a, bf16r(fmaxf(d[0], 0.f))));
    sg = __fadd_rn(sg, __fmul_rn(w2b, bf16r(fmaxf(d[1], 0.f))));
    sg8 = __fadd_rn(sg8, __fmul_rn(w2a, bf16r(fmaxf(d[2], 0.f))));
    sg8 = __fadd_rn(sg8, __fmul_rn(w2b, bf16r(fmaxf(d[3], 0.f))));
  }
  sg = __fadd_rn(sg, __shfl_xor_sync(kFull, sg, 1));
  sg = __fadd_rn(sg, __shfl_xor_sync(kFull, sg, 2));
  sg8 = __fadd_rn(sg8, __shfl_xor_sync(kFull, sg8, 1));
  sg8 = __fadd_rn(sg8, __shfl_xor_sync(kFull, sg8, 2));
  *s8 = sg8;
  return sg;
}

__device__ __forceinline__ void mlp_warp16(const __nv_bfloat16* __restrict__ wb, const uint32_t (&a_frag)[4][4],
                                           float* yg, float* yg8) {
  float p8[4], p[4];
#pragma unroll
  for (int grp = 0; grp < 4; grp++) p[grp] = mlp_group_sum(wb, a_frag, (uint32_t)grp, &p8[grp]);
  *yg = __fadd_rn(__fadd_rn(p[0], p[1]), __fadd_rn(p[2], p[3]));
  *yg8 = __fadd_rn(__fadd_rn(p8[0], p8[1]), __fadd_rn(p8[2], p8[3]));
}

// A fragments of 16 rows of FP32 features (row r at x + r * kFeat; rows >=
// nrows are zero), rounded to BF16.
__device__ __forceinline__ void mlp_a_frags(const float* __restrict__ x, uint32_t nrows, uint32_t (&a)[4][4]) {
  const uint32_t lane = threadIdx.x & 31u, g = lane >> 2, q = lane & 3u;
  const bool vg = g < nrows, vg8 = g + 8u < nrows;
  const float* xg = x + (size_t)g * kFeat + 2u * q;
  const float* xg8 = x + (size_t)(g + 8u) * kFeat + 2u * q;
#pragma unroll
  for (int ks = 0; ks < 4; ks++) {
    const int c = 16 * ks;
    a[ks][0] = vg ? pack_bf16x2(xg[c], xg[c + 1]) : 0u;
    a[ks][1] = vg8 ? pack_bf16x2(xg8[c], xg8[c + 1]) : 0u;
    a[ks][2] = vg ? pack_bf16x2(xg[c + 8], xg[c + 9]) : 0u;
    a[ks][3] = vg8 ? pack_bf16x2(xg8[c + 8], xg8[c + 9]) : 0u;
  }
}

// The MLP's output for row r of x given the quad sum s of mlp_warp16:
// (s + b2) + x[r][kResidF] (the residual input, BF16-rounded like the rest).
__device__ __forceinline__ float mlp_out(const __nv_bfloat16* __restrict__ wb, float s, const float* xr) {
  return __fadd_rn(__fadd_rn(s, __bfloat162float(wb[kOffB2])), bf16r(xr[kResidF]));
}

// Block-wide exclusive scan of cnt[0..n) (1024 threads, n <= 1024 * 64) into
// out[0..n], out[n] = total.
__device__ void block_scan_1024(const uint32_t* cnt, uint32_t* out, uint32_t n) {
  __shared__ uint32_t s[1024];
  const uint32_t per = (n + 1023) / 1024;
  const uint32_t b = threadIdx.x * per;
  uint32_t t = 0;
  for (uint32_t q = 0; q < per; q++)
    if (b + q < n) t += cnt[b + q];
  s[threadIdx.x] = t;
  __syncthreads();
  for (uint32_t o = 1; o < 1024; o <<= 1) {
    const uint32_t x = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += x;
    __syncthreads();
  }
  uint32_t run = s[threadIdx.x] - t;
  for (uint32_t q = 0; q < per; q++)
    if (b + q < n) {
      const uint32_t c = cnt[b + q];
      out[b + q] = run;
      run += c;
    }
  if (threadIdx.x == 1023) out[n] = s[1023];
  __syncthreads();
}

// Capacity (synapses) of tile j's compaction segment on a sparse tick.
__device__ __forceinline__ uint32_t tile_cap(const LearnCtl& c, float pred, uint32_t fan) {
  if (c.policy == 1) return fan;
  const float want = fmaxf(pred, 0.f) * (float)fan * (1.f + c.margin) + (float)c.slack;
  return want >= (float)fan ? fan : (uint32_t)want;
}

// The schedule of the next tick, by one thread, from totals over the tiles:
// ty / terr the finished tick's active synapses and prediction error (when
// the features kernel ran), tp the predicted active synapses and tnext the
// evaluated slots of the next tick, rate its input spike fraction.
__device__ void plan_serial(LearnCtl& c, unsigned long long row_sum, unsigned long long ty, unsigned long long terr,
                            unsigned long long tp, unsigned long long tnext, float rate, bool features_ran) {
  if (c.prev_learned && features_ran) {   // the finished tick, judged with exact counts
    const bool best_sparse = c.ratio * (float)ty < (float)c.eval_now;
    if (best_sparse != (c.prev_mode == 1u)) c.stat[kStMismatch]++;
    c.stat[kStJudged]++;
    c.stat[kStAbsErr] += terr;
    c.stat[kStActual] += ty;
  }
  if (features_ran) {
    if (c.collect && c.ticks_seen >= 1 && (c.ticks_seen % c.sample_every) == 0 && c.samples + c.T <= c.sample_cap)
      c.samples += c.T;
    c.ticks_seen++;
  } else {
    c.ticks_seen = 0;   // the feature history restarts
  }
  for (int q = 8; q > 0; q--) c.inrate[q] = c.inrate[q - 1];
  c.inrate[0] = rate;
  c.stale = (row_sum != c.row_sum) ? 1u : 0u;
  const bool learned = features_ran && c.policy < 0 && c.ticks_seen > 0 && !c.stale;
  bool sparse;
  if (c.stale) sparse = false;
  else if (c.policy == 1) sparse = true;
  else sparse = learned && c.ratio * (float)tp < (float)tnext;
  c.pred_total = (float)tp;
  c.eval_now = tnext;
  c.mode = sparse ? 1u : 0u;
  c.prev_mode = c.mode;
  c.prev_learned = learned ? 1u : 0u;
  c.overflow = 0;
  c.spk_count = 0;
}

// The control block is staged in shared memory around plan_serial, which
// would otherwise be a chain of dependent global-memory accesses.
__device__ __forceinline__ void ctl_load(LearnCtl* dst, const LearnCtl* src) {
  for (uint32_t q = threadIdx.x; q < sizeof(LearnCtl) / 4; q += blockDim.x)
    reinterpret_cast<uint32_t*>(dst)[q] = __ldcg(reinterpret_cast<const uint32_t*>(src) + q);
}
__device__ __forceinline__ void ctl_store(LearnCtl* dst, const LearnCtl* src) {
  for (uint32_t q = threadIdx.x; q < sizeof(LearnCtl) / 4; q += blockDim.x)
    reinterpret_cast<uint32_t*>(dst)[q] = reinterpret_cast<const uint32_t*>(src)[q];
}

// ---------------------------------------------------------------------------
// per tick 0: the schedule, by one block of 1024 threads, from the totals of
// the features kernel's per-tile partials (when it ran after the previous
// tick) on a shared-memory copy of the control block.
// ---------------------------------------------------------------------------
// Accounting of the tick about to run.
__device__ __forceinline__ void plan_commit(LearnCtl& c) {
  c.stat[kStTicks]++;
  if (c.stale) c.stat[kStStale]++;
  if (c.mode == 1u) c.stat[kStSparsePicked]++;
}

__global__ void __launch_bounds__(1024) k_learn_plan(LearnDev L, const float* __restrict__ pred,
                                                     const uint32_t* __restrict__ fan, uint32_t* __restrict__ cap,
                                                     const uint32_t* __restrict__ part,
                                                     const uint32_t* __restrict__ bits, uint32_t words, uint32_t nv,
                                                     const ShardCtl* __restrict__ sc) {
  LearnCtl& c = *L.ctl;
  __shared__ unsigned long long s_part[4][32];
  __shared__ uint32_t s_in[32];
  __shared__ LearnCtl s_c;
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  ctl_load(&s_c, &c);
  __syncthreads();
  const uint32_t T = s_c.T;
  const bool feat = s_c.feat_done != 0u;   // the features kernel ran after the previous tick
  // totals of the previous tick's features blocks, and this tick's input spikes
  unsigned long long a[4] = {0, 0, 0, 0};
  if (feat)
    for (uint32_t j = threadIdx.x; j < T; j += 1024)
#pragma unroll
      for (int k = 0; k < 4; k++) a[k] += part[(size_t)k * T + j];
  uint32_t ib = 0;
  for (uint32_t q = threadIdx.x; q < words; q += 1024) {
    uint32_t x = bits ? bits[q] : 0u;
    if (32u * q + 32u > nv) x &= (32u * q >= nv) ? 0u : ((1u << (nv - 32u * q)) - 1u);
    ib += __popc(x);
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const unsigned long long v = warp_sum(a[k]);
    if (lane == 0) s_part[k][w] = v;
  }
  ib = warp_sum(ib);
  if (lane == 0) s_in[w] = ib;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t[4] = {0, 0, 0, 0};
    uint32_t ti = 0;
    for (int q = 0; q < 32; q++) {
      for (int k = 0; k < 4; k++) t[k] += s_part[k][q];
      ti += s_in[q];
    }
    plan_serial(s_c, sc->row_sum, t[0], t[1], t[2], t[3], nv ? (float)ti / (float)nv : 0.f, feat);
    s_c.feat_done = 0;
    plan_commit(s_c);
  }
  __syncthreads();
  ctl_store(&c, &s_c);
  // tile capacities: the features kernel wrote them for the planned tick,
  // except without features (no prediction) or with exact buffers
  if (!feat || s_c.policy == 1)
    for (uint32_t j = threadIdx.x; j < T; j += 1024) cap[j] = tile_cap(s_c, pred[j], fan[j]);
  if (!feat)
    for (uint32_t j = threadIdx.x; j < T; j += 1024) {
      L.yacc[j] = 0;
      L.bacc[j] = 0;
      L.fill[j] = 0;
    }
}

// ---------------------------------------------------------------------------
// per tick 2s: the sparse gather.  The tiles' active axons, as one flat range,
// a warp per axon walking the axon's slots in the inverted index; hit slots of evaluated neurons add their weight to the
// neuron's input current (wrapping int32, order-independent).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_learn_scatter(LearnDev L, uint32_t T, const uint32_t* __restrict__ inv,
                                                       const uint8_t* __restrict__ inv_seg,
                                                       const uint2* __restrict__ mask2,
                                                       const int16_t* __restrict__ rw,
                                                       const uint8_t* __restrict__ posmap,
                                                       const uint8_t* __restrict__ flags,
                                                       const BurstHeads8* __restrict__ heads, uint32_t A,
                                                       int32_t* __restrict__ acc, ShardCtl* __restrict__ sc) {
  LearnCtl& c = *L.ctl;
  if (blockIdx.x == 0 && threadIdx.x == 0 && c.mode == 1u) c.stat[c.overflow ? kStOverflow : kStSparse]++;
  if (c.mode != 1u || c.overflow) return;
  __shared__ uint32_t s_prop[16];
  __shared__ uint32_t s_pmax;
  extern __shared__ uint32_t s_pre[];   // [T+1] prefix of the tiles' active-axon counts
  if (threadIdx.x < 16) s_prop[threadIdx.x] = VARIANT_LUT[threadIdx.x].signal_propagation_length;
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  // every block scans the fills itself: the tiles' active axons form one flat
  // range [0, total) that all warps of the grid share
  {
    const uint32_t per = (T + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t t = 0;
    for (uint32_t q = 0; q < per; q++)
      if (b0 + q < T) t += L.fill[b0 + q];
    __shared__ uint32_t s_part[256];
    s_part[threadIdx.x] = t;
    __syncthreads();
    for (uint32_t o = 1; o < blockDim.x; o <<= 1) {
      const uint32_t x = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0u;
      __syncthreads();
      s_part[threadIdx.x] += x;
      __syncthreads();
    }
    uint32_t run = s_part[threadIdx.x] - t;
    for (uint32_t q = 0; q < per; q++)
      if (b0 + q < T) {
        s_pre[b0 + q] = run;
        run += L.fill[b0 + q];
      }
    if (threadIdx.x == blockDim.x - 1) s_pre[T] = s_part[blockDim.x - 1];
    __syncthreads();
  }
  const uint32_t total = s_pre[T];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long hits = 0;
  for (uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < total; e += nwarps) {
    uint32_t lo = 0, hi = T;   // the tile holding flat position e
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (s_pre[mid] <= e) lo = mid; else hi = mid;
    }
    const uint32_t a = L.alist[(size_t)lo * kTileN + (e - s_pre[lo])];
    const uint2 m = __ldg(mask2 + a);
    const uint32_t r0 = __ldg(L.inv_off + a), r1 = __ldg(L.inv_off + a + 1);
    for (uint32_t r = r0 + lane; r < r1; r += 32) {
      const uint32_t s = inv_seg[r];
      const uint32_t slot = __ldg(inv + r);
      const uint32_t sh = min(s, 31u);
      if (!(((m.x | m.y) >> sh) & 1u)) continue;
      const uint32_t n = slot / kRowStride;
      const uint32_t evw = __ldg(L.evbits + (n >> 5));
      const uint32_t fl = flags[n];
      // the index holds columnar slots; the row copy keeps the slots whose weights
      // may still move first, so the weight sits at the row position the map gives
      const int32_t wv = rw[(size_t)n * kRowStride + __ldg(posmap + slot)];
      if (!((evw >> (n & 31u)) & 1u)) continue;
      const uint32_t prop = s_prop[fl >> 4];
      bool hit = true;
      if (s >= 31u || prop != s_pmax) hit = hit_exact(heads, A, a, s, prop);
      if (hit) {
        atomicAdd(acc + n, wv);
        hits++;
      }
    }
  }
  block_count(0, hits, 0, &sc->ctr[1]);
}

// per tick 3s: GLIF of every evaluated neuron from the scattered current;
// spikers push their axon and are listed for the row engine's GSOP passes
// exactly as k_rows_update lists them (the same per-warp slices of the
// evaluated list, 32 warps per SM).
__global__ void __launch_bounds__(256) k_learn_update(ShardVramPtrs P, LearnDev L, uint32_t A,
                                                      const uint16_t* __restrict__ cnt,
                                                      const uint32_t* __restrict__ eval, uint32_t* __restrict__ pend,
                                                      int32_t* __restrict__ acc, const uint8_t* __restrict__ lfz,
                                                      uint32_t* __restrict__ gs_n, uint32_t* __restrict__ gd_n,
                                                      uint32_t* __restrict__ wcnt, ShardCtl* __restrict__ ctl,
                                                      uint32_t k) {
  LearnCtl& c = *L.ctl;
  if (c.mode != 1u || c.overflow) return;
  __shared__ VariantParameters lut[16];
  lut_to_smem(lut);
  __syncthreads();
  const uint32_t tick = ctl->tick_base + k;
  const uint32_t ecount = ctl->eval_count[k & 1];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t per_warp = (((ecount + nwarps - 1) / nwarps) + 3) & ~3u;
  const uint32_t beg = min(wid * per_warp, ecount), end = min(beg + per_warp, ecount);
  unsigned long long ev_slots = 0, nspk = 0, nev = 0, gdone = 0;
  uint32_t err = 0, wc = 0, wd = 0;
  for (uint32_t b0 = beg; b0 < end; b0 += 32) {
    const uint32_t i = b0 + lane;
    const bool valid = i < end;
    bool spike = false;
    uint32_t n = 0, lf = 0;
    if (valid) {
      n = eval[i];
      const uint8_t flags = P.soma_flags[n];
      const uint32_t cw = cnt[n];
      lf = lfz[n];
      const int32_t i_in = acc[n];
      acc[n] = 0;
      const VariantParameters& p = lut[flags >> 4];
      const GlifOut o = glif_step(p, P.soma_voltage[n], P.threshold_offset[n], i_in, tick, n);
      spike = o.spike != 0;
      P.soma_voltage[n] = o.v;
      P.soma_flags[n] = (uint8_t)((flags & 0xF0) | (spike ? 0x05 : 0x00));
      P.threshold_offset[n] = o.thr;
      P.timers[n] = o.glif ? p.refractory_period : 0;
      ev_slots += cw & 0xFFu;
      nev++;
      if (cw & kRowBad) err |= AXC_ERR_TARGET_RANGE;
      if (spike) {
        nspk++;
        if (lf <= 8u) gdone += (cw & 0xFFu) - lf;   // frozen slots of rows k_rows_gsop takes, or all
        const uint32_t my_axon = P.soma_to_axon[n];
        if (my_axon != AXC_NO_AXON) {
          if (my_axon < A) atomicAdd(&pend[my_axon], 1u);
          else err |= AXC_ERR_SOMA_AXON;
        }
      }
    }
    const bool few = spike && lf > 0u && lf <= 8u, many = spike && lf > 8u;
    const uint32_t ab = __ballot_sync(kFull, few), db = __ballot_sync(kFull, many);
    const uint32_t below = (1u << lane) - 1u;
    if (few) gs_n[beg + wc + __popc(ab & below)] = n;
    if (many) gd_n[beg + wd + __popc(db & below)] = n;
    wc += __popc(ab);
    wd += __popc(db);
  }
  if (lane == 0) {
    wcnt[wid] = wc;
    wcnt[kMaxUpdateWarps + wid] = wd;
  }
  const uint32_t err_any = __reduce_or_sync(kFull, err);
  if (err_any && lane == 0) atomicOr(&ctl->err, err_any);
  block_count(ev_slots, 0, nspk, &ctl->ctr[1]);
  block_count(gdone, nev, 0, &ctl->ctr[4]);
}

// ---------------------------------------------------------------------------
// per tick 5: features of each tile after the tick, a recorded training pair
// when collecting, and the prediction for the next tick.  A 128-thread block
// per tile.
//
// Features (64): spikes, active-synapse fraction, heads in flight and
// evaluated neurons of ticks t..t-7 (4 x 8); the input spike fraction of ticks
// t..t-7 and t+1; the next tick's evaluated neurons and slots (exact: refractory
// timers after the tick); the refractory histogram (timer 1, 2, 3, >= 4); the
// tile's fan-out; a constant 1; zeros.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_learn_features(LearnDev L, ShardVramPtrs P, uint32_t N,
                                                        const uint16_t* __restrict__ cnt,
                                                        const uint32_t* __restrict__ fan,
                                                        const uint32_t* __restrict__ axn, float* __restrict__ hist,
                                                        float* __restrict__ feat, float* __restrict__ pred,
                                                        uint32_t* __restrict__ cap, uint32_t* __restrict__ part,
                                                        const __nv_bfloat16* __restrict__ wb, float* __restrict__ X,
                                                        float* __restrict__ Y, const uint32_t* __restrict__ bits_next,
                                                        uint32_t words, uint32_t nv, const ShardCtl* __restrict__ sc) {
  LearnCtl& c = *L.ctl;
  const uint32_t T = c.T;
  const uint32_t j = blockIdx.x;
  const uint32_t u = threadIdx.x, lane = u & 31, w = u >> 5;
  __shared__ uint32_t s_cnt[8][4];
  __shared__ float s_old[kHistF];
  const bool seen = c.ticks_seen > 0;   // x of the previous tick is in feat[]
  // 1. the tile's neurons after the tick: 8 consecutive neurons per thread,
  //    one vector load each of timers, flags and row counts when aligned
  uint32_t spk = 0, nxt = 0, nslots = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, ib = 0;
  const uint32_t n8 = j * kTileN + 8u * u;
  const bool vec = ((reinterpret_cast<uintptr_t>(P.timers) | reinterpret_cast<uintptr_t>(P.soma_flags)) & 7u) == 0 &&
                   n8 + 8u <= N;
  uint32_t tmw[2] = {0xFFFFFFFFu, 0xFFFFFFFFu}, flw[2] = {0, 0}, cw[4] = {0, 0, 0, 0};
  if (vec) {
    const uint2 tm8 = *reinterpret_cast<const uint2*>(P.timers + n8);
    const uint2 fl8 = *reinterpret_cast<const uint2*>(P.soma_flags + n8);
    const uint4 c8 = *reinterpret_cast<const uint4*>(cnt + n8);
    tmw[0] = tm8.x; tmw[1] = tm8.y; flw[0] = fl8.x; flw[1] = fl8.y;
    cw[0] = c8.x; cw[1] = c8.y; cw[2] = c8.z; cw[3] = c8.w;
  } else {
    for (int q = 0; q < 8; q++) {
      const uint32_t n = n8 + q;
      if (n >= N) break;
      const uint32_t sh = 8 * (q & 3);
      tmw[q >> 2] = (tmw[q >> 2] & ~(0xFFu << sh)) | ((uint32_t)P.timers[n] << sh);
      flw[q >> 2] |= (uint32_t)P.soma_flags[n] << sh;
      cw[q >> 1] |= (uint32_t)cnt[n] << (16 * (q & 1));
    }
  }
#pragma unroll
  for (int q = 0; q < 8; q++) {   // neurons past N are skipped
    const uint32_t tm = (tmw[q >> 2] >> (8 * (q & 3))) & 0xFFu;
    if (n8 + q >= N) continue;
    spk += (flw[q >> 2] >> (8 * (q & 3))) & 1u;
    if (tm == 0) { nxt++; nslots += (cw[q >> 1] >> (16 * (q & 1))) & 0xFFu; }
    t1 += tm == 1;
    t2 += tm == 2;
    t3 += tm == 3;
    t4 += tm >= 4;
  }
  for (uint32_t q = u; q < words; q += 128) {
    uint32_t x = bits_next ? bits_next[q] : 0u;
    if (32u * q + 32u > nv) x &= (32u * q >= nv) ? 0u : ((1u << (nv - 32u * q)) - 1u);
    ib += __popc(x);
  }
  const uint32_t vals[8] = {spk, nxt, nslots, t1, t2, t3, t4, ib};
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const uint32_t v = warp_sum(vals[q]);
    if (lane == 0) s_cnt[q][w] = v;
  }
  if (u < kHistF) s_old[u] = seen ? hist[(size_t)j * kHistF + u] : 0.f;
  const uint32_t ya = L.yacc[j], ba = L.bacc[j];
  const float pred_old = pred[j];
  __syncthreads();
  uint32_t tot[8];
#pragma unroll
  for (int q = 0; q < 8; q++) tot[q] = s_cnt[q][0] + s_cnt[q][1] + s_cnt[q][2] + s_cnt[q][3];
  const float fj = (float)max(fan[j], 1u);
  const float aj = (float)max(axn[j], 1u);
  const float y_now = (float)ya / fj;
  // 2. training pair (features of the previous tick, this tick's target)
  if (seen && c.collect && (c.ticks_seen % c.sample_every) == 0 && c.samples + T <= c.sample_cap) {
    const size_t row = (size_t)c.samples + j;
    if (u < kFeat) X[row * kFeat + u] = feat[(size_t)j * kFeat + u];
    if (u == 0) Y[row] = y_now;
  }
  // 3. history shift and the feature vector
  const float cur[kHistCh] = {(float)tot[0] / (float)kTileN, y_now, (float)ba / (8.f * aj),
                              s_old[kHistCh * kHistLen] / (float)kTileN};
  float x = 0.f;
  if (u < kHistCh * kHistLen) {
    const uint32_t ch = u / kHistLen, i = u % kHistLen;
    x = i == 0 ? cur[ch] : s_old[ch * kHistLen + i - 1];
  } else if (u < 40) {
    x = c.inrate[u - 32];
  } else if (u == 40) {
    x = nv ? (float)tot[7] / (float)nv : 0.f;
  } else if (u == 41) {
    x = (float)tot[1] / (float)kTileN;
  } else if (u == 42) {
    x = (float)tot[2] / (float)(kTileN * AXC_MAX_DENDRITES);
  } else if (u >= 43 && u <= 46) {
    x = (float)tot[3 + (u - 43)] / (float)kTileN;
  } else if (u == 47) {
    x = (float)fan[j] / (float)(kTileN * AXC_MAX_DENDRITES);
  } else if (u == 48) {
    x = 1.f;
  }
  __syncthreads();   // every read of feat[] / hist[] is done
  if (u < kHistCh * kHistLen) hist[(size_t)j * kHistF + u] = x;
  if (u == 0) hist[(size_t)j * kHistF + kHistCh * kHistLen] = (float)tot[1];
  if (u < kFeat) feat[(size_t)j * kFeat + u] = x;
  // 4. the tile's partial totals (k_learn_predict adds the prediction for the
  //    next tick); this tick's accumulators are cleared for the next
  if (u == 0) {
    const float err = (seen && c.policy < 0) ? fabsf(fmaxf(pred_old, 0.f) - y_now) * fj : 0.f;
    part[j] = ya;
    part[T + j] = (uint32_t)(err + 0.5f);
    part[3 * T + j] = tot[2];
    L.yacc[j] = 0;
    L.bacc[j] = 0;
    L.fill[j] = 0;
    if (j == 0) c.feat_done = 1u;
  }
}

// ---------------------------------------------------------------------------
// Inverted index (axon -> dendrite slots), built from the rows.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_inv_count(const uint32_t* __restrict__ rt, const uint16_t* __restrict__ cnt,
                                                   uint32_t N, uint32_t A, uint32_t* __restrict__ deg) {
  const size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (size_t)N * kRowStride) return;
  const uint32_t n = (uint32_t)(r / kRowStride), q = (uint32_t)(r % kRowStride);
  if (q >= (cnt[n] & 0xFFu)) return;
  const uint32_t a = (rt[r] & AXC_TARGET_AXON_MASK) - 1u;
  if (a < A) atomicAdd(deg + a, 1u);
}

__global__ void __launch_bounds__(256) k_inv_fill(const uint32_t* __restrict__ rt, const uint16_t* __restrict__ cnt,
                                                  uint32_t N, uint32_t A, uint32_t* __restrict__ cursor,
                                                  uint32_t* __restrict__ inv, uint8_t* __restrict__ inv_seg) {
  const size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (size_t)N * kRowStride) return;
  const uint32_t n = (uint32_t)(r / kRowStride), q = (uint32_t)(r % kRowStride);
  if (q >= (cnt[n] & 0xFFu)) return;
  const uint32_t t = rt[r];
  const uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
  if (a >= A) return;
  const uint32_t pos = atomicAdd(cursor + a, 1u);
  inv[pos] = (uint32_t)r;
  inv_seg[pos] = (uint8_t)(t >> AXC_TARGET_SEG_SHIFT);
}

// Exclusive scan of n <= 4096 * 4096 values: blocks of 4096, then the block sums.
__global__ void __launch_bounds__(1024) k_scan_blocks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                      uint32_t n, uint32_t* __restrict__ bsum) {
  __shared__ uint32_t s[1024];
  const uint32_t base = blockIdx.x * 4096u + threadIdx.x * 4u;
  uint32_t v[4], t = 0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    v[i] = base + i < n ? in[base + i] : 0u;
    t += v[i];
  }
  s[threadIdx.x] = t;
  __syncthreads();
  for (uint32_t o = 1; o < 1024; o <<= 1) {
    const uint32_t x = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += x;
    __syncthreads();
  }
  uint32_t run = s[threadIdx.x] - t;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == 1023) bsum[blockIdx.x] = s[1023];
}

__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* __restrict__ bsum, uint32_t nb,
                                                    uint32_t* __restrict__ out, uint32_t n) {
  __shared__ uint32_t tmp[4097];
  for (uint32_t i = threadIdx.x; i < nb; i += 1024) tmp[i] = bsum[i];
  __syncthreads();
  block_scan_1024(tmp, bsum, nb);   // bsum[0..nb] exclusive, bsum[nb] = total
  if (threadIdx.x == 0) out[n] = bsum[nb];
}

__global__ void __launch_bounds__(256) k_scan_add(uint32_t* __restrict__ out, uint32_t n,
                                                  const uint32_t* __restrict__ bsum) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += bsum[i / 4096u];
}

__global__ void __launch_bounds__(256) k_tile_fan(const uint32_t* __restrict__ off, uint32_t A, uint32_t T,
                                                  uint32_t* __restrict__ fan, uint32_t* __restrict__ axn) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= T) return;
  const uint32_t a0 = j * kTileN, a1 = min(a0 + kTileN, A);
  fan[j] = off[a1] - off[a0];
  axn[j] = a1 - a0;
}

__global__ void k_learn_index_done(LearnCtl* c, const ShardCtl* sc) {
  c->row_sum = sc->row_sum;
  c->ticks_seen = 0;
  c->feat_done = 0;
  c->prev_learned = 0;
  c->eval_next = 0;
  c->eval_now = 0;
  for (int q = 0; q < 9; q++) c->inrate[q] = 0.f;
}

// The output of the MLP for 16 rows of x by a block of 4 warps: warp p computes
// the sums of unit group p (mlp_group_sum) and the first 16 threads combine
// them in mlp_warp16's order, so the result equals mlp_warp16's; *y_out (row
// threadIdx.x, for threads < nrows) gets (s + b2) + x[kResidF].  All 128
// threads must call it.
__device__ __forceinline__ bool mlp_block16(const __nv_bfloat16* __restrict__ wb, const float* __restrict__ x,
                                            uint32_t nrows, float* y_out) {
  __shared__ float s_grp[4][16];
  const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31u, g = lane >> 2, q = lane & 3u;
  uint32_t a[4][4];
  mlp_a_frags(x, nrows, a);
  float s8;
  const float s0 = mlp_group_sum(wb, a, w, &s8);
  if (q == 0) {
    s_grp[w][g] = s0;
    s_grp[w][g + 8] = s8;
  }
  __syncthreads();
  const uint32_t r = threadIdx.x;
  bool ok = false;
  if (r < nrows) {
    const float s = __fadd_rn(__fadd_rn(s_grp[0][r], s_grp[1][r]), __fadd_rn(s_grp[2][r], s_grp[3][r]));
    *y_out = mlp_out(wb, s, x + (size_t)r * kFeat);
    ok = true;
  }
  __syncthreads();   // s_grp is free for the next call
  return ok;
}

// per tick 5b: the predictor on every tile's features, a block of 4 warps
// per 16 tiles on the tensor cores (mlp_block16): the next tick's predicted
// active-synapse fraction, the tile's compaction capacity and its predicted
// active synapses.
__global__ void __launch_bounds__(128) k_learn_predict(LearnDev L, const __nv_bfloat16* __restrict__ wb,
                                                       const float* __restrict__ feat, const uint32_t* __restrict__ fan,
                                                       float* __restrict__ pred, uint32_t* __restrict__ cap,
                                                       uint32_t* __restrict__ part) {
  const LearnCtl& c = *L.ctl;
  const uint32_t T = c.T;
  for (uint32_t r0 = 16u * blockIdx.x; r0 < T; r0 += 16u * gridDim.x) {
    float y;
    if (!mlp_block16(wb, feat + (size_t)r0 * kFeat, min(16u, T - r0), &y)) continue;
    const uint32_t j = r0 + threadIdx.x;
    const float fj = (float)max(fan[j], 1u);
    pred[j] = y;
    cap[j] = tile_cap(c, y, fan[j]);
    part[2 * T + j] = (uint32_t)fminf(fmaxf(y, 0.f) * fj, fj);
  }
}

// ---------------------------------------------------------------------------
// MLP training: one block of 4 warps per 16 samples, on the tensor cores.
// Forward: warp p computes the hidden units 32p .. 32p + 31 of the 16 samples
// (mlp_group_sum); the output is (((G0 + G1) + (G2 + G3)) + b2) + x[kResidF],
// as in inference.  Loss: mean squared error over the minibatch (count
// samples, 1/count).  Backward: dy = 2 (y - t) / count; gw2[u] and gb1[u] in
// FP32 (rows g, then g + 8, then over g by xor 4, 8, 16); dh[s][u] = dy[s] w2[u]
// where the pre-activation is positive, rounded to BF16 for the W1 gradient
// G1 = dh^T x, 16 units x 8 features per MMA over the 16 samples.  Each block
// writes its partial gradient; k_mlp_reduce sums them in block order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_mlp_grad(const __nv_bfloat16* __restrict__ wb, const float* __restrict__ X,
                                                  const float* __restrict__ Yt, const uint32_t* __restrict__ idx,
                                                  uint32_t count, float inv_count, float* __restrict__ partial) {
  __shared__ __align__(16) __nv_bfloat16 xs[16][kFeat + 8];    // the samples (forward A operand)
  __shared__ __align__(16) __nv_bfloat16 xt[kFeat][16 + 8];    // transposed (backward B operand)
  __shared__ __align__(16) __nv_bfloat16 dht[kHid][16 + 8];    // dh transposed (backward A operand)
  __shared__ float ysum[4][16];
  __shared__ float s_dy[16], s_loss[16], s_x8[16];
  const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31u, g = lane >> 2, q = lane & 3u;
  const uint32_t s0 = blockIdx.x * 16u;
  const uint32_t ns = min(16u, count - s0);
  for (uint32_t i = threadIdx.x; i < 16u * kFeat; i += 128u) {
    const uint32_t r = i / kFeat, f = i % kFeat;
    float v = 0.f;
    if (r < ns) v = X[(size_t)(idx ? idx[s0 + r] : s0 + r) * kFeat + f];
    const __nv_bfloat16 bv = __float2bfloat16_rn(v);
    xs[r][f] = bv;
    xt[f][r] = bv;
    if (f == kResidF) s_x8[r] = __bfloat162float(bv);
  }
  __syncthreads();
  uint32_t a[4][4];
#pragma unroll
  for (int ks = 0; ks < 4; ks++) {
    a[ks][0] = ld_bf16x2(&xs[g][16 * ks + 2 * q]);
    a[ks][1] = ld_bf16x2(&xs[g + 8][16 * ks + 2 * q]);
    a[ks][2] = ld_bf16x2(&xs[g][16 * ks + 8 + 2 * q]);
    a[ks][3] = ld_bf16x2(&xs[g + 8][16 * ks + 8 + 2 * q]);
  }
  float acc[4][4];   // pre-activations of units 32w + 8nt + 2q (+1), rows g and g + 8
  float sg8;
  const float sg = mlp_group_sum(wb, a, w, &sg8, acc);
  if (q == 0) {
    ysum[w][g] = sg;
    ysum[w][g + 8] = sg8;
  }
  __syncthreads();
  if (threadIdx.x < 16) {
    const uint32_t r = threadIdx.x;
    const float y = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(ysum[0][r], ysum[1][r]), __fadd_rn(ysum[2][r], ysum[3][r])),
                                        __bfloat162float(wb[kOffB2])),
                              s_x8[r]);
    float dy = 0.f, lr = 0.f;
    if (r < ns) {
      const float d = __fsub_rn(y, Yt[idx ? idx[s0 + r] : s0 + r]);
      dy = __fmul_rn(__fmul_rn(2.f, d), inv_count);
      lr = __fmul_rn(__fmul_rn(d, d), inv_count);
    }
    s_dy[r] = dy;
    s_loss[r] = lr;
  }
  __syncthreads();
  const float dyg = s_dy[g], dyg8 = s_dy[g + 8];
  float gw2[4][2], gb1[4][2];
#pragma unroll
  for (int nt = 0; nt < 4; nt++) {
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const uint32_t u = 32u * w + 8u * nt + 2u * q + j;
      const float w2u = __bfloat162float(wb[kOffW2 + u]);
      const float ag = acc[nt][j], ag8 = acc[nt][2 + j];
      gw2[nt][j] = __fadd_rn(__fmul_rn(dyg, bf16r(fmaxf(ag, 0.f))), __fmul_rn(dyg8, bf16r(fmaxf(ag8, 0.f))));
      const float dhg = ag > 0.f ? __fmul_rn(dyg, w2u) : 0.f, dhg8 = ag8 > 0.f ? __fmul_rn(dyg8, w2u) : 0.f;
      gb1[nt][j] = __fadd_rn(dhg, dhg8);
      dht[u][g] = __float2bfloat16_rn(dhg);
      dht[u][g + 8] = __float2bfloat16_rn(dhg8);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 4; nt++) {
#pragma unroll
    for (int j = 0; j < 2; j++) {
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) {
        gw2[nt][j] = __fadd_rn(gw2[nt][j], __shfl_xor_sync(kFull, gw2[nt][j], o));
        gb1[nt][j] = __fadd_rn(gb1[nt][j], __shfl_xor_sync(kFull, gb1[nt][j], o));
      }
    }
  }
  __syncthreads();
  float* Pp = partial + (size_t)blockIdx.x * (kParams + 1);
#pragma unroll
  for (int mt = 0; mt < 2; mt++) {
    const uint32_t ub = 32u * w + 16u * mt;
    const uint32_t am[4] = {ld_bf16x2(&dht[ub + g][2 * q]), ld_bf16x2(&dht[ub + g + 8][2 * q]),
                            ld_bf16x2(&dht[ub + g][8 + 2 * q]), ld_bf16x2(&dht[ub + g + 8][8 + 2 * q])};
#pragma unroll
    for (int nf = 0; nf < 8; nf++) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      mma_bf16_16816(d, am, ld_bf16x2(&xt[8 * nf + g][2 * q]), ld_bf16x2(&xt[8 * nf + g][8 + 2 * q]));
      const uint32_t f = 8u * nf + 2u * q;
      Pp[(size_t)(ub + g) * kFeat + f] = d[0];
      Pp[(size_t)(ub + g) * kFeat + f + 1] = d[1];
      Pp[(size_t)(ub + g + 8) * kFeat + f] = d[2];
      Pp[(size_t)(ub + g + 8) * kFeat + f + 1] = d[3];
    }
  }
  if (g == 0) {
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const uint32_t u = 32u * w + 8u * nt + 2u * q + j;
        Pp[kOffB1 + u] = gb1[nt][j];
        Pp[kOffW2 + u] = gw2[nt][j];
      }
    }
  }
  if (threadIdx.x == 0) {
    float gb2 = 0.f, loss = 0.f;
    for (int r = 0; r < 16; r++) {
      gb2 = __fadd_rn(gb2, s_dy[r]);
      loss = __fadd_rn(loss, s_loss[r]);
    }
    Pp[kOffB2] = gb2;
    Pp[kParams] = loss;
  }
}

__global__ void __launch_bounds__(256) k_mlp_reduce(const float* __restrict__ partial, uint32_t nb,
                                                    float* __restrict__ grad) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > kParams) return;
  float s = 0.f;
  for (uint32_t b = 0; b < nb; b++) s = __fadd_rn(s, partial[(size_t)b * (kParams + 1) + p]);
  grad[p] = s;
}

__global__ void __launch_bounds__(256) k_mlp_to_bf16(const float* __restrict__ master, __nv_bfloat16* __restrict__ wb) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kParams) wb[p] = __float2bfloat16_rn(master[p]);
}

__global__ void __launch_bounds__(256) k_mlp_adam(float* __restrict__ master, float* __restrict__ m1,
                                                  float* __restrict__ m2, const float* __restrict__ grad,
                                                  __nv_bfloat16* __restrict__ wb, float lr, float c1, float c2,
                                                  float* __restrict__ loss_acc) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0) *loss_acc += grad[kParams];
  if (p >= kParams) return;
  const float g = grad[p];
  const float a = 0.9f * m1[p] + 0.1f * g;
  const float b = 0.999f * m2[p] + 0.001f * g * g;
  m1[p] = a;
  m2[p] = b;
  const float w = master[p] - lr * (a * c1) / (sqrtf(b * c2) + 1e-8f);
  master[p] = w;
  wb[p] = __float2bfloat16_rn(w);
}

// Predictions for `count` rows of X (axc_mlp_predict), a block of 4 warps
// per 16 rows.
__global__ void __launch_bounds__(128) k_mlp_predict(const __nv_bfloat16* __restrict__ wb,
                                                     const float* __restrict__ X, uint32_t count,
                                                     float* __restrict__ out) {
  for (uint32_t r0 = 16u * blockIdx.x; r0 < count; r0 += 16u * gridDim.x) {
    float y;
    if (mlp_block16(wb, X + (size_t)r0 * kFeat, min(16u, count - r0), &y)) out[r0 + threadIdx.x] = y;
  }
}

}  // namespace
}  // namespace axc

// ===========================================================================
// host side
// ===========================================================================
#include <cmath>
#include <cstddef>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

namespace axc {
namespace {

// After chunks on the plain graph the features history is stale: the next
// learned tick plans without the previous tick's features (no prediction, dense).
__global__ void k_learn_resume(LearnCtl* c) { c->feat_done = 0; }

constexpr uint32_t kGateChunks = 64;   // chunks on the plain graph after a dense-only probe, at most

// What the gate reads back from the shard's control block around a chunk on
// the plain graph: the statistics counters through slot_total.
struct GateSnap {
  unsigned long long before[11], after[11];
};
constexpr size_t kGateSnapOff = offsetof(ShardCtl, ctr);
constexpr size_t kGateSnapBytes = offsetof(ShardCtl, slot_total) + sizeof(unsigned long long) - kGateSnapOff;
static_assert(kGateSnapBytes == sizeof(GateSnap::before), "GateSnap mirrors ShardCtl::ctr .. slot_total");

// Per chunk, before its graph: tick base, dopamine, and whether the chunk lays
// its rows out anew (always on learned chunks: force).
__global__ void k_learn_set_ctl(ShardCtl* ctl, uint32_t tick_base, int32_t dopamine, uint32_t force, uint32_t ticks) {
  ctl->tick_base = tick_base;
  ctl->dopamine = dopamine;
  layout_decide(ctl, force, ticks);
}

// splitmix64: seeded parameter init and minibatch order, identical on every host.
inline uint64_t smix(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

struct Learned {
  ShardVramPtrs v{};
  uint32_t N = 0, A = 0, voff = 0, nv = 0, words = 0, v_seg = 0, T = 0, tick_base = 0;
  int16_t dopamine = 0;
  const uint32_t* bits = nullptr;   // caller's device input bitmask [bits_ticks][words]
  uint32_t bits_ticks = 0;
  uint32_t sample_cap = 0;
  void* base = nullptr;
  LearnCtl* ctl = nullptr;
  uint32_t *inv_off = nullptr, *fan = nullptr, *axn = nullptr, *yacc = nullptr, *bacc = nullptr, *fill = nullptr;
  uint32_t *cap = nullptr, *part = nullptr, *alist = nullptr, *evbits = nullptr, *spk = nullptr;
  uint32_t *deg = nullptr, *bsum = nullptr, *idx = nullptr;
  int32_t* acc = nullptr;
  float *hist = nullptr, *feat = nullptr, *pred = nullptr, *X = nullptr, *Y = nullptr;
  float *master = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *loss_acc = nullptr;
  __nv_bfloat16* wb = nullptr;
  uint32_t* inv = nullptr;
  uint8_t* inv_seg = nullptr;
  size_t inv_cap = 0;
  uint32_t* stage = nullptr;
  uint32_t stage_ticks = 0;
  float* partial = nullptr;
  uint32_t partial_blocks = 0;
  uint32_t adam_step = 0;
  int32_t policy = -1;
  uint32_t collect = 0;
  // gate: after a chunk in which the predictor chose the dense form on every
  // tick, up to kGateChunks chunks run on a plain graph (no features, no plan,
  // no position map).  The plain graph's own exact counts end the gate early:
  // each gated chunk's evaluated slots and hits are read back (two chunks
  // behind, so the GPU never waits for the host), and a chunk in which the
  // sparse form could have won sends the next chunk back to the predictor.
  float ratio = 3.f;
  uint32_t gate_left = 0;
  uint64_t gated_ticks = 0;
  uint64_t chunk_no = 0;
  GateSnap* h_gate = nullptr;       // pinned, two slots (chunk number & 1)
  cudaEvent_t gate_ev[2] = {nullptr, nullptr};
  bool gate_pend[2] = {false, false};
  const void* rows_base = nullptr;   // the row cache the graphs were captured with
  std::map<std::tuple<uint32_t, uint32_t>, cudaGraphExec_t> graphs;
  cudaStream_t capture = nullptr;

  LearnDev dev() const {
    LearnDev d;
    d.ctl = ctl;
    d.inv_off = inv_off;
    d.yacc = yacc;
    d.bacc = bacc;
    d.fill = fill;
    d.cap = cap;
    d.alist = alist;
    d.evbits = evbits;
    return d;
  }
  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }
};

static void learned_free(Learned* L) {
  if (!L) return;
  L->drop_graphs();
  if (L->capture) cudaStreamDestroy(L->capture);
  for (cudaEvent_t ev : L->gate_ev)
    if (ev) cudaEventDestroy(ev);
  if (L->h_gate) cudaFreeHost(L->h_gate);
  void* ptrs[] = {L->base, L->inv, L->inv_seg, L->stage, L->partial};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete L;
}

static cudaError_t learned_partial(Learned& L, uint32_t blocks) {
  if (L.partial_blocks >= blocks) return cudaSuccess;
  if (L.partial) cudaFree(L.partial);
  L.partial = nullptr;
  L.partial_blocks = 0;
  cudaError_t e = cudaMalloc(&L.partial, (size_t)blocks * (kParams + 1) * 4);
  if (e == cudaSuccess) L.partial_blocks = blocks;
  return e;
}

// The inverted index of the current targets (and the tile fan-outs), built
// from the neuron-major rows; resets the feature history.
static cudaError_t learned_index(Learned& L, cudaStream_t st) {
  cudaError_t e;
  ShardScratch* s = scratch_for(&L.v, L.N, L.A, &e);
  if (!s) return e;
  e = rows_alloc(*s, L.N, L.A, true, st);
  if (e != cudaSuccess) return e;
  rows_touched(*s);   // slot-order rows replace the per-tick entry point's
  e = launch_rows_begin(L.v, *s, L.N, L.A, st, true, false);
  if (e != cudaSuccess) return e;
  const RowCache& r = *s->rows;
  e = cudaMemsetAsync(L.deg, 0, (size_t)L.A * 4, st);
  if (e != cudaSuccess) return e;
  const size_t slots = (size_t)L.N * kRowStride;
  const uint32_t gb = (uint32_t)((slots + 255) / 256);
  if (slots) k_inv_count<<<gb, 256, 0, st>>>(r.rt, r.cnt, L.N, L.A, L.deg);
  const uint32_t nb = (L.A + 4095) / 4096;
  if (nb > 4096) return cudaErrorInvalidValue;   // the two-level scan covers 16M axons
  k_scan_blocks<<<std::max(nb, 1u), 1024, 0, st>>>(L.deg, L.inv_off, L.A, L.bsum);
  k_scan_sums<<<1, 1024, 0, st>>>(L.bsum, std::max(nb, 1u), L.inv_off, L.A);
  k_scan_add<<<(L.A + 255) / 256, 256, 0, st>>>(L.inv_off, L.A, L.bsum);
  uint32_t total = 0;
  e = cudaMemcpyAsync(&total, L.inv_off + L.A, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (total > L.inv_cap || !L.inv) {
    if (L.inv) cudaFree(L.inv);
    if (L.inv_seg) cudaFree(L.inv_seg);
    L.inv = nullptr;
    L.inv_seg = nullptr;
    L.inv_cap = 0;
    const size_t want = std::max<size_t>(total, 1);
    e = cudaMalloc(&L.inv, want * 4);
    if (e == cudaSuccess) e = cudaMalloc(&L.inv_seg, want);
    if (e != cudaSuccess) return e;
    L.inv_cap = want;
    L.drop_graphs();
  }
  e = cudaMemcpyAsync(L.deg, L.inv_off, (size_t)L.A * 4, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  if (slots) k_inv_fill<<<gb, 256, 0, st>>>(r.rt, r.cnt, L.N, L.A, L.deg, L.inv, L.inv_seg);
  k_tile_fan<<<(L.T + 255) / 256, 256, 0, st>>>(L.inv_off, L.A, L.T, L.fan, L.axn);
  e = cudaMemsetAsync(L.hist, 0, (size_t)L.T * kHistF * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(L.yacc, 0, (size_t)L.T * 4, st);
  if (e != cudaSuccess) return e;
  k_learn_index_done<<<1, 1, 0, st>>>(L.ctl, s->ctl);
  return cudaGetLastError();
}

// The update forms of one tick: the dense update (it returns at once on a
// sparse tick that did not overflow) and the sparse kernels (they return at
// once on a dense tick), then the GSOP passes over the spikers either listed.
static void learned_update_forms(Learned& L, ShardScratch& s, uint32_t k, cudaStream_t st) {
  RowCache& r = *s.rows;
  const uint32_t N = L.N, A = L.A;
  const int sms = sm_count();
  const LearnDev D = L.dev();
  const uint32_t fix_cap = kFixCap;
  // dense: the plain engine's passes on the movable-first rows, GSOP inside them
  // (the 8-lane pass, or the lit-sum form when its lit set held)
  launch_rows_update<true>(L.v, s, N, A, k, fix_cap, L.ctl, st);
  k_rows_update_lsum<false><<<kLsumBlocks * sms, 256, 0, st>>>(L.v, A, r.rt, r.rw, r.cnt, r.mask2, r.eval, s.pend,
                                                               r.fix, s.ctl, k, fix_cap, r.lit, r.lfz, r.lsum,
                                                               ColWT{}, L.ctl);
  // sparse: the axon-driven gather, GLIF, and GSOP of the spikers it listed
  k_learn_scatter<<<8 * sms, 256, ((size_t)L.T + 1) * 4, st>>>(D, L.T, L.inv, L.inv_seg, r.mask2, r.rw, r.posmap,
                                                                L.v.soma_flags, L.v.axon_heads, A, L.acc, s.ctl);
  // 4 blocks of 256 per SM: the 32 warps per SM whose slices the GSOP passes read
  k_learn_update<<<4 * sms, 256, 0, st>>>(L.v, D, A, r.cnt, r.eval, s.pend, L.acc, r.lfz, r.gs_n, r.gd_n, r.wcnt,
                                          s.ctl, k);
  launch_rows_gsop(L.v, s, A, k, fix_cap, st, L.ctl);
}

// One tick: schedule, prologue, both update forms (the one not picked returns
// at once), fix-up, push, features + prediction.
static cudaError_t learned_tick(Learned& L, ShardScratch& s, uint32_t k, bool last, bool features_on,
                                cudaStream_t st) {
  RowCache& r = *s.rows;
  const uint32_t N = L.N, A = L.A;
  const int sms = sm_count();
  const LearnDev D = L.dev();
  const uint32_t* bits_k = L.nv ? L.stage + (size_t)k * L.words : nullptr;
  k_learn_plan<<<1, 1024, 0, st>>>(D, L.pred, L.fan, L.cap, L.part, bits_k, L.words, L.nv, s.ctl);
  const uint32_t G = std::max(A, N);
  const uint32_t raise = (bits_k && ((uint64_t)L.voff + L.nv > A)) ? AXC_ERR_VIRTUAL_RANGE : 0u;
  if (G)
    k_rows_prologue<true><<<(G + 255) / 256, 256, 0, st>>>(L.v.axon_heads, A, L.v_seg, bits_k, L.voff,
                                                           bits_k ? L.nv : 0u, s.incoming, nullptr, k, r.mask2,
                                                           r.mult, L.v.soma_flags, L.v.timers, N, r.eval, s.ctl,
                                                           raise, r.lit, D, k > 0 ? s.pend : nullptr, r.xlit);
  learned_update_forms(L, s, k, st);
  k_rows_fixup<<<2 * sms, 256, 0, st>>>(L.v, N, A, r.rt, r.rw, r.cnt, r.mask2, s.pend, r.eval, r.fix, s.ctl, k,
                                        nullptr, nullptr, 0, ColWT{});
  // soma pushes: by the next tick's prologue within a graph, here on its last tick
  if (last)
    k_rows_push<<<2 * sms, 256, 0, st>>>(L.v.axon_heads, L.v.soma_to_axon, A, s.pend, r.eval, L.v.soma_flags, N,
                                       nullptr, nullptr, 0, s.ctl, k);
  if (features_on && L.T)
    k_learn_features<<<L.T, 128, 0, st>>>(D, L.v, N, r.cnt, L.fan, L.axn, L.hist, L.feat, L.pred, L.cap, L.part,
                                          L.wb, L.X, L.Y, L.nv ? L.stage + (size_t)(k + 1) * L.words : nullptr,
                                          L.words, L.nv, s.ctl);
  if (features_on && L.T)
    k_learn_predict<<<(L.T + 15) / 16, 128, 0, st>>>(D, L.wb, L.feat, L.fan, L.pred, L.cap, L.part);
  return cudaGetLastError();
}

}  // namespace axc

using namespace axc;

extern "C" {

uint32_t axc_mlp_param_count(void) { return kParams; }

int32_t axc_learned_create(const AxcLearnedDesc* d, void** out_handle) {
  if (!d || !out_handle || !d->vram.axon_heads || d->total_axons == 0) return (int32_t)cudaErrorInvalidValue;
  if (d->d_input_bitmask && (d->words_per_tick == 0 || d->bitmask_ticks == 0)) return (int32_t)cudaErrorInvalidValue;
  Learned* L = new Learned();
  L->v = d->vram;
  L->N = d->padded_n;
  L->A = d->total_axons;
  L->voff = d->virtual_offset;
  L->nv = d->d_input_bitmask ? d->num_virtual : 0;
  L->words = d->words_per_tick;
  L->v_seg = d->v_seg;
  L->dopamine = d->dopamine;
  L->tick_base = d->tick_base;
  L->bits = d->d_input_bitmask;
  L->bits_ticks = d->d_input_bitmask ? d->bitmask_ticks : 0;
  L->sample_cap = d->sample_capacity;
  L->T = (L->A + kTileN - 1) / kTileN;
  const uint32_t T = L->T, N = L->N, A = L->A;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off = al(off + bytes); return o; };
  const size_t o_ctl = take(sizeof(LearnCtl));
  const size_t o_off = take(((size_t)A + 1) * 4), o_fan = take((size_t)T * 4), o_axn = take((size_t)T * 4);
  const size_t o_yacc = take((size_t)T * 4), o_bacc = take((size_t)T * 4), o_fill = take((size_t)T * 4);
  const size_t o_cap = take((size_t)T * 4), o_part = take((size_t)T * 16);
  const size_t o_alist = take((size_t)T * kTileN * 4), o_ev = take(((size_t)N / 32 + 2) * 4), o_spk = take((size_t)N * 4 + 4);
  const size_t o_deg = take((size_t)A * 4), o_bsum = take(4097 * 4), o_idx = take((size_t)L->sample_cap * 4 + 4);
  const size_t o_acc = take((size_t)N * 4 + 4);
  const size_t o_hist = take((size_t)T * kHistF * 4), o_feat = take((size_t)T * kFeat * 4);
  const size_t o_pred = take((size_t)T * 4);
  const size_t o_X = take((size_t)L->sample_cap * kFeat * 4), o_Y = take((size_t)L->sample_cap * 4);
  const size_t o_master = take((size_t)kParams * 4), o_m1 = take((size_t)kParams * 4), o_m2 = take((size_t)kParams * 4);
  const size_t o_grad = take(((size_t)kParams + 1) * 4), o_loss = take(4), o_wb = take((size_t)kParams * 2);
  cudaError_t e = cudaMalloc(&L->base, off);
  if (e == cudaSuccess) e = cudaMemset(L->base, 0, off);
  if (e != cudaSuccess) {
    learned_free(L);
    return (int32_t)e;
  }
  char* b = static_cast<char*>(L->base);
  L->ctl = reinterpret_cast<LearnCtl*>(b + o_ctl);
  L->inv_off = reinterpret_cast<uint32_t*>(b + o_off);
  L->fan = reinterpret_cast<uint32_t*>(b + o_fan);
  L->axn = reinterpret_cast<uint32_t*>(b + o_axn);
  L->yacc = reinterpret_cast<uint32_t*>(b + o_yacc);
  L->bacc = reinterpret_cast<uint32_t*>(b + o_bacc);
  L->fill = reinterpret_cast<uint32_t*>(b + o_fill);
  L->cap = reinterpret_cast<uint32_t*>(b + o_cap);
  L->part = reinterpret_cast<uint32_t*>(b + o_part);
  L->alist = reinterpret_cast<uint32_t*>(b + o_alist);
  L->evbits = reinterpret_cast<uint32_t*>(b + o_ev);
  L->spk = reinterpret_cast<uint32_t*>(b + o_spk);
  L->deg = reinterpret_cast<uint32_t*>(b + o_deg);
  L->bsum = reinterpret_cast<uint32_t*>(b + o_bsum);
  L->idx = reinterpret_cast<uint32_t*>(b + o_idx);
  L->acc = reinterpret_cast<int32_t*>(b + o_acc);
  L->hist = reinterpret_cast<float*>(b + o_hist);
  L->feat = reinterpret_cast<float*>(b + o_feat);
  L->pred = reinterpret_cast<float*>(b + o_pred);
  L->X = reinterpret_cast<float*>(b + o_X);
  L->Y = reinterpret_cast<float*>(b + o_Y);
  L->master = reinterpret_cast<float*>(b + o_master);
  L->m1 = reinterpret_cast<float*>(b + o_m1);
  L->m2 = reinterpret_cast<float*>(b + o_m2);
  L->grad = reinterpret_cast<float*>(b + o_grad);
  L->loss_acc = reinterpret_cast<float*>(b + o_loss);
  L->wb = reinterpret_cast<__nv_bfloat16*>(b + o_wb);
  // control block defaults
  LearnCtl hc;
  std::memset(&hc, 0, sizeof(hc));
  hc.sample_cap = L->sample_cap;
  hc.sample_every = 1;
  hc.policy = -1;
  hc.ratio = 3.f;
  hc.margin = 0.25f;
  hc.slack = 64;
  hc.T = T;
  // seeded uniform init of W1 (fan-in scaled); biases and w2 zero, so the
  // untrained network predicts the last-tick rule
  std::vector<float> w(kParams, 0.f);
  uint64_t sd = 0xA11CE5EEDull;
  for (uint32_t p = 0; p < kParams; p++) {
    const float u = (float)(smix(sd) >> 40) * (1.f / 16777216.f) * 2.f - 1.f;
    if (p < kOffB1) w[p] = u * 0.30618622f;   // sqrt(6 / 64)
  }
  e = cudaMemcpy(L->ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(L->master, w.data(), (size_t)kParams * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_mlp_to_bf16<<<(kParams + 255) / 256, 256>>>(L->master, L->wb);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L->capture, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaHostAlloc(&L->h_gate, 2 * sizeof(GateSnap), cudaHostAllocDefault);
  for (int q = 0; q < 2 && e == cudaSuccess; q++) e = cudaEventCreateWithFlags(&L->gate_ev[q], cudaEventDisableTiming);
  if (e == cudaSuccess && ((size_t)T + 1) * 4 > 48 * 1024)
    e = cudaFuncSetAttribute(k_learn_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(((size_t)T + 1) * 4));
  if (e == cudaSuccess) e = learned_index(*L, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    learned_free(L);
    return (int32_t)e;
  }
  *out_handle = L;
  return 0;
}

void axc_learned_destroy(void* handle) { learned_free(static_cast<Learned*>(handle)); }

int32_t axc_learned_refresh(void* handle, void* stream_v) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L) return (int32_t)cudaErrorInvalidValue;
  return (int32_t)learned_index(*L, static_cast<cudaStream_t>(stream_v));
}

int32_t axc_learned_set_policy(void* handle, int32_t policy, float ratio, float margin, uint32_t slack) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L || policy < -1 || policy > 1 || !(ratio >= 0.f) || !(margin >= 0.f)) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e = cudaDeviceSynchronize();
  LearnCtl hc;
  if (e == cudaSuccess) e = cudaMemcpy(&hc, L->ctl, sizeof(hc), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return (int32_t)e;
  hc.policy = policy;
  hc.ratio = ratio;
  hc.margin = margin;
  hc.slack = slack;
  L->policy = policy;
  L->ratio = ratio;
  L->gate_left = 0;
  L->gate_pend[0] = L->gate_pend[1] = false;
  return (int32_t)cudaMemcpy(L->ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice);
}

int32_t axc_learned_collect(void* handle, uint32_t enable, uint32_t sample_every, uint32_t reset) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L || sample_every == 0) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e = cudaDeviceSynchronize();
  LearnCtl hc;
  if (e == cudaSuccess) e = cudaMemcpy(&hc, L->ctl, sizeof(hc), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return (int32_t)e;
  // the pairs of the last tick collected are committed when the next tick is
  // planned; switching collection off commits them here
  if (hc.collect && !enable && hc.feat_done && hc.ticks_seen >= 1 && (hc.ticks_seen % hc.sample_every) == 0 &&
      hc.samples + hc.T <= hc.sample_cap)
    hc.samples += hc.T;
  hc.collect = enable ? 1u : 0u;
  hc.sample_every = sample_every;
  if (reset) hc.samples = 0;
  L->collect = hc.collect;
  return (int32_t)cudaMemcpy(L->ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice);
}

int32_t axc_learned_run(void* handle, uint32_t tick0, uint32_t ticks, uint32_t tpg, void* stream_v) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L || tpg == 0 || ticks % tpg) return (int32_t)cudaErrorInvalidValue;
  if (L->bits && (uint64_t)tick0 + ticks > L->bits_ticks) return (int32_t)cudaErrorInvalidValue;
  cudaStream_t st = static_cast<cudaStream_t>(stream_v);
  cudaError_t e;
  ShardScratch* s = scratch_for(&L->v, L->N, L->A, &e);
  if (!s) return (int32_t)e;
  e = rows_alloc(*s, L->N, L->A, true, st);
  if (e == cudaSuccess) e = rows_posmap(*s, st);
  if (e != cudaSuccess) return (int32_t)e;
  s->tick_rows_valid.store(false);   // this run's rows replace the per-tick entry point's
  if (L->rows_base != s->rows->base) {
    L->drop_graphs();
    L->rows_base = s->rows->base;
  }
  if (L->stage_ticks < tpg + 1) {
    if (L->stage) cudaFree(L->stage);
    L->stage = nullptr;
    L->stage_ticks = 0;
    e = cudaMalloc(&L->stage, (size_t)(tpg + 1) * std::max(L->words, 1u) * 4);
    if (e != cudaSuccess) return (int32_t)e;
    L->stage_ticks = tpg + 1;
    L->drop_graphs();
  }
  const bool features_on = L->policy < 0 || L->collect;
  // graph kinds: 0/1 learned (features off/on), 2 plain (the gate); the row
  // layout of each chunk follows the device's decision (layout_decide)
  auto graph_of = [&](uint32_t kind, cudaGraphExec_t* out) -> cudaError_t {
    const auto key = std::make_tuple(tpg, kind);
    auto it = L->graphs.find(key);
    if (it != L->graphs.end()) {
      *out = it->second;
      return cudaSuccess;
    }
    cudaError_t ce = cudaStreamBeginCapture(L->capture, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) return ce;
    // every layout of this engine writes the index checksum and the position
    // map (the sparse form reads the rows through it), when the device lays out
    cudaError_t le = launch_rows_begin(L->v, *s, L->N, L->A, L->capture, true, true, true, true);
    for (uint32_t k = 0; k < tpg && le == cudaSuccess; k++) {
      if (kind == 2) {   // the plain engine's tick on the staged bitmask rows
        TickArgs a{};
        a.padded_n = L->N;
        a.total_axons = L->A;
        a.v_seg = L->v_seg;
        a.input_bitmask = L->nv ? L->stage + (size_t)k * L->words : nullptr;
        a.virtual_offset = L->voff;
        a.num_virtual = a.input_bitmask ? L->nv : 0u;
        a.batch = true;
        a.k = k;
        a.rows = true;
        a.defer_push = k + 1 < tpg;
        a.fix_cap = kFixCap;
        le = launch_tick(L->v, *s, a, L->capture);
      } else {
        le = learned_tick(*L, *s, k, k + 1 == tpg, kind == 1, L->capture);
      }
    }
    if (le == cudaSuccess) le = launch_rows_end(L->v, *s, L->N, L->capture);
    cudaGraph_t g = nullptr;
    ce = cudaStreamEndCapture(L->capture, &g);
    if (le != cudaSuccess) ce = le;
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(out, g, 0);
    if (g) cudaGraphDestroy(g);
    if (ce == cudaSuccess) L->graphs[key] = *out;
    return ce;
  };
  const bool gate_on = L->policy < 0 && !L->collect;
  for (uint32_t c = 0; c < ticks / tpg && e == cudaSuccess; c++) {
    const uint32_t t0 = tick0 + c * tpg;
    const uint32_t slot = (uint32_t)(L->chunk_no++ & 1u);
    // the counts of the gated chunk two chunks back (its copies are done once
    // the chunk before this one started): could the sparse form have won?
    if (L->gate_pend[slot]) {
      L->gate_pend[slot] = false;
      e = cudaEventSynchronize(L->gate_ev[slot]);
      if (e != cudaSuccess) break;
      const GateSnap& g = L->h_gate[slot];
      const double ev_slots = (double)(g.after[1] - g.before[1]), hit = (double)(g.after[2] - g.before[2]);
      const double live = (double)g.after[10] * tpg;   // live slots x ticks: the active synapses scale with them
      if (gate_on && L->gate_left > 0 && ev_slots > 0 && (double)L->ratio * hit * live < ev_slots * ev_slots) {
        L->gate_left = 0;
        k_learn_resume<<<1, 1, 0, st>>>(L->ctl);   // the features history is stale
      }
    }
    const bool gated = gate_on && L->gate_left > 0;
    // the first chunk of a call lays the rows out (another path may have laid
    // them out without the position map since); later chunks keep them as the
    // batch path does
    const bool force = batch_rows_force(*s) || c == 0;
    cudaGraphExec_t exec = nullptr;
    e = graph_of(gated ? 2u : (features_on ? 1u : 0u), &exec);
    if (e != cudaSuccess) break;
    if (L->bits) {
      const uint32_t have = std::min(tpg + 1, L->bits_ticks - t0);
      e = cudaMemcpyAsync(L->stage, L->bits + (size_t)t0 * L->words, (size_t)have * L->words * 4,
                          cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess && have < tpg + 1)
        e = cudaMemsetAsync(L->stage + (size_t)have * L->words, 0, (size_t)(tpg + 1 - have) * L->words * 4, st);
      if (e != cudaSuccess) break;
    }
    k_learn_set_ctl<<<1, 1, 0, st>>>(s->ctl, L->tick_base + t0, (int32_t)L->dopamine, force ? 1u : 0u, tpg);
    e = launch_reset_burst(L->v, L->N, st);
    unsigned long long picked0 = 0, picked1 = 0;
    const size_t picked_at = offsetof(LearnCtl, stat) + kStSparsePicked * sizeof(unsigned long long);
    if (e == cudaSuccess && gate_on && !gated)
      e = cudaMemcpyAsync(&picked0, reinterpret_cast<char*>(L->ctl) + picked_at, 8, cudaMemcpyDeviceToHost, st);
    const char* snap_src = reinterpret_cast<const char*>(s->ctl) + kGateSnapOff;
    if (e == cudaSuccess && gated)
      e = cudaMemcpyAsync(L->h_gate[slot].before, snap_src, kGateSnapBytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
    if (e != cudaSuccess) break;
    if (gated) {
      e = cudaMemcpyAsync(L->h_gate[slot].after, snap_src, kGateSnapBytes, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaEventRecord(L->gate_ev[slot], st);
      if (e != cudaSuccess) break;
      L->gate_pend[slot] = true;
      L->gate_left--;
      L->gated_ticks += tpg;
      if (L->gate_left == 0) k_learn_resume<<<1, 1, 0, st>>>(L->ctl);   // the features history is stale
      continue;
    }
    if (!gate_on) continue;
    // a probe chunk: did the predictor choose the sparse form on any tick?
    e = cudaMemcpyAsync(&picked1, reinterpret_cast<char*>(L->ctl) + picked_at, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) break;
    if (picked1 == picked0) L->gate_left = kGateChunks;
  }
  return (int32_t)e;
}

int32_t axc_learned_stats(void* handle, uint64_t* out16) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L || !out16) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e = cudaDeviceSynchronize();
  LearnCtl hc;
  if (e == cudaSuccess) e = cudaMemcpy(&hc, L->ctl, sizeof(hc), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return (int32_t)e;
  for (int q = 0; q < 12; q++) out16[q] = hc.stat[q];
  out16[9] = L->gated_ticks;
  out16[12] = hc.samples;
  out16[13] = hc.ticks_seen;
  out16[14] = hc.T;
  out16[15] = L->inv_cap;
  return 0;
}

int32_t axc_learned_reset_stats(void* handle) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess)
    e = cudaMemset(reinterpret_cast<char*>(L->ctl) + offsetof(LearnCtl, stat), 0, sizeof(LearnCtl::stat));
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);   // cleared before a run on any stream
  L->gated_ticks = 0;
  return (int32_t)e;
}

int32_t axc_learned_params(void* handle, float* host_out, const float* host_in) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && host_out) e = cudaMemcpy(host_out, L->master, (size_t)kParams * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && host_in) {
    e = cudaMemcpy(L->master, host_in, (size_t)kParams * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(L->m1, 0, (size_t)kParams * 4);
    if (e == cudaSuccess) e = cudaMemset(L->m2, 0, (size_t)kParams * 4);
    if (e == cudaSuccess) {
      k_mlp_to_bf16<<<(kParams + 255) / 256, 256>>>(L->master, L->wb);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);   // in place before a run on any stream
    L->adam_step = 0;
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int32_t)e;
}

// Adam on the recorded pairs: the first 90% (in recording order) train, the
// last 10% validate.  out_loss[epoch] = mean training loss of the epoch.
int32_t axc_learned_train(void* handle, uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float* out_loss,
                          float* out_val, void* stream_v) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L || batch == 0 || !(lr > 0.f)) return (int32_t)cudaErrorInvalidValue;
  cudaStream_t st = static_cast<cudaStream_t>(stream_v);
  cudaError_t e = cudaDeviceSynchronize();
  uint32_t n = 0;
  if (e == cudaSuccess)
    e = cudaMemcpy(&n, reinterpret_cast<char*>(L->ctl) + offsetof(LearnCtl, samples), 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return (int32_t)e;
  const uint32_t nval = n / 10, ntr = n - nval;
  if (ntr == 0) return (int32_t)cudaErrorInvalidValue;
  const uint32_t maxb = std::max((std::min(batch, ntr) + kGradPer - 1) / kGradPer, (nval + kGradPer - 1) / kGradPer);
  e = learned_partial(*L, std::max(maxb, 1u));
  if (e != cudaSuccess) return (int32_t)e;
  std::vector<uint32_t> order(ntr);
  for (uint32_t i = 0; i < ntr; i++) order[i] = i;
  uint64_t sd = seed;
  for (uint32_t ep = 0; ep < epochs && e == cudaSuccess; ep++) {
    for (uint32_t i = ntr - 1; i > 0; i--) std::swap(order[i], order[(uint32_t)(smix(sd) % (uint64_t)(i + 1))]);
    e = cudaMemcpyAsync(L->idx, order.data(), (size_t)ntr * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(L->loss_acc, 0, 4, st);
    uint32_t steps = 0;
    for (uint32_t b0 = 0; b0 < ntr && e == cudaSuccess; b0 += batch) {
      const uint32_t cnt = std::min(batch, ntr - b0);
      const uint32_t nb = (cnt + kGradPer - 1) / kGradPer;
      k_mlp_grad<<<nb, 128, 0, st>>>(L->wb, L->X, L->Y, L->idx + b0, cnt, 1.f / (float)cnt, L->partial);
      k_mlp_reduce<<<(kParams + 1 + 255) / 256, 256, 0, st>>>(L->partial, nb, L->grad);
      L->adam_step++;
      const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)L->adam_step)));
      const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)L->adam_step)));
      k_mlp_adam<<<(kParams + 255) / 256, 256, 0, st>>>(L->master, L->m1, L->m2, L->grad, L->wb, lr, c1, c2,
                                                       L->loss_acc);
      e = cudaGetLastError();
      steps++;
    }
    float tot = 0.f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tot, L->loss_acc, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (out_loss) out_loss[ep] = steps ? tot / (float)steps : 0.f;
  }
  if (e == cudaSuccess && out_val) {
    *out_val = 0.f;
    if (nval) {
      const uint32_t nb = (nval + kGradPer - 1) / kGradPer;
      k_mlp_grad<<<nb, 128, 0, st>>>(L->wb, L->X + (size_t)ntr * kFeat, L->Y + ntr, nullptr, nval,
                                     1.f / (float)nval, L->partial);
      k_mlp_reduce<<<(kParams + 1 + 255) / 256, 256, 0, st>>>(L->partial, nb, L->grad);
      e = cudaMemcpyAsync(out_val, L->grad + kParams, 4, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
  }
  return (int32_t)e;
}

// Copies recorded pairs out (rows [first, first + count)).
int32_t axc_learned_samples(void* handle, uint32_t first, uint32_t count, float* host_x, float* host_y) {
  Learned* L = static_cast<Learned*>(handle);
  if (!L || (uint64_t)first + count > L->sample_cap) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && host_x)
    e = cudaMemcpy(host_x, L->X + (size_t)first * kFeat, (size_t)count * kFeat * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && host_y) e = cudaMemcpy(host_y, L->Y + first, (size_t)count * 4, cudaMemcpyDeviceToHost);
  return (int32_t)e;
}

// Stand-alone MLP entry points on caller buffers (FP32 parameters, rounded to
// BF16 inside): the mean squared error and its gradient, and predictions.
int32_t axc_mlp_loss_grad(const float* d_params, const float* d_x, const float* d_y, uint32_t count, float* d_grad,
                          float* d_loss, void* stream_v) {
  if (!d_params || !d_x || !d_y || !d_grad || count == 0) return (int32_t)cudaErrorInvalidValue;
  cudaStream_t st = static_cast<cudaStream_t>(stream_v);
  const uint32_t nb = (count + kGradPer - 1) / kGradPer;
  __nv_bfloat16* wb = nullptr;
  float *partial = nullptr, *grad = nullptr;
  cudaError_t e = cudaMalloc(&wb, (size_t)kParams * 2);
  if (e == cudaSuccess) e = cudaMalloc(&partial, (size_t)nb * (kParams + 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&grad, ((size_t)kParams + 1) * 4);
  if (e == cudaSuccess) {
    k_mlp_to_bf16<<<(kParams + 255) / 256, 256, 0, st>>>(d_params, wb);
    k_mlp_grad<<<nb, 128, 0, st>>>(wb, d_x, d_y, nullptr, count, 1.f / (float)count, partial);
    k_mlp_reduce<<<(kParams + 1 + 255) / 256, 256, 0, st>>>(partial, nb, grad);
    e = cudaMemcpyAsync(d_grad, grad, (size_t)kParams * 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && d_loss) e = cudaMemcpyAsync(d_loss, grad + kParams, 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (wb) cudaFree(wb);
  if (partial) cudaFree(partial);
  if (grad) cudaFree(grad);
  return (int32_t)e;
}

int32_t axc_mlp_predict(const float* d_params, const float* d_x, uint32_t count, float* d_out, void* stream_v) {
  if (!d_params || !d_x || !d_out) return (int32_t)cudaErrorInvalidValue;
  if (count == 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream_v);
  __nv_bfloat16* wb = nullptr;
  cudaError_t e = cudaMalloc(&wb, (size_t)kParams * 2);
  if (e == cudaSuccess) {
    k_mlp_to_bf16<<<(kParams + 255) / 256, 256, 0, st>>>(d_params, wb);
    k_mlp_predict<<<std::min((count + 15u) / 16u, 8192u), 128, 0, st>>>(wb, d_x, count, d_out);
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (wb) cudaFree(wb);
  return (int32_t)e;
}

}  // extern "C"
