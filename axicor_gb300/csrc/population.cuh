// population.cuh — many independent brains stepped together (compiled as part
// of day_phase.cu, with the row engine's helpers).
//
// Per tick the whole population runs five launches, captured once into a CUDA
// graph of several ticks:
//   k_pop_prologue  block -> brain map: each brain's axons and somas, as the row
//                   engine's prologue, with the brain's own bitmask row
//   k_pop_chunks    one block: cuts every brain's list of evaluated neurons into
//                   chunks of `chunk` neurons (the work list of the next stages)
//   k_pop_update    persistent grid over chunks; a block stages the chunk's brain
//                   descriptor, LUT, GSOP table and fully-lit bitmap in shared
//                   memory, then runs the row engine's update with GSOP of the
//                   movable slots, LANES lanes per neuron
//   k_pop_fixup     deferred GSOP slots of all brains
//   k_pop_push      the spikers' own-axon pushes, per chunk, on a graph's last
//                   tick (on the others the next prologue applies them)
// Batch prologue/epilogue (once per run): GSOP tables, soma multiplicity,
// neuron-major rows with their movable slots first, weight write-back, each
// as one launch over all brains.
// Every brain evolves exactly as it would alone in axc_step_day_phase_batch.

namespace axc {

struct PopBrain {
  ShardVramPtrs P;
  const uint32_t* bitmask;
  const VariantParameters* lut;
  int2* gtab;          // [16][16] GSOP (potentiation, depression), this batch's dopamine
  uint32_t* rt;
  int16_t* rw;
  uint16_t* cnt;
  uint2* mask2;
  uint32_t* mult;
  uint32_t* eval;
  uint32_t* pend;
  ShardCtl* ctl;
  uint32_t* lit;       // [A/32+1] the tick's fully-lit axons, one bit each
  uint8_t* lfz;        // [N] movable slots of each row (placed first by the row copy)
  uint4* amask;        // [N] their row positions
  uint4* omask;        // [N] the columnar slots placed first (for the write-back)
  uint32_t N, A, voff, nv, words, v_seg, tick_base, pmax;
  int32_t dopamine;
  uint32_t pad[3];
};

struct PopCtl {
  uint32_t tick0;          // bitmask row of tick k of the running graph = tick0 + k
  uint32_t nchunks[2];     // chunks of tick k in slot k & 1
  uint32_t fix_count, fix_overflow, err;
  uint32_t pad[2];
  unsigned long long ctr[8];
};

namespace {

constexpr uint32_t kPopChunk = 256;   // evaluated neurons per chunk
constexpr uint32_t kPopLitWords = 12288;   // 48 KB: brains of up to 393k axons stage their fully-lit bitmap

__device__ __forceinline__ uint32_t pmax_of(const VariantParameters* lut) {
  uint32_t m = 0;
  for (int v = 0; v < 16; v++) m = max(m, (uint32_t)lut[v].signal_propagation_length);
  return m;
}

// batch start, one block per brain: GSOP table, list counters, dummy mask entry,
// multiplicity reset.
__global__ void __launch_bounds__(256) k_pop_begin(PopBrain* __restrict__ brains) {
  PopBrain& b = brains[blockIdx.x];
  const uint32_t v = threadIdx.x >> 4, r = threadIdx.x & 15;
  const VariantParameters& p = b.lut[v];
  const GsopConsts g = gsop_consts((uint8_t)((v << 4) | 0x05), p, b.dopamine);
  const int32_t inertia = p.inertia_curve[r];
  b.gtab[threadIdx.x] =
      make_int2(wmul(wmul(g.raw_pot, inertia), g.bm) >> 7, wmul(wmul(g.final_dep, inertia), g.bm) >> 7);
  if (threadIdx.x == 0) {
    b.pmax = pmax_of(b.lut);
    b.ctl->row_smax = 0;
    b.ctl->seg_max = 0;
    b.ctl->eval_count[0] = 0;
    b.ctl->eval_count[1] = 0;
    b.mask2[b.A] = make_uint2(0u, 0x80000000u);
  }
  for (uint32_t a = threadIdx.x; a < b.A; a += blockDim.x) b.mult[a] = 0;
}

__device__ __forceinline__ uint32_t block_brain(const uint32_t* map, const uint32_t* first, uint32_t* local) {
  const uint32_t b = map[blockIdx.x];
  *local = blockIdx.x - first[b];
  return b;
}

__global__ void __launch_bounds__(256) k_pop_mult(const PopBrain* __restrict__ brains, const uint32_t* __restrict__ map,
                                                  const uint32_t* __restrict__ first) {
  uint32_t lb;
  const PopBrain& b = brains[block_brain(map, first, &lb)];
  const uint32_t n = lb * 256 + threadIdx.x;
  if (n >= b.N) return;
  const uint32_t a = b.P.soma_to_axon[n];
  if (a < b.A) atomicAdd(&b.mult[a], 1u);
}

// columnar -> rows for 32 neurons of one brain (build_row: movable slots
// first), and the batch's burst reset (genesis-compute/src/compute/shard.rs:71,
// physics.cu:25-30).
__global__ void __launch_bounds__(256) k_pop_build(const PopBrain* __restrict__ brains,
                                                   const uint32_t* __restrict__ map,
                                                   const uint32_t* __restrict__ first) {
  __shared__ uint32_t s_t[AXC_MAX_DENDRITES][33];
  __shared__ int16_t s_w[AXC_MAX_DENDRITES][34];
  __shared__ uint32_t s_cnt[32];
  uint32_t lb;
  const PopBrain& b = brains[block_brain(map, first, &lb)];
  const uint32_t N = b.N, A = b.A;
  const uint32_t n0 = lb * 32;
  const uint32_t col = threadIdx.x & 31, r0 = threadIdx.x >> 5;
  if (threadIdx.x < 32) {
    s_cnt[threadIdx.x] = AXC_MAX_DENDRITES;
    if (n0 + threadIdx.x < N) b.P.soma_flags[n0 + threadIdx.x] &= 0xF1;
  }
  __syncthreads();
  for (uint32_t ch = 0; ch < AXC_MAX_DENDRITES / 8; ch++) {
    const uint32_t r = ch * 8 + r0, n = n0 + col;
    uint32_t t = 0;
    int16_t w = 0;
    if (n < N) {
      t = __ldcs(b.P.dendrite_targets + (size_t)r * N + n);
      w = __ldcs(b.P.dendrite_weights + (size_t)r * N + n);
    }
    s_t[r][col] = t;
    s_w[r][col] = w;
    if (t == 0) atomicMin(&s_cnt[col], r);
    __syncthreads();
    const int mine = threadIdx.x < 32 ? (s_cnt[threadIdx.x] < (ch + 1) * 8) : 1;
    if (__syncthreads_and(mine)) break;
  }
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ uint32_t s_bc[8], s_bs[8];
  uint32_t wc = 0, ws = 0;
  for (uint32_t j = warp; j < 32; j += 8) {
    const uint32_t n = n0 + j;
    if (n >= N) continue;
    const uint32_t c = s_cnt[j];
    const RowBuilt rb = build_row(s_t, s_w, j, n, c, frozen_from(b.lut[b.P.soma_flags[n] >> 4]), A, false, true,
                                  b.rt, b.rw, b.cnt, b.amask, b.omask, b.lfz);
    if (lane == 0 && c) {
      wc = max(wc, c);
      ws = max(ws, rb.smx);
    }
  }
  if (lane == 0) { s_bc[warp] = wc; s_bs[warp] = ws; }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t bc = 0, bs = 0;
    for (int q = 0; q < 8; q++) { bc = max(bc, s_bc[q]); bs = max(bs, s_bs[q]); }
    if (bc) atomicMax(&b.ctl->row_smax, bc);
    if (bs) atomicMax(&b.ctl->seg_max, bs);
  }
}

__global__ void __launch_bounds__(256) k_pop_writeback(const PopBrain* __restrict__ brains,
                                                       const uint32_t* __restrict__ map,
                                                       const uint32_t* __restrict__ first) {
  __shared__ int16_t s_w[AXC_MAX_DENDRITES][34];
  __shared__ uint32_t s_c[32];
  uint32_t lb;
  const PopBrain& b = brains[block_brain(map, first, &lb)];
  writeback_tile(b.P.dendrite_weights, b.N, lb * 32, b.rw, b.cnt, b.omask, s_w, s_c);
}

// per tick 1/5: k_rows_prologue per brain (block -> brain map), with the
// brain's fully-lit bitmap.  apply_pend: the previous tick's soma pushes,
// deferred to here within a graph (pushes commute), go in with the input pushes.
__global__ void __launch_bounds__(256) k_pop_prologue(const PopBrain* __restrict__ brains,
                                                      const uint32_t* __restrict__ map,
                                                      const uint32_t* __restrict__ first,
                                                      PopCtl* __restrict__ pctl, uint32_t k, uint32_t apply_pend) {
  __shared__ uint32_t s_base;
  __shared__ uint32_t s_warp[8];
  uint32_t lb;
  const uint32_t bi = block_brain(map, first, &lb);
  const PopBrain& b = brains[bi];
  const uint32_t A = b.A, N = b.N;
  const uint32_t i = lb * 256 + threadIdx.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&pctl->ctr[0], 1ull);
    pctl->fix_count = 0;      // the previous tick's fix-up is done
    pctl->fix_overflow = 0;
  }
  bool lit = false;
  if (i < A) {
    uint4* p = reinterpret_cast<uint4*>(b.P.axon_heads + i);
    const uint4 x = p[0], y = p[1];
    uint32_t h[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
    uint32_t npush = 0;
    if (b.bitmask) {
      const uint32_t v = i - b.voff;
      if (v < b.nv)
        npush += (__ldg(b.bitmask + (size_t)(pctl->tick0 + k) * b.words + (v >> 5)) >> (v & 31u)) & 1u;
    }
    if (apply_pend) {
      const uint32_t c = b.pend[i];
      if (c) {
        npush += c;
        b.pend[i] = 0;
      }
    }
    push_n(h, npush);
    const uint32_t vs = b.v_seg;
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (h[j] != AXC_AXON_SENTINEL) h[j] += vs;
    p[0] = make_uint4(h[0], h[1], h[2], h[3]);
    p[1] = make_uint4(h[4], h[5], h[6], h[7]);
    const uint2 m = split_masks(h, b.pmax, b.mult[i]);
    b.mask2[i] = m;
    // fully lit: heads 0..6 hit every segment 1..seg_max the brain's slots use
    // and one soma at most owns the axon (as in k_rows_prologue)
    const uint32_t hi = min(b.ctl->seg_max, 30u);
    const uint32_t need = hi ? (((2u << hi) - 1u) & ~1u) : 0xFFFFFFFFu;
    lit = (m.x & need) == need && !(m.y >> 31);
  }
  {
    const uint32_t lbits = __ballot_sync(kFull, lit);
    if ((threadIdx.x & 31) == 0 && i < A) b.lit[i >> 5] = lbits;
  }
  bool ev = false;
  if (i < N) {
    const uint8_t t = b.P.timers[i];
    if (t > 0) {
      b.P.timers[i] = (uint8_t)(t - 1);
      b.P.soma_flags[i] = b.P.soma_flags[i] & 0xF0;
    } else {
      ev = true;
    }
  }
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t ballot = __ballot_sync(kFull, ev);
  if (lane == 0) s_warp[w] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int q = 0; q < 8; q++) { const uint32_t c = s_warp[q]; s_warp[q] = tot; tot += c; }
    s_base = tot ? atomicAdd(&b.ctl->eval_count[k & 1], tot) : 0u;
  }
  __syncthreads();
  if (ev) b.eval[s_base + s_warp[w] + __popc(ballot & ((1u << lane) - 1u))] = i;
}

// per tick 2/5: chunk list (brain, first list index) over all brains.
__global__ void __launch_bounds__(1024) k_pop_chunks(const PopBrain* __restrict__ brains, uint32_t count,
                                                     uint2* __restrict__ chunks, PopCtl* __restrict__ pctl,
                                                     uint32_t k, uint32_t chunk) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (count + 1023) / 1024;
  const uint32_t b0 = threadIdx.x * per;
  uint32_t s = 0;
  for (uint32_t b = b0; b < min(b0 + per, count); b++) s += (brains[b].ctl->eval_count[k & 1] + chunk - 1) / chunk;
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int i = 0; i < 1024; i++) { const uint32_t x = part[i]; part[i] = acc; acc += x; }
    pctl->nchunks[k & 1] = acc;
  }
  __syncthreads();
  uint32_t pos = part[threadIdx.x];
  for (uint32_t b = b0; b < min(b0 + per, count); b++) {
    const uint32_t e = brains[b].ctl->eval_count[k & 1];
    for (uint32_t st = 0; st < e; st += chunk) chunks[pos++] = make_uint2(b, st);
  }
}

// Shared-memory copy of one brain's constants for a block.
struct PopStage {
  PopBrain b;
  VariantParameters lut[16];
  int2 gtab[16][16];
  uint32_t brain;
};

// With lit_cap > 0 the brain's fully-lit bitmap (when it has at most lit_cap
// words) goes to s_lit too.
__device__ __forceinline__ void stage_brain(PopStage& st, const PopBrain* brains, uint32_t bi, uint32_t* s_lit,
                                            uint32_t lit_cap) {
  __syncthreads();
  if (st.brain != bi) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(brains + bi);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&st.b);
    for (uint32_t i = threadIdx.x; i < sizeof(PopBrain) / 4; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    const uint32_t words = (st.b.A >> 5) + 1;
    if (words <= lit_cap) {
      const uint32_t* lw = st.b.lit;
      for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) s_lit[i] = __ldg(lw + i);
    }
    const uint32_t* ls = reinterpret_cast<const uint32_t*>(st.b.lut);
    uint32_t* ld = reinterpret_cast<uint32_t*>(st.lut);
    for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) ld[i] = ls[i];
    int2* gd = &st.gtab[0][0];
    for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) gd[i] = st.b.gtab[i];
    if (threadIdx.x == 0) st.brain = bi;
  }
  __syncthreads();
}

// per tick 3/5: update + GSOP of every evaluated neuron of every brain,
// LANES lanes per neuron (lane g holds slots (4*LANES)*j + 4g .. +3).  Slots
// of fully-lit axons (the brain's bitmap staged in shared memory when it has
// at most lit_cap words) hit without a mask gather; a round whose slots are
// all fully lit skips the mask path warp-uniformly.  GSOP runs over the
// movable slots only, the first lfz of the row.
template <int LANES>
__global__ void __launch_bounds__(256, 3) k_pop_update(const PopBrain* __restrict__ brains, const uint2* __restrict__ chunks,
                                                    PopCtl* __restrict__ pctl, uint2* __restrict__ fix,
                                                    uint32_t k, uint32_t chunk, uint32_t fix_cap, uint32_t lit_cap) {
  extern __shared__ uint32_t s_lit[];
  constexpr int CH = 32 / LANES;      // chunks of 4 slots per lane
  constexpr int G = 32 / LANES;       // neurons per warp
  constexpr int SPAN = 4 * LANES;     // slots covered by one chunk of all lanes
  __shared__ PopStage st;
  if (threadIdx.x == 0) st.brain = 0xFFFFFFFFu;
  const uint32_t nch = pctl->nchunks[k & 1];
  const uint32_t lane = threadIdx.x & 31, gl = lane % LANES, grp = lane / LANES, warp = threadIdx.x >> 5;
  uint32_t ev_slots = 0, hits = 0, nspk = 0, gdone = 0, nev = 0, err = 0;
  for (uint32_t ci = blockIdx.x; ci < nch; ci += gridDim.x) {
    const uint2 cd = chunks[ci];
    stage_brain(st, brains, cd.x, s_lit, lit_cap);
    const PopBrain& b = st.b;
    const uint32_t A = b.A;
    const bool use_lit = (A >> 5) + 1 <= lit_cap;
    const uint32_t seg_hi = min(b.ctl->seg_max, 30u);   // lit bits cover segments 1..seg_hi
    const uint32_t tick = b.tick_base + pctl->tick0 + k;
    const uint32_t ecount = min(b.ctl->eval_count[k & 1] - cd.y, chunk);
    const uint32_t smax = b.ctl->row_smax;
    for (uint32_t off = warp * G; off < ecount; off += 8 * G) {
      const uint32_t idx = off + grp;
      const bool valid = idx < ecount;
      const uint32_t n = valid ? __ldg(b.eval + cd.y + idx) : 0u;
      const uint8_t flags = b.P.soma_flags[n];
      const uint32_t cw = valid ? b.cnt[n] : 0u;
      const uint32_t lf = valid ? b.lfz[n] : 0u;
      const int32_t thr0 = b.P.threshold_offset[n];
      const int32_t v0 = b.P.soma_voltage[n];
      const uint32_t* trow = b.rt + (size_t)n * kRowStride + 4u * gl;
      int16_t* wrow = b.rw + (size_t)n * kRowStride + 4u * gl;
      uint4 T[CH];
      uint2 W[CH];
#pragma unroll
      for (int j = 0; j < CH; j++) {
        if (valid && (uint32_t)(SPAN * j) + 4u * gl < smax) {
          T[j] = __ldg(reinterpret_cast<const uint4*>(trow + SPAN * j));
          W[j] = *reinterpret_cast<const uint2*>(wrow + SPAN * j);
        } else {
          T[j] = make_uint4(0, 0, 0, 0);
          W[j] = make_uint2(0, 0);
        }
      }
      const uint32_t c = cw & 0xFFu;
      const uint32_t var = flags >> 4;
      const VariantParameters& p = st.lut[var];
      const uint32_t prop = p.signal_propagation_length;
      const bool exact = prop == b.pmax;
      const bool gfast = exact && prop <= 16u;
      if (cw & kRowBad) err |= AXC_ERR_TARGET_RANGE;
      int32_t i_in = 0;
      uint32_t hitb = 0, slowb = 0;
      const bool glit = use_lit && gfast;
#pragma unroll
      for (int j = 0; j < CH; j++) {
        const uint32_t q0 = (uint32_t)(SPAN * j) + 4u * gl;
        uint2 m[4];
        bool lit[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const uint32_t t = word_of(T[j], i);
          const uint32_t ax = (t & AXC_TARGET_AXON_MASK) - 1u;
          lit[i] = glit && ((t >> AXC_TARGET_SEG_SHIFT) - 1u) < seg_hi && ((s_lit[ax >> 5] >> (ax & 31u)) & 1u);
          m[i] = (q0 + i < c && !lit[i]) ? __ldg(b.mask2 + ax) : make_uint2(0, 0);
        }
        uint32_t need = 0;   // live slots off the fully-lit path
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (q0 + i >= c) continue;
          if (lit[i]) {   // segment 1..30 of a fully lit axon: hit, fast GSOP
            i_in = wadd(i_in, (int32_t)half_of(W[j], i));
            hitb |= 1u << (4 * j + i);
          } else {
            need |= 1u << i;
          }
        }
        if (!__any_sync(kFull, need)) continue;
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (!((need >> i) & 1u)) continue;
          const uint32_t t = word_of(T[j], i);
          const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
          const uint32_t sh = min(s, 31u);
          const uint32_t bx = (m[i].x >> sh) & 1u, by = (m[i].y >> sh) & 1u;
          bool hit = (bx | by) != 0u;
          if (hit && (s >= 31u || !exact)) hit = hit_exact(b.P.axon_heads, A, (t & AXC_TARGET_AXON_MASK) - 1u, s, prop);
          if (hit) {
            i_in = wadd(i_in, (int32_t)half_of(W[j], i));
            hitb |= 1u << (4 * j + i);
          }
          const bool fast = gfast && s < 31u && !(m[i].y >> 31) && (bx || by == (s == 0u));
          slowb |= fast ? 0u : (1u << (4 * j + i));
        }
      }
#pragma unroll
      for (int o = 1; o < LANES; o <<= 1) i_in = wadd(i_in, __shfl_xor_sync(kFull, i_in, o));
      if (gl == 0 && valid) { ev_slots += c; nev++; }
      hits += __popc(hitb);
      int spike = 0;
      if (valid) {
        const int32_t decayed = wsub(thr0, (int32_t)p.homeostasis_decay);
        int32_t thr = decayed & ~(decayed >> 31);
        int32_t leak = p.leak_rate;
        if (p.adaptive_mode == 1) {
          leak = wadd(leak, wmul(thr, (int32_t)p.adaptive_leak_gain) >> 8);
          const int32_t over = wsub(leak, p.adaptive_leak_max);
          leak = wsub(leak, over & ~(over >> 31));
        }
        int32_t v = wadd(v0, i_in);
        const int32_t diff = wsub(v, p.rest_potential);
        const int32_t sign = (diff > 0) - (diff < 0);
        int32_t leaked = wsub(wmul(diff, sign), leak);
        leaked = leaked & ~(leaked >> 31);
        v = wadd(p.rest_potential, wmul(sign, leaked));
        const int glif = v >= wadd(p.threshold, thr) ? 1 : 0;
        const uint32_t period = p.spontaneous_firing_period_ticks;
        const int hb = (period > 0 && ((tick + n * 104729u) % period) == 0) ? 1 : 0;
        spike = glif | hb;
        if (glif) {
          v = p.rest_potential;
          thr = wadd(thr, p.homeostasis_penalty);
        }
        if (gl == 0) {
          b.P.soma_voltage[n] = v;
          b.P.soma_flags[n] = (uint8_t)((flags & 0xF0) | (spike ? 0x05 : 0x00));
          b.P.threshold_offset[n] = thr;
          b.P.timers[n] = glif ? p.refractory_period : 0;
          if (spike) {
            nspk++;
            const uint32_t my_axon = b.P.soma_to_axon[n];
            if (my_axon != AXC_NO_AXON) {
              if (my_axon < A) atomicAdd(&b.pend[my_axon], 1u);
              else err |= AXC_ERR_SOMA_AXON;
            }
          }
        }
      }
      // GSOP of the movable slots, the first lf of the row; the frozen ones
      // (GSOP leaves them as they are) are counted
      if (spike && gl == 0) gdone += c - lf;
      if (spike) {
#pragma unroll
        for (int j = 0; j < CH; j++) {
          const uint32_t q0 = (uint32_t)(SPAN * j) + 4u * gl;
          if (q0 >= lf) continue;
          uint2 wj = W[j];
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const uint32_t bit = 1u << (4 * j + i);
            if (q0 + i >= lf) continue;
            const int16_t w16 = half_of(wj, i);
            if (!(slowb & bit)) {
              const int32_t aw = w16 < 0 ? -(int32_t)w16 : (int32_t)w16;
              const int2 e = st.gtab[var][min((uint32_t)aw >> 11, 15u)];
              int32_t na = aw + ((hitb & bit) ? e.x : -e.y);
              na = min(max(na, 0), 32767);
              set_half(wj, i, (int16_t)(w16 < 0 ? -na : na));
              gdone++;
              continue;
            }
            const uint32_t t = __ldg(trow + SPAN * j + i);
            int16_t nw = w16;
            const int r = gsop_general(b.P.axon_heads, b.mask2, A, (t & AXC_TARGET_AXON_MASK) - 1u,
                                       t >> AXC_TARGET_SEG_SHIFT, p, flags, b.dopamine, &nw);
            if (r == 2) continue;
            gdone++;
            if (r == 1) {
              const uint32_t slot = atomicAdd(&pctl->fix_count, 1u);
              if (slot < fix_cap) fix[slot] = make_uint2(cd.x, (uint32_t)((size_t)n * kRowStride + q0 + i));
              else pctl->fix_overflow = 1u;
              continue;
            }
            set_half(wj, i, nw);
          }
          if (wj.x != W[j].x || wj.y != W[j].y) *reinterpret_cast<uint2*>(wrow + SPAN * j) = wj;
        }
      }
    }
  }
  const uint32_t err_any = __reduce_or_sync(kFull, err);
  if (err_any && lane == 0) atomicOr(&pctl->err, err_any);
  block_count(ev_slots, hits, nspk, &pctl->ctr[1]);
  block_count(gdone, nev, 0, &pctl->ctr[4]);
}

// per tick 4/5: deferred GSOP slots of all brains.
__global__ void __launch_bounds__(256) k_pop_fixup(const PopBrain* __restrict__ brains, uint32_t count,
                                                   const uint2* __restrict__ chunks, PopCtl* __restrict__ pctl,
                                                   const uint2* __restrict__ fix, uint32_t k, uint32_t chunk) {
  const uint32_t nfix = pctl->fix_count;
  const uint32_t overflow = pctl->fix_overflow;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  // the next tick's lists (the slot was last used two ticks ago)
  for (uint32_t b = tid; b < count; b += stride) brains[b].ctl->eval_count[(k + 1) & 1] = 0;
  if (nfix == 0 && !overflow) return;
  if (!overflow) {
    for (uint32_t i = tid; i < nfix; i += stride) {
      const PopBrain& b = brains[fix[i].x];
      fixup_slot(b.P, b.lut, b.A, b.rt, b.rw, b.pend, fix[i].y, b.dopamine);
    }
    return;
  }
  const uint32_t nch = pctl->nchunks[k & 1];
  for (uint32_t w = tid; w < nch * chunk * kRowStride; w += stride) {
    const uint32_t ci = w / (chunk * kRowStride), rem = w % (chunk * kRowStride);
    const uint2 cd = chunks[ci];
    const PopBrain& b = brains[cd.x];
    const uint32_t li = rem / kRowStride, q = rem % kRowStride;
    if (cd.y + li >= b.ctl->eval_count[k & 1]) continue;
    const uint32_t n = b.eval[cd.y + li];
    if (!(b.P.soma_flags[n] & 1) || q >= (b.cnt[n] & 0xFFu)) continue;
    const uint32_t r = n * kRowStride + q;
    const uint32_t t = b.rt[r];
    const uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
    if (a >= b.A) continue;
    const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
    const VariantParameters& p = b.lut[b.P.soma_flags[n] >> 4];
    const uint32_t prop = p.signal_propagation_length;
    const bool gfast = prop == b.pmax && prop <= 16u;
    const uint2 m = b.mask2[a];
    const uint32_t sh = min(s, 31u);
    const uint32_t bx = (m.x >> sh) & 1u, by = (m.y >> sh) & 1u;
    if (gfast && s < 31u && !(m.y >> 31) && (bx || by == (s == 0u))) continue;
    uint32_t md0, md1;
    md_pair(b.P.axon_heads, a, s, prop, &md0, &md1);
    if ((m.y >> 31) || md0 != md1) fixup_slot(b.P, b.lut, b.A, b.rt, b.rw, b.pend, r, b.dopamine);
  }
}

// per tick 5/5, on a graph's last tick only: the spikers' own-axon pushes,
// per chunk (on the other ticks the next prologue applies them).
__global__ void __launch_bounds__(256) k_pop_push(const PopBrain* __restrict__ brains, uint32_t count,
                                                  const uint2* __restrict__ chunks, PopCtl* __restrict__ pctl,
                                                  uint32_t k, uint32_t chunk) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t nch = pctl->nchunks[k & 1];
  for (uint32_t w = tid; w < nch * chunk; w += stride) {
    const uint2 cd = chunks[w / chunk];
    const PopBrain& b = brains[cd.x];
    const uint32_t li = cd.y + w % chunk;
    if (li >= b.ctl->eval_count[k & 1]) continue;
    const uint32_t n = b.eval[li];
    if (!(b.P.soma_flags[n] & 1)) continue;
    const uint32_t ax = b.P.soma_to_axon[n];
    if (ax >= b.A) continue;
    const uint32_t c = atomicExch(&b.pend[ax], 0u);
    if (!c) continue;
    uint4* p = reinterpret_cast<uint4*>(b.P.axon_heads + ax);
    uint4 x = p[0], y = p[1];
    uint32_t h[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
    push_n(h, c);
    p[0] = make_uint4(h[0], h[1], h[2], h[3]);
    p[1] = make_uint4(h[4], h[5], h[6], h[7]);
  }
}

__global__ void k_pop_set_tick0(PopCtl* pctl, uint32_t tick0) { pctl->tick0 = tick0; }

}  // namespace
}  // namespace axc

// ===========================================================================
// host side
// ===========================================================================
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

namespace axc {

static std::atomic<uint32_t> s_pop_fix_cap{kFixCap};
static inline uint32_t g_pop_fix_cap() { return s_pop_fix_cap.load(); }

namespace {

__global__ void k_pop_next_graph(PopBrain* __restrict__ brains, uint32_t count, PopCtl* __restrict__ pctl,
                                 uint32_t tick0) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) pctl->tick0 = tick0;
  if (i < count) {            // tick 0 of the graph appends into slot 0
    brains[i].ctl->eval_count[0] = 0;
    brains[i].ctl->eval_count[1] = 0;
  }
}

}  // namespace

struct Population {
  uint32_t count = 0;
  std::vector<PopBrain> hb;
  PopBrain* d_brains = nullptr;
  uint32_t *d_map_pro = nullptr, *d_first_pro = nullptr, nblk_pro = 0;
  uint32_t *d_map_tile = nullptr, *d_first_tile = nullptr, nblk_tile = 0;
  uint32_t *d_map_n = nullptr, *d_first_n = nullptr, nblk_n = 0;
  int2* d_gtab = nullptr;
  uint2* d_chunks = nullptr;
  uint2* d_fix = nullptr;
  PopCtl* d_ctl = nullptr;
  AxcPopSchedule sched{8, 4, 2};
  uint32_t chunk = kPopChunk;
  uint32_t lit_cap = 0;   // words of the largest fully-lit bitmap the update stages (<= kPopLitWords)
  std::vector<uint32_t> bm_ticks;   // per brain: bitmask rows (UINT32_MAX without a bitmask)
  std::vector<ShardScratch*> scr;   // per brain: the shard's scratch (its rows are this engine's while it runs)
  std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t>, cudaGraphExec_t> graphs;
  cudaStream_t capture = nullptr;
};

// Every brain's bitmask holds rows tick0 .. tick0 + ticks - 1.
static bool pop_ticks_ok(const Population& P, uint32_t tick0, uint64_t ticks) {
  for (uint32_t b : P.bm_ticks)
    if ((uint64_t)tick0 + ticks > b) return false;
  return true;
}

static cudaError_t pop_upload_map(const std::vector<uint32_t>& v, uint32_t** out) {
  cudaError_t e = cudaMalloc(out, std::max<size_t>(v.size(), 1) * 4);
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*out, v.data(), v.size() * 4, cudaMemcpyHostToDevice);
  return e;
}

// One tick of a graph of `ticks` ticks: the soma pushes of tick k go in with
// tick k+1's prologue, and the last tick pushes its own.
static cudaError_t pop_tick(Population& P, uint32_t k, uint32_t ticks, const AxcPopSchedule& sc, cudaStream_t st) {
  const int sms = sm_count();
  if (P.nblk_pro)
    k_pop_prologue<<<P.nblk_pro, 256, 0, st>>>(P.d_brains, P.d_map_pro, P.d_first_pro, P.d_ctl, k, k > 0 ? 1u : 0u);
  k_pop_chunks<<<1, 1024, 0, st>>>(P.d_brains, P.count, P.d_chunks, P.d_ctl, k, P.chunk);
  const uint32_t ub = std::max<uint32_t>(1, sc.update_blocks_per_sm) * sms;
  const uint32_t ab = std::max<uint32_t>(1, sc.aux_blocks_per_sm) * sms;
  const uint32_t cap = std::min(g_pop_fix_cap(), kFixCap);
  const size_t lit_bytes = (size_t)P.lit_cap * 4;
  if (sc.lanes_per_neuron == 16)
    k_pop_update<16><<<ub, 256, lit_bytes, st>>>(P.d_brains, P.d_chunks, P.d_ctl, P.d_fix, k, P.chunk, cap,
                                                 P.lit_cap);
  else
    k_pop_update<8><<<ub, 256, lit_bytes, st>>>(P.d_brains, P.d_chunks, P.d_ctl, P.d_fix, k, P.chunk, cap,
                                                P.lit_cap);
  k_pop_fixup<<<ab, 256, 0, st>>>(P.d_brains, P.count, P.d_chunks, P.d_ctl, P.d_fix, k, P.chunk);
  if (k + 1 == ticks) k_pop_push<<<ab, 256, 0, st>>>(P.d_brains, P.count, P.d_chunks, P.d_ctl, k, P.chunk);
  return cudaGetLastError();
}

static cudaError_t pop_begin(Population& P, cudaStream_t st) {
  k_pop_begin<<<P.count, 256, 0, st>>>(P.d_brains);
  if (P.nblk_n) k_pop_mult<<<P.nblk_n, 256, 0, st>>>(P.d_brains, P.d_map_n, P.d_first_n);
  if (P.nblk_tile) k_pop_build<<<P.nblk_tile, 256, 0, st>>>(P.d_brains, P.d_map_tile, P.d_first_tile);
  return cudaGetLastError();
}

static cudaError_t pop_end(Population& P, cudaStream_t st) {
  if (P.nblk_tile) k_pop_writeback<<<P.nblk_tile, 256, 0, st>>>(P.d_brains, P.d_map_tile, P.d_first_tile);
  return cudaGetLastError();
}

static void pop_free(Population* P) {
  if (!P) return;
  for (auto& kv : P->graphs) cudaGraphExecDestroy(kv.second);
  if (P->capture) cudaStreamDestroy(P->capture);
  void* ptrs[] = {P->d_brains, P->d_map_pro, P->d_first_pro, P->d_map_tile, P->d_first_tile, P->d_map_n,
                  P->d_first_n, P->d_gtab, P->d_chunks, P->d_fix, P->d_ctl};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete P;
}

}  // namespace axc

using namespace axc;

extern "C" {

int32_t axc_population_create(const AxcPopBrainDesc* brains, uint32_t count, void** out_handle) {
  if (!brains || !count || !out_handle) return (int32_t)cudaErrorInvalidValue;
  Population* P = new Population();
  P->count = count;
  P->hb.resize(count);
  P->bm_ticks.resize(count);
  cudaError_t e = cudaMalloc(&P->d_gtab, (size_t)count * 256 * sizeof(int2));
  std::vector<uint32_t> map_pro, first_pro(count), map_tile, first_tile(count), map_n, first_n(count);
  size_t max_chunks = count;
  for (uint32_t b = 0; b < count && e == cudaSuccess; b++) {
    const AxcPopBrainDesc& d = brains[b];
    ShardScratch* s = scratch_for(&d.vram, d.padded_n, d.total_axons, &e);
    if (!s) break;
    e = rows_alloc(*s, d.padded_n, d.total_axons, false, nullptr);
    if (e != cudaSuccess) break;
    rows_touched(*s);
    P->scr.push_back(s);
    PopBrain& h = P->hb[b];
    std::memset(&h, 0, sizeof(h));
    h.P = d.vram;
    h.bitmask = d.d_input_bitmask;
    h.lut = d.d_lut;
    h.gtab = P->d_gtab + (size_t)b * 256;
    h.rt = s->rows->rt;
    h.rw = s->rows->rw;
    h.cnt = s->rows->cnt;
    h.mask2 = s->rows->mask2;
    h.mult = s->rows->mult;
    h.eval = s->rows->eval;
    h.pend = s->pend;
    h.ctl = s->ctl;
    h.lit = s->rows->lit;
    h.lfz = s->rows->lfz;
    h.amask = s->rows->amask;
    h.omask = s->rows->omask;
    P->lit_cap = std::max(P->lit_cap, std::min((d.total_axons >> 5) + 1, kPopLitWords));
    h.N = d.padded_n;
    h.A = d.total_axons;
    h.voff = d.virtual_offset;
    h.nv = d.d_input_bitmask ? d.num_virtual : 0;
    h.words = d.words_per_tick;
    h.v_seg = d.v_seg;
    h.tick_base = d.tick_base;
    h.dopamine = d.dopamine;
    P->bm_ticks[b] = d.d_input_bitmask ? d.bitmask_ticks : 0xFFFFFFFFu;
    first_pro[b] = (uint32_t)map_pro.size();
    for (uint32_t i = 0; i < (std::max(d.padded_n, d.total_axons) + 255) / 256; i++) map_pro.push_back(b);
    first_tile[b] = (uint32_t)map_tile.size();
    for (uint32_t i = 0; i < (d.padded_n + 31) / 32; i++) map_tile.push_back(b);
    first_n[b] = (uint32_t)map_n.size();
    for (uint32_t i = 0; i < (d.padded_n + 255) / 256; i++) map_n.push_back(b);
    max_chunks += (d.padded_n + 127) / 128;
  }
  if (e == cudaSuccess) e = cudaMalloc(&P->d_brains, (size_t)count * sizeof(PopBrain));
  if (e == cudaSuccess) e = cudaMemcpy(P->d_brains, P->hb.data(), (size_t)count * sizeof(PopBrain), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = pop_upload_map(map_pro, &P->d_map_pro);
  if (e == cudaSuccess) e = pop_upload_map(first_pro, &P->d_first_pro);
  if (e == cudaSuccess) e = pop_upload_map(map_tile, &P->d_map_tile);
  if (e == cudaSuccess) e = pop_upload_map(first_tile, &P->d_first_tile);
  if (e == cudaSuccess) e = pop_upload_map(map_n, &P->d_map_n);
  if (e == cudaSuccess) e = pop_upload_map(first_n, &P->d_first_n);
  P->nblk_pro = (uint32_t)map_pro.size();
  P->nblk_tile = (uint32_t)map_tile.size();
  P->nblk_n = (uint32_t)map_n.size();
  if (e == cudaSuccess) e = cudaMalloc(&P->d_chunks, max_chunks * sizeof(uint2));
  if (e == cudaSuccess) e = cudaMalloc(&P->d_fix, (size_t)kFixCap * sizeof(uint2));
  if (e == cudaSuccess) e = cudaMalloc(&P->d_ctl, sizeof(PopCtl));
  if (e == cudaSuccess) e = cudaMemset(P->d_ctl, 0, sizeof(PopCtl));
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);   // zeroed before a run on any stream
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->capture, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    pop_free(P);
    return (int32_t)e;
  }
  *out_handle = P;
  return 0;
}

int32_t axc_population_set_schedule(void* handle, const AxcPopSchedule* sc) {
  if (!handle || !sc || (sc->lanes_per_neuron != 8 && sc->lanes_per_neuron != 16)) return (int32_t)cudaErrorInvalidValue;
  static_cast<Population*>(handle)->sched = *sc;
  return 0;
}

int32_t axc_population_run(void* handle, uint32_t tick0, uint32_t ticks, uint32_t tpg, void* stream_v) {
  Population* P = static_cast<Population*>(handle);
  if (!P || tpg == 0 || ticks % tpg || !pop_ticks_ok(*P, tick0, ticks)) return (int32_t)cudaErrorInvalidValue;
  cudaStream_t st = static_cast<cudaStream_t>(stream_v);
  for (ShardScratch* s : P->scr) rows_touched(*s);   // the per-tick entry point's row copies are replaced
  auto key = std::make_tuple(tpg, P->sched.lanes_per_neuron, P->sched.update_blocks_per_sm,
                             P->sched.aux_blocks_per_sm * 1000 + std::min(g_pop_fix_cap(), kFixCap) % 1000);
  cudaGraphExec_t exec = nullptr;
  auto it = P->graphs.find(key);
  cudaError_t e = cudaSuccess;
  if (it != P->graphs.end()) {
    exec = it->second;
  } else {
    e = cudaStreamBeginCapture(P->capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return (int32_t)e;
    cudaError_t le = cudaSuccess;
    for (uint32_t k = 0; k < tpg && le == cudaSuccess; k++) le = pop_tick(*P, k, tpg, P->sched, P->capture);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(P->capture, &g);
    if (le != cudaSuccess) e = le;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return (int32_t)e;
    P->graphs[key] = exec;
  }
  e = pop_begin(*P, st);
  for (uint32_t c = 0; c < ticks / tpg && e == cudaSuccess; c++) {
    k_pop_next_graph<<<(P->count + 255) / 256, 256, 0, st>>>(P->d_brains, P->count, P->d_ctl, tick0 + c * tpg);
    e = cudaGraphLaunch(exec, st);
  }
  if (e == cudaSuccess) e = pop_end(*P, st);
  return (int32_t)e;
}

int32_t axc_population_tune(void* handle, uint32_t tick0, uint32_t trial_ticks, void* stream_v,
                            AxcPopSchedule* chosen, float* out_ms, uint32_t max_out) {
  Population* P = static_cast<Population*>(handle);
  if (!P || !chosen || trial_ticks == 0) return (int32_t)cudaErrorInvalidValue;
  cudaStream_t st = static_cast<cudaStream_t>(stream_v);
  std::vector<AxcPopSchedule> cands;
  for (uint32_t lanes : {8u, 16u})
    for (uint32_t ub : {2u, 3u, 4u})
      for (uint32_t ab : {1u, 2u}) cands.push_back(AxcPopSchedule{lanes, ub, ab});
  if (!pop_ticks_ok(*P, tick0, (uint64_t)trial_ticks * cands.size())) return (int32_t)cudaErrorInvalidValue;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t e = pop_begin(*P, st);
  float best = 1e30f;
  uint32_t tick = tick0;
  for (size_t i = 0; i < cands.size() && e == cudaSuccess; i++) {
    k_pop_next_graph<<<(P->count + 255) / 256, 256, 0, st>>>(P->d_brains, P->count, P->d_ctl, tick);
    cudaEventRecord(e0, st);
    for (uint32_t k = 0; k < trial_ticks && e == cudaSuccess; k++) e = pop_tick(*P, k, trial_ticks, cands[i], st);
    cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (out_ms && i < max_out) out_ms[i] = ms;
    if (ms < best) { best = ms; *chosen = cands[i]; }
    tick += trial_ticks;
  }
  if (e == cudaSuccess) e = pop_end(*P, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e == cudaSuccess) P->sched = *chosen;
  return (int32_t)e;
}

int32_t axc_population_counters(void* handle, uint64_t out[8]) {
  Population* P = static_cast<Population*>(handle);
  if (!P || !out) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e = cudaDeviceSynchronize();
  PopCtl c;
  if (e == cudaSuccess) e = cudaMemcpy(&c, P->d_ctl, sizeof(c), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return (int32_t)e;
  for (int i = 0; i < 6; i++) out[i] = c.ctr[i];
  uint32_t err = c.err;
  for (uint32_t b = 0; b < P->count; b++) {
    uint32_t be = 0;
    if (cudaMemcpy(&be, &P->hb[b].ctl->err, 4, cudaMemcpyDeviceToHost) == cudaSuccess) err |= be;
  }
  out[6] = err;
  out[7] = 0;
  return 0;
}

void axc_population_destroy(void* handle) { pop_free(static_cast<Population*>(handle)); }

uint32_t axc_population_fix_capacity(uint32_t cap) { return s_pop_fix_cap.exchange(std::min(cap, kFixCap)); }

}  // extern "C"
