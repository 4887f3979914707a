// row_engine.cuh — the batch engine's neuron-major tick (compiled as part of
// day_phase.cu: it uses that translation unit's __constant__ LUT and helpers).
//
// Why: in the reference layout dendrite slot i of all neurons is one row
// ([slot][neuron], memory.rs:71-86), so a 32-byte sector holds 8 neurons'
// targets.  In steady state only the non-refractory quarter of the neurons is
// evaluated each tick, yet nearly every sector is fetched, and GSOP re-reads
// the spikers' slots with one sector per slot.  For the length of one batch the
// engine keeps a neuron-major copy ([neuron][128]) of targets and weights:
//
//   batch start  k_rows_mult       somas per axon (soma_to_axon multiplicity)
//                k_rows_build      columnar -> rows (the slots whose weights may
//                                  still move first), per-neuron counts and masks
//   per tick     k_rows_prologue   the previous tick's soma pushes, axon pushes +
//                                  propagation + split masks, fully-lit bitmap,
//                                  refractory countdown, list of evaluated neurons
//                k_rows_update     8 lanes per evaluated neuron: gather/sum, GLIF;
//                                  lists the spikers with movable slots
//                k_rows_gsop       GSOP of spikers with 1..8 movable slots
//                k_rows_gsop_rows  GSOP of spikers with more, 8 lanes per row
//                k_rows_fixup      readout, the GSOP slots whose result depends on
//                                  same-tick pushes
//                k_rows_push       the spikers' pushes (a batch's last tick only;
//                                  otherwise the next prologue applies them)
//   batch end    k_rows_writeback  weights rows -> columnar
//
// GSOP against same-tick pushes.  GSOP must see the heads after this tick's
// soma pushes (physics.cu:281-373 runs after the update kernel).  A push
// inserts a 0 head and drops h7, so for an axon owned by one soma the result
// can only change when segment 0 is involved or h7 is the only head in the
// tail.  The axon stage writes two masks per axon — hits of heads 0..6 and
// hits of head 7 — so GSOP knows, per slot, the "no push" and "one push"
// outcomes.  When they agree the weight is updated at once; otherwise the slot
// is left untouched and listed, and k_rows_fixup applies it with the actual
// push count (and from the original weight).  Axons owned by two or more
// somas, variants whose length differs from the LUT maximum or exceeds 16
// (where the cooling shift can be non-zero) and segments >= 31 take the exact
// general path.

namespace axc {
namespace {

constexpr uint32_t kRowStride = AXC_MAX_DENDRITES;   // slots per neuron row
constexpr uint32_t kInf = 0xFFFFFFFFu;

// Programmatic dependent launch inside a tick's kernel chain (prologue ->
// 8-lane pass -> lit-sum pass -> fix-up -> push).  A kernel
// launched with launch_chain(pdl = true) may be scheduled while the kernel
// before it on the stream still runs; its first statement is chain_wait(),
// which returns once that kernel has completed and its writes are visible, so
// only the launch and the block scheduling overlap.  Every block passes
// chain_wait() before it can exit, so a kernel's completion implies its
// predecessor's, and the chain stays ordered end to end.  chain_open() then
// lets the next kernel of the chain be scheduled (after this grid's last block
// started and passed its own wait); it only matters when that kernel is
// launched with the attribute.  In a kernel launched without it (the prologue,
// every kernel of a captured batch) chain_wait() returns at once: the stream
// finished the predecessor before the kernel started.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void chain_open() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... P, typename... Args>
static void launch_chain(void (*kern)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, bool pdl,
                         Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  // a failed launch also leaves its error for cudaGetLastError, which the
  // launch sequences return
  cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}
constexpr uint32_t kRowBad = 0x8000u;    // cnt flag: the row holds an invalid target

// Bytes of the fully-lit bitmap of A axons as staged in shared memory (one
// bit per axon and a spare word, rounded up to the bulk copy's 16 bytes; the
// global bitmap is allocated at least this large).
__host__ __device__ __forceinline__ uint32_t lit_smem_bytes(uint32_t A) { return (((A >> 5) + 1) * 4 + 15) & ~15u; }

// physics.cu:322-371 for one slot given the minimum in-tail distance md.
__device__ __forceinline__ int16_t gsop_weight(int16_t w16, uint32_t md, const VariantParameters& p, int32_t bm,
                                               int32_t raw_pot, int32_t final_dep) {
  const bool active = md != kInf;
  const int32_t sign = w16 >= 0 ? 1 : -1;
  int32_t abs_w = (int32_t)w16;
  if (abs_w < 0) abs_w = -abs_w;
  uint32_t rank = (uint32_t)abs_w >> 11;
  if (rank > 15) rank = 15;
  const int32_t inertia = p.inertia_curve[rank];
  const int32_t delta_pot = wmul(wmul(raw_pot, inertia), bm) >> 7;
  const int32_t delta_dep = wmul(wmul(final_dep, inertia), bm) >> 7;
  const uint32_t cs = active ? (md >> 4) : 0u;
  int32_t delta = active ? (delta_pot >> cs) : wsub(0, delta_dep);
  delta = wmul(delta, 128) >> (7u + cs);
  int32_t new_abs = wadd(abs_w, delta);
  new_abs = new_abs & ~(new_abs >> 31);
  if (new_abs > 32767) new_abs = 32767;
  return (int16_t)wmul(new_abs, sign);
}

__device__ __forceinline__ uint32_t md_of(const uint32_t h[8], uint32_t s, uint32_t len) {
  uint32_t md = kInf;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const uint32_t d = h[q] - s;
    md = min(md, d < len ? d : kInf);
  }
  return md;
}

// Minimum distances with no push and with one push (0, h0..h6).
__device__ __forceinline__ void md_pair(const BurstHeads8* heads, uint32_t a, uint32_t s, uint32_t len,
                                        uint32_t* md0, uint32_t* md1) {
  uint32_t h[8];
  load_heads(heads, a, h);
  uint32_t m06 = kInf;
#pragma unroll
  for (int q = 0; q < 7; q++) {
    const uint32_t d = h[q] - s;
    m06 = min(m06, d < len ? d : kInf);
  }
  const uint32_t d7 = h[7] - s;
  *md0 = min(m06, d7 < len ? d7 : kInf);
  const uint32_t dz = 0u - s;
  *md1 = min(m06, dz < len ? dz : kInf);
}

// Write-through of GSOP's weight changes to the reference's columnar blob
// (dendrite_weights[slot][N]), used by the per-tick entry point, whose row
// cache outlives the call: after every tick the blob must hold the weights the
// reference would hold.  w == nullptr: no write-through (the batch paths write
// every weight back at batch end).
struct ColWT {
  int16_t* w = nullptr;         // columnar weights of the shard
  const uint4* om = nullptr;    // per neuron: the columnar slots placed first in its row
  const uint16_t* cnt = nullptr;
  uint32_t N = 0;
};

// The r-th set bit (0-based) of a 128-bit mask.
__device__ __forceinline__ uint32_t nth_bit128(uint4 m, uint32_t r) {
  const uint32_t c0 = __popc(m.x);
  if (r < c0) return __fns(m.x, 0, r + 1);
  r -= c0;
  const uint32_t c1 = __popc(m.y);
  if (r < c1) return 32u + __fns(m.y, 0, r + 1);
  r -= c1;
  const uint32_t c2 = __popc(m.z);
  if (r < c2) return 64u + __fns(m.z, 0, r + 1);
  return 96u + __fns(m.w, 0, r - c2 + 1);
}

// Columnar slot of row position pos in a row of c used slots whose slots of om
// come first (in slot order) and the other used slots after them (in slot order).
__device__ __forceinline__ uint32_t col_of_pos(uint4 om, uint32_t pos, uint32_t c) {
  const uint32_t olf = __popc(om.x) + __popc(om.y) + __popc(om.z) + __popc(om.w);
  if (pos < olf) return nth_bit128(om, pos);
  const auto used = [c](uint32_t lo) { return c >= lo + 32u ? 0xFFFFFFFFu : (c > lo ? (1u << (c - lo)) - 1u : 0u); };
  const uint4 rest = make_uint4(used(0) & ~om.x, used(32) & ~om.y, used(64) & ~om.z, used(96) & ~om.w);
  return nth_bit128(rest, pos - olf);
}

__device__ __forceinline__ void col_write(const ColWT& wt, uint32_t n, uint32_t pos, int16_t w) {
  const uint32_t q = col_of_pos(wt.om[n], pos, wt.cnt[n] & 0xFFu);
  wt.w[(size_t)q * wt.N + n] = w;
}

// The lit-sum form runs tick k when the rows' tested prefixes are short (at most
// an eighth of the live slots: otherwise the 8-lane pass is faster) and every
// axon the row layout took as fully lit is fully lit this tick.  Every thread
// of both update kernels asks at its start; the three words were written by
// earlier kernels and no kernel that asks writes them, so plain loads (cached
// in L1 after the first warp of an SM) serve it: uncached loads sent every
// warp's request to the one L2 slice that holds the control block, a few
// microseconds per launch.
__device__ __forceinline__ bool lsum_tick(const ShardCtl* ctl, uint32_t k) {
  const unsigned long long p = ctl->pfx_total, c = ctl->slot_total;
  return c > 0 && p * 8ull <= c && ctl->dense[k & 1] == 0u;
}

// Per-neuron GSOP constants (physics.cu:290-345).
struct GsopConsts {
  int32_t bm, raw_pot, final_dep;
};

__device__ __forceinline__ GsopConsts gsop_consts(uint8_t flags, const VariantParameters& p, int32_t dopamine) {
  GsopConsts g;
  const uint32_t burst = (flags >> 1) & 0x07;
  g.bm = burst > 0 ? (int32_t)burst : 1;
  const int32_t pot_mod = wmul(dopamine, (int32_t)p.d1_affinity) >> 7;
  const int32_t dep_mod = wmul(dopamine, (int32_t)p.d2_affinity) >> 7;
  g.raw_pot = wadd((int32_t)p.gsop_potentiation, pot_mod);
  const int32_t raw_dep = wsub((int32_t)p.gsop_depression, dep_mod);
  g.final_dep = raw_dep & ~(raw_dep >> 31);
  return g;
}

// Split segment-hit masks of one axon's (propagated) heads for length P:
// x: bits 0..30 = segments hit by heads 0..6, bit 31 = some head (0..7) may hit
//    a segment >= 31;  y: bits 0..30 = segments hit by head 7, bit 31 = the axon
//    is owned by two or more somas.  An axon owned by no soma cannot be pushed
//    between update and GSOP, so its head-7 hits are folded into x.
__device__ __forceinline__ uint2 split_masks(const uint32_t h[8], uint32_t P, uint32_t mult) {
  uint32_t x = 0, y = 0;
  if (P != 0) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const uint32_t v = h[k];
      if (v < 255u + P) {
        const uint32_t lo = (v + 1u > P) ? v + 1u - P : 0u;
        uint32_t bits = 0;
        if (lo <= 30u) {
          const uint32_t top = min(v, 30u);
          bits = ((2u << top) - 1u) & ~((1u << lo) - 1u);
        }
        if (k < 7) x |= bits; else y |= bits;
        if (v >= 31u) x |= 0x80000000u;
      }
    }
  }
  if (mult == 0) { x |= y; y = 0; }
  if (mult >= 2) y |= 0x80000000u;
  return make_uint2(x, y);
}

// True when the update pass may apply GSOP to this slot on the spot.
// fast: hit/no-hit decides (variant length == LUT max <= 16, segment < 31,
// axon not multiply owned) and the one-push outcome equals the no-push one.
__device__ __forceinline__ bool fast_class(uint32_t s, uint2 m, bool gsop_fast) {
  return gsop_fast && s < 31u && !(m.y >> 31);
}

__device__ __forceinline__ bool fast_sensitive(uint32_t s, uint2 m) {
  const bool a0 = ((m.x | m.y) >> s) & 1u;
  const bool a1 = (s == 0u) || ((m.x >> s) & 1u);
  return a0 != a1;
}

// Control block and per-tick buffers of the learned-schedule engine
// (learned.cuh): the prologue accumulates per-tile activity into them and, on
// a sparse tick, compacts the active axons into per-tile segments whose sizes
// the predictor chose before the tick.
struct LearnCtl {
  uint32_t mode;          // this tick: 0 dense row pass, 1 sparse axon-driven gather
  uint32_t overflow;      // a tile outgrew its pre-sized segment: the tick runs dense
  uint32_t spk_count;     // sparse tick: spikers listed for GSOP
  uint32_t stale;         // the inverted index no longer matches the targets
  uint32_t ticks_seen;    // ticks completed with features since the history began
  uint32_t samples;       // (features, target) pairs recorded
  uint32_t sample_cap;
  uint32_t sample_every;  // record every k-th tick
  int32_t policy;         // -1 predictor, 0 always dense, 1 always sparse (exact capacities)
  uint32_t collect;       // record pairs while running
  float ratio;            // sparse when ratio * predicted active synapses < evaluated slots
  float margin;           // capacity = prediction * (1 + margin) + slack
  uint32_t slack;
  uint32_t T;             // tiles of 1024 axons (= neurons)
  uint32_t prev_mode;     // the previous tick's schedule
  uint32_t prev_learned;  // the previous tick's schedule came from the predictor
  uint32_t feat_done;     // the features kernel ran after the previous tick
  uint32_t pad0, pad1, pad2, pad3;
  unsigned long long eval_next;   // evaluated slots of the next tick (features kernel)
  unsigned long long eval_now;    // evaluated slots of this tick
  unsigned long long row_sum;     // targets checksum the inverted index was built from
  float pred_total;               // sum of the tile predictions for this tick (synapses)
  float inrate[9];                // input spike fraction of ticks t, t-1, ..., t-8
  unsigned long long stat[12];
};

struct LearnDev {
  LearnCtl* ctl;
  const uint32_t* inv_off;  // [A+1] inverted index offsets (slots whose target is axon a)
  uint32_t* yacc;           // [T] active synapses of the tile's axons this tick
  uint32_t* bacc;           // [T] heads in flight on the tile's axons this tick
  uint32_t* fill;           // [T] axons compacted into the tile's segment
  const uint32_t* cap;      // [T] the tile's capacity in synapses
  uint32_t* alist;          // active axons of a sparse tick, tile j at [1024 j, 1024 j + fill[j])
  uint32_t* evbits;         // [N/32+1] evaluated neurons of the tick
};

// 64-bit mix of one live slot for the targets checksum (order-independent sum).
__device__ __forceinline__ unsigned long long slot_mix(uint32_t t, uint32_t r) {
  unsigned long long x = ((unsigned long long)t << 32) ^ (unsigned long long)r;
  x *= 0x9E3779B97F4A7C15ull;
  x ^= x >> 31;
  x *= 0xBF58476D1CE4E5B9ull;
  return x ^ (x >> 29);
}

// ---------------------------------------------------------------------------
// batch start / end: the row copy
// ---------------------------------------------------------------------------
// Smallest |w| from which every inertia rank of variant v is 0 (0x10000:
// none): GSOP moves such a weight by 0 whatever the hit, distance, burst or
// dopamine (physics.cu:336-371), except -32768, which the clamp turns into
// -32767.
__device__ __forceinline__ int32_t frozen_from(const VariantParameters& p) {
  int r0 = 16;
  while (r0 > 0 && p.inertia_curve[r0 - 1] == 0) r0--;
  return r0 < 16 ? r0 * 2048 : 0x10000;
}

// thr <= |w| <= 32767, in plain signed comparisons (-32768 is not frozen: the
// clamp moves it).
__device__ __forceinline__ bool frozen_weight(int16_t w16, int32_t thr) {
  const int32_t w = w16;
  return w != -32768 && (w >= thr || w <= -thr);
}

// Row position of columnar slot q (lane = q & 31) when the slots of mask o
// come first, in slot order, and the others follow in slot order: word = the
// 32 bits of o holding q, pre = set bits of o before that word, lf = set bits
// of o in all.
__device__ __forceinline__ uint32_t row_pos(uint32_t word, uint32_t lane, uint32_t q, uint32_t pre, uint32_t lf) {
  const uint32_t below = pre + __popc(word & ((1u << lane) - 1u));
  return ((word >> lane) & 1u) ? below : lf + q - below;
}

// One neuron's row of the row copy, by one warp, from the columns staged in
// shared memory (column j, c used slots): invalid targets redirected, movable
// marks, placement, and the neuron's cnt / amask / omask / lfz.
// Placement with permute: the movable slots first, then (with xlit) the other
// slots the update pass must test each tick, then the lit-sum slots, each
// group in slot order; without permute every slot keeps its position.
// A lit-sum slot (xlit given, permute) is frozen (GSOP cannot move its weight),
// has a segment in 1..30, belongs to a neuron whose variant length is the LUT
// maximum, and targets an axon that xlit marks as fully lit: while that axon
// stays fully lit (the prologue checks it every tick) the slot is a hit, so the
// update pass adds the row's lit-sum weights as one precomputed wrapping sum
// (lsum[n].x) and tests only the first lsum[n].y positions.
// Returns, in every lane, the row's largest segment, (want_sum) its targets
// checksum and its tested-prefix length.
struct RowBuilt {
  uint32_t smx;
  unsigned long long hsum;
  uint32_t pfx;
};

__device__ __forceinline__ RowBuilt build_row(uint32_t (*s_t)[33], const int16_t (*s_w)[34], uint32_t j, uint32_t n,
                                              uint32_t c, int32_t fz, uint32_t A, bool want_sum, bool permute,
                                              uint32_t* __restrict__ rt, int16_t* __restrict__ rw,
                                              uint16_t* __restrict__ cnt, uint4* __restrict__ amask,
                                              uint4* __restrict__ omask, uint8_t* __restrict__ lfz,
                                              const uint32_t* __restrict__ xlit = nullptr, bool exact_var = false,
                                              int2* __restrict__ lsum = nullptr, uint8_t* __restrict__ posmap = nullptr) {
  const uint32_t lane = threadIdx.x & 31;
  const bool lsum_on = permute && xlit != nullptr && exact_var;
  bool bad = false;
  uint32_t smx = 0, rsum = 0;
  unsigned long long hsum = 0;
  uint32_t mv[4], rs[4], all[4];   // movable / lit-sum / used slots, by columnar position
#pragma unroll
  for (int ch = 0; ch < 4; ch++) {
    const uint32_t q = 32u * ch + lane;
    bool mov = false, rest = false;
    if (q < c) {
      uint32_t t = s_t[q][j];
      // an invalid axon id (field 0 or >= A) points at the dummy mask entry A,
      // which sends the slot down the exact path (hit_exact / gsop_general skip it)
      if ((t & AXC_TARGET_AXON_MASK) - 1u >= A) {
        t = (t & ~AXC_TARGET_AXON_MASK) | (A + 1u);
        s_t[q][j] = t;
        bad = true;
      }
      const uint32_t seg = t >> AXC_TARGET_SEG_SHIFT;
      smx = max(smx, seg);
      if (want_sum) hsum += slot_mix(t, n * kRowStride + q);
      mov = !frozen_weight(s_w[q][j], fz);
      if (lsum_on && !mov && seg - 1u < 30u) {
        const uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
        rest = a < A && ((__ldg(xlit + (a >> 5)) >> (a & 31u)) & 1u);
      }
      if (rest) rsum += (uint32_t)(int32_t)s_w[q][j];
    }
    mv[ch] = __ballot_sync(kFull, mov);
    rs[ch] = __ballot_sync(kFull, rest);
    all[ch] = __ballot_sync(kFull, q < c);
  }
  bad = __any_sync(kFull, bad);
  smx = __reduce_max_sync(kFull, smx);
  if (want_sum) hsum = warp_sum(hsum);
  rsum = warp_sum(rsum);
  if (bad) {
#pragma unroll
    for (int ch = 0; ch < 4; ch++) { mv[ch] = all[ch]; rs[ch] = 0u; }
    rsum = 0;
  }
  const uint32_t lf = __popc(mv[0]) + __popc(mv[1]) + __popc(mv[2]) + __popc(mv[3]);
  const uint32_t nrs = __popc(rs[0]) + __popc(rs[1]) + __popc(rs[2]) + __popc(rs[3]);
  const uint32_t pfx = c - nrs;   // row positions the update pass tests: movable, then the others
  // placement: movable (o), then tested (x), then lit-sum (rs) with permute; else the identity
  uint32_t o[4], x[4];
#pragma unroll
  for (int ch = 0; ch < 4; ch++) {
    o[ch] = permute ? mv[ch] : all[ch];
    x[ch] = permute ? (all[ch] & ~mv[ch] & ~rs[ch]) : 0u;
  }
  uint32_t po = 0, px = 0, pr = 0, am[4];
  const uint32_t below = (1u << lane) - 1u;
#pragma unroll
  for (int ch = 0; ch < 4; ch++) {
    const uint32_t q = 32u * ch + lane;
    const uint32_t bit = 1u << lane;
    uint32_t pos;
    if (o[ch] & bit) pos = po + __popc(o[ch] & below);
    else if (x[ch] & bit) pos = lf + px + __popc(x[ch] & below);
    else pos = pfx + pr + __popc(rs[ch] & below);
    po += __popc(o[ch]);
    px += __popc(x[ch]);
    pr += __popc(rs[ch]);
    if (q < c) {
      rt[(size_t)n * kRowStride + pos] = s_t[q][j];
      rw[(size_t)n * kRowStride + pos] = s_w[q][j];
      if (posmap) posmap[(size_t)n * kRowStride + q] = (uint8_t)pos;
    }
    // the movable slots by row position: the first lf positions, or mv itself
    const uint32_t lo = 32u * ch;
    am[ch] = permute ? (lf >= lo + 32u ? kFull : (lf > lo ? (1u << (lf - lo)) - 1u : 0u)) : mv[ch];
  }
  if (lane == 0) {
    cnt[n] = (uint16_t)(c | (bad ? kRowBad : 0u));
    amask[n] = make_uint4(am[0], am[1], am[2], am[3]);
    omask[n] = make_uint4(o[0], o[1], o[2], o[3]);
    lfz[n] = (uint8_t)lf;
    if (lsum) lsum[n] = make_int2((int32_t)rsum, (int32_t)pfx);
  }
  return RowBuilt{smx, hsum, pfx};
}

// Batch end, 32 neurons from n0 by a 256-thread block: weights rows -> columnar
// for the slots of omask (the first group of the row, in slot order).  Those
// are the only slots whose weights GSOP can have changed (the others are frozen
// or, without permute, omask holds every used slot).
__device__ __forceinline__ void writeback_tile(int16_t* __restrict__ weights, uint32_t N, uint32_t n0,
                                               const int16_t* __restrict__ rw, const uint16_t* __restrict__ cnt,
                                               const uint4* __restrict__ omask, int16_t (*s_w)[34],
                                               uint32_t* s_c) {
  __shared__ uint4 s_om[32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t j = warp; j < 32; j += 8) {
    const uint32_t n = n0 + j;
    const uint32_t c = n < N ? (cnt[n] & 0xFFu) : 0u;
    const uint4 om = c ? omask[n] : make_uint4(0, 0, 0, 0);
    if (lane == 0) {
      s_c[j] = (om.x | om.y | om.z | om.w) ? c : 0u;
      s_om[j] = om;
    }
    const uint32_t o[4] = {om.x, om.y, om.z, om.w};
    uint32_t pre = 0;
#pragma unroll
    for (int ch = 0; ch < 4; ch++) {
      const uint32_t q = 32u * ch + lane;
      if (q < c && ((o[ch] >> lane) & 1u))
        s_w[q][j] = rw[(size_t)n * kRowStride + pre + __popc(o[ch] & ((1u << lane) - 1u))];
      pre += __popc(o[ch]);
    }
  }
  __syncthreads();
  uint32_t cmax = 0;
  for (int j = 0; j < 32; j++) cmax = max(cmax, s_c[j]);
  const uint32_t c_mine = s_c[lane];
  const uint4 om = s_om[lane];
  const uint32_t o[4] = {om.x, om.y, om.z, om.w};
  for (uint32_t r = warp; r < cmax; r += 8)
    if (r < c_mine && ((o[r >> 5] >> (r & 31u)) & 1u)) weights[(size_t)r * N + n0 + lane] = s_w[r][lane];
}

// Batch start: columnar -> rows.  32 neurons per 256-thread block; the
// columns are read 8 slots at a time until every neuron of the tile has met
// its first empty target.  A slot whose weight GSOP may still move (not
// frozen_weight, or any slot of a row with an invalid target) is movable;
// weights only freeze, so the marks hold for the whole batch.  With permute
// the movable slots go first in the row, then the others (each group in slot
// order), so that GSOP reads a short prefix of the row; the dendrite sum (a
// wrapping i32 sum) and GSOP (per slot) do not depend on the order.
// Per neuron: cnt = used slots (| kRowBad), lfz = movable slots, amask = their
// row positions, omask = the columnar slots placed first (read by the
// write-back; every used slot when the row keeps the columnar order).
__global__ void __launch_bounds__(256) k_rows_build(const uint32_t* __restrict__ targets,
                                                    const int16_t* __restrict__ weights,
                                                    const uint8_t* __restrict__ flags, uint32_t N,
                                                    uint32_t* __restrict__ rt, int16_t* __restrict__ rw,
                                                    uint16_t* __restrict__ cnt, uint4* __restrict__ amask,
                                                    uint4* __restrict__ omask, uint8_t* __restrict__ lfz,
                                                    ShardCtl* __restrict__ ctl, uint32_t A, uint32_t want_sum,
                                                    uint32_t permute, const uint32_t* __restrict__ xlit,
                                                    int2* __restrict__ lsum, uint8_t* __restrict__ posmap,
                                                    uint32_t cond) {
  if (cond && !ctl->lay_now) return;   // the batch keeps the last layout
  __shared__ uint32_t s_t[AXC_MAX_DENDRITES][33];
  __shared__ int16_t s_w[AXC_MAX_DENDRITES][34];
  __shared__ uint32_t s_cnt[32];
  __shared__ uint32_t s_pmax;
  const uint32_t n0 = blockIdx.x * 32;
  const uint32_t col = threadIdx.x & 31, r0 = threadIdx.x >> 5;
  if (threadIdx.x < 32) s_cnt[threadIdx.x] = AXC_MAX_DENDRITES;
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  for (uint32_t ch = 0; ch < AXC_MAX_DENDRITES / 8; ch++) {
    const uint32_t r = ch * 8 + r0, n = n0 + col;
    uint32_t t = 0;
    int16_t w = 0;
    if (n < N) {
      t = __ldcs(targets + (size_t)r * N + n);
      w = __ldcs(weights + (size_t)r * N + n);
    }
    s_t[r][col] = t;
    s_w[r][col] = w;
    if (t == 0) atomicMin(&s_cnt[col], r);
    __syncthreads();
    const int mine = threadIdx.x < 32 ? (s_cnt[threadIdx.x] < (ch + 1) * 8) : 1;
    if (__syncthreads_and(mine)) break;
  }
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // the block's longest row, largest segment, tested and live slots and (when
  // asked) targets checksum, one atomic each per block
  __shared__ uint32_t s_bc[8], s_bs[8], s_bp[8], s_bl[8];
  __shared__ unsigned long long s_bh[8];
  uint32_t wc = 0, ws = 0, wp = 0, wl = 0;
  unsigned long long wh = 0;
  for (uint32_t j = warp; j < 32; j += 8) {
    const uint32_t n = n0 + j;
    if (n >= N) continue;
    const uint32_t c = s_cnt[j];
    const VariantParameters& vp = VARIANT_LUT[flags[n] >> 4];
    const RowBuilt rb = build_row(s_t, s_w, j, n, c, frozen_from(vp), A, want_sum != 0u, permute != 0u, rt, rw, cnt,
                                  amask, omask, lfz, xlit, vp.signal_propagation_length == s_pmax, lsum, posmap);
    if (lane == 0 && c) {
      wc = max(wc, c);
      ws = max(ws, rb.smx);
      wh += rb.hsum + slot_mix(c, n);
      wp += rb.pfx;
      wl += c;
    }
  }
  if (lane == 0) { s_bc[warp] = wc; s_bs[warp] = ws; s_bh[warp] = wh; s_bp[warp] = wp; s_bl[warp] = wl; }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t bc = 0, bs = 0, bp = 0, bl = 0;
    unsigned long long bh = 0;
    for (int q = 0; q < 8; q++) {
      bc = max(bc, s_bc[q]);
      bs = max(bs, s_bs[q]);
      bh += s_bh[q];
      bp += s_bp[q];
      bl += s_bl[q];
    }
    if (bc > *(volatile uint32_t*)&ctl->row_smax) atomicMax(&ctl->row_smax, bc);
    if (bs > *(volatile uint32_t*)&ctl->seg_max) atomicMax(&ctl->seg_max, bs);
    if (want_sum) atomicAdd(&ctl->row_sum, bh);
    if (bp) atomicAdd(&ctl->pfx_total, (unsigned long long)bp);
    if (bl) atomicAdd(&ctl->slot_total, (unsigned long long)bl);
  }
}

// Layout start: the owner counts cleared and, for permuted rows, the axons
// fully lit in the last tick the rows saw (the lit bitmap it left) taken as
// the lit set of the layout (the prologue checks every tick that they still
// are).
__global__ void __launch_bounds__(256) k_rows_prep(const ShardCtl* __restrict__ ctl, uint32_t* __restrict__ mult,
                                                   uint32_t A, const uint32_t* __restrict__ lit,
                                                   uint32_t* __restrict__ xlit, uint32_t cond) {
  if (cond && !ctl->lay_now) return;
  const uint32_t words = A / 32 + 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A; i += gridDim.x * blockDim.x) {
    mult[i] = 0u;
    if (xlit && i < words) xlit[i] = lit[i];
  }
}

__global__ void __launch_bounds__(256) k_rows_mult(const uint32_t* __restrict__ s2a, uint32_t N, uint32_t A,
                                                   uint32_t* __restrict__ mult, uint2* __restrict__ mask2,
                                                   ShardCtl* __restrict__ ctl, uint32_t cond) {
  if (cond && !ctl->lay_now) return;
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n == 0) {
    mask2[A] = make_uint2(0u, 0x80000000u);   // dummy entry of invalid targets: no hit, exact path
    ctl->row_smax = 0;
    ctl->seg_max = 0;
    ctl->row_sum = 0;
    ctl->pmax = lut_pmax();
    ctl->pfx_total = 0;
    ctl->slot_total = 0;
  }
  if (n >= N) return;
  const uint32_t a = s2a[n];
  if (a < A) atomicAdd(&mult[a], 1u);
}

// Batch end: weights rows -> columnar, a thread per neuron.  The k-th set bit
// of omask[n] (a columnar slot q) is row position k: the row's first group,
// the only slots whose weights GSOP can have changed.  A neuron without such
// slots (every neuron of a frozen row) costs one 16-byte load, so in a brain
// whose weights have mostly frozen the write-back reads 16 bytes a neuron
// instead of a tile's rows.  Where every slot is movable, neighbouring threads
// write the same slot of neighbouring neurons: 64 contiguous bytes a warp.
__global__ void __launch_bounds__(256) k_rows_writeback(int16_t* __restrict__ weights, uint32_t N,
                                                        const int16_t* __restrict__ rw,
                                                        const uint4* __restrict__ omask) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const uint4 om = omask[n];
  const uint32_t o[4] = {om.x, om.y, om.z, om.w};
  const int16_t* row = rw + (size_t)n * kRowStride;
  uint32_t k = 0;
#pragma unroll
  for (int ch = 0; ch < 4; ch++) {
    uint32_t b = o[ch];
    while (b) {
      const uint32_t q = 32u * ch + (uint32_t)(__ffs(b) - 1);
      b &= b - 1u;
      weights[(size_t)q * N + n] = row[k++];
    }
  }
}

// Learned engine, in the prologue: per-tile active synapses and heads in
// flight; on a sparse tick, the block's active axons go into its tile's
// segment (a 256-thread block lies inside one 1024-axon tile).  A tile whose
// active synapses exceed the capacity the predictor gave it sets the overflow
// flag.
__device__ __forceinline__ void learn_axons(const LearnDev& L, uint32_t i, uint32_t A, uint32_t fan,
                                            uint32_t inflight) {
  __shared__ uint32_t s_red[3][8];
  __shared__ uint32_t s_base2;
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool act = fan != 0u;
  const uint32_t ball = __ballot_sync(kFull, act);
  const uint32_t f = warp_sum(fan), b = warp_sum(inflight);
  if (lane == 0) { s_red[0][w] = f; s_red[1][w] = b; s_red[2][w] = __popc(ball); }
  __syncthreads();
  const uint32_t i0 = blockIdx.x * blockDim.x;
  const uint32_t j = i0 >> 10;
  const bool sparse = L.ctl->mode == 1u;
  if (threadIdx.x == 0) {
    uint32_t tf = 0, tb = 0, tc = 0;
    for (int q = 0; q < 8; q++) {
      tf += s_red[0][q];
      tb += s_red[1][q];
      const uint32_t c = s_red[2][q];
      s_red[2][q] = tc;
      tc += c;
    }
    s_base2 = 0;
    if (i0 < A) {
      const uint32_t old = atomicAdd(&L.yacc[j], tf);
      atomicAdd(&L.bacc[j], tb);
      if (sparse) {
        if (tc) s_base2 = atomicAdd(&L.fill[j], tc);
        if (old + tf > L.cap[j]) L.ctl->overflow = 1u;
      }
    }
  }
  __syncthreads();
  // an axon is appended once per tick, so a tile's segment never exceeds its 1024 axons
  if (sparse && act) L.alist[(size_t)j * 1024u + s_base2 + s_red[2][w] + __popc(ball & ((1u << lane) - 1u))] = i;
}

// ---------------------------------------------------------------------------
// per tick 1/4 of the learned engine (LEARN): axons (inject, network pushes,
// propagate, split masks) and somas (refractory countdown, list of neurons to
// evaluate), with learn_axons' per-tile activity and, on sparse ticks, the
// compaction of the active axons.  The list entry positions are reserved once
// per block.  The plain engine runs k_rows_prologue_plain.
// ---------------------------------------------------------------------------
template <bool LEARN>
__global__ void __launch_bounds__(256) k_rows_prologue(BurstHeads8* __restrict__ heads, uint32_t A, uint32_t v_seg,
                                                       const uint32_t* __restrict__ bitmask, uint32_t voff,
                                                       uint32_t nv, uint32_t* __restrict__ incoming,
                                                       const uint32_t* __restrict__ batch_counts, uint32_t k,
                                                       uint2* __restrict__ mask2, const uint32_t* __restrict__ mult,
                                                       uint8_t* __restrict__ flags, uint8_t* __restrict__ timers,
                                                       uint32_t N, uint32_t* __restrict__ eval,
                                                       ShardCtl* __restrict__ ctl, uint32_t raise_err,
                                                       uint32_t* __restrict__ lit_bits, LearnDev L,
                                                       uint32_t* __restrict__ pend_apply,
                                                       const uint32_t* __restrict__ xlit) {
  __shared__ uint32_t s_base;
  __shared__ uint32_t s_warp[8];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t xw = (xlit && i < A) ? __ldg(xlit + (i >> 5)) : 0u;   // axons the row layout took as fully lit
  // every load first, with no barrier before them: heads, owners, pending
  // pushes, input bit; the batch constants are read by every thread (the LUT's
  // largest length and the largest segment, both set by the row copy)
  uint4 hx = make_uint4(0, 0, 0, 0), hy = hx;
  uint32_t own = 0, pc = 0, ibit = 0;
  const uint8_t tm = i < N ? timers[i] : (uint8_t)0;
  if (i < A) {
    const uint4* p = reinterpret_cast<const uint4*>(heads + i);
    hx = p[0];
    hy = p[1];
    own = __ldg(mult + i);
    if (pend_apply) pc = pend_apply[i];   // the previous tick's soma pushes (pushes commute)
    if (bitmask) {
      const uint32_t v = i - voff;
      if (v < nv) ibit = (__ldg(bitmask + (v >> 5)) >> (v & 31u)) & 1u;
    }
  }
  const uint32_t pmax = ctl->pmax, seg_max = ctl->seg_max;
  const uint32_t hi = min(seg_max, 30u);   // segments 1..hi are the ones the batch's slots use
  const uint32_t need = hi ? (((2u << hi) - 1u) & ~1u) : 0xFFFFFFFFu;
  // segments the batch's slots use: 0..seg_max (bit 31: any segment >= 31)
  const uint32_t act = seg_max >= 31u ? 0xFFFFFFFFu : ((2u << seg_max) - 1u);
  const bool inc = batch_counts && batch_counts[k] > 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->ctr[0] += 1;
    if (raise_err) atomicOr(&ctl->err, raise_err);
    ctl->fix_count = 0;      // the previous tick's fix-up is done
    ctl->fix_overflow = 0;
  }
  bool lit = false;
  uint32_t fan = 0, inflight = 0;   // LEARN: active synapses and heads in flight of axon i
  if (i < A) {
    uint32_t h[8] = {hx.x, hx.y, hx.z, hx.w, hy.x, hy.y, hy.z, hy.w};
    uint32_t npush = ibit + pc;
    if (pc) pend_apply[i] = 0;
    if (inc) {
      const uint32_t c = incoming[i];
      if (c) { npush += c; incoming[i] = 0; }
    }
    push_n(h, npush);
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (h[j] != AXC_AXON_SENTINEL) h[j] += v_seg;
    uint4* p = reinterpret_cast<uint4*>(heads + i);
    p[0] = make_uint4(h[0], h[1], h[2], h[3]);
    p[1] = make_uint4(h[4], h[5], h[6], h[7]);
    const uint2 m = split_masks(h, pmax, own);
    mask2[i] = m;
    // fully lit: heads 0..6 hit every segment 1..seg_max the batch uses and at
    // most one soma owns the axon, so for those segments the hit is 1 and one
    // push cannot change it
    lit = (m.x & need) == need && !(m.y >> 31);
    if (LEARN) {
      // active: some head covers a segment that a slot of the batch uses
      if (((m.x | (m.y & 0x7FFFFFFFu)) & act) != 0u) fan = __ldg(L.inv_off + i + 1) - __ldg(L.inv_off + i);
#pragma unroll
      for (int j = 0; j < 8; j++) inflight += h[j] < 255u + pmax ? 1u : 0u;
    }
  }
  if (LEARN) learn_axons(L, i, A, fan, inflight);
  if (lit_bits) {
    const uint32_t lb = __ballot_sync(kFull, lit);
    if ((threadIdx.x & 31) == 0 && i < A) {
      lit_bits[i >> 5] = lb;
      if (xw & ~lb) atomicOr(&ctl->dense[k & 1], 1u);   // the lit-sum form cannot run this tick
    }
  }
  bool ev = false;
  if (i < N) {
    if (tm > 0) {                                 // physics.cu:168-174 after the burst reset
      timers[i] = (uint8_t)(tm - 1);
      flags[i] = flags[i] & 0xF0;
    } else {
      ev = true;
    }
  }
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t ballot = __ballot_sync(kFull, ev);
  if (LEARN && lane == 0 && i < N) L.evbits[i >> 5] = ballot;
  if (lane == 0) s_warp[w] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int q = 0; q < 8; q++) { const uint32_t c = s_warp[q]; s_warp[q] = tot; tot += c; }
    s_base = tot ? atomicAdd(&ctl->eval_count[k & 1], tot) : 0u;
  }
  __syncthreads();
  if (ev) eval[s_base + s_warp[w] + __popc(ballot & ((1u << lane) - 1u))] = i;
}

// ---------------------------------------------------------------------------
// per tick 2/4: 8 lanes per evaluated neuron, lane g holds slots
// 32j + 4g .. 32j + 4g + 3 (j = 0..3) of the neuron's row in registers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t word_of(const uint4& v, int i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}
__device__ __forceinline__ int16_t half_of(const uint2& v, int i) {
  const uint32_t w = (i < 2) ? v.x : v.y;
  return (int16_t)((i & 1) ? (w >> 16) : (w & 0xFFFFu));
}
__device__ __forceinline__ void set_half(uint2& v, int i, int16_t x) {
  uint32_t& w = (i < 2) ? v.x : v.y;
  w = (i & 1) ? ((w & 0x0000FFFFu) | ((uint32_t)(uint16_t)x << 16)) : ((w & 0xFFFF0000u) | (uint16_t)x);
}

// Rare paths of the update pass, kept out of line so that the hot loop keeps
// its registers.
__device__ __noinline__ bool hit_exact(const BurstHeads8* heads, uint32_t A, uint32_t a, uint32_t s,
                                       uint32_t prop) {
  return a < A && heads_hit(heads, a, s, prop);
}

// General GSOP of one slot with exact distances.  Returns 0 when applied, 1
// when the slot must be deferred to the fix-up stage (its result depends on
// same-tick pushes), 2 when the target is invalid (skipped, physics.cu would
// read out of bounds).
__device__ __noinline__ int gsop_general(const BurstHeads8* heads, const uint2* mask2, uint32_t A, uint32_t a,
                                         uint32_t s, const VariantParameters& p, uint8_t flags, int32_t dopamine,
                                         int16_t* w16) {
  if (a >= A) return 2;
  const uint2 m = __ldg(mask2 + a);
  uint32_t md, md1;
  md_pair(heads, a, s, p.signal_propagation_length, &md, &md1);
  if ((m.y >> 31) || md != md1) return 1;
  const GsopConsts gc = gsop_consts((uint8_t)((flags & 0xF0) | 0x05), p, dopamine);
  *w16 = gsop_weight(*w16, md, p, gc.bm, gc.raw_pot, gc.final_dep);
  return 0;
}

// GSOP deltas per variant and inertia rank for a spiker (flags type | 0b101:
// burst multiplier 2, physics.cu:255, 271-273, 290-291; physics.cu:336-349).
// Called by the first 256 threads of the block.
__device__ __forceinline__ void build_gtab(int2 (*gtab)[16], const VariantParameters* lut, int32_t dopamine) {
  if (threadIdx.x < 256) {
    const uint32_t v = threadIdx.x >> 4, r = threadIdx.x & 15;
    const GsopConsts g = gsop_consts((uint8_t)((v << 4) | 0x05), lut[v], dopamine);
    const int32_t inertia = lut[v].inertia_curve[r];
    gtab[v][r] = make_int2(wmul(wmul(g.raw_pot, inertia), g.bm) >> 7, wmul(wmul(g.final_dep, inertia), g.bm) >> 7);
  }
}

// How the 8 lanes of a neuron hold its row, from the shard's longest row
// smax: F full rounds of 32 slots (lane g: slots 32j+4g..32j+4g+3, one vector
// load each of targets and weights) and, for rows that end inside a round, TR
// single-slot rounds (lane g: slot 32F+g+8t) kept in the round-3 registers
// (T[3].x / T[3].y, the two halves of W[3].x).  A 100-slot row takes 3 full
// rounds and one single-slot round instead of 4 full rounds, three quarters of
// whose last round would be empty; a tail of more than 16 slots takes a full
// round.
struct RowShape {
  uint32_t F, TR;
};

__device__ __forceinline__ RowShape row_shape(uint32_t smax) {
  uint32_t F = smax >> 5, tail = smax & 31u;
  if (tail > 16u) {
    F++;
    tail = 0;
  }
  return RowShape{F, (tail + 7u) >> 3};
}

__device__ __forceinline__ void row_load(uint4 (&T)[4], uint2 (&W)[4], const uint32_t* rt_n, const int16_t* rw_n,
                                         uint32_t g8, bool valid, RowShape sh, uint32_t smax) {
#pragma unroll
  for (int j = 0; j < 4; j++) {
    T[j] = make_uint4(0, 0, 0, 0);
    W[j] = make_uint2(0, 0);
    if (valid && (uint32_t)j < sh.F && 32u * j + 4u * g8 < smax) {
      T[j] = __ldg(reinterpret_cast<const uint4*>(rt_n + 32 * j + 4 * g8));
      W[j] = *reinterpret_cast<const uint2*>(rw_n + 32 * j + 4 * g8);
    }
  }
  if (sh.F < 4u && valid) {
    const uint32_t q0 = 32u * sh.F + g8;
    if (sh.TR > 0u && q0 < smax) {
      T[3].x = __ldg(rt_n + q0);
      W[3].x = (uint16_t)rw_n[q0];
    }
    if (sh.TR > 1u && q0 + 8u < smax) {
      T[3].y = __ldg(rt_n + q0 + 8);
      W[3].x |= (uint32_t)(uint16_t)rw_n[q0 + 8] << 16;
    }
  }
}

// Bulk copy global -> shared completed on an mbarrier (cp.async.bulk, the
// untiled TMA path: 16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase `parity` of bar at most `tries` tries (default kWaitLimit); false: gave up.
constexpr uint32_t kWaitLimit = 1u << 16;
// Tries of the update pass's first wait for the staged bitmap
// (axc_row_engine_wait_limit; tests set 0 to take the give-up path).  The
// drain wait before the block exits always has kWaitLimit tries.
__device__ uint32_t g_first_wait_limit = kWaitLimit;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t tries = kWaitLimit) {
  for (uint32_t it = 0; it < tries; it++)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// The dendrite pass over the slots one lane holds (row_shape) of a row with c
// used slots: returns the lane's share of the input current and sets, per slot
// (bit 4j+i; single-slot round t: bit 12+t), hitb = the segment is hit and
// slowb = GSOP needs the exact path (physics.cu:186-207 for the hit test).
template <bool LIT>
__device__ __forceinline__ int32_t row_slots(const uint4 (&T)[4], const uint2 (&W)[4], uint32_t c, uint32_t g8,
                                             RowShape sh, const uint2* __restrict__ mask2, const uint32_t* s_lit,
                                             uint32_t seg_hi, bool exact, bool gfast, uint32_t prop,
                                             const BurstHeads8* heads, uint32_t A, uint32_t& hitb_out,
                                             uint32_t& slowb_out, bool lit_on = true) {
  int32_t i_in = 0;
  const bool glit = LIT && lit_on && gfast;   // the fully-lit shortcut applies
  uint32_t hitb = 0, slowb = 0;   // bit 4j+i
#pragma unroll
  for (int j = 0; j < 4; j++) {
    if ((uint32_t)j >= sh.F) continue;
    const uint32_t q0 = 32u * j + 4u * g8;
    uint2 m[4];
    bool lit[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const uint32_t t = word_of(T[j], i);
      const uint32_t ax = (t & AXC_TARGET_AXON_MASK) - 1u;   // invalid ids were redirected to A
      lit[i] = glit && ((t >> AXC_TARGET_SEG_SHIFT) - 1u) < seg_hi && ((s_lit[ax >> 5] >> (ax & 31u)) & 1u);
      m[i] = (q0 + i < c && !lit[i]) ? __ldg(mask2 + ax) : make_uint2(0, 0);
    }
    uint32_t need = 0;   // live slots off the fully-lit path
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (q0 + i >= c) continue;
      if (LIT && lit[i]) {                      // segment 1..30 of a fully lit axon: hit, fast GSOP
        i_in = wadd(i_in, (int32_t)half_of(W[j], i));
        hitb |= 1u << (4 * j + i);
      } else {
        need |= 1u << i;
      }
    }
    // warp-uniform: most rounds have every slot of the warp's four rows on the
    // fully-lit path, and skip the mask path as a whole
    if (LIT && !__any_sync(kFull, need)) continue;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (!((need >> i) & 1u)) continue;
      const uint32_t t = word_of(T[j], i);
      const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
      const uint32_t sh = min(s, 31u);
      const uint32_t bx = (m[i].x >> sh) & 1u, by = (m[i].y >> sh) & 1u;
      bool hit = (bx | by) != 0u;              // bit 31 (s >= 31): "may hit", tested below
      if (hit && (s >= 31u || !exact))
        hit = hit_exact(heads, A, (t & AXC_TARGET_AXON_MASK) - 1u, s, prop);
      if (hit) {
        i_in = wadd(i_in, (int32_t)half_of(W[j], i));
        hitb |= 1u << (4 * j + i);
      }
      // fast GSOP: hit decides, and one same-tick push could not change it
      const bool fast = gfast && s < 31u && !(m[i].y >> 31) && (bx || by == (s == 0u));
      slowb |= fast ? 0u : (1u << (4 * j + i));
    }
  }
  if (sh.F < 4u) {
    // single-slot tail rounds t = 0, 1: slot 32F + g8 + 8t, bit 12 + t
    uint2 m[2];
    uint32_t need = 0;
#pragma unroll
    for (int t = 0; t < 2; t++) {
      m[t] = make_uint2(0, 0);
      const uint32_t q = 32u * sh.F + g8 + 8u * t;
      if ((uint32_t)t >= sh.TR || q >= c) continue;
      const uint32_t tw = t ? T[3].y : T[3].x;
      const uint32_t ax = (tw & AXC_TARGET_AXON_MASK) - 1u;
      if (glit && ((tw >> AXC_TARGET_SEG_SHIFT) - 1u) < seg_hi && ((s_lit[ax >> 5] >> (ax & 31u)) & 1u)) {
        i_in = wadd(i_in, (int32_t)half_of(W[3], t));
        hitb |= 1u << (12 + t);
      } else {
        m[t] = __ldg(mask2 + ax);
        need |= 1u << t;
      }
    }
    if (!LIT || __any_sync(kFull, need)) {
#pragma unroll
      for (int t = 0; t < 2; t++) {
        if (!((need >> t) & 1u)) continue;
        const uint32_t tw = t ? T[3].y : T[3].x;
        const uint32_t b = 1u << (12 + t);
        const int32_t w = (int32_t)half_of(W[3], t);
        const uint32_t s = tw >> AXC_TARGET_SEG_SHIFT;
        const uint32_t shv = min(s, 31u);
        const uint32_t bx = (m[t].x >> shv) & 1u, by = (m[t].y >> shv) & 1u;
        bool hit = (bx | by) != 0u;
        if (hit && (s >= 31u || !exact)) hit = hit_exact(heads, A, (tw & AXC_TARGET_AXON_MASK) - 1u, s, prop);
        if (hit) {
          i_in = wadd(i_in, w);
          hitb |= b;
        }
        const bool fast = gfast && s < 31u && !(m[t].y >> 31) && (bx || by == (s == 0u));
        slowb |= fast ? 0u : b;
      }
    }
  }
  hitb_out = hitb;
  slowb_out = slowb;
  return i_in;
}

// GLIF of one evaluated (non-refractory) neuron, physics.cu:209-275.
struct GlifOut {
  int32_t v, thr;
  int glif, spike;
};

__device__ __forceinline__ GlifOut glif_step(const VariantParameters& p, int32_t v0, int32_t thr0, int32_t i_in,
                                             uint32_t tick, uint32_t n) {
  GlifOut o;
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
  if (glif) {
    v = p.rest_potential;
    thr = wadd(thr, p.homeostasis_penalty);
  }
  o.v = v;
  o.thr = thr;
  o.glif = glif;
  o.spike = glif | hb;
  return o;
}

// GSOP of a spiker's slots held by this lane (physics.cu:281-373): fast slots
// from the gtab deltas, slow ones on the exact path or deferred to the fix-up
// list.  Writes the changed weights back to the row (rt_n / rw_n: the
// neuron's row); returns the slots done.
template <bool WT = false>
__device__ __forceinline__ uint32_t row_gsop(uint2 (&W)[4], uint32_t hitb, uint32_t slowb,
                                             uint32_t c, uint32_t g8, RowShape sh, const int2 (*gtab)[16],
                                             uint32_t var, const uint32_t* rt_n, int16_t* rw_n,
                                             const BurstHeads8* heads, const uint2* mask2, uint32_t A,
                                             const VariantParameters& p, uint8_t flags, int32_t dopamine,
                                             ShardCtl* ctl, uint32_t* fix, uint32_t fix_cap, uint32_t n,
                                             const ColWT& wt = ColWT{}) {
  uint32_t gdone = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    if ((uint32_t)j >= sh.F) continue;
    const uint32_t q0 = 32u * j + 4u * g8;
    if (q0 >= c) continue;
    uint2 wj = W[j];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const uint32_t b = 1u << (4 * j + i);
      if (q0 + i >= c) continue;
      const int16_t w16 = half_of(wj, i);
      if (!(slowb & b)) {
        // cooling shift 0: delta = +potentiation or -depression of the weight's rank
        const int32_t aw = w16 < 0 ? -(int32_t)w16 : (int32_t)w16;
        const int2 e = gtab[var][min((uint32_t)aw >> 11, 15u)];
        int32_t na = aw + ((hitb & b) ? e.x : -e.y);
        na = min(max(na, 0), 32767);
        set_half(wj, i, (int16_t)(w16 < 0 ? -na : na));
        gdone++;
        continue;
      }
      const uint32_t t = __ldg(rt_n + q0 + i);
      int16_t nw = w16;
      const int r = gsop_general(heads, mask2, A, (t & AXC_TARGET_AXON_MASK) - 1u, t >> AXC_TARGET_SEG_SHIFT, p,
                                 flags, dopamine, &nw);
      if (r == 2) continue;
      gdone++;
      if (r == 1) {
        const uint32_t slot = atomicAdd(&ctl->fix_count, 1u);
        if (slot < fix_cap) fix[slot] = (uint32_t)((size_t)n * kRowStride + q0 + i);
        else ctl->fix_overflow = 1u;
        continue;
      }
      set_half(wj, i, nw);
    }
    if (wj.x != W[j].x || wj.y != W[j].y) {
      *reinterpret_cast<uint2*>(rw_n + q0) = wj;
      if (WT) {
#pragma unroll
        for (int i = 0; i < 4; i++)
          if (half_of(wj, i) != half_of(W[j], i)) col_write(wt, n, q0 + i, half_of(wj, i));
      }
    }
  }
  if (sh.F < 4u) {
#pragma unroll
    for (int t = 0; t < 2; t++) {
      if ((uint32_t)t >= sh.TR) continue;
      const uint32_t q = 32u * sh.F + g8 + 8u * t;
      if (q >= c) continue;
      const uint32_t b = 1u << (12 + t);
      const int16_t w16 = half_of(W[3], t);
      int16_t nw = w16;
      if (!(slowb & b)) {
        const int32_t aw = w16 < 0 ? -(int32_t)w16 : (int32_t)w16;
        const int2 e = gtab[var][min((uint32_t)aw >> 11, 15u)];
        int32_t na = aw + ((hitb & b) ? e.x : -e.y);
        na = min(max(na, 0), 32767);
        nw = (int16_t)(w16 < 0 ? -na : na);
        gdone++;
      } else {
        const uint32_t tw = __ldg(rt_n + q);
        const int r = gsop_general(heads, mask2, A, (tw & AXC_TARGET_AXON_MASK) - 1u, tw >> AXC_TARGET_SEG_SHIFT,
                                   p, flags, dopamine, &nw);
        if (r == 2) continue;
        gdone++;
        if (r == 1) {
          const uint32_t slot = atomicAdd(&ctl->fix_count, 1u);
          if (slot < fix_cap) fix[slot] = (uint32_t)((size_t)n * kRowStride + q);
          else ctl->fix_overflow = 1u;
          continue;
        }
      }
      if (nw != w16) {
        rw_n[q] = nw;
        if (WT) col_write(wt, n, q, nw);
      }
    }
  }
  return gdone;
}

// LIT: 1024-thread blocks (one per SM) that first copy the prologue's
// fully-lit bitmap (one bit per axon) into shared memory; slots whose axon is
// fully lit need no mask gather from L2.
// INLINE (rows with their movable slots first): GSOP of each spiker's movable
// slots on the weights still in registers; else the spikers with movable
// slots are listed for k_rows_gsop / k_rows_gsop_rows.
// WT: write GSOP's changes through to the columnar blob (the per-tick entry point).
template <bool LIT, bool INLINE, bool WT = false>
__global__ void __launch_bounds__(LIT ? 1024 : 256, LIT ? 1 : 4)
    k_rows_update(ShardVramPtrs P, uint32_t N, uint32_t A, const uint32_t* __restrict__ rt,
                  int16_t* __restrict__ rw, const uint16_t* __restrict__ cnt, const uint2* __restrict__ mask2,
                  const uint32_t* __restrict__ eval, uint32_t* __restrict__ pend, uint32_t* __restrict__ fix,
                  ShardCtl* __restrict__ ctl, uint32_t k, uint32_t fix_cap, const uint32_t* __restrict__ lit_bits,
                  const LearnCtl* __restrict__ lc, uint32_t* __restrict__ gs_n, uint32_t* __restrict__ gd_n,
                  const uint8_t* __restrict__ lfz, uint32_t* __restrict__ wcnt, ColWT wt) {
  __shared__ VariantParameters lut[16];
  __shared__ int2 gtab[16][16];
  __shared__ uint32_t s_pmax;
  __shared__ uint64_t s_bar;
  extern __shared__ __align__(128) uint32_t s_lit[];
  chain_wait();
  chain_open();
  if (lc && lc->mode == 1u && !lc->overflow) return;   // learned engine: this tick runs sparse
  if (INLINE && lsum_tick(ctl, k)) return;              // k_rows_update_lsum runs this tick
  if (LIT && threadIdx.x == 0) mbar_init(&s_bar, 1);
  lut_to_smem(lut);
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  // the fully-lit bitmap: one bulk copy into shared memory
  if (LIT && threadIdx.x == 0) bulk_to_smem(s_lit, lit_bits, lit_smem_bytes(A), &s_bar);
  const int32_t dopamine = (int32_t)(int16_t)ctl->dopamine;
  if (INLINE) {
    build_gtab(gtab, lut, dopamine);
    __syncthreads();
  }
  const uint32_t tick = ctl->tick_base + k;
  const uint32_t ecount = ctl->eval_count[k & 1];
  const uint32_t smax = ctl->row_smax;   // longest row of the shard: rows are loaded up to here
  const RowShape sh = row_shape(smax);
  const uint32_t seg_hi = min(ctl->seg_max, 30u);   // lit bits cover segments 1..seg_hi
  const uint32_t lane = threadIdx.x & 31, g8 = lane & 7, grp = lane >> 3;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // each warp owns a contiguous slice of the list, 4 neurons per step
  const uint32_t per_warp = (((ecount + nwarps - 1) / nwarps) + 3) & ~3u;
  const uint32_t beg = min(wid * per_warp, ecount), end = min(beg + per_warp, ecount);
  uint32_t ev_slots = 0, hits = 0, nspk = 0, gdone = 0, nev = 0, err = 0;
  uint32_t wc = 0, wd = 0;   // spikers this warp listed for the GSOP passes
  bool lit_on = true;
  if (LIT) {
    lit_on = mbar_wait_bounded(&s_bar, 0, g_first_wait_limit);
    if (!lit_on) err |= AXC_ERR_WAIT_LIMIT;   // then without the shortcut (results exact)
  }
  for (uint32_t base = beg; base < end; base += 32) {
    const uint32_t mine = (base + lane < end) ? __ldg(eval + base + lane) : 0u;
    for (uint32_t sub = 0; sub < 32 && base + sub < end; sub += 4) {
      const bool valid = base + sub + grp < end;
      const uint32_t n = __shfl_sync(kFull, mine, sub + grp);
      // every load of the neuron at once: state, count, and its row up to smax
      const uint8_t flags = P.soma_flags[n];
      const uint32_t cw = valid ? cnt[n] : 0u;
      const uint32_t lf = lfz[n];
      const int32_t thr0 = P.threshold_offset[n];
      const int32_t v0 = P.soma_voltage[n];
      const uint32_t* rt_n = rt + (size_t)n * kRowStride;
      int16_t* rw_n = rw + (size_t)n * kRowStride;
      uint4 T[4];
      uint2 W[4];
      row_load(T, W, rt_n, rw_n, g8, valid, sh, smax);
      const uint32_t c = cw & 0xFFu;
      const uint32_t var = flags >> 4;
      const VariantParameters& p = lut[var];
      const uint32_t prop = p.signal_propagation_length;
      const bool exact = prop == s_pmax;
      const bool gfast = exact && prop <= 16u;
      if (cw & kRowBad) err |= AXC_ERR_TARGET_RANGE;
      uint32_t hitb, slowb;
      // the fully-lit test reads the bitmap from shared memory (LIT) or, when it
      // did not fit there, from global memory (1 bit per axon: far fewer bytes
      // to keep in L1/L2 than the 8-byte masks)
      int32_t i_in = row_slots<true>(T, W, c, g8, sh, mask2, LIT ? s_lit : lit_bits, seg_hi, exact, gfast, prop,
                                     P.axon_heads, A, hitb, slowb, lit_on);
      i_in = wadd(i_in, __shfl_xor_sync(kFull, i_in, 1));
      i_in = wadd(i_in, __shfl_xor_sync(kFull, i_in, 2));
      i_in = wadd(i_in, __shfl_xor_sync(kFull, i_in, 4));
      if (g8 == 0 && valid) { ev_slots += c; nev++; }
      hits += __popc(hitb);
      // GLIF (physics.cu:209-275); the neuron is not refractory
      int spike = 0;
      if (valid) {
        const GlifOut o = glif_step(p, v0, thr0, i_in, tick, n);
        spike = o.spike;
        if (g8 == 0) {
          P.soma_voltage[n] = o.v;
          P.soma_flags[n] = (uint8_t)((flags & 0xF0) | (spike ? 0x05 : 0x00));
          P.threshold_offset[n] = o.thr;
          P.timers[n] = o.glif ? p.refractory_period : 0;
          if (spike) {
            nspk++;
            const uint32_t my_axon = P.soma_to_axon[n];
            if (my_axon != AXC_NO_AXON) {
              if (my_axon < A) atomicAdd(&pend[my_axon], 1u);
              else err |= AXC_ERR_SOMA_AXON;
            }
          }
        }
      }
      if (INLINE) {
        // GSOP (physics.cu:281-373) of the spiker's movable slots, the first lf
        // of its row; frozen slots (GSOP leaves them as they are) are counted
        if (spike && lf > 0u)
          gdone += row_gsop<WT>(W, hitb, slowb, lf, g8, sh, gtab, var, rt_n, rw_n, P.axon_heads, mask2, A, p,
                                flags, dopamine, ctl, fix, fix_cap, n, wt);
        if (spike && g8 == 0) gdone += c - lf;
        continue;
      }
      // GSOP (physics.cu:281-373) runs in k_rows_gsop / k_rows_gsop_rows over
      // the spikers listed here (those with slots that may move: a few, or
      // many), in this warp's segments of the lists; frozen slots (GSOP leaves
      // them as they are) of a row with a few movable ones or none are only
      // counted here
      const bool few = spike && lf > 0u && lf <= 8u, many = spike && lf > 8u;
      if (spike && lf <= 8u && g8 == 0) gdone += c - lf;
      const uint32_t ab = __ballot_sync(kFull, few && g8 == 0), db = __ballot_sync(kFull, many && g8 == 0);
      if (few && g8 == 0) gs_n[beg + wc + __popc(ab & ((1u << lane) - 1u))] = n;
      if (many && g8 == 0) gd_n[beg + wd + __popc(db & ((1u << lane) - 1u))] = n;
      wc += __popc(ab);
      wd += __popc(db);
    }
  }
  if (!INLINE && lane == 0) {
    wcnt[wid] = wc;
    wcnt[kMaxUpdateWarps + wid] = wd;
  }
  // a warp that gave up: the copy must land before the block exits
  if (LIT && !lit_on && !mbar_wait_bounded(&s_bar, 0)) err |= AXC_ERR_WAIT_LIMIT;
  const uint32_t err_any = __reduce_or_sync(kFull, err);
  if (err_any && lane == 0) atomicOr(&ctl->err, err_any);
  block_count(ev_slots, hits, nspk, &ctl->ctr[1]);
  block_count(gdone, nev, 0, &ctl->ctr[4]);
}

// Sums six per-thread counters over a 256-thread block into ctr[1..5] and
// ctr[7] (evaluated slots, hits, spikes, GSOP slots, evaluated neurons, tested
// slots): one barrier, one atomic per counter.
__device__ __forceinline__ void block_count256(uint32_t a1, uint32_t a2, uint32_t a3, uint32_t a4, uint32_t a5,
                                               uint32_t a7, unsigned long long* ctr) {
  __shared__ uint32_t red[6][8];
  const uint32_t v[6] = {__reduce_add_sync(kFull, a1), __reduce_add_sync(kFull, a2), __reduce_add_sync(kFull, a3),
                         __reduce_add_sync(kFull, a4), __reduce_add_sync(kFull, a5), __reduce_add_sync(kFull, a7)};
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 6; c++) red[c][w] = v[c];
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    unsigned long long sum = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) sum += red[threadIdx.x][q];
    if (sum) atomicAdd(ctr + (threadIdx.x == 5 ? 7 : threadIdx.x + 1), sum);
  }
}

// The hit test of one slot as the 8-lane pass makes it (row_slots): the
// fully-lit shortcut for segments 1..seg_hi of variants whose length is the LUT
// maximum (<= 16), else the tick's split masks and, where they do not decide,
// the eight heads.  *fast: GSOP may take the slot's delta from the gtab table
// (the hit decides and one same-tick push cannot change it).
__device__ __forceinline__ bool slot_hit(uint32_t t, bool exact, bool gfast, uint32_t prop, uint32_t seg_hi,
                                         const uint32_t* __restrict__ lit_bits, const uint2* __restrict__ mask2,
                                         const BurstHeads8* heads, uint32_t A, bool* fast) {
  const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
  const uint32_t ax = (t & AXC_TARGET_AXON_MASK) - 1u;   // invalid ids were redirected to A (dummy mask entry)
  if (gfast && (s - 1u) < seg_hi && ((__ldg(lit_bits + (ax >> 5)) >> (ax & 31u)) & 1u)) {
    *fast = true;
    return true;
  }
  const uint2 m = __ldg(mask2 + ax);
  const uint32_t sh = min(s, 31u);
  const uint32_t bx = (m.x >> sh) & 1u, by = (m.y >> sh) & 1u;
  bool hit = (bx | by) != 0u;
  if (hit && (s >= 31u || !exact)) hit = hit_exact(heads, A, ax, s, prop);
  *fast = gfast && s < 31u && !(m.y >> 31) && (bx || by == (s == 0u));
  return hit;
}

// ---------------------------------------------------------------------------
// per tick 2/4, lit-sum form (lsum_tick: short tested prefixes, and every axon
// the row layout took as fully lit is fully lit): a thread per evaluated
// neuron.  Its input current is the row's lit-sum (frozen slots on fully-lit
// axons with segments 1..30: hits whatever the tick, their weights summed once
// per batch; the dendrite sum is a wrapping i32 sum, so the order cannot change
// a bit) plus the hits among the first lsum[n].y row positions, tested as the
// 8-lane pass tests them (physics.cu:182-206); GLIF (physics.cu:209-275); then
// GSOP of a spiker's movable slots, the first lf positions (physics.cu:281-373),
// from the gtab deltas, on the exact path or deferred to the fix-up stage.
// WT: weight changes written through to the columnar blob (per-tick entry point).
// ---------------------------------------------------------------------------
constexpr int kLsumBlocks = 5;   // resident 256-thread blocks per SM (48 registers a thread)
template <bool WT>
__global__ void __launch_bounds__(256, kLsumBlocks) k_rows_update_lsum(ShardVramPtrs P, uint32_t A, const uint32_t* __restrict__ rt,
                                                          int16_t* __restrict__ rw, const uint16_t* __restrict__ cnt,
                                                          const uint2* __restrict__ mask2,
                                                          const uint32_t* __restrict__ eval, uint32_t* __restrict__ pend,
                                                          uint32_t* __restrict__ fix, ShardCtl* __restrict__ ctl,
                                                          uint32_t k, uint32_t fix_cap,
                                                          const uint32_t* __restrict__ lit_bits,
                                                          const uint8_t* __restrict__ lfz,
                                                          const int2* __restrict__ lsum, ColWT wt,
                                                          const LearnCtl* __restrict__ lc) {
  chain_wait();
  chain_open();
  if (lc && lc->mode == 1u && !lc->overflow) return;   // learned engine: this tick runs sparse
  if (!lsum_tick(ctl, k)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->ctr[6] += 1;   // ticks on the lit-sum form
  const uint32_t ecount = ctl->eval_count[k & 1];
  if (blockIdx.x * blockDim.x >= ecount) return;   // no neuron for this block: no table to build
  __shared__ VariantParameters lut[16];
  __shared__ int2 gtab[16][16];
  __shared__ uint32_t s_pmax;
  lut_to_smem(lut);
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  const int32_t dopamine = (int32_t)(int16_t)ctl->dopamine;
  build_gtab(gtab, lut, dopamine);
  __syncthreads();
  const uint32_t tick = ctl->tick_base + k;
  const uint32_t seg_hi = min(ctl->seg_max, 30u);
  uint32_t ev_slots = 0, hits = 0, nspk = 0, gdone = 0, nev = 0, err = 0, tested = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ecount; i += gridDim.x * blockDim.x) {
    const uint32_t n = eval[i];
    // every load of the neuron at once
    const uint8_t flags = P.soma_flags[n];
    const uint32_t cw = cnt[n];
    const uint32_t lf = lfz[n];
    const int2 ls = lsum[n];
    const int32_t thr0 = P.threshold_offset[n];
    const int32_t v0 = P.soma_voltage[n];
    const uint32_t my_axon = P.soma_to_axon[n];
    const uint32_t c = cw & 0xFFu, pfx = (uint32_t)ls.y;
    const uint32_t var = flags >> 4;
    const VariantParameters& p = lut[var];
    const uint32_t prop = p.signal_propagation_length;
    const bool exact = prop == s_pmax;
    const bool gfast = exact && prop <= 16u;
    if (cw & kRowBad) err |= AXC_ERR_TARGET_RANGE;
    const uint32_t* rt_n = rt + (size_t)n * kRowStride;
    int16_t* rw_n = rw + (size_t)n * kRowStride;
    int32_t i_in = ls.x;
    uint32_t h = c - pfx;   // the lit-sum slots are hits
    // the tests of row positions 0..31 (the movable slots come first), kept for GSOP
    uint32_t hit_bits = 0, fast_bits = 0;
    for (uint32_t q = 0; q < pfx; q += 4) {
      const uint4 T4 = *reinterpret_cast<const uint4*>(rt_n + q);
      const uint2 W4 = *reinterpret_cast<const uint2*>(rw_n + q);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        if (q + j >= pfx) break;
        bool fast;
        const bool hit = slot_hit(word_of(T4, j), exact, gfast, prop, seg_hi, lit_bits, mask2, P.axon_heads, A, &fast);
        if (hit) {
          i_in = wadd(i_in, (int32_t)half_of(W4, j));
          h++;
        }
        const uint32_t bit = (q + j < 32u) ? (1u << (q + j)) : 0u;
        hit_bits |= hit ? bit : 0u;
        fast_bits |= fast ? bit : 0u;
      }
    }
    ev_slots += c;
    hits += h;
    tested += pfx;
    nev++;
    const GlifOut o = glif_step(p, v0, thr0, i_in, tick, n);
    P.soma_voltage[n] = o.v;
    P.soma_flags[n] = (uint8_t)((flags & 0xF0) | (o.spike ? 0x05 : 0x00));
    P.threshold_offset[n] = o.thr;
    P.timers[n] = o.glif ? p.refractory_period : 0;
    if (!o.spike) continue;
    nspk++;
    if (my_axon != AXC_NO_AXON) {
      if (my_axon < A) atomicAdd(&pend[my_axon], 1u);
      else err |= AXC_ERR_SOMA_AXON;
    }
    // GSOP (physics.cu:281-373) of the movable slots; the frozen ones are left as they are
    gdone += c - lf;
    for (uint32_t q = 0; q < lf; q++) {
      const int16_t w16 = rw_n[q];
      bool fast, hit;
      if (q < 32u) {   // tested in the prefix loop (lf <= pfx)
        hit = (hit_bits >> q) & 1u;
        fast = (fast_bits >> q) & 1u;
      } else {
        hit = slot_hit(rt_n[q], exact, gfast, prop, seg_hi, lit_bits, mask2, P.axon_heads, A, &fast);
      }
      int16_t nw = w16;
      if (fast) {
        const int32_t aw = w16 < 0 ? -(int32_t)w16 : (int32_t)w16;
        const int2 e = gtab[var][min((uint32_t)aw >> 11, 15u)];
        int32_t na = aw + (hit ? e.x : -e.y);
        na = min(max(na, 0), 32767);
        nw = (int16_t)(w16 < 0 ? -na : na);
        gdone++;
      } else {
        const uint32_t t = rt_n[q];
        const int r = gsop_general(P.axon_heads, mask2, A, (t & AXC_TARGET_AXON_MASK) - 1u, t >> AXC_TARGET_SEG_SHIFT,
                                   p, flags, dopamine, &nw);
        if (r == 2) continue;
        gdone++;
        if (r == 1) {
          const uint32_t slot = atomicAdd(&ctl->fix_count, 1u);
          if (slot < fix_cap) fix[slot] = (uint32_t)((size_t)n * kRowStride + q);
          else ctl->fix_overflow = 1u;
          continue;
        }
      }
      if (nw != w16) {
        rw_n[q] = nw;
        if (WT) col_write(wt, n, q, nw);
      }
    }
  }
  const uint32_t err_any = __reduce_or_sync(kFull, err);
  if (err_any && (threadIdx.x & 31) == 0) atomicOr(&ctl->err, err_any);
  block_count256(ev_slots, hits, nspk, gdone, nev, tested, ctl->ctr);
}

// ---------------------------------------------------------------------------
// per tick 2b (learned engine): GSOP (physics.cu:281-373) of the listed
// spikers over the slots of amask only (the others are frozen: GSOP leaves
// them as they are), the (spiker, slot) items of 32 spikers spread over the
// warp's lanes.  Each slot is classified as in the update pass (fully lit,
// else the tick's hit masks; exact path for segments >= 31, other lengths,
// several owners, or a hit that one same-tick push could change) and updated
// from the gtab deltas, on the exact path, or deferred to the fix-up stage.
// Warp w of the listing pass listed its spikers at [beg_w, beg_w + wcnt[w]).
// ---------------------------------------------------------------------------
template <bool LIT>
__global__ void __launch_bounds__(256) k_rows_gsop(ShardVramPtrs P, uint32_t A, const uint32_t* __restrict__ rt,
                                                   int16_t* __restrict__ rw, const uint16_t* __restrict__ cnt,
                                                   const uint2* __restrict__ mask2, const uint32_t* __restrict__ lit_bits,
                                                   const uint4* __restrict__ amask, const uint32_t* __restrict__ gs_n,
                                                   const uint32_t* __restrict__ wcnt, uint32_t nwu,
                                                   uint32_t* __restrict__ fix, ShardCtl* __restrict__ ctl, uint32_t k,
                                                   uint32_t fix_cap, const LearnCtl* __restrict__ lc) {
  // the learned engine lists the spikers of its sparse ticks here; on its dense
  // ticks the update pass applied GSOP itself
  if (lc && !(lc->mode == 1u && !lc->overflow)) return;
  __shared__ VariantParameters lut[16];
  __shared__ int2 gtab[16][16];
  __shared__ uint32_t s_pmax;
  lut_to_smem(lut);
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  const int32_t dopamine = (int32_t)(int16_t)ctl->dopamine;
  build_gtab(gtab, lut, dopamine);
  __syncthreads();
  const uint32_t ecount = ctl->eval_count[k & 1];
  const uint32_t per_warp = (((ecount + nwu - 1) / nwu) + 3) & ~3u;
  const uint32_t seg_hi = min(ctl->seg_max, 30u);
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t ngw = (gridDim.x * blockDim.x) >> 5;
  unsigned long long gdone = 0;
  for (uint32_t uw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; uw < nwu; uw += ngw) {
    const uint32_t cntw = wcnt[uw];
    const uint32_t beg = min(uw * per_warp, ecount);
    for (uint32_t e0 = 0; e0 < cntw; e0 += 32) {
      // 32 listed spikers; their movable slots are spread over the lanes
      const bool has = e0 + lane < cntw;
      const uint32_t my_n = has ? gs_n[beg + e0 + lane] : 0u;
      const uint4 my_am = has ? amask[my_n] : make_uint4(0, 0, 0, 0);
      const uint32_t my_k = __popc(my_am.x) + __popc(my_am.y) + __popc(my_am.z) + __popc(my_am.w);
      uint32_t incl = my_k;   // inclusive prefix of the slot counts over the lanes
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(kFull, incl, o);
        if (lane >= (uint32_t)o) incl += x;
      }
      const uint32_t total = __shfl_sync(kFull, incl, 31);
      for (uint32_t it0 = 0; it0 < total; it0 += 32) {   // warp-uniform: every lane takes part in the shuffles
        const uint32_t it = it0 + lane;
        // the lane that owns item it: the first whose inclusive prefix exceeds it
        uint32_t owner = 0;
#pragma unroll
        for (int stp = 16; stp > 0; stp >>= 1) {
          const uint32_t v = __shfl_sync(kFull, incl, owner + stp - 1);
          if (v <= it) owner += stp;
        }
        owner = min(owner, 31u);
        const uint32_t n = __shfl_sync(kFull, my_n, owner);
        const uint32_t prev = __shfl_sync(kFull, incl - my_k, owner);
        const uint32_t am0 = __shfl_sync(kFull, my_am.x, owner), am1 = __shfl_sync(kFull, my_am.y, owner);
        const uint32_t am2 = __shfl_sync(kFull, my_am.z, owner), am3 = __shfl_sync(kFull, my_am.w, owner);
        if (it >= total) continue;
        uint32_t rank = it - prev, q;   // the rank-th set bit of the owner's mask
        const uint32_t c0 = __popc(am0), c1 = __popc(am1), c2 = __popc(am2);
        if (rank < c0) q = __fns(am0, 0, rank + 1);
        else if ((rank -= c0) < c1) q = 32u + __fns(am1, 0, rank + 1);
        else if ((rank -= c1) < c2) q = 64u + __fns(am2, 0, rank + 1);
        else q = 96u + __fns(am3, 0, rank - c2 + 1);
        const uint8_t flags = P.soma_flags[n];
        const uint32_t var = flags >> 4;
        const VariantParameters& p = lut[var];
        const uint32_t prop = p.signal_propagation_length;
        const bool exact = prop == s_pmax;
        const bool gfast = exact && prop <= 16u;
        const size_t r = (size_t)n * kRowStride + q;
        const uint32_t t = __ldg(rt + r);
        const int16_t w16 = rw[r];
        const uint32_t ax = (t & AXC_TARGET_AXON_MASK) - 1u;
        const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
        bool hit, fast;
        if (LIT && gfast && (s - 1u) < seg_hi && ((__ldg(lit_bits + (ax >> 5)) >> (ax & 31u)) & 1u)) {
          hit = true;
          fast = true;
        } else {
          const uint2 m = __ldg(mask2 + ax);
          const uint32_t sh = min(s, 31u);
          const uint32_t bx = (m.x >> sh) & 1u, by = (m.y >> sh) & 1u;
          hit = (bx | by) != 0u;
          if (hit && (s >= 31u || !exact)) hit = hit_exact(P.axon_heads, A, ax, s, prop);
          fast = gfast && s < 31u && !(m.y >> 31) && (bx || by == (s == 0u));
        }
        int16_t nw = w16;
        if (fast) {
          const int32_t aw = w16 < 0 ? -(int32_t)w16 : (int32_t)w16;
          const int2 d = gtab[var][min((uint32_t)aw >> 11, 15u)];
          int32_t na = aw + (hit ? d.x : -d.y);
          na = min(max(na, 0), 32767);
          nw = (int16_t)(w16 < 0 ? -na : na);
          gdone++;
        } else {
          const int res = gsop_general(P.axon_heads, mask2, A, ax, s, p, flags, dopamine, &nw);
          if (res == 2) continue;
          gdone++;
          if (res == 1) {
            const uint32_t slot = atomicAdd(&ctl->fix_count, 1u);
            if (slot < fix_cap) fix[slot] = (uint32_t)r;
            else ctl->fix_overflow = 1u;
            continue;
          }
        }
        if (nw != w16) rw[r] = nw;
      }
    }
  }
  block_count(gdone, 0, 0, &ctl->ctr[4]);
}

// GSOP of the listed spikers with many slots that may move, 8 lanes per row
// as in the update pass (row_load / row_slots / row_gsop; frozen slots get a
// zero delta).  Warp w of the update pass listed them at [beg_w, beg_w + wcnt[w]).
template <bool LIT>
__global__ void __launch_bounds__(256) k_rows_gsop_rows(ShardVramPtrs P, uint32_t A, const uint32_t* __restrict__ rt,
                                                        int16_t* __restrict__ rw, const uint16_t* __restrict__ cnt,
                                                        const uint2* __restrict__ mask2,
                                                        const uint32_t* __restrict__ lit_bits,
                                                        const uint32_t* __restrict__ gd_n,
                                                        const uint32_t* __restrict__ wcnt, uint32_t nwu,
                                                        uint32_t* __restrict__ fix, ShardCtl* __restrict__ ctl,
                                                        uint32_t k, uint32_t fix_cap, const LearnCtl* __restrict__ lc) {
  if (lc && !(lc->mode == 1u && !lc->overflow)) return;   // as k_rows_gsop
  __shared__ VariantParameters lut[16];
  __shared__ int2 gtab[16][16];
  __shared__ uint32_t s_pmax;
  lut_to_smem(lut);
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  const int32_t dopamine = (int32_t)(int16_t)ctl->dopamine;
  build_gtab(gtab, lut, dopamine);
  __syncthreads();
  const uint32_t ecount = ctl->eval_count[k & 1];
  const uint32_t per_warp = (((ecount + nwu - 1) / nwu) + 3) & ~3u;
  const uint32_t smax = ctl->row_smax;
  const RowShape sh = row_shape(smax);
  const uint32_t seg_hi = min(ctl->seg_max, 30u);
  const uint32_t lane = threadIdx.x & 31, g8 = lane & 7, grp = lane >> 3;
  const uint32_t ngw = (gridDim.x * blockDim.x) >> 5;
  unsigned long long gdone = 0;
  for (uint32_t uw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; uw < nwu; uw += ngw) {
    const uint32_t cntw = wcnt[uw];
    const uint32_t beg = min(uw * per_warp, ecount);
    for (uint32_t e = 0; e < cntw; e += 4) {
      const bool valid = e + grp < cntw;
      const uint32_t n = valid ? gd_n[beg + e + grp] : 0u;
      const uint8_t flags = P.soma_flags[n];
      const uint32_t c = valid ? (cnt[n] & 0xFFu) : 0u;
      const uint32_t var = flags >> 4;
      const VariantParameters& p = lut[var];
      const uint32_t prop = p.signal_propagation_length;
      const bool exact = prop == s_pmax;
      const bool gfast = exact && prop <= 16u;
      const uint32_t* rt_n = rt + (size_t)n * kRowStride;
      int16_t* rw_n = rw + (size_t)n * kRowStride;
      uint4 T[4];
      uint2 W[4];
      row_load(T, W, rt_n, rw_n, g8, valid, sh, smax);
      uint32_t hitb, slowb;
      (void)row_slots<LIT>(T, W, c, g8, sh, mask2, lit_bits, seg_hi, exact, gfast, prop, P.axon_heads, A, hitb,
                           slowb);
      if (valid)
        gdone += row_gsop(W, hitb, slowb, c, g8, sh, gtab, var, rt_n, rw_n, P.axon_heads, mask2, A, p, flags,
                          dopamine, ctl, fix, fix_cap, n);
    }
  }
  block_count(gdone, 0, 0, &ctl->ctr[4]);
}

// ---------------------------------------------------------------------------
// per tick 3/4: deferred GSOP slots, with the actual push count of the axon
// (pend, before the push stage consumes it) and the original weight.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fixup_slot(const ShardVramPtrs& P, const VariantParameters* lut, uint32_t A,
                                           const uint32_t* rt, int16_t* rw, const uint32_t* pend,
                                           uint32_t r, int32_t dopamine, const ColWT& wt = ColWT{}) {
  const uint32_t n = r / kRowStride;
  const uint32_t t = rt[r];
  const uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
  const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
  const uint8_t flags = P.soma_flags[n];
  const VariantParameters& p = lut[flags >> 4];
  uint32_t h[8];
  load_heads(P.axon_heads, a, h);
  push_n(h, pend[a]);
  const uint32_t md = md_of(h, s, p.signal_propagation_length);
  const GsopConsts gc = gsop_consts(flags, p, dopamine);
  const int16_t w0 = rw[r];
  const int16_t w1 = gsop_weight(w0, md, p, gc.bm, gc.raw_pot, gc.final_dep);
  if (w1 != w0) {
    rw[r] = w1;
    if (wt.w) col_write(wt, n, r % kRowStride, w1);
  }
}

__global__ void __launch_bounds__(256) k_rows_fixup(ShardVramPtrs P, uint32_t N, uint32_t A,
                                                    const uint32_t* __restrict__ rt, int16_t* __restrict__ rw,
                                                    const uint16_t* __restrict__ cnt,
                                                    const uint2* __restrict__ mask2, const uint32_t* __restrict__ pend,
                                                    const uint32_t* __restrict__ eval,
                                                    const uint32_t* __restrict__ fix, ShardCtl* __restrict__ ctl,
                                                    uint32_t k, const uint32_t* __restrict__ ids,
                                                    uint8_t* __restrict__ out, uint32_t num_outputs, ColWT wt) {
  chain_wait();
  chain_open();
  const uint32_t nfix = ctl->fix_count;
  const uint32_t overflow = ctl->fix_overflow;
  {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0) {
      ctl->eval_count[(k + 1) & 1] = 0;   // the next tick's list (last used two ticks ago)
      ctl->dense[(k + 1) & 1] = 0;
    }
    // readout of the tick (physics.cu:378-395): flags are final once the update pass is done
    uint32_t err = 0;
    for (uint32_t j = tid; j < num_outputs; j += stride) {
      const uint32_t id = ids[j];
      uint8_t v = 0;
      if (id != AXC_NO_AXON) {
        if (id < N) v = P.soma_flags[id] & 0x01;
        else err = AXC_ERR_READOUT_RANGE;
      }
      out[j] = v;
    }
    if (err) atomicOr(&ctl->err, err);
  }
  if (nfix == 0 && !overflow) return;
  __shared__ VariantParameters lut[16];
  __shared__ uint32_t s_pmax;
  lut_to_smem(lut);
  if (threadIdx.x == 0) s_pmax = lut_pmax();
  __syncthreads();
  const int32_t dopamine = (int32_t)(int16_t)ctl->dopamine;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (!overflow) {
    for (uint32_t i = tid; i < nfix; i += stride) fixup_slot(P, lut, A, rt, rw, pend, fix[i], dopamine, wt);
    return;
  }
  // the list overflowed: rescan every spiker's slots with the update pass's rule
  const uint32_t ecount = ctl->eval_count[k & 1];
  for (uint32_t w = tid; w < ecount * kRowStride; w += stride) {
    const uint32_t n = eval[w / kRowStride], q = w % kRowStride;
    if (!(P.soma_flags[n] & 1) || q >= (cnt[n] & 0xFFu)) continue;
    const uint32_t r = n * kRowStride + q;
    const uint32_t t = rt[r];
    const uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
    if (a >= A) continue;
    const uint32_t s = t >> AXC_TARGET_SEG_SHIFT;
    const VariantParameters& p = lut[P.soma_flags[n] >> 4];
    const uint32_t prop = p.signal_propagation_length;
    const bool gfast = prop == s_pmax && prop <= 16u;
    const uint2 m = mask2[a];
    const uint32_t sh = min(s, 31u);
    const uint32_t bx = (m.x >> sh) & 1u, by = (m.y >> sh) & 1u;
    const bool fast = gfast && s < 31u && !(m.y >> 31) && (bx || by == (s == 0u));
    if (fast) continue;
    uint32_t md0, md1;
    md_pair(P.axon_heads, a, s, prop, &md0, &md1);
    if ((m.y >> 31) || md0 != md1) fixup_slot(P, lut, A, rt, rw, pend, r, dopamine, wt);
  }
}

// per tick 4/4, on a batch's (or learned graph's) last tick: the spikers'
// own-axon pushes (physics.cu:257-261), found in the evaluated list; on the
// other ticks the next prologue applies them.
__global__ void __launch_bounds__(256) k_rows_push(BurstHeads8* __restrict__ heads, const uint32_t* __restrict__ s2a,
                                                   uint32_t A, uint32_t* __restrict__ pend,
                                                   const uint32_t* __restrict__ eval, const uint8_t* __restrict__ flags,
                                                   uint32_t N, const uint32_t* __restrict__ ids,
                                                   uint8_t* __restrict__ out, uint32_t num_outputs,
                                                   ShardCtl* __restrict__ ctl, uint32_t k) {
  chain_wait();
  chain_open();
  const uint32_t ecount = ctl->eval_count[k & 1];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid == 0) {
    ctl->eval_count[(k + 1) & 1] = 0;
    ctl->dense[(k + 1) & 1] = 0;
    ctl->fix_count = 0;
    ctl->fix_overflow = 0;
  }
  for (uint32_t i = tid; i < ecount; i += stride) {
    const uint32_t n = eval[i];
    if (!(flags[n] & 1)) continue;
    const uint32_t ax = s2a[n];
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

__global__ void k_rows_reset_lists(ShardCtl* ctl) {
  ctl->eval_count[0] = 0;
  ctl->eval_count[1] = 0;
  ctl->fix_count = 0;
  ctl->fix_overflow = 0;
  ctl->dense[0] = 0;
  ctl->dense[1] = 0;
}


// ---------------------------------------------------------------------------
// per tick 1/4 of the plain engine: k_rows_prologue without the learned
// engine's per-tile accounting, ITEMS axons and neurons per thread (items
// i0 + 256 r).  No barrier before the loads: every thread reads the batch
// constants (seg_max, the LUT's largest length, set at batch start) itself,
// next to its own loads.  The evaluated neurons are appended with one atomic
// per block.
// ---------------------------------------------------------------------------
// push_n for the common counts 0 and 1 without the general shift network
__device__ __forceinline__ void push_few(uint32_t h[8], uint32_t c) {
  if (c == 1u) {
#pragma unroll
    for (int q = 7; q > 0; q--) h[q] = h[q - 1];
    h[0] = 0u;
  } else if (c > 1u) {
    push_n(h, c);
  }
}

template <int ITEMS>
__global__ void __launch_bounds__(256) k_rows_prologue_plain(BurstHeads8* __restrict__ heads, uint32_t A,
                                                             uint32_t v_seg, const uint32_t* __restrict__ bitmask,
                                                             uint32_t voff, uint32_t nv,
                                                             uint32_t* __restrict__ incoming,
                                                             const uint32_t* __restrict__ batch_counts, uint32_t k,
                                                             uint2* __restrict__ mask2,
                                                             const uint32_t* __restrict__ mult,
                                                             uint8_t* __restrict__ flags,
                                                             uint8_t* __restrict__ timers, uint32_t N,
                                                             uint32_t* __restrict__ eval, ShardCtl* __restrict__ ctl,
                                                             uint32_t raise_err, uint32_t* __restrict__ lit_bits,
                                                             uint32_t* __restrict__ pend_apply, uint32_t inc_direct,
                                                             uint32_t set_tick, uint32_t tick_base, int32_t dopamine,
                                                             const uint32_t* __restrict__ xlit) {
  __shared__ uint32_t s_base;
  __shared__ uint32_t s_warp[ITEMS][8];
  chain_wait();
  chain_open();
  const uint32_t i0 = blockIdx.x * (256u * ITEMS) + threadIdx.x;
  // all loads first: heads, owners, pending pushes, input bits, timers, constants,
  // and the axons the row layout took as fully lit (xlit, 32 per warp)
  uint4 hx[ITEMS], hy[ITEMS];
  uint32_t own[ITEMS], npush[ITEMS], xw[ITEMS];
  uint8_t tm[ITEMS], fl[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; r++) {
    const uint32_t i = i0 + 256u * r;
    npush[r] = 0;
    own[r] = 0;
    tm[r] = 0;
    fl[r] = 0;
    xw[r] = (xlit && i < A) ? __ldg(xlit + (i >> 5)) : 0u;
    if (i < A) {
      const uint4* p = reinterpret_cast<const uint4*>(heads + i);
      hx[r] = p[0];
      hy[r] = p[1];
      own[r] = __ldg(mult + i);
      if (pend_apply) npush[r] = pend_apply[i];   // the previous tick's soma pushes
      if (bitmask) {
        const uint32_t v = i - voff;
        if (v < nv) npush[r] += (__ldg(bitmask + (v >> 5)) >> (v & 31u)) & 1u;
      }
    }
    if (i < N) {
      tm[r] = timers[i];
      fl[r] = flags[i];
    }
  }
  const uint32_t seg_max = ctl->seg_max, pmax = ctl->pmax;
  // network pushes this tick: per-tick calls say so directly, batches by the tick's count
  const bool inc = inc_direct || (batch_counts && batch_counts[k] > 0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->ctr[0] += 1;
    if (raise_err) atomicOr(&ctl->err, raise_err);
    ctl->fix_count = 0;      // the previous tick's fix-up is done
    ctl->fix_overflow = 0;
    if (set_tick) {          // per-tick calls: the tick number and dopamine the later stages read
      ctl->tick_base = tick_base;
      ctl->dopamine = dopamine;
    }
  }
  const uint32_t hi = min(seg_max, 30u);   // segments 1..hi are the ones the batch's slots use
  const uint32_t need = hi ? (((2u << hi) - 1u) & ~1u) : 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t evb[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; r++) {
    const uint32_t i = i0 + 256u * r;
    bool lit = false;
    if (i < A) {
      uint32_t c = npush[r];
      if (pend_apply && c) pend_apply[i] = 0;
      if (inc) {
        const uint32_t ci = incoming[i];
        if (ci) { c += ci; incoming[i] = 0; }
      }
      uint32_t h[8] = {hx[r].x, hx[r].y, hx[r].z, hx[r].w, hy[r].x, hy[r].y, hy[r].z, hy[r].w};
      push_few(h, c);
#pragma unroll
      for (int j = 0; j < 8; j++)
        if (h[j] != AXC_AXON_SENTINEL) h[j] += v_seg;
      uint4* p = reinterpret_cast<uint4*>(heads + i);
      p[0] = make_uint4(h[0], h[1], h[2], h[3]);
      p[1] = make_uint4(h[4], h[5], h[6], h[7]);
      const uint2 m = split_masks(h, pmax, own[r]);
      mask2[i] = m;
      // fully lit: heads 0..6 hit every segment 1..seg_max the batch uses and at
      // most one soma owns the axon (for those segments the hit is 1 and one
      // push cannot change it)
      lit = (m.x & need) == need && !(m.y >> 31);
    }
    const uint32_t lb = __ballot_sync(kFull, lit);
    if (lane == 0 && i < A) {
      lit_bits[i >> 5] = lb;
      // an axon the row layout summed as fully lit is not: this tick takes the full pass
      if (xw[r] & ~lb) atomicOr(&ctl->dense[k & 1], 1u);
    }
    bool ev = false;
    if (i < N) {
      if (tm[r] > 0) {                              // physics.cu:168-174 after the burst reset
        timers[i] = (uint8_t)(tm[r] - 1);
        if (fl[r] & 0x0Fu) flags[i] = fl[r] & 0xF0u;
      } else {
        ev = true;
      }
    }
    evb[r] = __ballot_sync(kFull, ev);
    if (lane == 0) s_warp[r][w] = __popc(evb[r]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int q = 0; q < ITEMS * 8; q++) {
      const uint32_t c = (&s_warp[0][0])[q];
      (&s_warp[0][0])[q] = tot;
      tot += c;
    }
    s_base = tot ? atomicAdd(&ctl->eval_count[k & 1], tot) : 0u;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ITEMS; r++)
    if ((evb[r] >> lane) & 1u)
      eval[s_base + s_warp[r][w] + __popc(evb[r] & ((1u << lane) - 1u))] = i0 + 256u * r;
}
// Items (an axon and a neuron each) per thread of k_rows_prologue_plain: two
// halve the blocks, and with them the list-append atomics on one counter and
// the per-block barriers (1.5M neurons: 18,162 against 17,733 ticks/s; four
// are slower, 16,717), where the grid at one item has at least kProWide
// blocks (four waves of 8 blocks per SM on 152 SMs); a smaller brain keeps one
// item per thread and twice the blocks (16k neurons: 66,644 ticks/s with one
// item and 64 blocks, 60,629 with two and 32).
constexpr uint32_t kProWide = 4864;

}  // namespace

uint32_t set_first_wait_limit(uint32_t tries) {
  static uint32_t current = kWaitLimit;
  const uint32_t prev = current;
  if (cudaMemcpyToSymbol(g_first_wait_limit, &tries, sizeof(tries)) == cudaSuccess) current = tries;
  return prev;
}

cudaError_t rows_alloc(ShardScratch& s, uint32_t N, uint32_t A, bool with_fix, cudaStream_t stream) {
  if (s.rows && s.rows->N >= N && s.rows->A >= A && (s.rows->fix || !with_fix)) return cudaSuccess;
  graph_cache_drop(&s);   // captured graphs hold the old buffers' addresses
  rows_touched(s);
  rows_free(s);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off = 0;
  const size_t o_rt = off; off = al(off + (size_t)N * kRowStride * 4);
  const size_t o_rw = off; off = al(off + (size_t)N * kRowStride * 2);
  const size_t o_cnt = off; off = al(off + (size_t)N * 2);
  const size_t o_m2 = off; off = al(off + ((size_t)A + 1) * 8);
  const size_t o_mult = off; off = al(off + (size_t)A * 4);
  const size_t o_eval = off; off = al(off + (size_t)N * 4 + 4);
  const size_t o_fix = off; off = al(off + (with_fix ? (size_t)kFixCap * 4 : 0));
  const size_t o_lit = off; off = al(off + ((size_t)std::max(A, N) / 32 + 2) * 4 + 16);
  const size_t o_gsn = off; off = al(off + (size_t)N * 4 + 4);
  const size_t o_gdn = off; off = al(off + (size_t)N * 4 + 4);
  const size_t o_am = off; off = al(off + (size_t)N * 16 + 16);
  const size_t o_lfz = off; off = al(off + (size_t)N + 4);
  const size_t o_om = off; off = al(off + (size_t)N * 16 + 16);
  const size_t o_wcnt = off; off = al(off + (size_t)kMaxUpdateWarps * 8);
  const size_t o_lsum = off; off = al(off + (size_t)N * 8 + 8);
  const size_t o_xlit = off; off = al(off + ((size_t)A / 32 + 2) * 4 + 16);
  void* base = nullptr;
  cudaError_t e = cudaMalloc(&base, off);
  if (e != cudaSuccess) return e;
  // zeroed in the order of the caller's stream: a blocking memset would go on
  // the legacy stream, which a non-blocking stream does not wait for (work
  // queued there before it, another shard's graph say, would delay the zeroing
  // into this shard's first batch)
  e = cudaMemsetAsync(base, 0, off, stream);
  if (e == cudaSuccess && stream == nullptr) e = cudaStreamSynchronize(nullptr);
  if (e != cudaSuccess) { cudaFree(base); return e; }
  RowCache* r = new RowCache();
  char* b = static_cast<char*>(base);
  r->N = N;
  r->A = A;
  r->base = base;
  r->rt = reinterpret_cast<uint32_t*>(b + o_rt);
  r->rw = reinterpret_cast<int16_t*>(b + o_rw);
  r->cnt = reinterpret_cast<uint16_t*>(b + o_cnt);
  r->mask2 = reinterpret_cast<uint2*>(b + o_m2);
  r->mult = reinterpret_cast<uint32_t*>(b + o_mult);
  r->eval = reinterpret_cast<uint32_t*>(b + o_eval);
  r->fix = with_fix ? reinterpret_cast<uint32_t*>(b + o_fix) : nullptr;
  r->lit = reinterpret_cast<uint32_t*>(b + o_lit);
  r->gs_n = reinterpret_cast<uint32_t*>(b + o_gsn);
  r->gd_n = reinterpret_cast<uint32_t*>(b + o_gdn);
  r->amask = reinterpret_cast<uint4*>(b + o_am);
  r->lfz = reinterpret_cast<uint8_t*>(b + o_lfz);
  r->omask = reinterpret_cast<uint4*>(b + o_om);
  r->wcnt = reinterpret_cast<uint32_t*>(b + o_wcnt);
  r->lsum = reinterpret_cast<int2*>(b + o_lsum);
  r->xlit = reinterpret_cast<uint32_t*>(b + o_xlit);
  s.rows = r;
  return cudaSuccess;
}

cudaError_t rows_posmap(ShardScratch& s, cudaStream_t stream) {
  if (!s.rows) return cudaErrorInvalidValue;
  if (s.rows->posmap) return cudaSuccess;
  const size_t bytes = (size_t)s.rows->N * kRowStride;
  cudaError_t e = cudaMalloc(&s.rows->posmap, bytes ? bytes : 1);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.rows->posmap, 0, bytes, stream);
  if (e == cudaSuccess) graph_cache_drop(&s);   // graphs captured without the map do not write it
  return e;
}

void rows_free(ShardScratch& s) {
  if (!s.rows) return;
  if (s.rows->posmap) cudaFree(s.rows->posmap);
  cudaFree(s.rows->base);
  delete s.rows;
  s.rows = nullptr;
}

cudaError_t launch_rows_begin(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, uint32_t A, cudaStream_t stream,
                              bool row_sum, bool permute, bool with_posmap, bool conditional) {
  RowCache& r = *s.rows;
  const uint32_t cond = conditional ? 1u : 0u;
  k_rows_reset_lists<<<1, 1, 0, stream>>>(s.ctl);
  if (A) k_rows_prep<<<std::min((A + 255) / 256, 4u * (uint32_t)sm_count()), 256, 0, stream>>>(
             s.ctl, r.mult, A, r.lit, permute ? r.xlit : nullptr, cond);
  if (N) {
    k_rows_mult<<<(N + 255) / 256, 256, 0, stream>>>(v.soma_to_axon, N, A, r.mult, r.mask2, s.ctl, cond);
    k_rows_build<<<(N + 31) / 32, 256, 0, stream>>>(v.dendrite_targets, v.dendrite_weights, v.soma_flags, N, r.rt,
                                                    r.rw, r.cnt, r.amask, r.omask, r.lfz, s.ctl, A,
                                                    row_sum ? 1u : 0u, permute ? 1u : 0u,
                                                    permute ? r.xlit : nullptr, permute ? r.lsum : nullptr,
                                                    with_posmap ? r.posmap : nullptr, cond);
  }
  return cudaGetLastError();
}

// Largest fully-lit bitmap the update kernel stages in shared memory (the
// 1024-thread variant also uses ~3.4 KB of static shared memory).
static size_t lit_smem_limit() {
  static size_t limit = [] {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    size_t lim = optin > 8192 ? (size_t)optin - 8192 : 0;
    if (cudaFuncSetAttribute(k_rows_update<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_rows_update<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_rows_update<true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)lim) != cudaSuccess) {
      cudaGetLastError();
      lim = 0;
    }
    return lim;
  }();
  return limit;
}

// The update pass (with the fully-lit bitmap in shared memory when it fits).
// lc: the learned engine's control block (the pass returns at once on its
// sparse ticks), or null.
static bool rows_lit(uint32_t A) { return (size_t)lit_smem_bytes(A) <= lit_smem_limit(); }

// inline: GSOP inside the pass (rows with their movable slots first), else
// the spikers are listed for launch_rows_gsop.
// pdl: launched into the tick's kernel chain (launch_chain).
template <bool INLINE>
static void launch_rows_update(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, uint32_t A, uint32_t k,
                               uint32_t fix_cap, const LearnCtl* lc, cudaStream_t stream, ColWT wt = ColWT{},
                               bool pdl = false) {
  RowCache& r = *s.rows;
  const int sms = sm_count();
  const bool lit = rows_lit(A);
  const dim3 grid(lit ? sms : 4 * sms), block(lit ? 1024 : 256);
  const size_t smem = lit ? lit_smem_bytes(A) : 0;
  auto go = [&](auto kern) {
    launch_chain(kern, grid, block, smem, stream, pdl, v, N, A, r.rt, r.rw, r.cnt, r.mask2, r.eval, s.pend, r.fix,
                 s.ctl, k, fix_cap, r.lit, lc, r.gs_n, r.gd_n, r.lfz, r.wcnt, wt);
  };
  if constexpr (INLINE) {
    if (wt.w) {   // the per-tick entry point: weight changes written through
      if (lit)
        go(k_rows_update<true, true, true>);
      else
        go(k_rows_update<false, true, true>);
      return;
    }
  }
  if (lit)
    go(k_rows_update<true, INLINE>);
  else
    go(k_rows_update<false, INLINE>);
}

// The GSOP passes over the spikers the tick's update pass listed (32 warps per
// SM, each with its slice of the evaluated list; a GSOP warp per slice).
static void launch_rows_gsop(const ShardVramPtrs& v, ShardScratch& s, uint32_t A, uint32_t k, uint32_t fix_cap,
                             cudaStream_t stream, const LearnCtl* lc = nullptr) {
  RowCache& r = *s.rows;
  const uint32_t nwu = (uint32_t)sm_count() * 32u;
  if (rows_lit(A)) {
    k_rows_gsop<true><<<nwu / 8, 256, 0, stream>>>(v, A, r.rt, r.rw, r.cnt, r.mask2, r.lit, r.amask, r.gs_n, r.wcnt,
                                                   nwu, r.fix, s.ctl, k, fix_cap, lc);
    k_rows_gsop_rows<true><<<nwu / 8, 256, 0, stream>>>(v, A, r.rt, r.rw, r.cnt, r.mask2, r.lit, r.gd_n,
                                                        r.wcnt + kMaxUpdateWarps, nwu, r.fix, s.ctl, k, fix_cap, lc);
  } else {
    k_rows_gsop<false><<<nwu / 8, 256, 0, stream>>>(v, A, r.rt, r.rw, r.cnt, r.mask2, r.lit, r.amask, r.gs_n, r.wcnt,
                                                    nwu, r.fix, s.ctl, k, fix_cap, lc);
    k_rows_gsop_rows<false><<<nwu / 8, 256, 0, stream>>>(v, A, r.rt, r.rw, r.cnt, r.mask2, r.lit, r.gd_n,
                                                         r.wcnt + kMaxUpdateWarps, nwu, r.fix, s.ctl, k, fix_cap, lc);
  }
}

// One tick of the row engine: prologue, update (+GSOP), fix-up, push.  In a
// batch (a.batch) the tick number, dopamine and network spike count come from
// the control block and the soma pushes may be deferred to the next tick's
// prologue; a per-tick call (cu_step_day_phase) passes them to the prologue,
// applies its pushes before it returns, and writes GSOP's weight changes
// through to the columnar blob (its row cache outlives the call).  ev
// (optional) gets the stage boundaries 2..5 recorded: after the prologue,
// after the 8-lane pass, after the lit-sum pass, after fix-up and push (GSOP
// is part of the update passes).
cudaError_t launch_tick_rows(const ShardVramPtrs& v, ShardScratch& s, const TickArgs& a, cudaStream_t stream,
                             cudaEvent_t* ev, bool have_incoming) {
  RowCache& r = *s.rows;
  const uint32_t N = a.padded_n, A = a.total_axons;
  const int sms = sm_count();
  const uint32_t* bitmask = (a.num_virtual > 0) ? a.input_bitmask : nullptr;
  uint32_t raise = 0;
  if (bitmask && ((uint64_t)a.virtual_offset + a.num_virtual > A)) raise |= AXC_ERR_VIRTUAL_RANGE;
  const uint32_t G = max(A, N);
  const bool per_tick = !a.batch;
  // The per-tick entry point launches the kernels after the prologue into the
  // kernel chain (launch_chain), which overlaps each stream launch with the
  // kernel before it: 4,841 against 4,617 calls/s at 1.5M neurons.  A batch's
  // captured graph gains nothing from it (16,955 against 17,073 ticks/s) and
  // keeps plain edges.  Never while stage events are recorded.
  const bool pdl = per_tick && ev == nullptr;
  if (G) {
    const bool wide = (G + 255) / 256 >= kProWide;
    launch_chain(wide ? k_rows_prologue_plain<2> : k_rows_prologue_plain<1>,
                 dim3(wide ? (G + 511) / 512 : (G + 255) / 256), dim3(256), 0, stream, false, v.axon_heads, A,
                 a.v_seg, bitmask, a.virtual_offset, a.num_virtual, s.incoming,
                 (have_incoming && !per_tick) ? s.batch_counts : nullptr, a.k, r.mask2, r.mult, v.soma_flags,
                 v.timers, N, r.eval, s.ctl, raise, r.lit, (a.k > 0 && !per_tick) ? s.pend : nullptr,
                 (have_incoming && per_tick) ? 1u : 0u, per_tick ? 1u : 0u, a.tick - a.k, (int32_t)a.dopamine,
                 r.xlit);
  }
  if (ev) cudaEventRecord(ev[2], stream);
  ColWT wt{};
  if (per_tick) {
    wt.w = v.dendrite_weights;
    wt.om = r.omask;
    wt.cnt = r.cnt;
    wt.N = N;
  }
  // stages: ev[2]..ev[3] the 8-lane pass, ev[3]..ev[4] the lit-sum pass (both
  // with GSOP; both are launched and each returns at once on the other's
  // ticks), ev[4]..ev[5] fix-up and push.
  const uint32_t fix_cap = min(a.fix_cap, kFixCap);
  launch_rows_update<true>(v, s, N, A, a.k, fix_cap, nullptr, stream, wt, pdl && G);
  if (ev) cudaEventRecord(ev[3], stream);
  launch_chain(per_tick ? k_rows_update_lsum<true> : k_rows_update_lsum<false>, dim3(kLsumBlocks * sms), dim3(256),
               0, stream, pdl, v, A, r.rt, r.rw, r.cnt, r.mask2, r.eval, s.pend, r.fix, s.ctl, a.k, fix_cap, r.lit,
               r.lfz, r.lsum, wt, (const LearnCtl*)nullptr);
  if (ev) cudaEventRecord(ev[4], stream);
  const bool readout = a.num_outputs > 0 && a.mapped_soma_ids && a.output_history;
  launch_chain(k_rows_fixup, dim3(2 * sms), dim3(256), 0, stream, pdl, v, N, A, r.rt, r.rw, r.cnt, r.mask2, s.pend,
               r.eval, r.fix, s.ctl, a.k, a.mapped_soma_ids, a.output_history, readout ? a.num_outputs : 0, wt);
  // the soma pushes: by the next tick's prologue within a batch, here on its last tick
  if (!a.defer_push)
    launch_chain(k_rows_push, dim3(8 * sms), dim3(256), 0, stream, pdl, v.axon_heads, v.soma_to_axon, A, s.pend,
                 r.eval, v.soma_flags, N, (const uint32_t*)nullptr, (uint8_t*)nullptr, 0u, s.ctl, a.k);
  if (ev) cudaEventRecord(ev[5], stream);
  return cudaGetLastError();
}

cudaError_t launch_rows_end(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, cudaStream_t stream) {
  RowCache& r = *s.rows;
  if (N) k_rows_writeback<<<(N + 255) / 256, 256, 0, stream>>>(v.dendrite_weights, N, r.rw, r.omask);
  return cudaGetLastError();
}

}  // namespace axc
