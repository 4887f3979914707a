/*
 * day_phase_oracle.c — CPU restatement of the reference Day Phase.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the CUDA engine is
 * compared against (tests, smoke check, and the timed CPU baseline of the
 * benchmark).  The engine never calls it.
 *
 * It restates, element by element and in plain C, the kernels of
 * genesis-compute/src/cuda/physics.cu and the side kernels of
 * genesis-compute/src/cuda/bindings.cu.  Every function cites the
 * reference lines it follows.  Integer semantics are those of the GPU:
 * 32-bit products and sums wrap (done here in uint32_t), `>>` on a negative
 * int32_t is arithmetic (gcc), u8/i16 stores truncate.
 *
 * One deliberate difference from the reference: snapshot semantics for the
 * soma pushes of a tick.  cu_update_neurons_kernel (physics.cu:159-276)
 * reads other neurons' axon heads (physics.cu:194) while spiking neurons
 * push their own heads in the same kernel (physics.cu:257-261), so which
 * value a reader sees depends on the schedule.  Here every read in the
 * update stage sees the heads as left by PropagateAxons, and the pushes are
 * applied after the whole update stage, before GSOP (which, in the
 * reference, runs in a later kernel and so sees all pushes).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "../include/axicor_day.h"

#define ORC_LUT_SIZE 16

/* ------------------------------------------------------------------ */
/* wrapping helpers (two's complement, as the GPU computes)            */
/* ------------------------------------------------------------------ */
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

static inline uint32_t h_get(const BurstHeads8* h, int k) { return ((const uint32_t*)h)[k]; }

/* physics.cu:32-41 — shift h0..h6 into h1..h7, new head 0. */
void orc_push_burst_head(BurstHeads8* h) {
  h->h7 = h->h6; h->h6 = h->h5; h->h5 = h->h4; h->h4 = h->h3;
  h->h3 = h->h2; h->h2 = h->h1; h->h1 = h->h0; h->h0 = 0;
}

/* physics.cu:198-201 — a dendrite segment is hit when any head h satisfies
 * (u32)(h - seg) < prop (genesis-core/src/signal.rs:22-25). */
int orc_segment_hit(const BurstHeads8* h, uint32_t seg, uint32_t prop) {
  int hit = 0;
  for (int k = 0; k < 8; k++) hit |= (uint32_t)(h_get(h, k) - seg) < prop;
  return hit;
}

/* physics.cu:311-318 — smallest in-tail distance, 0xFFFFFFFF when none. */
uint32_t orc_min_dist(const BurstHeads8* h, uint32_t seg, uint32_t prop) {
  uint32_t md = 0xFFFFFFFFu;
  for (int k = 0; k < 8; k++) {
    uint32_t d = h_get(h, k) - seg;
    uint32_t c = (d < prop) ? d : 0xFFFFFFFFu;
    if (c < md) md = c;
  }
  return md;
}

/* physics.cu:25-30 */
void orc_reset_burst_counters(uint8_t* flags, uint32_t padded_n) {
  for (uint32_t i = 0; i < padded_n; i++) flags[i] &= 0xF1;
}

/* physics.cu:88-108.  Returns AXC_ERR_VIRTUAL_RANGE when a set bit would push
 * past total_axons (the reference writes out of bounds there). */
uint32_t orc_inject_inputs(BurstHeads8* heads, uint32_t total_axons, const uint32_t* bitmask,
                           uint32_t virtual_offset, uint32_t num_virtual) {
  uint32_t err = 0;
  for (uint32_t v = 0; v < num_virtual; v++) {
    if ((bitmask[v / 32] >> (v % 32)) & 1u) {
      uint32_t a = virtual_offset + v;
      if (a >= total_axons || a < virtual_offset) { err |= AXC_ERR_VIRTUAL_RANGE; continue; }
      orc_push_burst_head(&heads[a]);
    }
  }
  return err;
}

/* physics.cu:114-132.  Ids >= total_axons are ignored (physics.cu:127).
 * Duplicate ids race in the reference; here each occurrence is one push. */
void orc_apply_spike_batch(BurstHeads8* heads, const uint32_t* ids, uint32_t count,
                           uint32_t total_axons) {
  for (uint32_t i = 0; i < count; i++)
    if (ids[i] < total_axons) orc_push_burst_head(&heads[ids[i]]);
}

/* physics.cu:137-154 */
void orc_propagate_axons(BurstHeads8* heads, uint32_t total_axons, uint32_t v_seg, int threads) {
#pragma omp parallel for schedule(static) num_threads(threads)
  for (int64_t a = 0; a < (int64_t)total_axons; a++) {
    uint32_t* h = (uint32_t*)&heads[a];
    for (int k = 0; k < 8; k++)
      if (h[k] != AXC_AXON_SENTINEL) h[k] += v_seg;
  }
}

/* physics.cu:159-276, one neuron.  Returns 1 when the neuron spiked (GLIF or
 * heartbeat).  Reads heads only (the caller applies the push afterwards).
 * *evaluated / *hits count the slots scanned and the slots that added a
 * weight (statistics only, not part of the reference). */
static int orc_update_one(const ShardVramPtrs* s, const VariantParameters* lut, uint32_t n,
                          uint32_t padded_n, uint32_t total_axons, uint32_t current_tick,
                          uint32_t* err, uint64_t* evaluated, uint64_t* hits) {
  uint8_t flags = s->soma_flags[n];
  uint8_t timer = s->timers[n];
  flags &= (uint8_t)~0x01;                                   /* :168 */
  if (timer > 0) {                                           /* :170-174 */
    s->timers[n] = (uint8_t)(timer - 1);
    s->soma_flags[n] = flags;
    return 0;
  }
  const VariantParameters* p = &lut[(flags >> 4) & 0x0F];    /* :176-177 */
  int32_t v = s->soma_voltage[n];
  int32_t i_in = 0;
  uint32_t prop = p->signal_propagation_length;
  for (uint32_t i = 0; i < AXC_MAX_DENDRITES; i++) {         /* :182-206 */
    uint64_t col = (uint64_t)i * padded_n + n;
    uint32_t t = s->dendrite_targets[col];
    if (t == 0) break;
    (*evaluated)++;
    uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
    uint32_t seg = t >> AXC_TARGET_SEG_SHIFT;
    if (a >= total_axons) { *err |= AXC_ERR_TARGET_RANGE; continue; }
    if (orc_segment_hit(&s->axon_heads[a], seg, prop)) {
      i_in = wadd(i_in, (int32_t)s->dendrite_weights[col]);
      (*hits)++;
    }
  }
  int32_t thr = s->threshold_offset[n];                      /* :209-213 */
  int32_t decayed = wsub(thr, (int32_t)p->homeostasis_decay);
  thr = decayed & ~(decayed >> 31);

  int32_t leak = p->leak_rate;                               /* :216-223 */
  if (p->adaptive_mode == 1) {
    int32_t add = wmul(thr, (int32_t)p->adaptive_leak_gain) >> 8;
    leak = wadd(leak, add);
    int32_t over = wsub(leak, p->adaptive_leak_max);
    leak = wsub(leak, over & ~(over >> 31));
  }

  v = wadd(v, i_in);                                         /* :225-235 */
  int32_t diff = wsub(v, p->rest_potential);
  int32_t sign = (diff > 0) - (diff < 0);
  int32_t abs_diff = wmul(diff, sign);
  int32_t leaked = wsub(abs_diff, leak);
  leaked = leaked & ~(leaked >> 31);
  v = wadd(p->rest_potential, wmul(sign, leaked));

  int32_t eff = wadd(p->threshold, thr);                     /* :237-245 */
  int32_t glif = (v >= eff) ? 1 : 0;
  uint32_t period = p->spontaneous_firing_period_ticks;
  int32_t hb = (period > 0 && ((current_tick + (n * 104729u)) % period) == 0) ? 1 : 0;
  int32_t spike = glif | hb;

  if (glif) v = p->rest_potential;                           /* :248-250 */
  thr = wadd(thr, wmul(glif, p->homeostasis_penalty));
  uint8_t new_timer = glif ? p->refractory_period : s->timers[n];

  if (spike) flags = (uint8_t)((flags & 0xFC) | 0x03);       /* :253-266 */
  else flags = (uint8_t)(flags & ~0x01);

  s->soma_voltage[n] = v;                                    /* :269-275 */
  uint8_t burst = (flags >> 1) & 0x07;
  burst = (uint8_t)(burst + (spike && burst < 7));
  s->soma_flags[n] = (uint8_t)((flags & 0xF0) | (burst << 1) | (uint8_t)spike);
  s->threshold_offset[n] = thr;
  s->timers[n] = new_timer;
  return spike;
}

/* physics.cu:159-276 over all neurons with snapshot semantics, then the
 * deferred soma pushes (physics.cu:257-261) in neuron order.
 * spiked (optional, padded_n bytes) receives 1 for each spiking neuron. */
uint32_t orc_update_neurons(const ShardVramPtrs* s, const VariantParameters* lut, uint32_t padded_n,
                            uint32_t total_axons, uint32_t current_tick, uint8_t* spiked,
                            uint64_t* stats, int threads) {
  uint8_t* sp = spiked ? spiked : (uint8_t*)malloc(padded_n ? padded_n : 1);
  uint32_t err = 0;
  uint64_t ev = 0, hi = 0;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) reduction(| : err) reduction(+ : ev, hi)
  for (int64_t n = 0; n < (int64_t)padded_n; n++) {
    uint32_t e = 0;
    uint64_t a = 0, b = 0;
    sp[n] = (uint8_t)orc_update_one(s, lut, (uint32_t)n, padded_n, total_axons, current_tick, &e, &a, &b);
    err |= e; ev += a; hi += b;
  }
  uint64_t nsp = 0;
  for (uint32_t n = 0; n < padded_n; n++) {
    if (!sp[n]) continue;
    nsp++;
    uint32_t my_axon = s->soma_to_axon[n];
    if (my_axon == AXC_NO_AXON) continue;
    if (my_axon >= total_axons) { err |= AXC_ERR_SOMA_AXON; continue; }
    orc_push_burst_head(&s->axon_heads[my_axon]);
  }
  if (stats) { stats[0] += ev; stats[1] += hi; stats[2] += nsp; }
  if (!spiked) free(sp);
  return err;
}

/* physics.cu:281-373, one neuron. Returns the number of slots updated. */
static uint32_t orc_gsop_one(const ShardVramPtrs* s, const VariantParameters* lut, uint32_t n,
                             uint32_t padded_n, uint32_t total_axons, int16_t dopamine, uint32_t* err) {
  uint8_t flags = s->soma_flags[n];
  if ((flags & 0x01) == 0) return 0;                         /* :286-287 */
  uint8_t burst = (flags >> 1) & 0x07;                       /* :290-291 */
  int32_t burst_mult = burst > 0 ? burst : 1;
  const VariantParameters* p = &lut[(flags >> 4) & 0x0F];
  uint32_t done = 0;
  for (uint32_t i = 0; i < AXC_MAX_DENDRITES; i++) {         /* :296-372 */
    uint64_t col = (uint64_t)i * padded_n + n;
    uint32_t t = s->dendrite_targets[col];
    if (t == 0) break;
    uint32_t a = (t & AXC_TARGET_AXON_MASK) - 1u;
    uint32_t seg = t >> AXC_TARGET_SEG_SHIFT;
    if (a >= total_axons) { *err |= AXC_ERR_TARGET_RANGE; continue; }
    uint32_t md = orc_min_dist(&s->axon_heads[a], seg, p->signal_propagation_length);
    int is_active = md != 0xFFFFFFFFu;

    int16_t w = s->dendrite_weights[col];                    /* :322-332 */
    int32_t sign = (w >= 0) ? 1 : -1;
    int32_t abs_w = (int32_t)w;
    if (abs_w < 0) abs_w = -abs_w;
    uint32_t rank = (uint32_t)abs_w >> 11;
    if (rank > 15) rank = 15;
    int32_t inertia = p->inertia_curve[rank];

    int32_t pot_mod = wmul((int32_t)dopamine, (int32_t)p->d1_affinity) >> 7;   /* :336-345 */
    int32_t dep_mod = wmul((int32_t)dopamine, (int32_t)p->d2_affinity) >> 7;
    int32_t raw_pot = wadd((int32_t)p->gsop_potentiation, pot_mod);
    int32_t raw_dep = wsub((int32_t)p->gsop_depression, dep_mod);
    int32_t final_dep = raw_dep & ~(raw_dep >> 31);

    int32_t delta_pot = wmul(wmul(raw_pot, inertia), burst_mult) >> 7;        /* :348-358 */
    int32_t delta_dep = wmul(wmul(final_dep, inertia), burst_mult) >> 7;
    uint32_t cs = is_active ? (md >> 4) : 0;
    int32_t delta = is_active ? (delta_pot >> cs) : wsub(0, delta_dep);
    delta = wmul(delta, 128) >> (7 + cs);

    int32_t new_abs = wadd(abs_w, delta);                   /* :361-371 */
    new_abs = new_abs & ~(new_abs >> 31);
    if (new_abs > 32767) new_abs = 32767;
    s->dendrite_weights[col] = (int16_t)wmul(new_abs, sign);
    done++;
  }
  return done;
}

/* physics.cu:281-373 over all neurons. */
uint32_t orc_apply_gsop(const ShardVramPtrs* s, const VariantParameters* lut, uint32_t padded_n,
                        uint32_t total_axons, int16_t dopamine, uint64_t* stats, int threads) {
  uint32_t err = 0;
  uint64_t done = 0;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) reduction(| : err) reduction(+ : done)
  for (int64_t n = 0; n < (int64_t)padded_n; n++) {
    uint32_t e = 0;
    done += orc_gsop_one(s, lut, (uint32_t)n, padded_n, total_axons, dopamine, &e);
    err |= e;
  }
  if (stats) stats[3] += done;
  return err;
}

/* physics.cu:378-395.  Ids >= padded_n (other than the sentinel) read out of
 * bounds in the reference; here they give 0 and AXC_ERR_READOUT_RANGE. */
uint32_t orc_record_readout(const uint8_t* flags, uint32_t padded_n, const uint32_t* ids,
                            uint8_t* out, uint32_t num_outputs) {
  uint32_t err = 0;
  for (uint32_t k = 0; k < num_outputs; k++) {
    uint32_t id = ids[k];
    uint8_t v = 0;
    if (id != AXC_NO_AXON) {
      if (id < padded_n) v = flags[id] & 0x01;
      else err |= AXC_ERR_READOUT_RANGE;
    }
    out[k] = v;
  }
  return err;
}

/* physics.cu:400-434.  The reference's warp order depends on atomics; the
 * restatement lists spiking ids in ascending order. Returns the count. */
uint32_t orc_extract_telemetry(const uint8_t* flags, uint32_t padded_n, uint32_t* out_ids) {
  uint32_t c = 0;
  for (uint32_t n = 0; n < padded_n; n++)
    if (flags[n] & 0x01) { if (out_ids) out_ids[c] = n; c++; }
  return c;
}

/* physics.cu:441-495: R, I, S, P, U (+ deferred pushes), G, O.
 * stats (optional, 4 x u64): evaluated slots, hits, spikes, GSOP slots.
 * Returns the AXC_ERR_* bits raised. */
uint32_t orc_step_day_phase(const ShardVramPtrs* s, const VariantParameters* lut,
                            uint32_t padded_n, uint32_t total_axons, uint32_t v_seg,
                            uint32_t current_tick, const uint32_t* input_bitmask,
                            uint32_t virtual_offset, uint32_t num_virtual_axons,
                            const uint32_t* incoming_spikes, uint32_t num_incoming_spikes,
                            const uint32_t* mapped_soma_ids, uint8_t* output_history,
                            uint32_t num_outputs, int16_t dopamine, uint64_t* stats, int threads) {
  uint32_t err = 0;
  if (threads <= 0) threads = omp_get_max_threads();
  orc_reset_burst_counters(s->soma_flags, padded_n);                              /* :458 */
  if (num_virtual_axons > 0 && input_bitmask)                                      /* :461-465 */
    err |= orc_inject_inputs(s->axon_heads, total_axons, input_bitmask, virtual_offset,
                             num_virtual_axons);
  if (num_incoming_spikes > 0 && incoming_spikes)                                  /* :468-472 */
    orc_apply_spike_batch(s->axon_heads, incoming_spikes, num_incoming_spikes, total_axons);
  orc_propagate_axons(s->axon_heads, total_axons, v_seg, threads);                 /* :475-477 */
  err |= orc_update_neurons(s, lut, padded_n, total_axons, current_tick, NULL, stats, threads); /* :480 */
  err |= orc_apply_gsop(s, lut, padded_n, total_axons, dopamine, stats, threads);  /* :484 */
  if (num_outputs > 0 && mapped_soma_ids && output_history)                        /* :487-492 */
    err |= orc_record_readout(s->soma_flags, padded_n, mapped_soma_ids, output_history, num_outputs);
  return err;
}

/* ------------------------------------------------------------------ */
/* Side kernels of bindings.cu                                          */
/* ------------------------------------------------------------------ */

/* bindings.cu:341-368 */
void orc_ghost_sync(const BurstHeads8* src, BurstHeads8* dst, const uint32_t* src_idx,
                    const uint32_t* dst_idx, uint32_t count) {
  for (uint32_t i = 0; i < count; i++)
    if (src_idx[i] < 0x80000000u) dst[dst_idx[i]] = src[src_idx[i]];
}

/* bindings.cu:378-436.  Events are listed in (index, head) order; the
 * reference's order follows its atomics.  Returns the event count. */
uint32_t orc_extract_outgoing_spikes(const BurstHeads8* heads, const uint32_t* src_idx,
                                     const uint32_t* dst_ghost, uint32_t count,
                                     uint32_t sync_batch_ticks, uint32_t v_seg,
                                     SpikeEvent* out, uint32_t capacity) {
  uint32_t c = 0;
  for (uint32_t i = 0; i < count; i++) {
    uint32_t a = src_idx[i];
    if (a >= 0x80000000u) continue;
    for (int k = 0; k < 8; k++) {
      uint32_t h = h_get(&heads[a], k);
      if (h >= 0x70000000u) continue;
      uint32_t ticks_since = h / v_seg;
      if (ticks_since < sync_batch_ticks) {
        if (c < capacity) {
          out[c].ghost_id = dst_ghost[i];
          out[c].tick_offset = sync_batch_ticks - 1 - ticks_since;
        }
        c++;
      }
    }
  }
  return c;
}

/* bindings.cu:450-515, one neuron per call of the inner body: clear burst
 * bits, stable insertion sort of the 128 slots by |weight| descending with
 * empty targets sinking, then zero every slot with |w| < threshold. */
void orc_sort_and_prune(const ShardVramPtrs* s, uint32_t padded_n, int16_t prune_threshold,
                        int threads) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
  for (int64_t nn = 0; nn < (int64_t)padded_n; nn++) {
    uint32_t n = (uint32_t)nn;
    s->soma_flags[n] &= 0xF1;                                              /* :456-458 */
    uint32_t tg[AXC_MAX_DENDRITES];
    int16_t wt[AXC_MAX_DENDRITES];
    uint8_t tm[AXC_MAX_DENDRITES];
    for (uint32_t i = 0; i < AXC_MAX_DENDRITES; i++) {                      /* :469-475 */
      uint64_t col = (uint64_t)i * padded_n + n;
      tg[i] = s->dendrite_targets[col];
      wt[i] = s->dendrite_weights[col];
      tm[i] = s->dendrite_timers[col];
    }
    for (int i = 1; i < (int)AXC_MAX_DENDRITES; i++) {                      /* :478-495 */
      uint32_t kt = tg[i];
      int16_t kw = wt[i];
      uint8_t km = tm[i];
      if (kt == 0) continue;
      int32_t kabs = kw >= 0 ? kw : -kw;
      int j = i - 1;
      while (j >= 0) {
        int32_t pabs = wt[j] >= 0 ? wt[j] : -wt[j];
        if (tg[j] != 0 && pabs >= kabs) break;
        tg[j + 1] = tg[j]; wt[j + 1] = wt[j]; tm[j + 1] = tm[j];
        j--;
      }
      tg[j + 1] = kt; wt[j + 1] = kw; tm[j + 1] = km;
    }
    for (uint32_t i = 0; i < AXC_MAX_DENDRITES; i++) {                      /* :498-506 */
      int32_t a = wt[i] >= 0 ? wt[i] : -wt[i];
      if (tg[i] != 0 && a < prune_threshold) { tg[i] = 0; wt[i] = 0; tm[i] = 0; }
    }
    for (uint32_t i = 0; i < AXC_MAX_DENDRITES; i++) {                      /* :510-514 */
      uint64_t col = (uint64_t)i * padded_n + n;
      s->dendrite_targets[col] = tg[i];
      s->dendrite_weights[col] = wt[i];
      s->dendrite_timers[col] = tm[i];
    }
  }
}

/* bindings.cu:560-568 */
void orc_init_sentinels(BurstHeads8* heads, uint32_t total_axons) {
  for (uint32_t a = 0; a < total_axons; a++) {
    uint32_t* h = (uint32_t*)&heads[a];
    for (int k = 0; k < 8; k++) h[k] = AXC_AXON_SENTINEL;
  }
}

/* genesis-compute/src/memory.rs:71-86 — slices a host .state blob into the
 * ShardVramPtrs fields (host pointers). */
void orc_slice_state(void* blob, uint32_t padded_n, BurstHeads8* heads, ShardVramPtrs* out) {
  uint8_t* b = (uint8_t*)blob;
  size_t n = padded_n, off = 0;
  out->soma_voltage = (int32_t*)(b + off); off += n * 4;
  out->soma_flags = (uint8_t*)(b + off); off += n;
  out->threshold_offset = (int32_t*)(b + off); off += n * 4;
  out->timers = (uint8_t*)(b + off); off += n;
  out->soma_to_axon = (uint32_t*)(b + off); off += n * 4;
  out->dendrite_targets = (uint32_t*)(b + off); off += n * AXC_MAX_DENDRITES * 4;
  out->dendrite_weights = (int16_t*)(b + off); off += n * AXC_MAX_DENDRITES * 2;
  out->dendrite_timers = (uint8_t*)(b + off);
  out->axon_heads = heads;
}

/* Runs `ticks` ticks of the batch loop of genesis-compute/src/compute/shard.rs:40-124
 * (burst reset once, then one step per tick with global tick = tick_base + k)
 * over a host blob.  input_bitmask holds words_per_tick words per tick (or is
 * NULL); outputs (optional) receive num_outputs bytes per tick; spike_raster
 * (optional) receives padded_n/8 bytes per tick, bit n%8 of byte n/8 = spike. */
uint32_t orc_run_ticks(void* state_blob, BurstHeads8* heads, const VariantParameters* lut,
                       uint32_t padded_n, uint32_t total_axons, uint32_t v_seg,
                       uint32_t tick_base, uint32_t ticks, const uint32_t* input_bitmask,
                       uint32_t words_per_tick, uint32_t virtual_offset, uint32_t num_virtual,
                       const uint32_t* mapped_soma_ids, uint8_t* outputs, uint32_t num_outputs,
                       int16_t dopamine, uint8_t* spike_raster, uint64_t* stats, int threads) {
  ShardVramPtrs s;
  orc_slice_state(state_blob, padded_n, heads, &s);
  if (threads <= 0) threads = omp_get_max_threads();
  uint32_t err = 0;
  orc_reset_burst_counters(s.soma_flags, padded_n);
  for (uint32_t k = 0; k < ticks; k++) {
    const uint32_t* bm = input_bitmask ? input_bitmask + (size_t)k * words_per_tick : NULL;
    uint8_t* out = outputs ? outputs + (size_t)k * num_outputs : NULL;
    err |= orc_step_day_phase(&s, lut, padded_n, total_axons, v_seg, tick_base + k, bm,
                              virtual_offset, num_virtual, NULL, 0, mapped_soma_ids, out,
                              num_outputs, dopamine, stats, threads);
    if (spike_raster) {
      uint8_t* r = spike_raster + (size_t)k * ((padded_n + 7) / 8);
      memset(r, 0, (padded_n + 7) / 8);
      for (uint32_t n = 0; n < padded_n; n++)
        if (s.soma_flags[n] & 1) r[n / 8] |= (uint8_t)(1u << (n % 8));
    }
  }
  return err;
}
