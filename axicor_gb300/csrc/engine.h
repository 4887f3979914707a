// engine.h — internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <tuple>
#include <type_traits>
#include <utility>

#include "../../include/axicor_day.h"

namespace axc {

// Launches kernel k and returns the status of that launch alone
// (cudaLaunchKernel's return value), without reading or clearing an error
// that an earlier call left pending.  Arguments convert to the kernel's
// parameter types.
template <typename... P, typename... A, size_t... I>
cudaError_t launch_k_impl(void (*k)(P...), dim3 g, dim3 b, cudaStream_t s, std::index_sequence<I...>, A&&... a) {
  std::tuple<std::decay_t<P>...> t(static_cast<std::decay_t<P>>(std::forward<A>(a))...);
  void* args[sizeof...(P) > 0 ? sizeof...(P) : 1] = {static_cast<void*>(&std::get<I>(t))...};
  return cudaLaunchKernel(reinterpret_cast<const void*>(k), g, b, args, 0, s);
}
template <typename... P, typename... A>
cudaError_t launch_k(void (*k)(P...), dim3 g, dim3 b, cudaStream_t s, A&&... a) {
  static_assert(sizeof...(P) == sizeof...(A), "one argument per kernel parameter");
  return launch_k_impl(k, g, b, s, std::index_sequence_for<P...>{}, std::forward<A>(a)...);
}

// Control block of one shard in device memory.
struct ShardCtl {
  uint32_t spike_count;   // spikers listed by the last update stage
  uint32_t err;           // AXC_ERR_* bits, sticky until read with clear
  uint32_t tick_base;     // batch mode: global tick of tick 0 of the batch
  int32_t dopamine;       // batch mode: dopamine of the batch
  uint32_t fix_count;     // row engine: GSOP slots deferred to the fix-up stage
  uint32_t fix_overflow;  // row engine: the fix-up list overflowed, rescan the spikers
  uint32_t eval_count[2]; // row engine: non-refractory neurons listed in tick k (slot k & 1)
  uint32_t row_smax;      // row engine: longest row (slots before the first empty) of the batch
  uint32_t seg_max;       // row engine: largest segment of a live slot in the batch
  unsigned long long row_sum;  // row engine: checksum of the batch's targets (slot order)
  uint32_t pmax;          // row engine: largest signal_propagation_length of the LUT (batch start)
  uint32_t pad2;
  unsigned long long ctr[8];  // statistics, see axc_shard_counters
  uint32_t dense[2];      // row engine: tick k (slot k & 1) has an axon off the lit set the row layout assumed
  unsigned long long pfx_total;   // row engine: slots outside the frozen lit-sum part of the rows (batch start)
  unsigned long long slot_total;  // row engine: live slots of the rows (batch start)
  uint32_t lay_now;       // row engine: this batch lays the row copy out anew (layout_decide)
  uint32_t lay_since;     // row engine: ticks since the last layout
  uint32_t lay_every;     // row engine: ticks between layouts while the lit-sum criterion holds
  uint32_t pad3;
};

// Neuron-major copy of the dendrites used by the batch engine for the length
// of one batch (row_engine.cuh).
struct RowCache {
  uint32_t N = 0, A = 0;
  void* base = nullptr;
  uint32_t* rt = nullptr;   // [N][128] targets, neuron-major
  int16_t* rw = nullptr;    // [N][128] weights, neuron-major
  uint16_t* cnt = nullptr;  // [N] slots before the first empty target; bit 15: an invalid target
  uint2* mask2 = nullptr;   // [A+1] split segment-hit masks (heads 0..6 | head 7); [A] dummy
  uint32_t* mult = nullptr; // [A] number of somas that own the axon
  uint32_t* eval = nullptr; // [N] non-refractory neurons of the tick
  uint32_t* fix = nullptr;  // [kFixCap] deferred GSOP slots (n*128 + slot)
  uint32_t* lit = nullptr;  // [A/32+1] fully-lit axons of the tick, one bit each
  uint32_t* gs_n = nullptr; // [N] spikers with 1..8 slots GSOP may move (a thread each)
  uint32_t* gd_n = nullptr; // [N] spikers with more (8 lanes each)
  uint4* amask = nullptr;   // [N] row positions (bit q) whose weights GSOP may move (set at batch start)
  uint8_t* lfz = nullptr;   // [N] number of those slots (set at batch start)
  uint4* omask = nullptr;   // [N] columnar slots placed first in the row (the movable ones; all when unpermuted)
  uint32_t* wcnt = nullptr; // [2][kMaxUpdateWarps] spikers each warp of the update pass listed (gs_n, gd_n)
  int2* lsum = nullptr;     // [N] x: wrapping sum of the row's lit-sum weights, y: row positions before them
  uint32_t* xlit = nullptr; // [A/32+1] axons taken as fully lit when the row layout was made
  uint8_t* posmap = nullptr;  // [N][128] row position of each columnar slot (learned engine only; own allocation)
};

// Per-shard scratch owned by the engine, next to the reference-visible
// state.  Sized for (padded_n, total_axons).
struct ShardScratch {
  uint32_t padded_n = 0;
  uint32_t total_axons = 0;
  void* base = nullptr;        // single allocation
  uint32_t* seg_mask = nullptr;  // [A] segment-hit mask of the propagated heads
  uint32_t* pend = nullptr;      // [A] soma pushes pending for the push stage
  uint32_t* incoming = nullptr;  // [A] network spike pushes pending for the axon stage
  uint32_t* spikers = nullptr;   // [N] ids of the neurons that spiked this tick
  ShardCtl* ctl = nullptr;
  uint32_t* batch_counts = nullptr;  // [batch_cap] per-tick network spike counts
  uint32_t batch_cap = 0;
  uint32_t* h_counts_pinned = nullptr;  // pinned staging for batch_counts / tick_base
  void* graph_cache = nullptr;          // batch engine graphs (batch_engine.cu)
  RowCache* rows = nullptr;             // batch engine neuron-major dendrites
  // Per-tick entry point (cu_step_day_phase): its row cache lives across calls.
  // It is valid while nothing else wrote the shard's targets, weights, flags or
  // soma_to_axon and the LUT is the one it was built with; every entry point
  // of this library that writes them clears the flag.
  std::atomic<bool> tick_rows_valid{false};
  uint64_t tick_rows_lut = 0;           // LUT generation the per-tick row cache was built with
  uint32_t tick_parity = 0;             // per-tick calls alternate the row engine's list slots
  uint32_t tick_since_build = 0;        // per-tick calls since the row copy was laid out
  const void* state_base = nullptr;     // the shard's .state allocation (invalidation by address)
  size_t state_bytes = 0;
  // Batch path: the row copy (layout, weights, lit-sum sums) is kept from one
  // batch to the next while it matches the shard's memory and the LUT (the
  // device decides each batch whether to lay it out anew: layout_decide).
  // Cleared by every route that clears tick_rows_valid, and by the per-tick
  // entry point; the next batch then lays the rows out for sure.
  std::atomic<bool> batch_rows_valid{false};
  uint64_t batch_rows_lut = 0;           // LUT generation of the batch layout
};

constexpr uint32_t kBatchRelayoutMin = 100, kBatchRelayoutMax = 1600;   // ticks between batch layouts

uint64_t lut_generation();

// Whether the next batch must lay the row copy out anew whatever the device
// decides (the kept copy is stale or from another LUT); marks the copy the
// batch leaves as valid.
inline bool batch_rows_force(ShardScratch& s) {
  const uint64_t gen = lut_generation();
  const bool force = !(s.batch_rows_valid.load() && s.batch_rows_lut == gen);
  s.batch_rows_lut = gen;
  s.batch_rows_valid.store(true);
  return force;
}

#ifdef __CUDACC__
// The device's layout decision for the next `ticks` ticks of a batch (one
// thread, before the batch): a new layout when forced, while the current one
// misses the lit-sum criterion (at most an eighth of the live slots outside
// the lit-sum groups: the weights are still freezing, or the axons taken as
// fully lit were not yet), and otherwise every lay_every ticks, doubling from
// kBatchRelayoutMin to kBatchRelayoutMax.  The layout kernels of the batch
// return at once when lay_now is 0.
__device__ __forceinline__ void layout_decide(ShardCtl* c, uint32_t force, uint32_t ticks) {
  const bool met = c->slot_total > 0 && c->pfx_total * 8ull <= c->slot_total;
  const bool build = force || !met || c->lay_since >= c->lay_every;
  if (build) {
    const uint32_t twice = 2u * c->lay_every;
    c->lay_every = (force || !met || c->lay_every < kBatchRelayoutMin) ? kBatchRelayoutMin
                   : twice < kBatchRelayoutMax                          ? twice
                                                                        : kBatchRelayoutMax;
    c->lay_since = 0;
  }
  c->lay_since += ticks;
  c->lay_now = build ? 1u : 0u;
}
#endif

constexpr uint32_t kFixCap = 1u << 22;  // deferred GSOP slots per tick before the rescan path
constexpr uint32_t kMaxUpdateWarps = 32u * 1024u;  // warps of the update pass (32 per SM)

// Row engine (row_engine.cuh, compiled in day_phase.cu).  A (re)allocation
// drops the batch engine's captured graphs, which hold the old addresses; the
// new buffers are zeroed on `stream` (the legacy stream: zeroed before return).
cudaError_t rows_alloc(ShardScratch& s, uint32_t N, uint32_t A, bool with_fix, cudaStream_t stream);
void rows_free(ShardScratch& s);
// Allocates the row copy's position map (row position of every columnar slot),
// written by every later row copy of the shard that asks for it.
cudaError_t rows_posmap(ShardScratch& s, cudaStream_t stream);
// row_sum: also compute the targets checksum (ShardCtl::row_sum) the learned engine checks its index against;
// with_posmap: also write the position map (when it is allocated); conditional: the layout kernels lay
// the rows out only when the device's decision (ShardCtl::lay_now, layout_decide) says so, and
// otherwise keep the copy (only the per-tick lists are reset).
cudaError_t launch_rows_begin(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, uint32_t A, cudaStream_t stream,
                              bool row_sum = false, bool permute = true, bool with_posmap = true,
                              bool conditional = false);
cudaError_t launch_rows_end(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, cudaStream_t stream);

// Tries of the update pass's first wait for its staged bitmap; returns the previous value.
uint32_t set_first_wait_limit(uint32_t tries);

// Registry keyed by the axon_heads pointer.  Created by cu_allocate_shard;
// created lazily (and sized) for shards whose memory the caller allocated.
ShardScratch* scratch_for(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                          cudaError_t* err);
void scratch_release(const void* heads_key);
void graph_cache_free(ShardScratch* s);  // batch_engine.cu
void graph_cache_drop(ShardScratch* s);  // batch_engine.cu: destroys the captured graphs only
uint32_t fix_capacity();                 // batch_engine.cu: deferred-GSOP list capacity in use

// The row caches of a shard (per-tick and batch) no longer match its memory (shard_api.cu).
inline void rows_touched(ShardScratch& s) {
  s.tick_rows_valid.store(false);
  s.batch_rows_valid.store(false);
}
// Marks every shard whose .state allocation overlaps [dst, dst + size).
void invalidate_overlapping(const void* dst, size_t size);
// Looks up a shard's scratch without creating it (nullptr if none).
ShardScratch* scratch_find(const ShardVramPtrs* vram);

// Tick stages (day_phase.cu).  When dctl_batch is true the tick number,
// dopamine and network spike count come from the shard's device control
// block (tick = ctl->tick_base + k, count = batch_counts[k]).
struct TickArgs {
  uint32_t padded_n, total_axons, v_seg, tick;
  const uint32_t* input_bitmask;
  uint32_t virtual_offset, num_virtual;
  const uint32_t* incoming_spikes;
  uint32_t num_incoming;      // per-tick mode
  uint32_t max_incoming;      // batch mode: capacity of the tick's schedule row
  const uint32_t* mapped_soma_ids;
  uint8_t* output_history;
  uint32_t num_outputs;
  int16_t dopamine;
  bool batch;                 // read tick/dopamine/count from the device control block
  uint32_t k;                 // tick index inside the batch
  bool rows;                  // use the neuron-major row engine (batch mode only)
  uint32_t fix_cap;           // row engine: deferred-GSOP list capacity (<= kFixCap)
  bool defer_push;            // row engine: leave this tick's soma pushes to the next tick's prologue
                              // (never on the last tick of a batch)
};

// ev (optional): 6 events recorded around the stages (incoming, axons,
// update, push, gsop) for per-kernel timing.
constexpr int kTickStages = 5;
cudaError_t launch_tick(const ShardVramPtrs& v, ShardScratch& s, const TickArgs& a, cudaStream_t stream,
                        cudaEvent_t* ev = nullptr);
cudaError_t launch_reset_burst(const ShardVramPtrs& v, uint32_t padded_n, cudaStream_t stream);

// One shard's batch: the arguments of axc_step_day_phase_batch (batch_engine.cu).
struct BatchArgs {
  const ShardVramPtrs* vram;
  uint32_t padded_n, total_axons, ticks;
  const AxcIoBuffers* io;
  const uint32_t *h_bm, *h_in, *h_counts;
  uint32_t voff, nv;
  const uint32_t* ids;
  uint32_t v_seg;
  int16_t dopamine;
  uint32_t tick_base;
};
cudaError_t batch_prepare(const BatchArgs& b, ShardScratch** out_s, uint32_t* out_rows, cudaStream_t stream);
cudaError_t batch_capture(const BatchArgs& b, ShardScratch& s, uint32_t rows, uint32_t fix_cap, cudaStream_t cap);
// dst[dst_indices[i]] = src[src_indices[i]] for src_indices[i] < 2^31 (side_kernels.cu, bindings.cu:341-368).
cudaError_t ghost_sync(const BurstHeads8* src_heads, BurstHeads8* dst_heads, const uint32_t* src_indices,
                       const uint32_t* dst_indices, uint32_t count, cudaStream_t stream);
cudaError_t launch_spike_list_sorted(const ShardVramPtrs& v, uint32_t padded_n, uint32_t* out_ids,
                                     uint32_t* out_count, cudaStream_t stream);

// Stand-alone stages for the legacy per-kernel launchers (ffi.rs:193-233).
cudaError_t launch_push_incoming(BurstHeads8* heads, ShardScratch& s, uint32_t A, const uint32_t* ids,
                                 uint32_t count, cudaStream_t stream);
cudaError_t launch_propagate_only(BurstHeads8* heads, uint32_t A, uint32_t v_seg, cudaStream_t stream);
cudaError_t launch_update_stage(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, uint32_t A, uint32_t tick,
                                cudaStream_t stream);
cudaError_t launch_gsop_stage(const ShardVramPtrs& v, ShardScratch& s, uint32_t N, uint32_t A, int16_t dopamine,
                              cudaStream_t stream);

// LUT access for host code (day_phase.cu owns the __constant__ symbol).  Every
// upload advances the LUT generation.
cudaError_t lut_upload(const VariantParameters* lut, cudaStream_t stream, bool async);
uint64_t lut_generation();

int sm_count();

}  // namespace axc
