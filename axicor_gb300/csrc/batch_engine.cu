// batch_engine.cu — the host batch loop of ShardEngine::step_day_phase_batch
// (genesis-compute/src/compute/shard.rs:40-124) with the per-tick launches
// captured once into a CUDA graph and replayed for every later batch of the
// same shape.
//
// Per batch: bulk H2D of the inputs (shard.rs:54-68), burst-counter reset
// (shard.rs:71), then `batch` ticks with global tick = tick_base + k
// (shard.rs:75-120).  Values that change from batch to batch (tick_base,
// dopamine, the per-tick network spike counts) live in device memory that the
// captured kernels read, so one graph serves every batch.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <map>
#include <mutex>
#include <tuple>

#include "engine.h"

namespace axc {

namespace {

struct GraphKey {
  uint32_t N, A, batch, voff, nv, v_seg, max_spikes, words, num_outputs, rows, fix_cap;
  const void *bitmask, *incoming, *out, *ids;
  bool operator<(const GraphKey& o) const {
    return std::tie(N, A, batch, voff, nv, v_seg, max_spikes, words, num_outputs, rows, fix_cap, bitmask, incoming,
                    out, ids) <
           std::tie(o.N, o.A, o.batch, o.voff, o.nv, o.v_seg, o.max_spikes, o.words, o.num_outputs, o.rows, o.fix_cap,
                    o.bitmask, o.incoming, o.out, o.ids);
  }
};

std::atomic<int> g_batch_mode{1};  // 1: neuron-major row engine, 0: columnar per-tick kernels
std::atomic<uint32_t> g_fix_cap{kFixCap};

struct GraphCache {
  std::mutex mu;
  std::map<GraphKey, cudaGraphExec_t> execs;
  cudaStream_t capture = nullptr;
};

__global__ void k_set_batch_ctl(ShardCtl* ctl, uint32_t tick_base, int32_t dopamine) {
  ctl->tick_base = tick_base;
  ctl->dopamine = dopamine;
}

cudaError_t ensure_counts(ShardScratch& s, uint32_t batch, bool* realloc) {
  if (s.batch_cap >= batch && s.batch_counts) return cudaSuccess;
  *realloc = true;
  if (s.batch_counts) cudaFree(s.batch_counts);
  s.batch_counts = nullptr;
  s.batch_cap = 0;
  cudaError_t e = cudaMalloc(&s.batch_counts, (size_t)batch * 4);
  if (e != cudaSuccess) return e;
  s.batch_cap = batch;
  return cudaMemset(s.batch_counts, 0, (size_t)batch * 4);
}

}  // namespace

void graph_cache_free(ShardScratch* s) {
  if (!s) return;
  rows_free(*s);
  if (!s->graph_cache) return;
  GraphCache* c = static_cast<GraphCache*>(s->graph_cache);
  for (auto& kv : c->execs) cudaGraphExecDestroy(kv.second);
  if (c->capture) cudaStreamDestroy(c->capture);
  delete c;
  s->graph_cache = nullptr;
}

void graph_cache_drop(ShardScratch* s) {
  if (!s || !s->graph_cache) return;
  GraphCache* c = static_cast<GraphCache*>(s->graph_cache);
  std::lock_guard<std::mutex> lk(c->mu);
  for (auto& kv : c->execs) cudaGraphExecDestroy(kv.second);
  c->execs.clear();
}

uint32_t fix_capacity() { return g_fix_cap.load(); }

}  // namespace axc

using namespace axc;

extern "C" int32_t axc_batch_engine_mode(int32_t mode) {
  if (mode < 0) return g_batch_mode.load();
  return g_batch_mode.exchange(mode == 0 ? 0 : 1);
}

extern "C" uint32_t axc_row_engine_fix_capacity(uint32_t cap) {
  return g_fix_cap.exchange(cap < kFixCap ? cap : kFixCap);
}

extern "C" int32_t axc_step_day_phase_batch(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                                            uint32_t sync_batch_ticks, const AxcIoBuffers* io,
                                            const uint32_t* h_input_bitmask, const uint32_t* h_incoming_spikes,
                                            const uint32_t* h_spike_counts, uint32_t virtual_offset,
                                            uint32_t num_virtual_axons, const uint32_t* mapped_soma_ids_device,
                                            uint32_t v_seg, int16_t dopamine, uint32_t tick_base,
                                            uint8_t* h_output_history, void* stream_v) {
  if (!vram || !io) return (int32_t)cudaErrorInvalidValue;
  if (sync_batch_ticks == 0) return 0;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  cudaError_t e;
  ShardScratch* s = scratch_for(vram, padded_n, total_axons, &e);
  if (!s) return (int32_t)e;
  rows_touched(*s);   // the batch's row copy replaces the per-tick entry point's
  // Captured graphs hold the addresses of the scratch buffers: any
  // reallocation below drops them.
  bool realloc = false;
  e = ensure_counts(*s, sync_batch_ticks, &realloc);
  if (e != cudaSuccess) return (int32_t)e;
  const uint32_t rows = g_batch_mode.load() == 1 ? 1u : 0u;
  if (rows) {
    const void* before = s->rows ? s->rows->base : nullptr;
    e = rows_alloc(*s, padded_n, total_axons);
    if (e != cudaSuccess) return (int32_t)e;
    realloc = realloc || (before != nullptr && before != s->rows->base);
  }
  if (realloc && s->graph_cache) {
    GraphCache* old = static_cast<GraphCache*>(s->graph_cache);
    std::lock_guard<std::mutex> lk(old->mu);
    for (auto& kv : old->execs) cudaGraphExecDestroy(kv.second);
    old->execs.clear();
  }

  // 1. bulk H2D of the batch's inputs (shard.rs:54-68)
  const uint32_t words = io->input_words_per_tick;
  const uint32_t total_words = words * sync_batch_ticks;
  const uint32_t total_sched = io->max_spikes_per_tick * sync_batch_ticks;
  // cudaMemcpyDefault: the sources may be host (pageable or pinned) or device memory.
  if (io->d_input_bitmask && h_input_bitmask && total_words)
    e = cudaMemcpyAsync(io->d_input_bitmask, h_input_bitmask, (size_t)total_words * 4, cudaMemcpyDefault, stream);
  if (e == cudaSuccess && io->d_incoming_spikes && h_incoming_spikes && total_sched)
    e = cudaMemcpyAsync(io->d_incoming_spikes, h_incoming_spikes, (size_t)total_sched * 4, cudaMemcpyDefault,
                        stream);
  if (e != cudaSuccess) return (int32_t)e;
  if (h_spike_counts && io->d_incoming_spikes)
    e = cudaMemcpyAsync(s->batch_counts, h_spike_counts, (size_t)sync_batch_ticks * 4, cudaMemcpyDefault,
                        stream);
  else
    e = cudaMemsetAsync(s->batch_counts, 0, (size_t)sync_batch_ticks * 4, stream);
  if (e != cudaSuccess) return (int32_t)e;
  k_set_batch_ctl<<<1, 1, 0, stream>>>(s->ctl, tick_base, (int32_t)dopamine);

  // 2. burst-counter reset before the batch (shard.rs:71)
  e = launch_reset_burst(*vram, padded_n, stream);
  if (e != cudaSuccess) return (int32_t)e;

  // 3. the tick loop, as one graph (shard.rs:75-120)
  GraphKey key{padded_n, total_axons, sync_batch_ticks, virtual_offset, num_virtual_axons, v_seg,
               io->max_spikes_per_tick, words, io->num_outputs, rows, g_fix_cap.load(), io->d_input_bitmask, io->d_incoming_spikes,
               io->d_output_history, mapped_soma_ids_device};
  if (!s->graph_cache) s->graph_cache = new GraphCache();
  GraphCache* gc = static_cast<GraphCache*>(s->graph_cache);
  cudaGraphExec_t exec = nullptr;
  {
    std::lock_guard<std::mutex> lk(gc->mu);
    auto it = gc->execs.find(key);
    if (it != gc->execs.end()) {
      exec = it->second;
    } else {
      if (!gc->capture) {
        e = cudaStreamCreateWithFlags(&gc->capture, cudaStreamNonBlocking);
        if (e != cudaSuccess) return (int32_t)e;
      }
      e = cudaStreamBeginCapture(gc->capture, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return (int32_t)e;
      cudaError_t le = rows ? launch_rows_begin(*vram, *s, padded_n, total_axons, gc->capture) : cudaSuccess;
      for (uint32_t k = 0; k < sync_batch_ticks && le == cudaSuccess; k++) {
        TickArgs a{};
        a.padded_n = padded_n;
        a.total_axons = total_axons;
        a.v_seg = v_seg;
        a.tick = 0;
        a.input_bitmask = io->d_input_bitmask ? io->d_input_bitmask + (size_t)k * words : nullptr;
        a.virtual_offset = virtual_offset;
        a.num_virtual = a.input_bitmask ? num_virtual_axons : 0;
        a.incoming_spikes = io->d_incoming_spikes ? io->d_incoming_spikes + (size_t)k * io->max_spikes_per_tick
                                                  : nullptr;
        a.num_incoming = 0;
        a.max_incoming = io->max_spikes_per_tick;
        a.mapped_soma_ids = mapped_soma_ids_device;
        a.output_history = io->d_output_history ? io->d_output_history + (size_t)k * io->num_outputs : nullptr;
        a.num_outputs = io->num_outputs;
        a.dopamine = 0;
        a.batch = true;
        a.k = k;
        a.rows = rows != 0;
        a.defer_push = rows != 0 && k + 1 < sync_batch_ticks;
        a.fix_cap = key.fix_cap;
        le = launch_tick(*vram, *s, a, gc->capture);
      }
      if (rows && le == cudaSuccess) le = launch_rows_end(*vram, *s, padded_n, gc->capture);
      cudaGraph_t graph = nullptr;
      e = cudaStreamEndCapture(gc->capture, &graph);
      if (le != cudaSuccess) e = le;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (e != cudaSuccess) return (int32_t)e;
      gc->execs[key] = exec;
    }
  }
  e = cudaGraphLaunch(exec, stream);
  if (e != cudaSuccess) return (int32_t)e;

  // 4. outputs (shard_thread.rs:208-227)
  if (h_output_history && io->d_output_history && io->num_outputs) {
    e = cudaMemcpyAsync(h_output_history, io->d_output_history, (size_t)io->num_outputs * sync_batch_ticks,
                        cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  }
  return (int32_t)e;
}

extern "C" int32_t axc_profile_ticks(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                                     uint32_t v_seg, uint32_t tick0, uint32_t ticks,
                                     const uint32_t* d_input_bitmask, uint32_t words_per_tick,
                                     uint32_t virtual_offset, uint32_t num_virtual, int16_t dopamine,
                                     int32_t engine, void* stream_v, float* out_ms, uint64_t* out_counts) {
  if (!vram || !out_ms || !out_counts) return (int32_t)cudaErrorInvalidValue;
  cudaError_t e;
  ShardScratch* s = scratch_for(vram, padded_n, total_axons, &e);
  if (!s) return (int32_t)e;
  const bool rows = engine == 1;
  cudaStream_t st = static_cast<cudaStream_t>(stream_v);
  rows_touched(*s);
  if (rows) {
    bool realloc = false;
    e = ensure_counts(*s, ticks ? ticks : 1, &realloc);
    if (e == cudaSuccess) e = rows_alloc(*s, padded_n, total_axons);
    if (e != cudaSuccess) return (int32_t)e;
    if (realloc && s->graph_cache) {
      GraphCache* old = static_cast<GraphCache*>(s->graph_cache);
      std::lock_guard<std::mutex> lk(old->mu);
      for (auto& kv : old->execs) cudaGraphExecDestroy(kv.second);
      old->execs.clear();
    }
    cudaMemsetAsync(s->batch_counts, 0, (size_t)ticks * 4, st);
    k_set_batch_ctl<<<1, 1, 0, st>>>(s->ctl, tick0, (int32_t)dopamine);
    e = launch_rows_begin(*vram, *s, padded_n, total_axons, st);
    if (e != cudaSuccess) return (int32_t)e;
  }
  cudaEvent_t ev[kTickStages + 1];
  for (int i = 0; i <= kTickStages; i++) cudaEventCreate(&ev[i]);
  unsigned long long c0[8], c1[8];
  e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpy(c0, s->ctl->ctr, sizeof(c0), cudaMemcpyDeviceToHost);
  for (int i = 0; i < kTickStages; i++) out_ms[i] = 0.f;
  for (uint32_t k = 0; k < ticks && e == cudaSuccess; k++) {
    TickArgs a{};
    a.padded_n = padded_n;
    a.total_axons = total_axons;
    a.v_seg = v_seg;
    a.tick = tick0 + k;
    a.input_bitmask = d_input_bitmask ? d_input_bitmask + (size_t)k * words_per_tick : nullptr;
    a.virtual_offset = virtual_offset;
    a.num_virtual = a.input_bitmask ? num_virtual : 0;
    a.dopamine = dopamine;
    a.batch = rows;
    a.k = k;
    a.rows = rows;
    a.defer_push = rows && k + 1 < ticks;
    a.fix_cap = g_fix_cap.load();
    e = launch_tick(*vram, *s, a, st, ev);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[kTickStages]);
    for (int i = 0; i < kTickStages && e == cudaSuccess; i++) {
      float ms = 0.f;
      e = cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
      out_ms[i] += ms;
    }
  }
  if (rows && e == cudaSuccess) e = launch_rows_end(*vram, *s, padded_n, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpy(c1, s->ctl->ctr, sizeof(c1), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    for (int i = 0; i < 5; i++) out_counts[i] = c1[i + 1] - c0[i + 1];
  for (int i = 0; i <= kTickStages; i++) cudaEventDestroy(ev[i]);
  return (int32_t)e;
}

