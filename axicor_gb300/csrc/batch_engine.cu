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

#include <algorithm>
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

// Per batch, before its graph: the tick base and dopamine the captured kernels
// read, and (row engine) whether the batch lays its row copy out anew.
__global__ void k_set_batch_ctl(ShardCtl* ctl, uint32_t tick_base, int32_t dopamine, uint32_t rows, uint32_t force,
                                uint32_t ticks) {
  ctl->tick_base = tick_base;
  ctl->dopamine = dopamine;
  if (rows) layout_decide(ctl, force, ticks);
}

cudaError_t ensure_counts(ShardScratch& s, uint32_t batch, bool* realloc, cudaStream_t stream) {
  if (s.batch_cap >= batch && s.batch_counts) return cudaSuccess;
  *realloc = true;
  if (s.batch_counts) cudaFree(s.batch_counts);
  s.batch_counts = nullptr;
  s.batch_cap = 0;
  cudaError_t e = cudaMalloc(&s.batch_counts, (size_t)batch * 4);
  if (e != cudaSuccess) return e;
  s.batch_cap = batch;
  return cudaMemsetAsync(s.batch_counts, 0, (size_t)batch * 4, stream);   // in the caller's stream order
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

extern "C" uint32_t axc_row_engine_wait_limit(uint32_t tries) { return set_first_wait_limit(tries); }

namespace axc {

// Prepares one shard for a batch (shard.rs:40-71): scratch and row cache, then
// on `stream` the bulk H2D of the batch's inputs, the batch's tick base and
// dopamine, and the burst-counter reset.  *out_rows: the kernels the batch runs
// (1 the neuron-major row engine, 0 the columnar per-tick kernels).
cudaError_t batch_prepare(const BatchArgs& b, ShardScratch** out_s, uint32_t* out_rows, cudaStream_t stream) {
  cudaError_t e;
  ShardScratch* s = scratch_for(b.vram, b.padded_n, b.total_axons, &e);
  if (!s) return e;
  s->tick_rows_valid.store(false);   // the batch's row copy replaces the per-tick entry point's
  // Captured graphs hold the addresses of the scratch buffers: any
  // reallocation below drops them.
  bool realloc = false;
  e = ensure_counts(*s, b.ticks, &realloc, stream);
  if (e != cudaSuccess) return e;
  const uint32_t rows = g_batch_mode.load() == 1 ? 1u : 0u;
  if (rows) {
    const void* before = s->rows ? s->rows->base : nullptr;
    e = rows_alloc(*s, b.padded_n, b.total_axons, true, stream);
    if (e != cudaSuccess) return e;
    realloc = realloc || (before != nullptr && before != s->rows->base);
  }
  if (realloc) graph_cache_drop(s);
  // the device decides whether the batch lays the rows out anew or keeps the
  // last batch's copy (written back, so it matches the .state blob); a copy
  // that something invalidated is laid out anew for sure
  const bool force = rows ? batch_rows_force(*s) : true;

  // bulk H2D of the batch's inputs (shard.rs:54-68)
  const AxcIoBuffers* io = b.io;
  const uint32_t words = io->input_words_per_tick;
  const uint32_t total_words = words * b.ticks;
  const uint32_t total_sched = io->max_spikes_per_tick * b.ticks;
  // cudaMemcpyDefault: the sources may be host (pageable or pinned) or device memory.
  if (io->d_input_bitmask && b.h_bm && total_words)
    e = cudaMemcpyAsync(io->d_input_bitmask, b.h_bm, (size_t)total_words * 4, cudaMemcpyDefault, stream);
  if (e == cudaSuccess && io->d_incoming_spikes && b.h_in && total_sched)
    e = cudaMemcpyAsync(io->d_incoming_spikes, b.h_in, (size_t)total_sched * 4, cudaMemcpyDefault, stream);
  if (e != cudaSuccess) return e;
  if (b.h_counts && io->d_incoming_spikes)
    e = cudaMemcpyAsync(s->batch_counts, b.h_counts, (size_t)b.ticks * 4, cudaMemcpyDefault, stream);
  else
    e = cudaMemsetAsync(s->batch_counts, 0, (size_t)b.ticks * 4, stream);
  if (e != cudaSuccess) return e;
  k_set_batch_ctl<<<1, 1, 0, stream>>>(s->ctl, b.tick_base, (int32_t)b.dopamine, rows, force ? 1u : 0u, b.ticks);
  // burst-counter reset before the batch (shard.rs:71)
  e = launch_reset_burst(*b.vram, b.padded_n, stream);
  if (e != cudaSuccess) return e;
  *out_s = s;
  *out_rows = rows;
  return cudaSuccess;
}

// Launches the shard's tick loop (shard.rs:75-120) on `cap`, a stream being
// captured: the row copy, `ticks` ticks with global tick = tick_base + k read
// from the control block, the weight write-back.
cudaError_t batch_capture(const BatchArgs& b, ShardScratch& s, uint32_t rows, uint32_t fix_cap, cudaStream_t cap) {
  const AxcIoBuffers* io = b.io;
  const uint32_t words = io->input_words_per_tick;
  cudaError_t le = cudaSuccess;
  if (rows) le = launch_rows_begin(*b.vram, s, b.padded_n, b.total_axons, cap, false, true, true, true);
  for (uint32_t k = 0; k < b.ticks && le == cudaSuccess; k++) {
    TickArgs a{};
    a.padded_n = b.padded_n;
    a.total_axons = b.total_axons;
    a.v_seg = b.v_seg;
    a.tick = 0;
    a.input_bitmask = io->d_input_bitmask ? io->d_input_bitmask + (size_t)k * words : nullptr;
    a.virtual_offset = b.voff;
    a.num_virtual = a.input_bitmask ? b.nv : 0;
    a.incoming_spikes = io->d_incoming_spikes ? io->d_incoming_spikes + (size_t)k * io->max_spikes_per_tick : nullptr;
    a.num_incoming = 0;
    a.max_incoming = io->max_spikes_per_tick;
    a.mapped_soma_ids = b.ids;
    a.output_history = io->d_output_history ? io->d_output_history + (size_t)k * io->num_outputs : nullptr;
    a.num_outputs = io->num_outputs;
    a.dopamine = 0;
    a.batch = true;
    a.k = k;
    a.rows = rows != 0;
    a.defer_push = rows != 0 && k + 1 < b.ticks;
    a.fix_cap = fix_cap;
    le = launch_tick(*b.vram, s, a, cap);
  }
  if (rows && le == cudaSuccess) le = launch_rows_end(*b.vram, s, b.padded_n, cap);
  return le;
}

}  // namespace axc

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
  const BatchArgs b{vram, padded_n, total_axons, sync_batch_ticks, io, h_input_bitmask, h_incoming_spikes,
                    h_spike_counts, virtual_offset, num_virtual_axons, mapped_soma_ids_device, v_seg, dopamine,
                    tick_base};
  ShardScratch* s = nullptr;
  uint32_t rows = 0;
  cudaError_t e = batch_prepare(b, &s, &rows, stream);
  if (e != cudaSuccess) return (int32_t)e;

  // the tick loop, as one graph (shard.rs:75-120), captured once per shape
  const uint32_t words = io->input_words_per_tick;
  GraphKey key{padded_n, total_axons, sync_batch_ticks, virtual_offset, num_virtual_axons, v_seg,
               io->max_spikes_per_tick, words, io->num_outputs, rows, g_fix_cap.load(), io->d_input_bitmask,
               io->d_incoming_spikes, io->d_output_history, mapped_soma_ids_device};
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
      const cudaError_t le = batch_capture(b, *s, rows, key.fix_cap, gc->capture);
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

  // outputs (shard_thread.rs:208-227)
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
    e = ensure_counts(*s, ticks ? ticks : 1, &realloc, st);
    if (e == cudaSuccess) e = rows_alloc(*s, padded_n, total_axons, true, st);
    if (e != cudaSuccess) return (int32_t)e;
    if (realloc && s->graph_cache) {
      GraphCache* old = static_cast<GraphCache*>(s->graph_cache);
      std::lock_guard<std::mutex> lk(old->mu);
      for (auto& kv : old->execs) cudaGraphExecDestroy(kv.second);
      old->execs.clear();
    }
    cudaMemsetAsync(s->batch_counts, 0, (size_t)ticks * 4, st);
    k_set_batch_ctl<<<1, 1, 0, st>>>(s->ctl, tick0, (int32_t)dopamine, 0u, 1u, ticks);   // layouts its own
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
    for (int i = 0; i < 7; i++) out_counts[i] = c1[i + 1] - c0[i + 1];
  for (int i = 0; i <= kTickStages; i++) cudaEventDestroy(ev[i]);
  return (int32_t)e;
}


// ---------------------------------------------------------------------------
// Double-buffered batch I/O.  The reference keeps a swapchain of two pinned
// input buffers between its network thread and the GPU
// (genesis-node/src/network/io_server.rs:20-85) and downloads each batch's
// output history after the batch with a stream sync
// (genesis-node/src/node/shard_thread.rs:208-227).  Here the device side is
// double-buffered too: two device input bitmasks and two output histories per
// shard, an upload stream and a download stream.  Batch b's bitmask goes up on
// the upload stream into buffer b & 1 (once batch b - 2 has finished reading
// it), the batch runs on the caller's stream once its upload landed, and its
// output history comes down on the download stream into pinned buffer b & 1
// once the batch is done.  So the upload of batch b + 1 overlaps batch b's
// ticks, and batch b's readout overlaps batch b + 1's ticks; nothing in a
// submit waits on the host.
// ---------------------------------------------------------------------------
namespace axc {
namespace {

struct IoPipeline {
  ShardVramPtrs vram{};
  uint32_t N = 0, A = 0, batch = 0, words = 0, num_outputs = 0, voff = 0, nv = 0, v_seg = 0;
  const uint32_t* ids = nullptr;
  uint32_t* d_in[2] = {nullptr, nullptr};
  uint8_t* d_out[2] = {nullptr, nullptr};
  uint8_t* h_out[2] = {nullptr, nullptr};
  cudaStream_t up = nullptr, down = nullptr;
  cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_run[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
  uint64_t submitted = 0;
};

void io_pipeline_free(IoPipeline* p) {
  if (!p) return;
  for (int i = 0; i < 2; i++) {
    if (p->d_in[i]) cudaFree(p->d_in[i]);
    if (p->d_out[i]) cudaFree(p->d_out[i]);
    if (p->h_out[i]) cudaFreeHost(p->h_out[i]);
    if (p->ev_in[i]) cudaEventDestroy(p->ev_in[i]);
    if (p->ev_run[i]) cudaEventDestroy(p->ev_run[i]);
    if (p->ev_out[i]) cudaEventDestroy(p->ev_out[i]);
  }
  if (p->up) cudaStreamDestroy(p->up);
  if (p->down) cudaStreamDestroy(p->down);
  delete p;
}

}  // namespace
}  // namespace axc

extern "C" int32_t axc_io_pipeline_create(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                                          uint32_t sync_batch_ticks, uint32_t input_words_per_tick,
                                          uint32_t num_outputs, const uint32_t* mapped_soma_ids_device,
                                          uint32_t virtual_offset, uint32_t num_virtual_axons, uint32_t v_seg,
                                          void** out_handle) {
  if (!vram || !out_handle || sync_batch_ticks == 0) return (int32_t)cudaErrorInvalidValue;
  IoPipeline* p = new IoPipeline();
  p->vram = *vram;
  p->N = padded_n;
  p->A = total_axons;
  p->batch = sync_batch_ticks;
  p->words = input_words_per_tick;
  p->num_outputs = mapped_soma_ids_device ? num_outputs : 0u;
  p->ids = mapped_soma_ids_device;
  p->voff = virtual_offset;
  p->nv = num_virtual_axons;
  p->v_seg = v_seg;
  cudaError_t e = cudaStreamCreateWithFlags(&p->up, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->down, cudaStreamNonBlocking);
  const size_t in_bytes = (size_t)p->words * p->batch * 4, out_bytes = (size_t)p->num_outputs * p->batch;
  for (int i = 0; i < 2 && e == cudaSuccess; i++) {
    if (in_bytes) e = cudaMalloc(&p->d_in[i], in_bytes);
    if (e == cudaSuccess && out_bytes) e = cudaMalloc(&p->d_out[i], out_bytes);
    if (e == cudaSuccess && out_bytes) e = cudaHostAlloc(&p->h_out[i], out_bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_in[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_run[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_out[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    io_pipeline_free(p);
    return (int32_t)e;
  }
  *out_handle = p;
  return 0;
}

extern "C" int32_t axc_io_pipeline_submit(void* handle, const uint32_t* h_input_bitmask, int16_t dopamine,
                                          uint32_t tick_base, void* stream_v) {
  IoPipeline* p = static_cast<IoPipeline*>(handle);
  if (!p) return (int32_t)cudaErrorInvalidValue;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  const uint32_t slot = (uint32_t)(p->submitted & 1u);
  const bool reuse = p->submitted >= 2;   // batch b - 2 used this slot's buffers
  cudaError_t e = cudaSuccess;
  const size_t in_bytes = (size_t)p->words * p->batch * 4, out_bytes = (size_t)p->num_outputs * p->batch;
  // upload: once batch b - 2 has read this slot's bitmask
  if (reuse) e = cudaStreamWaitEvent(p->up, p->ev_run[slot], 0);
  if (e == cudaSuccess && in_bytes && h_input_bitmask)
    e = cudaMemcpyAsync(p->d_in[slot], h_input_bitmask, in_bytes, cudaMemcpyDefault, p->up);
  if (e == cudaSuccess) e = cudaEventRecord(p->ev_in[slot], p->up);
  // the batch: once its upload landed and batch b - 2's readout left this slot's output history
  if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, p->ev_in[slot], 0);
  if (e == cudaSuccess && reuse && out_bytes) e = cudaStreamWaitEvent(stream, p->ev_out[slot], 0);
  if (e != cudaSuccess) return (int32_t)e;
  AxcIoBuffers io{p->d_in[slot], nullptr, p->d_out[slot], 0, p->words, p->num_outputs};
  e = (cudaError_t)axc_step_day_phase_batch(&p->vram, p->N, p->A, p->batch, &io, nullptr, nullptr, nullptr, p->voff,
                                            h_input_bitmask ? p->nv : 0u, p->ids, p->v_seg, dopamine, tick_base,
                                            nullptr, stream);
  if (e == cudaSuccess) e = cudaEventRecord(p->ev_run[slot], stream);
  // download: once the batch is done
  if (e == cudaSuccess && out_bytes) {
    e = cudaStreamWaitEvent(p->down, p->ev_run[slot], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->h_out[slot], p->d_out[slot], out_bytes, cudaMemcpyDeviceToHost,
                                              p->down);
  }
  if (e == cudaSuccess) e = cudaEventRecord(p->ev_out[slot], p->down);
  if (e == cudaSuccess) p->submitted++;
  return (int32_t)e;
}

extern "C" int32_t axc_io_pipeline_outputs(void* handle, uint32_t back, const uint8_t** out_history) {
  IoPipeline* p = static_cast<IoPipeline*>(handle);
  if (!p || !out_history || back > 1 || p->submitted <= back) return (int32_t)cudaErrorInvalidValue;
  const uint32_t slot = (uint32_t)((p->submitted - 1 - back) & 1u);
  const cudaError_t e = cudaEventSynchronize(p->ev_out[slot]);
  *out_history = e == cudaSuccess ? p->h_out[slot] : nullptr;
  return (int32_t)e;
}

extern "C" int32_t axc_io_pipeline_wait_input(void* handle) {
  IoPipeline* p = static_cast<IoPipeline*>(handle);
  if (!p) return (int32_t)cudaErrorInvalidValue;
  if (p->submitted == 0) return 0;
  return (int32_t)cudaEventSynchronize(p->ev_in[(p->submitted - 1) & 1u]);
}

extern "C" void axc_io_pipeline_destroy(void* handle) {
  IoPipeline* p = static_cast<IoPipeline*>(handle);
  if (!p) return;
  for (int i = 0; i < 2; i++) {
    if (p->ev_out[i]) cudaEventSynchronize(p->ev_out[i]);
    if (p->ev_run[i]) cudaEventSynchronize(p->ev_run[i]);
  }
  io_pipeline_free(p);
}
