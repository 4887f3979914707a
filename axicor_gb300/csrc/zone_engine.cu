// zone_engine.cu — one batch of every shard of a GPU, with the intra-GPU ghost
// sync fused behind it, as one CUDA graph.
//
// The reference's node loop (genesis-node/src/node/mod.rs:330-420) runs, per
// batch: each shard's ShardEngine::step_day_phase_batch on the shard's own
// stream (shard_thread.rs), a device-wide barrier (gpu_device_synchronize,
// mod.rs:388), then the intra-GPU ghost sync of every channel on the legacy
// stream (IntraGpuChannel::sync_ghosts -> launch_ghost_sync, intra_gpu.rs:84,
// bindings.cu:341-368) before the next batch.  Here the shards' tick loops are
// parallel branches of one graph (fork on an event, join on one event per
// shard) and the ghost-sync kernels are nodes after the join, so the barrier
// and the sync are part of the graph: one launch per batch for the whole zone,
// no host round trip between the batch and its sync.  The per-batch inputs
// (bulk H2D, tick base, burst reset) go on the caller's stream before the
// graph, as axc_step_day_phase_batch does.
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <vector>

#include "engine.h"

namespace axc {
namespace {

// The shape of a zone batch: everything the captured graph depends on.
struct ZoneKey {
  std::vector<uint64_t> v;
  bool operator<(const ZoneKey& o) const { return v < o.v; }
};

struct ZoneCache {
  std::mutex mu;
  std::map<ZoneKey, cudaGraphExec_t> execs;
  cudaStream_t root = nullptr;
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> events;   // [0] fork, [1 + i] join of branch i
};

ZoneCache& zone_cache() {
  static ZoneCache* c = new ZoneCache();
  return *c;
}

cudaError_t ensure_streams(ZoneCache& c, uint32_t n) {
  cudaError_t e = cudaSuccess;
  if (!c.root) e = cudaStreamCreateWithFlags(&c.root, cudaStreamNonBlocking);
  while (e == cudaSuccess && c.branch.size() < n) {
    cudaStream_t st = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) c.branch.push_back(st);
  }
  while (e == cudaSuccess && c.events.size() < n + 1) {
    cudaEvent_t ev = nullptr;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) c.events.push_back(ev);
  }
  return e;
}

constexpr size_t kMaxZoneGraphs = 64;

}  // namespace
}  // namespace axc

using namespace axc;

extern "C" int32_t axc_step_zone_batch(const AxcZoneShard* shards, uint32_t nshards, const AxcGhostRoute* routes,
                                       uint32_t nroutes, uint32_t sync_batch_ticks, uint32_t tick_base,
                                       void* stream_v) {
  if ((!shards && nshards) || (!routes && nroutes)) return (int32_t)cudaErrorInvalidValue;
  if (nshards == 0 || sync_batch_ticks == 0) return 0;
  for (uint32_t i = 0; i < nshards; i++) {
    if (!shards[i].vram.axon_heads) return (int32_t)cudaErrorInvalidValue;
    for (uint32_t j = 0; j < i; j++)
      if (shards[j].vram.axon_heads == shards[i].vram.axon_heads) return (int32_t)cudaErrorInvalidValue;
  }
  for (uint32_t r = 0; r < nroutes; r++)
    if (routes[r].src_shard >= nshards || routes[r].dst_shard >= nshards ||
        (routes[r].count && (!routes[r].d_src_indices || !routes[r].d_dst_indices)))
      return (int32_t)cudaErrorInvalidValue;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);

  // per-batch inputs of every shard, on the caller's stream
  std::vector<BatchArgs> args(nshards);
  std::vector<ShardScratch*> scr(nshards);
  std::vector<uint32_t> rows(nshards);
  for (uint32_t i = 0; i < nshards; i++) {
    const AxcZoneShard& z = shards[i];
    args[i] = BatchArgs{&z.vram, z.padded_n, z.total_axons, sync_batch_ticks, &z.io, z.h_input_bitmask,
                        z.h_incoming_spikes, z.h_spike_counts, z.virtual_offset, z.num_virtual_axons,
                        z.mapped_soma_ids_device, z.v_seg, z.dopamine, tick_base};
    cudaError_t e = batch_prepare(args[i], &scr[i], &rows[i], stream);
    if (e != cudaSuccess) return (int32_t)e;
  }

  // the graph of this zone shape: every pointer a captured node holds is in the key
  const uint32_t fix_cap = fix_capacity();
  ZoneKey key;
  key.v = {nshards, nroutes, sync_batch_ticks, fix_cap};
  for (uint32_t i = 0; i < nshards; i++) {
    const AxcZoneShard& z = shards[i];
    const ShardScratch& s = *scr[i];
    for (uint64_t x : {(uint64_t)(uintptr_t)z.vram.soma_voltage, (uint64_t)(uintptr_t)z.vram.axon_heads,
                       (uint64_t)z.padded_n, (uint64_t)z.total_axons, (uint64_t)(uintptr_t)z.io.d_input_bitmask,
                       (uint64_t)(uintptr_t)z.io.d_incoming_spikes, (uint64_t)(uintptr_t)z.io.d_output_history,
                       (uint64_t)z.io.max_spikes_per_tick, (uint64_t)z.io.input_words_per_tick,
                       (uint64_t)z.io.num_outputs, (uint64_t)z.virtual_offset, (uint64_t)z.num_virtual_axons,
                       (uint64_t)(uintptr_t)z.mapped_soma_ids_device, (uint64_t)z.v_seg, (uint64_t)rows[i],
                       (uint64_t)(uintptr_t)s.base, (uint64_t)(uintptr_t)s.batch_counts,
                       (uint64_t)(uintptr_t)(s.rows ? s.rows->base : nullptr)})
      key.v.push_back(x);
  }
  for (uint32_t r = 0; r < nroutes; r++)
    for (uint64_t x : {(uint64_t)routes[r].src_shard, (uint64_t)routes[r].dst_shard,
                       (uint64_t)(uintptr_t)routes[r].d_src_indices, (uint64_t)(uintptr_t)routes[r].d_dst_indices,
                       (uint64_t)routes[r].count})
      key.v.push_back(x);

  ZoneCache& c = zone_cache();
  std::lock_guard<std::mutex> lk(c.mu);
  cudaGraphExec_t exec = nullptr;
  auto it = c.execs.find(key);
  cudaError_t e = cudaSuccess;
  if (it != c.execs.end()) {
    exec = it->second;
  } else {
    if (c.execs.size() >= kMaxZoneGraphs) {
      for (auto& kv : c.execs) cudaGraphExecDestroy(kv.second);
      c.execs.clear();
    }
    e = ensure_streams(c, nshards);
    if (e != cudaSuccess) return (int32_t)e;
    e = cudaStreamBeginCapture(c.root, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return (int32_t)e;
    cudaError_t le = cudaEventRecord(c.events[0], c.root);
    // fork: every shard's tick loop on its own branch
    for (uint32_t i = 0; i < nshards && le == cudaSuccess; i++) {
      le = cudaStreamWaitEvent(c.branch[i], c.events[0], 0);
      if (le == cudaSuccess) le = batch_capture(args[i], *scr[i], rows[i], fix_cap, c.branch[i]);
      if (le == cudaSuccess) le = cudaEventRecord(c.events[1 + i], c.branch[i]);
      if (le == cudaSuccess) le = cudaStreamWaitEvent(c.root, c.events[1 + i], 0);
    }
    // join, then the ghost sync of every route (mod.rs:409-411)
    for (uint32_t r = 0; r < nroutes && le == cudaSuccess; r++) {
      const AxcGhostRoute& g = routes[r];
      le = ghost_sync(shards[g.src_shard].vram.axon_heads, shards[g.dst_shard].vram.axon_heads, g.d_src_indices,
                      g.d_dst_indices, g.count, c.root);
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(c.root, &graph);
    if (le != cudaSuccess) e = le;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return (int32_t)e;
    c.execs[key] = exec;
  }
  e = cudaGraphLaunch(exec, stream);
  if (e != cudaSuccess) return (int32_t)e;

  // outputs (shard_thread.rs:208-227)
  bool wait = false;
  for (uint32_t i = 0; i < nshards && e == cudaSuccess; i++) {
    const AxcZoneShard& z = shards[i];
    if (z.h_output_history && z.io.d_output_history && z.io.num_outputs) {
      e = cudaMemcpyAsync(z.h_output_history, z.io.d_output_history, (size_t)z.io.num_outputs * sync_batch_ticks,
                          cudaMemcpyDeviceToHost, stream);
      wait = true;
    }
  }
  if (e == cudaSuccess && wait) e = cudaStreamSynchronize(stream);
  return (int32_t)e;
}
