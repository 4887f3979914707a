// side_kernels.cu — the per-batch side kernels of genesis-compute/src/cuda/bindings.cu
// (Night-Phase sort-and-prune, inter-zone spike extraction and ghost sync),
// spike telemetry (physics.cu:400-434), and the legacy per-kernel launchers
// that ffi.rs:193-233 declares.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <mutex>

#include "engine.h"

namespace axc {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// sort_and_prune — bindings.cu:450-515.
// The reference runs one thread per neuron and insertion-sorts its 128 slots
// in shared memory.  Its result is a stable sort of the non-empty slots by
// |weight| descending, followed by the empty slots in their original order;
// then every non-empty slot with |w| < threshold is zeroed in place.
// Here a 256-thread block stages 32 neurons' slots in shared memory with
// coalesced row loads, each warp ranks one neuron's 128 slots at a time
// (lane L holds slots L, L+32, L+64, L+96), scatters them to their ranks,
// prunes, and the block writes the rows back coalesced.
// ---------------------------------------------------------------------------
constexpr int kSortNeurons = 32;

__global__ void __launch_bounds__(256) k_sort_and_prune(ShardVramPtrs v, uint32_t N, int16_t prune_threshold) {
  __shared__ uint32_t s_tg[AXC_MAX_DENDRITES][kSortNeurons + 1];
  __shared__ int16_t s_wt[AXC_MAX_DENDRITES][kSortNeurons + 1];
  __shared__ uint8_t s_tm[AXC_MAX_DENDRITES][kSortNeurons + 1];
  const uint32_t n0 = blockIdx.x * kSortNeurons;
  const uint32_t col = threadIdx.x & 31, row0 = threadIdx.x >> 5;
  for (uint32_t r = row0; r < AXC_MAX_DENDRITES; r += 8) {
    const uint32_t n = n0 + col;
    uint32_t t = 0; int16_t w = 0; uint8_t m = 0;
    if (n < N) {
      const size_t idx = (size_t)r * N + n;
      t = v.dendrite_targets[idx];
      w = v.dendrite_weights[idx];
      m = v.dendrite_timers[idx];
    }
    s_tg[r][col] = t; s_wt[r][col] = w; s_tm[r][col] = m;
  }
  if (threadIdx.x < kSortNeurons && n0 + threadIdx.x < N) v.soma_flags[n0 + threadIdx.x] &= 0xF1;  // :456-458
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t c = warp; c < kSortNeurons; c += 8) {
    uint32_t tg[4]; int16_t wt[4]; uint8_t tm[4]; int32_t aw[4]; bool ne[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const uint32_t q = lane + 32 * j;
      tg[j] = s_tg[q][c]; wt[j] = s_wt[q][c]; tm[j] = s_tm[q][c];
      aw[j] = wt[j] >= 0 ? wt[j] : -wt[j];
      ne[j] = tg[j] != 0;
    }
    uint32_t bal[4], nonempty = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) { bal[j] = __ballot_sync(kFull, ne[j]); nonempty += __popc(bal[j]); }
    uint32_t rank[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      // empties: after all non-empty slots, in original order
      uint32_t before = 0;
#pragma unroll
      for (int jj = 0; jj < 4; jj++) {
        const uint32_t eb = ~bal[jj];
        if (jj < j) before += __popc(eb);
        else if (jj == j) before += __popc(eb & ((1u << lane) - 1u));
      }
      rank[j] = nonempty + before;
    }
    uint32_t cnt[4] = {0, 0, 0, 0};
    for (int src = 0; src < 32; src++) {
#pragma unroll
      for (int jj = 0; jj < 4; jj++) {
        const int32_t oa = __shfl_sync(kFull, aw[jj], src);
        const bool one = __shfl_sync(kFull, ne[jj], src);
        const uint32_t oq = (uint32_t)src + 32u * jj;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const uint32_t q = lane + 32u * j;
          cnt[j] += (one && (oa > aw[j] || (oa == aw[j] && oq < q))) ? 1u : 0u;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (ne[j]) rank[j] = cnt[j];
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 4; j++) {
      uint32_t t = tg[j]; int16_t w = wt[j]; uint8_t m = tm[j];
      if (t != 0 && aw[j] < (int32_t)prune_threshold) { t = 0; w = 0; m = 0; }   // :498-506
      s_tg[rank[j]][c] = t; s_wt[rank[j]][c] = w; s_tm[rank[j]][c] = m;
    }
    __syncwarp();
  }
  __syncthreads();
  for (uint32_t r = row0; r < AXC_MAX_DENDRITES; r += 8) {
    const uint32_t n = n0 + col;
    if (n < N) {
      const size_t idx = (size_t)r * N + n;
      v.dendrite_targets[idx] = s_tg[r][col];
      v.dendrite_weights[idx] = s_wt[r][col];
      v.dendrite_timers[idx] = s_tm[r][col];
    }
  }
}

// ---------------------------------------------------------------------------
// ghost_sync — bindings.cu:341-368
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ghost_sync(const BurstHeads8* __restrict__ src, BurstHeads8* __restrict__ dst,
                                                    const uint32_t* __restrict__ si, const uint32_t* __restrict__ di,
                                                    uint32_t count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint32_t s = si[i];
  if (s < 0x80000000u) {
    const uint4* p = reinterpret_cast<const uint4*>(src + s);
    uint4* q = reinterpret_cast<uint4*>(dst + di[i]);
    const uint4 x = p[0], y = p[1];
    q[0] = x;
    q[1] = y;
  }
}

// ---------------------------------------------------------------------------
// extract_outgoing_spikes — bindings.cu:378-436, with a deterministic output
// order: per-entry event counts, a block scan and a one-block scan of the
// block totals, then each entry writes its events in head order.
// ---------------------------------------------------------------------------
constexpr uint32_t kExtBlock = 256;

__device__ __forceinline__ uint32_t outgoing_events(const BurstHeads8* heads, uint32_t a, uint32_t batch_ticks,
                                                    uint32_t v_seg, uint32_t out_ticks[8]) {
  const uint32_t* h = reinterpret_cast<const uint32_t*>(heads + a);
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const uint32_t head = h[k];
    if (head >= 0x70000000u) continue;                 // :405-406
    const uint32_t since = head / v_seg;               // :408
    if (since < batch_ticks) out_ticks[c++] = batch_ticks - 1 - since;
  }
  return c;
}

__global__ void __launch_bounds__(kExtBlock) k_ext_count(const BurstHeads8* __restrict__ heads,
                                                         const uint32_t* __restrict__ si, uint32_t count,
                                                         uint32_t batch_ticks, uint32_t v_seg,
                                                         uint32_t* __restrict__ block_totals) {
  const uint32_t i = blockIdx.x * kExtBlock + threadIdx.x;
  uint32_t c = 0;
  if (i < count) {
    const uint32_t a = si[i];
    uint32_t t[8];
    if (a < 0x80000000u) c = outgoing_events(heads, a, batch_ticks, v_seg, t);
  }
  __shared__ uint32_t part[kExtBlock / 32];
  uint32_t s = c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFull, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int w = 0; w < (int)(kExtBlock / 32); w++) tot += part[w];
    block_totals[blockIdx.x] = tot;
  }
}

__global__ void __launch_bounds__(1024) k_scan_totals(uint32_t* __restrict__ totals, uint32_t nblocks,
                                                      uint32_t* __restrict__ out_count, int accumulate) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (nblocks + 1023) / 1024;
  const uint32_t b0 = threadIdx.x * per;
  uint32_t s = 0;
  for (uint32_t b = b0; b < min(b0 + per, nblocks); b++) s += totals[b];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = accumulate ? *out_count : 0u;
    for (int i = 0; i < 1024; i++) { const uint32_t x = part[i]; part[i] = acc; acc += x; }
    *out_count = acc;
  }
  __syncthreads();
  uint32_t acc = part[threadIdx.x];
  for (uint32_t b = b0; b < min(b0 + per, nblocks); b++) { const uint32_t x = totals[b]; totals[b] = acc; acc += x; }
}

__global__ void __launch_bounds__(kExtBlock) k_ext_write(const BurstHeads8* __restrict__ heads,
                                                         const uint32_t* __restrict__ si,
                                                         const uint32_t* __restrict__ dg, uint32_t count,
                                                         uint32_t batch_ticks, uint32_t v_seg,
                                                         const uint32_t* __restrict__ block_offsets,
                                                         SpikeEvent* __restrict__ out) {
  const uint32_t i = blockIdx.x * kExtBlock + threadIdx.x;
  uint32_t c = 0, t[8];
  if (i < count) {
    const uint32_t a = si[i];
    if (a < 0x80000000u) c = outgoing_events(heads, a, batch_ticks, v_seg, t);
  }
  __shared__ uint32_t wsum[kExtBlock / 32];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = c;  // inclusive warp scan
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = block_offsets[blockIdx.x];
    for (int q = 0; q < (int)(kExtBlock / 32); q++) { const uint32_t y = wsum[q]; wsum[q] = acc; acc += y; }
  }
  __syncthreads();
  if (c) {
    const uint32_t base = wsum[w] + x - c;
    const uint32_t gid = dg[i];
    for (uint32_t k = 0; k < c; k++) {
      out[base + k].ghost_id = gid;
      out[base + k].tick_offset = t[k];
    }
  }
}

// ---------------------------------------------------------------------------
// Legacy per-kernel launchers (bindings.cu:106-207, 295-334)
// ---------------------------------------------------------------------------
// inject_inputs_kernel with input_stride 1 and virtual_offset 0, as
// launch_inject_inputs calls it (bindings.cu:106-135, 295-303).
__global__ void __launch_bounds__(256) k_legacy_inject(BurstHeads8* __restrict__ heads, uint32_t A,
                                                       const uint32_t* __restrict__ bitmask, uint32_t tick,
                                                       uint32_t total_virtual) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= total_virtual || tid >= A) return;
  const uint32_t words = (total_virtual + 31) / 32;
  const uint32_t word = bitmask[(size_t)tick * words + tid / 32];
  if ((word >> (tid % 32)) & 1u) {
    uint32_t* h = reinterpret_cast<uint32_t*>(heads + tid);
#pragma unroll
    for (int k = 7; k > 0; k--) h[k] = h[k - 1];
    h[0] = 0;
  }
}

// record_readout_kernel (bindings.cu:191-207), bounds-guarded.
__global__ void __launch_bounds__(256) k_legacy_readout(const uint8_t* __restrict__ flags, uint32_t N,
                                                        const uint32_t* __restrict__ ids, uint8_t* __restrict__ out,
                                                        uint32_t channels, uint32_t tick) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= channels) return;
  const uint32_t id = ids[tid];
  out[(size_t)tick * channels + tid] = id < N ? (flags[id] & 0x01) : 0;
}

// ---------------------------------------------------------------------------
// Scratch of the allocation-free spike extraction: the per-block event totals
// (then offsets) of one call, for up to AXC_NOALLOC_MAX_BOUNDARY_AXONS entries.
// Every GPU that loads this library holds these 16 KiB until the process
// exits.  Every call overwrites the totals of the blocks it uses before it
// reads them, so nothing has to start at zero; two calls that overlap on the
// GPU (for example on two streams) use the same array and race.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoAllocBlocks = AXC_NOALLOC_MAX_BOUNDARY_AXONS / kExtBlock;
static_assert(AXC_NOALLOC_MAX_BOUNDARY_AXONS % kExtBlock == 0, "whole blocks");
static __device__ __align__(256) uint32_t g_noalloc_block_totals[kNoAllocBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_block_totals on the current device.  Host code
// cannot pass the symbol itself: on the host it names a shadow variable, not
// device memory.  Looked up once per device, with that device current.
cudaError_t noalloc_scratch(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_block_totals);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace

cudaError_t ghost_sync(const BurstHeads8* src_heads, BurstHeads8* dst_heads, const uint32_t* src_indices,
                       const uint32_t* dst_indices, uint32_t count, cudaStream_t stream) {
  if (count == 0) return cudaSuccess;
  return launch_k(k_ghost_sync, dim3((count + 255) / 256), dim3(256), stream, src_heads, dst_heads, src_indices,
                  dst_indices, count);
}

namespace {

ShardVramPtrs from_legacy(const VramState& s) {
  ShardVramPtrs v;
  v.soma_voltage = s.voltage;
  v.soma_flags = s.flags;
  v.threshold_offset = s.threshold_offset;
  v.timers = s.refractory_timer;
  v.soma_to_axon = s.soma_to_axon;
  v.dendrite_targets = s.dendrite_targets;
  v.dendrite_weights = s.dendrite_weights;
  v.dendrite_timers = s.dendrite_timers;
  v.axon_heads = s.axon_heads;
  return v;
}

}  // namespace
}  // namespace axc

using namespace axc;

extern "C" {

void launch_sort_and_prune(const ShardVramPtrs* ptrs, uint32_t padded_n, int16_t prune_threshold) {
  if (!ptrs || padded_n == 0) return;
  if (ShardScratch* s = scratch_find(ptrs)) rows_touched(*s);   // targets and weights move
  k_sort_and_prune<<<(padded_n + kSortNeurons - 1) / kSortNeurons, 256>>>(*ptrs, padded_n, prune_threshold);
}

void launch_ghost_sync(const BurstHeads8* src_heads, BurstHeads8* dst_heads, const uint32_t* src_indices,
                       const uint32_t* dst_indices, uint32_t count, void* stream) {
  ghost_sync(src_heads, dst_heads, src_indices, dst_indices, count, static_cast<cudaStream_t>(stream));
}

void launch_extract_outgoing_spikes(const BurstHeads8* axon_heads, const uint32_t* src_indices,
                                    const uint32_t* dst_ghost_ids, uint32_t count, uint32_t sync_batch_ticks,
                                    uint32_t v_seg, void* out_events, uint32_t* out_count, void* stream_v) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  if (count == 0 || v_seg == 0) {
    cudaMemsetAsync(out_count, 0, sizeof(uint32_t), stream);
    return;
  }
  const uint32_t nb = (count + kExtBlock - 1) / kExtBlock;
  uint32_t* tmp = nullptr;
  // bindings.cu:431 clears the count before anything else: a call that fails
  // to get its scratch then reports 0 events, not the previous batch's count
  cudaMemsetAsync(out_count, 0, sizeof(uint32_t), stream);
  if (cudaMallocAsync(&tmp, (size_t)nb * 4, stream) != cudaSuccess) return;
  k_ext_count<<<nb, kExtBlock, 0, stream>>>(axon_heads, src_indices, count, sync_batch_ticks, v_seg, tmp);
  k_scan_totals<<<1, 1024, 0, stream>>>(tmp, nb, out_count, 0);
  k_ext_write<<<nb, kExtBlock, 0, stream>>>(axon_heads, src_indices, dst_ghost_ids, count, sync_batch_ticks, v_seg,
                                            tmp, static_cast<SpikeEvent*>(out_events));
  cudaFreeAsync(tmp, stream);
}

// The same extraction as launch_extract_outgoing_spikes, for callers that must
// not allocate device memory: its scratch is the file-scope array above, so the
// call launches kernels and nothing else (no cudaMalloc, cudaFree or pool
// allocation).  The first call on a device looks up the array's address.
int32_t axc_extract_outgoing_spikes_noalloc(const BurstHeads8* axon_heads, const uint32_t* src_indices,
                                            const uint32_t* dst_ghost_ids, uint32_t count, uint32_t sync_batch_ticks,
                                            uint32_t v_seg, void* out_events, uint32_t* out_count, void* stream_v) {
  if (count > AXC_NOALLOC_MAX_BOUNDARY_AXONS) {
    fprintf(stderr,
            "[axc_extract_outgoing_spikes_noalloc] %u boundary axons exceed the fixed scratch limit of %u; "
            "use launch_extract_outgoing_spikes or split the call\n",
            count, (unsigned)AXC_NOALLOC_MAX_BOUNDARY_AXONS);
    return (int32_t)cudaErrorInvalidValue;
  }
  if (!out_count || (count > 0 && (!axon_heads || !src_indices || !dst_ghost_ids || !out_events)))
    return (int32_t)cudaErrorInvalidValue;
  uint32_t* totals = nullptr;
  cudaError_t e = noalloc_scratch(&totals);
  if (e != cudaSuccess) return (int32_t)e;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  // Each launch reports its own status (cudaLaunchKernel's return), so an
  // error left pending by an earlier, unrelated call is neither blamed on this
  // one nor cleared: the caller still reads it with cudaGetLastError.
  if (count == 0 || v_seg == 0) {
    uint32_t zero = 0;
    int acc = 0;
    return (int32_t)launch_k(k_scan_totals, dim3(1), dim3(1024), stream, totals, zero, out_count, acc);  // *out_count = 0
  }
  uint32_t nb = (count + kExtBlock - 1) / kExtBlock;
  int acc = 0;
  SpikeEvent* events = static_cast<SpikeEvent*>(out_events);
  e = launch_k(k_ext_count, dim3(nb), dim3(kExtBlock), stream, axon_heads, src_indices, count, sync_batch_ticks, v_seg,
               totals);
  if (e == cudaSuccess) e = launch_k(k_scan_totals, dim3(1), dim3(1024), stream, totals, nb, out_count, acc);
  if (e == cudaSuccess)
    e = launch_k(k_ext_write, dim3(nb), dim3(kExtBlock), stream, axon_heads, src_indices, dst_ghost_ids, count,
                 sync_batch_ticks, v_seg, static_cast<const uint32_t*>(totals), events);
  return (int32_t)e;
}

// bindings.cu:780-782 is a no-op in the reference; so is this.
void gpu_reset_telemetry_count(const ShardVramPtrs* ptrs, void* stream) {
  (void)ptrs;
  (void)stream;
}

void launch_extract_telemetry(const ShardVramPtrs* ptrs, uint32_t padded_n, uint32_t* out_ids,
                              uint32_t* out_count_pinned, void* stream) {
  if (!out_ids || !out_count_pinned || !ptrs) return;  // bindings.cu:785
  launch_spike_list_sorted(*ptrs, padded_n, out_ids, out_count_pinned, static_cast<cudaStream_t>(stream));
}

void launch_inject_inputs(VramState vram, const uint32_t* bitmask, uint32_t current_tick,
                          uint32_t total_virtual_axons) {
  if (!bitmask || total_virtual_axons == 0) return;
  k_legacy_inject<<<(total_virtual_axons + 255) / 256, 256>>>(vram.axon_heads, vram.total_axons, bitmask,
                                                              current_tick, total_virtual_axons);
}

void launch_apply_spike_batch(VramState vram, const uint32_t* tick_schedule, uint32_t tick_spikes_count) {
  if (tick_spikes_count == 0 || !tick_schedule) return;
  ShardVramPtrs v = from_legacy(vram);
  cudaError_t e;
  ShardScratch* s = scratch_for(&v, vram.padded_n, vram.total_axons, &e);
  if (!s) return;
  launch_push_incoming(vram.axon_heads, *s, vram.total_axons, tick_schedule, tick_spikes_count, nullptr);
}

void launch_propagate_axons(VramState vram, uint32_t v_seg) {
  launch_propagate_only(vram.axon_heads, vram.total_axons, v_seg, nullptr);
}

void launch_update_neurons(VramState vram, const void* constants_ptr, uint32_t current_tick) {
  (void)constants_ptr;
  ShardVramPtrs v = from_legacy(vram);
  cudaError_t e;
  ShardScratch* s = scratch_for(&v, vram.padded_n, vram.total_axons, &e);
  if (!s) return;
  launch_update_stage(v, *s, vram.padded_n, vram.total_axons, current_tick, nullptr);
}

void launch_apply_gsop(VramState vram) {
  ShardVramPtrs v = from_legacy(vram);
  cudaError_t e;
  ShardScratch* s = scratch_for(&v, vram.padded_n, vram.total_axons, &e);
  if (!s) return;
  rows_touched(*s);   // columnar weights change
  launch_gsop_stage(v, *s, vram.padded_n, vram.total_axons, 0, nullptr);
}

void launch_record_readout(VramState vram, const uint32_t* mapped_soma_ids, uint8_t* output_history,
                           uint32_t current_tick, uint32_t total_pixels) {
  if (!mapped_soma_ids || !output_history || total_pixels == 0) return;
  k_legacy_readout<<<(total_pixels + 255) / 256, 256>>>(vram.flags, vram.padded_n, mapped_soma_ids,
                                                        output_history, total_pixels, current_tick);
}

}  // extern "C"
