// shard_api.cu — the drop-in C-ABI of genesis-compute/src/ffi.rs:50-273.
//
// Allocation, uploads and the per-tick entry point keep the reference's
// semantics (genesis-compute/src/cuda/bindings.cu:571-692 and
// physics.cu:441-506).  The engine keeps its own per-shard scratch (segment
// masks, pending pushes, spiker list, control block) in a registry keyed by
// the shard's axon_heads pointer, because ShardVramPtrs has a fixed layout.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <mutex>
#include <unordered_map>

#include "engine.h"

namespace axc {

namespace {

std::mutex g_mu;
std::unordered_map<const void*, ShardScratch*>& registry() {
  static auto* m = new std::unordered_map<const void*, ShardScratch*>();
  return *m;
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

cudaError_t scratch_alloc(ShardScratch* s, uint32_t N, uint32_t A) {
  size_t off = 0;
  const size_t o_mask = off; off = align256(off + (size_t)A * 4);
  const size_t o_pend = off; off = align256(off + (size_t)A * 4);
  const size_t o_inc = off; off = align256(off + (size_t)A * 4);
  const size_t o_spk = off; off = align256(off + (size_t)N * 4 + 4);
  const size_t o_ctl = off; off = align256(off + sizeof(ShardCtl));
  void* base = nullptr;
  cudaError_t e = cudaMalloc(&base, off);
  if (e != cudaSuccess) return e;
  // zeroed before return: the scratch may be created by a call on a
  // non-blocking stream, which would not wait for a memset on the legacy stream
  e = cudaMemset(base, 0, off);
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
  if (e != cudaSuccess) { cudaFree(base); return e; }
  char* b = static_cast<char*>(base);
  s->base = base;
  s->padded_n = N;
  s->total_axons = A;
  s->seg_mask = reinterpret_cast<uint32_t*>(b + o_mask);
  s->pend = reinterpret_cast<uint32_t*>(b + o_pend);
  s->incoming = reinterpret_cast<uint32_t*>(b + o_inc);
  s->spikers = reinterpret_cast<uint32_t*>(b + o_spk);
  s->ctl = reinterpret_cast<ShardCtl*>(b + o_ctl);
  return cudaSuccess;
}

void scratch_free(ShardScratch* s) {
  if (!s) return;
  graph_cache_free(s);
  if (s->base) cudaFree(s->base);
  if (s->batch_counts) cudaFree(s->batch_counts);
  if (s->h_counts_pinned) cudaFreeHost(s->h_counts_pinned);
  delete s;
}

__global__ void k_init_sentinels(BurstHeads8* heads, uint32_t total) {  // bindings.cu:560-568
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) {
    uint4 v = make_uint4(AXC_AXON_SENTINEL, AXC_AXON_SENTINEL, AXC_AXON_SENTINEL, AXC_AXON_SENTINEL);
    uint4* p = reinterpret_cast<uint4*>(heads + i);
    p[0] = v;
    p[1] = v;
  }
}

}  // namespace

size_t state_blob_bytes(uint32_t padded_n) {  // memory.rs:32-54
  return (size_t)padded_n * (4 + 1 + 4 + 1 + 4) + (size_t)padded_n * AXC_MAX_DENDRITES * (4 + 2 + 1);
}

ShardScratch* scratch_for(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                          cudaError_t* err) {
  *err = cudaSuccess;
  const void* key = vram->axon_heads;
  std::lock_guard<std::mutex> lk(g_mu);
  auto& m = registry();
  auto it = m.find(key);
  if (it != m.end()) {
    ShardScratch* s = it->second;
    if (s->padded_n >= padded_n && s->total_axons >= total_axons) {
      if (s->state_base != vram->soma_voltage) {   // the same heads with another state allocation
        s->state_base = vram->soma_voltage;
        rows_touched(*s);
      }
      return s;
    }
    m.erase(it);
    scratch_free(s);
  }
  ShardScratch* s = new ShardScratch();
  *err = scratch_alloc(s, padded_n, total_axons);
  if (*err != cudaSuccess) { delete s; return nullptr; }
  s->state_base = vram->soma_voltage;
  s->state_bytes = state_blob_bytes(padded_n);
  m[key] = s;
  return s;
}

ShardScratch* scratch_find(const ShardVramPtrs* vram) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto& m = registry();
  auto it = m.find(vram->axon_heads);
  return it == m.end() ? nullptr : it->second;
}

void invalidate_overlapping(const void* dst, size_t size) {
  if (!dst || size == 0) return;
  const uintptr_t lo = reinterpret_cast<uintptr_t>(dst), hi = lo + size;
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : registry()) {
    ShardScratch* s = kv.second;
    const uintptr_t b = reinterpret_cast<uintptr_t>(s->state_base);
    if (b && lo < b + s->state_bytes && b < hi) rows_touched(*s);
  }
}

void scratch_release(const void* key) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto& m = registry();
  auto it = m.find(key);
  if (it == m.end()) return;
  ShardScratch* s = it->second;
  m.erase(it);
  scratch_free(s);
}

static ShardScratch* scratch_lookup(const ShardVramPtrs* vram) { return scratch_find(vram); }

// Kernels of cu_step_day_phase: 1 the neuron-major row engine with a row cache
// kept across calls (default), 0 the columnar per-tick kernels.
static std::atomic<int> g_tick_mode{1};
// Per-tick calls between two layouts of the row copy: a new layout follows the
// weights that froze and the axons that became fully lit meanwhile (the copy is
// rebuilt from the .state blob, which the write-through keeps current).
constexpr uint32_t kTickRelayout = 64;

}  // namespace axc

using namespace axc;

extern "C" {

const char* axc_version(void) { return "axicor-gb300 0.1 (sm_103a)"; }

int32_t cu_allocate_shard(uint32_t padded_n, uint32_t total_axons, ShardVramPtrs* out_vram) {
  if (!out_vram) return (int32_t)cudaErrorInvalidValue;
  const size_t n = padded_n;
  const size_t total_state = state_blob_bytes(padded_n);
  void* base = nullptr;
  cudaError_t err = cudaMalloc(&base, total_state ? total_state : 256);
  if (err != cudaSuccess) {
    fprintf(stderr, "[cu_allocate_shard] cudaMalloc state failed: %s\n", cudaGetErrorString(err));
    return (int32_t)err;
  }
  err = cudaMemset(base, 0, total_state);
  if (err != cudaSuccess) { cudaFree(base); return (int32_t)err; }
  char* b = static_cast<char*>(base);
  size_t off = 0;
  out_vram->soma_voltage = reinterpret_cast<int32_t*>(b + off); off += n * 4;
  out_vram->soma_flags = reinterpret_cast<uint8_t*>(b + off); off += n;
  out_vram->threshold_offset = reinterpret_cast<int32_t*>(b + off); off += n * 4;
  out_vram->timers = reinterpret_cast<uint8_t*>(b + off); off += n;
  out_vram->soma_to_axon = reinterpret_cast<uint32_t*>(b + off); off += n * 4;
  out_vram->dendrite_targets = reinterpret_cast<uint32_t*>(b + off); off += n * AXC_MAX_DENDRITES * 4;
  out_vram->dendrite_weights = reinterpret_cast<int16_t*>(b + off); off += n * AXC_MAX_DENDRITES * 2;
  out_vram->dendrite_timers = reinterpret_cast<uint8_t*>(b + off);

  BurstHeads8* heads = nullptr;
  err = cudaMalloc(reinterpret_cast<void**>(&heads),
                   (size_t)(total_axons ? total_axons : 1) * sizeof(BurstHeads8));
  if (err != cudaSuccess) {
    fprintf(stderr, "[cu_allocate_shard] cudaMalloc axon_heads failed: %s\n", cudaGetErrorString(err));
    cudaFree(base);
    out_vram->soma_voltage = nullptr;
    return (int32_t)err;
  }
  out_vram->axon_heads = heads;
  if (total_axons) k_init_sentinels<<<(total_axons + 255) / 256, 256>>>(heads, total_axons);
  err = cudaGetLastError();
  if (err == cudaSuccess) {
    ShardScratch* s = scratch_for(out_vram, padded_n, total_axons, &err);
    (void)s;
  }
  if (err == cudaSuccess) err = cudaDeviceSynchronize();
  if (err != cudaSuccess) {
    scratch_release(heads);
    cudaFree(heads);
    cudaFree(base);
    out_vram->soma_voltage = nullptr;
    out_vram->axon_heads = nullptr;
    return (int32_t)err;
  }
  return 0;
}

void cu_reset_burst_counters(const ShardVramPtrs* ptrs, uint32_t padded_n, void* stream) {
  if (!ptrs) return;
  launch_reset_burst(*ptrs, padded_n, static_cast<cudaStream_t>(stream));
}

int32_t cu_upload_state_blob(const ShardVramPtrs* vram, const void* state_blob, size_t state_size) {
  if (!vram || !state_blob) return (int32_t)cudaErrorInvalidValue;
  ShardScratch* s = scratch_lookup(vram);
  if (s && state_size > state_blob_bytes(s->padded_n)) {
    fprintf(stderr, "[cu_upload_state_blob] blob of %zu bytes exceeds the shard (%zu)\n", state_size,
            state_blob_bytes(s->padded_n));
    return (int32_t)cudaErrorInvalidValue;
  }
  if (s) rows_touched(*s);
  cudaError_t err = cudaMemcpy(vram->soma_voltage, state_blob, state_size, cudaMemcpyHostToDevice);
  if (err != cudaSuccess)
    fprintf(stderr, "[cu_upload_state_blob] cudaMemcpy failed: %s\n", cudaGetErrorString(err));
  return (int32_t)err;
}

int32_t cu_upload_axons_blob(const ShardVramPtrs* vram, const void* axons_blob, size_t axons_size) {
  if (!vram || !axons_blob) return (int32_t)cudaErrorInvalidValue;
  ShardScratch* s = scratch_lookup(vram);
  if (s && axons_size > (size_t)s->total_axons * sizeof(BurstHeads8)) {
    fprintf(stderr, "[cu_upload_axons_blob] blob of %zu bytes exceeds the shard\n", axons_size);
    return (int32_t)cudaErrorInvalidValue;
  }
  cudaError_t err = cudaMemcpy(vram->axon_heads, axons_blob, axons_size, cudaMemcpyHostToDevice);
  if (err != cudaSuccess)
    fprintf(stderr, "[cu_upload_axons_blob] cudaMemcpy failed: %s\n", cudaGetErrorString(err));
  return (int32_t)err;
}

void cu_free_shard(ShardVramPtrs* vram) {
  if (!vram) return;
  if (vram->axon_heads) scratch_release(vram->axon_heads);
  if (vram->soma_voltage) {
    cudaFree(vram->soma_voltage);
    vram->soma_voltage = nullptr;
    vram->soma_flags = nullptr;
    vram->threshold_offset = nullptr;
    vram->timers = nullptr;
    vram->soma_to_axon = nullptr;
    vram->dendrite_targets = nullptr;
    vram->dendrite_weights = nullptr;
    vram->dendrite_timers = nullptr;
  }
  if (vram->axon_heads) {
    cudaFree(vram->axon_heads);
    vram->axon_heads = nullptr;
  }
}

int32_t cu_step_day_phase(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                          uint32_t v_seg, uint32_t current_tick, const uint32_t* input_bitmask,
                          uint32_t virtual_offset, uint32_t num_virtual_axons,
                          const uint32_t* incoming_spikes, uint32_t num_incoming_spikes,
                          const uint32_t* mapped_soma_ids, uint8_t* output_history,
                          uint32_t num_outputs, int16_t dopamine, void* stream) {
  if (!vram) return (int32_t)cudaErrorInvalidValue;
  cudaError_t err;
  ShardScratch* s = scratch_for(vram, padded_n, total_axons, &err);
  if (!s) return (int32_t)err;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // The row engine keeps its neuron-major copy of the dendrites across calls
  // (rebuilt when another entry point wrote the shard or the LUT changed) and
  // writes GSOP's weight changes through to the columnar blob, so the shard's
  // memory after every call is what the reference leaves.  Without room for the
  // copy the columnar kernels run the tick.
  bool rows = g_tick_mode.load() == 1 && padded_n > 0 && total_axons > 0;
  if (rows && !(s->rows && s->rows->N >= padded_n && s->rows->A >= total_axons)) {
    if (rows_alloc(*s, padded_n, total_axons, true, st) != cudaSuccess) {
      cudaGetLastError();   // the failed allocation's error is not this tick's
      rows = false;
    }
  }
  if (rows) {
    s->batch_rows_valid.store(false);   // the batch path lays its rows out anew after per-tick calls
    const uint64_t gen = lut_generation();
    if (!s->tick_rows_valid.load() || s->tick_rows_lut != gen || s->tick_since_build >= kTickRelayout) {
      err = launch_rows_begin(*vram, *s, padded_n, total_axons, st);
      if (err != cudaSuccess) return (int32_t)err;
      s->tick_rows_valid.store(true);
      s->tick_rows_lut = gen;
      s->tick_parity = 0;
      s->tick_since_build = 0;
    }
    s->tick_since_build++;
  }
  TickArgs a{};
  a.padded_n = padded_n;
  a.total_axons = total_axons;
  a.v_seg = v_seg;
  a.tick = current_tick;
  a.input_bitmask = input_bitmask;
  a.virtual_offset = virtual_offset;
  a.num_virtual = input_bitmask ? num_virtual_axons : 0;
  a.incoming_spikes = incoming_spikes;
  a.num_incoming = incoming_spikes ? num_incoming_spikes : 0;
  a.max_incoming = num_incoming_spikes;
  a.mapped_soma_ids = mapped_soma_ids;
  a.output_history = output_history;
  a.num_outputs = num_outputs;
  a.dopamine = dopamine;
  a.batch = false;
  a.k = 0;
  if (rows) {
    a.rows = true;
    a.k = s->tick_parity;
    a.defer_push = false;
    a.fix_cap = s->rows->fix ? fix_capacity() : 0u;   // no list (population rows): the fix-up rescans
    s->tick_parity ^= 1u;
  }
  return (int32_t)launch_tick(*vram, *s, a, st);
}

int32_t cu_upload_constant_memory(const VariantParameters* lut) {
  if (!lut) return (int32_t)cudaErrorInvalidValue;
  return (int32_t)lut_upload(lut, nullptr, false);
}

void gpu_load_constants(const void* host_ptr) {
  if (host_ptr) lut_upload(static_cast<const VariantParameters*>(host_ptr), nullptr, false);
}

void update_constant_memory_hot_reload(const VariantParameters* new_variants, void* stream) {
  if (new_variants) lut_upload(new_variants, static_cast<cudaStream_t>(stream), true);
}

// ---- memory / stream helpers (bindings.cu:214-265) ----------------------
void* gpu_malloc(size_t size) {
  void* p = nullptr;
  if (cudaMalloc(&p, size) != cudaSuccess) return nullptr;
  return p;
}
void gpu_free(void* p) { cudaFree(p); }
void* gpu_host_alloc(size_t size) {
  void* p = nullptr;
  if (cudaHostAlloc(&p, size, cudaHostAllocDefault) != cudaSuccess) return nullptr;
  return p;
}
void gpu_host_free(void* p) { cudaFreeHost(p); }
// Copies into a shard's .state (the Night Phase's sprouting upload,
// shard_thread.rs:339-350) make its per-tick row cache stale.
void gpu_memcpy_host_to_device_async(void* dst, const void* src, size_t size, void* stream) {
  invalidate_overlapping(dst, size);
  cudaMemcpyAsync(dst, src, size, cudaMemcpyHostToDevice, static_cast<cudaStream_t>(stream));
}
void gpu_memcpy_device_to_host_async(void* dst, const void* src, size_t size, void* stream) {
  cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream));
}
bool gpu_memcpy_host_to_device(void* dst, const void* src, size_t size) {
  invalidate_overlapping(dst, size);
  cudaError_t err = cudaMemcpy(dst, src, size, cudaMemcpyHostToDevice);
  if (err != cudaSuccess)
    fprintf(stderr, "[gpu_memcpy_host_to_device] %s (size %zu)\n", cudaGetErrorString(err), size);
  return err == cudaSuccess;
}
bool gpu_memcpy_device_to_host(void* dst, const void* src, size_t size) {
  cudaError_t err = cudaMemcpy(dst, src, size, cudaMemcpyDeviceToHost);
  if (err != cudaSuccess)
    fprintf(stderr, "[gpu_memcpy_device_to_host] %s (size %zu)\n", cudaGetErrorString(err), size);
  return err == cudaSuccess;
}
int32_t gpu_stream_create(void** out_stream) {
  return (int32_t)cudaStreamCreateWithFlags(reinterpret_cast<cudaStream_t*>(out_stream),
                                            cudaStreamNonBlocking);
}
int32_t gpu_stream_destroy(void* stream) {
  return (int32_t)cudaStreamDestroy(static_cast<cudaStream_t>(stream));
}
void gpu_stream_synchronize(void* stream) { cudaStreamSynchronize(static_cast<cudaStream_t>(stream)); }
void gpu_set_device(int32_t device_id) {
  cudaError_t err = cudaSetDevice(device_id);
  if (err != cudaSuccess) fprintf(stderr, "[gpu_set_device] %s\n", cudaGetErrorString(err));
}
void gpu_device_synchronize(void) { cudaDeviceSynchronize(); }
void gpu_synchronize(void) { cudaDeviceSynchronize(); }

// ---- I/O buffers (bindings.cu:717-778) -----------------------------------
int32_t cu_allocate_io_buffers(uint32_t input_words, uint32_t schedule_capacity,
                               uint32_t output_capacity, uint32_t** d_input_bitmask,
                               uint32_t** d_incoming_spikes, uint8_t** d_output_history) {
  if (!d_input_bitmask || !d_incoming_spikes || !d_output_history) return -1;
  *d_input_bitmask = nullptr;
  *d_incoming_spikes = nullptr;
  *d_output_history = nullptr;
  if (input_words > 0 &&
      cudaMalloc(reinterpret_cast<void**>(d_input_bitmask), (size_t)input_words * 4) != cudaSuccess)
    return -1;
  if (schedule_capacity > 0 &&
      cudaMalloc(reinterpret_cast<void**>(d_incoming_spikes), (size_t)schedule_capacity * 4) != cudaSuccess)
    return -1;
  if (output_capacity > 0 &&
      cudaMalloc(reinterpret_cast<void**>(d_output_history), (size_t)output_capacity) != cudaSuccess)
    return -1;
  return 0;
}

int32_t cu_dma_h2d_io(uint32_t* d_input_bitmask, const uint32_t* h_input_bitmask, uint32_t input_words,
                      uint32_t* d_incoming_spikes, const uint32_t* h_incoming_spikes,
                      uint32_t schedule_capacity, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (input_words > 0 && d_input_bitmask && h_input_bitmask)
    e = cudaMemcpyAsync(d_input_bitmask, h_input_bitmask, (size_t)input_words * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && schedule_capacity > 0 && d_incoming_spikes && h_incoming_spikes)
    e = cudaMemcpyAsync(d_incoming_spikes, h_incoming_spikes, (size_t)schedule_capacity * 4,
                        cudaMemcpyHostToDevice, st);
  return (int32_t)e;
}

int32_t cu_dma_d2h_io(uint8_t* h_output_history, const uint8_t* d_output_history, uint32_t output_capacity,
                      void* stream) {
  if (output_capacity > 0 && d_output_history && h_output_history)
    return (int32_t)cudaMemcpyAsync(h_output_history, d_output_history, output_capacity,
                                    cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream));
  return 0;
}

// ---- engine extras --------------------------------------------------------
int32_t axc_tick_engine_mode(int32_t mode) {
  if (mode < 0) return g_tick_mode.load();
  return g_tick_mode.exchange(mode == 0 ? 0 : 1);
}

int32_t axc_shard_invalidate(const ShardVramPtrs* vram) {
  if (!vram) return (int32_t)cudaErrorInvalidValue;
  ShardScratch* s = scratch_lookup(vram);
  if (s) rows_touched(*s);
  return 0;
}

int32_t axc_shard_error_flags(const ShardVramPtrs* vram, uint32_t clear, uint32_t* out_flags) {
  if (!vram || !out_flags) return (int32_t)cudaErrorInvalidValue;
  ShardScratch* s = scratch_lookup(vram);
  if (!s) { *out_flags = 0; return 0; }
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return (int32_t)e;
  e = cudaMemcpy(out_flags, &s->ctl->err, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && clear) e = cudaMemset(&s->ctl->err, 0, 4);
  if (e == cudaSuccess && clear) e = cudaDeviceSynchronize();   // cleared before any later stream's work
  return (int32_t)e;
}

int32_t axc_shard_counters(const ShardVramPtrs* vram, uint32_t reset, uint64_t out[8]) {
  if (!vram || !out) return (int32_t)cudaErrorInvalidValue;
  ShardScratch* s = scratch_lookup(vram);
  if (!s) { for (int i = 0; i < 8; i++) out[i] = 0; return 0; }
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return (int32_t)e;
  e = cudaMemcpy(out, s->ctl->ctr, 8 * sizeof(uint64_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && reset) e = cudaMemset(s->ctl->ctr, 0, 8 * sizeof(uint64_t));
  if (e == cudaSuccess && reset) e = cudaDeviceSynchronize();
  return (int32_t)e;
}

int32_t axc_last_spikes(const ShardVramPtrs* vram, uint32_t* out_count, uint32_t* out_ids, uint32_t capacity,
                        void* stream) {
  if (!vram || !out_count) return (int32_t)cudaErrorInvalidValue;
  ShardScratch* s = scratch_lookup(vram);
  if (!s) return (int32_t)cudaErrorInvalidResourceHandle;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint32_t* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, ((size_t)s->padded_n + 1) * 4, st);
  if (e != cudaSuccess) return (int32_t)e;
  cudaMemsetAsync(d, 0, 4, st);
  e = launch_spike_list_sorted(*vram, s->padded_n, d + 1, d, st);
  uint32_t cnt = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&cnt, d, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) {
    *out_count = cnt;
    if (out_ids && capacity) {
      uint32_t c = cnt < capacity ? cnt : capacity;
      if (c) e = cudaMemcpyAsync(out_ids, d + 1, (size_t)c * 4, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
  }
  cudaFreeAsync(d, st);
  cudaStreamSynchronize(st);
  return (int32_t)e;
}

}  // extern "C"
