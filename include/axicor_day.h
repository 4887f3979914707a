/*
 * axicor_day.h — C-ABI of the GB300 Day Phase engine.
 *
 * The first half of this header is the drop-in boundary: the same unmangled
 * symbols, argument orders and #[repr(C)] layouts that the Rust crate
 * genesis-compute binds in genesis-compute/src/ffi.rs:27-273 (link name
 * "genesis_cuda", ffi.rs:48).  A Rust build links this library in place of
 * the reference's physics.cu + bindings.cu without source changes.
 *
 * The second half (axc_* symbols) is new: a batch API with a CUDA-graph
 * captured tick loop, spike compaction, device error reporting, and the
 * brain generator used to build the synthetic benchmark brains.
 *
 * Conventions
 *  - A "stream" argument is a cudaStream_t passed as an opaque pointer
 *    (Rust: CudaStream = *mut c_void, ffi.rs:5).  NULL is the legacy stream.
 *  - int32_t returns are cudaError_t values (0 = success) unless stated.
 *  - Every pointer inside ShardVramPtrs is a device pointer.
 */
#ifndef AXICOR_DAY_H
#define AXICOR_DAY_H

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define AXC_MAX_DENDRITES 128u     /* genesis-core/src/constants.rs:9        */
#define AXC_AXON_SENTINEL 0x80000000u /* constants.rs:13                    */
#define AXC_TARGET_AXON_MASK 0x00FFFFFFu /* constants.rs:20                 */
#define AXC_TARGET_SEG_SHIFT 24u   /* constants.rs:21                        */
#define AXC_NO_AXON 0xFFFFFFFFu    /* soma_to_axon / mapped_soma_ids "none"  */

/* Eight-slot burst shift register of one axon (genesis-core/src/layout.rs:53-74). */
typedef struct __attribute__((aligned(32))) BurstHeads8 {
  uint32_t h0, h1, h2, h3, h4, h5, h6, h7;
} BurstHeads8;

/* Neuron-type parameters, 64 bytes (genesis-core/src/layout.rs:12-48). */
typedef struct __attribute__((aligned(64))) VariantParameters {
  int32_t threshold;                        /*  0 */
  int32_t rest_potential;                   /*  4 */
  int32_t leak_rate;                        /*  8 */
  int32_t homeostasis_penalty;              /* 12 */
  uint32_t spontaneous_firing_period_ticks; /* 16 */
  uint16_t initial_synapse_weight;          /* 20 */
  uint16_t gsop_potentiation;               /* 22 */
  uint16_t gsop_depression;                 /* 24 */
  uint16_t homeostasis_decay;               /* 26 */
  uint8_t refractory_period;                /* 28 */
  uint8_t synapse_refractory_period;        /* 29 */
  uint8_t signal_propagation_length;        /* 30 */
  uint8_t is_inhibitory;                    /* 31 */
  uint8_t inertia_curve[16];                /* 32 */
  int32_t adaptive_leak_max;                /* 48 */
  uint16_t adaptive_leak_gain;              /* 52 */
  uint8_t adaptive_mode;                    /* 54 */
  uint8_t _leak_pad[3];                     /* 55 */
  uint8_t d1_affinity;                      /* 58 */
  uint8_t d2_affinity;                      /* 59 */
  uint8_t _pad[4];                          /* 60 */
} VariantParameters;

/* Device pointers of one shard, field order == .state blob order
 * (genesis-compute/src/ffi.rs:25-42, memory.rs:71-86). */
typedef struct ShardVramPtrs {
  int32_t* soma_voltage;      /* [N]        base of the state allocation */
  uint8_t* soma_flags;        /* [N]        [7:4] variant, [3:1] burst, [0] spike */
  int32_t* threshold_offset;  /* [N] */
  uint8_t* timers;            /* [N]        refractory countdown */
  uint32_t* soma_to_axon;     /* [N] */
  uint32_t* dendrite_targets; /* [128][N]   (seg<<24) | (axon+1) */
  int16_t* dendrite_weights;  /* [128][N] */
  uint8_t* dendrite_timers;   /* [128][N]   not touched by the Day Phase */
  BurstHeads8* axon_heads;    /* [A]        separate allocation */
} ShardVramPtrs;

/* Legacy by-value state of the old per-kernel launchers (genesis-core/src/layout.rs:281-307). */
typedef struct VramState {
  uint32_t padded_n;
  uint32_t total_axons;
  int32_t* voltage;
  uint8_t* flags;
  int32_t* threshold_offset;
  uint8_t* refractory_timer;
  uint32_t* soma_to_axon;
  uint32_t* dendrite_targets;
  int16_t* dendrite_weights;
  uint8_t* dendrite_timers;
  BurstHeads8* axon_heads;
  uint32_t* input_bitmask;
  uint8_t* output_history;
  uint32_t* telemetry_count;
  uint32_t* telemetry_spikes;
} VramState;

/* Inter-node spike message record (genesis-core/src/ipc.rs:395-403, bindings.cu:371-374). */
typedef struct __attribute__((packed)) SpikeEvent {
  uint32_t ghost_id;
  uint32_t tick_offset;
} SpikeEvent;

/* ===================================================================== */
/* Drop-in boundary: genesis-compute/src/ffi.rs                           */
/* ===================================================================== */

/* ffi.rs:57 / bindings.cu:571-631.  One zero-filled state allocation sliced
 * in blob order, one heads allocation filled with the sentinel. */
int32_t cu_allocate_shard(uint32_t padded_n, uint32_t total_axons, ShardVramPtrs* out_vram);

/* ffi.rs:63 / physics.cu:497-501.  flags &= 0xF1 on the stream. */
void cu_reset_burst_counters(const ShardVramPtrs* ptrs, uint32_t padded_n, void* stream);

/* ffi.rs:72 / bindings.cu:638-653.  Synchronous copy of the whole .state blob. */
int32_t cu_upload_state_blob(const ShardVramPtrs* vram, const void* state_blob, size_t state_size);

/* ffi.rs:80 / bindings.cu:658-669.  Synchronous copy of a .axons blob (may be
 * shorter than total_axons; the rest keeps its sentinel fill). */
int32_t cu_upload_axons_blob(const ShardVramPtrs* vram, const void* axons_blob, size_t axons_size);

/* ffi.rs:87 / bindings.cu:675-692.  Frees both allocations, nulls the pointers. */
void cu_free_shard(ShardVramPtrs* vram);

/* ffi.rs:90-106 / physics.cu:441-495.  One Day Phase tick, asynchronous on
 * `stream`.  NULL pointers / zero counts skip the input, network and readout
 * stages.  Returns the launch status (the reference always returned 0). */
int32_t cu_step_day_phase(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                          uint32_t v_seg, uint32_t current_tick, const uint32_t* input_bitmask,
                          uint32_t virtual_offset, uint32_t num_virtual_axons,
                          const uint32_t* incoming_spikes, uint32_t num_incoming_spikes,
                          const uint32_t* mapped_soma_ids, uint8_t* output_history,
                          uint32_t num_outputs, int16_t dopamine, void* stream);

/* ffi.rs:109 / physics.cu:504-506.  Synchronous upload of the 16-entry LUT
 * shared by every shard in the process. */
int32_t cu_upload_constant_memory(const VariantParameters* lut);

/* ffi.rs:114-154 / bindings.cu:214-265.  Memory and stream helpers. */
void* gpu_malloc(size_t size);
void gpu_free(void* dev_ptr);
void* gpu_host_alloc(size_t size);
void gpu_host_free(void* ptr);
void gpu_memcpy_host_to_device_async(void* dst, const void* src, size_t size, void* stream);
void gpu_memcpy_device_to_host_async(void* dst, const void* src, size_t size, void* stream);
bool gpu_memcpy_host_to_device(void* dst_dev, const void* src_host, size_t size);
/* ffi.rs:140-144 declares bool; bindings.cu:248 defined void.  bool here. */
bool gpu_memcpy_device_to_host(void* dst_host, const void* src_dev, size_t size);
int32_t gpu_stream_create(void** out_stream); /* non-blocking stream, bindings.cu:257-259 */
int32_t gpu_stream_destroy(void* stream);
void gpu_stream_synchronize(void* stream);
void gpu_set_device(int32_t device_id);
void gpu_device_synchronize(void);
void gpu_synchronize(void);

/* ffi.rs:157-158 / bindings.cu:267-282.  LUT uploads (1024 bytes). */
void gpu_load_constants(const void* host_ptr);
void update_constant_memory_hot_reload(const VariantParameters* new_variants, void* stream);

/* ffi.rs:160-164 / bindings.cu:450-515,699-710.  Night Phase sort-and-prune
 * of every neuron's 128 slots (legacy stream, asynchronous). */
void launch_sort_and_prune(const ShardVramPtrs* ptrs, uint32_t padded_n, int16_t prune_threshold);

/* ffi.rs:166-176 / bindings.cu:378-436.  Emits one SpikeEvent per head born
 * inside the last `sync_batch_ticks` ticks of each boundary axon.  Resets
 * *out_count first.  Events are written in (axon order, head order) — a
 * deterministic order; the reference's atomic order was not. */
void launch_extract_outgoing_spikes(const BurstHeads8* axon_heads, const uint32_t* src_indices,
                                    const uint32_t* dst_ghost_ids, uint32_t count,
                                    uint32_t sync_batch_ticks, uint32_t v_seg, void* out_events,
                                    uint32_t* out_count, void* stream);

/* ffi.rs:178-185 / bindings.cu:341-368.  dst[dst_idx[i]] = src[src_idx[i]]
 * for src_idx < 2^31. */
void launch_ghost_sync(const BurstHeads8* src_heads, BurstHeads8* dst_heads,
                       const uint32_t* src_indices, const uint32_t* dst_indices, uint32_t count,
                       void* stream);

/* ffi.rs:193-233 / bindings.cu:106-207,295-334.  Legacy per-kernel launchers
 * on the legacy stream, kept linkable.  launch_update_neurons and
 * launch_apply_gsop are declared by ffi.rs:215-224 but defined nowhere in the
 * reference; here they run the same update / GSOP stages as cu_step_day_phase
 * (constants_ptr is ignored: the process LUT is used). */
void launch_inject_inputs(VramState vram, const uint32_t* bitmask, uint32_t current_tick,
                          uint32_t total_virtual_axons);
void launch_apply_spike_batch(VramState vram, const uint32_t* tick_schedule,
                              uint32_t tick_spikes_count);
void launch_propagate_axons(VramState vram, uint32_t v_seg);
void launch_update_neurons(VramState vram, const void* constants_ptr, uint32_t current_tick);
void launch_apply_gsop(VramState vram);
void launch_record_readout(VramState vram, const uint32_t* mapped_soma_ids, uint8_t* output_history,
                           uint32_t current_tick, uint32_t total_pixels);

/* ffi.rs:235-246 / bindings.cu:780-796, physics.cu:400-434.  Ballot/popc
 * compaction of the spiking soma ids into out_ids; *out_count is incremented
 * (the caller resets it, gpu_reset_telemetry_count resets the count of the
 * shard's internal list only).  Ids are written in ascending order. */
void gpu_reset_telemetry_count(const ShardVramPtrs* ptrs, void* stream);
void launch_extract_telemetry(const ShardVramPtrs* ptrs, uint32_t padded_n, uint32_t* out_ids,
                              uint32_t* out_count_pinned, void* stream);

/* ffi.rs:248-272 / bindings.cu:717-778.  Per-batch I/O buffers. */
int32_t cu_allocate_io_buffers(uint32_t input_words, uint32_t schedule_capacity,
                               uint32_t output_capacity, uint32_t** d_input_bitmask,
                               uint32_t** d_incoming_spikes, uint8_t** d_output_history);
int32_t cu_dma_h2d_io(uint32_t* d_input_bitmask, const uint32_t* h_input_bitmask,
                      uint32_t input_words, uint32_t* d_incoming_spikes,
                      const uint32_t* h_incoming_spikes, uint32_t schedule_capacity,
                      void* stream);
int32_t cu_dma_d2h_io(uint8_t* h_output_history, const uint8_t* d_output_history,
                      uint32_t output_capacity, void* stream);

/* ===================================================================== */
/* New entry points (axc_*)                                               */
/* ===================================================================== */

/* Error bits a tick can raise on the device.  The reference reads or writes
 * out of bounds in each of these cases; here the access is skipped, the bit
 * is set, and the host reads it with axc_shard_error_flags. */
#define AXC_ERR_TARGET_RANGE   0x1u /* dendrite target axon id >= total_axons or field 0 */
#define AXC_ERR_SOMA_AXON      0x2u /* soma_to_axon >= total_axons (and not 0xFFFFFFFF)  */
#define AXC_ERR_VIRTUAL_RANGE  0x4u /* virtual_offset + num_virtual_axons > total_axons   */
#define AXC_ERR_READOUT_RANGE  0x8u /* mapped_soma_id >= padded_n (and not 0xFFFFFFFF)   */
#define AXC_ERR_WAIT_LIMIT     0x10u /* a bounded on-device wait gave up; the kernel took
                                        its path without the staged data (results exact) */

/* Library version string. */
const char* axc_version(void);

/* Reads (and with clear != 0, clears) the error bits of a shard.  Synchronous. */
int32_t axc_shard_error_flags(const ShardVramPtrs* vram, uint32_t clear, uint32_t* out_flags);

/* Device spike list of the last tick of a shard: count and ascending ids.
 * out_ids may be NULL to read only the count.  Synchronous on `stream`. */
int32_t axc_last_spikes(const ShardVramPtrs* vram, uint32_t* out_count, uint32_t* out_ids,
                        uint32_t capacity, void* stream);

/* Batch engine: mirror of ShardEngine::step_day_phase_batch
 * (genesis-compute/src/compute/shard.rs:40-124).  Copies the batch's host
 * inputs (bitmask words_per_tick x batch, spike schedule max_spikes x batch)
 * into the device I/O buffers, resets the burst counters, then runs
 * `batch` ticks with global tick = tick_base + k.  The tick loop is captured
 * once into a CUDA graph per (shard, batch shape) and replayed.  The
 * neuron-major row copy the ticks run on is kept from one batch to the next
 * (its weights are written back to the .state blob at the end of every
 * batch).  The device decides before each batch whether to lay it out anew:
 * at every batch while the layout leaves more than an eighth of the live
 * slots outside its lit-sum groups (the weights are still freezing), then
 * after 100, 200, 400, ... up to every 1,600 ticks; and for sure after the
 * shard's memory or the LUT may have changed: after any entry point of this
 * library that writes them, per-tick calls, and axc_shard_invalidate.
 * h_output_history, when not NULL, receives num_outputs x batch bytes
 * (device to host on the stream).  h_spike_counts may be NULL (no network
 * spikes).  Asynchronous on `stream` unless h_output_history is given, in
 * which case the call returns after the output copy completed. */
typedef struct AxcIoBuffers {
  uint32_t* d_input_bitmask;
  uint32_t* d_incoming_spikes;
  uint8_t* d_output_history;
  uint32_t max_spikes_per_tick;
  uint32_t input_words_per_tick;
  uint32_t num_outputs;
} AxcIoBuffers;

int32_t axc_step_day_phase_batch(const ShardVramPtrs* vram, uint32_t padded_n,
                                 uint32_t total_axons, uint32_t sync_batch_ticks,
                                 const AxcIoBuffers* io, const uint32_t* h_input_bitmask,
                                 const uint32_t* h_incoming_spikes,
                                 const uint32_t* h_spike_counts, uint32_t virtual_offset,
                                 uint32_t num_virtual_axons, const uint32_t* mapped_soma_ids_device,
                                 uint32_t v_seg, int16_t dopamine, uint32_t tick_base,
                                 uint8_t* h_output_history, void* stream);

/* Zone batch: one batch of every shard of this GPU with the intra-GPU ghost
 * sync behind it, as one CUDA graph (captured once per zone shape).  It
 * equals, bit for bit, the reference node loop's batch
 * (genesis-node/src/node/mod.rs:330-420): ShardEngine::step_day_phase_batch
 * on every shard (here each shard's tick loop is a parallel branch of the
 * graph), the device barrier (mod.rs:388), then launch_ghost_sync for every
 * route in order (mod.rs:409-411), all before the call's stream moves on.
 * Each shard entry carries the arguments of axc_step_day_phase_batch; the
 * ghost routes copy heads src -> dst as launch_ghost_sync does.  A shard may
 * appear once.  Synchronous only when some shard asks for its output history
 * (as axc_step_day_phase_batch).  No counterpart call in the reference, which
 * issues these launches from the node loop one by one. */
typedef struct AxcZoneShard {
  ShardVramPtrs vram;
  uint32_t padded_n, total_axons;
  AxcIoBuffers io;
  const uint32_t* h_input_bitmask;    /* [batch][input_words_per_tick] or NULL */
  const uint32_t* h_incoming_spikes;  /* [batch][max_spikes_per_tick] or NULL */
  const uint32_t* h_spike_counts;     /* [batch] or NULL */
  uint32_t virtual_offset, num_virtual_axons;
  const uint32_t* mapped_soma_ids_device;
  uint32_t v_seg;
  int16_t dopamine;
  uint8_t* h_output_history;          /* num_outputs x batch bytes, or NULL */
} AxcZoneShard;

typedef struct AxcGhostRoute {
  uint32_t src_shard, dst_shard;      /* indices into the shard array */
  const uint32_t* d_src_indices;      /* device [count] */
  const uint32_t* d_dst_indices;      /* device [count] */
  uint32_t count;
} AxcGhostRoute;

int32_t axc_step_zone_batch(const AxcZoneShard* shards, uint32_t nshards, const AxcGhostRoute* routes,
                            uint32_t nroutes, uint32_t sync_batch_ticks, uint32_t tick_base, void* stream);

/* Double-buffered batch I/O for one shard: the device side of the
 * reference's input swapchain (genesis-node/src/network/io_server.rs:20-85)
 * and per-batch output download (genesis-node/src/node/shard_thread.rs:208-227).
 * The pipeline owns two device input bitmasks ([batch][words] u32), two
 * device output histories and two pinned host output histories
 * ([batch][num_outputs] u8), an upload stream and a download stream.
 * axc_io_pipeline_submit queues one batch and returns at once: the bitmask
 * goes up on the upload stream (into the buffer batch b - 2 used, once that
 * batch has read it), the batch runs on `stream` as axc_step_day_phase_batch
 * once its upload landed, and its output history comes down on the download
 * stream once it is done.  So the next batch's upload overlaps this batch's
 * ticks, and this batch's readout overlaps the next batch's ticks.  Pass the
 * bitmask from pinned memory for the copy to be asynchronous; the host buffer
 * may be rewritten after axc_io_pipeline_wait_input.  axc_io_pipeline_outputs
 * waits for the readout of the batch submitted `back` (0 or 1) submits ago and
 * returns its pinned output history, valid until two submits later.  No
 * counterpart call in the reference. */
int32_t axc_io_pipeline_create(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                               uint32_t sync_batch_ticks, uint32_t input_words_per_tick, uint32_t num_outputs,
                               const uint32_t* mapped_soma_ids_device, uint32_t virtual_offset,
                               uint32_t num_virtual_axons, uint32_t v_seg, void** out_handle);
int32_t axc_io_pipeline_submit(void* handle, const uint32_t* h_input_bitmask, int16_t dopamine,
                               uint32_t tick_base, void* stream);
int32_t axc_io_pipeline_outputs(void* handle, uint32_t back, const uint8_t** out_history);
int32_t axc_io_pipeline_wait_input(void* handle);
void axc_io_pipeline_destroy(void* handle);

/* Instrumented ticks for measurement: runs `ticks` ticks (tick = tick0 + k,
 * bitmask row k of the device array d_input_bitmask) without a graph, with
 * CUDA events recorded on `stream` around each stage.  engine 0: the
 * per-tick kernels of cu_step_day_phase; engine 1: the batch engine's
 * neuron-major kernels (the ticks then form one batch, rows built before and
 * weights written back after).  Sets out_ms[5] to the stage times in
 * milliseconds: engine 0 network ids, axons, update, push, GSOP; engine 1
 * network ids, prologue, the 8-lane pass, the lit-sum pass (both with GSOP;
 * each returns at once on the other's ticks), fix-up and push; and out_counts[7] to
 * the ticks' totals of evaluated slots, hits, spikes, GSOP slots, evaluated
 * (non-refractory) neurons, ticks on the lit-sum form and the slots that form
 * tested (the counters [1]..[7] of axc_shard_counters).  Synchronous. */
int32_t axc_profile_ticks(const ShardVramPtrs* vram, uint32_t padded_n, uint32_t total_axons,
                          uint32_t v_seg, uint32_t tick0, uint32_t ticks,
                          const uint32_t* d_input_bitmask, uint32_t words_per_tick,
                          uint32_t virtual_offset, uint32_t num_virtual, int16_t dopamine,
                          int32_t engine, void* stream, float* out_ms, uint64_t* out_counts);

/* Selects the kernels of axc_step_day_phase_batch: 1 (default) the
 * neuron-major batch engine, 0 the per-tick kernels of cu_step_day_phase.
 * A negative value only queries.  Returns the previous mode. */
int32_t axc_batch_engine_mode(int32_t mode);

/* Selects the kernels of cu_step_day_phase: 1 (default) the neuron-major row
 * engine, whose copy of the shard's dendrites (targets and weights by neuron,
 * the slots whose weights may still move first) lives across calls and whose
 * GSOP writes every weight it changes through to the .state blob, so that the
 * shard's memory after each tick is what the reference leaves; 0 the columnar
 * per-tick kernels.  The copy is rebuilt on the next tick after any entry
 * point of this library wrote the shard's .state (cu_upload_state_blob,
 * gpu_memcpy_host_to_device[_async] into it, launch_sort_and_prune,
 * launch_apply_gsop, the batch, population and learned engines) or uploaded
 * a LUT.  A negative value only queries.  Returns the previous mode. */
int32_t axc_tick_engine_mode(int32_t mode);

/* No counterpart in the reference.  A caller that writes a shard's targets,
 * weights, flags or soma_to_axon by other means than this library (its own
 * kernels, a raw cudaMemcpy) calls this before the next cu_step_day_phase or
 * axc_step_day_phase_batch, so that the row copy those entry points keep
 * (the per-tick copy across calls, the batch copy from one batch to the
 * next) is laid out anew.  Returns 0. */
int32_t axc_shard_invalidate(const ShardVramPtrs* vram);

/* Capacity of the batch engine's per-tick list of deferred GSOP slots
 * (default and maximum 4,194,304); beyond it the fix-up stage rescans every
 * spiker.  For tests of that path.  Returns the previous capacity. */
uint32_t axc_row_engine_fix_capacity(uint32_t cap);

/* Tries of the update pass's first wait for the fully-lit bitmap it stages
 * in shared memory (default 65,536).  A wait that runs out sets
 * AXC_ERR_WAIT_LIMIT and the pass continues without the bitmap (results
 * unchanged); before its block exits it waits again, always with the full
 * limit, so that no copy is left in flight.  0 makes every first wait give up
 * at once: for tests of that path.  Returns the previous value. */
uint32_t axc_row_engine_wait_limit(uint32_t tries);

/* Per-tick counters accumulated by the device since the last reset:
 *  [0] ticks, [1] evaluated slots (non-refractory neurons, up to first empty),
 *  [2] delivered hits, [3] GLIF+heartbeat spikes, [4] GSOP slots updated,
 *  [5] evaluated (non-refractory) neurons, [6] ticks the row engine ran on
 *  its lit-sum form (frozen slots on fully-lit axons added as one per-row
 *  sum; the other ticks scan every slot), [7] slots the lit-sum ticks tested
 *  one by one. */
int32_t axc_shard_counters(const ShardVramPtrs* vram, uint32_t reset, uint64_t out[8]);

/* Allocation-free outgoing-spike extraction.  No counterpart in the
 * reference: it is launch_extract_outgoing_spikes (same arguments, same
 * events in the same order) for callers that may not allocate device memory
 * at that point — for example a node loop that extracts spikes after every
 * batch while other shards keep their streams busy (cudaMalloc/cudaFree can
 * synchronize the whole device), or a deployment that reserves all device
 * memory at boot and forbids allocation in the per-batch loop.
 * Its scratch is a fixed 16 KiB device array inside this library, held by
 * every GPU that loads the library until the process exits; it covers at most
 * AXC_NOALLOC_MAX_BOUNDARY_AXONS boundary axons per call, and a larger
 * `count` returns cudaErrorInvalidValue without launching anything.
 * The first call on a device looks up the array's device address; make that
 * first call before any stream capture.  The address is kept for the life of
 * the process: after cudaDeviceReset it is stale, so a process that resets
 * a device must not call this entry point on that device again.  All calls
 * share the array: calls that overlap on the GPU (two streams, two threads)
 * race and must be serialised by the caller.  Returns 0 or the cudaError_t
 * of this call's own launches (an error left pending by an earlier call is
 * neither returned nor cleared). */
#define AXC_NOALLOC_MAX_BOUNDARY_AXONS (1u << 20)
int32_t axc_extract_outgoing_spikes_noalloc(const BurstHeads8* axon_heads,
                                            const uint32_t* src_indices,
                                            const uint32_t* dst_ghost_ids, uint32_t count,
                                            uint32_t sync_batch_ticks, uint32_t v_seg,
                                            void* out_events, uint32_t* out_count, void* stream);

/* ---- Batched population ------------------------------------------------ */
/* Many independent brains stepped together: every tick runs one launch per
 * stage for the whole population (axons + somas, update + GSOP, GSOP fix-up,
 * pushes), captured once into a CUDA graph of `ticks_per_graph` ticks.  Each
 * brain keeps its own state, heads, LUT, input bitmask and tick numbering, and
 * evolves exactly as if it ran alone through axc_step_day_phase_batch.  No
 * counterpart in the reference (which runs one brain per shard thread). */
typedef struct AxcPopBrainDesc {
  ShardVramPtrs vram;                 /* from cu_allocate_shard, state uploaded */
  uint32_t padded_n, total_axons;
  uint32_t virtual_offset, num_virtual;
  const uint32_t* d_input_bitmask;    /* device [ticks][words_per_tick], or NULL */
  uint32_t words_per_tick;
  uint32_t v_seg;
  const VariantParameters* d_lut;     /* device, 16 entries, this brain's LUT */
  int32_t dopamine;
  uint32_t tick_base;                 /* global tick of bitmask row 0 */
  uint32_t bitmask_ticks;             /* rows of d_input_bitmask: a run or tuning past them is
                                         refused with cudaErrorInvalidValue before any launch */
} AxcPopBrainDesc;

/* Kernel schedule of the population stages (chosen by axc_population_tune). */
typedef struct AxcPopSchedule {
  uint32_t lanes_per_neuron;   /* 8 or 16 */
  uint32_t update_blocks_per_sm;
  uint32_t aux_blocks_per_sm;  /* fix-up and push stages */
} AxcPopSchedule;

int32_t axc_population_create(const AxcPopBrainDesc* brains, uint32_t count, void** out_handle);
/* Runs ticks [tick0, tick0 + ticks) of every brain (bitmask row tick0 + t),
 * in graphs of ticks_per_graph ticks (ticks must be a multiple), with the
 * batch prologue/epilogue (row copy, weight write-back) once per call.
 * Refused (cudaErrorInvalidValue) when a brain's bitmask has fewer than
 * tick0 + ticks rows.  Asynchronous on `stream`. */
int32_t axc_population_run(void* handle, uint32_t tick0, uint32_t ticks, uint32_t ticks_per_graph,
                           void* stream);
/* Times every candidate schedule on `trial_ticks` ticks from the current
 * state and keeps the fastest (the trial ticks advance the brains like a run
 * would; states stay exact).  Writes the chosen schedule and, optionally, the
 * per-candidate milliseconds (out_ms[i] for candidate i, up to max_out). */
int32_t axc_population_tune(void* handle, uint32_t tick0, uint32_t trial_ticks, void* stream,
                            AxcPopSchedule* chosen, float* out_ms, uint32_t max_out);
int32_t axc_population_set_schedule(void* handle, const AxcPopSchedule* schedule);
/* Totals since creation: [0] ticks, [1] evaluated slots, [2] hits, [3] spikes,
 * [4] GSOP slots, [5] evaluated neurons; plus [6] the error bits of all brains. */
int32_t axc_population_counters(void* handle, uint64_t out[8]);
void axc_population_destroy(void* handle);
/* Capacity of the population's per-tick list of deferred GSOP slots (as
 * axc_row_engine_fix_capacity, for tests of the rescan path). */
uint32_t axc_population_fix_capacity(uint32_t cap);

/* ---- Learned-schedule engine ------------------------------------------- */
/* One brain stepped by the row engine, with a per-tile activity predictor (an
 * MLP 64 -> 128 -> 1, BF16 weights, FP32 accumulation; tiles of 1024 axons;
 * the output is a residual added to input 8, the tile's active-synapse
 * fraction of the tick just run, so zero weights are the last-tick rule)
 * choosing before every tick between the dense row pass and a sparse,
 * axon-driven gather through an inverted index, and sizing the per-tile
 * compaction buffers of the sparse form.  A tile that outgrows its buffer
 * makes the tick run dense, so every schedule gives the state of
 * axc_step_day_phase_batch bit for bit.  The LUT is the process LUT
 * (cu_upload_constant_memory).  No counterpart in the reference. */
typedef struct AxcLearnedDesc {
  ShardVramPtrs vram;                 /* from cu_allocate_shard, state uploaded */
  uint32_t padded_n, total_axons;
  uint32_t virtual_offset, num_virtual;
  const uint32_t* d_input_bitmask;    /* device [bitmask_ticks][words_per_tick], or NULL */
  uint32_t words_per_tick, bitmask_ticks;
  uint32_t v_seg;
  int32_t dopamine;
  uint32_t tick_base;                 /* global tick of bitmask row 0 */
  uint32_t sample_capacity;           /* (features, target) pairs kept for training */
} AxcLearnedDesc;

/* Builds the inverted index of the shard's current targets (synchronous). */
int32_t axc_learned_create(const AxcLearnedDesc* desc, void** out_handle);
/* Rebuilds the index after the targets changed (sort_and_prune, uploads).
 * Until then ticks whose targets checksum differs run dense (stat [8]). */
int32_t axc_learned_refresh(void* handle, void* stream);
/* policy -1: the predictor picks; 0: always dense; 1: always sparse with
 * exact (full fan-out) buffers.  Sparse is picked when
 * ratio * predicted active synapses < next tick's evaluated slots; a tile's
 * buffer holds prediction * (1 + margin) + slack synapses. */
int32_t axc_learned_set_policy(void* handle, int32_t policy, float ratio, float margin, uint32_t slack);
/* Records (features of tick t-1, active-synapse fraction of tick t) for every
 * tile on every sample_every-th tick while enabled; reset drops the pairs. */
int32_t axc_learned_collect(void* handle, uint32_t enable, uint32_t sample_every, uint32_t reset);
/* Runs ticks [tick0, tick0 + ticks) (bitmask rows), graphs of ticks_per_graph
 * ticks (ticks must be a multiple); asynchronous on `stream`. */
int32_t axc_learned_run(void* handle, uint32_t tick0, uint32_t ticks, uint32_t ticks_per_graph, void* stream);
/* Adam over the recorded pairs (first 90% train, last 10% validate):
 * out_loss[epochs] mean training MSE per epoch, *out_val validation MSE. */
int32_t axc_learned_train(void* handle, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                          float* out_loss, float* out_val, void* stream);
/* Host copies of the FP32 master parameters (W1[128][64], b1[128], w2[128],
 * b2); either pointer may be NULL.  Setting them resets the Adam moments. */
int32_t axc_learned_params(void* handle, float* host_out, const float* host_in);
int32_t axc_learned_samples(void* handle, uint32_t first, uint32_t count, float* host_x, float* host_y);
/* [0] ticks, [1] sparse ticks, [2] overflow re-runs, [3] schedule mismatches
 * against exact counts, [4] sum |predicted - actual| active synapses over
 * tiles, [5] sum actual, [6] judged ticks, [7] planned sparse, [8] stale-index
 * ticks, [9] ticks run with the predictor gated off, [12] recorded pairs,
 * [13] feature history length, [14] tiles, [15] index capacity.
 * Gate (policy -1, not collecting): a chunk of ticks_per_graph ticks in which
 * the predictor chose the dense form on every tick is followed by up to 64
 * chunks on the plain engine's graph (no features, no plan), then a probe
 * chunk with the predictor.  The gate ends early when a gated chunk's exact
 * counts say the sparse form could have won (ratio x hits x live slots <
 * evaluated slots squared, over the chunk); those counts are read back two
 * chunks behind, so the host never stalls the stream.  Dense ticks of both
 * graphs run the plain engine's passes, so the state is the same either way. */
int32_t axc_learned_stats(void* handle, uint64_t out[16]);
int32_t axc_learned_reset_stats(void* handle);
void axc_learned_destroy(void* handle);
uint32_t axc_mlp_param_count(void);
/* Mean squared error of the MLP (parameters FP32, rounded to BF16) over
 * count samples x[count][64], y[count], and its gradient d_grad[param_count]
 * (device buffers; synchronous). */
int32_t axc_mlp_loss_grad(const float* d_params, const float* d_x, const float* d_y, uint32_t count,
                          float* d_grad, float* d_loss, void* stream);
int32_t axc_mlp_predict(const float* d_params, const float* d_x, uint32_t count, float* d_out, void* stream);

/* ---- Synthetic brain generator (host) ---------------------------------- */
/* Neurons fill a dim_x*dim_y*dim_z voxel grid (x fastest, one per voxel);
 * neuron n owns axon n; input v owns virtual axon padded_n + v and sits on a
 * seeded distinct voxel.  Each neuron binds `slots` distinct presynaptic
 * axons (no self-synapse) drawn with probability proportional to
 * exp(-dist/lambda) over all neurons and inputs within `radius` voxels.  The
 * segment is 1 + floor(dist)/2 (two voxels per segment).  Weights are
 * uniform in [w_min, w_max], negative for inhibitory presynaptic neurons.  */
typedef struct AxcBrainSpec {
  uint32_t dim_x, dim_y, dim_z;
  uint32_t slots;              /* used dendrite slots per neuron (<= 128) */
  uint32_t num_inputs;         /* virtual input axons */
  uint32_t inhibitory_permille;/* 200 = 20% inhibitory */
  uint32_t radius;             /* sampling support, voxels */
  uint32_t lambda_voxels;      /* exp(-dist/lambda) */
  int32_t w_min, w_max;        /* |weight| range */
  uint64_t seed;
} AxcBrainSpec;

typedef struct AxcBrainLayout {
  uint32_t num_neurons;
  uint32_t padded_n;
  uint32_t total_axons;
  uint32_t virtual_offset;
  uint64_t state_bytes;
  uint64_t axons_bytes;
} AxcBrainLayout;

int32_t axc_brain_layout(const AxcBrainSpec* spec, AxcBrainLayout* out);
/* Writes the .state blob (layout.state_bytes) and .axons blob (all sentinel). */
int32_t axc_brain_generate(const AxcBrainSpec* spec, void* state_blob, void* axons_blob,
                           int32_t n_threads);
/* Seeded Bernoulli input bitmask, [ticks][ceil(num_inputs/32)] words; input v
 * fires at tick t when hash(seed, t, v) < p_q32[t % period] (p in Q0.32). */
int32_t axc_input_bitmask(uint64_t seed, uint32_t tick0, uint32_t ticks, uint32_t num_inputs,
                          const uint32_t* p_q32, uint32_t period, uint32_t* out_words);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* AXICOR_DAY_H */
