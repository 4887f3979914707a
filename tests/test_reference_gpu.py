"""The oracle against the reference's own CUDA kernels, run on the GPU.

The reference's update kernel reads other neurons' heads while spiking
neurons push theirs (physics.cu:194 vs :257-261); a neuron whose gather hit
result depends on whether such a push was already visible is "race-exposed".
The oracle fixes snapshot semantics, so it must agree with the reference on
every neuron that is not race-exposed, every tick.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from oracle import refgpu
from axicor_gb300 import _native as N
from axicor_gb300 import shard as S
from axicor_gb300 import workloads as W
from axicor_gb300.formats import StateView

pytestmark = pytest.mark.gpu
SENT = 0x80000000


def _push(h):
    h[..., 1:] = h[..., :-1].copy()
    h[..., 0] = 0


def exposed_neurons(state, heads, lut, N_, A, voff, nv, bm, v_seg, spikers):
    """Neurons whose gather differs between pre-push and post-push heads this tick."""
    H = heads.reshape(-1, 8).copy()
    if nv:
        bits = np.unpackbits(bm.view(np.uint8), bitorder="little")[:nv].astype(bool)
        idx = voff + np.nonzero(bits)[0]
        sub = H[idx].copy()
        _push(sub)
        H[idx] = sub
    live = H != SENT
    H[live] += np.uint32(v_seg)
    sv = StateView(state, N_)
    pushed = np.zeros(A, bool)
    s2a = sv.soma_to_axon[spikers]
    pushed[s2a[s2a < A]] = True
    Hp = H.copy()
    pa = np.nonzero(pushed)[0]
    tmp = Hp[pa].copy()
    _push(tmp)
    Hp[pa] = tmp
    T = sv.targets.astype(np.uint64)
    valid = np.cumprod(T != 0, axis=0).astype(bool)
    ax = ((T & 0xFFFFFF) - 1).astype(np.int64)
    seg = (T >> 24).astype(np.uint32)
    prop = lut["signal_propagation_length"][(sv.flags >> 4) & 15].astype(np.uint32)
    m = valid & (ax >= 0) & (ax < A) & pushed[np.clip(ax, 0, A - 1)]
    out = set()
    for i, n in zip(*np.nonzero(m)):
        a, s, p = ax[i, n], seg[i, n], prop[n]
        pre = np.any(((H[a] - s) & 0xFFFFFFFF) < p)
        post = np.any(((Hp[a] - s) & 0xFFFFFFFF) < p)
        if pre != post:
            out.add(int(n))
    return out


@pytest.mark.parametrize("case", ["default", "adaptive", "dopamine_inertia", "network"])
def test_oracle_matches_reference_kernels(gpu, case):
    if not refgpu.available():
        pytest.skip("reference cubin absent (built from the reference sources by oracle/build_ref.py)")
    from test_parity_gpu import lut_adaptive, lut_inertia
    rk = refgpu.ReferenceKernels()
    w = W.small(dims=(16, 16, 8), slots=64, inputs=64, p=0.1)
    dop = 0
    if case == "adaptive":
        w.lut = lut_adaptive()
    elif case == "dopamine_inertia":
        w.lut = lut_inertia()
        w.w_max = 5000
        dop = 90
    lay, state, heads = S.generate_brain(w.spec())
    rk.upload_lut(w.lut)
    Np, A = lay.padded_n, lay.total_axons
    vram = S.VramState(Np, A)
    lib = N.lib()
    words = (w.num_inputs + 31) // 32
    d_bm = lib.gpu_malloc(words * 4)
    ids = np.arange(Np, dtype=np.uint32)
    d_ids = S.device_array(ids)
    d_out = lib.gpu_malloc(Np)
    d_in = lib.gpu_malloc(4 * 256)
    rng = np.random.default_rng(9)
    h_state, h_heads = state.copy(), heads.copy()
    exposed_total, checked = 0, 0
    try:
        for t in range(80):
            vram.upload_state(h_state)
            vram.upload_axon_heads(h_heads)
            bm = S.input_bitmask(w.seed, t, 1, w.num_inputs, w.rate_q32)
            assert lib.gpu_memcpy_host_to_device(d_bm, N.ptr(bm), bm.nbytes)
            inc = None
            if case == "network":   # distinct ids: duplicates race in the reference (physics.cu:124-131)
                inc = rng.choice(A, size=64, replace=False).astype(np.uint32)
                assert lib.gpu_memcpy_host_to_device(d_in, N.ptr(inc), inc.nbytes)
            pre_state, pre_heads = h_state.copy(), h_heads.copy()
            rk.step(vram, Np, A, 1, t, d_bm, lay.virtual_offset, w.num_inputs, d_in if inc is not None else None,
                    0 if inc is None else inc.size, d_ids, d_out, Np, dop)
            g_state, g_heads = vram.download_state(), vram.download_heads()
            g_out = np.empty(Np, np.uint8)
            assert lib.gpu_memcpy_device_to_host(N.ptr(g_out), d_out, Np)
            o_out = np.empty(Np, np.uint8)
            oracle.step(h_state, h_heads, w.lut, Np, A, 1, t, bm, lay.virtual_offset, w.num_inputs, incoming=inc,
                        mapped_soma_ids=ids, outputs=o_out, dopamine=dop)
            assert np.array_equal(g_heads, h_heads), f"tick {t}: heads differ"
            if np.array_equal(g_state, h_state) and np.array_equal(g_out, o_out):
                checked += 1
                continue
            spikers = np.nonzero(StateView(h_state, Np).flags & 1)[0]
            exp = exposed_neurons(pre_state, pre_heads, w.lut, Np, A, lay.virtual_offset, w.num_inputs, bm, 1,
                                  spikers)
            gs, hs = StateView(g_state, Np), StateView(h_state, Np)
            bad = set(np.nonzero(gs.voltage != hs.voltage)[0]) | set(np.nonzero(gs.flags != hs.flags)[0]) | \
                set(np.nonzero((gs.weights != hs.weights).any(0))[0])
            assert bad <= exp, f"tick {t}: {len(bad - exp)} non-exposed neurons differ"
            exposed_total += len(bad)
            h_state, h_heads = g_state, g_heads    # continue from the reference's state
        assert checked >= 70, f"only {checked} of 80 ticks identical (race-exposed neurons: {exposed_total})"
    finally:
        for p in (d_bm, d_ids, d_out, d_in):
            lib.gpu_free(p)
        vram.free()


@pytest.mark.parametrize("config", ["config1", "config0"])
def test_reference_kernels_against_batch_path_on_config1(gpu, config):
    """The reference's own Day Phase kernels (physics.cu compiled for sm_103a, launched in
    cu_step_day_phase's order) and this engine's batch path on the 1.5M brain (and the 16k brain) in
    its steady state (after 700 ticks), the same 100 ticks from the same state on the same GPU, timed
    with CUDA events on each launching stream.  Prints one JSON line; the engine must be faster."""
    if not refgpu.available():
        pytest.skip("reference cubin absent (built from the reference sources by oracle/build_ref.py)")
    import json
    import torch
    w = getattr(W, config)()
    lay, state, heads = S.generate_brain(w.spec())
    S.upload_lut(w.lut)
    Np, A = lay.padded_n, lay.total_axons
    vram = S.VramState(Np, A)
    vram.upload_state(state)
    vram.upload_axon_heads(heads)
    del state, heads
    eng = S.ShardEngine(vram)
    lib = N.lib()
    words = (w.num_inputs + 31) // 32
    warm, T = 700, 100
    bm = S.input_bitmask(w.seed, 0, warm + T, w.num_inputs, w.rate_q32)
    io = S.IoDeviceBuffers(words, 0, 0, 100)
    for t in range(0, warm, 100):
        eng.step_day_phase_batch(100, io, bm[t * words:(t + 100) * words], None, None, lay.virtual_offset,
                                 w.num_inputs, None, 1, 0, t)
    eng.synchronize()
    st0, hd0 = vram.download_state(), vram.download_heads()
    rows = bm[warm * words:(warm + T) * words]
    d_bm = S.device_array(rows)
    try:
        # this engine: one batch of T ticks through axc_step_day_phase_batch (graph captured first, untimed)
        eng.step_day_phase_batch(T, io, rows, None, None, lay.virtual_offset, w.num_inputs, None, 1, 0, warm)
        eng.synchronize()
        vram.upload_state(st0)
        vram.upload_axon_heads(hd0)
        es = torch.cuda.ExternalStream(eng.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(es)
        assert lib.axc_step_day_phase_batch(C.byref(vram.ptrs), Np, A, T, C.byref(io.as_struct()), d_bm, None,
                                            None, lay.virtual_offset, w.num_inputs, None, 1, 0, warm, None,
                                            eng.stream) == 0
        e1.record(es)
        torch.cuda.synchronize()
        ours_s = e0.elapsed_time(e1) / 1e3
        # the reference's kernels: the same ticks from the same state, on the legacy default stream
        vram.upload_state(st0)
        vram.upload_axon_heads(hd0)
        rk = refgpu.ReferenceKernels()
        rk.upload_lut(w.lut)
        rk.step(vram, Np, A, 1, warm, d_bm, lay.virtual_offset, w.num_inputs, None, 0, None, None, 0, 0)  # warm
        vram.upload_state(st0)
        vram.upload_axon_heads(hd0)
        default = torch.cuda.default_stream()
        torch.cuda.synchronize()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(default)
        for k in range(T):
            rk.step(vram, Np, A, 1, warm + k, d_bm + k * words * 4, lay.virtual_offset, w.num_inputs, None, 0,
                    None, None, 0, 0, sync=False)
        r1.record(default)
        torch.cuda.synchronize()
        ref_s = r0.elapsed_time(r1) / 1e3
        synapses = int(np.count_nonzero(StateView(st0, Np).targets))
        print(json.dumps({"workload": w.name, "ticks": [warm, warm + T],
                          "reference_kernels_ticks_per_s": T / ref_s,
                          "reference_kernels_events_per_s": T * synapses / ref_s,
                          "engine_ticks_per_s": T / ours_s, "engine_events_per_s": T * synapses / ours_s,
                          "speedup": ref_s / ours_s}))
        assert ours_s < ref_s
    finally:
        lib.gpu_free(d_bm)
        vram.free()
