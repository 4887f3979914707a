// brain_gen.cpp — seeded synthetic brain generator (host).
//
// Writes the reference's on-disk formats directly:
//   .state  — SoA blob in ShardVramPtrs order, 910 B per padded neuron
//             (genesis-compute/src/memory.rs:71-86, genesis-baker/src/bake/layout.rs:127-159)
//   .axons  — BurstHeads8[total_axons], all heads at the sentinel
//             (bindings.cu:560-568, genesis-baker/src/bake/layout.rs:162-169)
// Axon numbering follows the runtime convention: neuron n owns axon n, input
// v owns virtual axon padded_n + v (virtual_offset = padded_n + ghosts, with
// no ghosts, genesis-compute/src/memory.rs:128-130), and
// total_axons = align32(padded_n + inputs) (genesis-node/src/boot.rs:64-71).
// Targets are packed as (seg << 24) | (axon + 1)
// (genesis-core/src/layout.rs:254-265).
//
// Every random draw is a counter-based hash (the wyhash-style entity_seed of
// genesis-core/src/seed.rs:50-57), so the bytes depend only on (spec, seed)
// and not on the thread count.  The distance weights use only IEEE basic
// operations (this file is compiled with -ffp-contract=off), so x86-64 and
// aarch64 hosts produce identical brains.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

#include "../../include/axicor_day.h"

namespace {

// genesis-core/src/seed.rs:50-57
inline uint64_t entity_seed(uint64_t master, uint32_t id) {
  uint64_t seed = master + (uint64_t)id + 0x60bee2bee120fc15ULL;
  __uint128_t tmp = (__uint128_t)seed * (__uint128_t)0xa3b195354a39b70dULL;
  __uint128_t m1 = (tmp >> 64) ^ tmp;
  tmp = m1 * (__uint128_t)0x1b03738712fad5c9ULL;
  return (uint64_t)((tmp >> 64) ^ tmp);
}

inline uint64_t mulhi64(uint64_t a, uint64_t b) {
  return (uint64_t)(((__uint128_t)a * (__uint128_t)b) >> 64);
}

// e^{-x} for x >= 0 from basic operations only: halve until x <= 1/16,
// 16-term Taylor series, square back.
double det_exp_neg(double x) {
  int k = 0;
  double y = x;
  while (y > 0.0625) { y *= 0.5; k++; }
  double term = 1.0, sum = 1.0;
  for (int i = 1; i <= 16; i++) { term = term * (-y) / (double)i; sum += term; }
  while (k-- > 0) sum = sum * sum;
  return sum;
}

uint32_t isqrt_u32(uint32_t v) {
  uint32_t r = (uint32_t)std::sqrt((double)v);
  while ((uint64_t)r * r > v) r--;
  while ((uint64_t)(r + 1) * (r + 1) <= v) r++;
  return r;
}

struct OffsetTable {
  // offsets grouped in shells of equal squared distance
  std::vector<int32_t> dx, dy, dz;
  std::vector<uint32_t> shell_d2, shell_start, shell_count;
  std::vector<uint64_t> shell_cdf;  // inclusive prefix of count*weight
  uint64_t total = 0;
};

OffsetTable build_offsets(uint32_t radius, uint32_t lambda) {
  OffsetTable t;
  const int R = (int)radius;
  const uint32_t r2max = radius * radius;
  std::vector<std::vector<int32_t>> by_d2(r2max + 1);
  for (int z = -R; z <= R; z++)
    for (int y = -R; y <= R; y++)
      for (int x = -R; x <= R; x++) {
        uint32_t d2 = (uint32_t)(x * x + y * y + z * z);
        if (d2 == 0 || d2 > r2max) continue;
        by_d2[d2].push_back(x);
        by_d2[d2].push_back(y);
        by_d2[d2].push_back(z);
      }
  uint64_t acc = 0;
  for (uint32_t d2 = 1; d2 <= r2max; d2++) {
    if (by_d2[d2].empty()) continue;
    double w = det_exp_neg(std::sqrt((double)d2) / (double)lambda);
    uint64_t wq = (uint64_t)(w * 1099511627776.0);  // 2^40
    if (wq == 0) continue;
    uint32_t cnt = (uint32_t)(by_d2[d2].size() / 3);
    t.shell_d2.push_back(d2);
    t.shell_start.push_back((uint32_t)t.dx.size());
    t.shell_count.push_back(cnt);
    for (uint32_t i = 0; i < cnt; i++) {
      t.dx.push_back(by_d2[d2][3 * i]);
      t.dy.push_back(by_d2[d2][3 * i + 1]);
      t.dz.push_back(by_d2[d2][3 * i + 2]);
    }
    acc += wq * cnt;
    t.shell_cdf.push_back(acc);
  }
  t.total = acc;
  return t;
}

bool spec_ok(const AxcBrainSpec* s) {
  if (!s) return false;
  uint64_t n = (uint64_t)s->dim_x * s->dim_y * s->dim_z;
  if (n == 0 || n > (1ull << 24) - 2) return false;
  if (s->slots > AXC_MAX_DENDRITES) return false;
  if (s->radius == 0 || s->radius > 124 || s->lambda_voxels == 0) return false;
  if (s->w_min < 0 || s->w_max < s->w_min || s->w_max > 32767) return false;
  if (s->inhibitory_permille > 1000) return false;
  uint64_t padded = (n + 63) & ~63ull;
  uint64_t axons = (padded + s->num_inputs + 31) & ~31ull;
  if (axons >= (1ull << 24) - 1) return false;  // 24-bit axon ids (layout.rs:256)
  return true;
}

}  // namespace

extern "C" {

int32_t axc_brain_layout(const AxcBrainSpec* spec, AxcBrainLayout* out) {
  if (!spec_ok(spec) || !out) return -1;
  uint64_t n = (uint64_t)spec->dim_x * spec->dim_y * spec->dim_z;
  uint64_t padded = (n + 63) & ~63ull;                       // layout.rs:77-79
  uint64_t axons = (padded + spec->num_inputs + 31) & ~31ull; // boot.rs:69-71
  out->num_neurons = (uint32_t)n;
  out->padded_n = (uint32_t)padded;
  out->total_axons = (uint32_t)axons;
  out->virtual_offset = (uint32_t)padded;
  out->state_bytes = padded * (4 + 1 + 4 + 1 + 4) + padded * AXC_MAX_DENDRITES * (4 + 2 + 1);
  out->axons_bytes = axons * sizeof(BurstHeads8);
  return 0;
}

int32_t axc_brain_generate(const AxcBrainSpec* spec, void* state_blob, void* axons_blob,
                           int32_t n_threads) {
  AxcBrainLayout L;
  if (axc_brain_layout(spec, &L) != 0 || !state_blob) return -1;
  const uint32_t N = L.num_neurons, P = L.padded_n;
  const uint32_t X = spec->dim_x, Y = spec->dim_y, Z = spec->dim_z;
  const uint32_t S = spec->slots, I = spec->num_inputs;
  if (n_threads <= 0) n_threads = omp_get_max_threads();

  uint8_t* b = (uint8_t*)state_blob;
  std::memset(b, 0, L.state_bytes);
  int32_t* voltage = (int32_t*)b;
  uint8_t* flags = b + (size_t)P * 4;
  uint32_t* s2a = (uint32_t*)(b + (size_t)P * 10);
  uint32_t* targets = (uint32_t*)(b + (size_t)P * 14);
  int16_t* weights = (int16_t*)(b + (size_t)P * 14 + (size_t)P * AXC_MAX_DENDRITES * 4);
  (void)voltage;  // rest potential 0 for every generated variant

  const uint64_t seed_type = entity_seed(spec->seed, 1);
  const uint64_t seed_syn = entity_seed(spec->seed, 2);
  const uint64_t seed_w = entity_seed(spec->seed, 3);
  const uint64_t seed_in = entity_seed(spec->seed, 4);

  // neuron types: variant 1 (inhibitory) with probability permille/1000
  std::vector<uint8_t> inhib(N);
#pragma omp parallel for schedule(static) num_threads(n_threads)
  for (int64_t n = 0; n < (int64_t)N; n++) {
    uint64_t h = entity_seed(seed_type, (uint32_t)n);
    inhib[n] = mulhi64(h, 1000) < spec->inhibitory_permille ? 1 : 0;
    flags[n] = (uint8_t)(inhib[n] << 4);  // flags = variant << 4 (baker topology.rs:167)
    s2a[n] = (uint32_t)n;
  }
  for (uint32_t n = N; n < P; n++) s2a[n] = AXC_NO_AXON;  // padding (bake/layout.rs:83)

  // inputs on distinct seeded voxels
  std::vector<int32_t> vox_input(N, -1);
  for (uint32_t v = 0; v < I; v++) {
    for (uint32_t att = 0;; att++) {
      uint64_t h = entity_seed(entity_seed(seed_in, v), att);
      uint32_t vox = (uint32_t)mulhi64(h, N);
      if (vox_input[vox] < 0) { vox_input[vox] = (int32_t)v; break; }
      if (att > 1000000u) return -2;  // more inputs than voxels
    }
  }

  const OffsetTable T = build_offsets(spec->radius, spec->lambda_voxels);
  std::vector<uint32_t> seg_of_d2(spec->radius * spec->radius + 1);
  for (uint32_t d2 = 0; d2 < seg_of_d2.size(); d2++)
    seg_of_d2[d2] = std::min<uint32_t>(63u, 1u + isqrt_u32(d2) / 2u);
  const uint32_t wspan = (uint32_t)(spec->w_max - spec->w_min + 1);
  const uint64_t max_attempts = 64ull * S + 4096;

#pragma omp parallel num_threads(n_threads)
  {
    uint32_t set[512];
#pragma omp for schedule(static, 256)
    for (int64_t nn = 0; nn < (int64_t)N; nn++) {
      const uint32_t n = (uint32_t)nn;
      const int32_t x = (int32_t)(n % X), y = (int32_t)((n / X) % Y), z = (int32_t)(n / (X * Y));
      std::memset(set, 0xFF, sizeof(set));
      const uint64_t base = entity_seed(seed_syn, n);
      const uint64_t wbase = entity_seed(seed_w, n);
      uint32_t cnt = 0;
      for (uint64_t att = 0; cnt < S && att < max_attempts; att++) {
        uint64_t u1 = entity_seed(base, (uint32_t)(2 * att));
        uint64_t u2 = entity_seed(base, (uint32_t)(2 * att + 1));
        uint64_t r = mulhi64(u1, T.total);
        size_t sh = (size_t)(std::upper_bound(T.shell_cdf.begin(), T.shell_cdf.end(), r) -
                             T.shell_cdf.begin());
        if (sh >= T.shell_cdf.size()) continue;
        uint32_t k = T.shell_start[sh] + (uint32_t)mulhi64(u2 >> 1, (uint64_t)T.shell_count[sh] << 1);
        int32_t tx = x + T.dx[k], ty = y + T.dy[k], tz = z + T.dz[k];
        if (tx < 0 || ty < 0 || tz < 0 || tx >= (int32_t)X || ty >= (int32_t)Y || tz >= (int32_t)Z)
          continue;
        uint32_t m = (uint32_t)tx + X * ((uint32_t)ty + Y * (uint32_t)tz);
        uint32_t axon;
        bool inhibitory = false;
        if ((u2 & 1) == 0) {
          if (m == n) continue;  // no self-synapse (dendrite_connect.rs:52)
          axon = m;
          inhibitory = inhib[m] != 0;
        } else {
          if (vox_input[m] < 0) continue;
          axon = P + (uint32_t)vox_input[m];
        }
        // distinct presynaptic axon per neuron (dendrite_connect.rs:62-65)
        uint32_t hsh = (axon * 2654435761u) >> 23;
        bool dup = false;
        while (set[hsh] != 0xFFFFFFFFu) {
          if (set[hsh] == axon) { dup = true; break; }
          hsh = (hsh + 1) & 511u;
        }
        if (dup) continue;
        set[hsh] = axon;
        uint32_t seg = seg_of_d2[T.shell_d2[sh]];
        uint64_t col = (uint64_t)cnt * P + n;
        targets[col] = (seg << AXC_TARGET_SEG_SHIFT) | (axon + 1u);
        uint64_t hw = entity_seed(wbase, cnt);
        int32_t aw = spec->w_min + (int32_t)mulhi64(hw, wspan);
        weights[col] = (int16_t)(inhibitory ? -aw : aw);
        cnt++;
      }
    }
  }

  if (axons_blob) {
    uint32_t* h = (uint32_t*)axons_blob;
    for (uint64_t i = 0; i < (uint64_t)L.total_axons * 8; i++) h[i] = AXC_AXON_SENTINEL;
  }
  return 0;
}

int32_t axc_input_bitmask(uint64_t seed, uint32_t tick0, uint32_t ticks, uint32_t num_inputs,
                          const uint32_t* p_q32, uint32_t period, uint32_t* out_words) {
  if (!p_q32 || period == 0 || !out_words) return -1;
  const uint32_t words = (num_inputs + 31) / 32;
  const uint64_t seed_bits = entity_seed(seed, 5);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)ticks; k++) {
    uint32_t t = tick0 + (uint32_t)k;
    uint64_t pq = p_q32[t % period];
    uint64_t tseed = entity_seed(seed_bits, t);
    uint32_t* w = out_words + (size_t)k * words;
    std::memset(w, 0, words * 4);
    for (uint32_t v = 0; v < num_inputs; v++) {
      uint64_t h = entity_seed(tseed, v);
      if ((h >> 32) < pq) w[v / 32] |= 1u << (v % 32);
    }
  }
  return 0;
}

}  // extern "C"
