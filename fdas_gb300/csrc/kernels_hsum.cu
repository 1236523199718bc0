// (d) harmonic summing, thresholding and candidate compaction; FP64 recheck of
// near-threshold cells; per-plane sort and the fixed-size candidate list.
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include <utility>
#include <type_traits>

#include "kernels.cuh"

namespace fdas {

template <typename F, int... I>
__device__ __forceinline__ void hs_sfor_impl(F &&f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void hs_sfor(F &&f) {
  hs_sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// one record appended to the global list (single-thread use)
__device__ __forceinline__ void global_append(unsigned long long *keys, float *pwrs, unsigned *total, int cap,
                                              int *status, unsigned long long key, float pwr) {
  const unsigned g = atomicAdd(total, 1u);
  if (g < (unsigned)cap) {
    keys[g] = key;
    pwrs[g] = pwr;
  } else {
    atomicOr(status, kStatusCandidateOverflow);
  }
}

// Per-CTA hit counts per plane (shared memory), added to the global counts
// when the CTA ends.
struct EmitBuf {
  unsigned pc[kMaxPlanes];  // hits per plane of this CTA
};

// Persistent harmonic summing.  Work item = (256-bin block, sign half),
// handed out dynamically through a global counter.  A CTA has NW consumer
// warps -- warp w owns templates |t| = 4w + k (k < 4), lane l the bins
// f0 + 4 l + c and f0 + 128 + 4 l + c (c < 4), i.e. a 4 x 8 tile of cells --
// and one producer warp.  For every item the producer issues one 2-D TMA
// tensor copy per plane (cp.async.bulk.tensor.2d): plane 1 as 256 bins x 4 NW
// rows, plane j >= 2 as the rows trunc(t/j) of the half over bins
// [(f0/j) & ~3, ...); rows and bins outside the FOP are zero-filled by the
// hardware (they only feed masked cells).  kHsStages stages deep: full / empty
// mbarriers, every wait bounded by %globaltimer.
//
// Planes 2, 4 and 8 read their values with 8- and 4-byte loads at
// compile-time offsets; for planes 3, 5, 6, 7 the eight bins map onto offsets
// from two divisions per plane and the four rows onto two staged rows split at
// a warp-uniform point, handled by a switch.
//
// HP_1 = FOP[t][f], HP_j = HP_{j-1} + FOP[trunc(t/j)][f/j] accumulated in FP32
// in this order -- hsum.py:95-120 / hms_baseline.cl.mako:55-84 -- so the
// values match hsum.py bit for bit for the same FOP.  A cell is a candidate of
// plane j if HP_j > thr_j (strict, hsum.py:134 / detect.cl.mako:185).  The fast
// path only tracks a bound of the tile maximum per plane and marks the planes
// where some lane of the warp reaches the lower edge of the band; at the end
// of the item, while the stage is still held, the warp recomputes its sums
// plane by plane (same values, same order) and emits at the marked planes.
struct HsItem {
  int f0, sgn, tlo;
};

__device__ __forceinline__ HsItem hs_item(const HsumParams &p, int it) {
  // items enumerate (block, half) over the enabled halves, highest blocks
  // first: a signal's harmonic images cover wider bin ranges at higher bins
  // (plane j sums f/k for k <= j), so the items that emit most are handed
  // out early and the light ones fill the end of the launch
  const bool neg = p.tlo[0] <= p.half, pos = p.tlo[1] <= p.half;
  const int nb = (p.n_bins + kHsBins - 1) / kHsBins;
  int blk, halfsel;
  if (neg && pos) { blk = it >> 1; halfsel = it & 1; }
  else { blk = it; halfsel = pos ? 1 : 0; }
  return HsItem{(nb - 1 - blk) * kHsBins, halfsel ? 1 : -1, p.tlo[halfsel]};
}

__device__ __forceinline__ int hs_n_items(const HsumParams &p) {
  const int nb = (p.n_bins + kHsBins - 1) / kHsBins;
  return nb * ((p.tlo[0] <= p.half) + (p.tlo[1] <= p.half));
}

__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
// maximum of the 32 cells of a tile (3-input max tree)
__device__ __forceinline__ float max32(const float (&a)[4][8]) {
  float m[4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    m[k] = fmax3(fmax3(a[k][0], a[k][1], a[k][2]), fmax3(a[k][3], a[k][4], a[k][5]), fmaxf(a[k][6], a[k][7]));
  return fmax3(m[0], m[1], fmaxf(m[2], m[3]));
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_wait_parity(uint64_t *bar, uint32_t parity, long long timeout_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity))
    if ((long long)(globaltimer_ns() - t0) > timeout_ns) return false;
  return true;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// smem row of staged row r (r = |t| or trunc(|t|/j)) in a box of bh rows: the
// boxes hold FOP rows in ascending order, i.e. reversed for the negative half
__device__ __forceinline__ int srow(int r, int bh, int sgn) { return sgn > 0 ? r : bh - 1 - r; }

// (a0, a1) += (b0, b1) as one packed FP32 pair instruction (add.rn.f32x2,
// sm_100 and later): each half is an ordinary round-to-nearest FP32 add, so
// the sums are the scalar ones bit for bit
__device__ __forceinline__ void add2(float &a0, float &a1, float b0, float b1) {
  unsigned long long a, b, d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "f"(a0), "f"(a1));
  asm("mov.b64 %0, {%1, %2};" : "=l"(b) : "f"(b0), "f"(b1));
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(d));
}

// acc[k][e] += (k < KS ? c0[e] : c1[e]), KS compile time
template <int KS>
__device__ __forceinline__ void add_rows(float (&acc)[4][8], const float (&c0)[8], const float (&c1)[8]) {
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      if (k < KS) add2(acc[k][e], acc[k][e + 1], c0[e], c0[e + 1]);
      else add2(acc[k][e], acc[k][e + 1], c1[e], c1[e + 1]);
    }
}

// Plane 1 of the warp's tile: 4 templates x 8 bins; cells outside the
// item's rows or beyond n_bins are -inf (they never reach a threshold)
template <int NW>
__device__ __forceinline__ void hs_load_plane1(float (&acc)[4][8], const float *stage, const HsumParams &p,
                                               int f0, int sgn, int tlo, int t0, int F) {
  const int H = p.half;
  const float *r1 = stage + p.soff[1] + (F - f0);
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const float *rr = r1 + srow(t0 + kk, 4 * NW, sgn) * kHsBins;
    const float4 q0 = *reinterpret_cast<const float4 *>(rr);
    const float4 q1 = *reinterpret_cast<const float4 *>(rr + 128);
    acc[kk][0] = q0.x; acc[kk][1] = q0.y; acc[kk][2] = q0.z; acc[kk][3] = q0.w;
    acc[kk][4] = q1.x; acc[kk][5] = q1.y; acc[kk][6] = q1.z; acc[kk][7] = q1.w;
    if (!((t0 + kk <= H) && (t0 + kk >= tlo))) {
#pragma unroll
      for (int e = 0; e < 8; ++e) acc[kk][e] = -CUDART_INF_F;
    }
  }
  if (f0 + kHsBins > p.n_bins) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
      for (int e = 0; e < 8; ++e)
        if (F + (e & 3) + ((e >> 2) << 7) >= p.n_bins) acc[kk][e] = -CUDART_INF_F;
  }
}

// Plane j >= 2 added for any j given at run time: the same values in the same
// order as the kernel's specialised per-plane code, so the sums are the same
// bit for bit
__device__ __forceinline__ void hs_add_plane_any(float (&acc)[4][8], const float *stage, const HsumParams &p,
                                                 int j, int f0, int sgn, int t0, int F) {
  const int a0 = (f0 / j) & ~3;
  const int bw = p.bw[j];
  const int rb = t0 / j;
  const int kstar = j - (t0 - rb * j);  // first k with trunc((t0+k)/j) = rb + 1
  const float *r0 = stage + p.soff[j] + srow(rb, p.bh[j], sgn) * bw - a0;
  const float *r1 = r0 + sgn * bw;
  // (F + c) / j = qa + [ra + c >= j] + [ra + c >= 2 j] for c < 4 <= 2 j
  const int qa = F / j, ra = F - qa * j;
  const int qb = (F + 128) / j, rg = F + 128 - qb * j;
  float c0[8], c1[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int r = (e < 4 ? ra : rg) + (e & 3);
    const int o = (e < 4 ? qa : qb) + (r >= j ? 1 : 0) + (r >= 2 * j ? 1 : 0);
    c0[e] = r0[o];
    c1[e] = kstar < 4 ? r1[o] : 0.f;
  }
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      const bool second = kk >= kstar;
      add2(acc[kk][e], acc[kk][e + 1], second ? c1[e] : c0[e], second ? c1[e + 1] : c0[e + 1]);
    }
}

// The lanes' cells of `mask` (bit c = cell 8 k + e: template |t| = t0 + k,
// bin F + (e & 3) + 128 (e >> 2)) get consecutive slots from `pos`, cell by
// cell, so every store instruction of the warp writes one contiguous run
template <typename Put>
__device__ __forceinline__ void hs_scatter(const float (&acc)[4][8], unsigned mask, unsigned pos, int row0, int sgn,
                                           int F, Put &&put) {
  const unsigned below = (1u << (threadIdx.x & 31)) - 1u;
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    const unsigned m = __ballot_sync(0xffffffffu, (mask >> c) & 1u);
    if (m) {
      if ((mask >> c) & 1u)
        put(pos + __popc(m & below), acc[c >> 3][c & 7], row0 + sgn * (c >> 3), F + (c & 3) + (((c >> 2) & 1) << 7));
      pos += __popc(m);
    }
  }
}

// Hits of plane `plane` (0-based) to the global list -- one reservation for
// the warp -- and cells within the band to the FP64 recheck list
__device__ __forceinline__ void hs_emit_plane(const float (&acc)[4][8], const HsumParams &p, EmitBuf *eb, int plane,
                                              int row0, int sgn, int F) {
  const int lane = threadIdx.x & 31;
  const float hi = p.hi[plane], lo = p.lo[plane];
  unsigned hmask = 0, nmask = 0;
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    const float a = acc[c >> 3][c & 7];
    if (a > hi) hmask |= 1u << c;
    else if (a >= lo) nmask |= 1u << c;
  }
  const unsigned nall = __reduce_add_sync(0xffffffffu, (unsigned)__popc(nmask));
  if (nall) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(p.rc_count, nall);
    uint4 *list = p.rc_list;
    const unsigned cap = (unsigned)p.rc_cap;
    int *status = p.status;
    hs_scatter(acc, nmask, __shfl_sync(0xffffffffu, base, 0), row0, sgn, F, [&](unsigned g, float, int row, int bin) {
      if (g < cap) list[g] = make_uint4((unsigned)plane, (unsigned)row, (unsigned)bin, 0u);
      else atomicOr(status, kStatusRecheckOverflow);
    });
  }
  const unsigned total = __reduce_add_sync(0xffffffffu, (unsigned)__popc(hmask));
  if (total) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(p.cand_total, total);
    base = __shfl_sync(0xffffffffu, base, 0);
    unsigned long long *keys = p.cand_key;
    float *pwrs = p.cand_pwr;
    const unsigned cap = (unsigned)p.cand_cap;
    hs_scatter(acc, hmask, base, row0, sgn, F, [&](unsigned g, float v, int row, int bin) {
      if (g < cap) {
        keys[g] = cand_key(plane, row, bin);
        pwrs[g] = v;
      }
    });
    if (lane == 0) {
      atomicAdd(&eb->pc[plane], total);
      if (base + total > cap) atomicOr(p.status, kStatusCandidateOverflow);
    }
  }
}

// Emission for one item (rare; the warp calls it together, before it releases
// the stage): the sums are recomputed plane by plane from the staged boxes
// and the planes marked in `need` (bit j - 1) are emitted.
template <int NW>
__device__ __forceinline__ void hs_emit_item_body(const HsumParams &p, const float *stage, EmitBuf *eb, int f0,
                                                  int sgn, int tlo, int t0, unsigned need) {
  const int F = f0 + 4 * (threadIdx.x & 31);
  const int row0 = p.half + sgn * t0;
  float acc[4][8];
  hs_load_plane1<NW>(acc, stage, p, f0, sgn, tlo, t0, F);
#pragma unroll 1
  for (int j = 1; j <= p.n_planes; ++j) {
    if (j > 1) hs_add_plane_any(acc, stage, p, j, f0, sgn, t0, F);
    if ((need >> (j - 1)) & 1u) hs_emit_plane(acc, p, eb, j - 1, row0, sgn, F);
    if (!(need >> j)) break;
  }
}

// The same out of line (the hot loop keeps its code and registers); `pp` is
// the CTA's shared-memory copy of the parameters.  Used where registers are
// plentiful: at the lean variant's 80 registers the call's saves would spill
// in the hot loop, so that variant inlines the body.
template <int NW>
__device__ __noinline__ void hs_emit_item(const HsumParams *pp, const float *stage, EmitBuf *eb, int f0, int sgn,
                                          int tlo, int t0, unsigned need) {
  hs_emit_item_body<NW>(*pp, stage, eb, f0, sgn, tlo, t0, need);
}

template <int MAXP, int NW, int kHsStages, int MINB>
__global__ void __launch_bounds__(32 * (NW + 1), MINB) hsum_kernel(const __grid_constant__ HsumParams p,
                                                                    const __grid_constant__ HsumMaps m) {
  extern __shared__ __align__(1024) float hs_smem[];
  // per stage: `full` completes when the plane-1 box has landed, `full2` when
  // the sub-harmonic boxes have, so the consumers start on plane 1 while the
  // rest of the stage is still arriving
  uint64_t *full = reinterpret_cast<uint64_t *>(hs_smem);  // [kHsStages]
  uint64_t *full2 = full + kHsStages;                        // [kHsStages]
  uint64_t *empty = full2 + kHsStages;                       // [kHsStages]
  int *item_id = reinterpret_cast<int *>(empty + kHsStages); // [kHsStages]
  HsumParams *sp = reinterpret_cast<HsumParams *>(hs_smem + 32);  // copy for the emitter
  float *stages = hs_smem + 256;                             // 1 KB header
  EmitBuf &eb = *reinterpret_cast<EmitBuf *>(stages + kHsStages * p.stage_floats);
  constexpr int kRows1 = 4 * NW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int H = p.half;
  const int P = p.n_planes;
  const int n_items = hs_n_items(p);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kHsStages; ++s) {
      mbar_init(full + s, 1);
      mbar_init(full2 + s, 1);
      mbar_init(empty + s, NW);
    }
    fence_mbar_init();
  }
  if (threadIdx.x < kMaxPlanes) eb.pc[threadIdx.x] = 0;
  static_assert(sizeof(HsumParams) % 4 == 0 && 128 + sizeof(HsumParams) <= 1024, "header holds the parameters");
  static_assert(kHsStages * (3 * 8 + 4) <= 128, "barriers and item ids before the parameter copy");
  for (int i = threadIdx.x; i < (int)(sizeof(HsumParams) / 4); i += blockDim.x)
    reinterpret_cast<int *>(sp)[i] = reinterpret_cast<const int *>(&p)[i];
  __syncthreads();

  if (warp == NW) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      // items are taken from the global counter one at a time, the next one
      // requested an item ahead so the atomic's latency is hidden (few items
      // reserved per CTA keeps the end of the launch even)
      constexpr int kChunk = 1;
      int cur = (int)atomicAdd(p.item_counter, (unsigned)kChunk);
      int nxt = (int)atomicAdd(p.item_counter, (unsigned)kChunk);
      int used = 0;
      // per stage: the use whose copies may still be in flight (-1: none).  A
      // stage's copies have landed once the consumers released it.
      int pending[kHsStages];
#pragma unroll
      for (int q = 0; q < kHsStages; ++q) pending[q] = -1;
      for (int s = 0;; ++s) {
        const int st = s % kHsStages, use = s / kHsStages;
        if (use >= 1 && !mbar_wait_parity(empty + st, (use - 1) & 1, p.timeout_ns)) {
          atomicOr(p.status, kStatusHsumTimeout);
          // let every copy in flight land (bounded), so that the stop mark
          // below arrives on a completed phase and no copy outlives the CTA
          bool drained = true;
#pragma unroll
          for (int q = 0; q < kHsStages; ++q)
            if (pending[q] >= 0) {
              drained &= mbar_wait_parity(full + q, pending[q] & 1, kDrainNs);
              drained &= mbar_wait_parity(full2 + q, pending[q] & 1, kDrainNs);
              pending[q] = -1;
            }
          // (a stage the test hook announced without copies has a phase that
          // never completes: no stop mark on it -- its consumers have left)
          if (drained && !(p.inject_stall && st == 0)) {
            item_id[st] = -1;
            mbar_arrive(full + st);
          }
          break;
        }
#pragma unroll
        for (int q = 0; q < kHsStages; ++q)
          if (q == st) pending[q] = -1;  // released by the consumers: its copies have landed
        if (used == kChunk) {
          cur = nxt;
          used = 0;
          if (cur < n_items) nxt = (int)atomicAdd(p.item_counter, (unsigned)kChunk);
        }
        const int it = cur + used++;
        if (it >= n_items) {
          item_id[st] = -1;
          mbar_arrive(full + st);  // plain arrival: the stage carries the stop mark
          break;
        }
        item_id[st] = it;
        const unsigned bytes1 = (unsigned)(p.bw[1] * p.bh[1]) * 4u;
        if (p.inject_stall && s == 0) {  // test hook: announced, never issued -- nothing in flight
          mbar_arrive_expect_tx(full + st, bytes1);
          mbar_arrive_expect_tx(full2 + st, p.stage_bytes - bytes1 + 16u);
          continue;
        }
#pragma unroll
        for (int q = 0; q < kHsStages; ++q)
          if (q == st) pending[q] = use;
        const HsItem item = hs_item(p, it);
        float *stage = stages + st * p.stage_floats;
        mbar_arrive_expect_tx(full + st, bytes1);
        tma_load_2d(stage + p.soff[1], &m.map[1], item.f0, item.sgn > 0 ? H : H - (kRows1 - 1), full + st);
        mbar_arrive_expect_tx(full2 + st, p.stage_bytes - bytes1);  // 0 bytes with one plane: a plain arrival
        hs_sfor<MAXP - 1>([&](auto JJ) {  // j known at compile time: divisions by constants
          constexpr int j = decltype(JJ)::value + 2;
          if (j <= P) {
            const int a0 = (item.f0 / j) & ~3;
            tma_load_2d(stage + p.soff[j], &m.map[j], a0, item.sgn > 0 ? H : H - (p.bh[j] - 1), full2 + st);
          }
        });
      }
      // consumers that stopped on a timeout leave stages unconsumed: their
      // copies land before the CTA ends (returns at once when they have)
#pragma unroll
      for (int q = 0; q < kHsStages; ++q)
        if (pending[q] >= 0) {
          mbar_wait_parity(full + q, pending[q] & 1, kDrainNs);
          mbar_wait_parity(full2 + q, pending[q] & 1, kDrainNs);
        }
    }
  } else {
    // ------------------------------------------------------------ consumers
    const int t0 = 4 * warp;
    for (int s = 0;; ++s) {
      const int st = s % kHsStages, use = s / kHsStages;
      if (!mbar_wait_parity(full + st, use & 1, p.timeout_ns)) {
        if (lane == 0) atomicOr(p.status, kStatusHsumTimeout);
        break;
      }
      const int it = item_id[st];
      if (it < 0) break;
      const HsItem item = hs_item(p, it);
      const int f0 = item.f0, sgn = item.sgn;
      const float *stage = stages + st * p.stage_floats;
      // lane l holds bins f0 + 4 l + {0..3} and f0 + 128 + 4 l + {0..3}: the
      // lanes of a warp read consecutive 16-byte words (no bank conflicts)
      const int F = f0 + 4 * lane;
      float acc[4][8];
      hs_load_plane1<NW>(acc, stage, p, f0, sgn, item.tlo, t0, F);
      unsigned need = 0;  // planes (bit j - 1) where some lane reached the band; warp-uniform
      // ub: an upper bound of the lane's tile maximum.  Rounded addition is
      // monotone, so ub + (largest value added) bounds every new sum, and the
      // exact maximum (a 3-input max tree) is only needed where the bound reaches
      // a plane's band
      float ub = max32(acc);
      unsigned need_lane = ub >= p.trig[0] ? 1u : 0u;  // this lane's marks; one vote per item
      if (!mbar_wait_parity(full2 + st, use & 1, p.timeout_ns)) {
        if (lane == 0) atomicOr(p.status, kStatusHsumTimeout);
        break;
      }
      hs_sfor<MAXP - 1>([&](auto JJ) {
        constexpr int j = decltype(JJ)::value + 2;
        if (j <= P) {
          const int a0 = (f0 / j) & ~3;
          const int bw = p.bw[j], bh = p.bh[j];
          const float *box = stage + p.soff[j];
          // f0 is a multiple of 256, so for j = 2, 4, 8 the box starts at f0 / j
          float vmax;
          if constexpr (j == 2) {
            const float *r0 = box + srow(t0 / 2, bh, sgn) * bw + 2 * lane;
            const float *r1 = r0 + sgn * bw;
            const float2 a0v = *reinterpret_cast<const float2 *>(r0), b0v = *reinterpret_cast<const float2 *>(r0 + 64);
            const float2 a1v = *reinterpret_cast<const float2 *>(r1), b1v = *reinterpret_cast<const float2 *>(r1 + 64);
            vmax = fmax3(fmax3(a0v.x, a0v.y, b0v.x), fmax3(b0v.y, a1v.x, a1v.y), fmaxf(b1v.x, b1v.y));
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const float2 va = kk < 2 ? a0v : a1v, vb = kk < 2 ? b0v : b1v;
              add2(acc[kk][0], acc[kk][1], va.x, va.x);
              add2(acc[kk][2], acc[kk][3], va.y, va.y);
              add2(acc[kk][4], acc[kk][5], vb.x, vb.x);
              add2(acc[kk][6], acc[kk][7], vb.y, vb.y);
            }
          } else if constexpr (j == 4) {
            const float *r0 = box + srow(t0 / 4, bh, sgn) * bw + lane;
            const float va = r0[0], vb = r0[32];
            vmax = fmaxf(va, vb);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
              for (int e = 0; e < 8; e += 2) add2(acc[kk][e], acc[kk][e + 1], e < 4 ? va : vb, e < 4 ? va : vb);
          } else if constexpr (j == 8) {
            const float *r0 = box + srow(t0 / 8, bh, sgn) * bw + (lane >> 1);
            const float va = r0[0], vb = r0[16];
            vmax = fmaxf(va, vb);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
              for (int e = 0; e < 8; e += 2) add2(acc[kk][e], acc[kk][e + 1], e < 4 ? va : vb, e < 4 ? va : vb);
          } else {
            const int rb = t0 / j;
            const int kstar = j - (t0 - rb * j);  // warp-uniform: first k with trunc((t0+k)/j) = rb + 1
            const float *r0 = box + srow(rb, bh, sgn) * bw - a0;
            const float *r1 = r0 + sgn * bw;
            float c0[8], c1[8];
            // bins F + c and F + 128 + c (c < 4) sit at (F + c) / j = qa + (ra + c >= j)
            // (ra + 3 < 2 j), and likewise for the second group: two divisions per
            // plane, and two staged values per group and row, qa and qa + 1
            // (inside the box: bw >= 255 / j + 6)
            const int qa = F / j, ra = F - qa * j;
            const int qb = (F + 128) / j, rg = F + 128 - qb * j;
            bool hi_a[4], hi_b[4];  // cell c takes the value at q + 1
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              hi_a[c] = ra + c >= j;
              hi_b[c] = rg + c >= j;
            }
            const float2 va = make_float2(r0[qa], r0[qa + 1]), vb = make_float2(r0[qb], r0[qb + 1]);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              c0[c] = hi_a[c] ? va.y : va.x;
              c0[c + 4] = hi_b[c] ? vb.y : vb.x;
            }
            // the bound may include a value no cell takes: still an upper bound
            vmax = fmaxf(fmaxf(va.x, va.y), fmaxf(vb.x, vb.y));
            if (kstar < 4) {  // the second row only where the four rows split
              const float2 wa = make_float2(r1[qa], r1[qa + 1]), wb = make_float2(r1[qb], r1[qb + 1]);
#pragma unroll
              for (int c = 0; c < 4; ++c) {
                c1[c] = hi_a[c] ? wa.y : wa.x;
                c1[c + 4] = hi_b[c] ? wb.y : wb.x;
              }
              vmax = fmax3(vmax, fmaxf(wa.x, wa.y), fmaxf(wb.x, wb.y));
            } else {
#pragma unroll
              for (int e = 0; e < 8; ++e) c1[e] = 0.f;
            }
            switch (kstar < 4 ? kstar : 4) {
              case 1: add_rows<1>(acc, c0, c1); break;
              case 2: add_rows<2>(acc, c0, c1); break;
              case 3: add_rows<3>(acc, c0, c1); break;
              default: add_rows<4>(acc, c0, c1); break;
            }
          }
          ub += vmax;
          if (ub >= p.trig[j - 1]) {  // per lane: no vote, no warp-wide branch in the plane loop
            ub = max32(acc);
            if (ub >= p.trig[j - 1]) need_lane |= 1u << (j - 1);
          }
        }
      });
      need = __reduce_or_sync(0xffffffffu, need_lane);
      if (need) {
        if constexpr (MINB >= 2) hs_emit_item_body<NW>(p, stage, &eb, f0, sgn, item.tlo, t0, need);
        else hs_emit_item<NW>(sp, stage, &eb, f0, sgn, item.tlo, t0, need);
      }

      // release the stage to the producer
      __syncwarp();
      if (lane == 0) mbar_arrive(empty + st);
    }
  }

  // ---- per-plane hit counts of the CTA
  __syncthreads();
  if (threadIdx.x < P && eb.pc[threadIdx.x]) atomicAdd(p.cand_count + threadIdx.x, eb.pc[threadIdx.x]);
}

constexpr int kSelUnroll = 4;  // records per thread in flight in the selection passes
constexpr int kRcUnroll = 8;   // taps per lane in flight in the FP64 recheck

// FP64 taps -> float pairs in place: (re hi, im hi, re lo, im lo) with
// hi = fl32(c), lo = fl32(c - hi), so c = hi + lo to 2^-48 relative.  The
// recheck then forms its products on the FP32 pipe; GB300's FP64 rate is
// about 1/64 of its FP32 rate.
__global__ void split_taps_kernel(double2 *taps, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 c = taps[i];
    const float hr = __double2float_rn(c.x), hm = __double2float_rn(c.y);
    const float lr = __double2float_rn(c.x - (double)hr), lm = __double2float_rn(c.y - (double)hm);
    reinterpret_cast<float4 *>(taps)[i] = make_float4(hr, hm, lr, lm);
  }
}

// (s, t) += a (bh + bl) in double-float arithmetic: a bh = p + pe exactly
// (FMA), s + p = u + e exactly (Knuth's two-sum), the small terms gathered in
// t.  Rounded intrinsics keep the compiler from fusing the error-free steps.
__device__ __forceinline__ void df_add_prod(float &s, float &t, float a, float bh, float bl) {
  const float pr = __fmul_rn(a, bh);
  const float pe = fmaf(a, bh, -pr);
  const float u = __fadd_rn(s, pr);
  const float bb = __fsub_rn(u, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(u, bb)), __fsub_rn(pr, bb));
  t = __fadd_rn(t, __fadd_rn(e, fmaf(a, bl, pe)));
  s = u;
}

// FP64-grade recheck: a CTA per entry (grid-stride), warp j computes the FOP
// cell FOP(trunc(t/(j+1)), bin/(j+1)) = |sum_q X[g - q] h_r[q]|^2
// (ft_conv.py:201-205) with its lanes over the taps -- per lane in
// double-float arithmetic (about 2^-44 relative), then in FP64 across the
// lanes; warp 0 sums the planes in order j = 1..k (hsum.py:95-120) in FP64
// and compares with the threshold.
__global__ void __launch_bounds__(512) recheck_kernel(RecheckParams p) {
  __shared__ double cell[kMaxPlanes];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const unsigned n = min(*p.rc_count, (unsigned)p.rc_cap);
  for (unsigned e = blockIdx.x; e < n; e += gridDim.x) {
    const uint4 ent = p.rc_list[e];
    const int plane = (int)ent.x, row = (int)ent.y, bin = (int)ent.z;
    const int t = row - p.half;
    for (int j = warp + 1; j <= plane + 1; j += nwarps) {
      const int tj = (t >= 0) ? t / j : -((-t) / j);
      const int r = p.half + tj;
      const int g = bin / j;
      const int qn = min(p.tap_len[r], g + 1);
      const float4 *h = p.taps + (long long)r * p.tap_pitch;
      float rs = 0.f, rt = 0.f, is = 0.f, it = 0.f;  // double-float sums of re and im
      // taps q = lane + 32 u in ascending order; the loads of a pass are all
      // issued before the arithmetic, so one memory latency covers 256 taps
      for (int q0 = 0; q0 < qn; q0 += 32 * kRcUnroll) {
        float2 x[kRcUnroll];
        float4 c[kRcUnroll];
#pragma unroll
        for (int u = 0; u < kRcUnroll; ++u) {
          const int q = q0 + lane + 32 * u;
          x[u] = q < qn ? p.input[g - q] : make_float2(0.f, 0.f);
          c[u] = q < qn ? h[q] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kRcUnroll; ++u) {
          if (q0 + lane + 32 * u < qn) {
            // re += x.re c.re - x.im c.im, im += x.re c.im + x.im c.re
            df_add_prod(rs, rt, x[u].x, c[u].x, c[u].z);
            df_add_prod(rs, rt, -x[u].y, c[u].y, c[u].w);
            df_add_prod(is, it, x[u].x, c[u].y, c[u].w);
            df_add_prod(is, it, x[u].y, c[u].x, c[u].z);
          }
        }
      }
      double re = (double)rs + (double)rt, im = (double)is + (double)it;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
      }
      if (lane == 0) cell[j - 1] = re * re + im * im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double hp = 0.0;
      for (int j = 0; j <= plane; ++j) hp += cell[j];
      if (hp > p.thr[plane]) {
        atomicAdd(p.cand_count + plane, 1u);
        global_append(p.cand_key, p.cand_pwr, p.cand_total, p.cand_cap, p.status, cand_key(plane, row, bin),
                      (float)hp);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------- deterministic top-K per plane
// The fixed-size list keeps, per plane, the K strongest hits (power
// descending, location ascending on ties) in location order.  Hits are stored
// unordered by the harmonic-summing kernel.  Selection: a histogram of each
// plane's powers over 2048 buckets (float bits 30..20, powers are >= 0) built
// in shared memory per CTA; the last CTA finds the bucket where the count from
// the top reaches K; the records above it ("sure") and in it ("boundary") are
// gathered; kFinSlices CTAs per plane each rank the boundary records and then
// order their slice of the kept ones by location, both by direct rank
// computation.

__device__ __forceinline__ int pwr_bucket(float pw) { return (int)((__float_as_uint(pw) >> 20) & 0x7ffu); }

__global__ void __launch_bounds__(1024) select_hist_kernel(SelectParams p) {
  extern __shared__ unsigned sh_hist[];  // [n_planes][kSelBuckets]
  __shared__ bool last;
  __shared__ bool over[kMaxPlanes];  // plane has more hits than K
  __shared__ int n_over;
  const int nb = p.n_planes * kSelBuckets;
  if (threadIdx.x == 0) n_over = 0;
  __syncthreads();
  if (threadIdx.x < kMaxPlanes) {
    over[threadIdx.x] = threadIdx.x < p.n_planes && p.cand_count[threadIdx.x] > (unsigned)p.per_plane;
    if (over[threadIdx.x]) atomicAdd(&n_over, 1);
  }
  __syncthreads();
  if (n_over == 0) {
    // every plane keeps all its hits: no histogram, no boundary bucket (the
    // counts are final, so every CTA takes this branch)
    if (blockIdx.x == 0 && threadIdx.x < p.n_planes) p.sel_bucket[threadIdx.x] = -1;
    return;
  }
  for (int i = threadIdx.x; i < nb; i += blockDim.x) sh_hist[i] = 0u;
  __syncthreads();
  const unsigned n = min(*p.cand_total, (unsigned)p.cand_cap);
  // warp-uniform loop, kSelUnroll records per lane in flight; lanes that hit
  // the same (plane, bucket) -- common, since a signal's hits have similar
  // powers -- add once, through their leader
  const unsigned ln = threadIdx.x & 31;
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += kSelUnroll * stride) {
    unsigned long long k[kSelUnroll];
    float w[kSelUnroll];
#pragma unroll
    for (int u = 0; u < kSelUnroll; ++u) {
      const unsigned i = base + u * stride + ln;
      k[u] = i < n ? p.cand_key[i] : ~0ull;
      w[u] = i < n ? p.cand_pwr[i] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kSelUnroll; ++u) {
      const int plane = (int)(k[u] >> 48);
      const unsigned slot = (k[u] != ~0ull && over[plane]) ? (unsigned)(plane * kSelBuckets + pwr_bucket(w[u]))
                                                            : 0xffffffffu;
      const unsigned peers = __match_any_sync(0xffffffffu, slot);
      if (slot != 0xffffffffu && ln == (unsigned)(__ffs(peers) - 1)) atomicAdd(sh_hist + slot, (unsigned)__popc(peers));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    if (sh_hist[i]) atomicAdd(p.hist + i, sh_hist[i]);
  // the last CTA to finish picks the boundary bucket of every plane
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(p.ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the summed histograms into shared memory (one coalesced pass), so the
  // boundary search below is not a chain of dependent global loads
  for (int i = threadIdx.x; i < nb; i += blockDim.x) sh_hist[i] = __ldcg(p.hist + i);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < p.n_planes) {
    const int plane = warp;
    const unsigned K = (unsigned)p.per_plane;
    if (!over[plane]) {
      if (lane == 0) p.sel_bucket[plane] = -1;
    } else {
      const unsigned *h = sh_hist + plane * kSelBuckets;
      // strongest first: chunk c covers buckets [2048 - 32 (c+1), 2048 - 32 c)
      unsigned above = 0;
      int found = -1;
      for (int c = 0; c < kSelBuckets / 32 && found < 0; ++c) {
        const int b = kSelBuckets - 1 - 32 * c - lane;
        unsigned v = h[b];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned u = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) v += u;
        }
        const unsigned hit = __ballot_sync(0xffffffffu, above + v >= K);
        if (hit) found = kSelBuckets - 1 - 32 * c - (__ffs(hit) - 1);
        else above += __shfl_sync(0xffffffffu, v, 31);
      }
      if (lane == 0) p.sel_bucket[plane] = found;  // -1: fewer stored than K (overflow), take all
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) p.hist[i] = 0u;
  if (threadIdx.x == 0) *p.ticket = 0u;
}

__global__ void __launch_bounds__(256) select_gather_kernel(SelectParams p) {
  __shared__ int sb_of[kMaxPlanes];
  if (threadIdx.x < kMaxPlanes) sb_of[threadIdx.x] = threadIdx.x < p.n_planes ? p.sel_bucket[threadIdx.x] : -1;
  __syncthreads();
  const unsigned n = min(*p.cand_total, (unsigned)p.cand_cap);
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned base = blockIdx.x * blockDim.x + threadIdx.x; base < n; base += kSelUnroll * stride) {
    unsigned long long k[kSelUnroll];
    float w[kSelUnroll];
#pragma unroll
    for (int u = 0; u < kSelUnroll; ++u) {
      const unsigned i = base + u * stride;
      k[u] = i < n ? p.cand_key[i] : ~0ull;
      w[u] = i < n ? p.cand_pwr[i] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kSelUnroll; ++u) {
      if (k[u] == ~0ull) continue;
      const unsigned long long key = k[u];
      const int plane = (int)(key >> 48);
      const float pw = w[u];
      const int sb = sb_of[plane];
      const int b = pwr_bucket(pw);
      int list = -1;
      unsigned *cnt = nullptr;
      if (sb < 0 || b > sb) { list = 0; cnt = p.sure_count + plane; }
      else if (b == sb) { list = 1; cnt = p.bound_count + plane; }
      if (list >= 0) {
        const unsigned idx = atomicAdd(cnt, 1u);
        if (idx < (unsigned)kSortCap) {
          const size_t o = ((size_t)plane * 2 + list) * kSortCap + idx;
          p.sel_key[o] = key;
          p.sel_pwr[o] = pw;
        } else {
          atomicOr(p.status, kStatusSelectionOverflow);
        }
      }
    }
  }
}

constexpr int kFinSlices = 8;  // CTAs per plane in the finalize (slices of the K entries)

// "a is stronger than b": power descending, key ascending on ties
__device__ __forceinline__ bool stronger(float pa, unsigned long long ka, float pb, unsigned long long kb) {
  return pa > pb || (pa == pb && ka < kb);
}

__global__ void __launch_bounds__(1024) select_finalize_kernel(SelectParams p) {
  extern __shared__ __align__(16) unsigned char fz_smem[];
  const int plane = blockIdx.x;
  const int K = p.per_plane;
  unsigned long long *bkey = reinterpret_cast<unsigned long long *>(fz_smem);  // [kSortCap] boundary
  float *bpwr = reinterpret_cast<float *>(bkey + kSortCap);
  unsigned long long *fin = reinterpret_cast<unsigned long long *>(bpwr + kSortCap);  // [kMaxCompat] kept
  float *finp = reinterpret_cast<float *>(fin + kMaxCompat);
  const int a = (int)min(p.sure_count[plane], (unsigned)kSortCap);
  const int b = (int)min(p.bound_count[plane], (unsigned)kSortCap);
  const size_t base = (size_t)plane * 2 * kSortCap;
  // the sure records are all kept (fewer than K unless every hit was taken)
  const int keep_a = min(a, K);
  for (int i = threadIdx.x; i < keep_a; i += blockDim.x) {
    fin[i] = p.sel_key[base + i];
    finp[i] = p.sel_pwr[base + i];
  }
  for (int i = threadIdx.x; i < b; i += blockDim.x) {
    bkey[i] = p.sel_key[base + kSortCap + i];
    bpwr[i] = p.sel_pwr[base + kSortCap + i];
  }
  __syncthreads();
  // boundary records: rank among themselves, keep the c strongest
  const int c = max(0, min(K - keep_a, b));
  for (int i = threadIdx.x; i < b; i += blockDim.x) {
    const unsigned long long ki = bkey[i];
    const float pi = bpwr[i];
    int rank = 0;
    for (int j = 0; j < b; ++j) rank += stronger(bpwr[j], bkey[j], pi, ki);
    if (rank < c) {
      fin[keep_a + rank] = ki;
      finp[keep_a + rank] = pi;
    }
  }
  __syncthreads();
  const int kept = keep_a + c;
  uint32_t *cl = p.compat_loc + (size_t)plane * K;
  float *cp = p.compat_pwr + (size_t)plane * K;
  // this CTA's slice [lo, hi) of the K entries: the kept records i in it are
  // placed, the unused positions in it (i >= kept) padded
  const int per = (K + (int)gridDim.y - 1) / (int)gridDim.y;
  const int lo = (int)blockIdx.y * per, hi = min(K, lo + per);
  // order the kept records by location: position = number of smaller keys,
  // counted by a warp per record (lanes over the other records)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int i = lo + warp; i < min(hi, kept); i += nwarps) {
    const unsigned long long ki = fin[i];
    unsigned pos = 0;
    for (int j = lane; j < kept; j += 32) pos += fin[j] < ki ? 1u : 0u;
    pos = __reduce_add_sync(0xffffffffu, pos);
    if (lane == 0) {
      const unsigned row = (unsigned)(ki >> 32) & 0xffffu, bin = (unsigned)(ki & 0xffffffffu);
      // gen_info.h:62-64: ((h-1)&7)<<29 | (row&0x7f)<<22 | (bin&0x3fffff)
      cl[pos] = (((unsigned)plane & 7u) << 29) | ((row & 0x7fu) << 22) | (bin & 0x3fffffu);
      cp[pos] = finp[i];
    }
  }
  for (int i = max(lo, kept) + (int)threadIdx.x; i < hi; i += blockDim.x) {
    cl[i] = p.invalid_location;
    cp[i] = -1.0f;
  }
}

// ----------------------------------------------------------------- launchers
int hsum_warps(int half) { return (half + 1 + 3) / 4 <= 11 ? 11 : 16; }
static int hsum_stages(const HsumParams &p) {
  return (p.lean || p.n_planes > 8 || hsum_warps(p.half) != 11) ? 2 : 3;
}

int hsum_smem_bytes(const HsumParams &p) {
  return 1024 + hsum_stages(p) * p.stage_floats * 4 + (int)sizeof(EmitBuf);
}

template <int MAXP, int NW, int STAGES, int MINB>
static cudaError_t launch_hsum_t(const HsumParams &p, const HsumMaps &m, cudaStream_t s) {
  const int smem = hsum_smem_bytes(p);
  cudaError_t e =
      cudaFuncSetAttribute(hsum_kernel<MAXP, NW, STAGES, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int n_sm = current_sm_count();
  const int items = (p.n_bins + kHsBins - 1) / kHsBins * 2;
  hsum_kernel<MAXP, NW, STAGES, MINB><<<items < n_sm ? items : n_sm, 32 * (NW + 1), smem, s>>>(p, m);
  return cudaGetLastError();
}

cudaError_t launch_hsum(const HsumParams &p, const HsumMaps &m, cudaStream_t s) {
  if (hsum_warps(p.half) == 11) {
    if (p.n_planes <= 8) {
      // lean: 2 stages and a register budget that fits next to one FT-convolution CTA
      if (p.lean) return launch_hsum_t<8, 11, 2, 2>(p, m, s);
      return launch_hsum_t<8, 11, 3, 1>(p, m, s);
    }
    return launch_hsum_t<16, 11, 2, 1>(p, m, s);
  }
  return launch_hsum_t<16, 16, 2, 1>(p, m, s);
}

cudaError_t launch_split_taps(double2 *taps, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = (n + 255) / 256;
  split_taps_kernel<<<(int)(blocks < 1024 ? blocks : 1024), 256, 0, s>>>(taps, n);
  return cudaGetLastError();
}

cudaError_t launch_recheck(const RecheckParams &p, cudaStream_t s) {
  recheck_kernel<<<4 * current_sm_count(), 32 * 8, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_select(const SelectParams &p, cudaStream_t s) {
  const int n_sm = current_sm_count();
  const int hsmem = p.n_planes * kSelBuckets * 4;
  cudaError_t e = cudaFuncSetAttribute(select_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, hsmem);
  if (e != cudaSuccess) return e;
  select_hist_kernel<<<n_sm, 1024, hsmem, s>>>(p);
  select_gather_kernel<<<4 * n_sm, 256, 0, s>>>(p);
  const int fsmem = (kSortCap + kMaxCompat) * (8 + 4);
  e = cudaFuncSetAttribute(select_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, fsmem);
  if (e != cudaSuccess) return e;
  select_finalize_kernel<<<dim3(p.n_planes, kFinSlices), 1024, fsmem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace fdas
