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
// TMA bulk copy global -> shared, completion signalled on the mbarrier
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait on phase 0 of the barrier; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, long long timeout_ns) {
  if (mbar_try_wait(bar, 0)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait(bar, 0)) return true;
    if ((long long)(globaltimer_ns() - t0) > timeout_ns) return false;
  }
}

// Candidate staging: each warp collects its records in a shared-memory
// buffer (warp ballot -> one slot range per batch) and moves a full buffer to
// the global list with a single atomic reservation.
constexpr int kWarpBuf = 64;
constexpr int kHsMaxWarps = 16;  // templates per half <= 64

struct EmitBuf {
  unsigned pc[kMaxPlanes];                 // hits per plane of this CTA
  unsigned long long key[kHsMaxWarps][kWarpBuf];
  float pwr[kHsMaxWarps][kWarpBuf];
};

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

// warp-synchronous: move this warp's staged records to the global list
__device__ __forceinline__ void warp_flush(EmitBuf &eb, int warp, unsigned &wcount, const HsumParams &p) {
  __syncwarp();
  const int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (lane == 0 && wcount) base = atomicAdd(p.cand_total, wcount);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (unsigned i = lane; i < wcount; i += 32) {
    const unsigned g = base + i;
    if (g < (unsigned)p.cand_cap) {
      p.cand_key[g] = eb.key[warp][i];
      p.cand_pwr[g] = eb.pwr[warp][i];
    }
  }
  if (lane == 0 && wcount && base + wcount > (unsigned)p.cand_cap) atomicOr(p.status, kStatusCandidateOverflow);
  __syncwarp();
  wcount = 0;
}

// warp-synchronous emission of the lanes in `hm` (all lanes call this)
__device__ __forceinline__ void warp_emit(EmitBuf &eb, int warp, unsigned &wcount, const HsumParams &p,
                                          unsigned hm, int plane, int row, int bin, float pwr) {
  const int lane = threadIdx.x & 31;
  const unsigned n = __popc(hm);
  if (wcount + n > (unsigned)kWarpBuf) warp_flush(eb, warp, wcount, p);
  if ((hm >> lane) & 1u) {
    const unsigned slot = wcount + __popc(hm & ((1u << lane) - 1u));
    eb.key[warp][slot] = cand_key(plane, row, bin);
    eb.pwr[warp][slot] = pwr;
  }
  if (lane == 0) atomicAdd(&eb.pc[plane], n);
  wcount += n;
}

__device__ __forceinline__ void warp_recheck(const HsumParams &p, unsigned nm, int plane, int row, int bin) {
  const int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (lane == 0) base = atomicAdd(p.rc_count, (unsigned)__popc(nm));
  base = __shfl_sync(0xffffffffu, base, 0);
  if ((nm >> lane) & 1u) {
    const unsigned idx = base + __popc(nm & ((1u << lane) - 1u));
    if (idx < (unsigned)p.rc_cap) p.rc_list[idx] = make_uint4((unsigned)plane, (unsigned)row, (unsigned)bin, 0u);
    else atomicOr(p.status, kStatusRecheckOverflow);
  }
}

// One CTA per (256-bin block, sign half), one warp per group of 4 templates:
// warp w owns |t| = 4w + k (k < 4), lane l the bins f0 + 128 i + 4 l + e
// (i < 2, e < 4), so every thread holds a 4 x 4 tile of cells aligned to 4 in
// both directions.  For planes j >= 2 the rows trunc(t/j) and bins
// [f0/j, (f0+255)/j] of the half are staged in shared memory by TMA bulk
// copies (one per plane and row, 16-byte aligned); plane 1 is read from global
// memory with 128-bit loads.  With the tile aligned to 4, planes 2, 4 and 8
// map the 4 x 4 tile onto 2 x 2, 1 x 1 and 1 x 1 staged values at
// compile-time offsets; planes 3, 5, 6, 7 onto a 2 x 2 window whose split
// points are computed once per thread.
//
// HP_1 = FOP[t][f], HP_j = HP_{j-1} + FOP[trunc(t/j)][f/j] accumulated in FP32
// in this order -- hsum.py:95-120 / hms_baseline.cl.mako:55-84 -- so the
// values match hsum.py bit for bit for the same FOP.  A cell is a candidate of
// plane j if HP_j > thr_j (strict, hsum.py:134 / detect.cl.mako:185).  The fast
// path only records, per thread, whether any cell reached the lower edge of a
// threshold band; such warps re-walk their cells warp-synchronously and emit
// through ballots.
struct HsGeom {
  const float *stage;
  int f0, w, lane;
};

// value of plane j (>= 2) for cell (k, e) of this thread's tile, from the staged rows
template <int J>
struct PlaneWindow {
  float v00, v01, v10, v11;
  int kstar, estar;
  __device__ __forceinline__ void load(const HsumParams &p, const HsGeom &g, int F) {
    const int a0 = (g.f0 / J) & ~3;
    const float *blk = g.stage + p.soff[J];
    const int sw = p.sw[J];
    const int t0 = 4 * g.w;
    const int rb = t0 / J;
    kstar = J - (t0 - rb * J);     // first k with trunc((t0+k)/J) = rb + 1
    const int bb = F / J;
    estar = J - (F - bb * J);      // first e with (F+e)/J = bb + 1
    const float *r0 = blk + rb * sw + (bb - a0);
    v00 = r0[0];
    v01 = r0[1];
    v10 = r0[sw];
    v11 = r0[sw + 1];
  }
  __device__ __forceinline__ float at(int k, int e) const {
    const float c0 = e < estar ? v00 : v01;
    const float c1 = e < estar ? v10 : v11;
    return k < kstar ? c0 : c1;
  }
};

template <int MAXP>
__global__ void __launch_bounds__(512) hsum_kernel(HsumParams p) {
  extern __shared__ __align__(128) float hs_smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(hs_smem);
  float *stage = hs_smem + 4;
  EmitBuf &eb = *reinterpret_cast<EmitBuf *>(hs_smem + 4 + ((p.smem_floats + 3) & ~3));
  const int halfsel = blockIdx.y;
  const int sgn = halfsel ? 1 : -1;
  const int tlo = p.tlo[halfsel];
  const int H = p.half;
  if (tlo > H) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int f0 = blockIdx.x * kHsBins;
  const int P = p.n_planes;
  const bool staged = p.stage_bytes > 0;

  if (threadIdx.x == 0 && staged) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (threadIdx.x < kMaxPlanes) eb.pc[threadIdx.x] = 0;
  __syncthreads();
  if (staged && warp == 0) {
    if (lane == 0) mbar_arrive_expect_tx(bar, p.stage_bytes);
    __syncwarp();
    for (int j = 2; j <= P; ++j) {
      const int a0 = (f0 / j) & ~3;
      const int w = p.sw[j];
      for (int r = lane; r < p.srows[j]; r += 32) {
        // rows past |t| = H only feed cells that are masked out; copy row H instead
        const float *src = p.fop + (long long)(H + sgn * min(r, H)) * p.stride + a0;
        bulk_g2s(stage + p.soff[j] + r * w, src, (uint32_t)w * 4u, bar);
      }
    }
  }

  // rows of this warp: |t| = 4 warp + k; invalid ones (|t| > H or < tlo) get -inf
  const int t0 = 4 * warp;
  bool rowok[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) rowok[k] = (t0 + k <= H) && (t0 + k >= tlo);

  // plane 1 for both bin sub-blocks (loads in flight while the staging lands)
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int F = f0 + 128 * i + 4 * lane;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float4 q = make_float4(-CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F);
      if (rowok[k]) q = __ldg(reinterpret_cast<const float4 *>(p.fop + (long long)(H + sgn * (t0 + k)) * p.stride + F));
      acc[i][k][0] = (F + 0 < p.n_bins) ? q.x : -CUDART_INF_F;
      acc[i][k][1] = (F + 1 < p.n_bins) ? q.y : -CUDART_INF_F;
      acc[i][k][2] = (F + 2 < p.n_bins) ? q.z : -CUDART_INF_F;
      acc[i][k][3] = (F + 3 < p.n_bins) ? q.w : -CUDART_INF_F;
    }
  }
  bool flag[2] = {false, false};
  {
    const float tr = p.trig[0];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int e = 0; e < 4; ++e) flag[i] |= acc[i][k][e] >= tr;
  }

  // the timeout decision is made uniform over the CTA before any warp vote
  bool ok = true;
  if (staged) ok = __syncthreads_and(mbar_wait_bounded(bar, p.timeout_ns)) != 0;
  if (!ok) {
    if (threadIdx.x == 0) atomicOr(p.status, kStatusHsumTimeout);
    mbar_wait_bounded(bar, p.timeout_ns);  // let copies in flight land (bounded)
    return;
  }
  const HsGeom g{stage, f0, warp, lane};

  // ---- fast path: planes 2..P, compile-time plane index
  hs_sfor<MAXP - 1>([&](auto JJ) {
    constexpr int j = decltype(JJ)::value + 2;
    if (j <= P) {
      const float tr = p.trig[j - 1];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int F = f0 + 128 * i + 4 * lane;
        if constexpr (j == 2 || j == 4 || j == 8) {
          const int a0 = (f0 / j) & ~3;
          const float *blk = stage + p.soff[j] + (F / j - a0);
          const int sw = p.sw[j];
          if constexpr (j == 2) {
            const float2 r0 = *reinterpret_cast<const float2 *>(blk + (t0 / 2) * sw);
            const float2 r1 = *reinterpret_cast<const float2 *>(blk + (t0 / 2 + 1) * sw);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const float2 r = k < 2 ? r0 : r1;
              acc[i][k][0] += r.x; acc[i][k][1] += r.x; acc[i][k][2] += r.y; acc[i][k][3] += r.y;
            }
          } else {
            const float v = blk[(t0 / j) * sw];
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
              for (int e = 0; e < 4; ++e) acc[i][k][e] += v;
          }
        } else {
          PlaneWindow<j> win;
          win.load(p, g, F);
#pragma unroll
          for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][k][e] += win.at(k, e);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
          for (int e = 0; e < 4; ++e) flag[i] |= acc[i][k][e] >= tr;
      }
    }
  });

  // ---- slow path (rare): warps with a flagged lane re-walk their cells in the
  // same order; every lane recomputes its own cell and emission goes through
  // warp ballots into the warp's record buffer
  unsigned wcount = 0;
  const unsigned flags = (flag[0] ? 1u : 0u) | (flag[1] ? 2u : 0u);
#pragma unroll 1
  for (int i = 0; i < 2; ++i) {
    const bool fl = (flags >> i) & 1u;
    if (!__any_sync(0xffffffffu, fl)) continue;
    const int F = f0 + 128 * i + 4 * lane;
#pragma unroll 1
    for (int c = 0; c < 16; ++c) {
      const int k = c >> 2, e = c & 3;
      const int t = t0 + k;
      const int f = F + e;
      const bool active = fl && t <= H && t >= tlo && f < p.n_bins;
      const int row = H + sgn * t;
      float a = active ? p.fop[(long long)row * p.stride + f] : 0.f;
      hs_sfor<MAXP>([&](auto JJ) {
        constexpr int j = decltype(JJ)::value + 1;
        if (j <= P) {
          if constexpr (j > 1) {
            const int a0 = (f0 / j) & ~3;
            if (active) a += stage[p.soff[j] + (t / j) * p.sw[j] + f / j - a0];
          }
          const bool hit = active && a > p.hi[j - 1];
          const bool near = active && !hit && a >= p.lo[j - 1];
          const unsigned hm = __ballot_sync(0xffffffffu, hit);
          if (hm) warp_emit(eb, warp, wcount, p, hm, j - 1, row, f, a);
          const unsigned nm = __ballot_sync(0xffffffffu, near);
          if (nm) warp_recheck(p, nm, j - 1, row, f);
        }
      });
    }
  }
  warp_flush(eb, warp, wcount, p);

  // ---- per-plane hit counts of the CTA
  __syncthreads();
  if (threadIdx.x < P && eb.pc[threadIdx.x]) atomicAdd(p.cand_count + threadIdx.x, eb.pc[threadIdx.x]);
  (void)nwarps;
}

// One warp per recheck entry: HP_j of the cell in FP64 from the spectrum and
// the FP64 taps, FOP(r, g) = |sum_q X[g - q] h_r[q]|^2 (ft_conv.py:201-205).
__global__ void __launch_bounds__(256) recheck_kernel(RecheckParams p) {
  const int lane = threadIdx.x & 31;
  const unsigned n = min(*p.rc_count, (unsigned)p.rc_cap);
  const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
  for (unsigned e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += nwarps) {
    const uint4 ent = p.rc_list[e];
    const int plane = (int)ent.x, row = (int)ent.y, bin = (int)ent.z;
    const int t = row - p.half;
    double hp = 0.0;
    for (int j = 1; j <= plane + 1; ++j) {
      const int tj = (t >= 0) ? t / j : -((-t) / j);
      const int r = p.half + tj;
      const int g = bin / j;
      const int len = p.tap_len[r];
      const double2 *h = p.taps + (long long)r * p.tap_pitch;
      double re = 0.0, im = 0.0;
      for (int q = lane; q < len && q <= g; q += 32) {
        const float2 x = p.input[g - q];
        const double2 c = h[q];
        re += (double)x.x * c.x - (double)x.y * c.y;
        im += (double)x.x * c.y + (double)x.y * c.x;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
      }
      hp += re * re + im * im;
    }
    if (lane == 0 && hp > p.thr[plane]) {
      atomicAdd(p.cand_count + plane, 1u);
      global_append(p.cand_key, p.cand_pwr, p.cand_total, p.cand_cap, p.status, cand_key(plane, row, bin),
                    (float)hp);
    }
  }
}

// ------------------------------------------- deterministic top-K per plane
// The fixed-size list keeps, per plane, the K strongest hits (power
// descending, location ascending on ties) in location order.  Hits are stored
// unordered by the harmonic-summing CTAs; the selection is a radix select on
// the power: a histogram of the top 16 bits of each plane's power keys, the
// bucket where the count from the top reaches K, a gather of the records at or
// above that bucket, and a one-CTA sort of the gathered records.

// order-preserving map of a float to an unsigned key
__device__ __forceinline__ unsigned float_key(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ unsigned stored_records(const SelectParams &p) {
  return min(*p.cand_total, (unsigned)p.cand_cap);
}

__global__ void __launch_bounds__(256) select_hist_kernel(SelectParams p) {
  const unsigned n = stored_records(p);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int plane = (int)(p.cand_key[i] >> 48);
    if (p.cand_count[plane] > (unsigned)p.per_plane)
      atomicAdd(p.hist + (size_t)plane * kSelBuckets + (float_key(p.cand_pwr[i]) >> 16), 1u);
  }
}

// One CTA (1024 threads) per plane: thread t owns buckets
// [kSelBuckets - 64 (t+1), kSelBuckets - 64 t), i.e. thread 0 the strongest.
__global__ void __launch_bounds__(1024) select_threshold_kernel(SelectParams p) {
  __shared__ unsigned part[1024];
  __shared__ unsigned found;
  const int plane = blockIdx.x;
  unsigned *h = p.hist + (size_t)plane * kSelBuckets;
  const unsigned K = (unsigned)p.per_plane;
  if (p.cand_count[plane] <= K) {
    if (threadIdx.x == 0) p.sel_lo[plane] = 0u;
    return;
  }
  const int t = threadIdx.x;
  const int hi_b = kSelBuckets - 64 * t;  // exclusive
  unsigned local = 0;
  for (int b = hi_b - 64; b < hi_b; ++b) local += h[b];
  part[t] = local;
  if (t == 0) found = 0u;
  __syncthreads();
  // inclusive scan over threads (strongest first)
  for (int o = 1; o < 1024; o <<= 1) {
    const unsigned v = t >= o ? part[t - o] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  const unsigned before = t ? part[t - 1] : 0u;
  if (before < K && part[t] >= K) {
    unsigned c = before;
    int b = hi_b - 1;
    for (; b >= hi_b - 64; --b) {
      c += h[b];
      if (c >= K) break;
    }
    p.sel_lo[plane] = (unsigned)b << 16;
    found = 1u;
  }
  __syncthreads();
  if (t == 0 && !found) p.sel_lo[plane] = 0u;  // fewer stored than K (overflow): take all
  // leave the histogram zeroed for the next search
  for (int b = hi_b - 64; b < hi_b; ++b)
    if (h[b]) h[b] = 0u;
}

__global__ void __launch_bounds__(256) select_gather_kernel(SelectParams p) {
  const unsigned n = stored_records(p);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long key = p.cand_key[i];
    const int plane = (int)(key >> 48);
    const float pw = p.cand_pwr[i];
    if (float_key(pw) >= p.sel_lo[plane]) {
      const unsigned idx = atomicAdd(p.sel_count + plane, 1u);
      if (idx < (unsigned)kSortCap) {
        p.sel_key[(size_t)plane * kSortCap + idx] = key;
        p.sel_pwr[(size_t)plane * kSortCap + idx] = pw;
      } else {
        atomicOr(p.status, kStatusSelectionOverflow);
      }
    }
  }
}

struct Rec {
  unsigned long long key;
  float pwr;
};

__device__ __forceinline__ bool less_key(const Rec &a, const Rec &b) { return a.key < b.key; }
// "stronger first": power descending, key ascending on ties
__device__ __forceinline__ bool less_pwr(const Rec &a, const Rec &b) {
  return (a.pwr > b.pwr) || (a.pwr == b.pwr && a.key < b.key);
}

template <bool BY_PWR>
__device__ void bitonic_sort(unsigned long long *keys, float *pwrs, int m) {
  for (int k = 2; k <= m; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          Rec a{keys[i], pwrs[i]}, b{keys[ixj], pwrs[ixj]};
          const bool up = (i & k) == 0;
          const bool swap = up ? (BY_PWR ? less_pwr(b, a) : less_key(b, a))
                               : (BY_PWR ? less_pwr(a, b) : less_key(a, b));
          if (swap) {
            keys[i] = b.key; pwrs[i] = b.pwr;
            keys[ixj] = a.key; pwrs[ixj] = a.pwr;
          }
        }
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(1024) select_finalize_kernel(SelectParams p) {
  extern __shared__ __align__(16) unsigned char fz_smem[];
  const int plane = blockIdx.x;
  const int n = (int)min(p.sel_count[plane], (unsigned)kSortCap);
  int m = 1;
  while (m < n) m <<= 1;
  unsigned long long *keys = reinterpret_cast<unsigned long long *>(fz_smem);
  float *pwrs = reinterpret_cast<float *>(keys + kSortCap);
  const unsigned long long *gk = p.sel_key + (size_t)plane * kSortCap;
  const float *gp = p.sel_pwr + (size_t)plane * kSortCap;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    keys[i] = i < n ? gk[i] : ~0ull;
    pwrs[i] = i < n ? gp[i] : -CUDART_INF_F;
  }
  __syncthreads();
  int kept = n;
  if (n > p.per_plane) {
    bitonic_sort<true>(keys, pwrs, m);
    kept = p.per_plane;
    for (int i = threadIdx.x; i < m; i += blockDim.x)
      if (i >= kept) { keys[i] = ~0ull; pwrs[i] = -CUDART_INF_F; }
    __syncthreads();
  }
  if (kept > 1) bitonic_sort<false>(keys, pwrs, m);
  uint32_t *cl = p.compat_loc + (size_t)plane * p.per_plane;
  float *cp = p.compat_pwr + (size_t)plane * p.per_plane;
  for (int i = threadIdx.x; i < p.per_plane; i += blockDim.x) {
    if (i < kept) {
      const unsigned row = (unsigned)(keys[i] >> 32) & 0xffffu, bin = (unsigned)(keys[i] & 0xffffffffu);
      // gen_info.h:62-64: ((h-1)&7)<<29 | (row&0x7f)<<22 | (bin&0x3fffff)
      cl[i] = (((unsigned)plane & 7u) << 29) | ((row & 0x7fu) << 22) | (bin & 0x3fffffu);
      cp[i] = pwrs[i];
    } else {
      cl[i] = p.invalid_location;
      cp[i] = -1.0f;
    }
  }
}

// ----------------------------------------------------------------- launchers
int hsum_smem_bytes(const HsumParams &p) {
  return 16 + ((p.smem_floats + 3) & ~3) * 4 + (int)sizeof(EmitBuf);
}

template <int MAXP>
static cudaError_t launch_hsum_t(const HsumParams &p, cudaStream_t s) {
  const int smem = hsum_smem_bytes(p);
  cudaError_t e = cudaFuncSetAttribute(hsum_kernel<MAXP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int groups = (p.half + 1 + 3) / 4;  // warps: 4 templates each
  dim3 grid((p.n_bins + kHsBins - 1) / kHsBins, 2);
  hsum_kernel<MAXP><<<grid, 32 * groups, smem, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_hsum(const HsumParams &p, cudaStream_t s) {
  if (p.n_planes <= 4) return launch_hsum_t<4>(p, s);
  if (p.n_planes <= 8) return launch_hsum_t<8>(p, s);
  return launch_hsum_t<16>(p, s);
}

cudaError_t launch_recheck(const RecheckParams &p, cudaStream_t s) {
  recheck_kernel<<<2 * 152, 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_select(const SelectParams &p, cudaStream_t s) {
  select_hist_kernel<<<4 * 152, 256, 0, s>>>(p);
  select_threshold_kernel<<<p.n_planes, 1024, 0, s>>>(p);
  select_gather_kernel<<<4 * 152, 256, 0, s>>>(p);
  const int smem = kSortCap * (8 + 4);
  cudaError_t e = cudaFuncSetAttribute(select_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  select_finalize_kernel<<<p.n_planes, 1024, smem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace fdas
