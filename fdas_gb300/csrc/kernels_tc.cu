// Precision form: the 2048-point DFTs of the search as two DFT-factor matrix
// products on the 5th-generation tensor cores (tcgen05.mma, accumulators in
// tensor memory), with split (hi + lo) BF16 or FP16 operands and FP32
// accumulation -- the inverse DFT of every (tile, template) item of the FT
// convolution, and (FWD) the forward DFT of every tile.
//
// With k = 32 k1 + k2 and n = n1 + 64 n2 (k1, n1 < 64; k2, n2 < 32):
//   y[n1 + 64 n2] = sum_k2 W32^(n2 k2) w^(n1 k2) sum_k1 W64^(n1 k1) Y[32 k1 + k2]
// (w = e^(+2 pi i / 2048)).  Stage A is a real GEMM with M = 128 (rows
// 2 n1 + re/im), K = 128 (re/im x k1) and N = 32 columns (k2) per item, four
// items per group; the twiddle w^(n1 k2) is applied on the CUDA cores while
// the stage-A result is read back from tensor memory; stage B is a real GEMM
// with M = 128 (two items x n1), K = 64 (re/im x k2), N = 64 (re/im x n2).
// Each product is hi*hi + hi*lo + lo*hi of the split operands (the lo*lo term,
// 2^-16 of the product for BF16, is dropped).  The operands are scaled by a
// power of two per group (FP16 range) and the power |y|^2 is scaled back
// exactly.  The forward transform (FWD) is the same with the conjugate
// factors (w = e^(-2 pi i / 2048)): Y is the tile's input (spectrum bins
// [i P - O, i P + P), zero outside [0, N)), y its spectrum, stored complex.
//
// Operands live in shared memory in the tensor core's canonical K-major layout
// without swizzle: 8 x 16-byte core matrices, K-adjacent ones 128 bytes apart,
// 8-row groups (K / 8) x 128 bytes apart.  One CTA of 8 warps per SM, one
// thread issues the MMAs; every mbarrier wait is bounded by %globaltimer.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace fdas {

namespace {

constexpr int kTcItems = 4;  // (tile, template) items per group
constexpr int kTcThreads = 256;
// shared-memory regions (bytes); stage B's A operands (4 x 16 KB) reuse the
// stage-A B operands once the stage-A products are done
constexpr int kAAh = 0, kAAl = 32768, kBAh = 65536, kBAl = 98304, kBBh = 131072, kBBl = 139264;
// + the inter-stage twiddles w^(n1 k2) at [k2][n1] (16 KB)
constexpr int kTW = 147456;
constexpr int kTcSmem = 163840;
// tensor memory: stage A hi*hi at columns 0..127, its correction terms (hi*lo + lo*hi)
// at 128..255; stage B hi*hi at 256 + 64 p, corrections at 384 + 64 p.  The small
// corrections get their own FP32 accumulators and are added on the CUDA cores.
constexpr int kTcTmemCols = 512;

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t tc_timer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// byte offset of element (row, k) of a K-major operand with K columns
__device__ __forceinline__ int kmaj(int row, int k, int K) {
  return (row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start >> 4, leading (K) byte offset 128,
// stride (8-row) byte offset, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, int K) {
  uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(((K * 16) >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: FP32 accumulator, A and B of one type
// (FP16 or BF16), both K-major, M x N
template <bool F16>
__device__ __forceinline__ uint32_t tc_idesc(int M, int N) {
  const uint32_t t = F16 ? 0u : 1u;
  return (1u << 4) | (t << 7) | (t << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// 32 consecutive tensor-memory columns of this thread's lane, one round trip
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// hi / lo split of two values at once (paired conversions), stored as two
// 32-bit words: element pair (x0, x1) of the hi and of the lo operand
template <bool F16>
__device__ __forceinline__ void store_pair(uint8_t *hi_base, uint8_t *lo_base, int off, float x0, float x1) {
  if constexpr (F16) {
    const __half2 h = __floats2half2_rn(x0, x1);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
    *reinterpret_cast<__half2 *>(hi_base + off) = h;
    *reinterpret_cast<__half2 *>(lo_base + off) = l;
  } else {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    *reinterpret_cast<__nv_bfloat162 *>(hi_base + off) = h;
    *reinterpret_cast<__nv_bfloat162 *>(lo_base + off) = l;
  }
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }  // -126 <= e <= 127

// bounded wait on the mbarrier phase; false on timeout
__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity, long long timeout_ns) {
  const uint64_t t0 = tc_timer();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(tc_smem(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if ((long long)(tc_timer() - t0) > timeout_ns) return false;
  }
}

template <bool F16, bool FWD>
__global__ void __launch_bounds__(kTcThreads, 1) ftc_tc_kernel(FtcParams p) {
  extern __shared__ __align__(1024) uint8_t tsm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ float red[kTcThreads / 32];
  __shared__ int stop;
  uint8_t *AAh = tsm + kAAh, *AAl = tsm + kAAl, *BAh = tsm + kBAh, *BAl = tsm + kBAl, *BBh = tsm + kBBh,
          *BBl = tsm + kBBl;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // ---- constant operands: the real forms of DFT-64 (stage A) and DFT-32 (stage B)
  for (int i = tid; i < 128 * 64; i += kTcThreads) {
    const int m = i >> 6, kp = (i & 63) * 2;  // element pair (kp, kp + 1) of row m
    const int n1 = m >> 1, part = m & 1;
    float v[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int kk = kp + u, pin = kk >> 6, k1 = kk & 63;
      float2 w = __ldg(p.twiddle + ((32 * n1 * k1) & 2047));
      if (FWD) w.y = -w.y;
      v[u] = part == 0 ? (pin == 0 ? w.x : -w.y) : (pin == 0 ? w.y : w.x);
    }
    store_pair<F16>(AAh, AAl, kmaj(m, kp, 128), v[0], v[1]);
  }
  for (int i = tid; i < 64 * 32; i += kTcThreads) {
    const int r = i >> 5, kp = (i & 31) * 2;
    const int pout = r >> 5, n2 = r & 31;
    float v[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int kk = kp + u, pin = kk >> 5, k2 = kk & 31;
      float2 w = __ldg(p.twiddle + ((64 * n2 * k2) & 2047));
      if (FWD) w.y = -w.y;
      v[u] = pout == 0 ? (pin == 0 ? w.x : -w.y) : (pin == 0 ? w.y : w.x);
    }
    store_pair<F16>(BBh, BBl, kmaj(r, kp, 64), v[0], v[1]);
  }
  float2 *TW = reinterpret_cast<float2 *>(tsm + kTW);
  for (int i = tid; i < 64 * 32; i += kTcThreads) {
    float2 w = __ldg(p.twiddle + (i & 63) * (i >> 6));
    if (FWD) w.y = -w.y;
    TW[i] = w;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    stop = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_slot)),
                 "r"(kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const int q = warp & 3, h = warp >> 2;  // TMEM lane quadrant, column half
  const uint32_t lane_addr = (uint32_t)(32 * q) << 16;
  const int n_items = FWD ? p.n_tiles : p.n_tiles * p.n_rows;
  const int n_groups = (n_items + kTcItems - 1) / kTcItems;
  uint32_t phase = 0;

  for (int g = blockIdx.x; g < n_groups; g += gridDim.x) {
    // ---- stage-A B operand: Y = tile spectrum x template spectrum, 4 items.
    // A warp fills whole 8 x 8 core matrices per store (no bank conflicts):
    // task t = (item, row group rg, K group kc); lane l: k2 = 8 rg + l / 4,
    // k1 = 8 kc + 2 (l % 4) and k1 + 1
    float4 y[16];
    float mx = 0.f;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int t = warp + 8 * j, item = t >> 5, rg = (t >> 3) & 3, kc = t & 7;
      const int k2 = 8 * rg + (lane >> 2), k1 = 8 * kc + 2 * (lane & 3);
      // loads are unconditional (a missing item reads item 0 and is zeroed), so
      // all 64 of a thread's loads are in flight together
      const int it = g * kTcItems + item, itc = it < n_items ? it : 0;
      const int k = 32 * k1 + k2;
      float4 v;
      if constexpr (FWD) {  // the tile's input bins (tile_input.cl.mako:42-94 / ft_conv.py:165-180)
        const long long b = (long long)itc * p.payload - p.overlap + k;
        const float2 zero = make_float2(0.f, 0.f);
        const float2 x0 = (b >= 0 && b < p.n_bins) ? __ldg(p.input + b) : zero;
        const float2 x1 = (b + 32 >= 0 && b + 32 < p.n_bins) ? __ldg(p.input + b + 32) : zero;
        v = make_float4(x0.x, x0.y, x1.x, x1.y);
      } else {
        const int tile = itc / p.n_rows, row = p.row_begin + (itc - tile * p.n_rows);
        const float2 *S = p.tiles + (long long)tile * kTile, *T = p.tmpl + (long long)row * kTile;
        const float2 s0 = __ldg(S + k), t0 = __ldg(T + k), s1 = __ldg(S + k + 32), t1 = __ldg(T + k + 32);
        v = make_float4(s0.x * t0.x - s0.y * t0.y, s0.x * t0.y + s0.y * t0.x, s1.x * t1.x - s1.y * t1.y,
                        s1.x * t1.y + s1.y * t1.x);
      }
      if (it >= n_items) v = make_float4(0.f, 0.f, 0.f, 0.f);
      y[j] = v;
      mx = fmaxf(mx, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) red[warp] = mx;
    __syncthreads();
    mx = red[0];
#pragma unroll
    for (int w = 1; w < kTcThreads / 32; ++w) mx = fmaxf(mx, red[w]);
    // scale so the largest component lies in [2^14, 2^15)
    // (sigma kept within +-56 so that 2^sigma and 2^(12 - 2 sigma) are normal floats)
    const int sigma = mx > 0.f ? max(-56, min(56, 14 - ilogbf(mx))) : 0;
    const float sa = pow2f(sigma);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int t = warp + 8 * j, item = t >> 5, rg = (t >> 3) & 3, kc = t & 7;
      const int k1 = 8 * kc + 2 * (lane & 3);
      const int r = item * 32 + 8 * rg + (lane >> 2);
      store_pair<F16>(BAh, BAl, kmaj(r, k1, 128), y[j].x * sa, y[j].z * sa);       // Re, k1 and k1 + 1
      store_pair<F16>(BAh, BAl, kmaj(r, 64 + k1, 128), y[j].y * sa, y[j].w * sa);  // Im
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // ---- stage A: D[2 n1 + part][item x 32 + k2], 3 split products x 8 K steps
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t idesc = tc_idesc<F16>(128, 128);
      const uint8_t *as[3] = {AAh, AAh, AAl}, *bs[3] = {BAh, BAl, BAh};
#pragma unroll 1
      for (int sp = 0; sp < 3; ++sp)
#pragma unroll 1
        for (int ks = 0; ks < 8; ++ks)
          tc_mma(tmem + (sp ? 128u : 0u), tc_desc(tc_smem(as[sp]) + ks * 256, 128),
                 tc_desc(tc_smem(bs[sp]) + ks * 256, 128), idesc, (sp == 2 || ks) ? 1u : 0u);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(&bar))
                   : "memory");
    }
    if (!tc_wait(&bar, phase, p.timeout_ns)) {
      if (tid == 0) atomicOr(p.status, kStatusFtcTimeout);
      stop = 1;
      tc_wait(&bar, phase, kDrainNs);  // bounded: the MMAs end before tensor memory is freed
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (stop) break;
    // ---- twiddle w^(n1 k2) / 64 on the stage-A result, into stage B's A operand
    {
      const int m = 32 * q + lane, n1 = m >> 1, part = m & 1;
#pragma unroll 1
      for (int c = 0; c < 2; ++c) {
        const int item = 2 * h + c, kb = 0;
        float v[32], vc[32];
        tc_ld32(tmem + lane_addr + (uint32_t)(64 * h + 32 * c), v);
        tc_ld32(tmem + lane_addr + (uint32_t)(128 + 64 * h + 32 * c), vc);
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) v[jj] += vc[jj];
        float z[32];
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) {
          const float other = __shfl_xor_sync(0xffffffffu, v[jj], 1);
          const float zr = part ? other : v[jj], zi = part ? v[jj] : other;
          const float2 w = TW[(kb + jj) * 64 + n1];
          z[jj] = (part == 0 ? zr * w.x - zi * w.y : zr * w.y + zi * w.x) * (1.0f / 64.0f);
        }
        uint8_t *abh = tsm + kBAh + h * 32768, *abl = abh + 16384;
        const int r = (item & 1) * 64 + n1;
#pragma unroll
        for (int jj = 0; jj < 32; jj += 2) store_pair<F16>(abh, abl, kmaj(r, part * 32 + kb + jj, 64), z[jj], z[jj + 1]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // ---- stage B: per item pair, D[item_in_pair x 64 + n1][re/im x 32 + n2]
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t idesc = tc_idesc<F16>(128, 64);
#pragma unroll 1
      for (int pr = 0; pr < 2; ++pr) {
        const uint8_t *abh = tsm + kBAh + pr * 32768, *abl = abh + 16384;
        const uint8_t *as[3] = {abh, abh, abl}, *bs[3] = {BBh, BBl, BBh};
#pragma unroll 1
        for (int sp = 0; sp < 3; ++sp)
#pragma unroll 1
          for (int ks = 0; ks < 4; ++ks)
            tc_mma(tmem + (sp ? 384u : 256u) + 64 * pr, tc_desc(tc_smem(as[sp]) + ks * 256, 64),
                   tc_desc(tc_smem(bs[sp]) + ks * 256, 64), idesc, (sp == 2 || ks) ? 1u : 0u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(&bar))
                   : "memory");
    }
    if (!tc_wait(&bar, phase, p.timeout_ns)) {
      if (tid == 0) atomicOr(p.status, kStatusFtcTimeout);
      stop = 1;
      tc_wait(&bar, phase, kDrainNs);  // bounded: the MMAs end before tensor memory is freed
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (stop) break;
    // ---- |y|^2, discard of the first O outputs, FOP store
    {
      const int m = 32 * q + lane, iip = m >> 6, n1 = m & 63;
      const int it = g * kTcItems + 2 * h + iip;
      float y[64];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        float cm[32];
        tc_ld32(tmem + lane_addr + (uint32_t)(256 + 64 * h + 32 * c), y + 32 * c);
        tc_ld32(tmem + lane_addr + (uint32_t)(384 + 64 * h + 32 * c), cm);
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) y[32 * c + jj] += cm[jj];
      }
      const float *yr = y, *yi = y + 32;
      if (FWD && it < n_items) {  // the tile's spectrum, natural order, unnormalised like fft2048_core
        float2 *out = p.tiles_out + (long long)it * kTile + n1;
        const float fs = pow2f(6 - sigma);
#pragma unroll
        for (int n2 = 0; n2 < 32; ++n2) out[64 * n2] = make_float2(yr[n2] * fs, yi[n2] * fs);
      } else if (!FWD && it < n_items) {
        const int tile = it / p.n_rows, row = p.row_begin + (it - tile * p.n_rows);
        float *out = p.fop + (long long)row * p.fop_stride;
        const long long base = (long long)tile * p.payload - p.overlap;
        const float fs = pow2f(12 - 2 * sigma);
#pragma unroll
        for (int n2 = 0; n2 < 32; ++n2) {
          const int n = n1 + 64 * n2;
          const long long b = base + n;
          if (n >= p.overlap && b < p.n_bins) out[b] = (yr[n2] * yr[n2] + yi[n2] * yi[n2]) * fs;
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols));
}

}  // namespace

cudaError_t launch_ftc_tc(const FtcParams &p, bool f16, cudaStream_t s) {
  if (p.n_rows <= 0 || p.n_tiles <= 0) return cudaSuccess;
  const int n_sm = current_sm_count();
  const long long groups = ((long long)p.n_tiles * p.n_rows + kTcItems - 1) / kTcItems;
  const int grid = (int)(groups < n_sm ? groups : n_sm);
  auto kern = f16 ? ftc_tc_kernel<true, false> : ftc_tc_kernel<false, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kTcThreads, kTcSmem, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_tile_tc(const TileParams &t, bool f16, int *status, long long timeout_ns, cudaStream_t s) {
  if (t.n_tiles <= 0) return cudaSuccess;
  FtcParams p{};
  p.input = t.input;
  p.tiles_out = t.tiles;
  p.n_bins = t.n_bins;
  p.n_tiles = t.n_tiles;
  p.overlap = t.overlap;
  p.payload = t.payload;
  p.n_rows = 1;
  p.twiddle = t.twiddle;
  p.status = status;
  p.timeout_ns = timeout_ns;
  const int n_sm = current_sm_count();
  const long long groups = ((long long)t.n_tiles + kTcItems - 1) / kTcItems;
  const int grid = (int)(groups < n_sm ? groups : n_sm);
  auto kern = f16 ? ftc_tc_kernel<true, true> : ftc_tc_kernel<false, true>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kTcThreads, kTcSmem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace fdas
