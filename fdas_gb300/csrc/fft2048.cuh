// Warp-level 2048-point complex FFT for sm_103a.
//
// One warp computes one 2048-point transform: each of the 32 lanes holds 64
// complex values in registers.  The transform is split as 2048 = 64 x 32 with
// a single shared-memory exchange:
//
//   inverse (sign +1), input Y[k] in natural order, k = 32 k' + kappa:
//     pass 1  lane kappa:  Z_kappa[m] = DFT64_k'( Y[32 k' + kappa] )      m in [0,64)
//     twiddle             V_kappa[m] = Z_kappa[m] * w^(m kappa),  w = e^(+2 pi i / 2048)
//     exchange            lane l gets V_kappa[l], V_kappa[l + 32] for all kappa
//     pass 2  lane l:     y[m + 64 d] = DFT32_kappa( V_kappa[m] ),  m in {l, l+32}
//   so lane l ends with outputs n = l + 32 c + 64 d (c in {0,1}, d in [0,32)):
//   for fixed (c, d) the 32 lanes hold 32 consecutive outputs.
//
//   forward (sign -1) is the mirror image: natural-order input x[m + 64 d] is
//   loaded with lane l holding m in {l, l+32}; DFT32 over d, twiddle
//   w^(-m kappa), exchange, DFT64 over m; lane kappa ends with X[32 k' + kappa].
//
// Global loads and stores of both directions are therefore unit-stride across
// the warp, which makes every access coalesced without any permutation of the
// spectra in memory.  The FPGA reference uses a radix-2^2 streaming engine with
// bit-reversed output instead (fft_4p.cl); only the transform is shared.
//
// Small DFTs (4, 8, 32 = 4x8, 64 = 8x8) are fully unrolled with compile-time
// twiddle constants (template variables evaluated by the host compiler), so
// trivial rotations cost no multiplies.
#pragma once

#include <cuda_runtime.h>
#include <utility>
#include <type_traits>

namespace fdas {

// ---------------------------------------------------------------- constants
constexpr double kTwoPi = 6.283185307179586476925286766559;

// cos / sin by Taylor series after reduction to [-pi/4, pi/4]; only ever
// evaluated by the host compiler when initialising constexpr template
// variables below.
constexpr double taylor_cos(double x) {
  double s = 0, t = 1;
  for (int i = 0; i < 24; ++i) { s += t; t *= -x * x / ((2.0 * i + 1) * (2.0 * i + 2)); }
  return s;
}
constexpr double taylor_sin(double x) {
  double s = 0, t = x;
  for (int i = 0; i < 24; ++i) { s += t; t *= -x * x / ((2.0 * i + 2) * (2.0 * i + 3)); }
  return s;
}
// cos(2 pi j / n), sin(2 pi j / n) for integer j, n using octant symmetry
constexpr double cexpr_cos_frac(long j, long n) {
  j = ((j % n) + n) % n;
  // reduce to the first octant with exact integer arithmetic on 8 j / n
  long e = 8 * j;  // angle in units of (2 pi / 8n)
  long oct = e / n;
  long rem = e - oct * n;  // angle = (oct + rem/n) * pi/4
  double a = (kTwoPi / 8.0) * (double)rem / (double)n;
  double b = (kTwoPi / 8.0) - a;
  switch (oct) {
    case 0: return taylor_cos(a);
    case 1: return taylor_sin(b);
    case 2: return -taylor_sin(a);
    case 3: return -taylor_cos(b);
    case 4: return -taylor_cos(a);
    case 5: return -taylor_sin(b);
    case 6: return taylor_sin(a);
    default: return taylor_cos(b);
  }
}
// sin(2 pi j / n) = cos(2 pi (4 j - n) / 4 n), exact for every n
constexpr double cexpr_sin_frac(long j, long n) { return cexpr_cos_frac(4 * j - n, 4 * n); }

template <int N, int J> constexpr float kCos = (float)cexpr_cos_frac(J, N);
template <int N, int J> constexpr float kSin = (float)cexpr_sin_frac(J, N);
constexpr float kRsqrt2 = 0.70710678118654752440f;

// ------------------------------------------------------------ static for
template <typename F, int... I>
__device__ __forceinline__ void sfor_impl(F &&f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void sfor(F &&f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// ------------------------------------------------------------ complex ops
// Complex add / subtract as one packed FP32 pair instruction (add.rn.f32x2 /
// sub.rn.f32x2, sm_100 and later): each half is an ordinary round-to-nearest
// FP32 add, so results equal two scalar adds.
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
// a + c b and a - c b for a real constant c, as packed fused multiply-adds
__device__ __forceinline__ float2 cfma_real(float c, float2 b, float2 a) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_pack(make_float2(c, c))), "l"(f2_pack(b)), "l"(f2_pack(a)));
  return f2_unpack(r);
}
// c b for a real c, as one packed multiply
__device__ __forceinline__ float2 cscale(float c, float2 b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(make_float2(c, c))), "l"(f2_pack(b)));
  return f2_unpack(r);
}
// t + S i d and t - S i d (rotation by +-90 degrees folded into scalar adds)
template <int S>
__device__ __forceinline__ void add_sub_i(float2 t, float2 d, float2 &plus, float2 &minus) {
  if constexpr (S > 0) {
    plus = make_float2(t.x - d.y, t.y + d.x);
    minus = make_float2(t.x + d.y, t.y - d.x);
  } else {
    plus = make_float2(t.x + d.y, t.y - d.x);
    minus = make_float2(t.x - d.y, t.y + d.x);
  }
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// v * e^(S i 2 pi J / N) with compile-time S, N, J.  Rotations by multiples of
// pi/4 use the cheap forms.
template <int S, int N, int J>
__device__ __forceinline__ float2 rot(float2 v) {
  constexpr int j = ((J % N) + N) % N;
  if constexpr (j == 0) {
    return v;
  } else if constexpr (2 * j == N) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (4 * j == N) {  // * (S i)
    return S > 0 ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  } else if constexpr (4 * j == 3 * N) {  // * (-S i)
    return S > 0 ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  } else if constexpr (8 * j == N) {  // r (1 + S i)
    return S > 0 ? make_float2(kRsqrt2 * (v.x - v.y), kRsqrt2 * (v.y + v.x))
                 : make_float2(kRsqrt2 * (v.x + v.y), kRsqrt2 * (v.y - v.x));
  } else if constexpr (8 * j == 3 * N) {  // r (-1 + S i)
    return S > 0 ? make_float2(-kRsqrt2 * (v.x + v.y), kRsqrt2 * (v.x - v.y))
                 : make_float2(kRsqrt2 * (v.y - v.x), -kRsqrt2 * (v.x + v.y));
  } else if constexpr (8 * j == 5 * N) {  // r (-1 - S i)
    return S > 0 ? make_float2(kRsqrt2 * (v.y - v.x), -kRsqrt2 * (v.x + v.y))
                 : make_float2(-kRsqrt2 * (v.x + v.y), kRsqrt2 * (v.x - v.y));
  } else if constexpr (8 * j == 7 * N) {  // r (1 - S i)
    return S > 0 ? make_float2(kRsqrt2 * (v.x + v.y), kRsqrt2 * (v.y - v.x))
                 : make_float2(kRsqrt2 * (v.x - v.y), kRsqrt2 * (v.y + v.x));
  } else {
    constexpr float c = kCos<N, j>;
    constexpr float s = S * kSin<N, j>;
    return make_float2(fmaf(v.x, c, -v.y * s), fmaf(v.x, s, v.y * c));
  }
}

// ------------------------------------------------------------ small DFTs
// In-place DFTs on v[OFF + STRIDE * i]; outputs in natural order.
template <int S, int OFF, int STRIDE>
__device__ __forceinline__ void dft2(float2 *v) {
  float2 a = v[OFF], b = v[OFF + STRIDE];
  v[OFF] = cadd(a, b);
  v[OFF + STRIDE] = csub(a, b);
}

template <int S, int OFF, int STRIDE>
__device__ __forceinline__ void dft4(float2 *v) {
  float2 x0 = v[OFF], x1 = v[OFF + STRIDE], x2 = v[OFF + 2 * STRIDE], x3 = v[OFF + 3 * STRIDE];
  float2 t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), d = csub(x1, x3);
  v[OFF] = cadd(t0, t2);
  v[OFF + 2 * STRIDE] = csub(t0, t2);
  add_sub_i<S>(t1, d, v[OFF + STRIDE], v[OFF + 3 * STRIDE]);
}

template <int S, int OFF, int STRIDE>
__device__ __forceinline__ void dft8(float2 *v) {
  // radix-2 decimation in time: two DFT4 on even / odd inputs
  float2 e[4] = {v[OFF], v[OFF + 2 * STRIDE], v[OFF + 4 * STRIDE], v[OFF + 6 * STRIDE]};
  float2 o[4] = {v[OFF + STRIDE], v[OFF + 3 * STRIDE], v[OFF + 5 * STRIDE], v[OFF + 7 * STRIDE]};
  dft4<S, 0, 1>(e);
  dft4<S, 0, 1>(o);
  // o1 w^1 = r (1 + S i) o1 = r u1, o3 w^3 = r (-1 + S i) o3 = r u3, o2 w^2 = S i o2
  const float2 u1 = S > 0 ? make_float2(o[1].x - o[1].y, o[1].y + o[1].x)
                          : make_float2(o[1].x + o[1].y, o[1].y - o[1].x);
  const float2 u3 = S > 0 ? make_float2(-(o[3].x + o[3].y), o[3].x - o[3].y)
                          : make_float2(o[3].y - o[3].x, -(o[3].x + o[3].y));
  v[OFF] = cadd(e[0], o[0]);
  v[OFF + 4 * STRIDE] = csub(e[0], o[0]);
  v[OFF + STRIDE] = cfma_real(kRsqrt2, u1, e[1]);
  v[OFF + 5 * STRIDE] = cfma_real(-kRsqrt2, u1, e[1]);
  add_sub_i<S>(e[2], o[2], v[OFF + 2 * STRIDE], v[OFF + 6 * STRIDE]);
  v[OFF + 3 * STRIDE] = cfma_real(kRsqrt2, u3, e[3]);
  v[OFF + 7 * STRIDE] = cfma_real(-kRsqrt2, u3, e[3]);
}

template <int S, int R, int OFF, int STRIDE>
__device__ __forceinline__ void dft_small(float2 *v) {
  if constexpr (R == 2) dft2<S, OFF, STRIDE>(v);
  else if constexpr (R == 4) dft4<S, OFF, STRIDE>(v);
  else dft8<S, OFF, STRIDE>(v);
}

// Composite DFT of size R1*R2 on v[OFF + STRIDE * n] (n natural order).
// Output X[k1 + R1 k2] is left in v[OFF + STRIDE * (R2 k1 + k2)].
template <int S, int R1, int R2, int OFF, int STRIDE>
__device__ __forceinline__ void dft_composite(float2 *v) {
  constexpr int N = R1 * R2;
  // step 1: R2 DFTs of size R1 over n1 (n = R2 n1 + n2)
  sfor<R2>([&](auto N2) {
    constexpr int n2 = decltype(N2)::value;
    dft_small<S, R1, OFF + STRIDE * n2, STRIDE * R2>(v);
  });
  // step 2: internal twiddles w_N^(n2 k1)
  sfor<R1>([&](auto K1) {
    constexpr int k1 = decltype(K1)::value;
    sfor<R2>([&](auto N2) {
      constexpr int n2 = decltype(N2)::value;
      constexpr int idx = OFF + STRIDE * (R2 * k1 + n2);
      v[idx] = rot<S, N, n2 * k1>(v[idx]);
    });
  });
  // step 3: R1 DFTs of size R2 over n2
  sfor<R1>([&](auto K1) {
    constexpr int k1 = decltype(K1)::value;
    dft_small<S, R2, OFF + STRIDE * R2 * k1, STRIDE>(v);
  });
}

// Register slot of output k for the 64 = 8x8 and 32 = 4x8 transforms.
__host__ __device__ constexpr int pos64(int k) { return 8 * (k % 8) + k / 8; }
__host__ __device__ constexpr int pos32(int k) { return 8 * (k % 4) + k / 4; }

template <int S, int OFF>
__device__ __forceinline__ void dft64(float2 *v) { dft_composite<S, 8, 8, OFF, 1>(v); }
template <int S, int OFF>
__device__ __forceinline__ void dft32(float2 *v) { dft_composite<S, 4, 8, OFF, 1>(v); }

// ------------------------------------------------------------ exchange
// Shared-memory buffer of one warp: 32 rows (kappa) x 64 columns (m), row
// pitch 66 complex values: 16-byte row starts and conflict-free access for
// both the 8-byte column-wise and 16-byte row-wise patterns below.
constexpr int kExPitch = 66;
constexpr int kExFloats = 32 * kExPitch * 2;  // floats per warp

// Per-lane twiddle bases for w^(m * lane), m = mlo + 8 mhi:
//   lo[j] = w^(j lane), hi[j] = w^(8 j lane), j in [0, 8).
// ``table`` holds e^(i 2 pi j / 2048), j in [0, 2048) (sign applied here).
struct TwiddleBases {
  float2 lo[8];
  float2 hi[8];
};

template <int S>
__device__ __forceinline__ TwiddleBases load_twiddle_bases(const float2 *__restrict__ table, int lane) {
  TwiddleBases tb;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float2 a = __ldg(table + ((j * lane) & 2047));
    float2 b = __ldg(table + ((8 * j * lane) & 2047));
    tb.lo[j] = make_float2(a.x, S * a.y);
    tb.hi[j] = make_float2(b.x, S * b.y);
  }
  return tb;
}

struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

// Inverse transform core: v[64] holds Y[32 k' + lane] at v[k'] on entry.  On
// exit v[32 c + pos32(d)] holds y[lane + 32 c + 64 d].  ``ex`` is this warp's
// exchange buffer (kExFloats floats, 16-byte aligned); ``after_exchange`` runs
// (on all lanes) once the buffer has been read back and is free again.
template <typename Hook = NoHook>
__device__ __forceinline__ void ifft2048_core(float2 *v, const TwiddleBases &tb, float *ex, int lane,
                                              Hook after_exchange = Hook()) {
  dft64<+1, 0>(v);
  // twiddle V[m] = Z[m] w^(m lane);  Z[m] sits at v[pos64(m)] = v[8 mlo + mhi]
  sfor<8>([&](auto MLO) {
    constexpr int mlo = decltype(MLO)::value;
    sfor<8>([&](auto MHI) {
      constexpr int mhi = decltype(MHI)::value;
      constexpr int idx = 8 * mlo + mhi;
      if constexpr (mlo == 0 && mhi == 0) {
      } else if constexpr (mlo == 0) {
        v[idx] = cmul(v[idx], tb.hi[mhi]);
      } else if constexpr (mhi == 0) {
        v[idx] = cmul(v[idx], tb.lo[mlo]);
      } else {
        v[idx] = cmul(v[idx], cmul(tb.lo[mlo], tb.hi[mhi]));
      }
    });
  });
  // exchange: row = lane (kappa), column m; 16-byte stores of (m, m+1)
  __syncwarp();  // every lane is done with whatever the buffer held before
  float4 *row = reinterpret_cast<float4 *>(ex + 2 * kExPitch * lane);
  sfor<32>([&](auto P) {
    constexpr int p = decltype(P)::value;  // m = 2p, 2p+1
    float2 a = v[pos64(2 * p)], b = v[pos64(2 * p + 1)];
    row[p] = make_float4(a.x, a.y, b.x, b.y);
  });
  __syncwarp();
  const float2 *col = reinterpret_cast<const float2 *>(ex);
  sfor<2>([&](auto C) {
    constexpr int c = decltype(C)::value;
    sfor<32>([&](auto K) {
      constexpr int kap = decltype(K)::value;
      v[32 * c + kap] = col[kExPitch * kap + lane + 32 * c];
    });
  });
  __syncwarp();
  after_exchange();
  dft32<+1, 0>(v);
  dft32<+1, 32>(v);
}

// Forward transform core: v[32 c + d] holds x[lane + 32 c + 64 d] on entry.
// On exit v[pos64(k')] holds X[32 k' + lane].
__device__ __forceinline__ void fft2048_core(float2 *v, const TwiddleBases &tb, float *ex, int lane) {
  dft32<-1, 0>(v);
  dft32<-1, 32>(v);
  // twiddle: U_m[kappa] * w^(-m kappa), m = lane + 32 c, kappa = klo + 8 khi.
  // w^(-(lane + 32c) kappa) = w^(-lane kappa) * e^(-2 pi i c kappa / 64)
  // per-lane part from the bases: kappa = klo + 8 khi -> lo[klo] * hi[khi]
  sfor<2>([&](auto C) {
    constexpr int c = decltype(C)::value;
    sfor<32>([&](auto K) {
      constexpr int kap = decltype(K)::value;
      constexpr int klo = kap % 8, khi = kap / 8;
      constexpr int idx = 32 * c + pos32(kap);
      float2 t = v[idx];
      if constexpr (klo != 0 && khi != 0) t = cmul(t, cmul(tb.lo[klo], tb.hi[khi]));
      else if constexpr (klo != 0) t = cmul(t, tb.lo[klo]);
      else if constexpr (khi != 0) t = cmul(t, tb.hi[khi]);
      if constexpr (c == 1) t = rot<-1, 64, kap>(t);
      v[idx] = t;
    });
  });
  // exchange: column writes (8-byte), row reads (16-byte)
  float2 *col = reinterpret_cast<float2 *>(ex);
  sfor<2>([&](auto C) {
    constexpr int c = decltype(C)::value;
    sfor<32>([&](auto K) {
      constexpr int kap = decltype(K)::value;
      col[kExPitch * kap + lane + 32 * c] = v[32 * c + pos32(kap)];
    });
  });
  __syncwarp();
  const float4 *row = reinterpret_cast<const float4 *>(ex + 2 * kExPitch * lane);
  sfor<32>([&](auto P) {
    constexpr int p = decltype(P)::value;
    float4 q = row[p];
    v[2 * p] = make_float2(q.x, q.y);
    v[2 * p + 1] = make_float2(q.z, q.w);
  });
  __syncwarp();
  dft64<-1, 0>(v);
}

}  // namespace fdas

namespace fdas {

// ---------------------------------------------------------------------------
// Two-warp inverse transform: 64 threads x 32 complex values (half the
// registers of the one-warp form, so twice the warps per SM).
//
//   thread p = 32 h + l (h: warp of the pair, l: lane), input Y[64 a + p]:
//   pass 1   Z_p[m] = DFT32_a( Y[64 a + p] ),            m in [0,32)
//   twiddle  V_p[m] = Z_p[m] w^(m p)
//   exchange (shared memory, across the two warps): thread (h, l) takes
//            m = 16 h + (l & 15), g = l >> 4 and the 32 values
//            V_{p1 + 8 p2}[m], p1 = 4 g + q (q < 4), p2 < 8
//   pass 2a  U_{p1}[d1] = DFT8_p2(V_{p1 + 8 p2}[m]) e^(2 pi i d1 p1 / 64)
//   exchange (register shuffle with lane l ^ 16): each thread keeps four d1
//            values for all eight p1
//   pass 2c  y[m + 32 d1 + 256 d2] = DFT8_p1( U_{p1}[d1] )
//
// Lanes with g = 1 modulate their pass-2a inputs by (-1)^p2, which moves
// their own d1 half (4..7) into register slots 0..3, so the shuffle pattern is
// the same for all lanes; they then feed their p1 halves to the last DFT8 in
// swapped order, which multiplies the outputs by (-1)^d2 -- harmless, since
// only |y|^2 is used.  The result is therefore given as |y|^2 only.
// Rows of 34 complex values (272 bytes): 16-byte aligned, so pass 1 writes
// pairs of values with 16-byte stores (the 8 lanes of a store phase hit banks
// 4 p mod 32, four wide: no conflicts), and the column reads of pass 2 stay
// conflict-free (a half-warp reads 16 consecutive values of one row).
constexpr int kEx2Pitch = 34;                 // complex values per row of the pair buffer
constexpr int kEx2Floats = 64 * kEx2Pitch * 2;  // floats per warp pair (>= 2048 complex)

// Twiddles w^(m p) of the two-warp transform, m < 32, p < 64, with the pair
// (m, m + 1), m even, of each p next to each other: w^(m p) at
// [128 (m / 2) + 2 p + (m & 1)], so a thread loads two with one 16-byte load
// (16 KB of shared memory per CTA, shared by its warp pairs).
constexpr int kTw2Floats = 2 * 32 * 64;

__device__ __forceinline__ void fill_twiddle2(float2 *twt, const float2 *__restrict__ table) {
  for (int i = threadIdx.x; i < 32 * 64; i += blockDim.x) {
    const int m = i >> 6, p = i & 63;
    twt[128 * (m >> 1) + 2 * p + (m & 1)] = __ldg(table + ((m * p) & 2047));
  }
}

// Pass 1 + twiddle + write to the pair buffer.  v[a] holds Y[64 a + p] on entry.
__device__ __forceinline__ void ifft2_pass1(float2 *v, const float2 *twt, float2 *buf, int p) {
  dft32<+1, 0>(v);
  // V_p[m] = Z_p[m] w^(m p); Z_p[m] sits in v[pos32(m)]; twiddles two at a time
  const float4 *tw4 = reinterpret_cast<const float4 *>(twt) + p;
  sfor<16>([&](auto M2) {
    constexpr int m = 2 * decltype(M2)::value;
    const float4 w = tw4[64 * (m >> 1)];
    if constexpr (m != 0) v[pos32(m)] = cmul(v[pos32(m)], make_float2(w.x, w.y));
    v[pos32(m + 1)] = cmul(v[pos32(m + 1)], make_float2(w.z, w.w));
  });
  float4 *row = reinterpret_cast<float4 *>(buf + kEx2Pitch * p);
  sfor<16>([&](auto M2) {
    constexpr int m = 2 * decltype(M2)::value;
    const float2 a = v[pos32(m)], b = v[pos32(m + 1)];
    row[m >> 1] = make_float4(a.x, a.y, b.x, b.y);
  });
}

// Passes 2a / 2c after the pair buffer has been written by both warps.  On
// exit pw[8 r + d2] holds |y[m + 32 (4 g + r) + 256 d2]|^2, m = 16 h + (l & 15).
template <typename Hook>
__device__ __forceinline__ void ifft2_pass2(const float2 *buf, int h, int lane, float *pw, Hook after_read) {
  const int m = 16 * h + (lane & 15);
  const int g = lane >> 4;
  float2 u[32];  // u[8 q + p2]
  sfor<4>([&](auto Q) {
    constexpr int q = decltype(Q)::value;
    sfor<8>([&](auto P2) {
      constexpr int p2 = decltype(P2)::value;
      u[8 * q + p2] = buf[kEx2Pitch * (4 * g + q + 8 * p2) + m];
    });
  });
  after_read();
  // lanes of group 1: (-1)^p2 modulation moves d1 = 4..7 to slots 0..3
  const float sg = g ? -1.f : 1.f;
  sfor<4>([&](auto Q) {
    constexpr int q = decltype(Q)::value;
    sfor<4>([&](auto P2) {
      constexpr int p2 = 2 * decltype(P2)::value + 1;
      u[8 * q + p2] = cscale(sg, u[8 * q + p2]);
    });
    dft8<+1, 8 * q, 1>(u);
    // twiddle e^(2 pi i d1 p1 / 64); constants differ per lane group
    sfor<8>([&](auto D) {
      constexpr int d = decltype(D)::value;
      constexpr float c0r = kCos<64, ((d & 7) * q)>, c0i = kSin<64, ((d & 7) * q)>;
      constexpr float c1r = kCos<64, (((d + 4) & 7) * (4 + q))>, c1i = kSin<64, (((d + 4) & 7) * (4 + q))>;
      const float2 c = make_float2(g ? c1r : c0r, g ? c1i : c0i);
      u[8 * q + d] = cmul(u[8 * q + d], c);
    });
  });
  // exchange with lane ^ 16: send slots 4..7, receive the partner's, in place
  sfor<4>([&](auto Q) {
    constexpr int q = decltype(Q)::value;
    sfor<4>([&](auto R) {
      constexpr int r = decltype(R)::value;
      float2 &x = u[8 * q + 4 + r];
      x.x = __shfl_xor_sync(0xffffffffu, x.x, 16);
      x.y = __shfl_xor_sync(0xffffffffu, x.y, 16);
    });
  });
  // pass 2c: for each own d1 slot r, DFT8 over p1 = (own q = 0..3, partner q = 0..3)
  sfor<4>([&](auto R) {
    constexpr int r = decltype(R)::value;
    float2 x[8];
    sfor<4>([&](auto Q) {
      constexpr int q = decltype(Q)::value;
      x[q] = u[8 * q + r];
      x[4 + q] = u[8 * q + 4 + r];
    });
    dft8<+1, 0, 1>(x);
    sfor<8>([&](auto D2) {
      constexpr int d2 = decltype(D2)::value;
      pw[8 * r + d2] = fmaf(x[d2].x, x[d2].x, x[d2].y * x[d2].y);
    });
  });
}

}  // namespace fdas
