// Upstream step: the normalised spectrum of a real time series
// (ft_conv.py:134-143: ``ft = fft(samples) / n_samp``, first N bins kept).
//
// The 2N real samples are read as N complex values z[n] = x[2n] + i x[2n+1]
// (no copy), transformed by an N-point complex FFT, and split into the
// spectrum of the real series:
//   X[k] = (Z[k] + conj Z[N-k]) / 2 - i e^(-i pi k / N) (Z[k] - conj Z[N-k]) / 2.
// The N-point FFT is a mixed-radix Stockham auto-sort FFT (radices 8, 4, 2, 3,
// 5, 7; one kernel launch per radix pass, ping-ponging between two device
// buffers), following the radix-R formulation of Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors" (SC 2008).
// FP32 arithmetic; the twiddle table e^(-i pi x / N), x < N, is computed on
// the device in FP64 and rounded once.
#include <cuda_runtime.h>

#include "fft2048.cuh"
#include "kernels.cuh"

namespace fdas {

// e^(-i pi x / N), x < N
__global__ void series_twiddle_kernel(float2 *tw, int n) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  double s, c;
  sincospi(-(double)x / (double)n, &s, &c);
  tw[x] = make_float2((float)c, (float)s);
}

// e^(-2 pi i m / N) for 0 <= m < N from the half-step table
__device__ __forceinline__ float2 tw_full(const float2 *__restrict__ tw, long long m, int n) {
  const long long x = 2 * m;
  if (x < n) return __ldg(tw + x);
  const float2 t = __ldg(tw + (x - n));
  return make_float2(-t.x, -t.y);
}

// forward DFT of odd size R on v[0..R) (direct, compile-time twiddles)
template <int R>
__device__ __forceinline__ void dft_odd(float2 *v) {
  float2 out[R];
  sfor<R>([&](auto K) {
    constexpr int k = decltype(K)::value;
    float2 acc = v[0];
    sfor<R - 1>([&](auto N1) {
      constexpr int n = decltype(N1)::value + 1;
      constexpr int j = (n * k) % R;
      acc = cadd(acc, rot<-1, R, j>(v[n]));
    });
    out[k] = acc;
  });
  sfor<R>([&](auto K) {
    constexpr int k = decltype(K)::value;
    v[k] = out[k];
  });
}

// One Stockham pass of radix R: for j < N / R, with k = j mod Ns,
//   v[r] = in[j + r N / R] e^(-2 pi i k r / (Ns R)),  v = DFT_R(v),
//   out[(j / Ns) Ns R + k + r Ns] = v[r].
template <int R>
__global__ void __launch_bounds__(256) stockham_kernel(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                       int n, int ns, const float2 *__restrict__ tw) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = n / R;
  if (j >= m) return;
  const int k = j % ns;
  float2 v[R];
  sfor<R>([&](auto Rr) {
    constexpr int r = decltype(Rr)::value;
    v[r] = __ldg(in + j + (long long)r * m);
  });
  if (ns > 1) {
    const long long step = (long long)k * (n / (ns * R));  // twiddle exponent unit for this j
    sfor<R - 1>([&](auto Rr) {
      constexpr int r = decltype(Rr)::value + 1;
      v[r] = cmul(v[r], tw_full(tw, step * r, n));
    });
  }
  if constexpr (R == 2 || R == 4 || R == 8) dft_small<-1, R, 0, 1>(v);
  else dft_odd<R>(v);
  const long long base = (long long)(j / ns) * ns * R + k;
  sfor<R>([&](auto Rr) {
    constexpr int r = decltype(Rr)::value;
    out[base + (long long)r * ns] = v[r];
  });
}

// Real-input split step, one thread per pair (k, N - k), 0 <= k <= N / 2;
// in place when z == x.
__global__ void __launch_bounds__(256) real_split_kernel(const float2 *z, float2 *x, int n, float scale,
                                                         const float2 *__restrict__ tw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > n / 2) return;
  const int kk = (n - k) % n;
  const float2 a = z[k], b = z[kk];
  auto bin = [&](float2 za, float2 zb, int q) {
    // Fe = (za + conj zb) / 2, Fo = (za - conj zb) / (2 i); X = Fe + e^(-i pi q / N) Fo
    const float2 fe = make_float2(0.5f * (za.x + zb.x), 0.5f * (za.y - zb.y));
    const float2 fo = make_float2(0.5f * (za.y + zb.y), -0.5f * (za.x - zb.x));
    const float2 w = __ldg(tw + q);
    const float2 r = cadd(fe, cmul(w, fo));
    return make_float2(scale * r.x, scale * r.y);
  };
  const float2 xk = bin(a, b, k);
  if (kk != k && k != 0) {
    const float2 xkk = bin(b, a, kk);
    x[kk] = xkk;
  }
  x[k] = xk;
}

namespace {
template <int R>
cudaError_t pass(const float2 *in, float2 *out, int n, int ns, const float2 *tw, cudaStream_t s) {
  const int m = n / R;
  stockham_kernel<R><<<(m + 255) / 256, 256, 0, s>>>(in, out, n, ns, tw);
  return cudaGetLastError();
}
}  // namespace

int series_radices(int n, int *radix, int max_passes) {
  int np = 0;
  const int pref[6] = {8, 4, 2, 3, 5, 7};
  while (n > 1) {
    int r = 0;
    for (int c : pref)
      if (n % c == 0) {
        r = c;
        break;
      }
    if (!r || np >= max_passes) return -1;
    radix[np++] = r;
    n /= r;
  }
  return np;
}

cudaError_t launch_series_twiddles(float2 *tw, int n, cudaStream_t s) {
  series_twiddle_kernel<<<(n + 255) / 256, 256, 0, s>>>(tw, n);
  return cudaGetLastError();
}

cudaError_t launch_series_spectrum(const SeriesParams &p, cudaStream_t s) {
  int radix[64];
  const int np = series_radices(p.n, radix, 64);
  if (np < 0) return cudaErrorInvalidValue;
  const float2 *cur = p.z;
  float2 *bufs[2] = {p.scratch, p.z};
  int ns = 1;
  for (int i = 0; i < np; ++i) {
    float2 *dst = bufs[i & 1];
    cudaError_t e;
    switch (radix[i]) {
      case 8: e = pass<8>(cur, dst, p.n, ns, p.tw, s); break;
      case 4: e = pass<4>(cur, dst, p.n, ns, p.tw, s); break;
      case 2: e = pass<2>(cur, dst, p.n, ns, p.tw, s); break;
      case 3: e = pass<3>(cur, dst, p.n, ns, p.tw, s); break;
      case 5: e = pass<5>(cur, dst, p.n, ns, p.tw, s); break;
      default: e = pass<7>(cur, dst, p.n, ns, p.tw, s); break;
    }
    if (e != cudaSuccess) return e;
    cur = dst;
    ns *= radix[i];
  }
  real_split_kernel<<<(p.n / 2 + 1 + 255) / 256, 256, 0, s>>>(cur, p.z, p.n, p.scale, p.tw);
  return cudaGetLastError();
}

}  // namespace fdas
