// SPOD Fourier stage: Welch blocks of the mean-removed snapshot matrix,
// windowed and transformed along time, written per frequency as the
// M x nBlks complex matrices the per-frequency SVDs consume.
//
// Reference behaviour (pyLowOrder pyLOM/SPOD/wrapper.py:24-85, _fft at :18):
//   block b starts at b*(nDFT - nolap); Xf = Y[:, i0:i0+nDFT] * window;
//   qk = winWeight/nDFT * fft(Xf)[:, :nf]; qk[:, 1:-1] *= 2;
//   Q_f = qk[:, f] over blocks, divided by sqrt(nBlks) before its SVD.
// Here `scale` = winWeight / nDFT / sqrt(nBlks) and the output layout is
// Q[f][i][b] (complex, interleaved re/im): Q_f is row-major M x nBlks.
//
// GB300 mapping: a CTA owns R consecutive points; each warp transforms whole
// windows (radix-2 decimation-in-time FFT in its own shared-memory buffer
// when nDFT is a power of two, a direct DFT from a twiddle table otherwise);
// results are staged in shared memory as [row][block][bin] and streamed out
// per frequency as contiguous R*nBlks runs.  HBM-bound: bytes = read M*N*s +
// write M*nBlks*nf*2s.
#include <algorithm>
#include <cmath>

#include "plom_common.cuh"
#include "plom_kernels.cuh"

namespace plom {

template <typename T>
struct c2 {
  T re, im;
};

template <typename T>
__global__ void __launch_bounds__(256) spod_fft_kernel(
    const T* __restrict__ Y, int64_t M, int64_t N, int64_t ldy, const T* __restrict__ mean,
    int nDFT, int log2n, int step, int nBlks, int nf, const T* __restrict__ window,
    const T* __restrict__ twr, const T* __restrict__ twi, T scale, int R, T* __restrict__ Q) {
  extern __shared__ unsigned char smem_raw[];
  T* sw = reinterpret_cast<T*>(smem_raw);                    // window  [nDFT]
  T* sc = sw + nDFT;                                          // cos     [nDFT]
  T* ss = sc + nDFT;                                          // sin     [nDFT]
  c2<T>* buf = reinterpret_cast<c2<T>*>(ss + nDFT);           // 8 warps x nDFT
  c2<T>* stage = buf + 8 * (size_t)nDFT;                      // R x nBlks x nf
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int j = tid; j < nDFT; j += blockDim.x) {
    sw[j] = window[j];
    sc[j] = twr[j];
    ss[j] = twi[j];
  }
  __syncthreads();
  const int64_t i0 = (int64_t)blockIdx.x * R;
  const int rows = (int)std::min<int64_t>((int64_t)R, M - i0);
  c2<T>* wb = buf + (size_t)warp * nDFT;
  const int nwin = rows * nBlks;
  for (int wdx = warp; wdx < nwin; wdx += 8) {
    const int r = wdx / nBlks, b = wdx % nBlks;
    const T* x = Y + (i0 + r) * ldy + (int64_t)b * step;
    const T mu = mean ? mean[i0 + r] : T(0);  // temporal mean removed on load
    c2<T>* out = stage + ((size_t)r * nBlks + b) * nf;
    if (log2n >= 0) {
      // windowed samples into bit-reversed positions
      for (int j = lane; j < nDFT; j += 32) {
        const unsigned rj = __brev((unsigned)j) >> (32 - log2n);
        wb[rj].re = (x[j] - mu) * sw[j];
        wb[rj].im = T(0);
      }
      __syncwarp();
      for (int s = 1; s <= log2n; ++s) {
        const int half = 1 << (s - 1);
        const int tstride = nDFT >> s;  // twiddle index step
        for (int bf = lane; bf < nDFT / 2; bf += 32) {
          const int grp = bf / half, pos = bf % half;
          const int a = grp * 2 * half + pos, c = a + half;
          const T wr = sc[pos * tstride], wi = ss[pos * tstride];  // e^{-2 pi i k / n}
          const c2<T> u = wb[a], v = wb[c];
          const T tr = v.re * wr - v.im * wi, ti = v.re * wi + v.im * wr;
          wb[a].re = u.re + tr;
          wb[a].im = u.im + ti;
          wb[c].re = u.re - tr;
          wb[c].im = u.im - ti;
        }
        __syncwarp();
      }
      for (int k = lane; k < nf; k += 32) {
        const T f = (k >= 1 && k <= nf - 2) ? T(2) * scale : scale;
        out[k].re = wb[k].re * f;
        out[k].im = wb[k].im * f;
      }
      __syncwarp();
    } else {
      // direct DFT (nDFT not a power of two)
      for (int j = lane; j < nDFT; j += 32) {
        wb[j].re = (x[j] - mu) * sw[j];
        wb[j].im = T(0);
      }
      __syncwarp();
      for (int k = lane; k < nf; k += 32) {
        T sr = 0, si = 0;
        int idx = 0;
        for (int j = 0; j < nDFT; ++j) {
          sr += wb[j].re * sc[idx];
          si += wb[j].re * ss[idx];
          idx += k;
          if (idx >= nDFT) idx -= nDFT;
        }
        const T f = (k >= 1 && k <= nf - 2) ? T(2) * scale : scale;
        out[k].re = sr * f;
        out[k].im = si * f;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  // stream out: Q[f][i0 + r][b]
  const int per_f = rows * nBlks;
  c2<T>* Qc = reinterpret_cast<c2<T>*>(Q);
  for (int64_t e = tid; e < (int64_t)nf * per_f; e += blockDim.x) {
    const int f = (int)(e / per_f), rb = (int)(e % per_f);
    const int r = rb / nBlks, b = rb % nBlks;
    Qc[((int64_t)f * M + i0 + r) * nBlks + b] = stage[((size_t)r * nBlks + b) * nf + f];
  }
}

// ---------------------------------------------------------------------------
// Fast path: FP32 data, nDFT = 32 E with E a power of two (1..32).  One warp
// transforms one window in registers: lane l holds samples l + 32 e; an
// E-point DIF FFT over its registers, twiddles w_N^(l k1), then a 32-point
// DIF FFT across the lanes with shuffles.  Lane l, register r ends with bin
// k1 + E k2, k1 = bitrev_E(r), k2 = bitrev_32(l).  Two real windows share one
// complex transform (z = x_a + i x_b; X_a[f] = (Z[f] + conj Z[N-f]) / 2,
// X_b[f] = (Z[f] - conj Z[N-f]) / 2i), which halves the FFT work.  A CTA owns
// one point (all its Welch blocks); the pair spectra are staged in shared
// memory in the register layout (one contiguous row per register across the
// warp) and written per frequency as contiguous runs of nBlks values.
// ---------------------------------------------------------------------------
template <int E>
__device__ __forceinline__ void warp_fft(float (&re)[E], float (&im)[E], int lane, int N,
                                         const float* __restrict__ tc,
                                         const float* __restrict__ ts) {
  // E-point DIF over the registers (twiddle w_{2h}^j = w_N^{j N / 2h})
#pragma unroll
  for (int h = E / 2; h >= 1; h >>= 1) {
#pragma unroll
    for (int blk = 0; blk < E; blk += 2 * h) {
#pragma unroll
      for (int j = 0; j < h; ++j) {
        const float ur = re[blk + j], ui = im[blk + j];
        const float vr = re[blk + j + h], vi = im[blk + j + h];
        re[blk + j] = ur + vr;
        im[blk + j] = ui + vi;
        const float dr = ur - vr, di = ui - vi;
        const int ti = j * (N / (2 * h));
        const float wr = tc[ti], wi = ts[ti];
        re[blk + j + h] = dr * wr - di * wi;
        im[blk + j + h] = dr * wi + di * wr;
      }
    }
  }
  // twiddles w_N^(l k1), k1 = bitrev_E(r)
#pragma unroll
  for (int r = 1; r < E; ++r) {
    const int k1 = (int)(__brev((unsigned)r) >> (32 - __ffs(E) + 1));
    const int ti = (lane * k1) & (N - 1);
    const float wr = tc[ti], wi = ts[ti];
    const float xr = re[r], xi = im[r];
    re[r] = xr * wr - xi * wi;
    im[r] = xr * wi + xi * wr;
  }
  // 32-point DIF across the lanes
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const bool upper = (lane & d) != 0;
    const int ti = (lane & (d - 1)) * (N / (2 * d));
    const float wr = tc[ti], wi = ts[ti];
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const float pr = __shfl_xor_sync(0xffffffffu, re[r], d);
      const float pi = __shfl_xor_sync(0xffffffffu, im[r], d);
      if (!upper) {
        re[r] += pr;
        im[r] += pi;
      } else {
        const float dr = pr - re[r], di = pi - im[r];
        re[r] = dr * wr - di * wi;
        im[r] = dr * wi + di * wr;
      }
    }
  }
}

template <int E>
__global__ void __launch_bounds__(256) spod_fft32_kernel(
    const float* __restrict__ Y, int64_t M, int64_t ldy, const float* __restrict__ mean, int step,
    int nBlks, int nf, const float* __restrict__ window, const float* __restrict__ twr,
    const float* __restrict__ twi, float scale, float* __restrict__ Q) {
  constexpr int N = 32 * E;
  extern __shared__ unsigned char smem_raw[];
  float* sw = reinterpret_cast<float*>(smem_raw);  // window [N]
  float* sc = sw + N;                              // cos    [N]
  float* ss = sc + N;                              // -sin   [N]
  // spectra of window pairs: [pair][N + 1] complex, bin f of a pair at slot
  // r(f) 32 + lane(f) (the register layout of warp_fft)
  float2* zs = reinterpret_cast<float2*>(ss + N);
  constexpr int ZP = N + 1;  // odd pitch: consecutive pairs start 2 banks apart
  const int npairs = (nBlks + 1) / 2;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int j = tid; j < N; j += blockDim.x) {
    sw[j] = window[j];
    sc[j] = twr[j];
    ss[j] = twi[j];
  }
  __syncthreads();
  constexpr int LOGE = (E == 1) ? 0 : (E == 2) ? 1 : (E == 4) ? 2 : (E == 8) ? 3 : (E == 16) ? 4 : 5;
  auto slot = [&](int f) -> int {  // f in [0, N)
    const int k1 = f % E, k2 = f / E;
    const int r = LOGE ? (int)(__brev((unsigned)k1) >> (32 - LOGE)) : 0;
    return r * 32 + (int)(__brev((unsigned)k2) >> 27);
  };
  for (int64_t row = blockIdx.x; row < M; row += gridDim.x) {
    const float* x = Y + row * ldy;
    const float mu = mean ? mean[row] : 0.f;  // temporal mean removed on load
    // two real windows per complex FFT: z = x_a + i x_b
    for (int p = warp; p < npairs; p += 8) {
      const float* xa = x + (int64_t)(2 * p) * step;
      const bool has_b = 2 * p + 1 < nBlks;
      const float* xb = xa + step;
      float re[E], im[E];
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int j = lane + 32 * e;
        re[e] = (__ldg(xa + j) - mu) * sw[j];
        im[e] = has_b ? (__ldg(xb + j) - mu) * sw[j] : 0.f;
      }
      warp_fft<E>(re, im, lane, N, sc, ss);
      float2* z = zs + (size_t)p * ZP;
#pragma unroll
      for (int r = 0; r < E; ++r) z[r * 32 + lane] = make_float2(re[r], im[r]);
    }
    __syncthreads();
    // Q[f][row][b]: one contiguous run of nBlks values per frequency, a warp
    // per frequency (its two spectrum slots and scale computed once), lanes
    // along the blocks.
    // X_a[f] = (Z[f] + conj Z[N-f]) / 2,  X_b[f] = (Z[f] - conj Z[N-f]) / (2i)
    c2<float>* Qc = reinterpret_cast<c2<float>*>(Q);
    for (int f = warp; f < nf; f += 8) {
      const int sk = slot(f), sn = slot((N - f) & (N - 1));
      const float g = 0.5f * ((f >= 1 && f <= nf - 2) ? 2.f * scale : scale);
      c2<float>* qrow = Qc + ((int64_t)f * M + row) * nBlks;
      for (int b = lane; b < nBlks; b += 32) {
        const float2* z = zs + (size_t)(b >> 1) * ZP;
        const float2 zk = z[sk], zn = z[sn];
        c2<float> v;
        if ((b & 1) == 0) {
          v.re = (zk.x + zn.x) * g;
          v.im = (zk.y - zn.y) * g;
        } else {
          v.re = (zk.y + zn.y) * g;
          v.im = (zn.x - zk.x) * g;
        }
        qrow[b] = v;
      }
    }
    __syncthreads();
  }
}

template <int E>
static int spod_fft32_launch(const float* Y, int64_t M, int64_t ldy, const float* mean, int step,
                             int nBlks, int nf,
                             const float* window, const float* twr, const float* twi, double scale,
                             float* Q, cudaStream_t st) {
  const size_t smem =
      sizeof(float) * 3 * 32 * E + sizeof(float2) * (size_t)((nBlks + 1) / 2) * (32 * E + 1);
  PLOM_CHECK_CUDA(cudaFuncSetAttribute(spod_fft32_kernel<E>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  PLOM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spod_fft32_kernel<E>,
                                                                256, smem));
  const int64_t grid = std::min<int64_t>(M, (int64_t)std::max(1, per_sm) * num_sms() * 8);
  spod_fft32_kernel<E><<<(unsigned)grid, 256, smem, st>>>(Y, M, ldy, mean, step, nBlks, nf, window,
                                                          twr,
                                                          twi, (float)scale, Q);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

template <typename T>
static int spod_fft_impl(const T* Y, int64_t M, int64_t N, int64_t ldy, const T* mean, int nDFT,
                         int step,
                         int nBlks, int nf, const T* window, const T* twr, const T* twi,
                         double scale, T* Q, cudaStream_t st) {
  int log2n = -1;
  if ((nDFT & (nDFT - 1)) == 0) {
    log2n = 0;
    while ((1 << log2n) < nDFT) ++log2n;
  }
  if constexpr (sizeof(T) == 4) {
    const size_t stage =
        sizeof(float2) * (size_t)((nBlks + 1) / 2) * (nDFT + 1) + sizeof(float) * 3 * nDFT;
    // the register FFT stages the one-sided spectrum (nf = nDFT / 2 + 1)
    if (log2n >= 5 && log2n <= 10 && nf == nDFT / 2 + 1 && stage <= 200 * 1024) {
      ProfScope prof("spod_fft", st, 5.0 * (double)M * nBlks * nDFT * log2n,
                     (double)sizeof(T) * ((double)M * N + 2.0 * M * nBlks * nf));
      switch (log2n) {
        case 5: return spod_fft32_launch<1>(Y, M, ldy, mean, step, nBlks, nf, window, twr, twi, scale, Q, st);
        case 6: return spod_fft32_launch<2>(Y, M, ldy, mean, step, nBlks, nf, window, twr, twi, scale, Q, st);
        case 7: return spod_fft32_launch<4>(Y, M, ldy, mean, step, nBlks, nf, window, twr, twi, scale, Q, st);
        case 8: return spod_fft32_launch<8>(Y, M, ldy, mean, step, nBlks, nf, window, twr, twi, scale, Q, st);
        case 9: return spod_fft32_launch<16>(Y, M, ldy, mean, step, nBlks, nf, window, twr, twi, scale, Q, st);
        default: return spod_fft32_launch<32>(Y, M, ldy, mean, step, nBlks, nf, window, twr, twi, scale, Q, st);
      }
    }
  }
  const size_t fixed = sizeof(T) * 3 * (size_t)nDFT + sizeof(c2<T>) * 8 * (size_t)nDFT;
  const size_t per_row = sizeof(c2<T>) * (size_t)nBlks * nf;
  const size_t cap = 200 * 1024;
  PLOM_REQUIRE(fixed + per_row <= cap, PLOM_ERR_UNSUPPORTED,
               "spod_fft: nDFT=%d with %d blocks does not fit one CTA", nDFT, nBlks);
  int R = (int)std::min<size_t>(8, (cap - fixed) / per_row);
  R = std::max(1, R);
  const size_t smem = fixed + per_row * R;
  PLOM_CHECK_CUDA(cudaFuncSetAttribute(spod_fft_kernel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = cdiv(M, R);
  PLOM_REQUIRE(grid < (1ll << 31), PLOM_ERR_ARG, "spod_fft: too many rows");
  ProfScope prof("spod_fft", st, 5.0 * (double)M * nBlks * nDFT * (log2n > 0 ? log2n : nDFT),
                 (double)sizeof(T) * ((double)M * N + 2.0 * M * nBlks * nf));
  spod_fft_kernel<T><<<(unsigned)grid, 256, smem, st>>>(Y, M, N, ldy, mean, nDFT, log2n, step, nBlks,
                                                        nf, window, twr, twi, (T)scale, R, Q);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// P[(b M + i) nf + f0 + g] = Re U_g[i][b] for the G frequencies f0 .. f0+G-1
// of one batched SVD (U_g: M x nBlks complex, interleaved, ustride complex
// elements apart): pyLOM's column layout of the modes, real(U) flattened in
// Fortran order into column ifreq of P (SPOD/wrapper.py:84).  A block stages
// one point's G x nBlks real parts and writes them back frequency-fastest, so
// both the reads (along b) and the writes (along f) are contiguous.
template <typename T>
__global__ void __launch_bounds__(256) spod_modes_kernel(const T* __restrict__ U, int64_t M,
                                                         int nBlks, int G, int64_t ustride,
                                                         T* __restrict__ P, int64_t nf, int64_t f0,
                                                         int pitch) {
  extern __shared__ __align__(16) unsigned char modes_sm[];
  T* tile = reinterpret_cast<T*>(modes_sm);  // [G][pitch]
  const int tot = G * nBlks;
  for (int64_t i = blockIdx.x; i < M; i += gridDim.x) {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int g = e / nBlks, b = e - g * nBlks;
      tile[g * pitch + b] = U[2 * ((int64_t)g * ustride + i * nBlks + b)];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int b = e / G, g = e - b * G;
      P[((int64_t)b * M + i) * nf + f0 + g] = tile[g * pitch + b];
    }
    __syncthreads();
  }
}

template <typename T>
static int spod_modes_impl(const T* U, int64_t G, int64_t M, int64_t nBlks, int64_t ustride, T* P,
                           int64_t nf, int64_t f0, cudaStream_t st) {
  const int pitch = (int)(nBlks | 1);  // odd pitch: the frequency-fastest reads spread over banks
  const size_t smem = sizeof(T) * (size_t)G * pitch;
  PLOM_REQUIRE(smem <= 200 * 1024, PLOM_ERR_UNSUPPORTED,
               "spod_modes: %lld frequencies x %lld blocks do not fit in shared memory",
               (long long)G, (long long)nBlks);
  if (smem > 48 * 1024)
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(spod_modes_kernel<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = std::min<int64_t>(M, (int64_t)num_sms() * 8);
  ProfScope prof("spod_modes", st, 0.0, (double)sizeof(T) * 3.0 * G * M * nBlks);
  spod_modes_kernel<T><<<(unsigned)grid, 256, smem, st>>>(U, M, (int)nBlks, (int)G, ustride, P, nf,
                                                          f0, pitch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// P[row][c] = T_k[row][g] for frequency f = order[c] = k G + g: the groups'
// modes, written group-major and dense (T_k: rows x G_k, G_k = min(G, nf - k
// G), T_k at T + k gstride), gathered into P's final column order.  A block
// stages RB whole rows: it reads each group's RB x G_k block (contiguous) and
// writes RB x nf contiguous values.
// Both phases move 16-byte vectors (the group blocks and the P rows of a
// block of RB rows are contiguous and 16-byte aligned when RB G_k and RB nf
// are multiples of 16 bytes / sizeof(T); the tail block falls back to
// scalars), several per thread in flight.
template <typename T>
__global__ void __launch_bounds__(256) spod_assemble_kernel(const T* __restrict__ Tg, int64_t rows,
                                                            int nf, int G, int64_t gstride,
                                                            const int* __restrict__ order,
                                                            T* __restrict__ P, int RB) {
  constexpr int V = 16 / sizeof(T);  // elements per 16-byte vector
  using Vec = uint4;
  extern __shared__ __align__(16) unsigned char asm_sm[];
  int* ord = reinterpret_cast<int*>(asm_sm);
  T* tile = reinterpret_cast<T*>(asm_sm + sizeof(int) * (((size_t)nf + 3) & ~(size_t)3));
  const int pitch = nf | 1;  // [RB][pitch], frequency order
  for (int c = threadIdx.x; c < nf; c += blockDim.x) ord[c] = order[c];
  const int ngroups = (nf + G - 1) / G;
  for (int64_t r0 = (int64_t)blockIdx.x * RB; r0 < rows; r0 += (int64_t)gridDim.x * RB) {
    const int nr = (int)min((int64_t)RB, rows - r0);
    __syncthreads();
    for (int k = 0; k < ngroups; ++k) {
      const int Gk = min(G, nf - k * G);
      const T* src = Tg + (int64_t)k * gstride + r0 * Gk;
      const int cnt = nr * Gk;
      const bool vec = (cnt % V) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0;
      if (vec) {
#pragma unroll 4
        for (int e4 = threadIdx.x; e4 < cnt / V; e4 += blockDim.x) {
          const Vec w = __ldg(reinterpret_cast<const Vec*>(src) + e4);
          const T* wv = reinterpret_cast<const T*>(&w);
          int r = (e4 * V) / Gk, g = e4 * V - r * Gk;  // one division a vector
#pragma unroll
          for (int q = 0; q < V; ++q) {
            tile[r * pitch + k * G + g] = wv[q];
            if (++g == Gk) {
              g = 0;
              ++r;
            }
          }
        }
      } else {
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
          const int r = e / Gk, g = e - r * Gk;
          tile[r * pitch + k * G + g] = src[e];
        }
      }
    }
    __syncthreads();
    T* dst = P + r0 * nf;
    const int cnt = nr * nf;
    if ((cnt % V) == 0 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
#pragma unroll 4
      for (int e4 = threadIdx.x; e4 < cnt / V; e4 += blockDim.x) {
        Vec w;
        T* wv = reinterpret_cast<T*>(&w);
        int r = (e4 * V) / nf, c = e4 * V - r * nf;  // one division a vector
#pragma unroll
        for (int q = 0; q < V; ++q) {
          wv[q] = tile[r * pitch + ord[c]];
          if (++c == nf) {
            c = 0;
            ++r;
          }
        }
        reinterpret_cast<Vec*>(dst)[e4] = w;
      }
    } else {
      for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int r = e / nf, c = e - r * nf;
        dst[e] = tile[r * pitch + ord[c]];
      }
    }
  }
}

template <typename T>
static int spod_assemble_impl(const T* Tg, int64_t rows, int nf, int G, int64_t gstride,
                              const int* order, T* P, cudaStream_t st) {
  const int RB = 64;
  const size_t smem = sizeof(int) * (((size_t)nf + 3) & ~(size_t)3) + sizeof(T) * RB * (nf | 1);
  PLOM_REQUIRE(smem <= 200 * 1024, PLOM_ERR_UNSUPPORTED, "spod_assemble: %d frequencies too many",
               nf);
  if (smem > 48 * 1024)
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(spod_assemble_kernel<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = std::min<int64_t>((rows + RB - 1) / RB, (int64_t)num_sms() * 8);
  ProfScope prof("spod_assemble", st, 0.0, 2.0 * sizeof(T) * rows * nf);
  spod_assemble_kernel<T><<<(unsigned)grid, 256, smem, st>>>(Tg, rows, nf, G, gstride, order, P,
                                                             RB);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

}  // namespace plom

using namespace plom;

extern "C" int plom_spod_assemble(int dtype, const void* Tg, int64_t rows, int64_t nf, int64_t G,
                                  int64_t gstride, const int* order, void* P, void* stream) {
  PLOM_REQUIRE(Tg && order && P, PLOM_ERR_ARG, "spod_assemble: null pointer");
  PLOM_REQUIRE(rows >= 1 && nf >= 1 && nf <= 8192 && G >= 1 && G <= nf && gstride >= G * rows,
               PLOM_ERR_ARG, "spod_assemble: bad sizes");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == PLOM_F32)
    return spod_assemble_impl<float>((const float*)Tg, rows, (int)nf, (int)G, gstride, order,
                                     (float*)P, st);
  if (dtype == PLOM_F64)
    return spod_assemble_impl<double>((const double*)Tg, rows, (int)nf, (int)G, gstride, order,
                                      (double*)P, st);
  set_error("spod_assemble: dtype must be F32 or F64");
  return PLOM_ERR_UNSUPPORTED;
}

extern "C" int plom_spod_fft(int dtype, const void* Y, int64_t M, int64_t N, int64_t ldy,
                             const void* mean, int64_t nDFT, int64_t step, int64_t nBlks, int64_t nf,
                             const void* window, const void* twr, const void* twi, double scale,
                             void* Q, void* stream) {
  PLOM_REQUIRE(Y && window && twr && twi && Q, PLOM_ERR_ARG, "spod_fft: null pointer");
  PLOM_REQUIRE(M >= 1 && nDFT >= 2 && nDFT <= 8192 && step >= 1 && nBlks >= 1 && nf >= 1 &&
                   nf <= nDFT && ldy >= N,
               PLOM_ERR_ARG, "spod_fft: bad sizes");
  PLOM_REQUIRE((nBlks - 1) * step + nDFT <= N, PLOM_ERR_ARG,
               "spod_fft: blocks run past the last snapshot");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == PLOM_F32)
    return spod_fft_impl<float>((const float*)Y, M, N, ldy, (const float*)mean, (int)nDFT,
                                (int)step, (int)nBlks,
                                (int)nf, (const float*)window, (const float*)twr,
                                (const float*)twi, scale, (float*)Q, st);
  if (dtype == PLOM_F64)
    return spod_fft_impl<double>((const double*)Y, M, N, ldy, (const double*)mean, (int)nDFT,
                                 (int)step, (int)nBlks,
                                 (int)nf, (const double*)window, (const double*)twr,
                                 (const double*)twi, scale, (double*)Q, st);
  set_error("spod_fft: dtype must be F32 or F64");
  return PLOM_ERR_UNSUPPORTED;
}

extern "C" int plom_spod_modes(int dtype, const void* U, int64_t G, int64_t M, int64_t nBlks,
                               int64_t ustride, void* P, int64_t nf, int64_t f0, void* stream) {
  PLOM_REQUIRE(U && P, PLOM_ERR_ARG, "spod_modes: null pointer");
  PLOM_REQUIRE(G >= 1 && M >= 1 && nBlks >= 1 && ustride >= M * nBlks && f0 >= 0 && f0 + G <= nf,
               PLOM_ERR_ARG, "spod_modes: bad sizes");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == PLOM_F32)
    return spod_modes_impl<float>((const float*)U, G, M, nBlks, ustride, (float*)P, nf, f0, st);
  if (dtype == PLOM_F64)
    return spod_modes_impl<double>((const double*)U, G, M, nBlks, ustride, (double*)P, nf, f0, st);
  set_error("spod_modes: dtype must be F32 or F64 (the real type of U)");
  return PLOM_ERR_UNSUPPORTED;
}
