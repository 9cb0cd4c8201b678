// Streaming row kernels: temporal mean, variance, mean subtraction and
// variance normalisation of the snapshot matrix X (m points x n snapshots,
// row-major, each row a time series).
//
// GB300 mapping: one warp per row, 16-byte vector loads/stores when the row
// start and length allow it.  f64 data accumulate in FP64; f32 data in FP32
// with compensated (Kahan) per-lane sums folded into FP64 across the warp (no
// per-element FP64 instruction: GB300's FP64 rate is 1/64 of FP32), and the
// mean is subtracted in FP32 as the reference's float32 path does.
// All modes are HBM-bound: algorithmic bytes = read m*n*s (+ write m*n*s when
// Y is produced).  A row is re-read from L1/L2 for the second and third
// sweeps (variance, write-out), never from HBM for rows up to ~64 KB.
//
// Reference behaviour (pyLowOrder): pyLOM/vmmath/src/averaging.c:10-157,
// pyLOM/vmmath/averaging.py:18-75.  Variance is the population variance
// (np.var, divide by n) and norm_variance divides by the variance itself.
#include "plom_common.cuh"

namespace plom {

enum : int { Y_NONE = 0, Y_SUB = 1, Y_NORM = 2 };

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int N = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int N = 2;
};

template <typename T>
__device__ __forceinline__ void vload(const T* p, double* out);
template <>
__device__ __forceinline__ void vload<float>(const float* p, double* out) {
  float4 v = __ldg(reinterpret_cast<const float4*>(p));
  out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
}
template <>
__device__ __forceinline__ void vload<double>(const double* p, double* out) {
  double2 v = __ldg(reinterpret_cast<const double2*>(p));
  out[0] = v.x; out[1] = v.y;
}
template <typename T>
__device__ __forceinline__ void vstore(T* p, const double* v);
template <>
__device__ __forceinline__ void vstore<float>(float* p, const double* v) {
  *reinterpret_cast<float4*>(p) = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
}
template <>
__device__ __forceinline__ void vstore<double>(double* p, const double* v) {
  *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// f32 rows: FP32 compensated sums (see the file comment)
template <bool VEC>
__global__ void __launch_bounds__(256) row_kernel_f32(const float* __restrict__ X, int64_t m,
                                                      int64_t n, int64_t ldx,
                                                      const float* __restrict__ mean_in,
                                                      const float* __restrict__ var_in,
                                                      float* __restrict__ mean_out,
                                                      float* __restrict__ var_out, int want_var,
                                                      int ymode, float* __restrict__ Y,
                                                      int64_t ldy) {
  const int lane = threadIdx.x & 31;
  const int64_t warps_total = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m;
       row += warps_total) {
    const float* x = X + row * ldx;
    float muf;
    if (mean_in) {
      muf = mean_in[row];
    } else {
      float s = 0.f, c = 0.f;
      if (VEC) {
        const int64_t nv = n / 4;
        int64_t j = lane;
        for (; j + 96 < nv; j += 128) {  // 4 vectors in flight per lane
          const float4 a = __ldg(reinterpret_cast<const float4*>(x + j * 4));
          const float4 b = __ldg(reinterpret_cast<const float4*>(x + (j + 32) * 4));
          const float4 d = __ldg(reinterpret_cast<const float4*>(x + (j + 64) * 4));
          const float4 e = __ldg(reinterpret_cast<const float4*>(x + (j + 96) * 4));
          kahan_add(s, c, (a.x + a.y) + (a.z + a.w));
          kahan_add(s, c, (b.x + b.y) + (b.z + b.w));
          kahan_add(s, c, (d.x + d.y) + (d.z + d.w));
          kahan_add(s, c, (e.x + e.y) + (e.z + e.w));
        }
        for (; j < nv; j += 32) {
          const float4 a = __ldg(reinterpret_cast<const float4*>(x + j * 4));
          kahan_add(s, c, (a.x + a.y) + (a.z + a.w));
        }
      } else {
        for (int64_t j = lane; j < n; j += 32) kahan_add(s, c, x[j]);
      }
      const double tot = warp_sum((double)s - (double)c);
      const double mu = tot / (double)n;
      muf = (float)mu;
      if (lane == 0 && mean_out) mean_out[row] = muf;
    }
    float var = 1.f;
    if (want_var) {
      float s2 = 0.f, c2 = 0.f;
      if (VEC) {
        const int64_t nv = n / 4;
        for (int64_t j = lane; j < nv; j += 32) {
          const float4 a = __ldg(reinterpret_cast<const float4*>(x + j * 4));
          const float d0 = a.x - muf, d1 = a.y - muf, d2 = a.z - muf, d3 = a.w - muf;
          kahan_add(s2, c2, fmaf(d0, d0, d1 * d1) + fmaf(d2, d2, d3 * d3));
        }
      } else {
        for (int64_t j = lane; j < n; j += 32) {
          const float d = x[j] - muf;
          kahan_add(s2, c2, d * d);
        }
      }
      const double tot = warp_sum((double)s2 - (double)c2);
      var = (float)(tot / (double)n);
      if (lane == 0 && var_out) var_out[row] = var;
    } else if (var_in) {
      var = var_in[row];
    }
    if (ymode != Y_NONE) {
      const float inv = (ymode == Y_NORM) ? 1.f / var : 1.f;
      float* y = Y + row * ldy;
      if (VEC) {
        const int64_t nv = n / 4;
        for (int64_t j = lane; j < nv; j += 32) {
          float4 a = __ldg(reinterpret_cast<const float4*>(x + j * 4));
          a.x -= muf;
          a.y -= muf;
          a.z -= muf;
          a.w -= muf;
          if (ymode == Y_NORM) {
            a.x *= inv;
            a.y *= inv;
            a.z *= inv;
            a.w *= inv;
          }
          *reinterpret_cast<float4*>(y + j * 4) = a;
        }
      } else {
        for (int64_t j = lane; j < n; j += 32) {
          const float d = x[j] - muf;
          y[j] = (ymode == Y_NORM) ? d * inv : d;
        }
      }
    }
  }
}

// One warp per row.  VEC: use 16-byte vectors (caller checked alignment).
template <typename T, bool VEC>
__global__ void __launch_bounds__(256) row_kernel(const T* __restrict__ X, int64_t m, int64_t n,
                                                  int64_t ldx, const T* __restrict__ mean_in,
                                                  const T* __restrict__ var_in,
                                                  T* __restrict__ mean_out,
                                                  T* __restrict__ var_out, int want_var,
                                                  int ymode, T* __restrict__ Y, int64_t ldy) {
  const int lane = threadIdx.x & 31;
  const int64_t warps_total = (int64_t)gridDim.x * (blockDim.x >> 5);
  constexpr int V = Vec16<T>::N;
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < m;
       row += warps_total) {
    const T* x = X + row * ldx;
    double mu;
    if (mean_in) {
      mu = (double)mean_in[row];
    } else {
      double s = 0.0;
      if (VEC) {
        const int64_t nv = n / V;
        int64_t j = lane;
        for (; j + 96 < nv; j += 128) {  // 4 vectors in flight per lane
          double a[V], b[V], c[V], d[V];
          vload<T>(x + j * V, a);
          vload<T>(x + (j + 32) * V, b);
          vload<T>(x + (j + 64) * V, c);
          vload<T>(x + (j + 96) * V, d);
#pragma unroll
          for (int k = 0; k < V; ++k) s += (a[k] + b[k]) + (c[k] + d[k]);
        }
        for (; j < nv; j += 32) {
          double a[V];
          vload<T>(x + j * V, a);
#pragma unroll
          for (int k = 0; k < V; ++k) s += a[k];
        }
      } else {
        for (int64_t j = lane; j < n; j += 32) s += (double)x[j];
      }
      s = warp_sum(s);
      mu = s / (double)n;
      if (lane == 0 && mean_out) mean_out[row] = (T)mu;
    }
    double var = 1.0;
    if (want_var) {
      double s2 = 0.0;
      if (VEC) {
        const int64_t nv = n / V;
        for (int64_t j = lane; j < nv; j += 32) {
          double a[V];
          vload<T>(x + j * V, a);
#pragma unroll
          for (int k = 0; k < V; ++k) {
            double d = a[k] - mu;
            s2 += d * d;
          }
        }
      } else {
        for (int64_t j = lane; j < n; j += 32) {
          double d = (double)x[j] - mu;
          s2 += d * d;
        }
      }
      s2 = warp_sum(s2);
      var = s2 / (double)n;
      if (lane == 0 && var_out) var_out[row] = (T)var;
    } else if (var_in) {
      var = (double)var_in[row];
    }
    if (ymode != Y_NONE) {
      const double inv = (ymode == Y_NORM) ? 1.0 / var : 1.0;
      T* y = Y + row * ldy;
      if (VEC) {
        const int64_t nv = n / V;
        for (int64_t j = lane; j < nv; j += 32) {
          double a[V];
          vload<T>(x + j * V, a);
#pragma unroll
          for (int k = 0; k < V; ++k) a[k] = (ymode == Y_NORM) ? (a[k] - mu) * inv : a[k] - mu;
          vstore<T>(y + j * V, a);
        }
      } else {
        for (int64_t j = lane; j < n; j += 32) {
          double d = (double)x[j] - mu;
          y[j] = (T)((ymode == Y_NORM) ? d * inv : d);
        }
      }
    }
  }
}

template <typename T>
static int launch_rows(const T* X, int64_t m, int64_t n, int64_t ldx, const T* mean_in,
                       const T* var_in, T* mean_out, T* var_out, int want_var, int ymode, T* Y,
                       int64_t ldy, cudaStream_t st) {
  PLOM_REQUIRE(m >= 0 && n >= 1 && ldx >= n, PLOM_ERR_ARG, "bad sizes m=%lld n=%lld ldx=%lld",
               (long long)m, (long long)n, (long long)ldx);
  PLOM_REQUIRE(ymode == Y_NONE || ldy >= n, PLOM_ERR_ARG, "ldy < n");
  if (m == 0) return PLOM_OK;
  constexpr int V = Vec16<T>::N;
  const bool vec = (n % V == 0) && (ldx % V == 0) &&
                   (reinterpret_cast<uintptr_t>(X) % 16 == 0) &&
                   (ymode == Y_NONE || ((ldy % V == 0) && reinterpret_cast<uintptr_t>(Y) % 16 == 0));
  const int threads = 256;
  const int64_t warps = m;
  int64_t blocks = cdiv(warps, threads / 32);
  const int64_t cap = (int64_t)num_sms() * 8 * 4;  // persistent-ish grid: 8 blocks/SM x 4 waves
  if (blocks > cap) blocks = cap;
  ProfScope prof("rows_mean_subtract", st, 0.0,
                 (double)m * n * sizeof(T) * (ymode == Y_NONE ? 1.0 : 2.0));
  if constexpr (sizeof(T) == 4) {
    if (vec)
      row_kernel_f32<true><<<(unsigned)blocks, threads, 0, st>>>(X, m, n, ldx, mean_in, var_in,
                                                                 mean_out, var_out, want_var,
                                                                 ymode, Y, ldy);
    else
      row_kernel_f32<false><<<(unsigned)blocks, threads, 0, st>>>(X, m, n, ldx, mean_in, var_in,
                                                                  mean_out, var_out, want_var,
                                                                  ymode, Y, ldy);
  } else {
    if (vec)
      row_kernel<T, true><<<(unsigned)blocks, threads, 0, st>>>(X, m, n, ldx, mean_in, var_in,
                                                                mean_out, var_out, want_var,
                                                                ymode, Y, ldy);
    else
      row_kernel<T, false><<<(unsigned)blocks, threads, 0, st>>>(X, m, n, ldx, mean_in, var_in,
                                                                 mean_out, var_out, want_var,
                                                                 ymode, Y, ldy);
  }
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

int rows_dispatch(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx, const void* mean_in,
                  const void* var_in, void* mean_out, void* var_out, int want_var, int ymode,
                  void* Y, int64_t ldy, cudaStream_t st) {
  if (dtype == PLOM_F32)
    return launch_rows<float>((const float*)X, m, n, ldx, (const float*)mean_in,
                              (const float*)var_in, (float*)mean_out, (float*)var_out, want_var,
                              ymode, (float*)Y, ldy, st);
  if (dtype == PLOM_F64)
    return launch_rows<double>((const double*)X, m, n, ldx, (const double*)mean_in,
                               (const double*)var_in, (double*)mean_out, (double*)var_out,
                               want_var, ymode, (double*)Y, ldy, st);
  set_error("averaging: dtype %d not supported (F32/F64 only)", dtype);
  return PLOM_ERR_UNSUPPORTED;
}

}  // namespace plom

using namespace plom;

extern "C" int plom_temporal_mean(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                                  void* mean, void* stream) {
  PLOM_REQUIRE(X && mean, PLOM_ERR_ARG, "null pointer");
  return rows_dispatch(dtype, X, m, n, ldx, nullptr, nullptr, mean, nullptr, 0, Y_NONE, nullptr, n,
                       (cudaStream_t)stream);
}

extern "C" int plom_subtract_mean(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                                  const void* mean, void* Y, int64_t ldy, void* stream) {
  PLOM_REQUIRE(X && mean && Y, PLOM_ERR_ARG, "null pointer");
  return rows_dispatch(dtype, X, m, n, ldx, mean, nullptr, nullptr, nullptr, 0, Y_SUB, Y, ldy,
                       (cudaStream_t)stream);
}

extern "C" int plom_temporal_variance(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                                      const void* mean, void* var, void* stream) {
  PLOM_REQUIRE(X && mean && var, PLOM_ERR_ARG, "null pointer");
  return rows_dispatch(dtype, X, m, n, ldx, mean, nullptr, nullptr, var, 1, Y_NONE, nullptr, n,
                       (cudaStream_t)stream);
}

extern "C" int plom_norm_variance(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                                  const void* mean, const void* var, void* Y, int64_t ldy,
                                  void* stream) {
  PLOM_REQUIRE(X && mean && var && Y, PLOM_ERR_ARG, "null pointer");
  return rows_dispatch(dtype, X, m, n, ldx, mean, var, nullptr, nullptr, 0, Y_NORM, Y, ldy,
                       (cudaStream_t)stream);
}

extern "C" int plom_remove_mean(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                                void* mean, void* var, int divide_variance, void* Y, int64_t ldy,
                                void* stream) {
  PLOM_REQUIRE(X && mean && Y, PLOM_ERR_ARG, "null pointer");
  PLOM_REQUIRE(!divide_variance || var, PLOM_ERR_ARG, "divide_variance needs a var buffer");
  return rows_dispatch(dtype, X, m, n, ldx, nullptr, nullptr, mean, var, divide_variance ? 1 : 0,
                       divide_variance ? Y_NORM : Y_SUB, Y, ldy, (cudaStream_t)stream);
}
