// vec.cu -- the Davidson / RQ-CG vector layer on the device.
//
// The reference runs these steps as BLAS calls on host arrays
// (davidson.c:133-255, CG.c:74-127).  Here they are fused passes over HBM:
//  * residual pass: x = V y, r = VA y - theta x, ||r||, the preconditioned
//    t = r / |diag - theta| (davidson.c:195-227; for a shifted operator
//    H - s the preconditioner uses diag - s - theta) and the first Gram-Schmidt
//    projections V^T t, all in one read of V and VA;
//  * Gram-Schmidt: classical GS applied twice (projection pass, update +
//    second projection pass, final update + normalisation), replacing the
//    single modified-GS sweep of davidson.c:139-146;
//  * subspace column V^T (H v_m) (davidson.c:178-193) as a multi-dot;
//  * deflation V <- V Y[:, :keep] in place (davidson.c:229-255);
//  * RQ-CG: the 2x2 Gram blocks of CG.c:102-103 in one pass, and the x/Ax/g
//    updates of CG.c:106-126 in one pass.
// Storage is double (FP64 mode) or float (FP32 basis of the mixed mode).
// FP64 storage: FP64 arithmetic throughout.  FP32 storage: FP32 arithmetic
// on the shifted operator, FP32 partial sums over short runs added into FP64
// accumulators (the *_f32 kernels).  Reductions are two-stage
// (per-block partials, then one block summing them in a fixed order), so
// results do not depend on timing.
#include <cuda_runtime.h>

#include <atomic>
#include <type_traits>

#include "internal.h"
#include "vec.h"

namespace doci {
namespace {

constexpr int kT = 256;
constexpr int kMaxK = 34;  // outputs of one reduction pass

int grid_blocks() { return device_sm_count() * 4; }

// Partial-sum buffer layout: [0] a block counter, [1, 1 + kMaxK) the
// results, then one row of nk partials per block.  Every reduction pass ends
// with block_reduce_store: each block writes its row, and the last block to
// finish (the counter) sums the rows in a fixed order (one warp per output,
// lanes over strided blocks, then a fixed shuffle tree) into the results and
// resets the counter -- results do not depend on timing, and no separate
// reduction launch is needed.
constexpr int kHeader = 1 + kMaxK;

template <int K>
__device__ __forceinline__ void block_reduce_store(double (&acc)[K], int nk, double *partials) {
  __shared__ double red[32][kMaxK];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (k < nk) {
      double v = acc[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][k] = v;
    }
  }
  __syncthreads();
  double *rows = partials + kHeader;
  if (threadIdx.x < nk) {
    double s = 0;
    for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
    rows[static_cast<size_t>(blockIdx.x) * nk + threadIdx.x] = s;
  }
  __threadfence();
  __syncthreads();
  unsigned int *counter = reinterpret_cast<unsigned int *>(partials);
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int k = warp; k < nk; k += nw) {
    double s = 0;
    for (unsigned b = lane; b < gridDim.x; b += 32) s += __ldcg(rows + static_cast<size_t>(b) * nk + k);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) partials[1 + k] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// partials of V_i . w for i < m
template <typename S, int K>
__global__ void __launch_bounds__(kT)
multidot_kernel(const S *__restrict__ V, size_t ld, int m, const S *__restrict__ w, size_t n,
                double *__restrict__ partials) {
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0;
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    const double wj = static_cast<double>(w[j]);
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < m) acc[k] += static_cast<double>(V[k * ld + j]) * wj;
  }
  block_reduce_store<K>(acc, m, partials);
}

// Residual pass.  Outputs (per block): [0] ||r||^2, [1] ||t||^2, [2..2+m) V_i . t
template <typename S, int K>
__global__ void __launch_bounds__(kT)
residual_kernel(const S *__restrict__ V, const S *__restrict__ VA, size_t ld, int m,
                const double *__restrict__ y, double theta, double pre_theta, const double *__restrict__ diag,
                size_t n, S *__restrict__ t, double *__restrict__ x_out, double *__restrict__ partials) {
  __shared__ double ys[K];
  if (threadIdx.x < K) ys[threadIdx.x] = threadIdx.x < m ? y[threadIdx.x] : 0.0;
  __syncthreads();
  double acc[K + 2];
#pragma unroll
  for (int k = 0; k < K + 2; ++k) acc[k] = 0;
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    double v[K];
    double xv = 0, av = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (k < m) {
        v[k] = static_cast<double>(V[k * ld + j]);
        xv += v[k] * ys[k];
        av += static_cast<double>(VA[k * ld + j]) * ys[k];
      }
    }
    const double r = av - theta * xv;
    acc[0] += r * r;
    if (x_out) x_out[j] = xv;
    const double d = fabs(diag[j] - pre_theta);
    const S ts = static_cast<S>(d > 1e-12 ? r / d : r / 1e-12);  // davidson.c:214-227
    t[j] = ts;
    const double td = static_cast<double>(ts);
    acc[1] += td * td;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < m) acc[2 + k] += v[k] * td;
  }
  block_reduce_store<K + 2>(acc, m + 2, partials);
}

// t <- t - sum_i c_i V_i; partials: [0] ||t||^2, [1..1+m) V_i . t
template <typename S, int K>
__global__ void __launch_bounds__(kT)
gs_update_kernel(const S *__restrict__ V, size_t ld, int m, const double *__restrict__ c, size_t n,
                 S *__restrict__ t, double *__restrict__ partials) {
  __shared__ double cs[K];
  if (threadIdx.x < K) cs[threadIdx.x] = threadIdx.x < m ? c[threadIdx.x] : 0.0;
  __syncthreads();
  double acc[K + 1];
#pragma unroll
  for (int k = 0; k < K + 1; ++k) acc[k] = 0;
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    double v[K];
    double tv = static_cast<double>(t[j]);
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < m) {
        v[k] = static_cast<double>(V[k * ld + j]);
        tv -= v[k] * cs[k];
      }
    const S ts = static_cast<S>(tv);
    t[j] = ts;
    const double td = static_cast<double>(ts);
    acc[0] += td * td;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < m) acc[1 + k] += v[k] * td;
  }
  block_reduce_store<K + 1>(acc, m + 1, partials);
}

// out = (t - sum_i c_i V_i) * scale; partials: [0] ||out||^2
template <typename S, int K>
__global__ void __launch_bounds__(kT)
gs_finish_kernel(const S *__restrict__ V, size_t ld, int m, const double *__restrict__ c, double scale,
                 size_t n, const S *__restrict__ t, S *__restrict__ out, double *__restrict__ partials) {
  __shared__ double cs[K];
  if (threadIdx.x < K) cs[threadIdx.x] = threadIdx.x < m ? c[threadIdx.x] : 0.0;
  __syncthreads();
  double acc[1] = {0};
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    double tv = static_cast<double>(t[j]);
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < m) tv -= static_cast<double>(V[k * ld + j]) * cs[k];
    const S o = static_cast<S>(tv * scale);
    out[j] = o;
    acc[0] += static_cast<double>(o) * static_cast<double>(o);
  }
  block_reduce_store<1>(acc, 1, partials);
}

// V[:, c] <- sum_k V[:, k] Y[k, c] for c < keep, in place (each element's
// row is read completely before it is written).
template <typename S, int K>
__global__ void __launch_bounds__(kT)
deflate_kernel(S *__restrict__ V, size_t ld, int mv, int keep, const double *__restrict__ Y, int ldy, size_t n) {
  __shared__ double Ys[K * K];
  for (int i = threadIdx.x; i < mv * keep; i += blockDim.x) Ys[i] = Y[(i / mv) * ldy + (i % mv)];
  __syncthreads();
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < mv) v[k] = static_cast<double>(V[k * ld + j]);
    for (int c = 0; c < keep; ++c) {
      double s = 0;
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < mv) s += v[k] * Ys[c * mv + k];
      V[c * ld + j] = static_cast<S>(s);
    }
  }
}

// x = V y (FP64 output)
template <typename S, int K>
__global__ void __launch_bounds__(kT)
combine_kernel(const S *__restrict__ V, size_t ld, int m, const double *__restrict__ y, size_t n,
               double *__restrict__ x) {
  __shared__ double ys[K];
  if (threadIdx.x < K) ys[threadIdx.x] = threadIdx.x < m ? y[threadIdx.x] : 0.0;
  __syncthreads();
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    double s = 0;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < m) s += static_cast<double>(V[k * ld + j]) * ys[k];
    x[j] = s;
  }
}

// ---- FP32-storage passes (the FP32 phase of the mixed mode) ---------------
// Arithmetic in FP32 (GB300's FP64 rate is a small fraction of its FP32
// rate, and these passes would be FP64-throughput bound); the operator is
// shifted (H - lowest diagonal element), so the residual's cancellation is
// mild.  Reductions add FP32 partial sums over kChunk elements of a thread
// into FP64 accumulators, so sums over 10^8+ elements stay accurate.
constexpr int kChunk = 16;

// Per-thread FP64 accumulators kept in shared memory ([k][thread], so the
// registers hold only the FP32 chunk sums); flushed once per chunk.  Blocks
// of BT threads: 256 for up to 16 basis vectors, 128 for up to 32 (18 or 34
// accumulators: 37 / 35 KB of static shared memory).
template <int K>
__host__ __device__ constexpr int f32_block() { return K <= 16 ? 256 : 128; }
// resident blocks per SM the register budget is set for (three, so at most
// 85 registers for 256-thread blocks), launched as one full wave.  Measured on
// GB300 (residual pass, 16 vectors, L=32 size): 87 registers and two resident
// blocks per SM 58.5 ms, 80 registers and three 15.9 ms.
template <int K>
__host__ __device__ constexpr int f32_minb() { return 3; }

template <int NK, int BT>
struct SmemAcc {
  double *a;
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int k = 0; k < NK; ++k) a[k * BT + threadIdx.x] = 0;
  }
  __device__ __forceinline__ void add(const float (&f)[NK], int nk) {
#pragma unroll
    for (int k = 0; k < NK; ++k)
      if (k < nk) a[k * BT + threadIdx.x] += f[k];
  }
  __device__ __forceinline__ void store(int nk, double *partials) {
    double acc[NK];
#pragma unroll
    for (int k = 0; k < NK; ++k) acc[k] = k < nk ? a[k * BT + threadIdx.x] : 0.0;
    block_reduce_store<NK>(acc, nk, partials);
  }
};

template <int K>
__global__ void __launch_bounds__(f32_block<K>(), f32_minb<K>())
multidot_f32_kernel(const float *__restrict__ V, size_t ld, int m, const float *__restrict__ w, size_t n,
                    double *__restrict__ partials) {
  __shared__ double acc_s[K * f32_block<K>()];
  SmemAcc<K, f32_block<K>()> acc{acc_s};
  acc.zero();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t j0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j0 < n; j0 += stride * kChunk) {
    float f[K];
#pragma unroll
    for (int k = 0; k < K; ++k) f[k] = 0.f;
#pragma unroll 4
    for (int u = 0; u < kChunk; ++u) {
      const size_t j = j0 + u * stride;
      if (j >= n) break;
      const float wj = w[j];
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < m) f[k] = fmaf(V[k * ld + j], wj, f[k]);
    }
    acc.add(f, m);
  }
  acc.store(m, partials);
}

template <int K>
__global__ void __launch_bounds__(f32_block<K>(), f32_minb<K>())
residual_f32_kernel(const float *__restrict__ V, const float *__restrict__ VA, size_t ld, int m,
                    const double *__restrict__ y, double theta, double pre_theta, const double *__restrict__ diag,
                    size_t n, float *__restrict__ t, double *__restrict__ x_out, double *__restrict__ partials) {
  __shared__ float ys[K];
  __shared__ double acc_s[(K + 2) * f32_block<K>()];
  if (threadIdx.x < K) ys[threadIdx.x] = threadIdx.x < m ? static_cast<float>(y[threadIdx.x]) : 0.f;
  SmemAcc<K + 2, f32_block<K>()> acc{acc_s};
  acc.zero();
  __syncthreads();
  const float th = static_cast<float>(theta);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t j0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j0 < n; j0 += stride * kChunk) {
    float f[K + 2];
#pragma unroll
    for (int k = 0; k < K + 2; ++k) f[k] = 0.f;
    for (int u = 0; u < kChunk; ++u) {
      const size_t j = j0 + u * stride;
      if (j >= n) break;
      float v[K];
      float xv = 0.f, av = 0.f;
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < m) {
          v[k] = V[k * ld + j];
          xv = fmaf(v[k], ys[k], xv);
          av = fmaf(VA[k * ld + j], ys[k], av);
        }
      const float r = fmaf(-th, xv, av);
      f[0] = fmaf(r, r, f[0]);
      if (x_out) x_out[j] = xv;
      const float d = fabsf(static_cast<float>(diag[j] - pre_theta));
      const float ts = d > 1e-12f ? r / d : r / 1e-12f;  // davidson.c:214-227
      t[j] = ts;
      f[1] = fmaf(ts, ts, f[1]);
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < m) f[2 + k] = fmaf(v[k], ts, f[2 + k]);
    }
    acc.add(f, m + 2);
  }
  acc.store(m + 2, partials);
}

template <int K>
__global__ void __launch_bounds__(f32_block<K>(), f32_minb<K>())
gs_update_f32_kernel(const float *__restrict__ V, size_t ld, int m, const double *__restrict__ c, size_t n,
                     float *__restrict__ t, double *__restrict__ partials) {
  __shared__ float cs[K];
  __shared__ double acc_s[(K + 1) * f32_block<K>()];
  if (threadIdx.x < K) cs[threadIdx.x] = threadIdx.x < m ? static_cast<float>(c[threadIdx.x]) : 0.f;
  SmemAcc<K + 1, f32_block<K>()> acc{acc_s};
  acc.zero();
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t j0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j0 < n; j0 += stride * kChunk) {
    float f[K + 1];
#pragma unroll
    for (int k = 0; k < K + 1; ++k) f[k] = 0.f;
    for (int u = 0; u < kChunk; ++u) {
      const size_t j = j0 + u * stride;
      if (j >= n) break;
      float v[K];
      float tv = t[j];
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < m) {
          v[k] = V[k * ld + j];
          tv = fmaf(-cs[k], v[k], tv);
        }
      t[j] = tv;
      f[0] = fmaf(tv, tv, f[0]);
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < m) f[1 + k] = fmaf(v[k], tv, f[1 + k]);
    }
    acc.add(f, m + 1);
  }
  acc.store(m + 1, partials);
}

template <int K>
__global__ void __launch_bounds__(kT)
gs_finish_f32_kernel(const float *__restrict__ V, size_t ld, int m, const double *__restrict__ c, double scale,
                     size_t n, const float *__restrict__ t, float *__restrict__ out, double *__restrict__ partials) {
  __shared__ float cs[K];
  if (threadIdx.x < K) cs[threadIdx.x] = threadIdx.x < m ? static_cast<float>(c[threadIdx.x]) : 0.f;
  __syncthreads();
  const float sc = static_cast<float>(scale);
  double acc[1] = {0};
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t j0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j0 < n; j0 += stride * kChunk) {
    float f = 0.f;
#pragma unroll 4
    for (int u = 0; u < kChunk; ++u) {
      const size_t j = j0 + u * stride;
      if (j >= n) break;
      float tv = t[j];
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < m) tv = fmaf(-cs[k], V[k * ld + j], tv);
      const float o = tv * sc;
      out[j] = o;
      f = fmaf(o, o, f);
    }
    acc[0] += f;
  }
  block_reduce_store<1>(acc, 1, partials);
}

template <int K>
__global__ void __launch_bounds__(kT)
deflate_f32_kernel(float *__restrict__ V, size_t ld, int mv, int keep, const double *__restrict__ Y, int ldy,
                   size_t n) {
  __shared__ float Ys[K * K];
  for (int i = threadIdx.x; i < mv * keep; i += blockDim.x) Ys[i] = static_cast<float>(Y[(i / mv) * ldy + (i % mv)]);
  __syncthreads();
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    float v[K];
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < mv) v[k] = V[k * ld + j];
    for (int cc = 0; cc < keep; ++cc) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (k < mv) s = fmaf(v[k], Ys[cc * mv + k], s);
      V[cc * ld + j] = s;
    }
  }
}

template <int K>
__global__ void __launch_bounds__(kT)
combine_f32_kernel(const float *__restrict__ V, size_t ld, int m, const double *__restrict__ y, size_t n,
                   double *__restrict__ x) {
  __shared__ float ys[K];
  if (threadIdx.x < K) ys[threadIdx.x] = threadIdx.x < m ? static_cast<float>(y[threadIdx.x]) : 0.f;
  __syncthreads();
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (k < m) s = fmaf(V[k * ld + j], ys[k], s);
    x[j] = s;
  }
}

// ---- FP64-storage passes with mixed arithmetic (FP64 phase of the mixed
// mode, whose correction vectors carry FP32-accurate sigmas) ----------------
// Column 0 of the basis (the anchor: the run's start vector, after a restart
// the lowest Ritz vector) is handled in FP64; columns >= 1 (corrections,
// whose coefficients are of the size of the residual) in FP32 arithmetic
// with FP64 accumulation of the reductions, as the FP32 passes above.  The
// FP32 rounding of a correction term then enters scaled by its small
// coefficient, like the FP32 rounding of its sigma.

template <int K>
__global__ void __launch_bounds__(f32_block<K>(), f32_minb<K>())
multidot_mix_kernel(const double *__restrict__ V, size_t ld, int m, const double *__restrict__ w, size_t n,
                    double *__restrict__ partials) {
  __shared__ double acc_s[K * f32_block<K>()];
  SmemAcc<K, f32_block<K>()> acc{acc_s};
  acc.zero();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  double a0 = 0;
  for (size_t j0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j0 < n; j0 += stride * kChunk) {
    float f[K];
#pragma unroll
    for (int k = 0; k < K; ++k) f[k] = 0.f;
    for (int u = 0; u < kChunk; ++u) {
      const size_t j = j0 + u * stride;
      if (j >= n) break;
      const double wj = w[j];
      a0 = fma(V[j], wj, a0);
      const float wf = static_cast<float>(wj);
#pragma unroll
      for (int k = 1; k < K; ++k)
        if (k < m) f[k] = fmaf(static_cast<float>(V[k * ld + j]), wf, f[k]);
    }
    acc.add(f, m);
  }
  acc.a[threadIdx.x] = a0;  // column 0's slot holds its FP64 sum (the FP32 chunks left it at 0)
  acc.store(m, partials);
}

template <int K>
__global__ void __launch_bounds__(f32_block<K>(), f32_minb<K>())
residual_mix_kernel(const double *__restrict__ V, const double *__restrict__ VA, size_t ld, int m,
                    const double *__restrict__ y, double theta, double pre_theta, const double *__restrict__ diag,
                    size_t n, double *__restrict__ t, double *__restrict__ x_out, double *__restrict__ partials) {
  __shared__ float ys[K];
  __shared__ double acc_s[(K + 2) * f32_block<K>()];
  if (threadIdx.x < K) ys[threadIdx.x] = threadIdx.x < m ? static_cast<float>(y[threadIdx.x]) : 0.f;
  SmemAcc<K + 2, f32_block<K>()> acc{acc_s};
  acc.zero();
  __syncthreads();
  const double y0 = y[0];
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  double r2 = 0, t2 = 0, d0 = 0;  // FP64: ||r||^2, ||t||^2, V_0 . t
  for (size_t j0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j0 < n; j0 += stride * kChunk) {
    float f[K + 2];
#pragma unroll
    for (int k = 0; k < K + 2; ++k) f[k] = 0.f;
    for (int u = 0; u < kChunk; ++u) {
      const size_t j = j0 + u * stride;
      if (j >= n) break;
      float v[K];
      float xs = 0.f, as = 0.f;  // correction parts
#pragma unroll
      for (int k = 1; k < K; ++k)
        if (k < m) {
          v[k] = static_cast<float>(V[k * ld + j]);
          xs = fmaf(v[k], ys[k], xs);
          as = fmaf(static_cast<float>(VA[k * ld + j]), ys[k], as);
        }
      const double v0 = V[j];
      const double xv = fma(v0, y0, static_cast<double>(xs));
      const double av = fma(VA[j], y0, static_cast<double>(as));
      const double r = av - theta * xv;
      r2 = fma(r, r, r2);
      if (x_out) x_out[j] = xv;
      const double d = fabs(diag[j] - pre_theta);
      const double tv = d > 1e-12 ? r / d : r / 1e-12;  // davidson.c:214-227
      t[j] = tv;
      t2 = fma(tv, tv, t2);
      d0 = fma(v0, tv, d0);
      const float tf = static_cast<float>(tv);
#pragma unroll
      for (int k = 1; k < K; ++k)
        if (k < m) f[2 + k] = fmaf(v[k], tf, f[2 + k]);
    }
    acc.add(f, m + 2);
  }
  acc.a[0 * f32_block<K>() + threadIdx.x] = r2;
  acc.a[1 * f32_block<K>() + threadIdx.x] = t2;
  acc.a[2 * f32_block<K>() + threadIdx.x] = d0;
  acc.store(m + 2, partials);
}

template <int K>
__global__ void __launch_bounds__(f32_block<K>(), f32_minb<K>())
gs_update_mix_kernel(const double *__restrict__ V, size_t ld, int m, const double *__restrict__ c, size_t n,
                     double *__restrict__ t, double *__restrict__ partials) {
  __shared__ float cs[K];
  __shared__ double acc_s[(K + 1) * f32_block<K>()];
  if (threadIdx.x < K) cs[threadIdx.x] = threadIdx.x < m ? static_cast<float>(c[threadIdx.x]) : 0.f;
  SmemAcc<K + 1, f32_block<K>()> acc{acc_s};
  acc.zero();
  __syncthreads();
  const double c0 = c[0];
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  double t2 = 0, d0 = 0;
  for (size_t j0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j0 < n; j0 += stride * kChunk) {
    float f[K + 1];
#pragma unroll
    for (int k = 0; k < K + 1; ++k) f[k] = 0.f;
    for (int u = 0; u < kChunk; ++u) {
      const size_t j = j0 + u * stride;
      if (j >= n) break;
      float v[K];
      float cs_sum = 0.f;
#pragma unroll
      for (int k = 1; k < K; ++k)
        if (k < m) {
          v[k] = static_cast<float>(V[k * ld + j]);
          cs_sum = fmaf(cs[k], v[k], cs_sum);
        }
      const double v0 = V[j];
      const double tv = t[j] - fma(c0, v0, static_cast<double>(cs_sum));
      t[j] = tv;
      t2 = fma(tv, tv, t2);
      d0 = fma(v0, tv, d0);
      const float tf = static_cast<float>(tv);
#pragma unroll
      for (int k = 1; k < K; ++k)
        if (k < m) f[1 + k] = fmaf(v[k], tf, f[1 + k]);
    }
    acc.add(f, m + 1);
  }
  acc.a[0 * f32_block<K>() + threadIdx.x] = t2;
  acc.a[1 * f32_block<K>() + threadIdx.x] = d0;
  acc.store(m + 1, partials);
}

template <int K>
__global__ void __launch_bounds__(kT)
gs_finish_mix_kernel(const double *__restrict__ V, size_t ld, int m, const double *__restrict__ c, double scale,
                     size_t n, const double *__restrict__ t, double *__restrict__ out,
                     double *__restrict__ partials) {
  __shared__ float cs[K];
  if (threadIdx.x < K) cs[threadIdx.x] = threadIdx.x < m ? static_cast<float>(c[threadIdx.x]) : 0.f;
  __syncthreads();
  const double c0 = m > 0 ? c[0] : 0.0;
  double acc[1] = {0};
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    float cs_sum = 0.f;
#pragma unroll
    for (int k = 1; k < K; ++k)
      if (k < m) cs_sum = fmaf(cs[k], static_cast<float>(V[k * ld + j]), cs_sum);
    const double o = (t[j] - fma(c0, V[j], static_cast<double>(cs_sum))) * scale;
    out[j] = o;
    acc[0] = fma(o, o, acc[0]);
  }
  block_reduce_store<1>(acc, 1, partials);
}

template <typename A, typename B>
__global__ void convert_kernel(const A *__restrict__ a, B *__restrict__ b, size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    b[j] = static_cast<B>(a[j]);
}

template <typename S>
__global__ void scale_kernel(const S *__restrict__ a, double s, S *__restrict__ b, size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    b[j] = static_cast<S>(static_cast<double>(a[j]) * s);
}

// ---- RQ-CG (CG.c) --------------------------------------------------------
// partials: x.Ax, p.Ax, x.Ap, p.Ap, x.x, x.p, p.p
__global__ void __launch_bounds__(kT)
cg_gram_kernel(const double *__restrict__ x, const double *__restrict__ p, const double *__restrict__ Ax,
               const double *__restrict__ Ap, size_t n, double *__restrict__ partials) {
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    const double xv = x[j], pv = p[j], ax = Ax[j], ap = Ap[j];
    acc[0] += xv * ax;
    acc[1] += pv * ax;
    acc[2] += xv * ap;
    acc[3] += pv * ap;
    acc[4] += xv * xv;
    acc[5] += xv * pv;
    acc[6] += pv * pv;
  }
  block_reduce_store<7>(acc, 7, partials);
}

// x <- a x + b p, Ax <- a Ax + b Ap (skipped when first), g = 2 (Ax - rho x);
// partials: [0] g.g, then g <- g * pinv, [1] g.g
__global__ void __launch_bounds__(kT)
cg_update_kernel(double a, double b, int first, double rho, double *__restrict__ x, const double *__restrict__ p,
                 double *__restrict__ Ax, const double *__restrict__ Ap, double *__restrict__ g,
                 const double *__restrict__ pinv, size_t n, double *__restrict__ partials) {
  double acc[2] = {0, 0};
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    double xv = x[j], ax = Ax[j];
    if (!first) {
      xv = a * xv + b * p[j];
      ax = a * ax + b * Ap[j];
      x[j] = xv;
      Ax[j] = ax;
    }
    double gv = 2 * (ax - rho * xv);
    acc[0] += gv * gv;
    if (pinv) gv *= pinv[j];
    g[j] = gv;
    acc[1] += gv * gv;
  }
  block_reduce_store<2>(acc, 2, partials);
}

// p <- beta p - g (first: p = -g)
__global__ void cg_direction_kernel(double beta, int first, double *__restrict__ p, const double *__restrict__ g,
                                    size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    p[j] = first ? -g[j] : beta * p[j] - g[j];
}

// CG.c:57-63
__global__ void precond_inverse_kernel(const double *__restrict__ diag, double *__restrict__ pinv, size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    pinv[j] = fabs(diag[j]) > 1e-12 ? 1.0 / diag[j] : 1.0 / 1e-12;
}


// ---- start vectors (executable.c:270-299) --------------------------------
// first index of the minimum (the reference scans with a strict <)
__global__ void argmin_partial_kernel(const double *__restrict__ d, size_t n, double *__restrict__ pv,
                                      int64_t *__restrict__ pi) {
  __shared__ double sv[kT];
  __shared__ int64_t si[kT];
  double best = INFINITY;
  int64_t bi = -1;
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    const double v = d[j];
    if (v < best) {
      best = v;
      bi = static_cast<int64_t>(j);
    }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      const double ov = sv[threadIdx.x + w];
      const int64_t oi = si[threadIdx.x + w];
      if (oi >= 0 && (si[threadIdx.x] < 0 || ov < sv[threadIdx.x] || (ov == sv[threadIdx.x] && oi < si[threadIdx.x]))) {
        sv[threadIdx.x] = ov;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    pv[blockIdx.x] = sv[0];
    pi[blockIdx.x] = si[0];
  }
}

__global__ void argmin_final_kernel(const double *__restrict__ pv, const int64_t *__restrict__ pi, int nb,
                                    int64_t *__restrict__ out) {
  if (threadIdx.x != 0) return;
  double best = INFINITY;
  int64_t bi = 0;
  bool any = false;
  for (int b = 0; b < nb; ++b) {
    if (pi[b] < 0) continue;
    if (!any || pv[b] < best || (pv[b] == best && pi[b] < bi)) {
      best = pv[b];
      bi = pi[b];
      any = true;
    }
  }
  *out = bi;
}

__global__ void set_unit_kernel(double *__restrict__ t, size_t n, const int64_t *__restrict__ idx) {
  const int64_t k = *idx;
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    t[j] = static_cast<int64_t>(j) == k ? 1.0 : 0.0;
}

// positive uniform numbers in (0, 1] from a counter-based hash (splitmix64)
__global__ void fill_random_kernel(double *__restrict__ t, size_t n, uint64_t seed) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + j + 1;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    t[j] = (static_cast<double>(z >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  }
}

// FP32-storage update passes (Gram-Schmidt finish, deflation, combination):
// one full wave (SMs x resident blocks of the kernel, at most 2
// grid_blocks()), so no partial last wave idles most SMs (measured: the
// finish pass at 16 vectors, L=32, 14.4 -> 10.7 ms).  The FP64 passes keep
// grid_blocks() (their summation order, hence the FP64 results, stay fixed).
template <typename KernelT>
int wave_grid(KernelT kern, int threads) {
  static std::atomic<int> per_sm{0};  // one value per kernel instantiation (the query is a driver call)
  int b = per_sm.load(std::memory_order_relaxed);
  if (b == 0) {
    if (kernel_blocks(reinterpret_cast<const void *>(kern), threads, 0, &b) != DOCI_OK || b < 1) b = 1;
    per_sm.store(b, std::memory_order_relaxed);
  }
  const int g = device_sm_count() * b;
  return g < 2 * grid_blocks() ? g : 2 * grid_blocks();
}

template <typename S, template <typename, int> class Kern, typename... Args>
int dispatch_k(int m, cudaStream_t st, Args... args) {
  const int g = grid_blocks();
  if (m <= 8) Kern<S, 8>::run(g, st, args...);
  else if (m <= 16) Kern<S, 16>::run(g, st, args...);
  else Kern<S, 32>::run(g, st, args...);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

template <typename S, int K>
struct MultidotL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const S *w, size_t n, double *p) {
    if constexpr (std::is_same<S, float>::value)
      multidot_f32_kernel<K><<<wave_grid(multidot_f32_kernel<K>, f32_block<K>()), f32_block<K>(), 0, st>>>(V, ld, m, w, n, p);
    else
      multidot_kernel<S, K><<<g, kT, 0, st>>>(V, ld, m, w, n, p);
  }
};
template <typename S, int K>
struct MultidotMixL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const S *w, size_t n, double *p) {
    if constexpr (std::is_same<S, double>::value)
      multidot_mix_kernel<K><<<wave_grid(multidot_mix_kernel<K>, f32_block<K>()), f32_block<K>(), 0, st>>>(V, ld, m, w, n, p);
  }
};
template <typename S, int K>
struct ResidualMixL {
  static void run(int g, cudaStream_t st, const S *V, const S *VA, size_t ld, int m, const double *y, double th,
                  double pre, const double *diag, size_t n, S *t, double *x, double *p) {
    if constexpr (std::is_same<S, double>::value)
      residual_mix_kernel<K><<<wave_grid(residual_mix_kernel<K>, f32_block<K>()), f32_block<K>(), 0, st>>>(V, VA, ld, m, y, th, pre, diag, n,
                                                                              t, x, p);
  }
};
template <typename S, int K>
struct GsUpdateMixL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const double *c, size_t n, S *t, double *p) {
    if constexpr (std::is_same<S, double>::value)
      gs_update_mix_kernel<K><<<wave_grid(gs_update_mix_kernel<K>, f32_block<K>()), f32_block<K>(), 0, st>>>(V, ld, m, c, n, t, p);
  }
};
template <typename S, int K>
struct GsFinishMixL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const double *c, double sc, size_t n,
                  const S *t, S *out, double *p) {
    if constexpr (std::is_same<S, double>::value)
      gs_finish_mix_kernel<K><<<wave_grid(gs_finish_mix_kernel<K>, kT), kT, 0, st>>>(V, ld, m, c, sc, n, t, out, p);
  }
};
template <typename S, int K>
struct MultidotExactL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const S *w, size_t n, double *p) {
    multidot_kernel<S, K><<<g, kT, 0, st>>>(V, ld, m, w, n, p);
  }
};
template <typename S, int K>
struct ResidualL {
  static void run(int g, cudaStream_t st, const S *V, const S *VA, size_t ld, int m, const double *y, double th,
                  double pre, const double *diag, size_t n, S *t, double *x, double *p) {
    if constexpr (std::is_same<S, float>::value)
      residual_f32_kernel<K><<<wave_grid(residual_f32_kernel<K>, f32_block<K>()), f32_block<K>(), 0, st>>>(V, VA, ld, m, y, th, pre, diag, n,
                                                                              t, x, p);
    else
      residual_kernel<S, K><<<g, kT, 0, st>>>(V, VA, ld, m, y, th, pre, diag, n, t, x, p);
  }
};
template <typename S, int K>
struct GsUpdateL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const double *c, size_t n, S *t, double *p) {
    if constexpr (std::is_same<S, float>::value)
      gs_update_f32_kernel<K><<<wave_grid(gs_update_f32_kernel<K>, f32_block<K>()), f32_block<K>(), 0, st>>>(V, ld, m, c, n, t, p);
    else
      gs_update_kernel<S, K><<<g, kT, 0, st>>>(V, ld, m, c, n, t, p);
  }
};
template <typename S, int K>
struct GsFinishL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const double *c, double sc, size_t n,
                  const S *t, S *out, double *p) {
    if constexpr (std::is_same<S, float>::value)
      gs_finish_f32_kernel<K><<<wave_grid(gs_finish_f32_kernel<K>, kT), kT, 0, st>>>(V, ld, m, c, sc, n, t, out, p);
    else
      gs_finish_kernel<S, K><<<g, kT, 0, st>>>(V, ld, m, c, sc, n, t, out, p);
  }
};
template <typename S, int K>
struct DeflateL {
  static void run(int g, cudaStream_t st, S *V, size_t ld, int mv, int keep, const double *Y, int ldy, size_t n) {
    if constexpr (std::is_same<S, float>::value)
      deflate_f32_kernel<K><<<wave_grid(deflate_f32_kernel<K>, kT), kT, 0, st>>>(V, ld, mv, keep, Y, ldy, n);
    else
      deflate_kernel<S, K><<<g, kT, 0, st>>>(V, ld, mv, keep, Y, ldy, n);
  }
};
template <typename S, int K>
struct CombineL {
  static void run(int g, cudaStream_t st, const S *V, size_t ld, int m, const double *y, size_t n, double *x) {
    if constexpr (std::is_same<S, float>::value)
      combine_f32_kernel<K><<<wave_grid(combine_f32_kernel<K>, kT), kT, 0, st>>>(V, ld, m, y, n, x);
    else
      combine_kernel<S, K><<<g, kT, 0, st>>>(V, ld, m, y, n, x);
  }
};

}  // namespace

// the largest grid a reduction pass launches is 2 grid_blocks()
int vec_partials_capacity() { return kHeader + 2 * grid_blocks() * kMaxK; }

int vec_partials_init(double *partials, cudaStream_t st) {
  DOCI_CUDA(cudaMemsetAsync(partials, 0, sizeof(double), st));
  return DOCI_OK;
}

const double *vec_results(const double *partials) { return partials + 1; }

int vec_reduction_blocks() { return grid_blocks(); }

namespace {
__global__ void shifted_diag_kernel(const double *__restrict__ d, double shift, float *__restrict__ out, size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    out[j] = static_cast<float>(d[j] - shift);
}
}  // namespace

namespace {
__global__ void copy16_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst, size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    dst[j] = src[j];
}
__global__ void copy4_kernel(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    dst[j] = src[j];
}
}  // namespace

int vec_copy(void *dst, const void *src, size_t bytes, cudaStream_t st) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src);
  if ((a % 16) == 0 && (bytes % 4) == 0) {
    // 16-byte words for the bulk (D x 4 bytes is rarely a multiple of 16:
    // copying all of it in 4-byte words over the host link is much slower),
    // then the last one to three words
    const size_t n16 = bytes / 16, tail = bytes - n16 * 16;
    if (n16)
      copy16_kernel<<<grid_blocks() * 2, kT, 0, st>>>(static_cast<const uint4 *>(src), static_cast<uint4 *>(dst), n16);
    if (tail)
      copy4_kernel<<<1, 32, 0, st>>>(reinterpret_cast<const uint32_t *>(static_cast<const char *>(src) + n16 * 16),
                                     reinterpret_cast<uint32_t *>(static_cast<char *>(dst) + n16 * 16), tail / 4);
  } else if ((a % 4) == 0 && (bytes % 4) == 0)
    copy4_kernel<<<grid_blocks() * 2, kT, 0, st>>>(static_cast<const uint32_t *>(src), static_cast<uint32_t *>(dst),
                                                   bytes / 4);
  else
    return DOCI_ERR_INVALID;
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

namespace {
__global__ void axpy_kernel(double a, const double *__restrict__ x, double *__restrict__ y, size_t n) {
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x)
    y[j] = fma(a, x[j], y[j]);
}
}  // namespace

int vec_axpy(double a, const double *x, double *y, size_t n, cudaStream_t st) {
  axpy_kernel<<<grid_blocks(), kT, 0, st>>>(a, x, y, n);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}


int vec_shifted_diag32(const double *d, double shift, float *out, size_t n, cudaStream_t st) {
  shifted_diag_kernel<<<grid_blocks(), kT, 0, st>>>(d, shift, out, n);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

int vec_reduce(const double *partials, int nk, double *out, cudaStream_t st) {
  // the pass itself reduced its partials; copy its results
  DOCI_CUDA(cudaMemcpyAsync(out, partials + 1, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
  return DOCI_OK;
}

template <typename S>
int vec_multidot(const S *V, size_t ld, int m, const S *w, size_t n, double *partials, cudaStream_t st,
                 bool fp64_products, bool mixed) {
  if (m < 1 || m > 32) return DOCI_ERR_INVALID;
  if (mixed && std::is_same<S, double>::value) return dispatch_k<S, MultidotMixL>(m, st, V, ld, m, w, n, partials);
  if (fp64_products) return dispatch_k<S, MultidotExactL>(m, st, V, ld, m, w, n, partials);
  return dispatch_k<S, MultidotL>(m, st, V, ld, m, w, n, partials);
}
template <typename S>
int vec_residual(const S *V, const S *VA, size_t ld, int m, const double *y, double theta, const double *diag,
                 size_t n, S *t, double *x, double *partials, cudaStream_t st, double diag_shift, bool mixed) {
  if (m < 1 || m > 32) return DOCI_ERR_INVALID;
  if (mixed && std::is_same<S, double>::value)
    return dispatch_k<S, ResidualMixL>(m, st, V, VA, ld, m, y, theta, theta + diag_shift, diag, n, t, x, partials);
  return dispatch_k<S, ResidualL>(m, st, V, VA, ld, m, y, theta, theta + diag_shift, diag, n, t, x, partials);
}
template <typename S>
int vec_gs_update(const S *V, size_t ld, int m, const double *c, size_t n, S *t, double *partials, cudaStream_t st,
                  bool mixed) {
  if (m < 1 || m > 32) return DOCI_ERR_INVALID;
  if (mixed && std::is_same<S, double>::value) return dispatch_k<S, GsUpdateMixL>(m, st, V, ld, m, c, n, t, partials);
  return dispatch_k<S, GsUpdateL>(m, st, V, ld, m, c, n, t, partials);
}
template <typename S>
int vec_gs_finish(const S *V, size_t ld, int m, const double *c, double scale, size_t n, const S *t, S *out,
                  double *partials, cudaStream_t st, bool mixed) {
  if (m < 0 || m > 32) return DOCI_ERR_INVALID;
  if (m == 0) {
    scale_kernel<S><<<grid_blocks(), kT, 0, st>>>(t, scale, out, n);
    DOCI_CUDA(cudaGetLastError());
    return DOCI_OK;
  }
  if (mixed && std::is_same<S, double>::value)
    return dispatch_k<S, GsFinishMixL>(m, st, V, ld, m, c, scale, n, t, out, partials);
  return dispatch_k<S, GsFinishL>(m, st, V, ld, m, c, scale, n, t, out, partials);
}
template <typename S>
int vec_deflate(S *V, size_t ld, int mv, int keep, const double *Y, int ldy, size_t n, cudaStream_t st) {
  if (mv < 1 || mv > 32 || keep < 1 || keep > mv) return DOCI_ERR_INVALID;
  return dispatch_k<S, DeflateL>(mv, st, V, ld, mv, keep, Y, ldy, n);
}
template <typename S>
int vec_combine(const S *V, size_t ld, int m, const double *y, size_t n, double *x, cudaStream_t st) {
  if (m < 1 || m > 32) return DOCI_ERR_INVALID;
  return dispatch_k<S, CombineL>(m, st, V, ld, m, y, n, x);
}
template <typename A, typename B>
int vec_convert(const A *a, B *b, size_t n, cudaStream_t st) {
  convert_kernel<A, B><<<grid_blocks(), kT, 0, st>>>(a, b, n);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}


int vec_argmin(const double *d, size_t n, int64_t *idx, cudaStream_t st) {
  const int g = grid_blocks();
  double *pv = nullptr;
  DOCI_CUDA(cudaMallocAsync(&pv, (sizeof(double) + sizeof(int64_t)) * g + sizeof(int64_t), st));
  int64_t *pi = reinterpret_cast<int64_t *>(pv + g), *out = pi + g;
  argmin_partial_kernel<<<g, kT, 0, st>>>(d, n, pv, pi);
  argmin_final_kernel<<<1, 32, 0, st>>>(pv, pi, g, out);
  DOCI_CUDA(cudaGetLastError());
  DOCI_CUDA(cudaMemcpyAsync(idx, out, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  DOCI_CUDA(cudaFreeAsync(pv, st));
  return DOCI_OK;
}

int vec_set_unit(double *t, size_t n, int64_t idx, cudaStream_t st) {
  int64_t *d_idx = nullptr;
  DOCI_CUDA(cudaMallocAsync(&d_idx, sizeof(int64_t), st));
  DOCI_CUDA(cudaMemcpyAsync(d_idx, &idx, sizeof(int64_t), cudaMemcpyHostToDevice, st));
  set_unit_kernel<<<grid_blocks(), kT, 0, st>>>(t, n, d_idx);
  DOCI_CUDA(cudaGetLastError());
  DOCI_CUDA(cudaFreeAsync(d_idx, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  return DOCI_OK;
}

int vec_fill_random(double *t, size_t n, uint64_t seed, cudaStream_t st) {
  fill_random_kernel<<<grid_blocks(), kT, 0, st>>>(t, n, seed);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

int cg_gram(const double *x, const double *p, const double *Ax, const double *Ap, size_t n, double *partials,
            cudaStream_t st) {
  cg_gram_kernel<<<grid_blocks(), kT, 0, st>>>(x, p, Ax, Ap, n, partials);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}
int cg_update(double a, double b, int first, double rho, double *x, const double *p, double *Ax, const double *Ap,
              double *g, const double *pinv, size_t n, double *partials, cudaStream_t st) {
  cg_update_kernel<<<grid_blocks(), kT, 0, st>>>(a, b, first, rho, x, p, Ax, Ap, g, pinv, n, partials);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}
int cg_direction(double beta, int first, double *p, const double *g, size_t n, cudaStream_t st) {
  cg_direction_kernel<<<grid_blocks(), kT, 0, st>>>(beta, first, p, g, n);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}
int precond_inverse(const double *diag, double *pinv, size_t n, cudaStream_t st) {
  precond_inverse_kernel<<<grid_blocks(), kT, 0, st>>>(diag, pinv, n);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

#define DOCI_VEC_INST(S)                                                                                   \
  template int vec_multidot<S>(const S *, size_t, int, const S *, size_t, double *, cudaStream_t, bool,     \
                               bool);                                                                       \
  template int vec_residual<S>(const S *, const S *, size_t, int, const double *, double, const double *,   \
                               size_t, S *, double *, double *, cudaStream_t, double, bool);                \
  template int vec_gs_update<S>(const S *, size_t, int, const double *, size_t, S *, double *, cudaStream_t, \
                                bool);                                                                      \
  template int vec_gs_finish<S>(const S *, size_t, int, const double *, double, size_t, const S *, S *,      \
                                double *, cudaStream_t, bool);                                              \
  template int vec_deflate<S>(S *, size_t, int, int, const double *, int, size_t, cudaStream_t);            \
  template int vec_combine<S>(const S *, size_t, int, const double *, size_t, double *, cudaStream_t);
DOCI_VEC_INST(double)
DOCI_VEC_INST(float)
template int vec_convert<double, float>(const double *, float *, size_t, cudaStream_t);
template int vec_convert<float, double>(const float *, double *, size_t, cudaStream_t);

}  // namespace doci
