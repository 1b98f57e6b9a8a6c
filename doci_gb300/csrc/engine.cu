// engine.cu -- block Davidson for many Hamiltonians at once, device-resident.
//
// The batch engine behind doci_batch_solve, doci_solve_roots and the request
// server's solves (no counterpart in the reference, whose Davidson is
// single-root and single-problem: davidson.c:33-128).  Every problem of a
// batch advances in lockstep: one iteration is a fixed sequence of batched
// launches, each covering all problems at once through a shared work space
// of determinant tiles (sigma) and vector chunks (the vector passes):
//
//   subspace eigenproblem (one warp per problem, cyclic Jacobi in FP64)
//   -> thick restart where the basis is full (deflation pass)
//   -> residuals and diagonal-preconditioned corrections of every root
//   -> convergence / stall decisions (one thread per problem)
//   -> classical Gram-Schmidt of each correction of an unconverged root
//      against the basis, a second pass when the first leaves less than half
//      of its norm (projection passes with FP64 sums)
//   -> sigma of the new basis vectors (one multi-problem, multi-vector pass)
//   -> the new columns of the subspace matrices.
//
// All control lives on the device (basis sizes, active roots, flags), so the
// host only replays the iteration -- captured once as a CUDA graph -- and
// reads one flag per problem after it.  Per-problem arithmetic never depends
// on the other problems of the batch: a problem's determinants and vector
// chunks are the same whatever else runs, every reduction finishes in a fixed
// order (per-chunk partial rows summed by the problem's last chunk to
// finish), and the batched sigma has no atomics -- so a result is
// bit-identical alone and in any batch.  Large problems (from 2^22
// determinants, or as the shape's autotuning decides) take their sigmas from
// the single-problem kernels (launch_sigma: the pair form for FP32) on
// staging buffers instead (each on one of up to eight streams forked from
// and joined back into the engine's stream, so that several problems'
// kernels overlap); their results still do not depend on the batch,
// but the FP32 pair form's atomic adds make their last bits vary from run to
// run.  Mixed mode: an FP32 phase on H - s (s = the lowest diagonal
// element; FP32 basis, sigma and vector arithmetic with FP64 sums), ending at
// mixed_tol or when the largest residual has not reached a new minimum for
// 15 iterations, then the FP64 phase from its Ritz vectors.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "addressing.cuh"
#include "engine.h"
#include "internal.h"

namespace doci {
namespace {

constexpr int kET = 256;                // threads per block of the batched passes
constexpr int kEPer = 32;               // vector-pass elements per thread (FP32 partial sums over them)
constexpr int kEChunk = kET * kEPer;    // vector-pass chunk
constexpr int kMaxR = 8;                // roots
constexpr int kMaxV = 32;               // basis vectors
constexpr int kLdp = kMaxV + 2;         // partial-row length

struct EProb {
  uint32_t D;
  int L, N, nh;
  const void *K;        // mirrored K (32 x 32) in the phase's type
  const void *diag_s;   // the sigma's diagonal in the phase's type (FP32 phase: diag - shift)
  const double *diag;   // FP64 diagonal (preconditioner)
  double shift;         // the operator is H - shift
  void *V, *VA, *T;     // basis and its sigmas (D x maxv), corrections (D x R), phase's type
  double *X;            // Ritz vectors (D x R, FP64)
  uint32_t tile0, chunk0, nchunks;
  int max_its;          // this problem's iteration limit in the phase
  int dpt;              // sigma tile: kET * dpt determinants, dpt per thread (autotuned per shape)
};

struct EState {
  int m, m0, its, done, converged, stall, restart, kk, nact, added, sigmas, idx0, need2;
  int act[kMaxR];
  double best, n0, n1, scale;
  double res[kMaxR];
  double w[kMaxV];
  double c[kMaxV];
  double S[kMaxV * kMaxV];  // subspace matrix, column-major, leading dimension kMaxV
  double Y[kMaxV * kMaxV];  // its eigenvectors (columns), ascending eigenvalues w
};

struct EArgs {
  int n, R, maxv, keep, max_its, stall_window;
  double tol;
  EProb *P;
  EState *St;
  const uint32_t *tile0;   // n + 1 prefix offsets (sigma tiles)
  const uint32_t *chunk0;  // n + 1 prefix offsets (vector chunks)
  double *part;            // chunk x kLdp partial rows
  unsigned *cnt;           // per-problem arrival counters (zero between passes)
  const uint32_t *binom;
  int *flags;              // per problem: 1 while running (host reads it)
};

// the problem that owns global index b of a prefix table (n + 1 entries)
__device__ __forceinline__ int owner(const uint32_t *pre, int n, uint32_t b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pre + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <typename S>
__device__ __forceinline__ S *colp(void *base, uint32_t D, int c) {
  return static_cast<S *>(base) + static_cast<size_t>(c) * D;
}

// Per-chunk sums of nk values (the block's threads each hold acc[k]) into the
// chunk's partial row; the problem's last chunk to arrive sums the rows in
// chunk order into out[0..nk) and returns true (in every thread of that
// block).  Results do not depend on timing or on the other problems.
template <int NK>
__device__ bool chunk_reduce(const double (&acc)[NK], int nk, const EArgs &a, const EProb &pb, int p, uint32_t chunk,
                             double *out) {
  __shared__ double red[kET / 32][NK];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    if (k < nk) {
      double v = acc[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][k] = v;
    }
  }
  __syncthreads();
  double *row = a.part + static_cast<size_t>(pb.chunk0 + chunk) * kLdp;
  if (threadIdx.x < nk) {
    double s = 0;
    for (int w = 0; w < kET / 32; ++w) s += red[w][threadIdx.x];
    row[threadIdx.x] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(a.cnt + p, 1u) == pb.nchunks - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // one warp per output, lanes over the rows (stride 32), then a fixed
  // shuffle tree: the order depends only on the problem's chunk count
  const double *r0 = a.part + static_cast<size_t>(pb.chunk0) * kLdp;
  for (int k = warp; k < nk; k += kET / 32) {
    double s = 0;
    for (uint32_t c = lane; c < pb.nchunks; c += 32) s += __ldcg(r0 + static_cast<size_t>(c) * kLdp + k);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[k] = s;
  }
  if (threadIdx.x == 0) a.cnt[p] = 0;
  __syncthreads();
  return true;
}

// ---------------------------------------------------------------- sigma
// VA[:, m0 + v] = (H - shift) V[:, m0 + v] for the v < m - m0 new basis
// vectors of every running problem: a tile of kET * dpt determinants per
// block (dpt per thread, a per-shape choice of the tile autotuner), the
// neighbours by the prefix-sum ranks of addressing.cuh, every vector at once.
// The tile shape changes no arithmetic: each determinant's sum is the same.
template <typename S, int NH>
__global__ void __launch_bounds__(kET) eng_sigma(EArgs a) {
  __shared__ uint32_t B[kBinomRows * kBinomCols];
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += kET) B[t] = a.binom[t];
  __syncthreads();
  if (blockIdx.x >= __ldg(a.tile0 + a.n)) return;
  const int p = owner(a.tile0, a.n, blockIdx.x);
  const EProb &pb = a.P[p];
  const EState &st = a.St[p];
  if (st.done) return;
  const int m0 = st.m0, nv = st.m - st.m0;
  if (nv <= 0) return;
  const S *K = static_cast<const S *>(pb.K);
  const S *x = colp<S>(pb.V, pb.D, m0);
  S *y = colp<S>(pb.VA, pb.D, m0);
  const uint32_t tile_first = (blockIdx.x - pb.tile0) * kET * pb.dpt + threadIdx.x;
  for (int e = 0; e < pb.dpt; ++e) {
  const uint32_t r = tile_first + e * kET;
  if (r >= pb.D) return;
  const uint32_t Dm1 = pb.D - 1, R = Dm1 - r;
  const uint32_t M = dev::colex_unrank<kBinomCols>(R, pb.L, pb.N, B);
  dev::Neighbours<NH, kBinomCols> nb;
  nb.precompute(M, R, pb.L, pb.nh, B);
  struct Acc {
    const S *K, *x;
    uint32_t D;
    int nv;
    const S *Krow;
    S acc[kMaxR];
    __device__ __forceinline__ void begin(int m) { Krow = K + m * 32; }
    __device__ __forceinline__ void hop(int, int q, uint32_t idx) {
      const S kv = __ldg(Krow + q);
#pragma unroll
      for (int v = 0; v < kMaxR; ++v)
        if (v < nv) acc[v] += kv * __ldg(x + static_cast<size_t>(v) * D + idx);
    }
  } f{K, x, pb.D, nv, K, {}};
  const S d = static_cast<const S *>(pb.diag_s)[r];
#pragma unroll
  for (int v = 0; v < kMaxR; ++v)
    if (v < nv) f.acc[v] = d * x[static_cast<size_t>(v) * pb.D + r];
  nb.visit(M, R, Dm1, pb.N, pb.nh, B, f);
#pragma unroll
  for (int v = 0; v < kMaxR; ++v)
    if (v < nv) y[static_cast<size_t>(v) * pb.D + r] = f.acc[v];
  }
}

// ---------------------------------------------------------------- vector passes
// three resident blocks per SM for the FP32 phase's passes (register
// budget 85; at two per SM the projection passes ran at ~2.4 TB/s); the
// FP64 phase's few iterations keep the registers their arrays need
template <typename S>
constexpr int eng_minb() { return sizeof(S) == 4 ? 3 : 1; }

// chunk-local element range of this thread: j = base + e * kET, e < kEPer
#define ENG_CHUNK_PROLOGUE                                      \
  const int p = owner(a.chunk0, a.n, blockIdx.x);               \
  const EProb &pb = a.P[p];                                     \
  EState &st = a.St[p];                                         \
  const uint32_t chunk = blockIdx.x - pb.chunk0;                \
  const uint32_t jbase = chunk * kEChunk + threadIdx.x;

// products summed over the thread's elements in S, then into FP64
template <typename S, int KM>
__global__ void __launch_bounds__(kET, eng_minb<S>()) eng_subcol(EArgs a, int j) {
  ENG_CHUNK_PROLOGUE
  if (st.done) return;
  const int i = st.m0 + j;
  if (i >= st.m) return;
  const S *V = static_cast<const S *>(pb.V);
  const S *w = colp<S>(pb.VA, pb.D, i);
  S f[KM];
#pragma unroll
  for (int k = 0; k < KM; ++k) f[k] = S(0);
#pragma unroll 4
  for (int e = 0; e < kEPer; ++e) {
    const uint32_t jj = jbase + e * kET;
    if (jj < pb.D) {
      const S wj = w[jj];
#pragma unroll
      for (int k = 0; k < KM; ++k)
        if (k <= i) f[k] += V[static_cast<size_t>(k) * pb.D + jj] * wj;
    }
  }
  double acc[KM];
#pragma unroll
  for (int k = 0; k < KM; ++k) acc[k] = static_cast<double>(f[k]);
  __shared__ double out[KM];
  if (chunk_reduce<KM>(acc, i + 1, a, pb, p, chunk, out)) {
    if (threadIdx.x <= i) {
      st.S[i * kMaxV + threadIdx.x] = out[threadIdx.x];
      st.S[threadIdx.x * kMaxV + i] = out[threadIdx.x];
    }
  }
}

// residual of root q: x = V y, r = VA y - theta x, t = r / |diag - shift - theta|
// (cutoff 1e-12, davidson.c:214-227); sums |r|^2
template <typename S, int KM>
__global__ void __launch_bounds__(kET) eng_residual(EArgs a, int q) {
  ENG_CHUNK_PROLOGUE
  if (st.done) return;
  const int m = st.m;
  if (q >= (a.R < m ? a.R : m)) return;
  __shared__ S ys[KM];
  if (threadIdx.x < KM) ys[threadIdx.x] = threadIdx.x < m ? static_cast<S>(st.Y[q * kMaxV + threadIdx.x]) : S(0);
  __syncthreads();
  const double th = st.w[q];
  const S ths = static_cast<S>(th);
  const double pre = th + pb.shift;
  const S *V = static_cast<const S *>(pb.V), *VA = static_cast<const S *>(pb.VA);
  S *t = colp<S>(pb.T, pb.D, q);
  S f = S(0);
  for (int e = 0; e < kEPer; ++e) {
    const uint32_t jj = jbase + e * kET;
    if (jj >= pb.D) break;
    S xv = S(0), av = S(0);
#pragma unroll
    for (int k = 0; k < KM; ++k)
      if (k < m) {
        xv += V[static_cast<size_t>(k) * pb.D + jj] * ys[k];
        av += VA[static_cast<size_t>(k) * pb.D + jj] * ys[k];
      }
    const S r = av - ths * xv;
    f += r * r;
    const S dd = static_cast<S>(fabs(pb.diag[jj] - pre));
    t[jj] = dd > S(1e-12) ? r / dd : r / S(1e-12);
  }
  double acc[1] = {static_cast<double>(f)};
  __shared__ double out[1];
  if (chunk_reduce<1>(acc, 1, a, pb, p, chunk, out))
    if (threadIdx.x == 0) st.res[q] = sqrt(out[0]);
}

// projections of correction act[q]: [t.t, V_k.t]; with `update` (1: first
// pass, 2: second pass) first t -= sum_k c_k V_k (c from the previous
// projection).  The second pass runs only when the first left less than half
// of the correction's norm (the Daniel-Gragg-Kaufman-Stewart test).
template <typename S, int KM>
__global__ void __launch_bounds__(kET, eng_minb<S>()) eng_gs(EArgs a, int q, int update) {
  ENG_CHUNK_PROLOGUE
  if (st.done || q >= st.nact) return;
  if (update == 2 && !st.need2) return;
  const int m = st.m;
  __shared__ S cs[KM];
  if (threadIdx.x < KM) cs[threadIdx.x] = (update && threadIdx.x < m) ? static_cast<S>(st.c[threadIdx.x]) : S(0);
  __syncthreads();
  const S *V = static_cast<const S *>(pb.V);
  S *t = colp<S>(pb.T, pb.D, st.act[q]);
  S f[KM + 1];
#pragma unroll
  for (int k = 0; k < KM + 1; ++k) f[k] = S(0);
  for (int e = 0; e < kEPer; ++e) {
    const uint32_t jj = jbase + e * kET;
    if (jj >= pb.D) break;
    S tv = t[jj];
    S v[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k)
      if (k < m) v[k] = V[static_cast<size_t>(k) * pb.D + jj];
    if (update) {
#pragma unroll
      for (int k = 0; k < KM; ++k)
        if (k < m) tv -= cs[k] * v[k];
      t[jj] = tv;
    }
    f[0] += tv * tv;
#pragma unroll
    for (int k = 0; k < KM; ++k)
      if (k < m) f[1 + k] += v[k] * tv;
  }
  double acc[KM + 1];
#pragma unroll
  for (int k = 0; k < KM + 1; ++k) acc[k] = static_cast<double>(f[k]);
  __shared__ double out[KM + 1];
  if (chunk_reduce<KM + 1>(acc, m + 1, a, pb, p, chunk, out)) {
    if (threadIdx.x < m) st.c[threadIdx.x] = out[1 + threadIdx.x];
    if (threadIdx.x == 0) {
      if (!update) {
        st.n0 = out[0];
      } else {
        st.n1 = out[0];
        if (update == 1) st.need2 = !(out[0] > 0.25 * st.n0);
      }
    }
  }
}

// V[:, m] = t * scale for an added correction
template <typename S>
__global__ void __launch_bounds__(kET) eng_gs_finish(EArgs a, int q) {
  ENG_CHUNK_PROLOGUE
  if (st.done || q >= st.nact || !st.added) return;
  const S *t = colp<S>(pb.T, pb.D, st.act[q]);
  S *out = colp<S>(pb.V, pb.D, st.m);
  const S sc = static_cast<S>(st.scale);
  for (int e = 0; e < kEPer; ++e) {
    const uint32_t jj = jbase + e * kET;
    if (jj >= pb.D) break;
    out[jj] = t[jj] * sc;
  }
}

// thick restart: V[:, c] = sum_k V[:, k] Y[k, c], c < kk, in place (each
// element's row is read before it is written), the same for VA
template <typename S, int KM>
__global__ void __launch_bounds__(kET) eng_deflate(EArgs a) {
  ENG_CHUNK_PROLOGUE
  if (st.done || !st.restart) return;
  const int m = st.m, kk = st.kk;
  __shared__ S Ys[KM * KM];
  for (int i = threadIdx.x; i < KM * KM; i += kET) {
    const int k = i % KM, c = i / KM;
    Ys[i] = (k < m && c < kk) ? static_cast<S>(st.Y[c * kMaxV + k]) : S(0);
  }
  __syncthreads();
  for (int which = 0; which < 2; ++which) {
    S *V = static_cast<S *>(which ? pb.VA : pb.V);
    for (int e = 0; e < kEPer; ++e) {
      const uint32_t jj = jbase + e * kET;
      if (jj >= pb.D) break;
      S v[KM];
#pragma unroll
      for (int k = 0; k < KM; ++k)
        if (k < m) v[k] = V[static_cast<size_t>(k) * pb.D + jj];
      for (int c = 0; c < kk; ++c) {
        S s = S(0);
#pragma unroll
        for (int k = 0; k < KM; ++k)
          if (k < m) s += v[k] * Ys[c * KM + k];
        V[static_cast<size_t>(c) * pb.D + jj] = s;
      }
    }
  }
}

// X[:, r] = V Y[:, r] (FP64) for r < min(R, m)
template <typename S, int KM>
__global__ void __launch_bounds__(kET) eng_combine(EArgs a) {
  ENG_CHUNK_PROLOGUE
  const int m = st.m, nr = a.R < m ? a.R : m;
  const S *V = static_cast<const S *>(pb.V);
  for (int e = 0; e < kEPer; ++e) {
    const uint32_t jj = jbase + e * kET;
    if (jj >= pb.D) break;
    for (int r = 0; r < nr; ++r) {
      double s = 0;
#pragma unroll
      for (int k = 0; k < KM; ++k)
        if (k < m) s += static_cast<double>(V[static_cast<size_t>(k) * pb.D + jj]) * st.Y[r * kMaxV + k];
      pb.X[static_cast<size_t>(r) * pb.D + jj] = s;
    }
  }
}

// large problems take their sigmas from the single-problem kernels
// (launch_sigma) on fixed staging buffers: the new basis vectors are copied in
// (xs[v] = V[:, m0 + v], v < m - m0) and the sigmas out (VA[:, m0 + v] = ys[v])
template <typename S>
__global__ void eng_stage(EArgs a, int p, S *xs, const S *ys, int out) {
  const EProb &pb = a.P[p];
  const EState &st = a.St[p];
  if (st.done) return;
  const int m0 = st.m0, nv = st.m - st.m0;
  const size_t n = static_cast<size_t>(nv > 0 ? nv : 0) * pb.D;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (out) static_cast<S *>(pb.VA)[static_cast<size_t>(m0) * pb.D + i] = ys[i];
    else xs[i] = static_cast<const S *>(pb.V)[static_cast<size_t>(m0) * pb.D + i];
  }
}

// start vectors: T[:, r] = unit vector on the r-th smallest diagonal element
// (the first on ties; davidson's HF start, executable.c:276-288, extended)
template <typename S>
__global__ void __launch_bounds__(kET) eng_unit(EArgs a) {
  ENG_CHUNK_PROLOGUE
  for (int r = 0; r < a.R; ++r) {
    S *t = colp<S>(pb.T, pb.D, r);
    const int idx = reinterpret_cast<const int *>(st.act)[r];
    for (int e = 0; e < kEPer; ++e) {
      const uint32_t jj = jbase + e * kET;
      if (jj >= pb.D) break;
      t[jj] = static_cast<int>(jj) == idx ? S(1) : S(0);
    }
  }
}

// ---------------------------------------------------------------- per-problem control
// round r of the start-vector choice: the r-th smallest diagonal element
// (the first index on ties, excluding the r already chosen), stored in
// act[r]; every chunk finds its minimum, the problem's last chunk to arrive
// takes the minimum over the chunks in chunk order
__global__ void __launch_bounds__(kET) eng_lowest(EArgs a, int r) {
  ENG_CHUNK_PROLOGUE
  const int R = a.R < static_cast<int>(pb.D) ? a.R : static_cast<int>(pb.D);
  if (r >= R) return;
  __shared__ double wv[kET / 32];
  __shared__ uint32_t wi[kET / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double v = 1e308;
  uint32_t id = 0xffffffffu;
  for (int e = 0; e < kEPer; ++e) {
    const uint32_t jj = jbase + e * kET;
    if (jj >= pb.D) break;
    bool taken = false;
    for (int q = 0; q < r; ++q) taken |= static_cast<uint32_t>(st.act[q]) == jj;
    const double d = pb.diag[jj];
    if (!taken && (d < v || (d == v && jj < id))) {
      v = d;
      id = jj;
    }
  }
  auto better = [](double v2, uint32_t i2, double v1, uint32_t i1) { return v2 < v1 || (v2 == v1 && i2 < i1); };
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_down_sync(0xffffffffu, v, o);
    const uint32_t i2 = __shfl_down_sync(0xffffffffu, id, o);
    if (better(v2, i2, v, id)) {
      v = v2;
      id = i2;
    }
  }
  if (lane == 0) {
    wv[warp] = v;
    wi[warp] = id;
  }
  __syncthreads();
  double *row = a.part + static_cast<size_t>(pb.chunk0 + chunk) * kLdp;
  if (threadIdx.x == 0) {
    double bv = wv[0];
    uint32_t bi = wi[0];
    for (int w = 1; w < kET / 32; ++w)
      if (better(wv[w], wi[w], bv, bi)) {
        bv = wv[w];
        bi = wi[w];
      }
    row[0] = bv;
    row[1] = static_cast<double>(bi);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(a.cnt + p, 1u) == pb.nchunks - 1;
  __syncthreads();
  if (!last || warp != 0) return;
  __threadfence();
  const double *r0 = a.part + static_cast<size_t>(pb.chunk0) * kLdp;
  v = 1e308;
  id = 0xffffffffu;
  for (uint32_t c = lane; c < pb.nchunks; c += 32) {
    const double v2 = __ldcg(r0 + static_cast<size_t>(c) * kLdp);
    const uint32_t i2 = static_cast<uint32_t>(__ldcg(r0 + static_cast<size_t>(c) * kLdp + 1));
    if (better(v2, i2, v, id)) {
      v = v2;
      id = i2;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_down_sync(0xffffffffu, v, o);
    const uint32_t i2 = __shfl_down_sync(0xffffffffu, id, o);
    if (better(v2, i2, v, id)) {
      v = v2;
      id = i2;
    }
  }
  if (lane == 0) {
    st.act[r] = static_cast<int>(id);
    if (r == 0) st.idx0 = static_cast<int>(id);
    a.cnt[p] = 0;
  }
}

// fresh state of a phase: empty basis, every start vector to be added
__global__ void eng_init_state(EArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  EState &st = a.St[p];
  st.m = st.m0 = st.its = st.done = st.converged = st.stall = st.restart = st.kk = st.added = st.sigmas = 0;
  st.best = 1e300;
  const int R = a.R < static_cast<int>(a.P[p].D) ? a.R : static_cast<int>(a.P[p].D);
  st.nact = R;
  for (int r = 0; r < kMaxR; ++r) {
    st.act[r] = r;
    st.res[r] = 1e300;
  }
  for (int i = 0; i < kMaxV * kMaxV; ++i) st.S[i] = st.Y[i] = 0.0;
  for (int i = 0; i < kMaxV; ++i) st.w[i] = st.c[i] = 0.0;
  a.flags[p] = 1;
}

// the subspace eigenproblem of every running problem: one warp, Jacobi in
// FP64 with the round-robin (tournament) ordering: each round rotates n/2
// disjoint index pairs at once (one lane computes each rotation, lanes then
// apply them over rows and columns), n-1 rounds a sweep, until the
// off-diagonal part is below 1e-30 of the whole; ascending eigenvalues; then
// the restart decision
__global__ void __launch_bounds__(32) eng_eig(EArgs a) {
  const int p = blockIdx.x;
  EState &st = a.St[p];
  if (st.done) return;
  __shared__ double A[kMaxV * kMaxV], Vv[kMaxV * kMaxV];
  __shared__ double rc[kMaxV / 2], rs[kMaxV / 2];
  __shared__ int rp[kMaxV / 2], rq[kMaxV / 2];
  __shared__ double wv[kMaxV];
  __shared__ int idx[kMaxV];
  const int n = st.m, lane = threadIdx.x;
  const int n2 = n + (n & 1), half = n2 / 2;
  for (int i = lane; i < kMaxV * kMaxV; i += 32) {
    const int r = i % kMaxV, c = i / kMaxV;
    A[i] = (r < n && c < n) ? st.S[i] : 0.0;
    Vv[i] = (r == c) ? 1.0 : 0.0;
  }
  __syncwarp();
  for (int sweep = 0; sweep < 100 && n > 1; ++sweep) {
    double off = 0, tot = 0;
    for (int i = lane; i < n * n; i += 32) {
      const int r = i % n, c = i / n;
      const double e = A[c * kMaxV + r] * A[c * kMaxV + r];
      tot += e;
      if (r != c) off += e;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (off == 0 || off <= 1e-30 * tot) break;
    for (int round = 0; round < n2 - 1; ++round) {
      if (lane < half) {
        auto player = [&](int k) { return k == 0 ? 0 : ((k - 1 + round) % (n2 - 1)) + 1; };
        int pp = player(lane), qq = player(n2 - 1 - lane);
        if (pp > qq) {
          const int t = pp;
          pp = qq;
          qq = t;
        }
        double cs = 1.0, sn = 0.0;
        if (qq < n) {
          const double apq = A[qq * kMaxV + pp];
          if (apq != 0) {
            const double theta = (A[qq * kMaxV + qq] - A[pp * kMaxV + pp]) / (2 * apq);
            const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
            cs = 1 / sqrt(t * t + 1);
            sn = t * cs;
          }
        }
        rp[lane] = pp;
        rq[lane] = qq;
        rc[lane] = cs;
        rs[lane] = sn;
      }
      __syncwarp();
      if (lane < n) {
        for (int i = 0; i < half; ++i) {  // columns p, q of row `lane`
          const int pp = rp[i], qq = rq[i];
          if (qq >= n || rs[i] == 0.0) continue;
          const double cs = rc[i], sn = rs[i];
          const double akp = A[pp * kMaxV + lane], akq = A[qq * kMaxV + lane];
          A[pp * kMaxV + lane] = cs * akp - sn * akq;
          A[qq * kMaxV + lane] = sn * akp + cs * akq;
          const double vkp = Vv[pp * kMaxV + lane], vkq = Vv[qq * kMaxV + lane];
          Vv[pp * kMaxV + lane] = cs * vkp - sn * vkq;
          Vv[qq * kMaxV + lane] = sn * vkp + cs * vkq;
        }
      }
      __syncwarp();
      if (lane < n) {
        for (int i = 0; i < half; ++i) {  // rows p, q of column `lane`
          const int pp = rp[i], qq = rq[i];
          if (qq >= n || rs[i] == 0.0) continue;
          const double cs = rc[i], sn = rs[i];
          const double apk = A[lane * kMaxV + pp], aqk = A[lane * kMaxV + qq];
          A[lane * kMaxV + pp] = cs * apk - sn * aqk;
          A[lane * kMaxV + qq] = sn * apk + cs * aqk;
        }
      }
      __syncwarp();
    }
  }
  __syncwarp();
  if (lane == 0) {
    for (int i = 0; i < n; ++i) idx[i] = i;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j)
        if (A[idx[j] * (kMaxV + 1)] < A[idx[i] * (kMaxV + 1)]) {
          const int tmp = idx[i];
          idx[i] = idx[j];
          idx[j] = tmp;
        }
    for (int i = 0; i < n; ++i) wv[i] = A[idx[i] * (kMaxV + 1)];
  }
  __syncwarp();
  for (int i = 0; i < n; ++i) {
    if (lane < n) st.Y[i * kMaxV + lane] = Vv[idx[i] * kMaxV + lane];
  }
  if (lane < n) st.w[lane] = wv[lane];
  if (lane == 0) {
    ++st.its;
    st.restart = n + a.R > a.maxv;
    st.kk = a.keep < n ? a.keep : n;
  }
}

// after a deflation: the basis holds the kk lowest Ritz vectors, so the
// subspace matrix is diag(w) and its eigenvectors the unit vectors
__global__ void eng_after_restart(EArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  EState &st = a.St[p];
  if (st.done || !st.restart) return;
  const int kk = st.kk;
  for (int c = 0; c < kMaxV; ++c)
    for (int r = 0; r < kMaxV; ++r) {
      st.S[c * kMaxV + r] = (r == c && c < kk) ? st.w[c] : 0.0;
      st.Y[c * kMaxV + r] = (r == c && c < kk) ? 1.0 : 0.0;
    }
  st.m = kk;
  st.restart = 0;
}

// convergence (every root's residual <= tol), iteration limit, stall window;
// the unconverged roots become the corrections to add
__global__ void eng_control(EArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  EState &st = a.St[p];
  if (st.done) return;
  const int nr = a.R < st.m ? a.R : st.m;
  double worst = 0;
  int nact = 0;
  for (int r = 0; r < nr; ++r) {
    worst = st.res[r] > worst ? st.res[r] : worst;
    if (st.res[r] > a.tol) st.act[nact++] = r;
  }
  st.nact = nact;
  st.m0 = st.m;
  if (worst <= a.tol) {
    st.done = 1;
    st.converged = 1;
  } else if (st.its >= a.P[p].max_its) {
    st.done = 1;
  } else if (a.stall_window > 0) {
    if (worst < st.best) {
      st.best = worst;
      st.stall = 0;
    } else if (++st.stall >= a.stall_window) {
      st.done = 1;
    }
  }
  if (st.done) a.flags[p] = 0;
}

// after the two projection passes of correction q: keep it if an
// independent direction is left
__global__ void eng_orth_decide(EArgs a, int q) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  EState &st = a.St[p];
  if (st.done || q >= st.nact) return;
  const double n0 = st.n0, n1 = st.n1;
  st.added = (n0 > 0) && (n1 > 0) && (n1 > 1e-20 * n0) && st.m < a.maxv;
  st.scale = st.added ? 1.0 / sqrt(n1) : 0.0;
}

// commit an added vector; after the last correction, a basis that did not
// grow ends the solve, else the new vectors get their sigmas
__global__ void eng_orth_commit(EArgs a, int q, int last) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  EState &st = a.St[p];
  if (st.done) return;
  if (q < st.nact && st.added) {
    ++st.m;
    st.added = 0;
  }
  if (last) {
    if (st.m == st.m0) {
      st.done = 1;
      a.flags[p] = 0;
    } else {
      st.sigmas += st.m - st.m0;
    }
  }
}

// ---------------------------------------------------------------- host side
template <typename T>
struct DBuf {
  T *p = nullptr;
  cudaStream_t st = nullptr;
  int alloc(size_t n, cudaStream_t s) {
    st = s;
    DOCI_CUDA(cudaMallocAsync(&p, sizeof(T) * (n ? n : 1), s));
    return DOCI_OK;
  }
  ~DBuf() {
    if (p) cudaFreeAsync(p, st);
  }
};

inline unsigned nblk(uint64_t n) { return static_cast<unsigned>(n < 1 ? 1 : n); }

constexpr size_t kSideStreams = 8;

// streams forked from the engine's stream and joined back into it
struct SideStreams {
  int n = 0;
  cudaStream_t s[kSideStreams] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kSideStreams] = {};
  int make(int count) {
    DOCI_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    for (int i = 0; i < count; ++i) {
      DOCI_CUDA(cudaStreamCreateWithFlags(&s[i], cudaStreamNonBlocking));
      DOCI_CUDA(cudaEventCreateWithFlags(&join_ev[i], cudaEventDisableTiming));
      n = i + 1;
    }
    return DOCI_OK;
  }
  cudaError_t fork(cudaStream_t st) {
    cudaError_t e = cudaEventRecord(fork_ev, st);
    for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(s[i], fork_ev, 0);
    return e;
  }
  cudaError_t join(cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < n && e == cudaSuccess; ++i) {
      e = cudaEventRecord(join_ev[i], s[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, join_ev[i], 0);
    }
    return e;
  }
  ~SideStreams() {
    for (int i = 0; i < n; ++i) {
      cudaStreamDestroy(s[i]);
      cudaEventDestroy(join_ev[i]);
    }
    if (fork_ev) cudaEventDestroy(fork_ev);
  }
};

// a problem whose sigmas come from launch_sigma (its handle, or the FP32
// phase's shifted view of it) through staging buffers of R vectors
struct BigProb {
  int p;
  const doci_ham *h;
  void *xs, *ys;
  size_t D;
};

template <typename S, int KM, int NH>
int run_phase(EArgs &a, uint32_t ntiles, uint32_t nchunks, cudaStream_t st, bool unit_start,
              const std::vector<BigProb> &big) {
  const int n = a.n, R = a.R;
  const int prec = sizeof(S) == 8 ? DOCI_FP64 : DOCI_FP32;
  std::vector<char> big_running(big.size(), 1);
  const unsigned small = (n + 127) / 128;
  // side streams for the large problems' sigmas: each problem's copies and
  // kernels run on one of them, so that several problems' kernels overlap
  // (forked from and joined back into st with events, also inside the graph)
  SideStreams side;
  if (big.size() > 1) {
    const int ns = static_cast<int>(std::min<size_t>(big.size(), kSideStreams));
    if (const int se = side.make(ns)) return se;
  }
  eng_init_state<<<small, 128, 0, st>>>(a);
  if (unit_start) {
    for (int r = 0; r < R; ++r) eng_lowest<<<nblk(nchunks), kET, 0, st>>>(a, r);
    eng_unit<S><<<nblk(nchunks), kET, 0, st>>>(a);
    eng_init_state<<<small, 128, 0, st>>>(a);
  }
  DOCI_CUDA(cudaGetLastError());
  // the orthonormalisation of the corrections and the sigmas and subspace
  // columns of the vectors added (the start block is the first "corrections")
  auto extend = [&]() -> int {
    for (int q = 0; q < R; ++q) {
      eng_gs<S, KM><<<nblk(nchunks), kET, 0, st>>>(a, q, 0);
      eng_gs<S, KM><<<nblk(nchunks), kET, 0, st>>>(a, q, 1);
      eng_gs<S, KM><<<nblk(nchunks), kET, 0, st>>>(a, q, 2);
      eng_orth_decide<<<small, 128, 0, st>>>(a, q);
      eng_gs_finish<S><<<nblk(nchunks), kET, 0, st>>>(a, q);
      eng_orth_commit<<<small, 128, 0, st>>>(a, q, q == R - 1);
    }
    if (ntiles > 0) eng_sigma<S, NH><<<nblk(ntiles), kET, 0, st>>>(a);
    if (side.n > 0) DOCI_CUDA(side.fork(st));
    for (size_t b = 0, k = 0; b < big.size(); ++b) {
      if (!big_running[b]) continue;
      const BigProb &bp = big[b];
      cudaStream_t sb = side.n > 0 ? side.s[k++ % side.n] : st;
      eng_stage<S><<<nblk(std::min<uint64_t>((bp.D * R + 255) / 256, 4096)), 256, 0, sb>>>(
          a, bp.p, static_cast<S *>(bp.xs), nullptr, 0);
      for (int v = 0; v < R; ++v) {
        const int sv = launch_sigma(bp.h, static_cast<S *>(bp.xs) + v * bp.D, static_cast<S *>(bp.ys) + v * bp.D,
                                    prec, sb);
        if (sv) return sv;
      }
      eng_stage<S><<<nblk(std::min<uint64_t>((bp.D * R + 255) / 256, 4096)), 256, 0, sb>>>(
          a, bp.p, nullptr, static_cast<const S *>(bp.ys), 1);
    }
    if (side.n > 0) DOCI_CUDA(side.join(st));
    for (int j = 0; j < R; ++j) eng_subcol<S, KM><<<nblk(nchunks), kET, 0, st>>>(a, j);
    DOCI_CUDA(cudaGetLastError());
    return DOCI_OK;
  };
  int s = extend();
  if (s) return s;
  // one iteration, captured and replayed (captured again when a large
  // problem finishes, so that its sigmas are no longer launched)
  cudaGraphExec_t exec = nullptr;
  auto capture = [&]() -> int {
    if (exec) {
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    DOCI_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    eng_eig<<<n, 32, 0, st>>>(a);
    eng_deflate<S, KM><<<nblk(nchunks), kET, 0, st>>>(a);
    eng_after_restart<<<small, 128, 0, st>>>(a);
    for (int q = 0; q < R; ++q) eng_residual<S, KM><<<nblk(nchunks), kET, 0, st>>>(a, q);
    eng_control<<<small, 128, 0, st>>>(a);
    const int se = extend();
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (se) {
      if (graph) cudaGraphDestroy(graph);
      return se;
    }
    DOCI_CUDA(ce);
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    DOCI_CUDA(ce);
    return DOCI_OK;
  };
  s = capture();
  if (s) return s;
  std::vector<int> flags(n);
  int status = DOCI_OK;
  for (int it = 0; it <= a.max_its + 1; ++it) {
    cudaError_t e = cudaGraphLaunch(exec, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags.data(), a.flags, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      status = cuda_status(e, "batch engine iteration");
      break;
    }
    if (std::none_of(flags.begin(), flags.end(), [](int f) { return f != 0; })) break;
    bool changed = false;
    for (size_t b = 0; b < big.size(); ++b)
      if (big_running[b] && !flags[big[b].p]) {
        big_running[b] = 0;
        changed = true;
      }
    if (changed && (status = capture())) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (status) return status;
  eng_combine<S, KM><<<nblk(nchunks), kET, 0, st>>>(a);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

template <typename S, int KM>
int run_phase_nh(EArgs &a, int nh_max, uint32_t ntiles, uint32_t nchunks, cudaStream_t st, bool unit_start,
                 const std::vector<BigProb> &big) {
  if (nh_max <= 8) return run_phase<S, KM, 8>(a, ntiles, nchunks, st, unit_start, big);
  if (nh_max <= 16) return run_phase<S, KM, 16>(a, ntiles, nchunks, st, unit_start, big);
  if (nh_max <= 24) return run_phase<S, KM, 24>(a, ntiles, nchunks, st, unit_start, big);
  return run_phase<S, KM, 32>(a, ntiles, nchunks, st, unit_start, big);
}

template <typename S>
int run_phase_km(EArgs &a, int nh_max, uint32_t ntiles, uint32_t nchunks, cudaStream_t st, bool unit_start,
                 const std::vector<BigProb> &big) {
  if (a.maxv <= 8) return run_phase_nh<S, 8>(a, nh_max, ntiles, nchunks, st, unit_start, big);
  if (a.maxv <= 16) return run_phase_nh<S, 16>(a, nh_max, ntiles, nchunks, st, unit_start, big);
  return run_phase_nh<S, 32>(a, nh_max, ntiles, nchunks, st, unit_start, big);
}

__global__ void shifted_diag32_kernel(const double *d, double shift, float *out, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = static_cast<float>(d[i] - shift);
}

// sigma choice per (device, L, N): the tile shape of the batched pass
// (determinants per thread: 1, 2 or 4) and whether the problem's sigmas come
// from the single-problem kernels instead (untuned: from 2^22 determinants,
// where those kernels' row tilings beat the per-determinant gather)
struct TileChoice {
  int dpt = 1;
  int kernels = -1;  // -1 untuned
};
std::mutex g_tile_mu;
std::map<std::tuple<int, int, int>, TileChoice> g_tile;
constexpr uint32_t kBigD = 1u << 22;

TileChoice tile_choice(const doci_ham *h) {
  std::lock_guard<std::mutex> lk(g_tile_mu);
  auto it = g_tile.find(std::make_tuple(h->device, h->L, h->N));
  TileChoice c = it == g_tile.end() ? TileChoice{} : it->second;
  if (c.kernels < 0) c.kernels = h->D >= kBigD ? 1 : 0;
  return c;
}

__global__ void eng_tune_state(EState *st, int nv) {
  st->m0 = 0;
  st->m = nv;
  st->done = 0;
}

template <int NH>
void launch_tune_sigma(const EArgs &a, unsigned ntiles, cudaStream_t st) {
  eng_sigma<float, NH><<<ntiles, kET, 0, st>>>(a);
}

}  // namespace

int engine_tune(doci_ham *h, int nv, int *dpt_out) {
  if (!h || nv < 1 || nv > kMaxR) return DOCI_ERR_INVALID;
  cudaStream_t st = h->stream;
  const size_t D = h->D;
  DBuf<float> V, VA;
  DBuf<EProb> dP;
  DBuf<EState> dS;
  DBuf<uint32_t> dT0;
  int s;
  if ((s = V.alloc(D * nv, st)) || (s = VA.alloc(D * nv, st)) || (s = dP.alloc(1, st)) || (s = dS.alloc(1, st)) ||
      (s = dT0.alloc(2, st)))
    return s;
  DOCI_CUDA(cudaMemsetAsync(V.p, 0, sizeof(float) * D * nv, st));
  eng_tune_state<<<1, 1, 0, st>>>(dS.p, nv);
  EProb pb{};
  pb.D = h->D;
  pb.L = h->L;
  pb.N = h->N;
  pb.nh = h->nh;
  pb.K = h->d_Kmir32;
  pb.diag_s = h->d_diag32;
  pb.diag = h->d_diag;
  pb.V = V.p;
  pb.VA = VA.p;
  pb.tile0 = 0;
  EArgs a{};
  a.n = 1;
  a.R = nv;
  a.P = dP.p;
  a.St = dS.p;
  a.tile0 = dT0.p;
  a.binom = h->d_binom;
  cudaEvent_t e0, e1;
  DOCI_CUDA(cudaEventCreate(&e0));
  DOCI_CUDA(cudaEventCreate(&e1));
  int best = 1;
  float best_ms = 1e30f;
  for (int dpt : {1, 2, 4}) {
    pb.dpt = dpt;
    const uint32_t nt = static_cast<uint32_t>((D + static_cast<size_t>(kET) * dpt - 1) / (static_cast<size_t>(kET) * dpt));
    const uint32_t t0[2] = {0, nt};
    if (cudaMemcpyAsync(dP.p, &pb, sizeof pb, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dT0.p, t0, sizeof t0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      break;
    auto run = [&] {
      if (h->nh <= 8) launch_tune_sigma<8>(a, nt, st);
      else if (h->nh <= 16) launch_tune_sigma<16>(a, nt, st);
      else if (h->nh <= 24) launch_tune_sigma<24>(a, nt, st);
      else launch_tune_sigma<32>(a, nt, st);
    };
    run();  // warm-up
    cudaEventRecord(e0, st);
    for (int k = 0; k < 3; ++k) run();
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = dpt;
    }
  }
  // the single-problem kernels on the same vectors, one sigma per vector
  int kernels = 0;
  {
    bool ok = true;
    for (int k = 0; k < 4 && ok; ++k) {  // warm-up, then three timed rounds
      if (k == 1) cudaEventRecord(e0, st);
      for (int v = 0; v < nv && ok; ++v)
        ok = launch_sigma(h, V.p + static_cast<size_t>(v) * D, VA.p + static_cast<size_t>(v) * D, DOCI_FP32, st) ==
             DOCI_OK;
    }
    cudaEventRecord(e1, st);
    float ms = 1e30f;
    if (ok && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    kernels = ms < best_ms ? 1 : 0;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  DOCI_CUDA(cudaGetLastError());
  {
    std::lock_guard<std::mutex> lk(g_tile_mu);
    TileChoice c;
    c.dpt = best;
    c.kernels = kernels;
    g_tile[std::make_tuple(h->device, h->L, h->N)] = c;
  }
  if (dpt_out) *dpt_out = kernels ? 0 : best;
  return DOCI_OK;
}

int64_t engine_footprint(int L, int N, const doci_batch_opts &o) {
  if (L < 1 || L > 32 || N < 0 || N > L) return -1;
  const int64_t D = static_cast<int64_t>(binom64(L, N));
  const int64_t R = std::max(1, std::min(o.nroots, kMaxR));
  const int64_t mv = std::min(kMaxV, std::max(o.max_vec, 2 * o.nroots));
  const int64_t ham = D * 12 + (16ll << 20);  // the handle's diagonals and tables
  const int64_t x = D * R * 8;                 // Ritz vectors
  const int64_t p64 = 2 * mv * D * 8 + R * D * 8 + 2 * R * D * 8;  // + staging of a large problem
  const int64_t p32 = o.mode == DOCI_MODE_MIXED ? 2 * mv * D * 4 + R * D * 4 + D * 4 + 2 * R * D * 4 : 0;
  return ham + x + p64 + p32 + (1ll << 20);
}

int engine_solve(int n, doci_ham *const *hams, const doci_batch_opts &o, cudaStream_t st, doci_root_result *res,
                 double *const *vecs) {
  if (n < 1) return DOCI_OK;
  const int R = o.nroots;
  if (R < 1 || R > kMaxR) return DOCI_ERR_INVALID;
  EArgs a{};
  a.n = n;
  a.R = R;
  a.maxv = std::min(kMaxV, std::max(o.max_vec, 2 * R));
  // thick restart: by default keep 2 nroots Ritz vectors, at least a quarter
  // of the basis (keeping only the nroots wanted ones restarts every few
  // blocks and stalls the higher roots)
  a.keep = o.keep > 0 ? o.keep : std::max(2 * R, a.maxv / 4);
  if (a.keep < R) a.keep = R;
  if (a.keep > a.maxv - R) a.keep = a.maxv - R;
  a.tol = o.tol;
  std::vector<uint32_t> tile0(n + 1, 0), chunk0(n + 1, 0);
  std::vector<int> dpt(n, 1), big_idx;
  size_t total = 0;
  int nh_max = 1;
  for (int i = 0; i < n; ++i) {
    const doci_ham *h = hams[i];
    if (!h || static_cast<int64_t>(h->D) < 1) return DOCI_ERR_INVALID;
    const TileChoice tc = tile_choice(h);
    dpt[i] = tc.dpt;
    if (tc.kernels) big_idx.push_back(i);
    tile0[i + 1] = tile0[i] + (tc.kernels ? 0u : static_cast<uint32_t>((h->D + kET * dpt[i] - 1) / (kET * dpt[i])));
    chunk0[i + 1] = chunk0[i] + (h->D + kEChunk - 1) / kEChunk;
    total += h->D;
    nh_max = std::max(nh_max, h->nh);
  }
  const uint32_t ntiles = tile0[n], nchunks = chunk0[n];
  DBuf<EProb> dP;
  DBuf<EState> dS;
  DBuf<uint32_t> dT0, dC0;
  DBuf<double> dpart, dX;
  DBuf<unsigned> dcnt;
  DBuf<int> dflags;
  int s;
  if ((s = dP.alloc(n, st)) || (s = dS.alloc(n, st)) || (s = dT0.alloc(n + 1, st)) || (s = dC0.alloc(n + 1, st)) ||
      (s = dpart.alloc(static_cast<size_t>(nchunks) * kLdp, st)) || (s = dcnt.alloc(n, st)) ||
      (s = dflags.alloc(n, st)) || (s = dX.alloc(total * R, st)))
    return s;
  DOCI_CUDA(cudaMemcpyAsync(dT0.p, tile0.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, st));
  DOCI_CUDA(cudaMemcpyAsync(dC0.p, chunk0.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, st));
  DOCI_CUDA(cudaMemsetAsync(dcnt.p, 0, sizeof(unsigned) * n, st));
  a.St = dS.p;
  a.tile0 = dT0.p;
  a.chunk0 = dC0.p;
  a.part = dpart.p;
  a.cnt = dcnt.p;
  a.flags = dflags.p;
  a.binom = hams[0]->d_binom;
  a.P = dP.p;
  std::vector<EProb> P(n);
  std::vector<EState> host_st(n);
  auto upload = [&]() -> int {
    DOCI_CUDA(cudaMemcpyAsync(dP.p, P.data(), sizeof(EProb) * n, cudaMemcpyHostToDevice, st));
    return DOCI_OK;
  };
  auto fill_common = [&](size_t elem, void *V, void *VA, void *T) {
    size_t off = 0;
    for (int i = 0; i < n; ++i) {
      const doci_ham *h = hams[i];
      EProb &pb = P[i];
      pb.D = h->D;
      pb.L = h->L;
      pb.N = h->N;
      pb.nh = h->nh;
      pb.diag = h->d_diag;
      pb.V = static_cast<char *>(V) + off * a.maxv * elem;
      pb.VA = static_cast<char *>(VA) + off * a.maxv * elem;
      pb.T = static_cast<char *>(T) + off * R * elem;
      pb.X = dX.p + off * R;
      pb.tile0 = tile0[i];
      pb.dpt = dpt[i];
      pb.chunk0 = chunk0[i];
      pb.nchunks = chunk0[i + 1] - chunk0[i];
      off += h->D;
    }
  };
  std::vector<double> e32(static_cast<size_t>(n) * R, 0.0);
  std::vector<int> its32v(n, 0), sig32(n, 0);
  bool have_start = false;  // the FP64 phase starts from the FP32 phase's Ritz vectors
  if (o.mode == DOCI_MODE_MIXED) {
    DBuf<float> V, VA, T, d32;
    if ((s = V.alloc(total * a.maxv, st)) || (s = VA.alloc(total * a.maxv, st)) || (s = T.alloc(total * R, st)) ||
        (s = d32.alloc(total, st)))
      return s;
    fill_common(sizeof(float), V.p, VA.p, T.p);
    // shift = the lowest diagonal element of each problem
    {
      for (int i = 0; i < n; ++i) {
        P[i].K = hams[i]->d_Kmir32;
        P[i].shift = 0;
        P[i].diag_s = nullptr;
      }
      if ((s = upload())) return s;
      eng_init_state<<<(n + 127) / 128, 128, 0, st>>>(a);
      eng_lowest<<<nblk(nchunks), kET, 0, st>>>(a, 0);
      DOCI_CUDA(cudaGetLastError());
      DOCI_CUDA(cudaMemcpyAsync(host_st.data(), dS.p, sizeof(EState) * n, cudaMemcpyDeviceToHost, st));
      DOCI_CUDA(cudaStreamSynchronize(st));
      size_t off = 0;
      for (int i = 0; i < n; ++i) {
        double sh = 0;
        DOCI_CUDA(cudaMemcpyAsync(&sh, hams[i]->d_diag + host_st[i].idx0, sizeof(double), cudaMemcpyDeviceToHost,
                                  st));
        DOCI_CUDA(cudaStreamSynchronize(st));
        P[i].shift = sh;
        P[i].diag_s = d32.p + off;
        shifted_diag32_kernel<<<nblk(std::min<uint64_t>((hams[i]->D + 255) / 256, 4096)), 256, 0, st>>>(
            hams[i]->d_diag, sh, d32.p + off, hams[i]->D);
        off += hams[i]->D;
      }
      DOCI_CUDA(cudaGetLastError());
      if ((s = upload())) return s;
    }
    // large problems: shifted views (FP32 diagonal - shift) and staging
    std::vector<std::unique_ptr<doci_ham>> views;
    std::vector<std::unique_ptr<DBuf<float>>> stg;
    std::vector<BigProb> big;
    for (int i : big_idx) {
      views.emplace_back(new doci_ham(*hams[i]));
      views.back()->d_diag32 = static_cast<float *>(const_cast<void *>(P[i].diag_s));
      views.back()->sigma_kernel = hams[i]->sigma_kernel;
      stg.emplace_back(new DBuf<float>());
      if ((s = stg.back()->alloc(2 * static_cast<size_t>(hams[i]->D) * R, st))) return s;
      big.push_back(BigProb{i, views.back().get(), stg.back()->p, stg.back()->p + static_cast<size_t>(hams[i]->D) * R,
                            hams[i]->D});
    }
    EArgs a32 = a;
    a32.tol = o.mixed_tol > o.tol ? o.mixed_tol : o.tol;
    a32.stall_window = 15;
    a32.max_its = o.max_its;
    for (int i = 0; i < n; ++i) P[i].max_its = o.max_its;
    if ((s = upload())) return s;
    s = run_phase_km<float>(a32, nh_max, ntiles, nchunks, st, true, big);
    if (s) return s;
    DOCI_CUDA(cudaMemcpyAsync(host_st.data(), dS.p, sizeof(EState) * n, cudaMemcpyDeviceToHost, st));
    DOCI_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i) {
      its32v[i] = host_st[i].its;
      sig32[i] = host_st[i].sigmas;
      for (int r = 0; r < R; ++r) e32[static_cast<size_t>(i) * R + r] = host_st[i].w[r] + P[i].shift;
    }
    have_start = true;
  }
  // FP64 phase
  {
    DBuf<double> V, VA, T;
    if ((s = V.alloc(total * a.maxv, st)) || (s = VA.alloc(total * a.maxv, st)) || (s = T.alloc(total * R, st)))
      return s;
    fill_common(sizeof(double), V.p, VA.p, T.p);
    for (int i = 0; i < n; ++i) {
      P[i].K = hams[i]->d_Kmir64;
      P[i].diag_s = hams[i]->d_diag;
      P[i].shift = 0;
    }
    if ((s = upload())) return s;
    if (have_start) DOCI_CUDA(cudaMemcpyAsync(T.p, dX.p, sizeof(double) * total * R, cudaMemcpyDeviceToDevice, st));
    EArgs a64 = a;
    a64.stall_window = 0;
    // the FP64 phase may run max_its less the problem's FP32 iterations
    int max64 = 1;
    for (int i = 0; i < n; ++i) {
      P[i].max_its = have_start ? std::max(1, o.max_its - its32v[i]) : o.max_its;
      max64 = std::max(max64, P[i].max_its);
    }
    if ((s = upload())) return s;
    a64.max_its = max64;
    std::vector<std::unique_ptr<DBuf<double>>> stg;
    std::vector<BigProb> big;
    for (int i : big_idx) {
      stg.emplace_back(new DBuf<double>());
      if ((s = stg.back()->alloc(2 * static_cast<size_t>(hams[i]->D) * R, st))) return s;
      big.push_back(BigProb{i, hams[i], stg.back()->p, stg.back()->p + static_cast<size_t>(hams[i]->D) * R,
                            hams[i]->D});
    }
    s = run_phase_km<double>(a64, nh_max, ntiles, nchunks, st, !have_start, big);
    if (s) return s;
    DOCI_CUDA(cudaMemcpyAsync(host_st.data(), dS.p, sizeof(EState) * n, cudaMemcpyDeviceToHost, st));
    DOCI_CUDA(cudaStreamSynchronize(st));
  }
  size_t off = 0;
  for (int i = 0; i < n; ++i) {
    doci_root_result &r = res[i];
    const EState &es = host_st[i];
    const int nr = std::min(R, es.m);
    r.nroots = R;
    for (int k = 0; k < nr; ++k) {
      r.energy[k] = es.w[k];
      r.residual[k] = es.res[k];
      r.energy_fp32[k] = e32[static_cast<size_t>(i) * R + k];
    }
    r.iterations = es.its + its32v[i];
    r.iterations_fp32 = its32v[i];
    r.sigmas = es.sigmas + sig32[i];
    r.converged = es.converged;
    r.status = DOCI_OK;
    if (vecs && vecs[i]) {
      DOCI_CUDA(cudaMemcpyAsync(vecs[i], dX.p + off * R, sizeof(double) * hams[i]->D * R, cudaMemcpyDeviceToHost,
                                st));
    }
    off += hams[i]->D;
  }
  DOCI_CUDA(cudaStreamSynchronize(st));
  return DOCI_OK;
}

}  // namespace doci
