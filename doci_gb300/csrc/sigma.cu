// sigma.cu -- DOCI sigma = H x on the GPU, the diagonal and the addressing kernels.
//
// H[T,T]             = diag[T]                      (doci.c:550-628)
// H[T, T\i u a]      = K_ia = (ia|ia), i in T, a not in T   (doci.c:216-222)
//
// The reference enumerates the lower triangle and scatters into per-thread
// copies of sigma (doci.c:164-238).  Here every determinant gathers all of its
// N(L-N) neighbours instead (the race-free form of the commented
// doci_full_matvec, doci.c:314-376): one thread per determinant, no atomics,
// no partial vectors, sigma written once with coalesced stores.
#include <cuda_runtime.h>

#include "addressing.cuh"
#include "internal.h"

namespace doci {

namespace {

constexpr int kThreads = 256;

struct SigmaShape {
  uint32_t D;
  int L, N, nh;
};

// Shared tables: binomials and the mirrored K matrix (K[m][q] with m, q
// mirrored orbitals).
template <typename Real>
struct SigmaSmem {
  uint32_t binom[kBinomRows * kBinomCols];
  Real K[32 * 32];
};

// One determinant per thread (grid-stride).  NH is the compile-time bound on
// the number of holes L-N, so the per-hole terms E1/E2/q live in registers.
template <typename Real, int NH>
__global__ void __launch_bounds__(kThreads)
sigma_gather_kernel(SigmaShape s, const uint32_t *__restrict__ g_binom, const Real *__restrict__ g_K,
                    const Real *__restrict__ diag, const Real *__restrict__ x, Real *__restrict__ y) {
  __shared__ SigmaSmem<Real> sm;
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += blockDim.x) sm.binom[t] = g_binom[t];
  for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) sm.K[t] = g_K[t];
  __syncthreads();
  const uint32_t *B = sm.binom;
  const uint32_t Dm1 = s.D - 1;

  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < s.D; r += gridDim.x * blockDim.x) {
    const uint32_t R = Dm1 - r;
    const uint32_t M = dev::colex_unrank<kBinomCols>(R, s.L, s.N, B);
    dev::Neighbours<NH, kBinomCols> nb;
    nb.precompute(M, R, s.L, s.nh, B);
    struct Acc {
      const Real *K, *x;
      const Real *Krow;
      Real acc;
      __device__ __forceinline__ void begin(int m) { Krow = K + m * 32; }
      __device__ __forceinline__ void hop(int, int q, uint32_t idx) { acc += Krow[q] * __ldg(x + idx); }
    } f{sm.K, x, sm.K, diag[r] * x[r]};
    nb.visit(M, R, Dm1, s.N, s.nh, B, f);
    y[r] = f.acc;
  }
}

template <typename Real, int NH>
int launch_nh(const doci_ham *h, const void *x, void *y, cudaStream_t st) {
  const SigmaShape s{h->D, h->L, h->N, h->nh};
  static int blocks_per_sm = 0;
  if (!blocks_per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, sigma_gather_kernel<Real, NH>, kThreads, 0);
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  const uint64_t need = (static_cast<uint64_t>(h->D) + kThreads - 1) / kThreads;
  uint64_t grid = static_cast<uint64_t>(device_sm_count()) * blocks_per_sm;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  const Real *K = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_Kmir64)
                                                   : reinterpret_cast<const Real *>(h->d_Kmir32);
  const Real *dg = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_diag)
                                                    : reinterpret_cast<const Real *>(h->d_diag32);
  sigma_gather_kernel<Real, NH><<<static_cast<unsigned>(grid), kThreads, 0, st>>>(
      s, h->d_binom, K, dg, static_cast<const Real *>(x), static_cast<Real *>(y));
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

template <typename Real>
int launch_typed(const doci_ham *h, const void *x, void *y, cudaStream_t st) {
  const int nh = h->nh;
  if (nh <= 4) return launch_nh<Real, 4>(h, x, y, st);
  if (nh <= 8) return launch_nh<Real, 8>(h, x, y, st);
  if (nh <= 12) return launch_nh<Real, 12>(h, x, y, st);
  if (nh <= 16) return launch_nh<Real, 16>(h, x, y, st);
  if (nh <= 20) return launch_nh<Real, 20>(h, x, y, st);
  if (nh <= 24) return launch_nh<Real, 24>(h, x, y, st);
  if (nh <= 28) return launch_nh<Real, 28>(h, x, y, st);
  return launch_nh<Real, 32>(h, x, y, st);
}

// ---------------------------------------------------------------------------
// Diagonal, doci.c:550-628: for the occupied orbitals from the highest down,
// 2 h'_ii, then over all orbitals j ascending 2 (ii|jj) if j is occupied or
// (ij|ji) if it is empty.  Same additions in the same order as the
// reference, so the FP64 result is bit-identical; the terms the reference
// multiplies by zero are skipped (adding +-0 leaves the sum unchanged).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
diagonal_kernel(SigmaShape s, double core, const uint32_t *__restrict__ g_binom,
                const double *__restrict__ tab, double *__restrict__ out, float *__restrict__ out32) {
  __shared__ uint32_t binom[kBinomRows * kBinomCols];
  __shared__ double h2[32], J2[32 * 32], Kx[32 * 32];
  const int L = s.L;
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += blockDim.x) binom[t] = g_binom[t];
  for (int t = threadIdx.x; t < L; t += blockDim.x) h2[t] = tab[t];
  for (int t = threadIdx.x; t < L * L; t += blockDim.x) {
    J2[t] = tab[L + t];
    Kx[t] = tab[L + L * L + t];
  }
  __syncthreads();
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < s.D; r += gridDim.x * blockDim.x) {
    const uint32_t M = dev::colex_unrank<kBinomCols>(s.D - 1 - r, L, s.N, binom);
    const uint32_t bits = dev::mirror_bits(M, L);
    double t = core;
    uint32_t rem = bits;
    while (rem) {
      const int o1 = 31 - __clz(rem);
      rem &= ~(1u << o1);
      t += h2[o1];
      const double *jrow = J2 + o1 * L, *krow = Kx + o1 * L;
      for (int o2 = 0; o2 < L; ++o2) t += ((bits >> o2) & 1u) ? jrow[o2] : krow[o2];
    }
    out[r] = t;
    out32[r] = static_cast<float>(t);
  }
}

__global__ void bitstrings_kernel(SigmaShape s, const uint32_t *__restrict__ g_binom, uint64_t first,
                                  uint64_t count, uint32_t *__restrict__ out) {
  __shared__ uint32_t binom[kBinomRows * kBinomCols];
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += blockDim.x) binom[t] = g_binom[t];
  __syncthreads();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = static_cast<uint32_t>(first + i);
    out[i] = dev::mirror_bits(dev::colex_unrank<kBinomCols>(s.D - 1 - r, s.L, s.N, binom), s.L);
  }
}

// rank of each bitstring; -1 for a string that is not an N-subset of L orbitals
__global__ void ranks_kernel(SigmaShape s, const uint32_t *__restrict__ g_binom, const uint32_t *__restrict__ bits,
                             uint64_t count, int64_t *__restrict__ out) {
  __shared__ uint32_t binom[kBinomRows * kBinomCols];
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += blockDim.x) binom[t] = g_binom[t];
  __syncthreads();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t b = bits[i];
    if ((b & ~dev::low_mask(s.L)) || __popc(b) != s.N) {
      out[i] = -1;
      continue;
    }
    out[i] = static_cast<int64_t>(s.D - 1 - dev::colex_rank<kBinomCols>(dev::mirror_bits(b, s.L), binom));
  }
}

unsigned grid_for(uint64_t n) {
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = static_cast<uint64_t>(device_sm_count()) * 8;
  if (g > cap) g = cap;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

}  // namespace

int launch_sigma(const doci_ham *h, const void *x, void *y, int precision, cudaStream_t st) {
  if (precision == DOCI_FP64) return launch_typed<double>(h, x, y, st);
  if (precision == DOCI_FP32) return launch_typed<float>(h, x, y, st);
  return DOCI_ERR_INVALID;
}

int launch_diagonal(doci_ham *h, cudaStream_t st) {
  const SigmaShape s{h->D, h->L, h->N, h->nh};
  diagonal_kernel<<<grid_for(h->D), kThreads, 0, st>>>(s, h->core, h->d_binom, h->d_tab64, h->d_diag, h->d_diag32);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

int launch_bitstrings(const doci_ham *h, int64_t first, int64_t count, uint32_t *out, cudaStream_t st) {
  if (first < 0 || count < 0 || static_cast<uint64_t>(first) + static_cast<uint64_t>(count) > h->D)
    return DOCI_ERR_INVALID;
  if (count == 0) return DOCI_OK;
  const SigmaShape s{h->D, h->L, h->N, h->nh};
  bitstrings_kernel<<<grid_for(count), kThreads, 0, st>>>(s, h->d_binom, first, count, out);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

int launch_ranks(const doci_ham *h, const uint32_t *bits, int64_t count, int64_t *out, cudaStream_t st) {
  if (count < 0) return DOCI_ERR_INVALID;
  if (count == 0) return DOCI_OK;
  const SigmaShape s{h->D, h->L, h->N, h->nh};
  ranks_kernel<<<grid_for(count), kThreads, 0, st>>>(s, h->d_binom, bits, count, out);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

}  // namespace doci
