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

#include <cstdlib>

#include <mutex>
#include <map>
#include <tuple>
#include <set>
#include <type_traits>
#include <vector>

#include "addressing.cuh"
#include "ff.cuh"
#include "internal.h"

namespace doci {

#define DOCI_TRY_S(expr)            \
  do {                              \
    const int _st = (expr);         \
    if (_st != DOCI_OK) return _st; \
  } while (0)

namespace {

constexpr int kThreads = 256;

// Launch configuration shared by the dynamic-shared-memory kernels: once per
// kernel (under a lock: solves run concurrently from several host threads)
// the dynamic shared-memory limit is raised to what the device allows next to
// the kernel's static shared memory; the resident blocks per SM are queried
// per launch (a host-side computation).
std::mutex g_attr_mu;
std::map<const void *, size_t> g_attr_limit;

template <typename KernelT>
int blocks_for(KernelT kern, int threads, size_t dyn, int *blocks) {
  return kernel_blocks(reinterpret_cast<const void *>(kern), threads, dyn, blocks);
}

}  // namespace

int kernel_blocks(const void *key, int threads, size_t dyn, int *blocks) {
  {
    std::lock_guard<std::mutex> lock(g_attr_mu);
    auto it = g_attr_limit.find(key);
    if (it == g_attr_limit.end()) {
      int dev = 0, optin = 0;
      DOCI_CUDA(cudaGetDevice(&dev));
      DOCI_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
      cudaFuncAttributes fa;
      DOCI_CUDA(cudaFuncGetAttributes(&fa, key));
      const size_t limit = static_cast<size_t>(optin) > fa.sharedSizeBytes ? optin - fa.sharedSizeBytes : 0;
      DOCI_CUDA(cudaFuncSetAttribute(key, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(limit)));
      it = g_attr_limit.emplace(key, limit).first;
    }
    if (dyn > it->second) return DOCI_ERR_INVALID;
  }
  int b = 0;
  DOCI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, key, threads, dyn));
  *blocks = b < 1 ? 1 : b;
  return DOCI_OK;
}

namespace {

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
  int blocks_per_sm = 1;
  DOCI_TRY_S(blocks_for(sigma_gather_kernel<Real, NH>, kThreads, 0, &blocks_per_sm));
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

// Several vectors at once (block methods): x_v = x + v ldx, y_v = y + v ldy,
// v < nv <= NV.  The unrank, neighbour ranks and weights are computed once
// per determinant and hop and applied to every vector.
template <typename Real, int NH, int NV>
__global__ void __launch_bounds__(kThreads)
sigma_gather_multi_kernel(SigmaShape s, const uint32_t *__restrict__ g_binom, const Real *__restrict__ g_K,
                          const Real *__restrict__ diag, const Real *__restrict__ x, size_t ldx,
                          Real *__restrict__ y, size_t ldy, int nv) {
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
      size_t ldx;
      int nv;
      const Real *Krow;
      Real acc[NV];
      __device__ __forceinline__ void begin(int m) { Krow = K + m * 32; }
      __device__ __forceinline__ void hop(int, int q, uint32_t idx) {
        const Real kv = Krow[q];
#pragma unroll
        for (int v = 0; v < NV; ++v)
          if (v < nv) acc[v] += kv * __ldg(x + v * ldx + idx);
      }
    } f{sm.K, x, ldx, nv, sm.K, {}};
    const Real d = diag[r];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      if (v < nv) f.acc[v] = d * x[v * ldx + r];
    nb.visit(M, R, Dm1, s.N, s.nh, B, f);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      if (v < nv) y[v * ldy + r] = f.acc[v];
  }
}

template <typename Real, int NH>
int launch_gather_multi(const doci_ham *h, const void *x, size_t ldx, void *y, size_t ldy, int nv, cudaStream_t st) {
  const SigmaShape s{h->D, h->L, h->N, h->nh};
  int blocks_per_sm = 1;
  DOCI_TRY_S(blocks_for(sigma_gather_multi_kernel<Real, NH, 4>, kThreads, 0, &blocks_per_sm));
  const uint64_t need = (static_cast<uint64_t>(h->D) + kThreads - 1) / kThreads;
  uint64_t grid = static_cast<uint64_t>(device_sm_count()) * blocks_per_sm;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  const Real *K = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_Kmir64)
                                                   : reinterpret_cast<const Real *>(h->d_Kmir32);
  const Real *dg = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_diag)
                                                    : reinterpret_cast<const Real *>(h->d_diag32);
  sigma_gather_multi_kernel<Real, NH, 4><<<static_cast<unsigned>(grid), kThreads, 0, st>>>(
      s, h->d_binom, K, dg, static_cast<const Real *>(x), ldx, static_cast<Real *>(y), ldy, nv);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

template <typename Real>
int launch_gather_multi_typed(const doci_ham *h, const void *x, size_t ldx, void *y, size_t ldy, int nv,
                              cudaStream_t st) {
  const int nh = h->nh;
  if (nh <= 8) return launch_gather_multi<Real, 8>(h, x, ldx, y, ldy, nv, st);
  if (nh <= 16) return launch_gather_multi<Real, 16>(h, x, ldx, y, ldy, nv, st);
  if (nh <= 24) return launch_gather_multi<Real, 24>(h, x, ldx, y, ldy, nv, st);
  return launch_gather_multi<Real, 32>(h, x, ldx, y, ldy, nv, st);
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


// ---------------------------------------------------------------------------
// Row kernel.  Mirrored orbitals [0, split) form the column part, [split, L)
// the row part.  A row (fixed row-part occupation R, k elements; j = N - k in
// the column part) is a contiguous rank range of n = C(split, j) determinants;
// column c of the row holds colex_B = n - 1 - c of its column-part set.  One
// block handles one row at a time: it stages x[row] in shared memory and every
// thread computes whole columns, split into the four hop classes:
//   column part -> column part : gathers from the staged row (shared memory);
//   row part    -> row part    : the same column of another row of the same
//                                length (one coalesced load per hop);
//   row part    -> column part : column c' of row R\m (one more column element,
//                                colex of M_B u q = E1[h] + PVtot);
//   column part -> row part    : column c' of row R u q (colex of
//                                M_B \ m_k = PW(k) + PUtot - PU(k+1)).
// The rows' starts come from a table indexed by the row-part mask.
// ---------------------------------------------------------------------------
constexpr int kRowThreads = 256;
constexpr int kMaxRowPart = 24;                  // L - split
constexpr int kMaxIntraRow = 12 * 12;            // k (na - k) <= (na / 2)^2

struct RowShape {
  uint32_t D;
  int L, N, split, na, nrows;
};

template <typename Real>
struct RowTables {
  uint32_t binom[kBinomRows * kBinomCols];
  Real K[32 * 32];
  uint32_t aa_rs[kMaxIntraRow];  // row part -> row part: start of R \ m u q
  Real aa_K[kMaxIntraRow];
  uint32_t ab_rs[kMaxRowPart];   // row part -> column part: start of R \ m
  int ab_m[kMaxRowPart];
  uint32_t ba_rs[kMaxRowPart];   // column part -> row part: start of R u q
  int ba_q[kMaxRowPart];
  int n_aa, n_ab, n_ba;
};

template <typename Real, int NHB>
__global__ void __launch_bounds__(kRowThreads, 3)
sigma_row_kernel(RowShape s, int with_across, const uint2 *__restrict__ rows, const uint32_t *__restrict__ rowstart_of,
                 const uint32_t *__restrict__ g_binom, const Real *__restrict__ g_K, const Real *__restrict__ diag,
                 const Real *__restrict__ x, Real *__restrict__ y) {
  __shared__ RowTables<Real> tb;
  extern __shared__ __align__(16) unsigned char row_smem[];
  Real *xs = reinterpret_cast<Real *>(row_smem);
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += blockDim.x) tb.binom[t] = g_binom[t];
  for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) tb.K[t] = g_K[t];
  const uint32_t *B = tb.binom;
  const int sp = s.split, na = s.na;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  for (int row = blockIdx.x; row < s.nrows; row += gridDim.x) {
    const uint2 rw = rows[row];
    const uint32_t rstart = rw.x, mask = rw.y & 0xffffffu;
    const int k = static_cast<int>(rw.y >> 24), j = s.N - k;
    __syncthreads();  // previous row finished with xs and the tables
    if (warp == 0) {
      // row-part elements and holes, compacted with ballots
      const bool live = lane < na;
      const bool in_r = live && ((mask >> lane) & 1u);
      const bool hole = live && !in_r;
      const uint32_t eb = __ballot_sync(0xffffffffu, in_r), hb = __ballot_sync(0xffffffffu, hole);
      const uint32_t below = (1u << lane) - 1u;
      if (in_r) {
        const int e = __popc(eb & below);
        tb.ab_rs[e] = rowstart_of[mask & ~(1u << lane)];
        tb.ab_m[e] = sp + lane;
      }
      if (hole) {
        const int h = __popc(hb & below);
        tb.ba_rs[h] = rowstart_of[mask | (1u << lane)];
        tb.ba_q[h] = sp + lane;
      }
      const int ne = __popc(eb), nhl = __popc(hb);
      if (lane == 0) {
        tb.n_ab = j < sp ? ne : 0;   // a column-part hole must exist
        tb.n_ba = j > 0 ? nhl : 0;   // a column-part element must exist
        tb.n_aa = with_across ? ne * nhl : 0;
      }
      // row part -> row part pairs (element e, hole h)
      for (int t = lane; with_across && t < ne * nhl; t += 32) {
        const int e = t / nhl, h = t % nhl;
        const int a_e = __fns(eb, 0, e + 1), a_h = __fns(hb, 0, h + 1);
        tb.aa_rs[t] = rowstart_of[(mask & ~(1u << a_e)) | (1u << a_h)];
        tb.aa_K[t] = g_K[(sp + a_e) * 32 + sp + a_h];
      }
    }
    const uint32_t n = B[sp * kBinomCols + j];
    for (uint32_t c = threadIdx.x; c < n; c += blockDim.x) xs[c] = x[rstart + c];
    __syncthreads();

    const int n_aa = tb.n_aa, n_ab = tb.n_ab, n_ba = tb.n_ba;
    struct Acc {
      const RowTables<Real> &tb;
      const Real *xs, *x;
      const Real *Krow;
      Real acc;
      __device__ __forceinline__ void begin(int m) { Krow = tb.K + m * 32; }
      __device__ __forceinline__ void inrow(int, int q, uint32_t cc) { acc += Krow[q] * xs[cc]; }
      __device__ __forceinline__ void down(int t, int, int q, uint32_t cc) {
        acc += Krow[q] * __ldg(x + tb.ba_rs[t] + cc);
      }
      __device__ __forceinline__ void up(int t, int m, int q, uint32_t cc) {
        acc += tb.K[m * 32 + q] * __ldg(x + tb.ab_rs[t] + cc);
      }
      __device__ __forceinline__ void across(int t, uint32_t cc) { acc += tb.aa_K[t] * __ldg(x + tb.aa_rs[t] + cc); }
    };
    for (uint32_t c = threadIdx.x; c < n; c += blockDim.x) {
      Acc f{tb, xs, x, tb.K, diag[rstart + c] * xs[c]};
      dev::row_column_hops<NHB, kBinomCols>(c, n, sp, j, B, n_ab, tb.ab_m, n_ba, tb.ba_q, n_aa, f);
      y[rstart + c] = f.acc;
    }
  }
}

template <typename Real, int NHB, int NV>
__global__ void __launch_bounds__(kRowThreads, 2)
sigma_row_multi_kernel(RowShape s, int nv, size_t ldx, size_t ldy, uint32_t row_pad, const uint2 *__restrict__ rows, const uint32_t *__restrict__ rowstart_of,
                 const uint32_t *__restrict__ g_binom, const Real *__restrict__ g_K, const Real *__restrict__ diag,
                 const Real *__restrict__ x, Real *__restrict__ y) {
  __shared__ RowTables<Real> tb;
  extern __shared__ __align__(16) unsigned char row_smem[];
  Real *xs = reinterpret_cast<Real *>(row_smem);
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += blockDim.x) tb.binom[t] = g_binom[t];
  for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) tb.K[t] = g_K[t];
  const uint32_t *B = tb.binom;
  const int sp = s.split, na = s.na;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  for (int row = blockIdx.x; row < s.nrows; row += gridDim.x) {
    const uint2 rw = rows[row];
    const uint32_t rstart = rw.x, mask = rw.y & 0xffffffu;
    const int k = static_cast<int>(rw.y >> 24), j = s.N - k;
    __syncthreads();  // previous row finished with xs and the tables
    if (warp == 0) {
      // row-part elements and holes, compacted with ballots
      const bool live = lane < na;
      const bool in_r = live && ((mask >> lane) & 1u);
      const bool hole = live && !in_r;
      const uint32_t eb = __ballot_sync(0xffffffffu, in_r), hb = __ballot_sync(0xffffffffu, hole);
      const uint32_t below = (1u << lane) - 1u;
      if (in_r) {
        const int e = __popc(eb & below);
        tb.ab_rs[e] = rowstart_of[mask & ~(1u << lane)];
        tb.ab_m[e] = sp + lane;
      }
      if (hole) {
        const int h = __popc(hb & below);
        tb.ba_rs[h] = rowstart_of[mask | (1u << lane)];
        tb.ba_q[h] = sp + lane;
      }
      const int ne = __popc(eb), nhl = __popc(hb);
      if (lane == 0) {
        tb.n_ab = j < sp ? ne : 0;   // a column-part hole must exist
        tb.n_ba = j > 0 ? nhl : 0;   // a column-part element must exist
        tb.n_aa = ne * nhl;
      }
      // row part -> row part pairs (element e, hole h)
      for (int t = lane; t < ne * nhl; t += 32) {
        const int e = t / nhl, h = t % nhl;
        const int a_e = __fns(eb, 0, e + 1), a_h = __fns(hb, 0, h + 1);
        tb.aa_rs[t] = rowstart_of[(mask & ~(1u << a_e)) | (1u << a_h)];
        tb.aa_K[t] = g_K[(sp + a_e) * 32 + sp + a_h];
      }
    }
    const uint32_t n = B[sp * kBinomCols + j];
    for (int v = 0; v < nv; ++v)
      for (uint32_t c = threadIdx.x; c < n; c += blockDim.x) xs[v * row_pad + c] = x[v * ldx + rstart + c];
    __syncthreads();

    const int n_aa = tb.n_aa, n_ab = tb.n_ab, n_ba = tb.n_ba;
    struct Acc {
      const RowTables<Real> &tb;
      const Real *xs, *x;
      size_t ldx;
      uint32_t pad;
      int nv;
      const Real *Krow;
      Real acc[NV];
      __device__ __forceinline__ void begin(int m) { Krow = tb.K + m * 32; }
      __device__ __forceinline__ void inrow(int, int q, uint32_t cc) {
        const Real kv = Krow[q];
#pragma unroll
        for (int v = 0; v < NV; ++v)
          if (v < nv) acc[v] += kv * xs[v * pad + cc];
      }
      __device__ __forceinline__ void down(int t, int, int q, uint32_t cc) {
        const Real kv = Krow[q];
        const Real *src = x + tb.ba_rs[t] + cc;
#pragma unroll
        for (int v = 0; v < NV; ++v)
          if (v < nv) acc[v] += kv * __ldg(src + v * ldx);
      }
      __device__ __forceinline__ void up(int t, int m, int q, uint32_t cc) {
        const Real kv = tb.K[m * 32 + q];
        const Real *src = x + tb.ab_rs[t] + cc;
#pragma unroll
        for (int v = 0; v < NV; ++v)
          if (v < nv) acc[v] += kv * __ldg(src + v * ldx);
      }
      __device__ __forceinline__ void across(int t, uint32_t cc) {
        const Real kv = tb.aa_K[t];
        const Real *src = x + tb.aa_rs[t] + cc;
#pragma unroll
        for (int v = 0; v < NV; ++v)
          if (v < nv) acc[v] += kv * __ldg(src + v * ldx);
      }
    };
    for (uint32_t c = threadIdx.x; c < n; c += blockDim.x) {
      Acc f{tb, xs, x, ldx, row_pad, nv, tb.K, {}};
      const Real d = diag[rstart + c];
#pragma unroll
      for (int v = 0; v < NV; ++v)
        if (v < nv) f.acc[v] = d * xs[v * row_pad + c];
      dev::row_column_hops<NHB, kBinomCols>(c, n, sp, j, B, n_ab, tb.ab_m, n_ba, tb.ba_q, n_aa, f);
#pragma unroll
      for (int v = 0; v < NV; ++v)
        if (v < nv) y[v * ldy + rstart + c] = f.acc[v];
    }
  }
}


template <typename Real>
int launch_row_multi(const doci_ham *h, const void *x, size_t ldx, void *y, size_t ldy, int nv, cudaStream_t st) {
  const RowShape s{h->D, h->L, h->N, h->split, h->L - h->split, h->nrows};
  const uint32_t pad = (static_cast<uint32_t>(h->max_row) + 3u) & ~3u;
  const size_t dyn = static_cast<size_t>(nv) * pad * sizeof(Real);
  int blocks_per_sm = 1;
  DOCI_TRY_S(blocks_for(sigma_row_multi_kernel<Real, 16, 4>, kRowThreads, dyn, &blocks_per_sm));
  int grid = device_sm_count() * blocks_per_sm;
  if (grid > h->nrows) grid = h->nrows;
  const Real *K = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_Kmir64)
                                                   : reinterpret_cast<const Real *>(h->d_Kmir32);
  const Real *dg = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_diag)
                                                    : reinterpret_cast<const Real *>(h->d_diag32);
  sigma_row_multi_kernel<Real, 16, 4><<<grid, kRowThreads, dyn, st>>>(
      s, nv, ldx, ldy, pad, reinterpret_cast<const uint2 *>(h->d_rows), h->d_rowstart, h->d_binom, K, dg,
      static_cast<const Real *>(x), static_cast<Real *>(y));
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

template <typename Real>
int launch_row(const doci_ham *h, const void *x, void *y, cudaStream_t st, int with_across) {
  const RowShape s{h->D, h->L, h->N, h->split, h->L - h->split, h->nrows};
  const size_t dyn = static_cast<size_t>(h->max_row) * sizeof(Real);
  auto kern = sigma_row_kernel<Real, 16>;
  int blocks_per_sm = 1;
  DOCI_TRY_S(blocks_for(kern, kRowThreads, dyn, &blocks_per_sm));
  int grid = device_sm_count() * blocks_per_sm;
  if (grid > h->nrows) grid = h->nrows;
  const Real *K = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_Kmir64)
                                                   : reinterpret_cast<const Real *>(h->d_Kmir32);
  const Real *dg = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_diag)
                                                    : reinterpret_cast<const Real *>(h->d_diag32);
  kern<<<grid, kRowThreads, dyn, st>>>(s, with_across, reinterpret_cast<const uint2 *>(h->d_rows), h->d_rowstart,
                                       h->d_binom, K, dg, static_cast<const Real *>(x), static_cast<Real *>(y));
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

bool row_kernel_fits(const doci_ham *h, size_t elem) {
  if (h->split < 1 || h->nrows < 1) return false;
  if (h->L - h->split > kMaxRowPart || (h->L - h->split) > 32) return false;
  if (h->split - 0 > 16) return false;
  // largest (row-part elements x holes) product must fit the pair table
  const int na = h->L - h->split;
  if ((na / 2) * (na - na / 2) > kMaxIntraRow) return false;
  return static_cast<size_t>(h->max_row) * elem <= 160 * 1024;
}

// ---------------------------------------------------------------------------
// Phase-ordered row pass.  Same row tiling as sigma_row_kernel, but the
// cross hops are taken one source row at a time: each of the rows R u q
// (column part -> row part) and R \ m (row part -> column part) is staged in
// shared memory with cp.async, and every column of the output row gathers
// its neighbours from it, with the neighbour columns read from the
// precomputed tables (build_cross_tables).  The output row accumulates in
// shared memory across phases.  Phase 0 does the diagonal, the column-part
// hops (own row staged) and, when asked, the row-part hops (aligned loads).
// ---------------------------------------------------------------------------
constexpr int kRowxThreads = 256;

template <typename Real>
struct RowxTables {
  uint32_t binom[17 * kBinomCols];  // binomials C(n, k), n <= 16 (the column part)
  Real Kb[16 * 16];                 // K between column-part orbitals
  Real Kx[16];                      // K row of the current cross phase
  uint32_t aa_rs[kMaxIntraRow];
  Real aa_K[kMaxIntraRow];
  uint32_t ab_rs[kMaxRowPart];
  int ab_m[kMaxRowPart];
  uint32_t ba_rs[kMaxRowPart];
  int ba_q[kMaxRowPart];
  int n_aa, n_ab, n_ba;
};

template <int Bytes>
__device__ __forceinline__ void cp_async(void *smem, const void *g) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(g), "n"(Bytes));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename Real>
__device__ __forceinline__ void stage_row(Real *buf, const Real *src, uint32_t n) {
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) cp_async<sizeof(Real)>(buf + i, src + i);
  cp_async_wait_all();
}

// acc[c] += sum over the first `cnt` table entries (neighbour column << 8 | orbital)
template <typename Real>
__device__ __forceinline__ Real table_gather(const uint32_t *__restrict__ ent, int cnt, const Real *Kx, const Real *buf) {
  Real a = 0;
  const uint4 *e4 = reinterpret_cast<const uint4 *>(ent);
#pragma unroll
  for (int i4 = 0; i4 < 4; ++i4) {
    if (4 * i4 < cnt) {
      const uint4 v = __ldg(e4 + i4);
      a += Kx[v.x & 255u] * buf[v.x >> 8];
      if (4 * i4 + 1 < cnt) a += Kx[v.y & 255u] * buf[v.y >> 8];
      if (4 * i4 + 2 < cnt) a += Kx[v.z & 255u] * buf[v.z >> 8];
      if (4 * i4 + 3 < cnt) a += Kx[v.w & 255u] * buf[v.w >> 8];
    }
  }
  return a;
}

// Real: the arithmetic (double, float, or float-float with double tables,
// diagonal and output and a float-float x: Io<Real>)
template <typename Real, int NHB>
__global__ void __launch_bounds__(kRowxThreads, 2)
sigma_rowx_kernel(RowShape s, int with_across, uint32_t row_pad, const uint2 *__restrict__ rows,
                  const uint32_t *__restrict__ rowstart_of, const uint32_t *__restrict__ g_binom,
                  const typename Io<Real>::T *__restrict__ g_K, const uint32_t *__restrict__ rem_tab,
                  const uint32_t *__restrict__ ins_tab, const uint32_t *__restrict__ tab_off,
                  const typename Io<Real>::T *__restrict__ diag, const Real *__restrict__ x,
                  typename Io<Real>::T *__restrict__ y) {
  using IO = Io<Real>;
  __shared__ RowxTables<Real> tb;
  extern __shared__ __align__(16) unsigned char rowx_smem[];
  Real *acc = reinterpret_cast<Real *>(rowx_smem);
  Real *buf = acc + row_pad;
  const int sp = s.split, na = s.na;
  for (int t = threadIdx.x; t < 17 * kBinomCols; t += blockDim.x) tb.binom[t] = g_binom[t];
  for (int t = threadIdx.x; t < 256; t += blockDim.x) {
    const int m = t >> 4, q = t & 15;
    tb.Kb[t] = (m < sp && q < sp) ? IO::in(g_K[m * 32 + q]) : Real(0);
  }
  const uint32_t *B = tb.binom;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  for (int row = blockIdx.x; row < s.nrows; row += gridDim.x) {
    const uint2 rw = rows[row];
    const uint32_t rstart = rw.x, mask = rw.y & 0xffffffu;
    const int k = static_cast<int>(rw.y >> 24), j = s.N - k;
    __syncthreads();
    if (warp == 0) {
      const bool live = lane < na;
      const bool in_r = live && ((mask >> lane) & 1u);
      const bool hole = live && !in_r;
      const uint32_t eb = __ballot_sync(0xffffffffu, in_r), hb = __ballot_sync(0xffffffffu, hole);
      const uint32_t below = (1u << lane) - 1u;
      if (in_r) {
        const int e = __popc(eb & below);
        tb.ab_rs[e] = rowstart_of[mask & ~(1u << lane)];
        tb.ab_m[e] = sp + lane;
      }
      if (hole) {
        const int h = __popc(hb & below);
        tb.ba_rs[h] = rowstart_of[mask | (1u << lane)];
        tb.ba_q[h] = sp + lane;
      }
      const int ne = __popc(eb), nhl = __popc(hb);
      if (lane == 0) {
        tb.n_ab = j < sp ? ne : 0;
        tb.n_ba = j > 0 ? nhl : 0;
        tb.n_aa = with_across ? ne * nhl : 0;
      }
      for (int t = lane; with_across && t < ne * nhl; t += 32) {
        const int e = t / nhl, h = t % nhl;
        const int a_e = __fns(eb, 0, e + 1), a_h = __fns(hb, 0, h + 1);
        tb.aa_rs[t] = rowstart_of[(mask & ~(1u << a_e)) | (1u << a_h)];
        tb.aa_K[t] = IO::in(g_K[(sp + a_e) * 32 + sp + a_h]);
      }
    }
    const uint32_t n = B[sp * kBinomCols + j];
    stage_row(buf, x + rstart, n);
    __syncthreads();
    // phase 0: diagonal, column-part hops from the staged own row, row-part hops
    const int n_aa = tb.n_aa, n_ab = tb.n_ab, n_ba = tb.n_ba;
    for (uint32_t c = threadIdx.x; c < n; c += blockDim.x) {
      const uint32_t p = n - 1 - c;
      const uint32_t Mb = dev::colex_unrank<kBinomCols>(p, sp, j, B);
      dev::Neighbours<NHB, kBinomCols> nb;
      nb.precompute(Mb, p, sp, sp - j, B);
      struct In {
        const Real *Kb, *buf;
        const Real *Krow;
        Real a;
        __device__ __forceinline__ void begin(int m) { Krow = Kb + m * 16; }
        __device__ __forceinline__ void hop(int, int q, uint32_t cc) { a += Krow[q] * buf[cc]; }
      } f{tb.Kb, buf, tb.Kb, IO::in(diag[rstart + c]) * buf[c]};
      nb.visit(Mb, p, n - 1, j, sp - j, B, f);
      Real a2 = 0;
      int t = 0;
      for (; t + 4 <= n_aa; t += 4) {
        const Real v0 = ldg_val(x + tb.aa_rs[t] + c), v1 = ldg_val(x + tb.aa_rs[t + 1] + c);
        const Real v2 = ldg_val(x + tb.aa_rs[t + 2] + c), v3 = ldg_val(x + tb.aa_rs[t + 3] + c);
        a2 += tb.aa_K[t] * v0 + tb.aa_K[t + 1] * v1 + tb.aa_K[t + 2] * v2 + tb.aa_K[t + 3] * v3;
      }
      for (; t < n_aa; ++t) a2 += tb.aa_K[t] * ldg_val(x + tb.aa_rs[t] + c);
      acc[c] = f.a + a2;
    }
    // column part -> row part: sources R u q, one at a time
    if (n_ba > 0) {
      const uint32_t n_dn = B[sp * kBinomCols + j - 1];
      const uint32_t *remj = rem_tab + tab_off[j];
      for (int t = 0; t < n_ba; ++t) {
        __syncthreads();
        if (threadIdx.x < 16) tb.Kx[threadIdx.x] = threadIdx.x < sp ? IO::in(g_K[threadIdx.x * 32 + tb.ba_q[t]]) : Real(0);
        stage_row(buf, x + tb.ba_rs[t], n_dn);
        __syncthreads();
        for (uint32_t c = threadIdx.x; c < n; c += blockDim.x) acc[c] += table_gather(remj + 16 * c, j, tb.Kx, buf);
      }
    }
    // row part -> column part: sources R \ m, one at a time
    if (n_ab > 0) {
      const uint32_t n_up = B[sp * kBinomCols + j + 1];
      const uint32_t *insj = ins_tab + tab_off[j];
      for (int t = 0; t < n_ab; ++t) {
        __syncthreads();
        if (threadIdx.x < 16) tb.Kx[threadIdx.x] = threadIdx.x < sp ? IO::in(g_K[tb.ab_m[t] * 32 + threadIdx.x]) : Real(0);
        stage_row(buf, x + tb.ab_rs[t], n_up);
        __syncthreads();
        for (uint32_t c = threadIdx.x; c < n; c += blockDim.x)
          acc[c] += table_gather(insj + 16 * c, sp - j, tb.Kx, buf);
      }
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < n; c += blockDim.x) y[rstart + c] = IO::out(acc[c]);
  }
}

template <typename Real>
int launch_rowx(const doci_ham *h, const void *x, void *y, cudaStream_t st, int with_across) {
  const RowShape s{h->D, h->L, h->N, h->split, h->L - h->split, h->nrows};
  const uint32_t pad = (static_cast<uint32_t>(h->max_row) + 3u) & ~3u;
  const size_t dyn = 2 * static_cast<size_t>(pad) * sizeof(Real);
  auto kern = sigma_rowx_kernel<Real, 16>;
  int blocks_per_sm = 1;
  DOCI_TRY_S(blocks_for(kern, kRowxThreads, dyn, &blocks_per_sm));
  int grid = device_sm_count() * blocks_per_sm;
  if (grid > h->nrows) grid = h->nrows;
  const Real *K = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_Kmir64)
                                                   : reinterpret_cast<const Real *>(h->d_Kmir32);
  const Real *dg = std::is_same<Real, double>::value ? reinterpret_cast<const Real *>(h->d_diag)
                                                    : reinterpret_cast<const Real *>(h->d_diag32);
  kern<<<grid, kRowxThreads, dyn, st>>>(s, with_across, pad, reinterpret_cast<const uint2 *>(h->d_rows),
                                        h->d_rowstart, h->d_binom, K, h->d_rem, h->d_ins, h->d_tab_off, dg,
                                        static_cast<const Real *>(x), static_cast<Real *>(y));
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

unsigned grid_for(uint64_t n);

__global__ void to_ff_kernel(const double *__restrict__ x, ff *__restrict__ out, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = ff_from(x[i]);
}

// FP64-accurate sigma in float-float arithmetic: x converted to float-float
// once (stream-ordered scratch of D x 8 bytes), the phase-ordered row pass
// on it, double diagonal and output
int launch_rowx_ff(const doci_ham *h, const double *x, double *y, cudaStream_t st) {
  const RowShape s{h->D, h->L, h->N, h->split, h->L - h->split, h->nrows};
  const uint32_t pad = (static_cast<uint32_t>(h->max_row) + 3u) & ~3u;
  const size_t dyn = 2 * static_cast<size_t>(pad) * sizeof(ff);
  auto kern = sigma_rowx_kernel<ff, 16>;
  int blocks_per_sm = 1;
  DOCI_TRY_S(blocks_for(kern, kRowxThreads, dyn, &blocks_per_sm));
  int grid = device_sm_count() * blocks_per_sm;
  if (grid > h->nrows) grid = h->nrows;
  ff *xf = nullptr;
  DOCI_CUDA(cudaMallocAsync(&xf, sizeof(ff) * static_cast<size_t>(h->D), st));
  to_ff_kernel<<<grid_for(h->D), kThreads, 0, st>>>(x, xf, h->D);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    kern<<<grid, kRowxThreads, dyn, st>>>(s, 1, pad, reinterpret_cast<const uint2 *>(h->d_rows), h->d_rowstart,
                                          h->d_binom, h->d_Kmir64, h->d_rem, h->d_ins, h->d_tab_off, h->d_diag, xf,
                                          y);
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(xf, st);
  DOCI_CUDA(e);
  DOCI_CUDA(ef);
  return DOCI_OK;
}

bool rowx_fits(const doci_ham *h, size_t elem) {
  if (!h->d_rem || h->split > 16) return false;
  return 2 * (static_cast<size_t>(h->max_row) + 3) * elem <= 210 * 1024;
}

unsigned grid_for(uint64_t n) {
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = static_cast<uint64_t>(device_sm_count()) * 8;
  if (g > cap) g = cap;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

}  // namespace

namespace {

// ---------------------------------------------------------------------------
// Autotuning: the kernel path per problem shape, chosen by timing the
// candidates (doci_ham_autotune).  Choices are kept per (device, L, N,
// precision, vectors, pair form allowed) for the whole process: the kernels'
// speed depends on the shape, not on the integrals.
// ---------------------------------------------------------------------------
struct TuneKey {
  int device, L, N, precision, nv, allow_pair;
  bool operator<(const TuneKey &o) const {
    return std::tie(device, L, N, precision, nv, allow_pair) <
           std::tie(o.device, o.L, o.N, o.precision, o.nv, o.allow_pair);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tuned;

TuneKey tune_key(const doci_ham *h, int precision, int nv, bool allow_pair) {
  return TuneKey{h->device, h->L, h->N, precision, nv, allow_pair ? 1 : 0};
}

int tuned_choice(const doci_ham *h, int precision, int nv, bool allow_pair) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(tune_key(h, precision, nv, allow_pair));
  return it == g_tuned.end() ? 0 : it->second;
}

// The path of kind `kind` (0 = the heuristics) for this handle; a kind that
// does not fit falls back as described at doci_ham_set_sigma_kernel.
SigmaPlan plan_kind(const doci_ham *h, int precision, bool allow_pair, int kind) {
  const size_t elem = precision == DOCI_FP64 ? 8 : 4;
  if (precision == DOCI_FP64 && (kind == 6 || kind == 8)) kind = 0;  // FP32-only forms: the automatic FP64 path
  if (allow_pair && precision == DOCI_FP32) {
    // tensor-core pair form with TMA-staged hole rows: on request (kind 8)
    if (kind == 8 && tc_fits(h)) return {8, tc_launches(h)};
    // mma.sync pair form: the automatic FP32 choice where it fits and the
    // space gives every SM blocks of work (measured fastest there)
    const bool want_pair = kind == 6 || kind == 8 || (kind == 0 && h->npblocks >= device_sm_count());
    if (want_pair && pair_fits(h)) return {6, 2};  // init pass + pair pass
  }
  // float-float sigma (FP64 accuracy in FP32 arithmetic): the pair form, or
  // the phase-ordered row pass where the pair tiling does not fit; the x
  // conversion (with sigma = diag x for the pair form) and the pass
  if (kind == 9 && precision == DOCI_FP64 && (pair_ff_fits(h) || (h->nrows >= 1 && rowx_fits(h, sizeof(ff)))))
    return {9, 2};
  // the automatic FP64 choice where the pair tiling gives every SM blocks of
  // work: the float-float pair form (measured 3.2x faster than the row pass
  // at L=32, N=16: 138.6 ms against 444.9 ms)
  if (kind == 0 && allow_pair && precision == DOCI_FP64 && h->npblocks >= device_sm_count() && pair_ff_fits(h))
    return {9, 2};
  // row kernel when the row tiling exists, fits, and gives every SM work
  bool row = kind >= 3 || (kind == 0 && h->nrows >= device_sm_count());
  if (row && !row_kernel_fits(h, elem)) row = false;
  if (!row) return {1, 1};
  // automatic: the phase-ordered pass for FP64 (measured faster there), the
  // single row pass for FP32 (measured faster there)
  const bool want_rowx = kind == 4 || (kind == 0 && precision == DOCI_FP64);
  if (want_rowx && rowx_fits(h, elem)) return {4, 1};
  return {3, 1};
}

}  // namespace

SigmaPlan plan_sigma(const doci_ham *h, int precision, bool allow_pair) {
  int kind = h->sigma_kernel;
  if (precision == DOCI_FP64 && (kind == 6 || kind == 8)) kind = 0;  // FP32-only forms: the automatic FP64 path
  if (precision == DOCI_FP32 && kind == 9) kind = 0;                 // FP64-only form: the automatic FP32 path
  if (kind == 0) kind = tuned_choice(h, precision, 1, allow_pair);  // a tuned shape: its measured best
  return plan_kind(h, precision, allow_pair, kind);
}

// try_wait iterations per device wait of the tensor-core sigma; the
// environment variable DOCI_TC_SPIN_LIMIT (read once) lowers it, so that a
// test can make every wait run out and check the reported status
long tc_spin_limit() {
  static const long v = [] {
    const char *e = std::getenv("DOCI_TC_SPIN_LIMIT");
    return e ? std::strtol(e, nullptr, 10) : kTcSpinLimit;
  }();
  return v;
}

int launch_sigma(const doci_ham *h, const void *x, void *y, int precision, cudaStream_t st, bool allow_pair) {
  if (precision != DOCI_FP64 && precision != DOCI_FP32) return DOCI_ERR_INVALID;
  const bool f64 = precision == DOCI_FP64;
  const SigmaPlan p = plan_sigma(h, precision, allow_pair);
  switch (p.kind) {
    case 8:
      if ((reinterpret_cast<uintptr_t>(x) & 15u) == 0)
        return launch_tc(h, static_cast<const float *>(x), static_cast<float *>(y), st, h->d_tc_err, tc_spin_limit());
      // bulk copies need a 16-byte aligned x: the mma.sync pair form instead
      return pair_fits(h) ? launch_pair(h, static_cast<const float *>(x), static_cast<float *>(y), st)
                          : launch_row<float>(h, x, y, st, 1);
    case 6:
      return launch_pair(h, static_cast<const float *>(x), static_cast<float *>(y), st);
    case 1:
      return f64 ? launch_typed<double>(h, x, y, st) : launch_typed<float>(h, x, y, st);
    case 4:
      return f64 ? launch_rowx<double>(h, x, y, st, 1) : launch_rowx<float>(h, x, y, st, 1);
    case 9:
      // the pair form where it fits, else the phase-ordered row pass, both in float-float
      if (pair_ff_fits(h)) return launch_pair_ff(h, static_cast<const double *>(x), static_cast<double *>(y), st);
      return launch_rowx_ff(h, static_cast<const double *>(x), static_cast<double *>(y), st);
    default:  // 3
      return f64 ? launch_row<double>(h, x, y, st, 1) : launch_row<float>(h, x, y, st, 1);
  }
}

namespace {

// multi-vector methods
constexpr int kMultiRow = 1, kMultiGather = 2, kMultiSingle = 3;

int multi_row_group(const doci_ham *h, size_t elem) {
  // every vector's row staged in shared memory: the group is what fits
  // beside the static tables (at most 212 KB of rows), up to 4
  const size_t row_bytes = static_cast<size_t>((h->max_row + 3) & ~3) * elem;
  const int fit = static_cast<int>((212u * 1024u) / row_bytes);
  return !row_kernel_fits(h, elem) || fit < 2 ? 0 : fit < 4 ? fit : 4;
}

int multi_method_auto(const doci_ham *h, int precision) {
  const size_t elem = precision == DOCI_FP64 ? 8 : 4;
  // same choice of family as the single-vector dispatch
  const bool want_row = h->sigma_kernel >= 2 || (h->sigma_kernel == 0 && h->nrows >= device_sm_count());
  if (want_row && multi_row_group(h, elem) >= 2) return kMultiRow;
  if (!want_row || !row_kernel_fits(h, elem)) return kMultiGather;
  return kMultiSingle;
}

int run_multi(const doci_ham *h, int method, const void *x, size_t ldx, void *y, size_t ldy, int nv, int precision,
              cudaStream_t st) {
  const size_t elem = precision == DOCI_FP64 ? 8 : 4;
  const char *xc = static_cast<const char *>(x);
  char *yc = static_cast<char *>(y);
  if (method == kMultiRow) {
    const int group = multi_row_group(h, elem);
    if (group < 2) return DOCI_ERR_INVALID;
    for (int v0 = 0; v0 < nv; v0 += group) {
      const int k = nv - v0 < group ? nv - v0 : group;
      const void *xv = xc + v0 * ldx * elem;
      void *yv = yc + v0 * ldy * elem;
      const int r = k == 1 ? launch_sigma(h, xv, yv, precision, st, false)
                    : precision == DOCI_FP64 ? launch_row_multi<double>(h, xv, ldx, yv, ldy, k, st)
                                             : launch_row_multi<float>(h, xv, ldx, yv, ldy, k, st);
      if (r != DOCI_OK) return r;
    }
    return DOCI_OK;
  }
  if (method == kMultiGather)
    return precision == DOCI_FP64 ? launch_gather_multi_typed<double>(h, x, ldx, y, ldy, nv, st)
                                  : launch_gather_multi_typed<float>(h, x, ldx, y, ldy, nv, st);
  for (int v = 0; v < nv; ++v) {  // one vector at a time
    const int r = launch_sigma(h, xc + v * ldx * elem, yc + v * ldy * elem, precision, st, false);
    if (r) return r;
  }
  return DOCI_OK;
}

}  // namespace

int launch_sigma_multi(const doci_ham *h, const void *x, size_t ldx, void *y, size_t ldy, int nv, int precision,
                       cudaStream_t st) {
  if (nv < 1 || nv > 4 || ldx < h->D || ldy < h->D) return DOCI_ERR_INVALID;
  if (precision != DOCI_FP64 && precision != DOCI_FP32) return DOCI_ERR_INVALID;
  // the block solves stay run-to-run reproducible: no pair form here
  if (nv == 1) return launch_sigma(h, x, y, precision, st, false);
  int method = h->sigma_kernel == 0 ? tuned_choice(h, precision, nv, false) : 0;
  if (method == 0) method = multi_method_auto(h, precision);
  return run_multi(h, method, x, ldx, y, ldy, nv, precision, st);
}

int autotune_sigma(doci_ham *h, int precision, int nv, cudaStream_t st, int *choice) {
  if (nv < 1 || nv > 4 || (precision != DOCI_FP64 && precision != DOCI_FP32)) return DOCI_ERR_INVALID;
  const size_t elem = precision == DOCI_FP64 ? 8 : 4, D = h->D;
  void *buf = nullptr;
  DOCI_CUDA(cudaMallocAsync(&buf, 2 * D * nv * elem, st));
  char *x = static_cast<char *>(buf), *y = x + D * nv * elem;
  DOCI_CUDA(cudaMemsetAsync(x, 0, D * nv * elem, st));  // the timing does not depend on the values
  cudaEvent_t e0, e1;
  DOCI_CUDA(cudaEventCreate(&e0));
  DOCI_CUDA(cudaEventCreate(&e1));
  const int saved = h->sigma_kernel;
  doci_ham *hm = h;
  auto time_it = [&](auto &&run) -> double {
    if (run() != DOCI_OK) return 1e30;  // warm-up; a path that does not apply is skipped
    cudaEventRecord(e0, st);
    for (int r = 0; r < 2; ++r)
      if (run() != DOCI_OK) return 1e30;
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
  };
  int best = 0;
  if (nv == 1) {
    for (int allow = 0; allow < 2; ++allow) {
      double best_ms = 1e30;
      int pick = 0;
      for (int kind : {1, 3, 4, 6, 8, 9}) {
        if ((kind == 6 || kind == 8) && (!allow || precision != DOCI_FP32)) continue;
        if (kind == 9 && precision != DOCI_FP64) continue;
        hm->sigma_kernel = kind;
        const SigmaPlan p = plan_sigma(h, precision, allow != 0);
        if (p.kind != kind) continue;  // the path does not fit this shape
        const double ms = time_it([&] { return launch_sigma(h, x, y, precision, st, allow != 0); });
        if (ms < best_ms) {
          best_ms = ms;
          pick = kind;
        }
      }
      hm->sigma_kernel = saved;
      if (pick) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[tune_key(h, precision, 1, allow != 0)] = pick;
      }
      if (allow) best = pick;
    }
  } else {
    double best_ms = 1e30;
    hm->sigma_kernel = 0;
    for (int method : {kMultiRow, kMultiGather, kMultiSingle}) {
      if (method == kMultiRow && multi_row_group(h, elem) < 2) continue;
      const double ms = time_it([&] { return run_multi(h, method, x, D, y, D, nv, precision, st); });
      if (ms < best_ms) {
        best_ms = ms;
        best = method;
      }
    }
    hm->sigma_kernel = saved;
    if (best) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tuned[tune_key(h, precision, nv, false)] = best;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  DOCI_CUDA(cudaFreeAsync(buf, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  if (choice) *choice = best;
  return best ? DOCI_OK : DOCI_ERR_INVALID;
}

bool sigma_tuned(const doci_ham *h, int precision, int nv) { return tuned_choice(h, precision, nv, false) != 0; }

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
