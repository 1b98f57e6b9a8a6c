// sigma_pair.cu -- FP32 sigma in the (N-1)-pair intermediate form.
//
// Every off-diagonal element of the DOCI Hamiltonian is a pair hop
// T -> T \ i u a with weight K_ia = (ia|ia) (doci.c:216-222).  Writing
// S = T \ i (a set of N-1 pairs), the hop sum regroups as
//
//   sigma[T] = diag[T] x[T] + sum_{i in T} Y_{T \ i}[i],
//   Y_S[i]   = sum_a K_ia X_S[a],   X_S[a] = x[S u a] (0 when a in S),
//
// so each (N-1)-set S needs one gather of its L neighbours X_S, a dense
// L x L product with K (the tensor cores, 3xTF32 for FP32 accuracy), and one
// scatter-add of Y_S to the same L determinants S u i.  Per S that is
// L - N + 1 loads and adds instead of N (L - N) hops per determinant.
//
// Sets S are grouped by their row part R' (the mirrored orbitals
// [split, L) of the row tiling): the determinants S u a with a in the
// column part lie in row R' (one contiguous rank range, accumulated in
// shared memory and added to sigma once per block), those with a in the row
// part lie at the same column position of the rows R' u a (coalesced loads
// and atomic adds).  sigma is first set to diag * x; all hop contributions
// are atomic adds, so the FP32 summation order (and the last bits of the
// result) varies from run to run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "addressing.cuh"
#include "internal.h"

namespace doci {
namespace {

constexpr int kPairThreads = 256;
constexpr int kPairWarps = kPairThreads / 32;
constexpr int kTileStride = 36;  // floats per tile row: conflict-free fragment loads and float4 row access
constexpr uint32_t kNone = 0xffffffffu;

struct PairShape {
  uint32_t D;
  int L, N, split, na, nblocks;
};

struct PairSmem {
  uint32_t binom[kBinomRows * kBinomCols];
  uint4 kfrag[4 * 4 * 32];                   // [k step][n tile][lane]: {b0 hi, b1 hi, b0 lo, b1 lo}
  float tile[kPairWarps][32][kTileStride];   // per warp: X rows, then Y rows, one per thread
  uint32_t sup[32];                          // row bit b: start of row R' u b plus n_s - 1, or kNone
};

__device__ __forceinline__ uint32_t to_tf32(float f) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
  return r;
}

// D += A B, m16n8k8, A row-major 16 x 8 and B column-major 8 x 8 in TF32
__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void pair_init_kernel(uint32_t D, const float *__restrict__ diag, const float *__restrict__ x,
                                 float *__restrict__ y) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < D; t += gridDim.x * blockDim.x)
    y[t] = diag[t] * x[t];
}

__global__ void __launch_bounds__(kPairThreads, 2)
sigma_pair_kernel(PairShape s, const uint2 *__restrict__ blocks, const uint32_t *__restrict__ rowstart_of,
                  const uint32_t *__restrict__ g_binom, const uint4 *__restrict__ g_kfrag,
                  const float *__restrict__ x, float *__restrict__ y) {
  __shared__ __align__(16) PairSmem sm;
  extern __shared__ __align__(16) float acc[];  // own row: hop sums into row R'
  for (int t = threadIdx.x; t < kBinomRows * kBinomCols; t += blockDim.x) sm.binom[t] = g_binom[t];
  for (int t = threadIdx.x; t < 4 * 4 * 32; t += blockDim.x) sm.kfrag[t] = g_kfrag[t];
  const uint32_t *B = sm.binom;
  const int sp = s.split;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tq = lane & 3;
  float(*tile)[kTileStride] = sm.tile[warp];

  for (int blk = blockIdx.x; blk < s.nblocks; blk += gridDim.x) {
    const uint2 bw = blocks[blk];
    const uint32_t own = bw.x, mask = bw.y & 0xffffffu;
    const int kp = static_cast<int>(bw.y >> 24), jp = s.N - 1 - kp;
    __syncthreads();  // previous block's flush is done with acc and sup
    const uint32_t n_s = B[sp * kBinomCols + jp];
    const uint32_t n_own = jp + 1 <= sp ? B[sp * kBinomCols + jp + 1] : 0u;
    if (threadIdx.x < 32) {
      const int b = threadIdx.x;
      uint32_t v = kNone;
      if (b < s.na && !((mask >> b) & 1u)) v = rowstart_of[mask | (1u << b)] + n_s - 1u;
      sm.sup[b] = v;
    }
    for (uint32_t c = threadIdx.x; c < n_own; c += blockDim.x) acc[c] = 0.f;
    __syncthreads();
    const uint32_t own_last = own + n_own - 1u;

    for (uint32_t s0 = 0; s0 < n_s; s0 += kPairThreads) {
      if (s0 + 32u * warp >= n_s) break;  // this warp's rows are all past the block (warp-uniform)
      const uint32_t sidx = s0 + threadIdx.x;
      const bool live = sidx < n_s;
      const uint32_t Cm = live ? dev::colex_unrank<kBinomCols>(sidx, sp, jp, B) : 0u;
      // gather X_S into this thread's tile row
      {
        float xv[32];
#pragma unroll
        for (int o = 0; o < 32; ++o) xv[o] = 0.f;
        if (live)
          dev::pair_neighbours<kBinomCols>(sidx, Cm, jp, sp, s.L, B, sm.sup, [&](int o, int kind, uint32_t where) {
            xv[o] = __ldg(x + (kind == 0 ? own_last - where : where));
          });
#pragma unroll
        for (int q = 0; q < 8; ++q)
          *reinterpret_cast<float4 *>(&tile[lane][4 * q]) = make_float4(xv[4 * q], xv[4 * q + 1], xv[4 * q + 2], xv[4 * q + 3]);
      }
      __syncwarp();
      // Y = X K on the tensor cores: 3xTF32 (lo*hi + hi*lo + hi*hi)
      float c[2][4][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
          for (int e = 0; e < 4; ++e) c[mt][nt][e] = 0.f;
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        uint32_t ah[2][4], al[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int r0 = 16 * mt + g, c0 = 8 * kt + tq;
          const float f[4] = {tile[r0][c0], tile[r0 + 8][c0], tile[r0][c0 + 4], tile[r0 + 8][c0 + 4]};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            ah[mt][e] = to_tf32(f[e]);
            al[mt][e] = to_tf32(f[e] - __uint_as_float(ah[mt][e]));
          }
        }
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
          const uint4 b = sm.kfrag[(kt * 4 + nt) * 32 + lane];
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            mma_tf32(c[mt][nt], al[mt], b.x, b.y);
            mma_tf32(c[mt][nt], ah[mt], b.z, b.w);
            mma_tf32(c[mt][nt], ah[mt], b.x, b.y);
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
          const int r0 = 16 * mt + g, c0 = 8 * nt + 2 * tq;
          *reinterpret_cast<float2 *>(&tile[r0][c0]) = make_float2(c[mt][nt][0], c[mt][nt][1]);
          *reinterpret_cast<float2 *>(&tile[r0 + 8][c0]) = make_float2(c[mt][nt][2], c[mt][nt][3]);
        }
      __syncwarp();
      // scatter Y_S back to the same determinants
      if (live) {
        float yv[32];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float4 v = *reinterpret_cast<const float4 *>(&tile[lane][4 * q]);
          yv[4 * q] = v.x;
          yv[4 * q + 1] = v.y;
          yv[4 * q + 2] = v.z;
          yv[4 * q + 3] = v.w;
        }
        dev::pair_neighbours<kBinomCols>(sidx, Cm, jp, sp, s.L, B, sm.sup, [&](int o, int kind, uint32_t where) {
          if (kind == 0)
            atomicAdd(&acc[n_own - 1u - where], yv[o]);
          else
            atomicAdd(y + where, yv[o]);
        });
      }
      __syncwarp();  // the tile is rewritten by the next round's gather
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < n_own; c += blockDim.x) atomicAdd(y + own + c, acc[c]);
  }
}

float round_tf32(double v) {
  // nearest TF32 (10-bit mantissa), ties away from zero, as cvt.rna
  float f = static_cast<float>(v);
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u = (u + 0x1000u) & 0xffffe000u;
  std::memcpy(&f, &u, 4);
  return f;
}

}  // namespace

bool pair_fits(const doci_ham *h) {
  if (h->split < 1 || h->nrows < 1 || !h->d_pblocks || h->npblocks < 1) return false;
  if (h->L - h->split > 24) return false;
  return static_cast<size_t>(h->max_row) * sizeof(float) <= 100 * 1024;
}

int ham_build_pairs(doci_ham *h, const std::vector<uint32_t> &start) {
  const int L = h->L, N = h->N, sp = h->split, na = L - sp;
  // K in mma B-fragment order, split into TF32 high and low parts (from FP64)
  std::vector<uint32_t> kf(4 * 4 * 32 * 4);
  for (int kt = 0; kt < 4; ++kt)
    for (int nt = 0; nt < 4; ++nt)
      for (int lane = 0; lane < 32; ++lane) {
        const int gg = lane >> 2, t = lane & 3, i = 8 * nt + gg;
        const int a0 = 8 * kt + t, a1 = a0 + 4;
        auto K = [&](int a, int b) -> double {
          return a < L && b < L ? h->Kp[(L - 1 - a) * L + (L - 1 - b)] : 0.0;
        };
        const double k0 = K(a0, i), k1 = K(a1, i);
        const float h0 = round_tf32(k0), h1 = round_tf32(k1);
        const float l0 = round_tf32(k0 - h0), l1 = round_tf32(k1 - h1);
        uint32_t *e = &kf[((kt * 4 + nt) * 32 + lane) * 4];
        std::memcpy(e + 0, &h0, 4);
        std::memcpy(e + 1, &h1, 4);
        std::memcpy(e + 2, &l0, 4);
        std::memcpy(e + 3, &l1, 4);
      }
  // one block per row part R' of an (N-1)-set, largest first
  std::vector<std::pair<uint64_t, std::pair<uint32_t, uint32_t>>> bl;
  for (uint32_t mask = 0; mask < (1u << na); ++mask) {
    const int kp = __builtin_popcount(mask), jp = N - 1 - kp;
    if (jp < 0 || jp > sp) continue;
    const uint32_t own = jp + 1 <= sp ? start[mask] : kNone;
    bl.push_back({binom64(sp, jp), {own, mask | (static_cast<uint32_t>(kp) << 24)}});
  }
  std::stable_sort(bl.begin(), bl.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
  std::vector<uint32_t> flat;
  flat.reserve(bl.size() * 2);
  for (auto &e : bl) {
    flat.push_back(e.second.first);
    flat.push_back(e.second.second);
  }
  h->npblocks = static_cast<int>(bl.size());
  DOCI_CUDA(cudaMallocAsync(&h->d_kfrag, kf.size() * sizeof(uint32_t), h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_kfrag, kf.data(), kf.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  if (!flat.empty()) {
    DOCI_CUDA(cudaMallocAsync(&h->d_pblocks, flat.size() * sizeof(uint32_t), h->stream));
    DOCI_CUDA(cudaMemcpyAsync(h->d_pblocks, flat.data(), flat.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                              h->stream));
  }
  DOCI_CUDA(cudaStreamSynchronize(h->stream));
  return DOCI_OK;
}

int launch_pair(const doci_ham *h, const float *x, float *y, cudaStream_t st) {
  if (!pair_fits(h)) return DOCI_ERR_INVALID;
  const int sms = device_sm_count();
  {
    uint64_t grid = (static_cast<uint64_t>(h->D) + 255) / 256;
    const uint64_t cap = static_cast<uint64_t>(sms) * 8;
    if (grid > cap) grid = cap;
    pair_init_kernel<<<static_cast<unsigned>(grid), 256, 0, st>>>(h->D, h->d_diag32, x, y);
    DOCI_CUDA(cudaGetLastError());
  }
  const PairShape s{h->D, h->L, h->N, h->split, h->L - h->split, h->npblocks};
  const size_t dyn = static_cast<size_t>(h->max_row) * sizeof(float);
  int per_sm = 1;
  const int r = kernel_blocks(reinterpret_cast<const void *>(sigma_pair_kernel), kPairThreads, dyn, &per_sm);
  if (r != DOCI_OK) return r;
  int grid = sms * per_sm;
  if (grid > h->npblocks) grid = h->npblocks;
  sigma_pair_kernel<<<grid, kPairThreads, dyn, st>>>(s, reinterpret_cast<const uint2 *>(h->d_pblocks),
                                                     h->d_rowstart, h->d_binom,
                                                     reinterpret_cast<const uint4 *>(h->d_kfrag), x, y);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

}  // namespace doci
