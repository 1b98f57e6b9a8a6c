// sigma_pair.cu -- FP32 sigma in the (N-1)-pair intermediate form on the
// warp-level mma.sync path (kind 6, the automatic FP32 choice once the
// tiling gives every SM a unit), and the FP64-accurate float-float version
// of the same form (kind 9).  The tcgen05 version of the FP32 form is
// sigma_tc.cu (kind 8).
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
// column part lie in row R' (one contiguous rank range, random accesses and
// atomic adds within it), those with a in the row part lie at the same column
// position of the rows R' u a (coalesced loads and atomic adds).  sigma is first set to diag * x; all hop contributions
// are atomic adds, so the FP32 summation order (and the last bits of the
// result) varies from run to run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "addressing.cuh"
#include "ff.cuh"
#include "internal.h"

namespace doci {
namespace {

constexpr int kPairThreads = 256;
constexpr int kPairWarps = kPairThreads / 32;
constexpr uint32_t kNone = 0xffffffffu;
// tile[q][c] (orbital-major; set s of the warp's 32 at column
// c = 16 (s >> 4) + 2 (s & 7) + ((s >> 3) & 1), so the sets g and g + 8 of an
// m-tile, which one mma lane holds, are neighbours): the 8-byte mma fragment
// loads (bank 8t + 2g), the 8-byte result stores (output slots permuted, see
// the K fragments) and the same-orbital writes of a warp's 32 sets are free
// of bank conflicts
constexpr int kTileStride = 40;

struct PairShape {
  uint32_t D;
  int L, N, split, na, nblocks;
};

struct PairSmem {  // 49.4 KB of static shared memory
  uint4 kfrag[4 * 4 * 32];                   // this block's K, [k step][n tile][lane]: {b0 hi, b1 hi, b0 lo, b1 lo}
  float tile[kPairWarps][32][kTileStride];   // per warp: X_S then Y_S, column s = the warp's 32 sets
  uint32_t hole_rs[32];                      // row-part holes b of R': start of row R' u b
  int hole_o[32];                            // and their mirrored orbitals split + b
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

__device__ __forceinline__ uint32_t lane_of(const uint4 &v, int i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

__global__ void pair_init_kernel(uint32_t D, const float *__restrict__ diag, const float *__restrict__ x,
                                 float *__restrict__ y) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < D; t += gridDim.x * blockDim.x)
    y[t] = diag[t] * x[t];
}

// One block of sets S = (R', C') per iteration: C' runs over the jp-subsets
// of the column orbitals (column position c in a row of C(split, jp)
// columns).  The MMA's orbital axis is compacted to the column orbitals
// followed by the row-part holes of R' (the row-part elements of R' are in
// every S, so their X entries are zero).  Own-row sums by global atomics, one
// m-tile of the product at a time and the insertion entries re-read for the
// scatter (four 16-byte loads per set, quad-interleaved so that a warp's
// load covers 512 consecutive bytes), so that four blocks fit an SM
// (registers <= 64): 32 warps per SM hide the gathers' latency.
__global__ void __launch_bounds__(kPairThreads, 4)
sigma_pair_kernel(PairShape s, const uint2 *__restrict__ blocks, const uint32_t *__restrict__ rowstart_of,
                  const uint32_t *__restrict__ g_binom, const float *__restrict__ g_ksplit,
                  const uint32_t *__restrict__ ins_t, const uint32_t *__restrict__ ins_off,
                  const float *__restrict__ x, float *__restrict__ y) {
  __shared__ __align__(16) PairSmem sm;
  const uint32_t *B = g_binom;
  const int sp = s.split;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tq = lane & 3;
  float(*tile)[kTileStride] = sm.tile[warp];
  const int pc = 16 * (lane >> 4) + 2 * (lane & 7) + ((lane >> 3) & 1);  // this lane's set column
  {
    float4 *tz = reinterpret_cast<float4 *>(&tile[0][0]);
    for (int z = lane; z < 32 * kTileStride / 4; z += 32) tz[z] = make_float4(0.f, 0.f, 0.f, 0.f);
  }

  for (int blk = blockIdx.x; blk < s.nblocks; blk += gridDim.x) {
    const uint2 bw = blocks[blk];
    const uint32_t own = bw.x, mask = bw.y & 0xffffffu;
    const int kp = static_cast<int>(bw.y >> 24), jp = s.N - 1 - kp;
    const int nhr = s.na - kp, keff = sp + nhr, nk = (keff + 7) >> 3, nch = sp - jp;
    __syncthreads();  // the previous block is done with the holes and fragments
    const uint32_t n_s = __ldg(B + sp * kBinomCols + jp);
    if (warp == 0) {
      const bool hole = lane < s.na && !((mask >> lane) & 1u);
      const uint32_t hb = __ballot_sync(0xffffffffu, hole);
      if (hole) {
        const int h = __popc(hb & ((1u << lane) - 1u));
        sm.hole_rs[h] = rowstart_of[mask | (1u << lane)];
        sm.hole_o[h] = sp + lane;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 4 * 4 * 32; e += blockDim.x) {
      const int kt = e >> 7, nt = (e >> 5) & 3, ln = e & 31;
      // product column j of n tile nt is output slot 8 nt + (j >> 1) + 4 (j & 1):
      // a lane's two result columns 2t, 2t + 1 land in slot rows t and t + 4,
      // which keeps the result stores free of bank conflicts
      const int a0 = 8 * kt + (ln & 3), a1 = a0 + 4, j = ln >> 2, i = 8 * nt + (j >> 1) + 4 * (j & 1);
      auto orb = [&](int col) { return col < sp ? col : col < keff ? sm.hole_o[col - sp] : -1; };
      const int o0 = orb(a0), o1 = orb(a1), oi = orb(i);
      const bool v0 = o0 >= 0 && oi >= 0, v1 = o1 >= 0 && oi >= 0;
      const float *khi = g_ksplit, *klo = g_ksplit + 32 * 32;
      sm.kfrag[e] = make_uint4(v0 ? __float_as_uint(__ldg(khi + o0 * 32 + oi)) : 0u,
                               v1 ? __float_as_uint(__ldg(khi + o1 * 32 + oi)) : 0u,
                               v0 ? __float_as_uint(__ldg(klo + o0 * 32 + oi)) : 0u,
                               v1 ? __float_as_uint(__ldg(klo + o1 * 32 + oi)) : 0u);
    }
    __syncthreads();
    const uint32_t *ins_blk = ins_t + ins_off[jp];

    for (uint32_t s0 = 0; s0 < n_s; s0 += kPairThreads) {
      if (s0 + 32u * warp >= n_s) break;  // this warp's sets are all past the block (warp-uniform)
      const uint32_t c = s0 + threadIdx.x;
      const bool live = c < n_s;
      {
        // X_S is zero on the column orbitals in S: clear the column-part rows
        // (the row-part rows are written for every live set; rows past the
        // block's orbitals meet zero K rows and only need to be finite, which
        // the clear at kernel start and the later Y values are)
        float4 *tz = reinterpret_cast<float4 *>(&tile[0][0]);
        for (int z = lane; z < sp * (kTileStride / 4); z += 32) tz[z] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      __syncwarp();
      // gather X_S: column holes of C' (row R', positions from the insertion
      // table) and the row-part holes of R' (rows R' u b, column c)
      uint4 ent[4];
      if (live) {
        const uint4 *ip = reinterpret_cast<const uint4 *>(ins_blk);
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (4 * u < nch) ent[u] = __ldg(ip + (c + u * n_s));
#pragma unroll
        for (int h = 0; h < 16; ++h)
          if (h < nch) {
            const uint32_t e = lane_of(ent[h >> 2], h & 3);
            tile[e & 0xffu][pc] = __ldg(x + own + (e >> 8));
          }
        for (int h = 0; h < nhr; ++h) tile[sp + h][pc] = __ldg(x + sm.hole_rs[h] + c);
      }
      __syncwarp();
      // Y = X K on the tensor cores: 3xTF32 (lo*hi + hi*lo + hi*hi)
      {
        // one m-tile (16 sets) at a time: its columns of the tile are disjoint
        // from the other m-tile's, so its Y may overwrite its X at once
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          float cc[4][4];
#pragma unroll
          for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) cc[nt][e] = 0.f;
          const int r0 = 16 * mt + 2 * g;  // columns of the sets 16 mt + g and 16 mt + g + 8
#pragma unroll
          for (int kt = 0; kt < 4; ++kt) {
            if (kt < nk) {
              uint32_t ah[4], al[4];
              const int k0 = 8 * kt + tq;
              const float2 p0 = *reinterpret_cast<const float2 *>(&tile[k0][r0]);
              const float2 p1 = *reinterpret_cast<const float2 *>(&tile[k0 + 4][r0]);
              const float f[4] = {p0.x, p0.y, p1.x, p1.y};
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                ah[e] = to_tf32(f[e]);
                al[e] = to_tf32(f[e] - __uint_as_float(ah[e]));
              }
#pragma unroll
              for (int nt = 0; nt < 4; ++nt)
                if (nt < nk) {
                  const uint4 b = sm.kfrag[(kt * 4 + nt) * 32 + lane];
                  mma_tf32(cc[nt], al, b.x, b.y);
                  mma_tf32(cc[nt], ah, b.z, b.w);
                  mma_tf32(cc[nt], ah, b.x, b.y);
                }
            }
          }
          __syncwarp();
#pragma unroll
          for (int nt = 0; nt < 4; ++nt)
            if (nt < nk) {
              const int q0 = 8 * nt + tq;  // columns 2t, 2t + 1 are slots t, t + 4
              *reinterpret_cast<float2 *>(&tile[q0][r0]) = make_float2(cc[nt][0], cc[nt][2]);
              *reinterpret_cast<float2 *>(&tile[q0 + 4][r0]) = make_float2(cc[nt][1], cc[nt][3]);
            }
        }
      }
      __syncwarp();
      // scatter Y_S back to the same determinants
      if (live) {
        {
          const uint4 *ip = reinterpret_cast<const uint4 *>(ins_blk);
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (4 * u < nch) ent[u] = __ldg(ip + (c + u * n_s));
        }
#pragma unroll
        for (int h = 0; h < 16; ++h)
          if (h < nch) {
            const uint32_t e = lane_of(ent[h >> 2], h & 3);
            atomicAdd(y + own + (e >> 8), tile[e & 0xffu][pc]);
          }
        for (int h = 0; h < nhr; ++h) atomicAdd(y + sm.hole_rs[h] + c, tile[sp + h][pc]);
      }
      __syncwarp();  // the tile is cleared by the next round
    }
  }
}

// ---------------------------------------------------------------------------
// FP64-accurate pair form in float-float arithmetic (kind 9).  Same blocks
// and neighbour tables as the kernel above; per set (one per thread) the
// L - N + 1 open slots (the column-part holes of C', from the insertion
// table, then the row-part holes of R') hold X_S, and every output
// Y_S[i] = sum_a K_ia X_S[a] over the open slots is formed in float-float
// (ff.cuh: about 48 significant bits) from x pre-converted to float-float,
// converted to double once and added to sigma with an FP64 atomic add
// (sigma starts as diag * x in FP64).  GB300's FP64 units run at a small
// fraction of its FP32 rate: the products and sums go to the FP32 units.
template <int NO>
__global__ void __launch_bounds__(kPairThreads, 2)
sigma_pair_ff_kernel(PairShape s, const uint2 *__restrict__ blocks, const uint32_t *__restrict__ rowstart_of,
                     const uint32_t *__restrict__ g_binom, const double *__restrict__ g_K,
                     const uint32_t *__restrict__ ins_t, const uint32_t *__restrict__ ins_off, const ff *__restrict__ x,
                     double *__restrict__ y) {
  __shared__ ff Kc[32 * 32];  // K on the block's slots: [output slot][input slot]
  __shared__ uint32_t hole_rs[32];
  __shared__ int hole_o[32];
  const uint32_t *B = g_binom;
  const int sp = s.split, lane = threadIdx.x & 31;
  for (int blk = blockIdx.x; blk < s.nblocks; blk += gridDim.x) {
    const uint2 bw = blocks[blk];
    const uint32_t own = bw.x, mask = bw.y & 0xffffffu;
    const int kp = static_cast<int>(bw.y >> 24), jp = s.N - 1 - kp;
    const int nhr = s.na - kp, keff = sp + nhr, nch = sp - jp, nopen = nch + nhr;
    __syncthreads();  // the previous block is done with the tables
    if (threadIdx.x < 32) {
      const bool hole = lane < s.na && !((mask >> lane) & 1u);
      const uint32_t hb = __ballot_sync(0xffffffffu, hole);
      if (hole) {
        const int h = __popc(hb & ((1u << lane) - 1u));
        hole_rs[h] = rowstart_of[mask | (1u << lane)];
        hole_o[h] = sp + lane;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
      const int i = e >> 5, a = e & 31;
      const int oi = i < sp ? i : i < keff ? hole_o[i - sp] : -1;
      const int oa = a < sp ? a : a < keff ? hole_o[a - sp] : -1;
      Kc[e] = (oi >= 0 && oa >= 0) ? ff_from(g_K[oi * 32 + oa]) : ff(0);
    }
    __syncthreads();
    const uint32_t n_s = __ldg(B + sp * kBinomCols + jp);
    const uint32_t *ins_blk = ins_t + ins_off[jp];
    for (uint32_t c = threadIdx.x; c < n_s; c += blockDim.x) {
      ff X[NO];
      uint32_t tgt[NO];
      int slot[NO];
#pragma unroll
      for (int t = 0; t < NO; ++t) {
        if (t < nch) {
          const uint32_t e = __ldg(ins_blk + 4 * ((t >> 2) * n_s + c) + (t & 3));
          slot[t] = static_cast<int>(e & 0xffu);
          tgt[t] = own + (e >> 8);
        } else if (t < nopen) {
          slot[t] = sp + (t - nch);
          tgt[t] = hole_rs[t - nch] + c;
        } else {
          slot[t] = 0;
          tgt[t] = 0;
        }
        X[t] = t < nopen ? ldg_val(x + tgt[t]) : ff(0);
      }
#pragma unroll
      for (int to = 0; to < NO; ++to) {
        if (to < nopen) {
          const ff *Krow = Kc + slot[to] * 32;
          ff acc(0);
#pragma unroll
          for (int ti = 0; ti < NO; ++ti)  // K_ii = 0: the diagonal term is skipped (same sum, bit for bit)
            if (ti < nopen && ti != to) acc += Krow[slot[ti]] * X[ti];
          atomicAdd(y + tgt[to], ff_to(acc));
        }
      }
    }
  }
}

__global__ void pair_init64_kernel(uint32_t D, const double *__restrict__ diag, const double *__restrict__ x,
                                   double *__restrict__ y, ff *__restrict__ xf) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < D; t += gridDim.x * blockDim.x) {
    const double v = x[t];
    y[t] = diag[t] * v;
    xf[t] = ff_from(v);
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
  if (h->split < 1 || h->split > 16 || h->nrows < 1 || !h->d_pblocks || h->npblocks < 1) return false;
  if (!h->d_ins || !h->d_ins_t || !h->d_tab_off) return false;
  if (h->L - h->split > 24) return false;
  return static_cast<size_t>(h->max_row) * sizeof(float) <= 100 * 1024;
}

int ham_build_pairs(doci_ham *h, const std::vector<uint32_t> &start) {
  const int L = h->L, N = h->N, sp = h->split, na = L - sp;
  // K (mirrored orbitals, zero outside 0..L-1) split into TF32 high and low
  // parts from the FP64 values: [hi 32 x 32 | lo 32 x 32]
  std::vector<float> ks(2 * 32 * 32, 0.f);
  for (int a = 0; a < L; ++a)
    for (int b = 0; b < L; ++b) {
      const double k = h->Kp[(L - 1 - a) * L + (L - 1 - b)];
      const float hi = round_tf32(k);
      ks[a * 32 + b] = hi;
      ks[32 * 32 + a * 32 + b] = round_tf32(k - hi);
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
  // host-buffer path: pieces of the vector, units by the pieces their rows
  // reach, the group schedule and its launch steps (host_plan.h)
  hostplan::pieces(h->D, h->chunk_off);
  std::vector<hostplan::Unit> hu;
  hu.reserve(bl.size());
  for (auto &e : bl) {
    const uint32_t mask = e.second.second & 0xffffffu;
    const int kp = static_cast<int>(e.second.second >> 24), jp = N - 1 - kp;
    uint32_t touched = 0;
    if (e.second.first != kNone) touched |= hostplan::row_pieces(h->chunk_off, e.second.first, binom64(sp, jp + 1));
    for (int b = 0; b < na; ++b)
      if (!(mask >> b & 1u)) touched |= hostplan::row_pieces(h->chunk_off, start[mask | (1u << b)], binom64(sp, jp));
    hu.push_back({e.second.first, e.second.second, binom64(sp, jp), touched});
  }
  std::vector<uint32_t> flat_host;
  hostplan::schedule(hu, h->D, h->host_groups, flat_host);
  h->host_steps = hostplan::steps(h->host_groups);
  DOCI_CUDA(cudaMallocAsync(&h->d_kfrag, ks.size() * sizeof(float), h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_kfrag, ks.data(), ks.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  if (!flat.empty()) {
    DOCI_CUDA(cudaMallocAsync(&h->d_pblocks, flat.size() * sizeof(uint32_t), h->stream));
    DOCI_CUDA(cudaMemcpyAsync(h->d_pblocks, flat.data(), flat.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                              h->stream));
    DOCI_CUDA(cudaMallocAsync(&h->d_pblocks_host, flat_host.size() * sizeof(uint32_t), h->stream));
    DOCI_CUDA(cudaMemcpyAsync(h->d_pblocks_host, flat_host.data(), flat_host.size() * sizeof(uint32_t),
                              cudaMemcpyHostToDevice, h->stream));
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
  int per_sm = 1;
  const int r = kernel_blocks(reinterpret_cast<const void *>(sigma_pair_kernel), kPairThreads, 0, &per_sm);
  if (r != DOCI_OK) return r;
  int grid = sms * per_sm;
  if (grid > h->npblocks) grid = h->npblocks;
  sigma_pair_kernel<<<grid, kPairThreads, 0, st>>>(s, reinterpret_cast<const uint2 *>(h->d_pblocks), h->d_rowstart,
                                                   h->d_binom, reinterpret_cast<const float *>(h->d_kfrag), h->d_ins_t,
                                                   h->d_tab_off, x, y);
  DOCI_CUDA(cudaGetLastError());
  return DOCI_OK;
}

namespace {

// One host-buffer sigma on the plan of host_plan.h (h->host_steps): the
// pieces of hx go up in order on the copy stream; per step, on its compute
// stream (the handle's stream st or the side stream), the wait for its last
// piece, init(a, n, stream) for the diagonal passes it runs first (each
// followed by the piece's init event), the waits for diagonal passes run on
// the other stream, group(first, count, stream) for its units and the
// group's event; with hy, the pieces final after the step go down on the
// copy stream.  st waits for the side stream and the downloads at the end.
template <typename T, typename Init, typename Group>
int run_host_schedule(doci_ham *h, const T *hx, T *dx, T *dy, T *hy, cudaStream_t st, Init init, Group group) {
  constexpr int NC = doci_ham::kHostChunks;
  const int ng = static_cast<int>(h->host_steps.size());
  if (!h->copy_stream) {
    DOCI_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    DOCI_CUDA(cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking));
    for (auto &e : h->up_ev) DOCI_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : h->init_ev) DOCI_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    DOCI_CUDA(cudaEventCreateWithFlags(&h->start_ev, cudaEventDisableTiming));
    DOCI_CUDA(cudaEventCreateWithFlags(&h->end_ev, cudaEventDisableTiming));
    DOCI_CUDA(cudaEventCreateWithFlags(&h->side_ev, cudaEventDisableTiming));
  }
  while (static_cast<int>(h->group_ev.size()) < ng) {
    cudaEvent_t e = nullptr;
    DOCI_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->group_ev.push_back(e);
  }
  cudaStream_t cs = h->copy_stream;
  cudaStream_t run[2] = {st, h->side_stream};
  // everything starts after the stream's earlier work (dx may still be read)
  DOCI_CUDA(cudaEventRecord(h->start_ev, st));
  DOCI_CUDA(cudaStreamWaitEvent(cs, h->start_ev, 0));
  DOCI_CUDA(cudaStreamWaitEvent(run[1], h->start_ev, 0));
  for (int k = 0; k < NC; ++k) {
    const uint64_t a = h->chunk_off[k], n = h->chunk_off[k + 1] - a;
    if (n) DOCI_CUDA(cudaMemcpyAsync(dx + a, hx + a, n * sizeof(T), cudaMemcpyHostToDevice, cs));
    DOCI_CUDA(cudaEventRecord(h->up_ev[k], cs));
  }
  for (int gi = 0; gi < ng; ++gi) {
    const hostplan::Step &p = h->host_steps[gi];
    const hostplan::Group &g = h->host_groups[gi];
    cudaStream_t s = run[p.stream];
    if (p.wait_up >= 0) DOCI_CUDA(cudaStreamWaitEvent(s, h->up_ev[p.wait_up], 0));
    for (int k = 0; k < NC; ++k) {
      if (!(p.init >> k & 1u)) continue;
      const uint64_t a = h->chunk_off[k], n = h->chunk_off[k + 1] - a;
      if (n) {
        const int rc = init(a, n, s);
        if (rc != DOCI_OK) return rc;
      }
      DOCI_CUDA(cudaEventRecord(h->init_ev[k], s));
    }
    for (int k = 0; k < NC; ++k)
      if (p.wait_init >> k & 1u) DOCI_CUDA(cudaStreamWaitEvent(s, h->init_ev[k], 0));
    if (g.count > 0) {
      const int rc = group(g.first, g.count, s);
      if (rc != DOCI_OK) return rc;
    }
    DOCI_CUDA(cudaEventRecord(h->group_ev[gi], s));
    if (!hy) continue;
    for (const hostplan::Down &d : p.down) {
      const uint64_t a = h->chunk_off[d.piece], n = h->chunk_off[d.piece + 1] - a;
      DOCI_CUDA(cudaStreamWaitEvent(cs, h->group_ev[gi], 0));
      if (d.other_group >= 0) DOCI_CUDA(cudaStreamWaitEvent(cs, h->group_ev[d.other_group], 0));
      if (d.wait_init) DOCI_CUDA(cudaStreamWaitEvent(cs, h->init_ev[d.piece], 0));
      if (n) DOCI_CUDA(cudaMemcpyAsync(hy + a, dy + a, n * sizeof(T), cudaMemcpyDeviceToHost, cs));
    }
  }
  DOCI_CUDA(cudaEventRecord(h->side_ev, run[1]));
  DOCI_CUDA(cudaStreamWaitEvent(st, h->side_ev, 0));
  if (hy) {
    DOCI_CUDA(cudaEventRecord(h->end_ev, cs));
    DOCI_CUDA(cudaStreamWaitEvent(st, h->end_ev, 0));
  }
  return DOCI_OK;
}

unsigned init_grid(uint64_t n) {
  const uint64_t cap = static_cast<uint64_t>(device_sm_count()) * 8;
  return static_cast<unsigned>(std::min((n + 255) / 256, cap));
}

template <int NO>
int launch_pair_ff_host_no(doci_ham *h, const double *hx, double *dx, double *dy, double *hy, cudaStream_t st) {
  int per_sm = 1;
  int r = kernel_blocks(reinterpret_cast<const void *>(sigma_pair_ff_kernel<NO>), kPairThreads, 0, &per_sm);
  if (r != DOCI_OK) return r;
  const int slots = device_sm_count() * per_sm;
  ff *xf = nullptr;
  DOCI_CUDA(cudaMallocAsync(&xf, sizeof(ff) * static_cast<size_t>(h->D), st));
  const uint2 *blocks = reinterpret_cast<const uint2 *>(h->d_pblocks_host);
  r = run_host_schedule<double>(
      h, hx, dx, dy, hy, st,
      [&](uint64_t a, uint64_t n, cudaStream_t s) {
        pair_init64_kernel<<<init_grid(n), 256, 0, s>>>(static_cast<uint32_t>(n), h->d_diag + a, dx + a, dy + a,
                                                         xf + a);
        DOCI_CUDA(cudaGetLastError());
        return static_cast<int>(DOCI_OK);
      },
      [&](int first, int count, cudaStream_t s) {
        const PairShape ps{h->D, h->L, h->N, h->split, h->L - h->split, count};
        sigma_pair_ff_kernel<NO><<<std::min(slots, count), kPairThreads, 0, s>>>(
            ps, blocks + first, h->d_rowstart, h->d_binom, h->d_Kmir64, h->d_ins_t, h->d_tab_off, xf, dy);
        DOCI_CUDA(cudaGetLastError());
        return static_cast<int>(DOCI_OK);
      });
  // the side stream's groups read xf: st is ordered after them (the
  // schedule's own join is skipped when it returns early with an error)
  if (r != DOCI_OK && h->side_stream) {
    cudaEventRecord(h->side_ev, h->side_stream);
    cudaStreamWaitEvent(st, h->side_ev, 0);
  }
  const cudaError_t ef = cudaFreeAsync(xf, st);
  if (r != DOCI_OK) return r;
  DOCI_CUDA(ef);
  return DOCI_OK;
}

}  // namespace

int launch_pair_host(doci_ham *h, const float *hx, float *dx, float *dy, float *hy, cudaStream_t st) {
  if (!pair_fits(h) || !h->d_pblocks_host || h->host_steps.empty()) return DOCI_ERR_INVALID;
  int per_sm = 1;
  const int r = kernel_blocks(reinterpret_cast<const void *>(sigma_pair_kernel), kPairThreads, 0, &per_sm);
  if (r != DOCI_OK) return r;
  const int slots = device_sm_count() * per_sm;
  const uint2 *blocks = reinterpret_cast<const uint2 *>(h->d_pblocks_host);
  return run_host_schedule<float>(
      h, hx, dx, dy, hy, st,
      [&](uint64_t a, uint64_t n, cudaStream_t s) {
        pair_init_kernel<<<init_grid(n), 256, 0, s>>>(static_cast<uint32_t>(n), h->d_diag32 + a, dx + a, dy + a);
        DOCI_CUDA(cudaGetLastError());
        return static_cast<int>(DOCI_OK);
      },
      [&](int first, int count, cudaStream_t s) {
        const PairShape ps{h->D, h->L, h->N, h->split, h->L - h->split, count};
        sigma_pair_kernel<<<std::min(slots, count), kPairThreads, 0, s>>>(
            ps, blocks + first, h->d_rowstart, h->d_binom, reinterpret_cast<const float *>(h->d_kfrag), h->d_ins_t,
            h->d_tab_off, dx, dy);
        DOCI_CUDA(cudaGetLastError());
        return static_cast<int>(DOCI_OK);
      });
}

int launch_pair_ff_host(doci_ham *h, const double *hx, double *dx, double *dy, double *hy, cudaStream_t st) {
  if (!pair_ff_fits(h) || !h->d_pblocks_host || h->host_steps.empty()) return DOCI_ERR_INVALID;
  const int no = h->L - h->N + 1;
  if (no <= 8) return launch_pair_ff_host_no<8>(h, hx, dx, dy, hy, st);
  if (no <= 17) return launch_pair_ff_host_no<17>(h, hx, dx, dy, hy, st);
  if (no <= 24) return launch_pair_ff_host_no<24>(h, hx, dx, dy, hy, st);
  return launch_pair_ff_host_no<32>(h, hx, dx, dy, hy, st);
}

bool pair_ff_fits(const doci_ham *h) { return pair_fits(h) && h->L - h->N + 1 <= 32; }

// open slots per set: L - N + 1
template <int NO>
int launch_pair_ff_no(const doci_ham *h, const double *x, double *y, cudaStream_t st) {
  const int sms = device_sm_count();
  ff *xf = nullptr;
  DOCI_CUDA(cudaMallocAsync(&xf, sizeof(ff) * static_cast<size_t>(h->D), st));
  {
    uint64_t grid = (static_cast<uint64_t>(h->D) + 255) / 256;
    const uint64_t cap = static_cast<uint64_t>(sms) * 8;
    if (grid > cap) grid = cap;
    pair_init64_kernel<<<static_cast<unsigned>(grid), 256, 0, st>>>(h->D, h->d_diag, x, y, xf);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    const PairShape s{h->D, h->L, h->N, h->split, h->L - h->split, h->npblocks};
    int per_sm = 1;
    const int r = kernel_blocks(reinterpret_cast<const void *>(sigma_pair_ff_kernel<NO>), kPairThreads, 0, &per_sm);
    if (r != DOCI_OK) {
      cudaFreeAsync(xf, st);
      return r;
    }
    int grid = sms * per_sm;
    if (grid > h->npblocks) grid = h->npblocks;
    sigma_pair_ff_kernel<NO><<<grid, kPairThreads, 0, st>>>(s, reinterpret_cast<const uint2 *>(h->d_pblocks),
                                                            h->d_rowstart, h->d_binom, h->d_Kmir64, h->d_ins_t,
                                                            h->d_tab_off, xf, y);
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(xf, st);
  DOCI_CUDA(e);
  DOCI_CUDA(ef);
  return DOCI_OK;
}

int launch_pair_ff(const doci_ham *h, const double *x, double *y, cudaStream_t st) {
  if (!pair_ff_fits(h)) return DOCI_ERR_INVALID;
  const int no = h->L - h->N + 1;
  if (no <= 8) return launch_pair_ff_no<8>(h, x, y, st);
  if (no <= 17) return launch_pair_ff_no<17>(h, x, y, st);
  if (no <= 24) return launch_pair_ff_no<24>(h, x, y, st);
  return launch_pair_ff_no<32>(h, x, y, st);
}

}  // namespace doci
