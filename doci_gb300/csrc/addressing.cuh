// addressing.cuh -- lexical determinant addressing on the device.
//
// The reference orders the C(L, N) determinants lexicographically by their
// sorted occupation lists (doci.c:472-548; the last pair is advanced first)
// and addresses them through the differenced string-graph weights Y
// (doci.c:384-434).  The same order has a closed form: with c_0 < ... < c_{N-1}
// the occupied orbitals,
//     rank(T) = D - 1 - sum_e C(L-1-c_e, N-e).
// Mirroring the orbitals (d = L-1-c) turns the sum into the combinatorial
// number system ("colex rank") of the mirrored set M = {d_j ascending}:
//     colex(M) = sum_j C(d_j, j+1),       rank(T) = D - 1 - colex(M).
// In the mirrored picture the determinant's bits are brev(bits) >> (32 - L).
//
// Neighbour ranks.  For T' = T \ i u a (pair hop i -> a) let m_k be the
// mirrored occupied orbital removed and q the mirrored hole filled.  With the
// prefix sums over M of W_j = C(m_j, j+1), U_j = C(m_j, j), V_j = C(m_j, j+2)
// and b = number of elements of M below q:
//   q < m_k: colex(T') = [PW(b) - PV(b) + C(q, b+1)] + [PV(k) + R - PW(k+1)]
//   q > m_k: colex(T') = [PU(b) + R - PW(b) + C(q, b)] + [PW(k) - PU(k+1)]
// where R = colex(M).  The first bracket depends only on the hole (E1/E2
// below), the second only on the removed element (c1/c2): every one of the
// N(L-N) neighbour ranks costs one compare and one add, the job the
// reference's incremental Y-walk does in prev_bitstring (doci.c:851-978).
#pragma once

#include <cstdint>
#include <vector>

namespace doci {
namespace dev {

#ifdef __CUDA_ARCH__
#define DOCI_HD __host__ __device__ __forceinline__
__device__ __forceinline__ int ffs32(uint32_t v) { return __ffs(static_cast<int>(v)); }
#else
#define DOCI_HD __host__ __device__ inline
inline int ffs32(uint32_t v) { return __builtin_ffs(static_cast<int>(v)); }
#endif

__host__ __device__ __forceinline__ uint32_t low_mask(int L) {
  return L >= 32 ? 0xffffffffu : ((1u << L) - 1u);
}

// colex unrank: the N-subset of {0..L-1} (mirrored orbitals) with colex rank R
template <int BC>
DOCI_HD uint32_t colex_unrank(uint32_t R, int L, int N, const uint32_t *binom) {
  uint32_t M = 0;
  int d = L - 1;
  for (int j = N; j >= 1; --j) {
    while (binom[d * BC + j] > R) --d;
    R -= binom[d * BC + j];
    M |= 1u << d;
    --d;
  }
  return M;
}

template <int BC>
DOCI_HD uint32_t colex_rank(uint32_t M, const uint32_t *binom) {
  uint32_t s = 0;
  int j = 0;
  while (M) {
    const int d = ffs32(M) - 1;
    M &= M - 1;
    s += binom[d * BC + j + 1];
    ++j;
  }
  return s;
}

DOCI_HD uint32_t mirror_bits(uint32_t bits, int L) {
#ifdef __CUDA_ARCH__
  return __brev(bits) >> (32 - L);
#else
  uint32_t r = 0;
  for (int o = 0; o < L; ++o)
    if (bits >> o & 1u) r |= 1u << (L - 1 - o);
  return r;
#endif
}

// Neighbour enumeration of one determinant (rank r, colex R = D-1-r, mirrored
// occupation M).  Precompute() fills the per-hole terms; then for every
// occupied element k (ascending mirrored orbital m) and hole h (ascending q),
// visit(m, q, rank(T')) is called.  Shared by the sigma kernels and by the
// host-side index check.
template <int NH, int BC>
struct Neighbours {
  uint32_t E1[NH], E2[NH];
  int Q[NH];
  DOCI_HD void precompute(uint32_t M, uint32_t R, int L, int nh, const uint32_t *B) {
    uint32_t holes = ~M & low_mask(L), mrem = M, PW = 0, PU = 0, PV = 0;
    int j = 0;
#pragma unroll
    for (int h = 0; h < NH; ++h) {
      if (h < nh) {
        const int q = ffs32(holes) - 1;
        holes &= holes - 1;
        while (mrem && (ffs32(mrem) - 1) < q) {
          const int m = ffs32(mrem) - 1;
          mrem &= mrem - 1;
          PW += B[m * BC + j + 1];
          PU += B[m * BC + j];
          PV += B[m * BC + j + 2];
          ++j;
        }
        // j == q - h elements of M lie below q
        E1[h] = PW - PV + B[q * BC + j + 1];
        E2[h] = PU + R - PW + B[q * BC + j];
        Q[h] = q;
      } else {
        E1[h] = E2[h] = 0;
        Q[h] = 0;
      }
    }
  }
  template <typename F>
  DOCI_HD void visit(uint32_t M, uint32_t R, uint32_t Dm1, int N, int nh, const uint32_t *B, F &&f) const {
    uint32_t mrem = M, PW = 0, PU = 0, PV = 0;
    for (int k = 0; k < N; ++k) {
      const int m = ffs32(mrem) - 1;
      mrem &= mrem - 1;
      const uint32_t W = B[m * BC + k + 1], U = B[m * BC + k], V = B[m * BC + k + 2];
      // rank(T') = D-1 - (E + c)
      const uint32_t base1 = Dm1 - (PV + R - (PW + W));
      const uint32_t base2 = Dm1 - (PW - (PU + U));
      f.begin(m);
#pragma unroll
      for (int h = 0; h < NH; ++h) {
        if (h < nh) f.hop(m, Q[h], Q[h] < m ? base1 - E1[h] : base2 - E2[h]);
      }
      PW += W;
      PU += U;
      PV += V;
    }
  }
};

// One column of a row in the row-tiled sigma (mirrored orbitals [0, sp) =
// column part, [sp, L) = row part).  The row has row-part occupation R with
// j = N - |R| elements left for the column part, n = C(sp, j) columns;
// column c holds the column-part set of colex n-1-c.  Calls
//   f.inrow(m, q, c')      hop m -> q inside the column part: column c' of this row
//   f.up(t, m, q, c')      hop of row-part element ab_m[t] = m to column-part hole q:
//                          column c' of row R \ m (start ab_rs[t])
//   f.down(t, m, q, c')    hop of column-part element m to row-part hole ba_q[t] = q:
//                          column c' of row R u q
//   f.across(t, c)         row-part hop t (table entry): same column c of another row
template <int NHB, int BC, typename F>
DOCI_HD void row_column_hops(uint32_t c, uint32_t n, int sp, int j, const uint32_t *B, int n_ab, const int *ab_m,
                             int n_ba, const int *ba_q, int n_aa, F &f) {
  const uint32_t p = n - 1 - c;
  const uint32_t Mb = colex_unrank<BC>(p, sp, j, B);
  Neighbours<NHB, BC> nb;
  nb.precompute(Mb, p, sp, sp - j, B);
  const int nhB = sp - j;
  const uint32_t n_up_m1 = (j < sp ? B[sp * BC + j + 1] : 1u) - 1u;
  const uint32_t n_dn_m1 = (j > 0 ? B[sp * BC + j - 1] : 1u) - 1u;
  uint32_t PVtot = 0, PUtot = 0;
  {
    uint32_t mr = Mb;
    for (int i = 0; i < j; ++i) {
      const int m = ffs32(mr) - 1;
      mr &= mr - 1;
      PVtot += B[m * BC + i + 2];
      PUtot += B[m * BC + i];
    }
  }
  uint32_t mrem = Mb, PW = 0, PU = 0, PV = 0;
  for (int kk = 0; kk < j; ++kk) {
    const int m = ffs32(mrem) - 1;
    mrem &= mrem - 1;
    const uint32_t W = B[m * BC + kk + 1], U = B[m * BC + kk], V = B[m * BC + kk + 2];
    const uint32_t base1 = n - 1 - (PV + p - (PW + W));
    const uint32_t base2 = n - 1 - (PW - (PU + U));
    f.begin(m);
#pragma unroll
    for (int h = 0; h < NHB; ++h) {
      if (h < nhB) f.inrow(m, nb.Q[h], nb.Q[h] < m ? base1 - nb.E1[h] : base2 - nb.E2[h]);
    }
    // colex(M_B \ m) = PW(kk) + PUtot - PU(kk+1)
    const uint32_t cdn = n_dn_m1 - (PW + PUtot - (PU + U));
    for (int t = 0; t < n_ba; ++t) f.down(t, m, ba_q[t], cdn);
    PW += W;
    PU += U;
    PV += V;
  }
  if (n_ab > 0) {
#pragma unroll
    for (int h = 0; h < NHB; ++h) {
      if (h < nhB) {
        // colex(M_B u q) = E1[h] + PVtot
        const uint32_t cup = n_up_m1 - (nb.E1[h] + PVtot);
        for (int t = 0; t < n_ab; ++t) f.up(t, ab_m[t], nb.Q[h], cup);
      }
    }
  }
  for (int t = 0; t < n_aa; ++t) f.across(t, c);
}

// Cross-hop index tables of the phase-ordered row pass, for a column part of
// sp <= 16 orbitals.  For every column count j and column c (column-part set
// M_B with colex n_j - 1 - c), 16 entries each (stride 16):
//   rem[off[j] + 16 c + e] = (c' << 8) | m_e  for the e-th element m_e of M_B:
//                            column c' of M_B \ m_e among the C(sp, j-1) sets;
//   ins[off[j] + 16 c + h] = (c' << 8) | q_h  for the h-th hole q_h of M_B:
//                            column c' of M_B u q_h among the C(sp, j+1) sets.
// Host code (built once per handle); off has sp + 2 entries.
inline void build_cross_tables(int sp, const uint32_t *B, int BCstride, std::vector<uint32_t> &rem,
                               std::vector<uint32_t> &ins, std::vector<uint32_t> &off) {
  off.assign(sp + 2, 0);
  for (int j = 0; j <= sp; ++j) off[j + 1] = off[j] + 16u * B[sp * BCstride + j];
  rem.assign(off[sp + 1], 0xffffffffu);
  ins.assign(off[sp + 1], 0xffffffffu);
  auto colex = [&](uint32_t M) {
    uint32_t s = 0;
    int t = 0;
    for (int d = 0; d < sp; ++d)
      if (M >> d & 1u) s += B[d * BCstride + (++t)];
    return s;
  };
  for (int j = 0; j <= sp; ++j) {
    const uint32_t n = B[sp * BCstride + j];
    const uint32_t n_dn = j > 0 ? B[sp * BCstride + j - 1] : 0, n_up = j < sp ? B[sp * BCstride + j + 1] : 0;
    for (uint32_t c = 0; c < n; ++c) {
      // colex unrank of n - 1 - c
      uint32_t R = n - 1 - c, M = 0;
      int d = sp - 1;
      for (int i = j; i >= 1; --i) {
        while (B[d * BCstride + i] > R) --d;
        R -= B[d * BCstride + i];
        M |= 1u << d;
        --d;
      }
      int e = 0, h = 0;
      for (int o = 0; o < sp; ++o) {
        if (M >> o & 1u) {
          rem[off[j] + 16 * c + e++] = ((n_dn - 1 - colex(M & ~(1u << o))) << 8) | static_cast<uint32_t>(o);
        } else {
          ins[off[j] + 16 * c + h++] = ((n_up - 1 - colex(M | (1u << o))) << 8) | static_cast<uint32_t>(o);
        }
      }
    }
  }
}

}  // namespace dev
}  // namespace doci
