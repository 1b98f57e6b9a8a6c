// sigma_tc.cu -- FP32 sigma in the (N-1)-pair form on the 5th-generation
// tensor cores (tcgen05.mma kind::tf32 with the A operand and the
// accumulators in tensor memory, TMA bulk loads of the streamed rows).
//
// The Hamiltonian's off-diagonal elements are the pair hops T -> T \ i u a
// with weight K_ia (doci.c:216-222, the hops prev_bitstring enumerates,
// doci.c:851-978).  With S = T \ i (N-1 pairs) the hop sum regroups as
//
//   sigma[T] = diag[T] x[T] + sum_{i in T} Y_S[i],   Y_S = X_S K,
//   X_S[a] = x[S u a] for a not in S (0 for a in S),
//
// every hop counted once (S = T n T').  Determinants are tiled by the row
// tiling of the rank space: the mirrored orbitals [0, sp) form the column
// part A, the rest the row part B; all determinants with the same row-part
// set R form one contiguous row of C(sp, |C|) columns.  A unit is the row
// part R' of the sets S (|R'| = kp, jp = N-1-kp column-part elements):
//
//   * the "own row" R' (column count jp+1) holds S u a for a in A: it is
//     staged in shared memory (x and the hop sums, at most C(16,8) = 12,870
//     elements each), so those gathers and scatter-adds are on-chip;
//   * the "hole rows" R' u b (b a row-part hole of R', column count jp) hold
//     S u b at the set's own column index c: consecutive sets read and add
//     consecutive elements, streamed with TMA bulk copies (x) and coalesced
//     reductions (sigma).
//
// Per tile of 128 sets (the MMA's M; one set per thread of a 4-warp group,
// which is also the set's tensor-memory lane) the 32-wide rows X_S (columns
// 0..15: the column-part orbitals, 16..31: the unit's row-part holes) are
// split into TF32 high and low parts and stored straight into tensor memory
// (tcgen05.st), where the MMA reads its A operand; the unit's 32 x 32 K
// (also split) is the B operand in shared memory (128-byte swizzled,
// K-major).  Three tcgen05.mma passes (hi*hi + hi*lo + lo*hi, FP32
// accumulation in tensor memory) give FP32 accuracy.
//
// Ordering instead of atomics for the own rows: the units of one row-part
// size kp run in one launch, launches go from the largest kp down.  Own row
// R' (size kp) is written once, with its diagonal term, by its own unit; the
// hole rows (size kp+1) were written by the previous launch and only take
// reductions.  Rows with no column element (no own unit) get diag*x from a
// first small launch.  So sigma needs no zero fill and each own row crosses
// HBM once each way; the hole rows' reductions are the only read-modify-write
// traffic.  The reduction order of the hole rows varies from run to run (the
// result's last bits with it).  Units run in colex order of their row part,
// so the units resident at one time share many hole rows in L2.
//
// Warp roles of a block (one block per SM): warps 0-15 form four groups of
// four that gather, split and scatter alternate tiles (four tiles in flight,
// each with its own 96 columns of tensor memory), warp 16 issues the TMA
// loads of the hole rows, warp 17 issues the MMAs.  All waits are bounded: a
// wait that runs out sets the block's abort flag and the launch's error word,
// every role then leaves its loop, in-flight copies and MMAs are drained
// (again bounded) and the tensor memory is freed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "addressing.cuh"
#include "internal.h"
#include "tc_index.cuh"

namespace doci {
namespace {

constexpr int kGroups = 4;                       // tiles in flight
constexpr int kGatherWarps = 4 * kGroups;        // warps 0-15
constexpr int kProdWarp = kGatherWarps;          // warp 16: TMA producer
constexpr int kMmaWarp = kGatherWarps + 1;       // warp 17: MMA issue
constexpr int kTcThreads = 32 * (kGatherWarps + 2);
constexpr int kTile = 128;                       // sets per tile (the MMA's M)
constexpr int kStages = 6;                       // hole-row stages in flight
constexpr int kSlot = 136;                       // floats per hole segment slot (128 + alignment slack)
constexpr uint32_t kTmemCols = 512;              // per group: A hi 32 | A lo 32 | D 32 (stride 128)
// tcgen05 instruction descriptor: D FP32 (bits 4-5 = 1), A and B TF32 (bits
// 7-9, 10-12 = 2), both K-major, N = 32 (bits 17-22 = N >> 3), M = 128
// (bits 24-28 = M >> 4)
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

struct TcShape {
  uint32_t D;        // determinants (x and sigma length)
  int sp, na, lo;    // column orbitals, row orbitals, low column orbitals (<= 8)
  int kp, jp;        // this launch: row-part size of the sets, column elements of the sets
  uint32_t n_s;      // sets per unit = C(sp, jp) = columns of a hole row
  uint32_t n_own;    // columns of the own row = C(sp, jp + 1) (0: no own row)
  uint32_t n_units;  // C(na, kp)
  uint32_t cset_off; // offset of column count jp in the column-set table
  int nhr;           // row-part holes per unit = na - kp
  long spin_limit;   // try_wait iterations before a wait gives up
};

// shared-memory layout (dynamic; the base is 1024-byte aligned)
constexpr int kOffB = 0;                                     // K: hi, lo 4 KB each (swizzled)
constexpr int kOffStage = kOffB + 2 * 4096;                  // [stage][hole][kSlot] floats
constexpr int kStageBytes = 16 * kSlot * 4;
constexpr int kOffBar = kOffStage + kStages * kStageBytes;   // mbarriers (8 B each)
constexpr int kNumBars = 2 * kStages + 2 * kGroups + 1;      // hx_full, hx_empty, a_full, acc_full, drain
constexpr int kOffMisc = kOffBar + 8 * kNumBars;             // tmem slot, abort flag, hole rows / orbitals
constexpr int kOffTables = kOffMisc + 16 + 2 * 16 * 4;       // c8 (256 B) then G
constexpr int kTablesBytes = tc::kTablesBytes;
constexpr int kOffCset = (kOffTables + kTablesBytes + 15) & ~15;  // this launch's column sets (u16)
constexpr int kCsetMax = 12870;                              // C(16, 8)
constexpr int kOffRows = (kOffCset + 2 * kCsetMax + 15) & ~15;    // x_own, then sigma_own
// at least this much shared memory per block, so that one block runs per SM
// (each block allocates all 512 tensor-memory columns)
constexpr size_t kMinSmem = 120 * 1024;

__host__ __device__ constexpr size_t tc_smem_bytes(uint32_t n_own) {
  return static_cast<size_t>(kOffRows) + 2 * ((static_cast<size_t>(n_own) * 4 + 15) & ~size_t(15));
}

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t su32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
// one poll of an mbarrier phase; the thread may be suspended (up to about a
// microsecond) until the phase completes, so a waiting warp issues few
// instructions
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(a), "r"(parity), "r"(1000u)
      : "memory");
  return ok != 0;
}
// bounded wait; false when it ran out or the block aborts (then the flag is set)
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, long limit, volatile int *abort_flag,
                                          int *err, int code) {
  for (long i = 0; i < limit; ++i) {
    if (mbar_try(a, parity)) return true;
    if ((i & 63) == 63 && *abort_flag) return false;
  }
  *abort_flag = 1;
  atomicCAS(err, 0, code);
  return false;
}
// the same wait by every lane of a warp, with one outcome for the warp (the
// .sync.aligned tensor-memory instructions that follow need the whole warp)
__device__ __forceinline__ bool warp_wait(uint32_t a, uint32_t parity, long limit, volatile int *abort_flag, int *err,
                                          int code) {
  const bool r = mbar_wait(a, parity, limit, abort_flag, err, code);
  return __all_sync(0xffffffffu, r);
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  // K-major, 128-byte swizzle: leading offset unused (16 B), 8-row groups 1024 B apart, version 1
  return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (static_cast<uint64_t>(1) << 16) |
         (static_cast<uint64_t>(1024 >> 4) << 32) | (static_cast<uint64_t>(1) << 46) |
         (static_cast<uint64_t>(2) << 61);
}
// D (tensor memory) [+]= A (tensor memory) x B (shared memory descriptor)
__device__ __forceinline__ void tc_mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t db, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(db), "r"(kIdesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// 32 columns of this warp's 32 tensor-memory lanes, one lane per thread
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&y)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) y[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
      "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
      "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ uint32_t tf32_rna(float f) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
  return r;
}

// byte offset of element (row r, column k) of a 128-byte-swizzled K-major
// tile with 32 FP32 per row: 8-row atoms of 1024 B, the 16-byte chunk index
// XORed with the row inside the atom
__host__ __device__ __forceinline__ uint32_t sw128(uint32_t r, uint32_t k) {
  return (r >> 3) * 1024u + (r & 7u) * 128u + ((((k >> 2) ^ r) & 7u) << 4) + (k & 3u) * 4u;
}

// colex unrank of an na-bit mask with kp elements (the unit's row part)
__device__ __forceinline__ uint32_t unit_mask(uint32_t u, int na, int kp, const uint32_t *B) {
  return dev::colex_unrank<kBinomCols>(u, na, kp, B);
}

// ---------------------------------------------------------------- kernels
// rows with no column element (all N pairs in the row part): no own unit,
// sigma starts as diag * x there
__global__ void tc_rows0_kernel(const uint32_t *__restrict__ starts, int n, const float *__restrict__ diag,
                                const float *__restrict__ x, float *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t r = starts[i];
    y[r] = diag[r] * x[r];
  }
}

__global__ void __launch_bounds__(kTcThreads, 1)
sigma_tc_kernel(TcShape s, const uint32_t *__restrict__ g_binom, const uint32_t *__restrict__ rowstart_of,
                const uint16_t *__restrict__ cset, const uint8_t *__restrict__ g_tables,
                const float *__restrict__ g_ksplit, const float *__restrict__ diag, const float *__restrict__ x,
                float *__restrict__ y, int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t base = su32(sm);
  if (base & 1023u) {  // the swizzled K tiles need a 1024-byte aligned base
    if (tid == 0) atomicCAS(err, 0, 3);
    return;
  }
  uint64_t *bars = reinterpret_cast<uint64_t *>(sm + kOffBar);
  auto bar = [&](int i) { return su32(bars + i); };
  const int B_HXF = 0, B_HXE = kStages, B_AF = 2 * kStages, B_ACC = 2 * kStages + kGroups,
            B_DRAIN = 2 * kStages + 2 * kGroups;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + kOffMisc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kOffMisc + 4);
  uint32_t *hole_rs = reinterpret_cast<uint32_t *>(sm + kOffMisc + 16);
  int *hole_orb = reinterpret_cast<int *>(sm + kOffMisc + 16 + 64);
  const uint8_t *c8 = sm + kOffTables;
  const uint16_t *Gt = reinterpret_cast<const uint16_t *>(sm + kOffTables + 256);
  uint16_t *cs_sm = reinterpret_cast<uint16_t *>(sm + kOffCset);
  const size_t row_bytes = ((static_cast<size_t>(s.n_own) * 4 + 15) & ~size_t(15));
  float *x_own = reinterpret_cast<float *>(sm + kOffRows);
  float *s_own = reinterpret_cast<float *>(sm + kOffRows + row_bytes);
  float *stage = reinterpret_cast<float *>(sm + kOffStage);

  const int lo = s.lo, sp = s.sp, nhr = s.nhr;
  const bool has_own = s.n_own > 0;
  const uint32_t Dl = s.D & ~3u;  // end of the vector's last whole 16-byte chunk

  // per-launch tables: c8[P] (colex of the low part), G[Q][p], the column sets
  for (int i = tid; i < kTablesBytes; i += kTcThreads) sm[kOffTables + i] = g_tables[i];
  for (uint32_t i = tid; i < s.n_s; i += kTcThreads) cs_sm[i] = cset[s.cset_off + i];
  if (tid == 0) {
    for (int i = 0; i < kNumBars; ++i) {
      const uint32_t cnt = (i >= B_HXE && i < B_AF) ? 4u : (i >= B_AF && i < B_ACC) ? 4u : 1u;
      mbar_init(bar(i), cnt);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  const uint32_t ntiles = (s.n_s + kTile - 1) / kTile;
  uint32_t T0 = 0;        // tiles of earlier units (phase bookkeeping of the barriers)
  uint32_t mma_issued = 0;
  uint32_t loads_issued = 0;  // producer: tiles whose hole segments were requested (T = 0 .. loads_issued-1)
  bool ok = true;

  for (uint32_t u = blockIdx.x; u < s.n_units; u += gridDim.x) {
    // ---- unit set-up: holes, K tiles, own row
    const uint32_t mask = unit_mask(u, s.na, s.kp, g_binom);
    __syncthreads();  // the previous unit's flush is done with the own row
    if (warp == 0) {
      const bool hole = lane < s.na && !((mask >> lane) & 1u);
      const uint32_t hb = __ballot_sync(0xffffffffu, hole);
      if (hole) {
        const int h = __popc(hb & ((1u << lane) - 1u));
        hole_rs[h] = rowstart_of[mask | (1u << lane)];
        hole_orb[h] = sp + lane;
      }
    }
    __syncthreads();
    // K tiles (B operand, N rows of K): row n = output column, column k = input column;
    // column j < 16: column orbital j (if j < sp); j >= 16: hole j - 16
    for (int e = tid; e < 32 * 32; e += kTcThreads) {
      const int n = e >> 5, k = e & 31;
      auto orb = [&](int j) { return j < 16 ? (j < sp ? j : -1) : (j - 16 < nhr ? hole_orb[j - 16] : -1); };
      const int on = orb(n), ok2 = orb(k);
      float vh = 0.f, vl = 0.f;
      if (on >= 0 && ok2 >= 0) {
        vh = g_ksplit[on * 32 + ok2];
        vl = g_ksplit[32 * 32 + on * 32 + ok2];
      }
      *reinterpret_cast<float *>(sm + kOffB + sw128(n, k)) = vh;
      *reinterpret_cast<float *>(sm + kOffB + 4096 + sw128(n, k)) = vl;
    }
    if (has_own) {
      const uint32_t own = rowstart_of[mask];
      for (uint32_t c = tid; c < s.n_own; c += kTcThreads) {
        const float v = x[own + c];
        x_own[c] = v;
        s_own[c] = diag[own + c] * v;
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (warp < kGatherWarps && ok) {
      // ---- gather / split into tensor memory / MMA hand-off / scatter:
      // group g takes the tiles T = T0 + t with T % 4 == g
      const int g = warp >> 2, q = warp & 3, gt = 32 * q + lane;
      const uint32_t t_grp = tmem + static_cast<uint32_t>(128 * g) + (static_cast<uint32_t>(32 * q) << 16);
      for (uint32_t t = static_cast<uint32_t>(g - static_cast<int>(T0 & 3u) + 4) & 3u; t < ntiles; t += 4) {
        const uint32_t T = T0 + t;
        const uint32_t st = T % kStages, use = T / kStages;
        if (!warp_wait(bar(B_HXF + st), use & 1u, s.spin_limit, abort_flag, err, 10)) { ok = false; break; }
        const uint32_t c0 = t * kTile, c = c0 + gt;
        const bool live = c < s.n_s;
        float v[32];
        uint32_t pos[16];
        uint32_t C = 0xffffu;
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0.f;
        if (live) {
          C = cs_sm[c];
          if (has_own) {
            // own-row position of C u a (tc::own_pos with its per-set terms hoisted)
            const uint32_t lomask = (1u << lo) - 1u, P = C & lomask, Q = C >> lo;
            const int p = __popc(P);
            const uint32_t top = s.n_own - 1u;
            const uint32_t base_lo = top - Gt[Q * tc::gw(lo) + p + 1];
            const uint32_t base_hi = top - c8[P];
#pragma unroll
            for (int a = 0; a < 16; ++a) {
              if (a < sp && !((C >> a) & 1u)) {
                pos[a] = a < lo ? base_lo - c8[P | (1u << a)]
                                : base_hi - Gt[(Q | (1u << (a - lo))) * tc::gw(lo) + p];
                v[a] = x_own[pos[a]];
              }
            }
          }
          // hole rows: the staged segment of row h starts at its 16-byte
          // chunk, (rs + c0) & 3 elements before this tile's first set
          const float *sg = stage + st * (16 * kSlot) + gt;
#pragma unroll
          for (int h = 0; h < 16; ++h) {
            if (h < nhr) {
              const uint32_t rs = hole_rs[h], gidx = rs + c;
              v[16 + h] = gidx < Dl ? sg[h * kSlot + ((rs + c0) & 3u)] : x[gidx];
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(B_HXE + st));
        // split into TF32 high and low parts, both into this set's lane
        {
          uint32_t hv[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) hv[j] = tf32_rna(v[j]);
          tc_st32(t_grp, hv);
#pragma unroll
          for (int j = 0; j < 32; ++j) hv[j] = __float_as_uint(v[j] - __uint_as_float(hv[j]));
          tc_st32(t_grp + 32, hv);
        }
        tc_wait_st();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(B_AF + g));
        if (!warp_wait(bar(B_ACC + g), (T >> 2) & 1u, s.spin_limit, abort_flag, err, 11)) { ok = false; break; }
        tc_fence_after();
        float yv[32];
        tc_ld32(t_grp + 64, yv);
        tc_fence_before();
        if (live) {
          if (has_own) {
#pragma unroll
            for (int a = 0; a < 16; ++a)
              if (a < sp && !((C >> a) & 1u)) atomicAdd(s_own + pos[a], yv[a]);
          }
#pragma unroll
          for (int h = 0; h < 16; ++h)
            if (h < nhr) atomicAdd(y + hole_rs[h] + c, yv[16 + h]);
        }
      }
    } else if (warp == kProdWarp && ok) {
      // ---- producer: the hole-row segments of every tile of this unit
      for (uint32_t t = 0; t < ntiles; ++t) {
        const uint32_t T = T0 + t, st = T % kStages, use = T / kStages;
        if (use > 0 && !warp_wait(bar(B_HXE + st), (use - 1) & 1u, s.spin_limit, abort_flag, err, 12)) {
          ok = false;
          break;
        }
        const uint32_t c0 = t * kTile, c1 = min(c0 + kTile, s.n_s);
        uint32_t a0 = 0, a1 = 0;
        if (lane < nhr) tc::hole_segment(hole_rs[lane], c0, c1, s.D, &a0, &a1);
        uint32_t bytes = (a1 - a0) * 4u;
        uint32_t total = bytes;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
        if (lane == 0) mbar_expect_tx(bar(B_HXF + st), total);
        __syncwarp();
        if (lane < nhr && bytes > 0)
          bulk_load(su32(stage + st * (16 * kSlot) + lane * kSlot), x + a0, bytes, bar(B_HXF + st));
        loads_issued = T + 1;
      }
    } else if (warp == kMmaWarp && ok) {
      // ---- MMA issue (one thread): 3 passes x the k-steps that hold columns
      for (uint32_t t = 0; t < ntiles; ++t) {
        const uint32_t T = T0 + t, g = T & 3u;
        if (!warp_wait(bar(B_AF + g), (T >> 2) & 1u, s.spin_limit, abort_flag, err, 13)) {
          ok = false;
          break;
        }
        tc_fence_after();
        if (lane == 0) {
          const uint32_t a_hi = tmem + 128u * g, a_lo = a_hi + 32u, d = a_hi + 64u;
          const uint32_t b_hi = base + kOffB, b_lo = b_hi + 4096;
          uint32_t acc = 0;
#pragma unroll
          for (int pass = 0; pass < 3; ++pass) {
            const uint32_t a = pass == 1 ? a_lo : a_hi, b = pass == 2 ? b_lo : b_hi;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const bool used = ks == 0 ? true : ks == 1 ? sp > 8 : ks == 2 ? nhr > 0 : nhr > 8;
              if (used) {
                tc_mma_ts(d, a + 8u * ks, smem_desc(b + ks * 32), acc);
                acc = 1;
              }
            }
          }
          tc_commit(bar(B_ACC + g));
        }
        __syncwarp();
        ++mma_issued;
      }
    }
    T0 += ntiles;
    tc_fence_before();
    __syncthreads();  // every tile of the unit is scattered
    tc_fence_after();
    if (*abort_flag) ok = false;
    if (!ok) break;
    // ---- own row: its first and only write (diagonal term included)
    if (has_own) {
      const uint32_t own = rowstart_of[mask];
      for (uint32_t c = tid; c < s.n_own; c += kTcThreads) y[own + c] = s_own[c];
    }
  }

  // ---- drain: after an abort, wait (bounded, with the fixed limit: these are
  // copies and MMAs that complete by themselves) for what is in flight, then
  // free the tensor memory
  __syncthreads();
  if (*abort_flag && warp == kProdWarp && lane == 0) {
    // the latest request of each stage is complete once that use's phase has completed
    for (uint32_t st = 0; st < kStages; ++st) {
      if (loads_issued > st) {
        const uint32_t last_T = loads_issued - 1 - ((loads_issued - 1 - st) % kStages);
        const uint32_t use = last_T / kStages;
        for (long i = 0; i < kTcSpinLimit && !mbar_try(bar(B_HXF + st), use & 1u); ++i) {
        }
      }
    }
  }
  if (warp == kMmaWarp) {
    if (lane == 0 && mma_issued > 0) {
      tc_commit(bar(B_DRAIN));
      for (long i = 0; i < kTcSpinLimit && !mbar_try(bar(B_DRAIN), 0); ++i) {
      }
    }
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == kMmaWarp)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// ---------------------------------------------------------------- host side
struct TcTables {
  uint16_t *cset = nullptr;      // all column sets of sp orbitals, by column count then column index
  std::vector<uint32_t> cset_off;
  uint8_t *tables = nullptr;     // c8 (256 B) + G (256 x 10 u16)
};

int tc_tables(int device, int sp, const TcTables **out) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, TcTables> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(device, sp);
  auto it = cache.find(key);
  if (it == cache.end()) {
    TcTables t;
    std::vector<uint32_t> B(kBinomRows * kBinomCols);
    fill_binom_table(B.data());
    std::vector<uint16_t> cs;
    std::vector<uint8_t> tb;
    tc::build_tables(sp, B.data(), kBinomCols, cs, t.cset_off, tb);
    DOCI_CUDA(cudaMalloc(&t.cset, cs.size() * sizeof(uint16_t)));
    DOCI_CUDA(cudaMalloc(&t.tables, tb.size()));
    DOCI_CUDA(cudaMemcpy(t.cset, cs.data(), cs.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    DOCI_CUDA(cudaMemcpy(t.tables, tb.data(), tb.size(), cudaMemcpyHostToDevice));
    it = cache.emplace(key, std::move(t)).first;
  }
  *out = &it->second;
  return DOCI_OK;
}

// rows with no column element, per handle shape (device, L, N, split)
int tc_rows0(const doci_ham *h, const uint32_t **rows, int *n) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, std::pair<uint32_t *, int>> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_tuple(h->device, h->L, h->N, h->split);
  auto it = cache.find(key);
  if (it == cache.end()) {
    std::vector<uint32_t> B(kBinomRows * kBinomCols);
    fill_binom_table(B.data());
    const std::vector<uint32_t> v = tc::rows_without_columns(h->L, h->N, h->split, h->D, B.data(), kBinomCols);
    uint32_t *d = nullptr;
    if (!v.empty()) {
      DOCI_CUDA(cudaMalloc(&d, v.size() * sizeof(uint32_t)));
      DOCI_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    }
    it = cache.emplace(key, std::make_pair(d, static_cast<int>(v.size()))).first;
  }
  *rows = it->second.first;
  *n = it->second.second;
  return DOCI_OK;
}

}  // namespace

bool tc_fits(const doci_ham *h) {
  if (h->split < 1 || h->split > 16 || !h->d_rowstart || !h->d_kfrag) return false;
  const int na = h->L - h->split;
  if (na < 0 || na > 16) return false;  // holes per unit <= 16 (columns 16..31 of the tile)
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) return false;  // built for sm_103a only
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return std::max(tc_smem_bytes(static_cast<uint32_t>(h->max_row)), kMinSmem) <= static_cast<size_t>(optin);
}

// launches of one sigma: the no-column rows (if any) and one per row-part
// size of the sets
int tc_launches(const doci_ham *h) {
  const int L = h->L, N = h->N, sp = h->split, na = L - sp;
  int n = N <= na ? 1 : 0;
  for (int kp = std::min(na, N - 1); kp >= 0; --kp) {
    const int jp = N - 1 - kp;
    if (jp >= 0 && jp <= sp && binom64(sp, jp) > 0 && binom64(na, kp) > 0) ++n;
  }
  return n;
}

int launch_tc(const doci_ham *h, const float *x, float *y, cudaStream_t st, int *d_err, long spin_limit) {
  if (!tc_fits(h)) return DOCI_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(x) & 15u) != 0) return DOCI_ERR_INVALID;  // bulk copies need 16-byte alignment
  const TcTables *tb = nullptr;
  int r = tc_tables(h->device, h->split, &tb);
  if (r != DOCI_OK) return r;
  const uint32_t *rows0 = nullptr;
  int n0 = 0;
  r = tc_rows0(h, &rows0, &n0);
  if (r != DOCI_OK) return r;
  if (n0 > 0) {
    tc_rows0_kernel<<<(n0 + 255) / 256, 256, 0, st>>>(rows0, n0, h->d_diag32, x, y);
    DOCI_CUDA(cudaGetLastError());
  }
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    attr_err = cudaFuncSetAttribute(sigma_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  });
  DOCI_CUDA(attr_err);
  const int L = h->L, N = h->N, sp = h->split, na = L - sp;
  std::vector<uint32_t> B(kBinomRows * kBinomCols);
  fill_binom_table(B.data());
  auto C = [&](int n, int k) -> uint32_t { return (k < 0 || n < 0 || k > n) ? 0u : B[n * kBinomCols + k]; };
  const int sms = device_sm_count();
  for (int kp = std::min(na, N - 1); kp >= 0; --kp) {
    const int jp = N - 1 - kp;
    if (jp < 0 || jp > sp) continue;
    TcShape s{};
    s.D = h->D;
    s.sp = sp;
    s.na = na;
    s.lo = sp < 8 ? sp : 8;
    s.kp = kp;
    s.jp = jp;
    s.n_s = C(sp, jp);
    s.n_own = jp + 1 <= sp ? C(sp, jp + 1) : 0u;
    s.n_units = C(na, kp);
    s.cset_off = tb->cset_off[jp];
    s.nhr = na - kp;
    s.spin_limit = spin_limit;
    if (s.n_units == 0 || s.n_s == 0) continue;
    const size_t smem = std::max(tc_smem_bytes(s.n_own), kMinSmem);
    const int grid = static_cast<int>(std::min<uint32_t>(s.n_units, static_cast<uint32_t>(sms)));
    sigma_tc_kernel<<<grid, kTcThreads, smem, st>>>(s, h->d_binom, h->d_rowstart, tb->cset, tb->tables,
                                                    reinterpret_cast<const float *>(h->d_kfrag), h->d_diag32, x, y,
                                                    d_err);
    DOCI_CUDA(cudaGetLastError());
  }
  return DOCI_OK;
}

}  // namespace doci
