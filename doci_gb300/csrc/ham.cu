// ham.cu -- device Hamiltonian: integral tables, addressing tables, diagonal.
//
// Setup of doci.c:69-134 (fill_doci_data) on the GPU: the lexical string-graph
// tables (doci.c:384-470) become one binomial table, the D-sized bitstring
// table (doci.c:472-548) is never built (kernels unrank on the fly), and the
// diagonal (doci.c:550-628) is computed by a kernel into HBM, in FP64 and as
// an FP32 copy for the FP32 sigma.
#include <cuda_runtime.h>

#include <cstdlib>
#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <cstring>
#include <utility>

#include "addressing.cuh"
#include "internal.h"

namespace doci {

static thread_local char g_last_cuda_error[256];

int cuda_status(cudaError_t e, const char *what) {
  std::snprintf(g_last_cuda_error, sizeof g_last_cuda_error, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();  // clear the sticky-free allocation error
    return DOCI_ERR_OUT_OF_MEMORY;
  }
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return DOCI_ERR_NO_DEVICE;
  return DOCI_ERR_CUDA;
}

const char *last_cuda_error() { return g_last_cuda_error; }

int device_sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
  }
  return sms;
}

// Device buffers of a handle come from the stream-ordered allocator on the
// handle's stream: creating and destroying handles while other solves run
// (the request server) then never synchronises the whole device.
static void release_async(void *p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

// The error word of the tensor-core sigma's bounded device waits: read on the
// stream (synchronising it), cleared; DOCI_ERR_DEVICE_TIMEOUT when a wait ran
// out since the last check.
int ham_device_error(doci_ham *h, cudaStream_t st) {
  if (!h->d_tc_err) return DOCI_OK;
  int v = 0;
  DOCI_CUDA(cudaMemcpyAsync(&v, h->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  if (v == 0) return DOCI_OK;
  DOCI_CUDA(cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), st));
  DOCI_CUDA(cudaStreamSynchronize(st));
  return DOCI_ERR_DEVICE_TIMEOUT;
}

void ham_release(doci_ham *h) {
  if (!h) return;
  cudaStream_t st = h->stream;
  void *bufs[] = {h->d_binom, h->d_Kmir64, h->d_Kmir32, h->d_tab64, h->d_diag, h->d_diag32, h->d_stage_x,
                  h->d_stage_y, h->d_rows, h->d_rowstart, h->d_pblocks, h->d_pblocks_host, h->d_kfrag, h->d_tc_err};  // d_rem/d_ins/d_ins_t/d_tab_off are shared (per-process cache)
  for (void *p : bufs) release_async(p, st);
  if (h->h_diag) cudaFreeHost(h->h_diag);
  if (st) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (cudaStream_t *s : {&h->copy_stream, &h->side_stream}) {
    if (*s) {
      cudaStreamSynchronize(*s);
      cudaStreamDestroy(*s);
    }
    *s = nullptr;
  }
  for (cudaEvent_t *e : {&h->start_ev, &h->end_ev, &h->side_ev}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
  for (auto &e : h->up_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  for (auto &e : h->init_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  for (auto &e : h->group_ev)
    if (e) cudaEventDestroy(e);
  h->group_ev.clear();
  h->d_pblocks_host = nullptr;
  h->host_groups.clear();
  h->host_steps.clear();
  h->d_binom = nullptr;
  h->d_Kmir64 = h->d_tab64 = h->d_diag = nullptr;
  h->d_Kmir32 = h->d_diag32 = nullptr;
  h->d_stage_x = h->d_stage_y = nullptr;
  h->d_rows = h->d_rowstart = nullptr;
  h->d_pblocks = nullptr;
  h->d_kfrag = nullptr;
  h->d_tc_err = nullptr;
  h->npblocks = 0;
  h->d_rem = h->d_ins = h->d_ins_t = h->d_tab_off = nullptr;
  h->h_diag = nullptr;
  h->stream = nullptr;
}

// keep freed memory in the device's default pool for reuse
void keep_pool_memory() {
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t threshold = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    cudaGetLastError();
  });
}

int ham_stage(doci_ham *h, size_t bytes) {
  if (h->stage_bytes >= bytes) return DOCI_OK;
  release_async(h->d_stage_x, h->stream);
  release_async(h->d_stage_y, h->stream);
  h->d_stage_x = h->d_stage_y = nullptr;
  h->stage_bytes = 0;
  DOCI_CUDA(cudaMallocAsync(&h->d_stage_x, bytes, h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_stage_y, bytes, h->stream));
  h->stage_bytes = bytes;
  return DOCI_OK;
}

// `in` holds the raw integrals (as read from an FCIDUMP); the transform is
// applied to a copy.
int ham_build(doci_ham *h, const Integrals &in) {
  const int L = in.L;
  if (L < 1) return DOCI_ERR_INVALID;
  if (L > kMaxOrbitals) return DOCI_ERR_TOO_MANY_ORBITALS;
  if (in.Na != in.Nb) return DOCI_ERR_NALPHA_NBETA;
  if (in.Na < 0 || in.Na > L) return DOCI_ERR_INVALID;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count < 1) {
    cudaGetLastError();
    return DOCI_ERR_NO_DEVICE;
  }
  std::vector<double> one(in.one), two(in.two);
  transform_integrals(one.data(), two.data(), L);
  const size_t n = L, n2 = n * n, n3 = n2 * n;
  h->L = L;
  h->N = in.Na;
  h->nh = L - in.Na;
  h->core = in.core;
  h->D = combination(static_cast<unsigned>(in.Na), static_cast<unsigned>(L));
  h->h2.assign(n, 0);
  h->J2.assign(n2, 0);
  h->Kx.assign(n2, 0);
  h->Kp.assign(n2, 0);
  for (size_t i = 0; i < n; ++i) {
    h->h2[i] = 2 * one[i * (n + 1)];
    for (size_t j = 0; j < n; ++j) {
      h->J2[i * n + j] = 2 * two[i + i * n + j * n2 + j * n3];  // 2 (ii|jj)
      h->Kx[i * n + j] = two[i + j * n + j * n2 + i * n3];      // (ij|ji)
      h->Kp[i * n + j] = i == j ? 0.0 : two[i + j * n + i * n2 + j * n3];  // (ij|ij)
    }
  }
  cudaGetDevice(&h->device);
  keep_pool_memory();
  DOCI_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));

  std::vector<uint32_t> binom(kBinomRows * kBinomCols);
  fill_binom_table(binom.data());
  std::vector<double> kmir(32 * 32, 0.0);
  std::vector<float> kmir32(32 * 32, 0.0f);
  for (int m = 0; m < L; ++m)
    for (int q = 0; q < L; ++q) {
      kmir[m * 32 + q] = h->Kp[(L - 1 - m) * n + (L - 1 - q)];
      kmir32[m * 32 + q] = static_cast<float>(kmir[m * 32 + q]);
    }
  std::vector<double> tab(n + 2 * n2);
  std::memcpy(tab.data(), h->h2.data(), n * sizeof(double));
  std::memcpy(tab.data() + n, h->J2.data(), n2 * sizeof(double));
  std::memcpy(tab.data() + n + n2, h->Kx.data(), n2 * sizeof(double));

  DOCI_CUDA(cudaMallocAsync(&h->d_binom, binom.size() * sizeof(uint32_t), h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_Kmir64, 32 * 32 * sizeof(double), h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_Kmir32, 32 * 32 * sizeof(float), h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_tab64, tab.size() * sizeof(double), h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_diag, static_cast<size_t>(h->D) * sizeof(double), h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_diag32, static_cast<size_t>(h->D) * sizeof(float), h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_tc_err, sizeof(int), h->stream));
  DOCI_CUDA(cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_binom, binom.data(), binom.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_Kmir64, kmir.data(), kmir.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_Kmir32, kmir32.data(), kmir32.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_tab64, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int st = launch_diagonal(h, h->stream);
  if (st) return st;
  st = ham_build_rows(h);
  if (st) return st;
  DOCI_CUDA(cudaStreamSynchronize(h->stream));
  return DOCI_OK;
}

// Row table for the row sigma kernel.  The column part takes the lowest
// `split` mirrored orbitals (split <= 16, so a row of C(split, j) elements
// fits in shared memory); the split shrinks until there are enough rows to
// spread over the SMs.  For a row-part occupation R (bit a = mirrored
// orbital split + a) with k elements and j = N - k in the column part, the
// colex ranks of the row are [base, base + C(split, j)) with
// base = sum_t C(split + a_t, j + t + 1) over R's elements a_0 < a_1 < ...,
// i.e. ranks [D - base - C(split, j), D - 1 - base].
int ham_build_rows(doci_ham *h) {
  const int L = h->L, N = h->N;
  int split = L < 16 ? L : 16;
  auto count_rows = [&](int sp) {
    const int na = L - sp;
    long n = 0;
    for (int k = 0; k <= na; ++k) {
      const int j = N - k;
      if (j >= 0 && j <= sp) n += static_cast<long>(binom64(na, k));
    }
    return n;
  };
  while (split > 8 && count_rows(split) < 8L * device_sm_count()) --split;
  const int na = L - split;
  if (na > 24) return DOCI_ERR_INVALID;
  h->split = split;
  std::vector<uint32_t> rows, start(size_t(1) << na, 0xffffffffu);
  int max_row = 0;
  for (uint32_t mask = 0; mask < (1u << na); ++mask) {
    const int k = __builtin_popcount(mask);
    const int j = N - k;
    if (j < 0 || j > split) continue;
    uint64_t base = 0;
    int t = 0;
    for (int a = 0; a < na; ++a)
      if (mask >> a & 1u) {
        base += binom64(split + a, j + t + 1);
        ++t;
      }
    const uint64_t len = binom64(split, j);
    const uint64_t rs = static_cast<uint64_t>(h->D) - base - len;
    start[mask] = static_cast<uint32_t>(rs);
    rows.push_back(static_cast<uint32_t>(rs));
    rows.push_back(mask | (static_cast<uint32_t>(k) << 24));
    if (static_cast<int>(len) > max_row) max_row = static_cast<int>(len);
  }
  // process rows in rank order
  std::vector<std::pair<uint32_t, uint32_t>> order;
  for (size_t i = 0; i < rows.size(); i += 2) order.emplace_back(rows[i], rows[i + 1]);
  std::sort(order.begin(), order.end());
  rows.clear();
  for (auto &p : order) {
    rows.push_back(p.first);
    rows.push_back(p.second);
  }
  h->nrows = static_cast<int>(order.size());
  h->max_row = max_row;
  DOCI_CUDA(cudaMallocAsync(&h->d_rows, rows.size() * sizeof(uint32_t), h->stream));
  DOCI_CUDA(cudaMallocAsync(&h->d_rowstart, start.size() * sizeof(uint32_t), h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_rows, rows.data(), rows.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  DOCI_CUDA(cudaMemcpyAsync(h->d_rowstart, start.data(), start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                            h->stream));
  {
    // cross-hop tables depend only on (device, split): built once per process
    static std::mutex mu;
    static std::map<std::pair<int, int>, std::array<uint32_t *, 4>> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(h->device, split);
    auto it = cache.find(key);
    if (it == cache.end()) {
      std::vector<uint32_t> B(kBinomRows * kBinomCols), rem, ins, toff;
      fill_binom_table(B.data());
      dev::build_cross_tables(split, B.data(), kBinomCols, rem, ins, toff);
      std::vector<uint32_t> ins_t(ins.size());
      for (int j = 0; j <= split; ++j) {
        const uint32_t n = B[split * kBinomCols + j];
        for (uint32_t c = 0; c < n; ++c)
          for (uint32_t e = 0; e < 16; ++e) ins_t[toff[j] + ((e >> 2) * n + c) * 4 + (e & 3)] = ins[toff[j] + 16 * c + e];
      }
      std::array<uint32_t *, 4> t{};
      DOCI_CUDA(cudaMalloc(&t[0], rem.size() * sizeof(uint32_t)));
      DOCI_CUDA(cudaMalloc(&t[1], ins.size() * sizeof(uint32_t)));
      DOCI_CUDA(cudaMalloc(&t[2], toff.size() * sizeof(uint32_t)));
      DOCI_CUDA(cudaMalloc(&t[3], ins_t.size() * sizeof(uint32_t)));
      DOCI_CUDA(cudaMemcpy(t[0], rem.data(), rem.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
      DOCI_CUDA(cudaMemcpy(t[1], ins.data(), ins.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
      DOCI_CUDA(cudaMemcpy(t[2], toff.data(), toff.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
      DOCI_CUDA(cudaMemcpy(t[3], ins_t.data(), ins_t.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
      it = cache.emplace(key, t).first;
    }
    h->d_rem = it->second[0];
    h->d_ins = it->second[1];
    h->d_tab_off = it->second[2];
    h->d_ins_t = it->second[3];
  }
  DOCI_CUDA(cudaStreamSynchronize(h->stream));
  return ham_build_pairs(h, start);
}

}  // namespace doci
