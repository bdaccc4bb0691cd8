// fuelg_lloyd.cu -- Lloyd k-means (src/cluster/kmeans/lloyd.rs:12-202) on GB300.
//
// One iteration = assign + centre update:
//   assign   every point's nearest centre under the reference's own distance
//            order (iteration 1: the pairwise kernel order of
//            vec_pairwise_sqdist, lloyd.rs:76; later iterations: math::sqdist,
//            lloyd.rs:166-172), first index wins ties (strict '<').  This is
//            the exact linear-scan top-1 of fuelg_knn.cu with centres as the
//            index and points as the queries.
//   update   centre_j = (f32)(sum_j / count_j), sums in FP64 over the members
//            of cluster j in ascending point order (stable radix sort by
//            label, then fixed 32-row chunk partials reduced in chunk order):
//            deterministic and atomics-free on the floating-point path.
//            Empty clusters keep their centre (lloyd.rs:138-146).
// The loop stops when no label changed (lloyd.rs:197) or at max_iter
// (initialisation counts as iteration 1, util.rs:40); the reported inertia is
// the FP64 sum of squared distances of every point to the centre it was
// assigned to in the final pass (the f32 `lastsum` of lloyd.rs:196, computed
// exactly).
#include <algorithm>
#include <cmath>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <vector>

#include "../../include/fuelg.h"
#include "fuelg_common.cuh"
#include "fuelg_internal.h"
#include "fuelg_prep.cuh"
#include "fuelg_sums.cuh"

namespace fuelg {

// Middle Lloyd passes captured into one CUDA graph (see lloyd_run).
constexpr int kPassesPerGraph = 8;

struct TcLloydState;
TcLloydState* lloyd_tc_new();
void lloyd_tc_delete(TcLloydState*);
bool lloyd_tc_supported(int d, int k);
int lloyd_tc_prepare(const LloydParams& p, TcLloydState* st, cudaStream_t stream);
int lloyd_assign_tc(const LloydParams& p, TcLloydState* st, const float* centers, bool first, int32_t* lab_new,
                    int* dev_status, cudaStream_t stream);
struct ExactSums;
ExactSums* exact_sums_new();
void exact_sums_delete(ExactSums*);
int exact_sums_init(ExactSums* s, const float* X, int64_t n, int d, int k, cudaStream_t stream);
int exact_sums_step(ExactSums* s, const float* X, const int32_t* lab_new, int32_t* labels, bool first,
                    bool write_centers, float* centers, int32_t* changed, int* dev_status, cudaStream_t stream,
                    const CentrePrep* cp);
int exact_sums_update(ExactSums* s, const float* X, bool write_centers, float* centers, int32_t* changed,
                      const CentrePrep* cp, cudaStream_t stream, bool plan_in_scatter);
void exact_sums_commit_view(ExactSums* s, SumsCommit* v);
int lloyd_tc_rescored_total(TcLloydState* st, cudaStream_t stream, int64_t* out);
int lloyd_tc_pass_fused(const LloydParams& p, TcLloydState* st, const float* centers, int32_t* labels,
                        const SumsCommit& sc, int* dev_status, cudaStream_t stream);
CentrePrep lloyd_tc_centre_prep(TcLloydState* st);
bool lloyd_tc_scaled(const TcLloydState* st);

namespace {

constexpr int kChunk = 32;  // rows per FP64 partial-sum chunk

__global__ void keys_to_labels_kernel(const uint64_t* __restrict__ keys, int64_t n, int32_t* __restrict__ lab) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lab[i] = (int32_t)key_idx(keys[i]);
}

__global__ void post_assign_kernel(const int32_t* __restrict__ lab_new, int64_t n, int32_t* __restrict__ labels,
                                   int first, int32_t* __restrict__ changed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (i < n) {
    const int32_t a = lab_new[i];
    if (first || labels[i] != a) c = 1;
    labels[i] = a;
  }
  c = __syncthreads_count(c);
  if (threadIdx.x == 0 && c) atomicAdd(changed, c);  // integer: order-independent
}

__global__ void iota_kernel(int32_t* __restrict__ v, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (int32_t)i;
}

__global__ void count_global_kernel(const int32_t* __restrict__ labels, int64_t n, int32_t* __restrict__ counts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&counts[labels[i]], 1);  // integer: order-independent
}

__global__ void count_kernel(const int32_t* __restrict__ labels, int64_t n, int k, int32_t* __restrict__ counts) {
  extern __shared__ int32_t hist[];
  for (int j = threadIdx.x; j < k; j += blockDim.x) hist[j] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&hist[labels[i]], 1);
  __syncthreads();
  for (int j = threadIdx.x; j < k; j += blockDim.x)
    if (hist[j]) atomicAdd(&counts[j], hist[j]);
}

// Per cluster: member offset, number of 32-row chunks.
__global__ void chunk_count_kernel(const int32_t* __restrict__ counts, int k, int32_t* __restrict__ nchunks) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) nchunks[j] = (counts[j] + kChunk - 1) / kChunk;
}

__global__ void chunk_table_kernel(const int32_t* __restrict__ chunk_off, const int32_t* __restrict__ nchunks, int k,
                                   int32_t* __restrict__ chunk_cluster) {
  const int j = blockIdx.x;
  for (int c = threadIdx.x; c < nchunks[j]; c += blockDim.x) chunk_cluster[chunk_off[j] + c] = j;
}

// partial[c][t] = sum over the <=32 member rows of chunk c, in member order.
__global__ void chunk_sum_kernel(const float* __restrict__ X, int d, const int32_t* __restrict__ perm,
                                 const int32_t* __restrict__ mem_off, const int32_t* __restrict__ counts,
                                 const int32_t* __restrict__ chunk_off, const int32_t* __restrict__ chunk_cluster,
                                 const int32_t* __restrict__ total_chunks, double* __restrict__ partial) {
  const int c = blockIdx.x;
  if (c >= *total_chunks) return;  // grid sized for the upper bound n/32 + k + 1
  const int j = chunk_cluster[c];
  const int r0 = (c - chunk_off[j]) * kChunk;
  const int rows = min(kChunk, counts[j] - r0);
  const int32_t* members = perm + mem_off[j] + r0;
  __shared__ int32_t mrow[kChunk];
  if (threadIdx.x < rows) mrow[threadIdx.x] = members[threadIdx.x];
  __syncthreads();
  for (int t = blockIdx.y * blockDim.x + threadIdx.x; t < d; t += gridDim.y * blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < rows; r++) s += (double)__ldg(X + (int64_t)mrow[r] * d + t);
    partial[(int64_t)c * d + t] = s;
  }
}

// centre_j[t] = (f32)(sum over chunks of j, in chunk order / count_j); empty clusters keep theirs.
__global__ void reduce_update_kernel(const double* __restrict__ partial, int d, int k,
                                     const int32_t* __restrict__ counts, const int32_t* __restrict__ chunk_off,
                                     const int32_t* __restrict__ nchunks, float* __restrict__ centers) {
  const int j = blockIdx.x;
  const int cnt = counts[j];
  if (cnt == 0) return;
  const int c0 = chunk_off[j], nc = nchunks[j];
  for (int t = blockIdx.y * blockDim.x + threadIdx.x; t < d; t += gridDim.y * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nc; c++) s += partial[(int64_t)(c0 + c) * d + t];
    centers[(int64_t)j * d + t] = __double2float_rn(__ddiv_rn(s, (double)cnt));
  }
}

// Per-block FP64 partials of sum_i ||x_i - c_{l_i}||^2, to near-FP64
// accuracy on FP32 arithmetic (one SqDiffAcc per lane, renormalised every
// 32 terms at most, converted to FP64 once).
__global__ void inertia_partial_kernel(const float* __restrict__ X, int64_t n, int d, const float* __restrict__ C,
                                       const int32_t* __restrict__ labels, double* __restrict__ partial) {
  __shared__ double red[32];
  double acc = 0.0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const bool vec = (d & 3) == 0 && ((reinterpret_cast<uintptr_t>(X) | reinterpret_cast<uintptr_t>(C)) & 15) == 0;
  SqDiffAcc sa;  // this lane's terms over all its rows, renormalised every <= 32 terms
  for (int64_t i = (int64_t)blockIdx.x * nw + warp; i < n; i += (int64_t)gridDim.x * nw) {
    const float* x = X + i * d;
    const float* c = C + (int64_t)labels[i] * d;
    if (vec) {
      // up to 8 float4 of the row and of its centre per lane in flight at once
      for (int cb = 4 * lane; cb < d; cb += 128 * 8) {
        float4 xv[8], cv[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const int c0 = cb + 128 * u;
          if (c0 < d) {
            xv[u] = __ldg(reinterpret_cast<const float4*>(x + c0));
            cv[u] = __ldg(reinterpret_cast<const float4*>(c + c0));
          }
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
          if (cb + 128 * u >= d) break;
          sa.add(xv[u].x, cv[u].x);
          sa.add(xv[u].y, cv[u].y);
          sa.add(xv[u].z, cv[u].z);
          sa.add(xv[u].w, cv[u].w);
        }
        sa.renorm();
      }
    } else {
      for (int t0 = lane; t0 < d; t0 += 32 * 32) {
        const int t1 = min(d, t0 + 32 * 32);
#pragma unroll 4
        for (int t = t0; t < t1; t += 32) sa.add(__ldg(x + t), __ldg(c + t));
        sa.renorm();
      }
    }
  }
  acc = sa.value();
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < nw; w++) s += red[w];
    partial[blockIdx.x] = s;
  }
}

// Fixed-shape tree reduction of the per-block partials (deterministic).
__global__ void sum_partials_kernel(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  __shared__ double red[1024];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// FP64 ||C_new - C_old||_F^2 and ||C_old||_F^2 for the tol>0 stop rule
// (lloyd.rs:136-153).
__global__ void frob_kernel(const float* __restrict__ Cold, const float* __restrict__ Cnew, int64_t kd,
                            double* __restrict__ out2) {
  __shared__ double s1[256], s2[256];
  double a = 0.0, b = 0.0;
  for (int64_t e = threadIdx.x; e < kd; e += blockDim.x) {
    const double o = Cold[e], w = Cnew[e];
    a += (w - o) * (w - o);
    b += o * o;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0.0, y = 0.0;
    for (int t = 0; t < (int)blockDim.x; t++) {
      x += s1[t];
      y += s2[t];
    }
    out2[0] = x;
    out2[1] = y;
  }
}

int end_bit_for(int k) {
  int b = 1;
  while ((1 << b) < k) b++;
  return b;
}

// ---- FP64 fallback sums (data whose exponent range exceeds 128 bits) -----
struct Fp64Sums {
  int64_t n = 0;
  int d = 0, k = 0, ebit = 0;
  int64_t max_chunks = 0;
  size_t sort_bytes = 0, scan_bytes = 0;
  Scratch perm_in, perm, lab_sorted, counts, offs, nchunks, chunk_off, chunk_cluster, partial, tmp;
};

int fp64_sums_init(Fp64Sums* f, int64_t n, int d, int k, int32_t* labels, cudaStream_t stream) {
  f->n = n;
  f->d = d;
  f->k = k;
  f->ebit = end_bit_for(k);
  f->max_chunks = n / kChunk + k + 1;
  FUELG_TRY(f->perm_in.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(f->perm.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(f->lab_sorted.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(f->counts.alloc(sizeof(int32_t) * (k + 1), stream));
  FUELG_TRY(f->offs.alloc(sizeof(int32_t) * (k + 1), stream));
  FUELG_TRY(f->nchunks.alloc(sizeof(int32_t) * (k + 1), stream));
  FUELG_TRY(f->chunk_off.alloc(sizeof(int32_t) * (k + 1), stream));
  FUELG_TRY(f->chunk_cluster.alloc(sizeof(int32_t) * f->max_chunks, stream));
  FUELG_TRY(f->partial.alloc(sizeof(double) * f->max_chunks * d, stream));
  FUELG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, f->sort_bytes, labels, f->lab_sorted.as<int32_t>(),
                                             f->perm_in.as<int32_t>(), f->perm.as<int32_t>(), (int)n, 0, f->ebit,
                                             stream));
  FUELG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, f->scan_bytes, f->counts.as<int32_t>(), f->offs.as<int32_t>(),
                                           k + 1, stream));
  FUELG_TRY(f->tmp.alloc(std::max(f->sort_bytes, f->scan_bytes), stream));
  iota_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(f->perm_in.as<int32_t>(), n); ::fuelg::note_launch();
  return ST_OK;
}

// centre_j = (f32)(FP64 sum of member rows in ascending point order / count)
int fp64_sums_update(Fp64Sums* f, const float* X, const int32_t* labels, float* C, cudaStream_t stream) {
  const int64_t n = f->n;
  const int d = f->d, k = f->k;
  FUELG_CUDA(cudaMemsetAsync(f->counts.p, 0, sizeof(int32_t) * (k + 1), stream));
  if (k <= 8192) {
    count_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, sizeof(int32_t) * k, stream>>>(
        labels, n, k, f->counts.as<int32_t>()); ::fuelg::note_launch();
  } else {
    count_global_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, stream>>>(
        labels, n, f->counts.as<int32_t>()); ::fuelg::note_launch();
  }
  size_t sb = f->sort_bytes;
  FUELG_CUDA(cub::DeviceRadixSort::SortPairs(f->tmp.p, sb, labels, f->lab_sorted.as<int32_t>(),
                                             f->perm_in.as<int32_t>(), f->perm.as<int32_t>(), (int)n, 0, f->ebit,
                                             stream));
  size_t scb = f->scan_bytes;
  FUELG_CUDA(cub::DeviceScan::ExclusiveSum(f->tmp.p, scb, f->counts.as<int32_t>(), f->offs.as<int32_t>(), k + 1,
                                           stream));
  chunk_count_kernel<<<(k + 255) / 256, 256, 0, stream>>>(f->counts.as<int32_t>(), k, f->nchunks.as<int32_t>()); ::fuelg::note_launch();
  FUELG_CUDA(cudaMemsetAsync(f->nchunks.as<int32_t>() + k, 0, sizeof(int32_t), stream));
  scb = f->scan_bytes;
  FUELG_CUDA(cub::DeviceScan::ExclusiveSum(f->tmp.p, scb, f->nchunks.as<int32_t>(), f->chunk_off.as<int32_t>(),
                                           k + 1, stream));
  chunk_table_kernel<<<k, 128, 0, stream>>>(f->chunk_off.as<int32_t>(), f->nchunks.as<int32_t>(), k,
                                            f->chunk_cluster.as<int32_t>()); ::fuelg::note_launch();
  const int ty = (d + 255) / 256;
  dim3 g1((unsigned)f->max_chunks, ty);
  chunk_sum_kernel<<<g1, 256, 0, stream>>>(X, d, f->perm.as<int32_t>(), f->offs.as<int32_t>(),
                                           f->counts.as<int32_t>(), f->chunk_off.as<int32_t>(),
                                           f->chunk_cluster.as<int32_t>(), f->chunk_off.as<int32_t>() + k,
                                           f->partial.as<double>()); ::fuelg::note_launch();
  dim3 g2(k, ty);
  reduce_update_kernel<<<g2, 256, 0, stream>>>(f->partial.as<double>(), d, k, f->counts.as<int32_t>(),
                                               f->chunk_off.as<int32_t>(), f->nchunks.as<int32_t>(), C); ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

}  // namespace

int lloyd_run(const LloydParams& p, LloydResult* r, int* dev_status, cudaStream_t stream) {
  const int64_t n = p.n;
  const int d = p.d, k = p.k;
  if (n <= 0 || d <= 0 || k <= 0) {
    set_error("lloyd: n, d and k must be positive (n=%lld d=%d k=%d)", (long long)n, d, k);
    return ST_EINVAL;
  }
  if (n >= (1ll << 31)) {
    set_error("lloyd: n=%lld exceeds the 2^31-1 row limit", (long long)n);
    return ST_ENOTSUP;
  }
  float* C = r->centers;
  int32_t* labels = r->labels;
  FUELG_CUDA(cudaMemcpyAsync(C, p.init, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, stream));

  Scratch keys, lab_new, changed, frob, cold, inert_part, inert;
  FUELG_TRY(lab_new.alloc(sizeof(int32_t) * n, stream));
  // one changed-count slot (2 words apart) per pass of a multi-pass graph
  FUELG_TRY(changed.alloc(sizeof(int32_t) * 2 * (kPassesPerGraph + 1), stream));
  FUELG_TRY(frob.alloc(sizeof(double) * 2, stream));
  if (p.tol > 0) FUELG_TRY(cold.alloc(sizeof(float) * k * d, stream));
  const int inert_blocks = 4 * 152;
  FUELG_TRY(inert_part.alloc(sizeof(double) * inert_blocks, stream));
  FUELG_TRY(inert.alloc(sizeof(double), stream));

  int32_t* h_changed = nullptr;
  FUELG_CUDA(cudaMallocHost(&h_changed, sizeof(int32_t) * 2 * kPassesPerGraph));
  struct HostFree {
    void* p;
    ~HostFree() {
      if (p) cudaFreeHost(p);
    }
  } hf{h_changed};

  // Exact integer centroid sums (fuelg_sums.cu); FP64 sums when the data's
  // exponent range does not fit 128 bits.
  ExactSums* es = exact_sums_new();
  struct EsFree {
    ExactSums* e;
    ~EsFree() { exact_sums_delete(e); }
  } esf{es};
  const bool exact = exact_sums_init(es, p.X, n, d, k, stream) == ST_OK;
  r->exact_sums = exact;
  Fp64Sums fs;
  if (!exact) FUELG_TRY(fp64_sums_init(&fs, n, d, k, labels, stream));

  // Tensor-core tier: BF16 (or hi+lo BF16) screen + exact re-score, for d >= 32 and k <= 256.
  TcLloydState* tc = nullptr;
  struct TcFree {
    TcLloydState*& t;
    ~TcFree() {
      if (t) lloyd_tc_delete(t);
    }
  } tcf{tc};
  r->precision_used = 0;
  // TMA row coordinates are 32-bit: the tile-major copy needs n * ceil(d/64) < 2^31
  const bool tc_fits = n * (int64_t)((d + 63) / 64) < (1ll << 31) - 4096;
  if (p.precision != 0 && lloyd_tc_supported(d, k) && tc_fits) {
    tc = lloyd_tc_new();
    FUELG_TRY(lloyd_tc_prepare(p, tc, stream));
    r->precision_used = lloyd_tc_scaled(tc) ? FUELG_PREC_SPLIT_BF16_SCALED : p.precision;
  } else {
    FUELG_TRY(keys.alloc(sizeof(uint64_t) * n, stream));
  }

  cudaEvent_t ev0, ev1;
  FUELG_CUDA(cudaEventCreate(&ev0));
  FUELG_CUDA(cudaEventCreate(&ev1));
  FUELG_CUDA(cudaEventRecord(ev0, stream));

  // nearest centre of every point -> lab_new
  auto assign = [&](bool first) -> int {
    if (tc) return lloyd_assign_tc(p, tc, C, first, lab_new.as<int32_t>(), dev_status, stream);
    ExactScanParams sp;
    sp.A = p.X;
    sp.m = n;
    sp.B = C;
    sp.n = k;
    sp.d = d;
    sp.kind = first ? KIND_PAIRWISE : KIND_SQDIST;
    sp.order = p.order;
    sp.metric = METRIC_SQEUCLIDEAN;
    sp.kk = 1;
    FUELG_TRY(exact_topk(sp, keys.as<uint64_t>(), dev_status, stream));
    keys_to_labels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(keys.as<uint64_t>(), n,
                                                                          lab_new.as<int32_t>()); ::fuelg::note_launch();
    FUELG_CUDA(cudaGetLastError());
    return ST_OK;
  };
  // one pass: assign, commit labels, update sums, and (if another pass
  // follows) the centres it will use
  // Tensor-core tier with exact sums: every pass after the first is one
  // fused screen launch (labels committed) and its re-score of the undecided
  // points, then the sum update -- its scatter kernel plans the buckets, its
  // centre kernel also writes the next pass's BF16 centre copies.
  CentrePrep cprep;
  if (tc) cprep = lloyd_tc_centre_prep(tc);
  SumsCommit scv{};
  if (exact) exact_sums_commit_view(es, &scv);
  auto pass = [&](bool first, bool write_centers, int32_t* chg) -> int {
    const bool fused = tc && exact && !first && d <= 1024;
    if (fused) FUELG_TRY(lloyd_tc_pass_fused(p, tc, C, labels, scv, dev_status, stream));
    else FUELG_TRY(assign(first));
    if (p.tol > 0 && write_centers)
      FUELG_CUDA(cudaMemcpyAsync(cold.p, C, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, stream));
    if (fused) return exact_sums_update(es, p.X, write_centers, C, chg, &cprep, stream, true);
    if (exact)
      return exact_sums_step(es, p.X, lab_new.as<int32_t>(), labels, first, write_centers, C, chg, dev_status, stream,
                             tc ? &cprep : nullptr);
    FUELG_CUDA(cudaMemsetAsync(chg, 0, sizeof(int32_t), stream));
    post_assign_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(lab_new.as<int32_t>(), n, labels,
                                                                       first ? 1 : 0, chg); ::fuelg::note_launch();
    FUELG_CUDA(cudaGetLastError());
    if (write_centers) FUELG_TRY(fp64_sums_update(&fs, p.X, labels, C, stream));
    return ST_OK;
  };

  // Middle passes (another pass follows) replay captured CUDA graphs from the
  // second iteration on -- kPassesPerGraph consecutive passes per graph where
  // that many middle passes remain (and no tol check runs between passes), so
  // the screen of each pass can start its point loads while the centre update
  // of the previous one finishes; one pass per graph otherwise.  The first
  // pass and the last few run as plain launches, so the screen kernel's
  // launches are timed individually in the steady state.  Pass j of a graph
  // writes its changed count to slot 2j: a
  // pass that changed nothing leaves sums, centres and labels as they were,
  // so the passes after it in the same graph repeat it exactly and the loop
  // stops at the first such pass (lloyd.rs:197).
  // The two instantiated graphs (one pass, kPassesPerGraph passes) are kept per
  // thread and device between calls: a later call captures its passes again
  // (their arguments differ) and updates the kept graph in place, which costs
  // far less than instantiating it; a graph of another shape is replaced.
  // They belong to the device and context they were made in, and
  // fuelg_release destroys every thread's (a new generation: this thread's
  // handles are then forgotten).
  struct KeptGraphs {
    int dev = -1;
    CUcontext ctx = nullptr;
    uint64_t gen = 0;
    cudaGraphExec_t g[2] = {nullptr, nullptr};
    void drop() {
      for (int i = 0; i < 2; i++) {
        if (g[i]) drop_graph(g[i]);
        g[i] = nullptr;
      }
    }
    ~KeptGraphs() {
      if (gen == cache_generation()) drop();
    }
  };
  thread_local KeptGraphs kept;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    const CUcontext ctx = current_context();
    const uint64_t gen = cache_generation();
    if (kept.gen != gen) {
      kept.g[0] = kept.g[1] = nullptr;
      kept.gen = gen;
    }
    if (kept.dev != dev || kept.ctx != ctx) {
      kept.drop();
      kept.dev = dev;
      kept.ctx = ctx;
    }
  }
  bool ready[2] = {false, false};  // captured and updated for this call
  int64_t graph_launches[2] = {0, 0};
  auto graph_pass = [&](int npass) -> int {
    const int gi = npass == 1 ? 0 : 1;
    if (!ready[gi]) {
      HotTimer* saved = hot_timer();
      hot_timer() = nullptr;
      cudaGraph_t g = nullptr;
      FUELG_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed));
      const int64_t l0 = launch_count();
      int rc = ST_OK;
      for (int j = 0; j < npass && rc == ST_OK; j++) rc = pass(false, true, changed.as<int32_t>() + 2 * j);
      const cudaError_t ce = cudaStreamEndCapture(stream, &g);
      hot_timer() = saved;
      graph_launches[gi] = launch_count() - l0;
      note_launch((int)-graph_launches[gi]);  // counted per replay
      if (rc != ST_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      FUELG_CUDA(ce);
      bool updated = false;
      if (kept.g[gi]) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(kept.g[gi], g, &info) == cudaSuccess;
        if (!updated) {
          cudaGetLastError();
          drop_graph(kept.g[gi]);
          kept.g[gi] = nullptr;
        }
      }
      cudaError_t ie = cudaSuccess;
      if (!updated) {
        ie = cudaGraphInstantiate(&kept.g[gi], g, 0);
        if (ie == cudaSuccess)
          keep_graph(kept.g[gi]);
        else
          kept.g[gi] = nullptr;
      }
      cudaGraphDestroy(g);
      FUELG_CUDA(ie);
      ready[gi] = true;
    }
    FUELG_CUDA(cudaGraphLaunch(kept.g[gi], stream));
    note_launch((int)graph_launches[gi]);
    return ST_OK;
  };

  const float* inertia_centers = C;
  FUELG_TRY(pass(true, p.max_iter > 1, changed.as<int32_t>()));
  int iters = 1;
  // The last kTimedPasses passes before the final one (and the final one)
  // run as plain launches: their screen launches are the ones timed
  // individually (events around a launch inside a graph are not possible).
  constexpr int kTimedPasses = 3;
  while (iters < p.max_iter) {
    if (p.tol <= 0 && iters + kPassesPerGraph + kTimedPasses < p.max_iter) {
      // kPassesPerGraph middle passes in one graph
      FUELG_TRY(graph_pass(kPassesPerGraph));
      const int before = iters;
      iters += kPassesPerGraph;
      if (!p.fixed_iters) {
        FUELG_CUDA(cudaMemcpyAsync(h_changed, changed.p, sizeof(int32_t) * 2 * kPassesPerGraph,
                                   cudaMemcpyDeviceToHost, stream));
        FUELG_CUDA(cudaStreamSynchronize(stream));
        int stop = -1;
        for (int j = 0; j < kPassesPerGraph && stop < 0; j++)
          if (h_changed[2 * j] == 0) stop = j;
        if (stop >= 0) {
          iters = before + stop + 1;
          break;
        }
      }
      continue;
    }
    iters++;
    if (p.tol > 0) {
      frob_kernel<<<1, 256, 0, stream>>>(cold.as<float>(), C, (int64_t)k * d, frob.as<double>()); ::fuelg::note_launch();
      double h2[2];
      FUELG_CUDA(cudaMemcpyAsync(h2, frob.p, sizeof(double) * 2, cudaMemcpyDeviceToHost, stream));
      FUELG_CUDA(cudaStreamSynchronize(stream));
      const double diff = std::sqrt(h2[0]), oldn = std::sqrt(h2[1]);
      const double rel = oldn == 0.0 ? diff : diff / oldn;
      if (rel <= p.tol) {
        // lloyd.rs:147-152: stop before re-assigning; the returned centres are
        // the updated ones, labels and inertia stay those of the previous
        // pass (against the previous centres).
        inertia_centers = cold.as<float>();
        break;
      }
    }
    if (iters + kTimedPasses < p.max_iter) FUELG_TRY(graph_pass(1));
    else FUELG_TRY(pass(false, iters < p.max_iter, changed.as<int32_t>()));
    if (!p.fixed_iters) {
      FUELG_CUDA(cudaMemcpyAsync(h_changed, changed.p, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
      FUELG_CUDA(cudaStreamSynchronize(stream));
      if (*h_changed == 0) break;
    }
  }
  r->iters = iters;
  FUELG_CUDA(cudaEventRecord(ev1, stream));
  if (tc) FUELG_TRY(lloyd_tc_rescored_total(tc, stream, &r->rescored));
  inertia_partial_kernel<<<inert_blocks, 256, 0, stream>>>(p.X, n, d, inertia_centers, labels, inert_part.as<double>()); ::fuelg::note_launch();
  sum_partials_kernel<<<1, 1024, 0, stream>>>(inert_part.as<double>(), inert_blocks, inert.as<double>()); ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  double h_inert = 0.0;
  FUELG_CUDA(cudaMemcpyAsync(&h_inert, inert.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
  FUELG_CUDA(cudaStreamSynchronize(stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  r->kernel_ms = ms;
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  r->inertia = h_inert;
  return ST_OK;
}

}  // namespace fuelg
