// Deterministic counting sort of particles by node key, giving the CSR that the
// deposit gathers walk (cell_start over the ghosted node grid + sorted particle
// indices), and the per-step reorder of particle storage by that sort.
//
// Order within a node is fixed by an explicit secondary key (the particle's
// position in the reference's vectors, or its storage index), so the CSR -- and
// every sum taken over it -- is identical from run to run.
#include "pstep_internal.cuh"

namespace pstep {
namespace {

constexpr int kScanItems = 16;                       // per thread
constexpr int kScanTile = kThreads * kScanItems;     // per block

__global__ void k_count(const uint32_t *__restrict__ keys, int shift, int64_t n, int32_t *__restrict__ counts) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < n;
  uint32_t node = valid ? (keys[i] >> shift) : 0xffffffffu;
  // warp-aggregated increments: lanes with the same node add once
  unsigned active = __ballot_sync(0xffffffffu, valid);
  if (!valid) return;
  unsigned peers = __match_any_sync(active, node);
  int leader = __ffs(peers) - 1;
  if ((int)(threadIdx.x & 31) == leader) atomicAdd(&counts[node], __popc(peers));
}

__device__ inline int32_t block_excl_scan(int32_t v, int32_t *smem, int32_t &total) {
  // smem: kThreads/32 ints
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t s = lane < (kThreads / 32) ? smem[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < (kThreads / 32)) smem[lane] = s;
  }
  __syncthreads();
  int32_t warp_off = w > 0 ? smem[w - 1] : 0;
  total = smem[kThreads / 32 - 1];
  __syncthreads();
  return warp_off + x - v;
}

// phase 1: per-tile sums
__global__ void k_scan_reduce(const int32_t *__restrict__ in, int64_t n, int32_t *__restrict__ block_sums) {
  __shared__ int32_t sm[kThreads / 32];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int32_t s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    int64_t i = base + (int64_t)q * kThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  int32_t total;
  block_excl_scan(s, sm, total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// phase 2: exclusive scan of the tile sums (one block, sequential over chunks)
__global__ void k_scan_blocks(int32_t *__restrict__ sums, int64_t nb) {
  __shared__ int32_t sm[kThreads / 32];
  int32_t carry = 0;
  for (int64_t base = 0; base < nb; base += kThreads) {
    int64_t i = base + threadIdx.x;
    int32_t v = i < nb ? sums[i] : 0;
    int32_t total;
    int32_t e = block_excl_scan(v, sm, total);
    if (i < nb) sums[i] = carry + e;
    carry += total;
  }
}

// phase 3: per-tile exclusive scan in blocked order; writes out[0..n] (out[n] = total)
__global__ void k_scan_apply(const int32_t *__restrict__ in, int64_t n, const int32_t *__restrict__ block_off,
                             int32_t *__restrict__ out, int32_t *__restrict__ out2) {
  static_assert(kScanItems % 4 == 0, "whole 16-byte vectors per thread");
  __shared__ int32_t sm[kThreads / 32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  // whole tiles move as 16-byte vectors (the arrays are 16-byte aligned and base is a
  // multiple of 4 elements); the ragged last tile element by element
  const bool whole = base + kScanItems <= n && (((uintptr_t)in | (uintptr_t)out | (uintptr_t)out2) & 15) == 0;
  int32_t v[kScanItems];
  int32_t s = 0;
  if (whole) {
#pragma unroll
    for (int q = 0; q < kScanItems; q += 4) {
      const int4 a = *reinterpret_cast<const int4 *>(in + base + q);
      v[q] = a.x; v[q + 1] = a.y; v[q + 2] = a.z; v[q + 3] = a.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) v[q] = base + q < n ? in[base + q] : 0;
  }
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) s += v[q];
  int32_t total;
  int32_t e = block_excl_scan(s, sm, total) + block_off[blockIdx.x];
  if (whole) {
#pragma unroll
    for (int q = 0; q < kScanItems; q += 4) {
      int4 o;
      o.x = e; e += v[q];
      o.y = e; e += v[q + 1];
      o.z = e; e += v[q + 2];
      o.w = e; e += v[q + 3];
      *reinterpret_cast<int4 *>(out + base + q) = o;
      if (out2) *reinterpret_cast<int4 *>(out2 + base + q) = o;
    }
    if (base + kScanItems == n) out[n] = e;
  } else {
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
      int64_t i = base + q;
      if (i < n) {
        out[i] = e;
        if (out2) out2[i] = e;
      }
      e += v[q];
      if (i == n - 1) out[n] = e;
    }
  }
}

__global__ void k_scatter(const uint32_t *__restrict__ keys, int shift, int64_t n, int32_t *__restrict__ cursor,
                          int32_t *__restrict__ sidx) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < n;
  uint32_t node = valid ? (keys[i] >> shift) : 0xffffffffu;
  unsigned active = __ballot_sync(0xffffffffu, valid);
  if (!valid) return;
  unsigned peers = __match_any_sync(active, node);
  int lane = threadIdx.x & 31;
  int leader = __ffs(peers) - 1;
  int32_t basepos = 0;
  if (lane == leader) basepos = atomicAdd(&cursor[node], __popc(peers));
  basepos = __shfl_sync(peers, basepos, leader);
  int32_t rank = __popc(peers & ((1u << lane) - 1u));
  sidx[basepos + rank] = (int32_t)i;
}

// Order every node's segment by a 64-bit secondary key: short segments (<= kSmallSeg)
// by one thread (insertion sort), longer ones are listed for k_segsort_big.
constexpr int kSmallSeg = 16;
constexpr int kBigSegMax = 16384;  // per-node particles sortable on chip (12 B each in shared memory)

__device__ inline uint64_t seckey(const int32_t *__restrict__ order, const uint32_t *__restrict__ keys, int32_t v) {
  // an explicit secondary key (reference position, or particle id), else (h bits, storage index)
  if (order) return (uint64_t)(uint32_t)order[v];
  return ((uint64_t)(keys[v] & 7u) << 32) | (uint32_t)v;
}

__global__ void k_segsort_small(const int32_t *__restrict__ cell_start, int64_t gsize, int32_t *__restrict__ sidx,
                                const int32_t *__restrict__ order, const uint32_t *__restrict__ keys,
                                int32_t *__restrict__ big_list, int32_t *__restrict__ big_count,
                                int32_t *__restrict__ err) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= gsize) return;
  int32_t a = cell_start[c], b = cell_start[c + 1];
  int32_t len = b - a;
  if (len < 2) return;
  if (len > kSmallSeg) {
    if (len > kBigSegMax) atomicOr(err, kErrCapacity);
    int32_t slot = atomicAdd(big_count, 1);
    big_list[slot] = (int32_t)c;
    return;
  }
  int32_t v[kSmallSeg];
  uint64_t k[kSmallSeg];
  for (int q = 0; q < len; ++q) {
    v[q] = sidx[a + q];
    k[q] = seckey(order, keys, v[q]);
  }
  for (int p = 1; p < len; ++p) {
    int32_t vv = v[p];
    uint64_t kv = k[p];
    int q = p - 1;
    while (q >= 0 && k[q] > kv) {
      k[q + 1] = k[q];
      v[q + 1] = v[q];
      --q;
    }
    k[q + 1] = kv;
    v[q + 1] = vv;
  }
  for (int q = 0; q < len; ++q) sidx[a + q] = v[q];
}

// one block per listed long segment: bitonic sort in shared memory
__global__ void __launch_bounds__(512) k_segsort_big(const int32_t *__restrict__ cell_start, int32_t *__restrict__ sidx,
                                                     const int32_t *__restrict__ order,
                                                     const uint32_t *__restrict__ keys,
                                                     const int32_t *__restrict__ big_list,
                                                     const int32_t *__restrict__ big_count) {
  extern __shared__ unsigned char smraw[];
  uint64_t *sk = (uint64_t *)smraw;
  int32_t *sv = (int32_t *)(sk + kBigSegMax);
  const int32_t nbig = *big_count;
  for (int32_t w = blockIdx.x; w < nbig; w += gridDim.x) {
    const int32_t c = big_list[w];
    const int32_t a = cell_start[c], b = cell_start[c + 1];
    const int32_t len = b - a;
    if (len > kBigSegMax) continue;  // reported by k_segsort_small
    int32_t m = 1;
    while (m < len) m <<= 1;
    for (int32_t q = threadIdx.x; q < m; q += blockDim.x) {
      if (q < len) {
        int32_t v = sidx[a + q];
        sv[q] = v;
        sk[q] = seckey(order, keys, v);
      } else {
        sv[q] = -1;
        sk[q] = ~0ull;
      }
    }
    __syncthreads();
    for (int32_t kk = 2; kk <= m; kk <<= 1) {
      for (int32_t j = kk >> 1; j > 0; j >>= 1) {
        for (int32_t q = threadIdx.x; q < m; q += blockDim.x) {
          int32_t r = q ^ j;
          if (r > q) {
            bool up = (q & kk) == 0;
            uint64_t x = sk[q], y = sk[r];
            if ((x > y) == up) {
              sk[q] = y; sk[r] = x;
              int32_t t = sv[q]; sv[q] = sv[r]; sv[r] = t;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int32_t q = threadIdx.x; q < len; q += blockDim.x) sidx[a + q] = sv[q];
    __syncthreads();
  }
}

}  // namespace

template <typename T>
__global__ void k_gather(const T *__restrict__ src, const int32_t *__restrict__ idx, int64_t n, T *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}
template __global__ void k_gather<float>(const float *, const int32_t *, int64_t, float *);
template __global__ void k_gather<uint32_t>(const uint32_t *, const int32_t *, int64_t, uint32_t *);
template __global__ void k_gather<int32_t>(const int32_t *, const int32_t *, int64_t, int32_t *);

namespace {

__global__ void k_invert(const int32_t *__restrict__ ref_of_phys, int64_t n, int32_t *__restrict__ phys_of_ref) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) phys_of_ref[ref_of_phys[i]] = (int32_t)i;
}

inline int blocks_for(int64_t n, int per = kThreads) { return (int)((n + per - 1) / per); }

}  // namespace

int exclusive_scan(pstep_ctx *h, const int32_t *in, int64_t n, int32_t *out, int32_t *out2) {
  int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb > h->scan_nblocks) {
    snprintf(h->err, sizeof h->err, "scan scratch too small");
    return PSTEP_ERR_STATE;
  }
  k_scan_reduce<<<(int)nb, kThreads, 0, h->stream>>>(in, n, h->scan_blocks);
  PSTEP_LAUNCHED(h);
  k_scan_blocks<<<1, kThreads, 0, h->stream>>>(h->scan_blocks, nb);
  PSTEP_LAUNCHED(h);
  k_scan_apply<<<(int)nb, kThreads, 0, h->stream>>>(in, n, h->scan_blocks, out, out2);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

int64_t scan_blocks_needed(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

// Counting sort of the h->np particles by (keys[i] >> shift) into nkeys buckets:
// cell_start[0..nkeys] and sidx, every bucket ordered by the secondary key.
int csr_sort(pstep_ctx *h, const uint32_t *keys, int shift, int64_t nkeys, const int32_t *order, int32_t *cell_start,
             int32_t *sidx, int order_within) {
  PSTEP_CUDA(cudaMemsetAsync(h->counts, 0, sizeof(int32_t) * nkeys, h->stream));
  if (h->np > 0) {
    k_count<<<blocks_for(h->np), kThreads, 0, h->stream>>>(keys, shift, h->np, h->counts);
    PSTEP_LAUNCHED(h);
  }
  int rc = exclusive_scan(h, h->counts, nkeys, cell_start, h->cursor);
  if (rc) return rc;
  if (h->np > 0) {
    k_scatter<<<blocks_for(h->np), kThreads, 0, h->stream>>>(keys, shift, h->np, h->cursor, sidx);
    PSTEP_LAUNCHED(h);
    if (!order_within) return PSTEP_OK;
    PSTEP_CUDA(cudaMemsetAsync(h->big_count, 0, sizeof(int32_t), h->stream));
    k_segsort_small<<<blocks_for(nkeys), kThreads, 0, h->stream>>>(cell_start, nkeys, sidx, order, keys, h->big_list,
                                                                    h->big_count, h->err_word);
    PSTEP_LAUNCHED(h);
    const size_t smem = (size_t)kBigSegMax * (sizeof(uint64_t) + sizeof(int32_t));
    PSTEP_CUDA(cudaFuncSetAttribute(k_segsort_big, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_segsort_big<<<2 * h->num_sms, 512, smem, h->stream>>>(cell_start, sidx, order, keys, h->big_list, h->big_count);
    PSTEP_LAUNCHED(h);
  }
  return PSTEP_OK;
}

// the cell-start table of keys already in non-decreasing order (no permutation needed):
// the counts and their exclusive scan, as csr_sort makes them
int csr_count(pstep_ctx *h, const uint32_t *keys, int shift, int64_t nkeys, int32_t *cell_start) {
  PSTEP_CUDA(cudaMemsetAsync(h->counts, 0, sizeof(int32_t) * nkeys, h->stream));
  if (h->np > 0) {
    k_count<<<blocks_for(h->np), kThreads, 0, h->stream>>>(keys, shift, h->np, h->counts);
    PSTEP_LAUNCHED(h);
  }
  return exclusive_scan(h, h->counts, nkeys, cell_start, nullptr);
}

int sort_by_node(pstep_ctx *h, const uint32_t *keys, Csr &out) {
  const int32_t *order =
      ((h->cfg.flags & PSTEP_TRACK_ORDER) && (h->cfg.flags & PSTEP_REFERENCE_SUMS)) ? h->ref_of_phys : nullptr;
  int rc = csr_sort(h, keys, 3, h->geom.gsize, order, out.cell_start, out.sidx, 1);
  out.identity = 0;
  return rc;
}

// Reorder particle storage by csr_prev.sidx (the sort of the positions the next
// stage starts from): every per-particle array is gathered through the
// permutation into scratch and the pointers swapped.
int f64_reorder(pstep_ctx *h) {
  const int64_t n = h->np;
  if (n == 0) return PSTEP_OK;
  const int32_t *idx = h->csr_prev.sidx;
  const int bl = blocks_for(n);
  double *tmp = (double *)h->perm_tmp;
  // each array is gathered into the free buffer, which then takes the array's place
  auto gd = [&](double *&arr) {
    k_gather<double><<<bl, kThreads, 0, h->stream>>>(arr, idx, n, tmp);
    h->launches++;
    double *old = arr;
    arr = tmp;
    tmp = old;
  };
  for (int q = 0; q < 7; ++q) gd(h->s.base[q]);
  gd(h->s.rhs_t);
  if (h->s.itp) gd(h->s.itp);
  for (int d = 0; d < 3; ++d) gd(h->s.frac_prev[d]);
  h->perm_tmp = tmp;
  PSTEP_LAUNCHED(h);
  h->launches--;
  int32_t *itmp = (int32_t *)h->perm_tmp;
  // int arrays through the same scratch (as int32), copied back
  k_gather<int32_t><<<bl, kThreads, 0, h->stream>>>(h->s.flag, idx, n, itmp);
  PSTEP_LAUNCHED(h);
  PSTEP_CUDA(cudaMemcpyAsync(h->s.flag, itmp, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, h->stream));
  k_gather<uint32_t><<<bl, kThreads, 0, h->stream>>>(h->s.key_prev, idx, n, (uint32_t *)itmp);
  PSTEP_LAUNCHED(h);
  PSTEP_CUDA(cudaMemcpyAsync(h->s.key_prev, itmp, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, h->stream));
  if (h->cfg.flags & PSTEP_TRACK_ORDER) {
    k_gather<int32_t><<<bl, kThreads, 0, h->stream>>>(h->ref_of_phys, idx, n, itmp);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaMemcpyAsync(h->ref_of_phys, itmp, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, h->stream));
    k_invert<<<bl, kThreads, 0, h->stream>>>(h->ref_of_phys, n, h->phys_of_ref);
    PSTEP_LAUNCHED(h);
  }
  h->csr_prev.identity = 1;
  return PSTEP_OK;
}

}  // namespace pstep
