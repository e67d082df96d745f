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

__global__ void k_count(const uint32_t *__restrict__ keys, int64_t n, int32_t *__restrict__ counts) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < n;
  uint32_t node = valid ? (keys[i] >> 3) : 0xffffffffu;
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
  __shared__ int32_t sm[kThreads / 32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    int64_t i = base + q;
    v[q] = i < n ? in[i] : 0;
    s += v[q];
  }
  int32_t total;
  int32_t e = block_excl_scan(s, sm, total) + block_off[blockIdx.x];
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

__global__ void k_scatter(const uint32_t *__restrict__ keys, int64_t n, int32_t *__restrict__ cursor,
                          int32_t *__restrict__ sidx) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < n;
  uint32_t node = valid ? (keys[i] >> 3) : 0xffffffffu;
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

// Order every node's segment by the secondary key (insertion sort; segments are short).
__global__ void k_segsort(const int32_t *__restrict__ cell_start, int64_t gsize, int32_t *__restrict__ sidx,
                          const int32_t *__restrict__ sortkey) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= gsize) return;
  int32_t a = cell_start[c], b = cell_start[c + 1];
  if (b - a < 2) return;
  for (int32_t p = a + 1; p < b; ++p) {
    int32_t v = sidx[p];
    int32_t kv = sortkey ? sortkey[v] : v;
    int32_t q = p - 1;
    while (q >= a) {
      int32_t u = sidx[q];
      int32_t ku = sortkey ? sortkey[u] : u;
      if (ku <= kv) break;
      sidx[q + 1] = u;
      --q;
    }
    sidx[q + 1] = v;
  }
}

template <typename T>
__global__ void k_gather(const T *__restrict__ src, const int32_t *__restrict__ idx, int64_t n, T *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

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

int sort_by_node(pstep_ctx *h, const uint32_t *keys, Csr &out) {
  const int64_t gsize = h->geom.gsize;
  PSTEP_CUDA(cudaMemsetAsync(h->counts, 0, sizeof(int32_t) * gsize, h->stream));
  if (h->np > 0) {
    k_count<<<blocks_for(h->np), kThreads, 0, h->stream>>>(keys, h->np, h->counts);
    PSTEP_LAUNCHED(h);
  }
  int rc = exclusive_scan(h, h->counts, gsize, out.cell_start, h->cursor);
  if (rc) return rc;
  if (h->np > 0) {
    k_scatter<<<blocks_for(h->np), kThreads, 0, h->stream>>>(keys, h->np, h->cursor, out.sidx);
    PSTEP_LAUNCHED(h);
    const int32_t *sk = (h->cfg.flags & PSTEP_TRACK_ORDER) ? h->ref_of_phys : nullptr;
    k_segsort<<<blocks_for(gsize), kThreads, 0, h->stream>>>(out.cell_start, gsize, out.sidx, sk);
    PSTEP_LAUNCHED(h);
  }
  out.identity = 0;
  return PSTEP_OK;
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
