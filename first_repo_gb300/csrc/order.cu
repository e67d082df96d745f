// Reference particle order (PSTEP_TRACK_ORDER): the permutation that the
// reference's single-rank Send_Recv leaves in its vectors (particle.cpp:150-311,
// 745-858), kept as a map between the reference's positions and device storage.
//
// One pass per dimension (z, then y, then x). In a pass, with n particles of
// which l leave the slab (SortValid*: x_new > xh or < xl), m = n - l:
//  - front leavers (position < m) are overwritten, in ascending order, by the
//    stayers of the back region [m, n) taken in descending order (the
//    swap-with-last of SortValid*);
//  - the leavers are emitted in the order the swap loop meets them. Writing
//    each leaver's emission index as s = n - a, the "anchor" a is
//      front leaver of rank r:     a = (r == 0) ? n : q_(r-1)
//      back leaver at q:           a = q,  except q == m (only possible when
//                                  no back stayer lies below it): a = E,
//    where q_0 > q_1 > ... are the back stayers and E = q_(F-1) (or n when
//    there are none). Anchors are distinct, so sorting by descending anchor
//    is a scatter into l+1 slots;
//  - FromBuf appends the low-side leavers first (Rbuf0 carries what was sent to
//    the low neighbour, which is this rank), then the high-side ones, each in
//    emission order.
// All work is O(l) apart from one bitmap pass over n, and nothing waits on the
// host: the counts stay on the device and the kernels loop over them.
#include "pstep_internal.cuh"

namespace pstep {

int exclusive_scan(pstep_ctx *h, const int32_t *in, int64_t n, int32_t *out, int32_t *out2);

namespace {

constexpr int kLoopBlocks = 592;  // 4 x 148-152 SMs; the loops below stride over l

// scratch layout inside h->ord_scratch (all int32, length cap + 64 each)
struct OrdBuf {
  uint32_t *bitmap;  // n/32 words
  int32_t *wcount;   // n/32 words
  int32_t *wscan;    // n/32 + 1
  int32_t *lpos;     // leaver positions, ascending
  int32_t *bsphys;   // back stayers (descending) -> storage index
  int32_t *slots;    // l + 1 anchor slots -> storage index of the leaver, -1 empty
  int32_t *newpos;   // l + 1 -> destination position of the slot's leaver
  int32_t *cnt;      // [0] = l, [1] = F, [2] = l_lo
};

__global__ void k_bitmap(const int32_t *__restrict__ phys_of_ref, const uint8_t *__restrict__ code, int bitlo,
                         int64_t n, uint32_t *__restrict__ bitmap, int32_t *__restrict__ wcount) {
  int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nw = (n + 31) / 32;
  if (w >= nw) return;
  uint32_t bits = 0;
  for (int b = 0; b < 32; ++b) {
    int64_t r = w * 32 + b;
    if (r < n && (code[phys_of_ref[r]] >> bitlo) & 3u) bits |= 1u << b;
  }
  bitmap[w] = bits;
  wcount[w] = __popc(bits);
}

__global__ void k_compact_leavers(const uint32_t *__restrict__ bitmap, const int32_t *__restrict__ wscan, int64_t n,
                                  int32_t *__restrict__ lpos, int32_t *__restrict__ cnt) {
  int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nw = (n + 31) / 32;
  if (w == 0) {
    int32_t l = wscan[nw];
    cnt[0] = l;
  }
  if (w >= nw) return;
  uint32_t bits = bitmap[w];
  int32_t o = wscan[w];
  while (bits) {
    int b = __ffs(bits) - 1;
    lpos[o++] = (int32_t)(w * 32 + b);
    bits &= bits - 1;
  }
}

__device__ inline bool is_leaver(const uint32_t *bitmap, int64_t q) { return (bitmap[q >> 5] >> (q & 31)) & 1u; }

// # set bits in [0, q]
__device__ inline int32_t rank_incl(const uint32_t *bitmap, const int32_t *wscan, int64_t q) {
  uint32_t word = bitmap[q >> 5];
  int b = (int)(q & 31);
  uint32_t mask = (b == 31) ? 0xffffffffu : ((1u << (b + 1)) - 1u);
  return wscan[q >> 5] + __popc(word & mask);
}

// F = # leavers below m (binary search in the ascending leaver list)
__global__ void k_front_count(const int32_t *__restrict__ lpos, int64_t n, int32_t *__restrict__ cnt) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int32_t l = cnt[0];
  int64_t m = n - l;
  int32_t lo = 0, hi = l;
  while (lo < hi) {
    int32_t mid = (lo + hi) / 2;
    if (lpos[mid] < m) lo = mid + 1; else hi = mid;
  }
  cnt[1] = lo;
}

// back region [m, n): stayers -> bsphys[rank], leavers -> anchor slot (not the q == m tail case yet)
__global__ void k_back(const uint32_t *__restrict__ bitmap, const int32_t *__restrict__ wscan,
                       const int32_t *__restrict__ phys_of_ref, int64_t n, const int32_t *__restrict__ cnt,
                       int32_t *__restrict__ bsphys, int32_t *__restrict__ slots) {
  const int32_t l = cnt[0];
  const int64_t m = n - l;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < l; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = m + t;
    int32_t above_leavers = l - rank_incl(bitmap, wscan, q);  // leavers with position > q
    if (!is_leaver(bitmap, q)) {
      int64_t r = (n - 1 - q) - above_leavers;                 // back stayers above q
      bsphys[r] = phys_of_ref[q];
    } else if (q != m) {
      slots[q - m] = phys_of_ref[q];
    }
  }
}

// front leavers (rank r < F) and the q == m tail leaver; needs bsphys complete
__global__ void k_front(const int32_t *__restrict__ lpos, const int32_t *__restrict__ phys_of_ref,
                        const uint32_t *__restrict__ bitmap, const int32_t *__restrict__ wscan, int64_t n,
                        const int32_t *__restrict__ cnt, int32_t *__restrict__ slots, int32_t *__restrict__ bspos) {
  const int32_t l = cnt[0], F = cnt[1];
  const int64_t m = n - l;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= F; r += (int64_t)gridDim.x * blockDim.x) {
    if (r < F) {
      // anchor of front leaver r: q_(r-1) (position of the back stayer of rank r-1), or n
      int64_t a = n;
      if (r > 0) a = bspos[r - 1];
      slots[a - m] = phys_of_ref[lpos[r]];
    } else if (l > 0 && is_leaver(bitmap, m)) {
      int64_t E = F > 0 ? bspos[F - 1] : n;
      slots[E - m] = phys_of_ref[m];
    }
  }
  (void)wscan;
}

// positions of the back stayers in descending order (bspos[r] = q_r)
__global__ void k_back_pos(const uint32_t *__restrict__ bitmap, const int32_t *__restrict__ wscan, int64_t n,
                           const int32_t *__restrict__ cnt, int32_t *__restrict__ bspos) {
  const int32_t l = cnt[0];
  const int64_t m = n - l;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < l; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = m + t;
    if (!is_leaver(bitmap, q)) {
      int32_t above_leavers = l - rank_incl(bitmap, wscan, q);
      int64_t r = (n - 1 - q) - above_leavers;
      bspos[r] = (int32_t)q;
    }
  }
}

__device__ inline int32_t block_scan_excl(int32_t v, int32_t *sm, int32_t &total) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t s = lane < (kThreads / 32) ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < (kThreads / 32)) sm[lane] = s;
  }
  __syncthreads();
  int32_t off = w > 0 ? sm[w - 1] : 0;
  total = sm[kThreads / 32 - 1];
  __syncthreads();
  return off + x - v;
}

// one block: walk the slots from the highest anchor down (= emission order), assign
// destinations m + rank among low-side leavers, then m + l_lo + rank among high-side ones
__global__ void k_assign(const int32_t *__restrict__ slots, const uint8_t *__restrict__ code, int bitlo, int64_t n,
                         const int32_t *__restrict__ cnt, int32_t *__restrict__ newpos) {
  __shared__ int32_t sm[kThreads / 32];
  const int32_t l = cnt[0];
  const int64_t m = n - l;
  int32_t nlo = 0;
  for (int pass = 0; pass < 2; ++pass) {
    int32_t carry = 0;
    for (int64_t base = 0; base <= l; base += kThreads) {
      int64_t t = base + threadIdx.x;   // t-th slot from the top
      int64_t s = (int64_t)l - t;       // slot index
      int32_t p = (t <= l) ? slots[s] : -1;
      int lo = 0, hi = 0;
      if (p >= 0) {
        uint32_t c = (code[p] >> bitlo) & 3u;
        lo = (c & 2u) ? 1 : 0;
        hi = (c & 1u) ? 1 : 0;
      }
      int mine = pass == 0 ? lo : hi;
      int32_t total;
      int32_t e = block_scan_excl(mine, sm, total);
      if (mine) newpos[s] = (int32_t)(m + (pass == 0 ? 0 : nlo) + carry + e);
      carry += total;
    }
    if (pass == 0) nlo = carry;
  }
  if (threadIdx.x == 0) ((int32_t *)cnt)[2] = nlo;
}

// apply: front leaver slots receive the back stayers; leavers go to their destinations
__global__ void k_apply(const int32_t *__restrict__ lpos, const int32_t *__restrict__ bsphys,
                        int32_t *__restrict__ slots, const int32_t *__restrict__ newpos, int64_t n,
                        const int32_t *__restrict__ cnt, int32_t *__restrict__ phys_of_ref,
                        int32_t *__restrict__ ref_of_phys) {
  const int32_t l = cnt[0], F = cnt[1];
  const int64_t m = n - l;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= l; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < F) {
      int32_t p = lpos[t];
      int32_t ph = bsphys[t];
      phys_of_ref[p] = ph;
      ref_of_phys[ph] = p;
    }
    int32_t ph = slots[t];
    slots[t] = -1;
    if (ph >= 0) {
      int32_t dst = newpos[t];
      phys_of_ref[dst] = ph;
      ref_of_phys[ph] = dst;
    }
  }
  (void)m;
}

__global__ void k_iota(int32_t *__restrict__ a, int32_t *__restrict__ b, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    a[i] = (int32_t)i;
    b[i] = (int32_t)i;
  }
}

OrdBuf bufs(pstep_ctx *h) {
  OrdBuf b;
  int64_t L = h->ord_scratch_len;
  int32_t *base = h->ord_scratch;
  b.bitmap = (uint32_t *)(base);
  b.wcount = base + L;
  b.wscan = base + 2 * L;
  b.lpos = base + 3 * L;
  b.bsphys = base + 4 * L;
  b.slots = base + 5 * L;
  b.newpos = base + 6 * L;
  b.cnt = h->ord_count;
  return b;
}

}  // namespace

int64_t order_scratch_words(int64_t cap) { return 7 * (cap + 64); }

int order_init(pstep_ctx *h) {
  if (h->np == 0) return PSTEP_OK;
  k_iota<<<(int)((h->np + kThreads - 1) / kThreads), kThreads, 0, h->stream>>>(h->ref_of_phys, h->phys_of_ref, h->np);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

// the three Send_Recv passes (z, y, x) of one stage
int order_passes(pstep_ctx *h) {
  const int64_t n = h->np;
  if (n == 0) return PSTEP_OK;
  OrdBuf b = bufs(h);
  const int64_t nw = (n + 31) / 32;
  // back-stayer positions live in wcount, which is dead once the word counts are scanned
  int32_t *bspos = b.wcount;
  for (int d = 2; d >= 0; --d) {
    const int bitlo = 2 * d;
    k_bitmap<<<(int)((nw + kThreads - 1) / kThreads), kThreads, 0, h->stream>>>(h->phys_of_ref, h->leave_code, bitlo,
                                                                               n, b.bitmap, b.wcount);
    PSTEP_LAUNCHED(h);
    int rc = exclusive_scan(h, b.wcount, nw, b.wscan, nullptr);
    if (rc) return rc;
    k_compact_leavers<<<(int)((nw + kThreads - 1) / kThreads), kThreads, 0, h->stream>>>(b.bitmap, b.wscan, n, b.lpos,
                                                                                        b.cnt);
    PSTEP_LAUNCHED(h);
    k_front_count<<<1, 32, 0, h->stream>>>(b.lpos, n, b.cnt);
    PSTEP_LAUNCHED(h);
    // slots are all -1 on entry: set once at creation, restored by k_apply after use
    k_back<<<kLoopBlocks, kThreads, 0, h->stream>>>(b.bitmap, b.wscan, h->phys_of_ref, n, b.cnt, b.bsphys, b.slots);
    PSTEP_LAUNCHED(h);
    k_back_pos<<<kLoopBlocks, kThreads, 0, h->stream>>>(b.bitmap, b.wscan, n, b.cnt, bspos);
    PSTEP_LAUNCHED(h);
    k_front<<<kLoopBlocks, kThreads, 0, h->stream>>>(b.lpos, h->phys_of_ref, b.bitmap, b.wscan, n, b.cnt, b.slots,
                                                     bspos);
    PSTEP_LAUNCHED(h);
    k_assign<<<1, kThreads, 0, h->stream>>>(b.slots, h->leave_code, bitlo, n, b.cnt, b.newpos);
    PSTEP_LAUNCHED(h);
    k_apply<<<kLoopBlocks, kThreads, 0, h->stream>>>(b.lpos, b.bsphys, b.slots, b.newpos, n, b.cnt, h->phys_of_ref,
                                                     h->ref_of_phys);
    PSTEP_LAUNCHED(h);
  }
  return PSTEP_OK;
}

}  // namespace pstep
