// FP32 mixed form of the particle step (PSTEP_FP32).
//
// Storage (structure of arrays, 32 B per particle and set):
//   cell   uint32  trunc cell, 10 bits per dimension (i | j << 10 | k << 20)
//   ox,oy,oz float offset inside the cell in cell units, [0, 1)
//   u,v,w,T  float
// for the sets base, *_int, *_new and *_np1, plus RHS_T, 1/tau_p and the id.
// A position is x = (i + ox) * dx; the reference's trunc cell is i and its
// fractional part ox, its round() node is i + (ox >= 0.5). The periodic wrap is
// the cell index modulo n, so positions never leave [0, L).
//
// Temperatures (particle and gas) are stored as offsets from a reference
// temperature t_ref taken from the first data the handle sees (the first
// particle's T at upload, or the first interior cell of the first bound T
// field). The heat-transfer RHS is a difference of two nearly equal
// temperatures, (Tg - T_p); with offsets of size |T - t_ref| the fp32 rounding
// of that difference shrinks by the same factor (the trilinear weights sum to
// one, so interpolating the offset is exact algebra).
//
// Arithmetic: fields, offsets and the ODE in fp32. Deposits are summed exactly
// in 64-bit fixed point (each fp32 contribution scaled by a power of two chosen
// from device-side bounds, so no sum can overflow) and converted to fp64 with
// integer operations; integer addition is associative, so the result does not
// depend on the order of the adds and is the same on every run. Every brick of
// 8^3 cells is owned by one CTA that walks the particles of its cells and a
// two-cell halo (particles are sorted by cell once per step and move less than
// a cell per stage), accumulating in shared memory: no global atomics, no
// per-stage sort. The interior mean of RHS_Part_Temp is an fp64 reduction.
//
// FP64 on GB300 runs at a small fraction of the fp32 rate, so this form keeps
// fp64 out of every per-particle operation: the only fp64 arithmetic left is
// the balance reduction over the grid.
#include <stdlib.h>
#include "pstep_internal.cuh"

namespace pstep {
int interior_mean(pstep_ctx *h, const double *f, double *out_dev);
int exclusive_scan(pstep_ctx *h, const int32_t *in, int64_t n, int32_t *out, int32_t *out2);
int fold_fields(pstep_ctx *h, double *const *f, int nf, int refresh);
}  // namespace pstep

namespace pstep {

enum { SBASE = 0, SINT = 1, SNEW = 2, SNP1 = 3 };
constexpr int kBr = 8;            // brick edge (cells) for the sort order and the deposit CTAs
constexpr int kHalo = 2;          // source cells beyond the brick
constexpr int kSrc = kBr + 2 * kHalo;
constexpr int kDepThreads = 256;
constexpr int kMaxN = 1024;       // 10 bits per cell coordinate

struct Set32 {
  uint32_t *cell;
  float *o[3];
  float *v[4];  // u v w T
};

struct F32Form {
  Set32 set[4];
  float *rhs_t;
  float *itp;      // per-particle 1/tau_p or nullptr
  float *rhs_u[3];
  float *uf[3], *tf;  // fp32 ghosted copies of the bound fields
  uint32_t *key;      // brick-major cell id of the base position
  int32_t *cell_start;  // n^3 + 1, brick-major order (per step)
  int32_t *sidx;
  float *tmpf;        // permutation scratch
  uint32_t *bounds;   // [0..2] max |RHS_u| per component (float bits), [3] max |RHS_T|, [4] max per-cell count
  int32_t *se;        // fixed-point scale exponents per field
  int sorted;
  int tref_set;
  double tref;        // temperature reference (see above)
};

namespace {

__host__ __device__ inline uint32_t pack(int i, int j, int k) { return (uint32_t)i | ((uint32_t)j << 10) | ((uint32_t)k << 20); }
__host__ __device__ inline int ci_(uint32_t c) { return (int)(c & 1023u); }
__host__ __device__ inline int cj_(uint32_t c) { return (int)((c >> 10) & 1023u); }
__host__ __device__ inline int ck_(uint32_t c) { return (int)(c >> 20); }

// brick-major id of interior cell (i,j,k)
__host__ __device__ inline uint32_t brick_id(const Geom &G, int i, int j, int k) {
  const int nbx = G.n[0] / kBr, nby = G.n[1] / kBr;
  const int bx = i / kBr, by = j / kBr, bz = k / kBr;
  const int lx = i % kBr, ly = j % kBr, lz = k % kBr;
  return ((uint32_t)((bz * nby + by) * nbx + bx) * (kBr * kBr * kBr)) + (uint32_t)((lz * kBr + ly) * kBr + lx);
}

__device__ inline int wrapi(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// offset o in cell units on top of cell index i: renormalise to [0, 1) and wrap
__device__ inline void renorm(int &i, float &o, int n) {
  float f = floorf(o);
  o -= f;
  i += (int)f;
  if (o >= 1.0f) { o -= 1.0f; i += 1; }
  i = wrapi(i, n);
}

__device__ inline long long glin3(const Geom &G, int i, int j, int k) { return glin(G, i, j, k); }

__device__ inline void atomic_max_abs(uint32_t *w, float v) {
  // non-negative floats order like their bit patterns
  atomicMax(w, __float_as_uint(fabsf(v)));
}

struct C32 {
  float dt_pre, dt_post, dt_pre_is, dt_post_is;
  float dpre_idx[3], dpost_idx[3];  // dt*pre/dx, dt*post/dx per dimension
  float itp, g[3], alpha, itth;
};

template <int K>
__global__ void __launch_bounds__(256) k_advance32(Geom G, F32Form f, C32 c, int twc, int64_t n,
                                                   int32_t *__restrict__ err) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float mu0 = 0.f, mu1 = 0.f, mu2 = 0.f, mt = 0.f;
  if (p < n) {
    const Set32 &B = f.set[SBASE];
    const Set32 &I = (K == 0) ? f.set[SBASE] : f.set[SINT];
    const Set32 &A = (K == 0) ? f.set[SBASE] : f.set[SNP1];
    const uint32_t cb = B.cell[p];
    const uint32_t cint = I.cell[p];
    uint32_t cacc = A.cell[p];
    float ob[3], oin[3], oac[3], vb[4], vin[4], vac[4];
#pragma unroll
    for (int d = 0; d < 3; ++d) { ob[d] = B.o[d][p]; oin[d] = I.o[d][p]; oac[d] = A.o[d][p]; }
#pragma unroll
    for (int q = 0; q < 4; ++q) { vb[q] = B.v[q][p]; vin[q] = I.v[q][p]; vac[q] = A.v[q][p]; }
    const float rhs_t_old = f.rhs_t[p];
    const float itp = f.itp ? f.itp[p] : c.itp;

    // face-normal interpolation at x_int (particle.cpp:340-360)
    const int ii = ci_(cint) + 1, jj = cj_(cint) + 1, kk = ck_(cint) + 1;
    const float xl = oin[0], yl = oin[1], zl = oin[2];
    const float ug = xl * f.uf[0][glin3(G, ii + 1, jj, kk)] + (1.f - xl) * f.uf[0][glin3(G, ii, jj, kk)];
    const float vg = yl * f.uf[1][glin3(G, ii, jj + 1, kk)] + (1.f - yl) * f.uf[1][glin3(G, ii, jj, kk)];
    const float wg = zl * f.uf[2][glin3(G, ii, jj, kk + 1)] + (1.f - zl) * f.uf[2][glin3(G, ii, jj, kk)];
    const float gas[3] = {ug, vg, wg};

    // positions (particle.cpp:314-338) in cell units
    int ia[3] = {ci_(cacc), cj_(cacc), ck_(cacc)};
    int ib[3] = {ci_(cb), cj_(cb), ck_(cb)};
    int in_[3];
    float on[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      oac[d] += c.dpost_idx[d] * vin[d];
      renorm(ia[d], oac[d], G.n[d]);
      if (K != 3) {
        on[d] = ob[d] + c.dpre_idx[d] * vin[d];
        in_[d] = ib[d];
        renorm(in_[d], on[d], G.n[d]);
      } else {
        on[d] = oac[d];
        in_[d] = ia[d];
      }
    }
    // velocity and temperature (particle.cpp:362-399, 480-496)
    float rhs[3], vn[4];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      rhs[d] = (gas[d] - vin[d]) * itp;
      vac[d] += c.dt_post * (rhs[d] + c.g[d]);
      vn[d] = (K != 3) ? vb[d] + c.dt_pre * (rhs[d] + c.g[d]) : vac[d];
    }
    vac[3] += c.dt_post_is * (rhs_t_old + c.alpha);
    vn[3] = (K != 3) ? vb[3] + c.dt_pre_is * (rhs_t_old + c.alpha) : vac[3];

    // trilinear T at x_new (particle.cpp:430-456): node = cell + h, x_l = o - h + 1/2
    const int hx = on[0] >= 0.5f, hy = on[1] >= 0.5f, hz = on[2] >= 0.5f;
    const float tx = on[0] - hx + 0.5f, ty = on[1] - hy + 0.5f, tz = on[2] - hz + 0.5f;
    const int ni = in_[0] + hx + 1, nj = in_[1] + hy + 1, nk = in_[2] + hz + 1;  // ghosted node
    const float *T = f.tf;
    const float tg = tx * ty * tz * T[glin3(G, ni, nj, nk)] + (1.f - tx) * ty * tz * T[glin3(G, ni - 1, nj, nk)] +
                     tx * (1.f - ty) * tz * T[glin3(G, ni, nj - 1, nk)] + tx * ty * (1.f - tz) * T[glin3(G, ni, nj, nk - 1)] +
                     (1.f - tx) * (1.f - ty) * tz * T[glin3(G, ni - 1, nj - 1, nk)] +
                     (1.f - tx) * ty * (1.f - tz) * T[glin3(G, ni - 1, nj, nk - 1)] +
                     tx * (1.f - ty) * (1.f - tz) * T[glin3(G, ni, nj - 1, nk - 1)] +
                     (1.f - tx) * (1.f - ty) * (1.f - tz) * T[glin3(G, ni - 1, nj - 1, nk - 1)];
    const float rhs_t_new = (tg - vn[3]) * c.itth;
    if (!isfinite(rhs_t_new) || !isfinite(vn[0]) || !isfinite(vn[1]) || !isfinite(vn[2]) || !isfinite(on[0]) ||
        !isfinite(on[1]) || !isfinite(on[2]))
      atomicOr(err, kErrNonFinite);

    // stores
    const Set32 &N = f.set[SNEW];
    const Set32 &P = f.set[SNP1];
    N.cell[p] = pack(in_[0], in_[1], in_[2]);
    P.cell[p] = pack(ia[0], ia[1], ia[2]);
#pragma unroll
    for (int d = 0; d < 3; ++d) { N.o[d][p] = on[d]; P.o[d][p] = oac[d]; }
#pragma unroll
    for (int q = 0; q < 4; ++q) { N.v[q][p] = vn[q]; P.v[q][p] = vac[q]; }
    if (twc) {
#pragma unroll
      for (int d = 0; d < 3; ++d) f.rhs_u[d][p] = rhs[d];
    }
    f.rhs_t[p] = rhs_t_new;
    mu0 = rhs[0]; mu1 = rhs[1]; mu2 = rhs[2]; mt = rhs_t_new;
  }
  // bounds for the fixed-point scales (order-independent maxima)
  float a0 = fabsf(mu0), a1 = fabsf(mu1), a2 = fabsf(mu2), a3 = fabsf(mt);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 = fmaxf(a0, __shfl_xor_sync(0xffffffffu, a0, o));
    a1 = fmaxf(a1, __shfl_xor_sync(0xffffffffu, a1, o));
    a2 = fmaxf(a2, __shfl_xor_sync(0xffffffffu, a2, o));
    a3 = fmaxf(a3, __shfl_xor_sync(0xffffffffu, a3, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_abs(&f.bounds[0], a0);
    atomic_max_abs(&f.bounds[1], a1);
    atomic_max_abs(&f.bounds[2], a2);
    atomic_max_abs(&f.bounds[3], a3);
  }
}

// the prime (grid.cpp:223-226) at the base positions: Tg, RHS_T
__global__ void k_prime32(Geom G, F32Form f, float itth, int64_t n) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float mt = 0.f;
  if (p < n) {
    const Set32 &B = f.set[SBASE];
    const uint32_t cb = B.cell[p];
    const float o0 = B.o[0][p], o1 = B.o[1][p], o2 = B.o[2][p];
    const int hx = o0 >= 0.5f, hy = o1 >= 0.5f, hz = o2 >= 0.5f;
    const float tx = o0 - hx + 0.5f, ty = o1 - hy + 0.5f, tz = o2 - hz + 0.5f;
    const int ni = ci_(cb) + hx + 1, nj = cj_(cb) + hy + 1, nk = ck_(cb) + hz + 1;
    const float *T = f.tf;
    const float tg = tx * ty * tz * T[glin3(G, ni, nj, nk)] + (1.f - tx) * ty * tz * T[glin3(G, ni - 1, nj, nk)] +
                     tx * (1.f - ty) * tz * T[glin3(G, ni, nj - 1, nk)] + tx * ty * (1.f - tz) * T[glin3(G, ni, nj, nk - 1)] +
                     (1.f - tx) * (1.f - ty) * tz * T[glin3(G, ni - 1, nj - 1, nk)] +
                     (1.f - tx) * ty * (1.f - tz) * T[glin3(G, ni - 1, nj, nk - 1)] +
                     tx * (1.f - ty) * (1.f - tz) * T[glin3(G, ni, nj - 1, nk - 1)] +
                     (1.f - tx) * (1.f - ty) * (1.f - tz) * T[glin3(G, ni - 1, nj - 1, nk - 1)];
    mt = (tg - B.v[3][p]) * itth;
    f.rhs_t[p] = mt;
  }
  float a3 = fabsf(mt);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a3 = fmaxf(a3, __shfl_xor_sync(0xffffffffu, a3, o));
  if ((threadIdx.x & 31) == 0) atomic_max_abs(&f.bounds[3], a3);
}

// exponents of the fixed-point scales: max|sum| <= bound = max|contribution| * 8 * 27 * max count per cell
__global__ void k_scales(F32Form f) {
  if (threadIdx.x != 0) return;
  const float cnt = 8.f * 27.f * fmaxf(1.f, (float)f.bounds[4]);
  const float b[5] = {cnt, __uint_as_float(f.bounds[0]) * cnt, __uint_as_float(f.bounds[1]) * cnt,
                      __uint_as_float(f.bounds[2]) * cnt, __uint_as_float(f.bounds[3]) * cnt};
  for (int q = 0; q < 5; ++q) {
    int e = 0;
    if (b[q] > 0.f && isfinite(b[q])) frexpf(b[q], &e);  // b < 2^e
    int se = 61 - e;
    if (se > 100) se = 100;
    f.se[q] = se;
  }
}

// max particles per cell of the step sort (bound for the scales)
__global__ void k_max_count(const int32_t *__restrict__ cs, int64_t ncell, uint32_t *__restrict__ out) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t m = 0;
  if (c < ncell) m = (uint32_t)(cs[c + 1] - cs[c]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// exact conversion of a scaled 64-bit integer sum q * 2^-se to fp64 with integer operations
__device__ inline double fixed_to_f64(long long q, int se) {
  if (q == 0) return 0.0;
  unsigned long long sgn = q < 0 ? 1ull : 0ull;
  unsigned long long m = sgn ? (unsigned long long)(-q) : (unsigned long long)q;
  int lz = __clzll(m);
  m <<= lz;  // leading one at bit 63: value = (m / 2^63) * 2^(63 - lz - se)
  long long ex = (long long)(63 - lz - se) + 1023;
  unsigned long long man = (m >> 11) & ((1ull << 52) - 1ull);
  unsigned long long rb = m & 0x7ffull;
  if (rb > 0x400ull || (rb == 0x400ull && (man & 1ull))) {
    man += 1ull;
    if (man == (1ull << 52)) { man = 0; ex += 1; }
  }
  if (ex <= 0) return 0.0;  // below the normal range (not reached for physical scales)
  return __longlong_as_double((long long)((sgn << 63) | ((unsigned long long)ex << 52) | man));
}

__device__ inline long long to_fixed(float v, int se) { return __float2ll_rn(ldexpf(v, se)); }

// Warp-cooperative exact add into shared int64 accumulators: lanes with the same
// slot (slot < 0: nothing to add) are summed first, in three 21-bit pieces whose
// sums over 32 lanes cannot overflow, and the group's lowest lane adds once.
// Must be called by all 32 lanes.
__device__ inline void warp_add_fixed(long long *acc, int slot, long long v) {
  const unsigned peers = __match_any_sync(0xffffffffu, slot);
  if (slot < 0) return;
  const unsigned long long u = (unsigned long long)v;
  const unsigned lo = (unsigned)(u & 0x1fffffu);
  const unsigned mid = (unsigned)((u >> 21) & 0x1fffffu);
  const int hi = (int)(v >> 42);  // arithmetic shift: signed top part
  const unsigned slo = __reduce_add_sync(peers, lo);
  const unsigned smid = __reduce_add_sync(peers, mid);
  const int shi = (int)__reduce_add_sync(peers, (unsigned)hi);
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
    const long long sum = ((long long)shi << 42) + ((long long)smid << 21) + (long long)slo;
    atomicAdd((unsigned long long *)&acc[slot], (unsigned long long)sum);
  }
}

// Deposit into the CTA's brick of 8^3 interior cells. mode 0: concentration + face
// momentum at the *_int positions; mode 1: RHS_T at the *_new positions.
template <int MODE>
__global__ void __launch_bounds__(kDepThreads) k_dep32(Geom G, F32Form f, Set32 S, int twc, double *__restrict__ out0,
                                                       double *__restrict__ ox_, double *__restrict__ oy_,
                                                       double *__restrict__ oz_) {
  constexpr int NF = MODE == 0 ? 4 : 1;
  __shared__ long long acc[NF][kBr * kBr * kBr];
  __shared__ int32_t pre[kSrc * kSrc * kSrc + 1];
  __shared__ int32_t beg[kSrc * kSrc * kSrc];
  const int nbx = G.n[0] / kBr, nby = G.n[1] / kBr;
  const int bx = (int)(blockIdx.x % nbx) * kBr;
  const int by = (int)((blockIdx.x / nbx) % nby) * kBr;
  const int bz = (int)(blockIdx.x / (nbx * nby)) * kBr;
  for (int s = threadIdx.x; s < NF * kBr * kBr * kBr; s += blockDim.x) (&acc[0][0])[s] = 0;
  // source cells [b-2, b+B+2): counts -> exclusive prefix (flat particle index space)
  constexpr int NS = kSrc * kSrc * kSrc;
  for (int s = threadIdx.x; s < NS; s += blockDim.x) {
    const int lx = s % kSrc, ly = (s / kSrc) % kSrc, lz = s / (kSrc * kSrc);
    const int i = wrapi(bx - kHalo + lx, G.n[0]), j = wrapi(by - kHalo + ly, G.n[1]), k = wrapi(bz - kHalo + lz, G.n[2]);
    const uint32_t id = brick_id(G, i, j, k);
    const int32_t a = f.cell_start[id], e = f.cell_start[id + 1];
    beg[s] = a;
    pre[s + 1] = e - a;
  }
  if (threadIdx.x == 0) pre[0] = 0;
  __syncthreads();
  // sequential-by-warp prefix over NS entries (small)
  if (threadIdx.x < 32) {
    int32_t carry = 0;
    for (int base = 0; base < NS; base += 32) {
      int idx = base + threadIdx.x + 1;
      int32_t v = idx <= NS ? pre[idx] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)threadIdx.x >= o) v += y;
      }
      if (idx <= NS) pre[idx] = v + carry;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
  }
  __syncthreads();
  const int32_t total = pre[NS];
  int se[4];
#pragma unroll
  for (int q = 0; q < NF; ++q) se[q] = f.se[MODE == 0 ? q : 4];
  // every lane runs the same number of iterations (the adds are warp-cooperative)
  const int32_t rounds = (total + (int32_t)blockDim.x - 1) / (int32_t)blockDim.x;
  for (int32_t it = 0; it < rounds; ++it) {
    const int32_t t = it * (int32_t)blockDim.x + (int32_t)threadIdx.x;
    const bool live = t < total;
    // find the source cell: last s with pre[s] <= t
    int lo = 0, hi = NS;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (pre[mid] <= t) lo = mid; else hi = mid;
    }
    const int32_t p = live ? beg[lo] + (t - pre[lo]) : 0;  // dead lanes read particle 0 (total > 0 here)
    const uint32_t c = S.cell[p];
    const float o0 = S.o[0][p], o1 = S.o[1][p], o2 = S.o[2][p];
    const int c3[3] = {ci_(c), cj_(c), ck_(c)};
    const int b3[3] = {bx, by, bz};
    // trilinear: node = cell + h; targets node - o (periodic); factor o ? 1 - x_l : x_l
    const int h3[3] = {o0 >= 0.5f, o1 >= 0.5f, o2 >= 0.5f};
    const float xl3[3] = {o0 - h3[0] + 0.5f, o1 - h3[1] + 0.5f, o2 - h3[2] + 0.5f};
    int lt[3][2];  // local brick coordinate of target node - o, or -1
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int o = 0; o < 2; ++o) {
        int tt = wrapi(c3[d] + h3[d] - o, G.n[d]) - b3[d];
        lt[d][o] = (tt >= 0 && tt < kBr) ? tt : -1;
      }
    const float val = MODE == 0 ? 1.0f : f.rhs_t[p];
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int ox = (o >> 2) & 1, oy = (o >> 1) & 1, oz = o & 1;
      const bool in = live && lt[0][ox] >= 0 && lt[1][oy] >= 0 && lt[2][oz] >= 0;
      const float w = (ox ? 1.f - xl3[0] : xl3[0]) * (oy ? 1.f - xl3[1] : xl3[1]) * (oz ? 1.f - xl3[2] : xl3[2]) * val;
      const int slot = in ? (lt[2][oz] * kBr + lt[1][oy]) * kBr + lt[0][ox] : -1;
      warp_add_fixed(acc[0], slot, in ? to_fixed(w, se[0]) : 0ll);
    }
    if (MODE == 0 && twc) {
      // face-normal (particle.cpp:498-524): face c gets (1 - x_l) R, face c + 1 gets x_l R
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int p1 = (d + 1) % 3, p2 = (d + 2) % 3;
        const int a1 = c3[p1] - b3[p1], a2 = c3[p2] - b3[p2];
        const bool across = live && a1 >= 0 && a1 < kBr && a2 >= 0 && a2 < kBr;
        const float r = f.rhs_u[d][p];
        const float xl = d == 0 ? o0 : (d == 1 ? o1 : o2);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const int tt = wrapi(c3[d] + side, G.n[d]) - b3[d];
          const bool in = across && tt >= 0 && tt < kBr;
          int l3[3];
          l3[d] = in ? tt : 0; l3[p1] = in ? a1 : 0; l3[p2] = in ? a2 : 0;
          const float w = side ? xl * r : (1.f - xl) * r;
          const int slot = in ? (l3[2] * kBr + l3[1]) * kBr + l3[0] : -1;
          warp_add_fixed(acc[1 + d], slot, in ? to_fixed(w, se[1 + d]) : 0ll);
        }
      }
    }
  }
  __syncthreads();
  for (int s = threadIdx.x; s < kBr * kBr * kBr; s += blockDim.x) {
    const int lx = s % kBr, ly = (s / kBr) % kBr, lz = s / (kBr * kBr);
    const long long g = glin3(G, bx + lx + 1, by + ly + 1, bz + lz + 1);
    out0[g] = fixed_to_f64(acc[0][s], se[0]);
    if (MODE == 0) {
      if (twc) {
        ox_[g] = fixed_to_f64(acc[1][s], se[1]);
        oy_[g] = fixed_to_f64(acc[2][s], se[2]);
        oz_[g] = fixed_to_f64(acc[3][s], se[3]);
      } else {
        ox_[g] = 0.0; oy_[g] = 0.0; oz_[g] = 0.0;
      }
    }
  }
}

__global__ void k_to_f32(const double *__restrict__ src, int64_t n, double shift, float *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)(src[i] - shift);
}

// upload: absolute fp64 positions -> cell + fp32 offset (the reference's trunc cell)
__global__ void k_from_f64(Geom G, F32Form f, const double *__restrict__ x, const double *__restrict__ y,
                           const double *__restrict__ z, const double *__restrict__ u, const double *__restrict__ v,
                           const double *__restrict__ w, const double *__restrict__ t, double tref, int64_t n,
                           int32_t *__restrict__ err) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double X[3] = {x[p], y[p], z[p]};
  int c[3];
  float o[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double xi = X[d] * G.idx[d];
    if (!isfinite(xi)) { atomicOr(err, kErrNonFinite); xi = 0.0; }
    double fl = floor(xi);
    int i = (int)fl;
    float of = (float)(xi - fl);
    if (of >= 1.0f) { of = 0.0f; i += 1; }
    c[d] = wrapi(i, G.n[d]);
    o[d] = of;
  }
  const Set32 &B = f.set[SBASE];
  B.cell[p] = pack(c[0], c[1], c[2]);
#pragma unroll
  for (int d = 0; d < 3; ++d) B.o[d][p] = o[d];
  B.v[0][p] = (float)u[p];
  B.v[1][p] = (float)v[p];
  B.v[2][p] = (float)w[p];
  B.v[3][p] = (float)(t[p] - tref);
}

// download: one array of a set as fp64 (positions back to absolute coordinates)
__global__ void k_to_f64_arr(Geom G, Set32 S, int comp, double tref, int64_t n, double *__restrict__ dst) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (comp < 3) {
    const uint32_t c = S.cell[p];
    const int i = comp == 0 ? ci_(c) : (comp == 1 ? cj_(c) : ck_(c));
    dst[p] = ((double)i + (double)S.o[comp][p]) * (G.l[comp] / G.n[comp]);
  } else if (comp < 6) {
    dst[p] = (double)S.v[comp - 3][p];
  } else {
    dst[p] = (double)S.v[3][p] + tref;
  }
}

__global__ void k_keys32(Geom G, Set32 S, int64_t n, uint32_t *__restrict__ key) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t c = S.cell[p];
  key[p] = brick_id(G, ci_(c), cj_(c), ck_(c));
}

template <typename T>
__global__ void k_perm(const T *__restrict__ src, const int32_t *__restrict__ idx, int64_t n, T *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

__global__ void k_f32_to_f64(const float *__restrict__ src, int64_t n, double *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}

__global__ void k_recip32(const double *__restrict__ tau, int64_t n, float *__restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)(1. / tau[i]);
}

inline int nb(int64_t n) { return (int)((n + kThreads - 1) / kThreads); }

C32 make_c32(const pstep_ctx *h, int k, double pre, double post) {
  const pstep_config &cfg = h->cfg;
  C32 c;
  const double dt = cfg.dt;
  const double iS = 1. / (cfg.mp * cfg.cvp);
  c.dt_pre = (float)(dt * pre);
  c.dt_post = (float)(dt * post);
  c.dt_pre_is = (float)(dt * pre * iS);
  c.dt_post_is = (float)(dt * post * iS);
  for (int d = 0; d < 3; ++d) {
    c.dpre_idx[d] = (float)(dt * pre * h->geom.idx[d]);
    c.dpost_idx[d] = (float)(dt * post * h->geom.idx[d]);
  }
  c.itp = cfg.tp != 0 ? (float)(1. / cfg.tp) : 0.f;
  c.g[0] = (float)(cfg.particle_gravity * cfg.gx);
  c.g[1] = (float)(cfg.particle_gravity * cfg.gy);
  c.g[2] = (float)(cfg.particle_gravity * cfg.gz);
  c.alpha = (float)(0.25 * cfg.epsilonp * kPi * cfg.dp * cfg.dp * cfg.i0);
  c.itth = (float)(cfg.nu * kPi * cfg.dp * cfg.k);
  (void)k;
  return c;
}

template <typename T>
int dalloc32(pstep_ctx *h, T *&p, size_t count) {
  p = nullptr;
  cudaError_t e = cudaMalloc((void **)&p, sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) {
    p = nullptr;
    snprintf(h->err, sizeof h->err, "cudaMalloc: %s", cudaGetErrorString(e));
    cudaGetLastError();
    return PSTEP_ERR_NOMEM;
  }
  return PSTEP_OK;
}
template <typename T>
void dfree32(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

#define TRY32(x)                       \
  do {                                 \
    int rc_ = (x);                     \
    if (rc_ != PSTEP_OK) return rc_;   \
  } while (0)

int dep_all(pstep_ctx *h, int mode);

int sort_step(pstep_ctx *h) {
  // particles by brick-major cell of the base position; storage reordered; per-cell CSR kept
  F32Form &f = *h->f32;
  const Geom &G = h->geom;
  const int64_t n = h->np;
  const int64_t ncell = (int64_t)G.n[0] * G.n[1] * G.n[2];
  if (n > 0) {
    k_keys32<<<nb(n), kThreads, 0, h->stream>>>(G, f.set[SBASE], n, f.key);
    PSTEP_LAUNCHED(h);
  }
  // within a cell, by particle id (deterministic storage order)
  TRY32(csr_sort(h, f.key, 0, ncell, h->s.flag, f.cell_start, f.sidx));
  if (n > 0) {
    Set32 &B = f.set[SBASE];
    auto permf = [&](float *&a) {
      k_perm<float><<<nb(n), kThreads, 0, h->stream>>>(a, f.sidx, n, f.tmpf);
      float *t = a; a = f.tmpf; f.tmpf = t;
    };
    for (int d = 0; d < 3; ++d) permf(B.o[d]);
    for (int q = 0; q < 4; ++q) permf(B.v[q]);
    permf(f.rhs_t);
    if (f.itp) permf(f.itp);
    {
      k_perm<uint32_t><<<nb(n), kThreads, 0, h->stream>>>(B.cell, f.sidx, n, (uint32_t *)f.tmpf);
      uint32_t *t = B.cell; B.cell = (uint32_t *)f.tmpf; f.tmpf = (float *)t;
    }
    {
      k_perm<int32_t><<<nb(n), kThreads, 0, h->stream>>>(h->s.flag, f.sidx, n, (int32_t *)f.tmpf);
      int32_t *t = h->s.flag; h->s.flag = (int32_t *)f.tmpf; f.tmpf = (float *)t;
    }
    h->launches += 9;
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaMemsetAsync(&f.bounds[4], 0, sizeof(uint32_t), h->stream));
    k_max_count<<<nb(ncell), kThreads, 0, h->stream>>>(f.cell_start, ncell, &f.bounds[4]);
    PSTEP_LAUNCHED(h);
  }
  f.sorted = 1;
  return PSTEP_OK;
}

}  // namespace

int f32_create(pstep_ctx *h) {
  const Geom &G = h->geom;
  for (int d = 0; d < 3; ++d) {
    if (G.n[d] > kMaxN || G.n[d] % kBr != 0) {
      snprintf(h->err, sizeof h->err, "FP32 form needs cells per side a multiple of %d and at most %d", kBr, kMaxN);
      return PSTEP_ERR_CONFIG;
    }
  }
  F32Form *f = new F32Form();
  memset((void *)f, 0, sizeof(F32Form));
  h->f32 = f;
  const size_t cap = (size_t)h->cap;
  for (int s = 0; s < 4; ++s) {
    TRY32(dalloc32(h, f->set[s].cell, cap));
    for (int d = 0; d < 3; ++d) TRY32(dalloc32(h, f->set[s].o[d], cap));
    for (int q = 0; q < 4; ++q) TRY32(dalloc32(h, f->set[s].v[q], cap));
  }
  TRY32(dalloc32(h, f->rhs_t, cap));
  for (int d = 0; d < 3; ++d) TRY32(dalloc32(h, f->rhs_u[d], cap));
  const size_t gs = (size_t)G.gsize;
  for (int d = 0; d < 3; ++d) TRY32(dalloc32(h, f->uf[d], gs));
  TRY32(dalloc32(h, f->tf, gs));
  TRY32(dalloc32(h, f->key, cap));
  const size_t ncell = (size_t)G.n[0] * G.n[1] * G.n[2];
  TRY32(dalloc32(h, f->cell_start, ncell + 1));
  TRY32(dalloc32(h, f->sidx, cap));
  TRY32(dalloc32(h, f->tmpf, cap));
  TRY32(dalloc32(h, f->bounds, 8));
  TRY32(dalloc32(h, f->se, 8));
  TRY32(dalloc32(h, h->s.flag, cap));
  PSTEP_CUDA(cudaMemsetAsync(f->bounds, 0, 8 * sizeof(uint32_t), h->stream));
  return PSTEP_OK;
}

int f32_destroy(pstep_ctx *h) {
  F32Form *f = h->f32;
  if (!f) return PSTEP_OK;
  for (int s = 0; s < 4; ++s) {
    dfree32(f->set[s].cell);
    for (int d = 0; d < 3; ++d) dfree32(f->set[s].o[d]);
    for (int q = 0; q < 4; ++q) dfree32(f->set[s].v[q]);
  }
  dfree32(f->rhs_t); dfree32(f->itp);
  for (int d = 0; d < 3; ++d) { dfree32(f->rhs_u[d]); dfree32(f->uf[d]); }
  dfree32(f->tf); dfree32(f->key); dfree32(f->cell_start); dfree32(f->sidx); dfree32(f->tmpf);
  dfree32(f->bounds); dfree32(f->se);
  delete f;
  h->f32 = nullptr;
  return PSTEP_OK;
}

int f32_upload(pstep_ctx *h, const double *x, const double *y, const double *z, const double *u, const double *v,
               const double *w, const double *t, int on_device) {
  F32Form &f = *h->f32;
  const int64_t n = h->np;
  dfree32(f.itp);
  f.sorted = 0;
  if (n == 0) return PSTEP_OK;
  if (!f.tref_set) {
    double t0 = 0.0;
    if (on_device) PSTEP_CUDA(cudaMemcpy(&t0, t, sizeof(double), cudaMemcpyDeviceToHost));
    else t0 = t[0];
    f.tref = (double)(float)t0;
    f.tref_set = 1;
  }
  const double *src[7] = {x, y, z, u, v, w, t};
  double *tmp[7] = {nullptr};
  if (!on_device) {
    for (int q = 0; q < 7; ++q) {
      TRY32(dalloc32(h, tmp[q], (size_t)n));
      PSTEP_CUDA(cudaMemcpyAsync(tmp[q], src[q], sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
      src[q] = tmp[q];
    }
  }
  k_from_f64<<<nb(n), kThreads, 0, h->stream>>>(h->geom, f, src[0], src[1], src[2], src[3], src[4], src[5], src[6],
                                                f.tref, n, h->err_word);
  PSTEP_LAUNCHED(h);
  if (!on_device) {
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    for (int q = 0; q < 7; ++q) dfree32(tmp[q]);
  }
  return PSTEP_OK;
}

int f32_set_tau(pstep_ctx *h, const double *tau, int on_device) {
  F32Form &f = *h->f32;
  if (!tau) {
    dfree32(f.itp);
    return PSTEP_OK;
  }
  if (f.sorted) {
    snprintf(h->err, sizeof h->err, "tau_p must be set before pstep_prime");
    return PSTEP_ERR_STATE;
  }
  if (!f.itp) TRY32(dalloc32(h, f.itp, (size_t)h->cap));
  const int64_t n = h->np;
  if (n == 0) return PSTEP_OK;
  const double *src = tau;
  double *tmp = nullptr;
  if (!on_device) {
    TRY32(dalloc32(h, tmp, (size_t)n));
    PSTEP_CUDA(cudaMemcpyAsync(tmp, tau, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    src = tmp;
  }
  k_recip32<<<nb(n), kThreads, 0, h->stream>>>(src, n, f.itp);
  PSTEP_LAUNCHED(h);
  if (tmp) {
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    dfree32(tmp);
  }
  return PSTEP_OK;
}

int f32_bind_fields(pstep_ctx *h) {
  F32Form &f = *h->f32;
  const int64_t gs = h->geom.gsize;
  if (h->tf && !f.tref_set) {
    double t0 = 0.0;  // first interior cell
    PSTEP_CUDA(cudaMemcpyAsync(&t0, h->tf + glin(h->geom, 1, 1, 1), sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    f.tref = (double)(float)t0;
    f.tref_set = 1;
  }
  const double *src[4] = {h->ux, h->uy, h->uz, h->tf};
  float *dst[4] = {f.uf[0], f.uf[1], f.uf[2], f.tf};
  for (int q = 0; q < 4; ++q) {
    if (!src[q]) continue;
    k_to_f32<<<nb(gs), kThreads, 0, h->stream>>>(src[q], gs, q == 3 ? f.tref : 0.0, dst[q]);
    PSTEP_LAUNCHED(h);
  }
  return PSTEP_OK;
}

int f32_prime(pstep_ctx *h) {
  F32Form &f = *h->f32;
  TRY32(sort_step(h));
  const C32 c = make_c32(h, 0, 0.5, 1. / 6.);
  PSTEP_CUDA(cudaMemsetAsync(f.bounds, 0, 4 * sizeof(uint32_t), h->stream));
  if (h->np > 0) {
    k_prime32<<<nb(h->np), kThreads, 0, h->stream>>>(h->geom, f, c.itth, h->np);
    PSTEP_LAUNCHED(h);
  }
  // part2gas_Temp_int at the base positions: the *_new set holds them for the deposit
  const int64_t n = h->np;
  if (n > 0) {
    Set32 &B = f.set[SBASE], &N = f.set[SNEW];
    PSTEP_CUDA(cudaMemcpyAsync(N.cell, B.cell, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, h->stream));
    for (int d = 0; d < 3; ++d)
      PSTEP_CUDA(cudaMemcpyAsync(N.o[d], B.o[d], sizeof(float) * n, cudaMemcpyDeviceToDevice, h->stream));
  }
  return dep_all(h, 1);
}

int f32_stage(pstep_ctx *h, int k, double pre, double post) {
  F32Form &f = *h->f32;
  const C32 c = make_c32(h, k, pre, post);
  const int64_t n = h->np;
  PSTEP_CUDA(cudaMemsetAsync(f.bounds, 0, 4 * sizeof(uint32_t), h->stream));
  prof_begin(h, PSTEP_PHASE_ADVANCE);
  if (n > 0) {
    switch (k) {
      case 0: k_advance32<0><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
      case 1: k_advance32<1><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
      case 2: k_advance32<2><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
      default: k_advance32<3><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
    }
    PSTEP_LAUNCHED(h);
  }
  prof_end(h, PSTEP_PHASE_ADVANCE);
  prof_begin(h, PSTEP_PHASE_DEPOSIT_INT);
  TRY32(dep_all(h, 0));
  prof_end(h, PSTEP_PHASE_DEPOSIT_INT);
  prof_begin(h, PSTEP_PHASE_DEPOSIT_TEMP);
  TRY32(dep_all(h, 1));
  prof_end(h, PSTEP_PHASE_DEPOSIT_TEMP);
  return PSTEP_OK;
}

namespace {
int dep_all(pstep_ctx *h, int mode) {
  F32Form &f = *h->f32;
  const Geom &G = h->geom;
  k_scales<<<1, 32, 0, h->stream>>>(f);
  PSTEP_LAUNCHED(h);
  const int nbr = (G.n[0] / kBr) * (G.n[1] / kBr) * (G.n[2] / kBr);
  if (mode == 0) {
    // positions of the stage's *_int set (the base itself at stage 0: the FP32 form never shifts it)
    const Set32 S = f.set[h->int_is_base ? SBASE : SINT];
    k_dep32<0><<<nbr, kDepThreads, 0, h->stream>>>(G, f, S, h->cfg.twc, h->dep[PSTEP_FIELD_C], h->dep[PSTEP_FIELD_RU_X],
                                                   h->dep[PSTEP_FIELD_RU_Y], h->dep[PSTEP_FIELD_RU_Z]);
    PSTEP_LAUNCHED(h);
    double *all[4] = {h->dep[PSTEP_FIELD_C], h->dep[PSTEP_FIELD_RU_X], h->dep[PSTEP_FIELD_RU_Y], h->dep[PSTEP_FIELD_RU_Z]};
    // interior values are final (periodic targets): refresh the ghost layers only
    return fold_fields(h, all, 4, 2);
  }
  k_dep32<1><<<nbr, kDepThreads, 0, h->stream>>>(G, f, f.set[SNEW], h->cfg.twc, h->dep[PSTEP_FIELD_PART_TEMP], nullptr, nullptr,
                                                 nullptr);
  PSTEP_LAUNCHED(h);
  double *e[1] = {h->dep[PSTEP_FIELD_PART_TEMP]};
  TRY32(fold_fields(h, e, 1, 2));
  return interior_mean(h, h->dep[PSTEP_FIELD_PART_TEMP], h->emean_dev);
}
}  // namespace

int f32_end_stage(pstep_ctx *h) {
  F32Form &f = *h->f32;
  Set32 t = f.set[SINT];
  f.set[SINT] = f.set[SNEW];
  f.set[SNEW] = t;
  return PSTEP_OK;
}

int f32_end_step(pstep_ctx *h) {
  F32Form &f = *h->f32;
  Set32 t = f.set[SBASE];
  f.set[SBASE] = f.set[SNP1];
  f.set[SNP1] = t;
  prof_begin(h, PSTEP_PHASE_REORDER);
  int rc = sort_step(h);
  prof_end(h, PSTEP_PHASE_REORDER);
  return rc;
}

int f32_get_array(pstep_ctx *h, int id, void *dst, int on_device) {
  F32Form &f = *h->f32;
  const int64_t n = h->np;
  int set = SBASE, comp = 0;
  if (id <= PSTEP_T) { set = SBASE; comp = id - PSTEP_X; }
  else if (id <= PSTEP_T_INT) { set = h->int_is_base ? SBASE : SINT; comp = id - PSTEP_X_INT; }
  else if (id <= PSTEP_T_NEW) { set = h->phase != 0 ? SNEW : (h->int_is_base ? SBASE : SINT); comp = id - PSTEP_X_NEW; }
  else if (id <= PSTEP_T_NP1) { set = h->np1_is_base ? SBASE : SNP1; comp = id - PSTEP_X_NP1; }
  else set = -1;
  double *tmp = nullptr;
  TRY32(dalloc32(h, tmp, (size_t)n));
  if (set >= 0) {
    k_to_f64_arr<<<nb(n), kThreads, 0, h->stream>>>(h->geom, f.set[set], comp, f.tref, n, tmp);
  } else {
    k_f32_to_f64<<<nb(n), kThreads, 0, h->stream>>>(f.rhs_t, n, tmp);  // RHS_T
  }
  PSTEP_LAUNCHED(h);
  PSTEP_CUDA(cudaMemcpyAsync(dst, tmp, sizeof(double) * n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             h->stream));
  PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  dfree32(tmp);
  return PSTEP_OK;
}

}  // namespace pstep
