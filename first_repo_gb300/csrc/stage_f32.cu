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
#include <cuda_bf16.h>
#include <stdlib.h>
#include "pstep_internal.cuh"
#include "tc05.cuh"

namespace pstep {
int interior_mean(pstep_ctx *h, const double *f, double *out_dev);
int exclusive_scan(pstep_ctx *h, const int32_t *in, int64_t n, int32_t *out, int32_t *out2);
int fold_fields(pstep_ctx *h, double *const *f, int nf, int refresh);
}  // namespace pstep

namespace pstep {

enum { SBASE = 0, SINT = 1, SNEW = 2, SNP1 = 3 };
constexpr int kBr = 8;            // brick edge (cells) of the sort order
constexpr int kHalo = 2;          // source cells beyond a deposit brick
constexpr int kMaxN = 1024;       // 10 bits per cell coordinate
constexpr int kBoundSlots = 1024;

struct Set32 {
  uint32_t *cell;
  float *o[3];
  float *v[4];  // u v w T
};

// Deposit bricks (the cells one CTA owns) are BR x BR x BZ = 16^3 where the grid
// allows (every side a multiple of 16 and at least 32 cells: the source window of
// the brick and two cells around it must not wrap onto itself), else 8^3. A
// brick's source particles (those whose step-start cell lies within two cells of
// it) are visited about (BR+4)^2 (BZ+4) / (BR^2 BZ) times each: 1.95 at 16^3, 3.4 at
// 8^3. Every contribution is added once, by the brick that holds its target: the
// shared-memory adds, not the visits, bound the kernel.
//
// Work list of the deposit: one item per deposit brick, or -- for bricks whose
// source window holds more than kChunkMax particles -- several items, each a
// slice of at most kChunkMax of the window's particles. Items of split bricks
// come first (largest work first), then the rest; CTAs take items in order from
// an atomic counter. kVisit bounds the visits per particle (windows overlap), so
// at most kVisit * particles / kChunkMax bricks split.
template <int BR, int BZ> struct DepTraits;
template <> struct DepTraits<8, 8> {
  static constexpr int kThreads = 256, kVisit = 4;  // (12/8)^3 = 3.4
};
template <> struct DepTraits<16, 16> {
  static constexpr int kThreads = 1024, kVisit = 2;  // (20/16)^3 = 1.95
};

struct Work {
  long long *items;     // (brick << 32) | chunk, or -1 (skip)
  int32_t *nchunk;      // per brick
  int32_t *slot;        // per brick: index of its global tile, or -1
  int32_t *cnt_a, *cnt_b, *cnt_s, *off_a, *off_b, *off_s;  // per brick (+1) scan arrays
  int32_t *n_items;     // device scalar
  int32_t *next;        // device counters, one per deposit launch
  int32_t *done;        // per slot: items finished
  long long *tiles;     // per slot: 5 x BR^2 BZ int64
  int64_t slot_cap;
  int br, bz;           // deposit brick edges: 16^3 or 8^3
  int nbd;              // number of deposit bricks
  int32_t *err;         // device error word (kErrCapacity)
};

struct F32Form {
  Set32 set[4];
  float *rhs_t;
  float *itp;      // per-particle 1/tau_p or nullptr
  float *pp[7];    // per-particle mass ratio, itth, 1/(m Cvp), alpha, body acceleration x y z (or nullptr)
  float *gas[4];   // ug vg wg at x_int and Tg - t_ref at x_new of the last stage (PSTEP_KEEP_GAS)
  uint2 *drive;    // learned correction: the slip (3) and T_new - Tg the last stage's drag and heat transfer
                   // used, bf16 x 4 (a lagged estimate: bf16's 3 significant digits serve it)
  uint2 *corr_y;   // learned correction: the network output of the step's stage 0 (bf16 x 4)
  float *rhs_u[3];
  float *uf[3], *tf;  // fp32 ghosted copies of the bound fields
  uint32_t *key;      // brick-major cell id of the base position
  int32_t *cell_start;  // n^3 + 1, brick-major order (per step)
  int32_t *sidx;
  uint32_t *bounds;   // [0..2] max |RHS_u| per component (float bits), [3] max |RHS_T|, [4] max per-cell count
  uint32_t *slots;    // kBoundSlots x 4 partial maxima (spread so blocks do not contend on one word)
  uint32_t *pslots;   // kBoundSlots x 2: the last stage's max u and max ug (order-preserving keys)
  int pmax_state;     // 0: none; 1: filled by this step's last stage; 2: valid for the base state
  int32_t *unsorted;  // sort_step's storage-order test word
  int32_t *se;        // fixed-point scale exponents per field
  unsigned long long *totals;  // exact integer sums, maxima, minima of the five fields (last deposit)
  double *fstat;               // per field: max, min, interior sum as fp64 (k_totals)
  int ext_ok[5];               // per field: its last deposit gathered the extrema too
  Work work;
  int launch_no;      // deposit launches since the last work-list build (counter index)
  void *corr_mem;     // learned correction: packed weight image + biases (device), or nullptr
  int sorted;
  int tref_set;
  double tref;        // temperature reference (see above)
  // host transfers: two staging slots of kStageArrays x kStageChunk doubles, filled and
  // drained on a copy stream of their own so that the copy of one chunk overlaps the
  // conversion of the other (created at the first host upload or download)
  double *stage[2];
  cudaStream_t copy_stream;
  cudaEvent_t ev_copied[2], ev_used[2];
};
constexpr int64_t kStageChunk = 1 << 22;  // particles per staged chunk
constexpr int kStageArrays = 7;

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

// block maximum of 4 non-negative values into slot blockIdx % kBoundSlots
__device__ inline void block_max4(uint32_t *slots, float a0, float a1, float a2, float a3) {
  __shared__ float red[4][32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 = fmaxf(a0, __shfl_xor_sync(0xffffffffu, a0, o));
    a1 = fmaxf(a1, __shfl_xor_sync(0xffffffffu, a1, o));
    a2 = fmaxf(a2, __shfl_xor_sync(0xffffffffu, a2, o));
    a3 = fmaxf(a3, __shfl_xor_sync(0xffffffffu, a3, o));
  }
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = a0; red[1][w] = a1; red[2][w] = a2; red[3][w] = a3; }
  __syncthreads();
  if (threadIdx.x < 4) {
    float m = 0.f;
    for (int q = 0; q < nw; ++q) m = fmaxf(m, red[threadIdx.x][q]);
    atomic_max_abs(&slots[(blockIdx.x % kBoundSlots) * 4 + threadIdx.x], m);
  }
}

// order-preserving 32-bit key of a float (larger float, larger key; 0 is below every key)
__device__ __forceinline__ uint32_t order_key(float v) {
  const uint32_t b = __float_as_uint(v);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// block maximum of 2 signed values into slot blockIdx % kBoundSlots as order keys (a block
// with no particle leaves its slots alone)
__device__ inline void block_max2_signed(uint32_t *slots, float a0, float a1) {
  __shared__ float red2[2][32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 = fmaxf(a0, __shfl_xor_sync(0xffffffffu, a0, o));
    a1 = fmaxf(a1, __shfl_xor_sync(0xffffffffu, a1, o));
  }
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) { red2[0][w] = a0; red2[1][w] = a1; }
  __syncthreads();
  if (threadIdx.x < 2) {
    float m = -INFINITY;
    for (int q = 0; q < nw; ++q) m = fmaxf(m, red2[threadIdx.x][q]);
    if (m > -INFINITY) atomicMax(&slots[(blockIdx.x % kBoundSlots) * 2 + threadIdx.x], order_key(m));
  }
}

struct C32 {
  float dt_pre, dt_post, dt_pre_is, dt_post_is;
  float dpre_idx[3], dpost_idx[3];  // dt*pre/dx, dt*post/dx per dimension
  float itp, g[3], alpha, itth;
  float is;  // 1/(mp*Cvp) (particle.cpp:485)
};

enum { PP_MASS = 0, PP_ITTH, PP_HEAT_IS, PP_ALPHA, PP_ACC };  // F32Form::pp slots (PP_ACC + d)

// learned correction: the drive slip / temperature difference at most 10x the plain one
constexpr float kDriveCap = 10.f;

// One particle's stage: everything the advance kernels read, and the gas velocity
// interpolated at x_int (particle.cpp:340-360).
struct Adv {
  uint32_t cb, cint, cacc;
  float ob[3], oin[3], oac[3], vb[4], vin[4], vac[4];
  float rhs_t_old, itp, itth, alpha, dpre_is, dpost_is, gacc[3];
  float gas[3];
};

// the particle's x_int cell, offsets and velocity and the gas velocity there (particle.cpp:340-360)
template <int K>
__device__ __forceinline__ void adv_load_gas(const Geom &G, const F32Form &f, int64_t p, Adv &a) {
  const Set32 &I = (K == 0) ? f.set[SBASE] : f.set[SINT];
  a.cint = I.cell[p];
#pragma unroll
  for (int d = 0; d < 3; ++d) { a.oin[d] = I.o[d][p]; a.vin[d] = I.v[d][p]; }
  const int ii = ci_(a.cint) + 1, jj = cj_(a.cint) + 1, kk = ck_(a.cint) + 1;
  const float xl = a.oin[0], yl = a.oin[1], zl = a.oin[2];
  a.gas[0] = xl * f.uf[0][glin3(G, ii + 1, jj, kk)] + (1.f - xl) * f.uf[0][glin3(G, ii, jj, kk)];
  a.gas[1] = yl * f.uf[1][glin3(G, ii, jj + 1, kk)] + (1.f - yl) * f.uf[1][glin3(G, ii, jj, kk)];
  a.gas[2] = zl * f.uf[2][glin3(G, ii, jj, kk + 1)] + (1.f - zl) * f.uf[2][glin3(G, ii, jj, kk)];
}

// everything else the stage reads
template <int K>
__device__ __forceinline__ void adv_load_rest(const Geom &G, const F32Form &f, const C32 &c, int64_t p, Adv &a) {
  const Set32 &B = f.set[SBASE];
  const Set32 &I = (K == 0) ? f.set[SBASE] : f.set[SINT];
  const Set32 &A = (K == 0) ? f.set[SBASE] : f.set[SNP1];
  a.cb = B.cell[p];
  a.cacc = A.cell[p];
#pragma unroll
  for (int d = 0; d < 3; ++d) { a.ob[d] = B.o[d][p]; a.oac[d] = A.o[d][p]; }
#pragma unroll
  for (int q = 0; q < 4; ++q) { a.vb[q] = B.v[q][p]; a.vac[q] = A.v[q][p]; }
  a.vin[3] = I.v[3][p];
  a.rhs_t_old = f.rhs_t[p];
  a.itp = f.itp ? f.itp[p] : c.itp;
  a.itth = f.pp[PP_ITTH] ? f.pp[PP_ITTH][p] : c.itth;
  a.alpha = f.pp[PP_ALPHA] ? f.pp[PP_ALPHA][p] : c.alpha;
  a.dpre_is = f.pp[PP_HEAT_IS] ? c.dt_pre * f.pp[PP_HEAT_IS][p] : c.dt_pre_is;
  a.dpost_is = f.pp[PP_HEAT_IS] ? c.dt_post * f.pp[PP_HEAT_IS][p] : c.dt_post_is;
#pragma unroll
  for (int d = 0; d < 3; ++d) a.gacc[d] = f.pp[PP_ACC + d] ? f.pp[PP_ACC + d][p] : c.g[d];
}

template <int K>
__device__ __forceinline__ void adv_load(const Geom &G, const F32Form &f, const C32 &c, int64_t p, Adv &a) {
  adv_load_gas<K>(G, f, p, a);
  adv_load_rest<K>(G, f, c, p, a);
}

// The rest of the stage for one particle, with a.gas the gas velocity to use; with
// ty != 0 the interpolated gas temperature Tg is replaced by Tg - ty * dT, dT the
// previous stage's T_new - Tg (td_prev, or the current T_new - Tg when there is
// none): the learned correction of the particle's own heating. Returns the
// T_new - Tg the heat transfer used.
template <int K>
__device__ __forceinline__ float adv_finish_t(const Geom &G, const F32Form &f, const C32 &c, int twc, int64_t p, Adv &a,
                                              float ty, float td_prev, int32_t *__restrict__ err, float &mu0, float &mu1,
                                              float &mu2, float &mt) {
  // positions (particle.cpp:314-338) in cell units
  int ia[3] = {ci_(a.cacc), cj_(a.cacc), ck_(a.cacc)};
  int ib[3] = {ci_(a.cb), cj_(a.cb), ck_(a.cb)};
  int in_[3];
  float on[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    a.oac[d] += c.dpost_idx[d] * a.vin[d];
    renorm(ia[d], a.oac[d], G.n[d]);
    if (K != 3) {
      on[d] = a.ob[d] + c.dpre_idx[d] * a.vin[d];
      in_[d] = ib[d];
      renorm(in_[d], on[d], G.n[d]);
    } else {
      on[d] = a.oac[d];
      in_[d] = ia[d];
    }
  }
  // x_new within one cell of the step-start cell on every axis: the deposit's source
  // windows (two cells around a brick) hold a particle's x_int and x_new cells only then
  {
    bool far = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int r = in_[d] - ib[d];
      r += (r < -(G.n[d] >> 1)) ? G.n[d] : 0;
      r -= (r > (G.n[d] >> 1)) ? G.n[d] : 0;
      far |= (r < -1 || r > 1);
    }
    if (far) atomicOr(err, kErrMove);
  }
  // velocity and temperature (particle.cpp:362-399, 480-496)
  float rhs[3], vn[4];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rhs[d] = (a.gas[d] - a.vin[d]) * a.itp;
    a.vac[d] += c.dt_post * (rhs[d] + a.gacc[d]);
    vn[d] = (K != 3) ? a.vb[d] + c.dt_pre * (rhs[d] + a.gacc[d]) : a.vac[d];
  }
  a.vac[3] += a.dpost_is * (a.rhs_t_old + a.alpha);
  vn[3] = (K != 3) ? a.vb[3] + a.dpre_is * (a.rhs_t_old + a.alpha) : a.vac[3];

  // trilinear T at x_new (particle.cpp:430-456): node = cell + h, x_l = o - h + 1/2
  const int hx = on[0] >= 0.5f, hy = on[1] >= 0.5f, hz = on[2] >= 0.5f;
  const int ni = in_[0] + hx + 1, nj = in_[1] + hy + 1, nk = in_[2] + hz + 1;  // ghosted node
  const float *T = f.tf;
  const float wx = on[0] - hx + 0.5f, wy = on[1] - hy + 0.5f, wz = on[2] - hz + 0.5f;
  float tg = wx * wy * wz * T[glin3(G, ni, nj, nk)] + (1.f - wx) * wy * wz * T[glin3(G, ni - 1, nj, nk)] +
             wx * (1.f - wy) * wz * T[glin3(G, ni, nj - 1, nk)] + wx * wy * (1.f - wz) * T[glin3(G, ni, nj, nk - 1)] +
             (1.f - wx) * (1.f - wy) * wz * T[glin3(G, ni - 1, nj - 1, nk)] +
             (1.f - wx) * wy * (1.f - wz) * T[glin3(G, ni - 1, nj, nk - 1)] +
             wx * (1.f - wy) * (1.f - wz) * T[glin3(G, ni, nj - 1, nk - 1)] +
             (1.f - wx) * (1.f - wy) * (1.f - wz) * T[glin3(G, ni - 1, nj - 1, nk - 1)];
  if (ty != 0.f) {
    const float dtn = vn[3] - tg;
    const float cap = kDriveCap * fabsf(dtn);
    const float td = td_prev != 0.f ? (fabsf(td_prev) <= cap ? td_prev : copysignf(cap, td_prev)) : dtn;
    tg -= ty * td;
  }
  const float rhs_t_new = (tg - vn[3]) * a.itth;
  if (!isfinite(rhs_t_new) || !isfinite(vn[0]) || !isfinite(vn[1]) || !isfinite(vn[2]) || !isfinite(on[0]) ||
      !isfinite(on[1]) || !isfinite(on[2]))
    atomicOr(err, kErrNonFinite);

  // stores
  const Set32 &N = f.set[SNEW];
  const Set32 &P = f.set[SNP1];
  N.cell[p] = pack(in_[0], in_[1], in_[2]);
  P.cell[p] = pack(ia[0], ia[1], ia[2]);
#pragma unroll
  for (int d = 0; d < 3; ++d) { N.o[d][p] = on[d]; P.o[d][p] = a.oac[d]; }
#pragma unroll
  for (int q = 0; q < 4; ++q) { N.v[q][p] = vn[q]; P.v[q][p] = a.vac[q]; }
  // the momentum deposit carries the particle's mass relative to cfg.mp
  const float mrel = f.pp[PP_MASS] ? f.pp[PP_MASS][p] : 1.f;
  if (twc) {
#pragma unroll
    for (int d = 0; d < 3; ++d) f.rhs_u[d][p] = rhs[d] * mrel;
  }
  f.rhs_t[p] = rhs_t_new;
  if (f.gas[0]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) f.gas[d][p] = a.gas[d];
    f.gas[3][p] = tg;
  }
  mu0 = fmaxf(mu0, fabsf(rhs[0] * mrel));
  mu1 = fmaxf(mu1, fabsf(rhs[1] * mrel));
  mu2 = fmaxf(mu2, fabsf(rhs[2] * mrel));
  mt = fmaxf(mt, fabsf(rhs_t_new));
  return vn[3] - tg;
}

template <int K>
__device__ __forceinline__ void adv_finish(const Geom &G, const F32Form &f, const C32 &c, int twc, int64_t p, Adv &a,
                                           int32_t *__restrict__ err, float &mu0, float &mu1, float &mu2, float &mt) {
  (void)adv_finish_t<K>(G, f, c, twc, p, a, 0.f, 0.f, err, mu0, mu1, mu2, mt);
}

template <int K>
__device__ __forceinline__ float adv_finish_mlp(const Geom &G, const F32Form &f, const C32 &c, int twc, int64_t p,
                                                Adv &a, float ty, float td_prev, int32_t *__restrict__ err, float &mu0,
                                                float &mu1, float &mu2, float &mt) {
  return adv_finish_t<K>(G, f, c, twc, p, a, ty, td_prev, err, mu0, mu1, mu2, mt);
}

template <int K>
__global__ void __launch_bounds__(256) k_advance32(Geom G, F32Form f, C32 c, int twc, int64_t n,
                                                   int32_t *__restrict__ err) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float mu0 = 0.f, mu1 = 0.f, mu2 = 0.f, mt = 0.f, umax = -INFINITY, gmax = -INFINITY;
  if (p < n) {
    Adv a;
    adv_load<K>(G, f, c, p, a);
    adv_finish<K>(G, f, c, twc, p, a, err, mu0, mu1, mu2, mt);
    umax = a.vac[0];
    gmax = a.gas[0];
  }
  // bounds for the fixed-point scales (order-independent maxima)
  block_max4(f.slots, mu0, mu1, mu2, mt);
  // the last stage: max u of the step's result and max ug (grid.cpp:726-727)
  if (K == 3) block_max2_signed(f.pslots, umax, gmax);
}

// ----------------------------------------------------------------------------
// The learned correction (pstep_set_correction).
//
// The network runs in its own kernel, k_corr_net, at stage 0 of every step (or at
// every stage, pstep_correction.every_stage): persistent CTAs of two warpgroups;
// each warpgroup owns tiles of 128 particles, one particle per thread, and thread
// t's network row is tensor-memory lane t of the warpgroup's 64 columns. Per tile:
// the plain interpolation at x_int and the features in registers, the feature row
// as bf16 to shared memory, three tcgen05 MMAs (16 -> 64 -> 64 -> 16 columns; each
// layer's accumulator reuses the columns of the one before, which has been read),
// bias and SiLU between them on 16-column chunks, and the network output (bf16 x 4,
// zero for particles outside the training ranges) to memory. The two warpgroups
// synchronise with named barriers only, so one's MMAs overlap the other's loads and
// epilogues; four CTAs per SM keep eight warpgroups in flight. The advance of every
// stage (k_advance32_corr) applies the kept output with that stage's own drive slip
// and prior: within a step a particle moves a few hundredths of a cell and its slip
// hardly changes, so one inference per step serves the step's four stages.
// Particles outside the training ranges keep the plain interpolation.
namespace corr {
constexpr int kRows = 128, kInP = 16, kHid = 64, kOutP = 16, kGroups = 2, kThreads = kRows * kGroups;
// shared memory: weight image W1 | W2 | W3 (bf16 tiles), biases, then per warpgroup
// X [128 x 16], H [128 x 64] (layer 1, then layer 2 output), its MMA mbarrier and an
// idle mbarrier that nothing signals (the wait-timeout test, pstep_set_wait_limit)
constexpr uint32_t W1 = 0, W2 = W1 + kHid * kInP * 2, W3 = W2 + kHid * kHid * 2, kImage = W3 + kOutP * kHid * 2;
constexpr uint32_t BIAS = kImage, GROUPS = 13 * 1024;
constexpr uint32_t G_XA = 0, G_H = G_XA + kRows * kInP * 2, G_BAR = G_H + kRows * kHid * 2, G_IDLE = G_BAR + 8,
                   kGroupStride = 21 * 1024;
constexpr uint32_t TSLOT = GROUPS + kGroups * kGroupStride, kBytes = TSLOT + 16;
static_assert(BIAS + (kHid + kHid + kOutP) * 4 <= GROUPS, "correction smem");
static_assert(G_IDLE + 8 <= kGroupStride, "correction group smem");
// with this much shared memory at most 4 CTAs fit on an SM (228 KB), so their
// 4 x 128 tensor-memory columns never exceed the 512 an SM has and no allocation waits
constexpr uint32_t kAlloc = kBytes;
static_assert(5 * (kAlloc + 1024) > 228 * 1024, "more than 4 correction CTAs per SM");
constexpr uint32_t kWaitLimit = 1u << 22;
}  // namespace corr

struct CorrDev {
  const uint4 *image;  // kImage bytes
  const float *bias;   // b1[64] b2[64] b3[16]
  float shift[10], scale[10], lo[4], hi[4];
  float inv_nu;        // 1 / kinematic viscosity of the gas
  float inv_prior_re;  // 1 / prior_re (0: outputs not scaled by the prior)
  float dp_per_itth;   // d_p = itth * dp_per_itth (1 / (Nu PI k)), per-particle diameters
  float dp;            // scalar diameter (no per-particle itth)
  float idx;           // 1 / dx
  uint32_t wait_limit; // polls of each MMA completion wait (the drain before freeing tensor memory
                       // always allows corr::kWaitLimit)
  uint32_t idle_first; // 1: each warpgroup's first completion wait polls the idle barrier (test)
  float drive_cap;     // the drive slip at most this many times the plain slip
};

static_assert(sizeof(CorrDev) <= sizeof(((pstep_ctx *)nullptr)->corr_dev), "correction constants");

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// warpgroup-local barrier (named barrier 1 + group, 128 threads; immediate ids)
__device__ __forceinline__ void group_bar(int wg) {
  if (wg == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
  else asm volatile("bar.sync 2, 128;" ::: "memory");
}
__device__ __forceinline__ bool group_and(int wg, bool v) {
  uint32_t out;
  if (wg == 0)
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, 1, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(out)
        : "r"(v ? 1u : 0u)
        : "memory");
  else
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, 2, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(out)
        : "r"(v ? 1u : 0u)
        : "memory");
  return out != 0;
}
__device__ __forceinline__ void group_sync_mma(int wg) {
  tc05::fence_smem_async();
  tc05::fence_before();
  group_bar(wg);
  tc05::fence_after();
}
__device__ __forceinline__ bool group_wait(int wg, uint64_t *mbar, uint32_t &phase, uint32_t limit) {
  const bool ok = tc05::mbar_wait(mbar, phase, limit);
  tc05::fence_after();
  const bool all = group_and(wg, ok);
  if (all) phase ^= 1u;
  return all;
}

// 16 accumulator columns + bias -> SiLU -> bf16, into row r, columns [c0, c0+16) of a 64-column tile
// SiLU z * sigmoid(z) = u (1 + tanh u) = u tanh(u) + u with u = z/2 and the hardware
// tanh approximation; with the halved bias hb, u = v/2 + hb is one fma
__device__ __forceinline__ float silu_half(float v, float hb) {
  const float u = fmaf(v, 0.5f, hb);
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return fmaf(u, t, u);
}

// bias: the layer's bias halved
__device__ __forceinline__ void silu_chunk_to_tile(uint8_t *tile, int r, int c0, const float (&v)[16],
                                                   const float *bias) {
  float h[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) h[q] = silu_half(v[q], bias[c0 + q]);
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    uint4 w;
    w.x = pack_bf16x2(h[half * 8 + 0], h[half * 8 + 1]);
    w.y = pack_bf16x2(h[half * 8 + 2], h[half * 8 + 3]);
    w.z = pack_bf16x2(h[half * 8 + 4], h[half * 8 + 5]);
    w.w = pack_bf16x2(h[half * 8 + 6], h[half * 8 + 7]);
    *reinterpret_cast<uint4 *>(tile + tc05::tile_off(r, c0 + half * 8, corr::kHid)) = w;
  }
}

// the drive slip: the previous stage's (at most `cap` x the plain one), or the plain slip
__device__ __forceinline__ void drive_slip(const uint2 dw, const float (&s)[3], float smag, float cap, float &sdrv,
                                           float (&dir)[3], float &dmag_used) {
  const float d0 = bf16_lo(dw.x), d1 = bf16_hi(dw.x), d2 = bf16_lo(dw.y);
  const float dmag = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
  if (dmag > 0.f) {
    sdrv = fminf(dmag, cap * smag);
    dir[0] = d0; dir[1] = d1; dir[2] = d2;
    dmag_used = dmag;
  } else {
    sdrv = smag;
    dir[0] = s[0]; dir[1] = s[1]; dir[2] = s[2];
    dmag_used = smag;
  }
}

__device__ __forceinline__ float prior_of(const CorrDev &cd, float dpdx, float rep) {
  return cd.inv_prior_re > 0.f ? dpdx / (1.f + rep / dpdx * cd.inv_prior_re) : 1.f;
}

__device__ __forceinline__ float particle_dp(const F32Form &f, const CorrDev &cd, int64_t p, float itth) {
  return f.pp[PP_ITTH] ? itth * cd.dp_per_itth : cd.dp;
}

// A particle's network inputs as loaded from memory (x_int cell, offsets and velocity,
// the drive state), fetched one tile ahead so that their memory round trip overlaps the
// current tile's tensor-core work
struct NetRaw {
  uint32_t cell;
  float o[3], v[3];
  uint2 drive;
};
template <int K>
__device__ __forceinline__ void net_raw_load(const F32Form &f, int64_t p, int64_t n, NetRaw &r) {
  if (p >= n) return;
  const Set32 &I = (K == 0) ? f.set[SBASE] : f.set[SINT];
  r.cell = I.cell[p];
#pragma unroll
  for (int d = 0; d < 3; ++d) { r.o[d] = I.o[d][p]; r.v[d] = I.v[d][p]; }
  r.drive = f.drive[p];
}

// The network of every particle at its x_int position: features from the plain
// interpolation and the drive state of the previous stage, three tcgen05 layers,
// the output (bf16 x 4) to f.corr_y (zero outside the training ranges).
template <int K>
__global__ void __launch_bounds__(corr::kThreads, 4) k_corr_net(Geom G, F32Form f, C32 c, int64_t n,
                                                                int32_t *__restrict__ err, CorrDev cd) {
  extern __shared__ __align__(1024) uint8_t sm[];
  using namespace tc05;
  const int tid = threadIdx.x, wg = tid >> 7, lt = tid & (corr::kRows - 1), warp = tid >> 5;
  uint8_t *W1 = sm + corr::W1, *W2 = sm + corr::W2, *W3 = sm + corr::W3;
  float *b1 = reinterpret_cast<float *>(sm + corr::BIAS), *b2 = b1 + corr::kHid, *b3 = b2 + corr::kHid;
  uint8_t *gbase = sm + corr::GROUPS + wg * corr::kGroupStride;
  uint8_t *XA = gbase + corr::G_XA, *H = gbase + corr::G_H;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(gbase + corr::G_BAR);
  uint64_t *idle = reinterpret_cast<uint64_t *>(gbase + corr::G_IDLE);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + corr::TSLOT);
  const uint32_t limit = cd.wait_limit ? cd.wait_limit : corr::kWaitLimit;
  for (uint32_t q = tid; q < corr::kImage / 16; q += corr::kThreads) reinterpret_cast<uint4 *>(sm)[q] = cd.image[q];
  // hidden-layer biases halved for silu_half (exact: a power-of-two scale)
  for (int q = tid; q < corr::kHid + corr::kHid + corr::kOutP; q += corr::kThreads)
    b1[q] = q < 2 * corr::kHid ? 0.5f * cd.bias[q] : cd.bias[q];
  if (lt == 0) {
    mbar_init(mbar, 1);
    mbar_init(idle, 1);
  }
  if (warp == 0) tmem_alloc(tslot, 128);
  tc05::fence_smem_async();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t tcol = *tslot + (uint32_t)(wg * 64);
  const uint32_t tl = tcol + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's lane quadrant
  const uint32_t id64 = idesc_bf16(128, 64), id16 = idesc_bf16(128, 16);
  const uint32_t sX = smem_u32(XA), sH = smem_u32(H), sW1 = smem_u32(W1), sW2 = smem_u32(W2), sW3 = smem_u32(W3);
  uint32_t phase = 0;
  bool ok = true;
  bool first = cd.idle_first != 0;
  const int64_t ntiles = (n + corr::kRows - 1) / corr::kRows;
  const int64_t tstride = (int64_t)gridDim.x * corr::kGroups;
  NetRaw raw{};
  net_raw_load<K>(f, ((int64_t)blockIdx.x * corr::kGroups + wg) * corr::kRows + lt, n, raw);
  for (int64_t tile = (int64_t)blockIdx.x * corr::kGroups + wg; tile < ntiles && ok; tile += tstride) {
    const int64_t p = tile * corr::kRows + lt;
    const bool live = p < n;
    bool use = false;
    {
      float x[corr::kInP];
#pragma unroll
      for (int j = 0; j < corr::kInP; ++j) x[j] = 0.f;
      if (live) {
        // the plain interpolation at x_int (particle.cpp:340-360) from the prefetched inputs
        const int ii = ci_(raw.cell) + 1, jj = cj_(raw.cell) + 1, kk = ck_(raw.cell) + 1;
        const float gas[3] = {
            raw.o[0] * f.uf[0][glin3(G, ii + 1, jj, kk)] + (1.f - raw.o[0]) * f.uf[0][glin3(G, ii, jj, kk)],
            raw.o[1] * f.uf[1][glin3(G, ii, jj + 1, kk)] + (1.f - raw.o[1]) * f.uf[1][glin3(G, ii, jj, kk)],
            raw.o[2] * f.uf[2][glin3(G, ii, jj, kk + 1)] + (1.f - raw.o[2]) * f.uf[2][glin3(G, ii, jj, kk)]};
        const float s[3] = {raw.v[0] - gas[0], raw.v[1] - gas[1], raw.v[2] - gas[2]};
        const float smag = sqrtf(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
        float sdrv, dir[3], dmag;
        drive_slip(raw.drive, s, smag, cd.drive_cap, sdrv, dir, dmag);
        const float itth = f.pp[PP_ITTH] ? f.pp[PP_ITTH][p] : c.itth;
        const float itp = f.itp ? f.itp[p] : c.itp;
        const float alpha = f.pp[PP_ALPHA] ? f.pp[PP_ALPHA][p] : c.alpha;
        const float his = f.pp[PP_HEAT_IS] ? f.pp[PP_HEAT_IS][p] : c.is;
        const float dpdx = particle_dp(f, cd, p, itth) * cd.idx;
        const float rep = sdrv * particle_dp(f, cd, p, itth) * cd.inv_nu;
        const float q = alpha * his;
        const float taup = 1.f / itp;
        use = smag > 0.f && dmag > 0.f && dpdx >= cd.lo[0] && dpdx <= cd.hi[0] && rep >= cd.lo[1] &&
              rep <= cd.hi[1] && q >= cd.lo[2] && q <= cd.hi[2] && taup >= cd.lo[3] && taup <= cd.hi[3];
        if (use) {
          const float inv = 1.f / dmag;
          const float fin[10] = {raw.o[0], raw.o[1], raw.o[2], dir[0] * inv, dir[1] * inv, dir[2] * inv, dpdx,
                                 logf(rep), q, logf(taup)};
#pragma unroll
          for (int j = 0; j < 10; ++j) x[j] = (fin[j] - cd.shift[j]) * cd.scale[j];
        }
      }
#pragma unroll
      for (int cb = 0; cb < 2; ++cb) {
        uint4 w;
        w.x = pack_bf16x2(x[cb * 8 + 0], x[cb * 8 + 1]);
        w.y = pack_bf16x2(x[cb * 8 + 2], x[cb * 8 + 3]);
        w.z = pack_bf16x2(x[cb * 8 + 4], x[cb * 8 + 5]);
        w.w = pack_bf16x2(x[cb * 8 + 6], x[cb * 8 + 7]);
        *reinterpret_cast<uint4 *>(XA + tile_off(lt, cb * 8, corr::kInP)) = w;
      }
    }
    group_sync_mma(wg);
    if (lt == 0) {
      mma_bf16(tcol, tile_desc(sX, corr::kInP, 0, 0), tile_desc(sW1, corr::kInP, 0, 0), id64, 0);
      commit(mbar);
    }
    net_raw_load<K>(f, (tile + tstride) * corr::kRows + lt, n, raw);  // the next tile's inputs, in flight
    // (the timeout test polls the idle barrier here, as a completion that never arrives;
    // the MMA's own completion is then drained below before the tensor memory is freed)
    ok = group_wait(wg, first ? idle : mbar, phase, limit);
    first = false;
    if (!ok) break;
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      float v[16];
      tmem_ld16(tl + cc * 16, v);
      silu_chunk_to_tile(H, lt, cc * 16, v, b1);
    }
    group_sync_mma(wg);
    if (lt == 0) {  // layer 2 into the same columns (layer 1 has been read)
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        mma_bf16(tcol, tile_desc(sH, corr::kHid, 0, ks), tile_desc(sW2, corr::kHid, 0, ks), id64, ks);
      commit(mbar);
    }
    ok = group_wait(wg, mbar, phase, limit);
    if (!ok) break;
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {  // layer 2 output overwrites layer 1's in H (its MMA is done)
      float v[16];
      tmem_ld16(tl + cc * 16, v);
      silu_chunk_to_tile(H, lt, cc * 16, v, b2);
    }
    group_sync_mma(wg);
    if (lt == 0) {
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        mma_bf16(tcol, tile_desc(sH, corr::kHid, 0, ks), tile_desc(sW3, corr::kHid, 0, ks), id16, ks);
      commit(mbar);
    }
    ok = group_wait(wg, mbar, phase, limit);
    if (!ok) break;
    float y[16];
    tmem_ld16(tl, y);
    tc05::fence_before();  // the accumulator reads before the warpgroup's next MMA
    if (live) {
      float yo[4] = {0.f, 0.f, 0.f, 0.f};
      if (use) {
#pragma unroll
        for (int d = 0; d < 4; ++d) yo[d] = y[d] + b3[d];
      }
      f.corr_y[p] = make_uint2(pack_bf16x2(yo[0], yo[1]), pack_bf16x2(yo[2], yo[3]));
    }
  }
  if (!ok) {
    if (lt == 0) atomicOr(err, kErrTimeout);
    tc05::mbar_wait(mbar, phase, corr::kWaitLimit);  // the MMA issued before the wait ran out
  }
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  if (warp == 0) tmem_dealloc(*tslot, 128);
}

// every stage with the correction: the kept network output, applied with this stage's
// drive slip and prior
template <int K>
__global__ void __launch_bounds__(256, 5) k_advance32_corr(Geom G, F32Form f, C32 c, int twc, int64_t n,
                                                        int32_t *__restrict__ err, CorrDev cd) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float mu0 = 0.f, mu1 = 0.f, mu2 = 0.f, mt = 0.f, umax = -INFINITY, gmax = -INFINITY;
  if (p < n) {
    Adv a;
    adv_load<K>(G, f, c, p, a);
    const uint2 yw = f.corr_y[p];
    const float yo[4] = {bf16_lo(yw.x), bf16_hi(yw.x), bf16_lo(yw.y), bf16_hi(yw.y)};
    float ty = 0.f, td = 0.f;
    if (yo[0] != 0.f || yo[1] != 0.f || yo[2] != 0.f || yo[3] != 0.f) {
      const float s[3] = {a.vin[0] - a.gas[0], a.vin[1] - a.gas[1], a.vin[2] - a.gas[2]};
      const float smag = sqrtf(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
      float sdrv, dir[3], dmag;
      const uint2 dw = f.drive[p];
      drive_slip(dw, s, smag, cd.drive_cap, sdrv, dir, dmag);
      const float dp = particle_dp(f, cd, p, a.itth);
      const float prior = prior_of(cd, dp * cd.idx, sdrv * dp * cd.inv_nu);
#pragma unroll
      for (int d = 0; d < 3; ++d) a.gas[d] -= sdrv * prior * yo[d];
      ty = prior * yo[3];
      td = bf16_hi(dw.y);
    }
    const float dv[3] = {a.vin[0] - a.gas[0], a.vin[1] - a.gas[1], a.vin[2] - a.gas[2]};
    const float dt_drive = adv_finish_mlp<K>(G, f, c, twc, p, a, ty, td, err, mu0, mu1, mu2, mt);
    f.drive[p] = make_uint2(pack_bf16x2(dv[0], dv[1]), pack_bf16x2(dv[2], dt_drive));
    umax = a.vac[0];
    gmax = a.gas[0];
  }
  block_max4(f.slots, mu0, mu1, mu2, mt);
  if (K == 3) block_max2_signed(f.pslots, umax, gmax);
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
    mt = (tg - B.v[3][p]) * (f.pp[PP_ITTH] ? f.pp[PP_ITTH][p] : itth);
    f.rhs_t[p] = mt;
  }
  block_max4(f.slots, 0.f, 0.f, 0.f, fabsf(mt));
}

// exponents of the fixed-point scales
__global__ void k_scales(F32Form f) {
  // fold the spread partial maxima, then clear them for the next stage
  for (int q = 0; q < 4; ++q) {
    uint32_t m = 0;
    for (int s = threadIdx.x; s < kBoundSlots; s += blockDim.x) m = max(m, f.slots[s * 4 + q]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) f.bounds[q] = m;
  }
  __syncwarp();
  for (int s = threadIdx.x; s < kBoundSlots * 4; s += blockDim.x) f.slots[s] = 0;
  if (threadIdx.x != 0) return;
  // largest contribution of each field: concentration weights <= 1, momentum |RHS_u|,
  // energy |RHS_T| (weights <= 1); its magnitude maps to at most 2^24
  const float b[5] = {1.f, __uint_as_float(f.bounds[0]), __uint_as_float(f.bounds[1]), __uint_as_float(f.bounds[2]),
                      __uint_as_float(f.bounds[3])};
  for (int q = 0; q < 5; ++q) {
    int e = 0;
    if (b[q] > 0.f && isfinite(b[q])) frexpf(b[q], &e);  // b < 2^e
    int se = 24 - e;
    if (se > 100) se = 100;
    f.se[q] = se;
  }
}

// max particles per cell of the step sort (bound for the scales): grid-stride, one
// atomic per block
__global__ void k_max_count(const int32_t *__restrict__ cs, int64_t ncell, uint32_t *__restrict__ out) {
  __shared__ uint32_t red[32];
  uint32_t m = 0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (int64_t)gridDim.x * blockDim.x)
    m = max(m, (uint32_t)(cs[c + 1] - cs[c]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) m = max(m, red[q]);
    m = max(m, red[0]);
    if (m) atomicMax(out, m);
  }
}

// exact conversion of a scaled 64-bit integer sum q * 2^-se to fp64 with integer operations
__device__ inline double fixed_to_f64(long long q, int se) {
  if (q == 0) return 0.0;
  if (q == (long long)(int)q) {  // |q| < 2^31: the same steps in 32-bit operations, exact (no rounding)
    const unsigned sgn = q < 0 ? 1u : 0u;
    unsigned m = (unsigned)(sgn ? -q : q);
    const int lz = __clz(m);
    m <<= lz;  // leading one at bit 31: value = (m / 2^31) * 2^(31 - lz - se)
    const int ex = 31 - lz - se + 1023;
    if (ex <= 0) return 0.0;
    return __hiloint2double((int)((sgn << 31) | ((unsigned)ex << 20) | ((m >> 11) & 0xfffffu)), (int)(m << 21));
  }
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

// c - b taken periodically into (-n/2, n/2]
__device__ inline int rel_local(int c, int b, int n) {
  int r = c - b;
  const int half = n >> 1;
  r += (r <= -half) ? n : 0;
  r -= (r > half) ? n : 0;
  return r;
}

// Exact sums with 32-bit shared-memory atomics. Every contribution is scaled so
// that the largest magnitude is 2^24 (the fp32 values carry 24 significant bits,
// so nothing beyond their own rounding is lost) and rounded to an integer v with
// |v| < 2^25. A slot holds two 32-bit words: the low word sums v mod 2^16
// (unsigned, below 2^16 each), the high word sums v >> 16 (signed, |.| < 2^9).
// Both adds are fire-and-forget (no returned value, no carry handling). The low
// word cannot wrap while a slot receives at most 2^16 contributions, and a slot
// receives at most one per particle the work item visits: work items visit at
// most kChunkMax = 2^16 particles. The sum is hi * 2^16 + lo, exact whatever the
// order of the adds.
constexpr int32_t kChunkMax = 1 << 16;
__device__ __forceinline__ void add_fixed32(uint32_t *lo, uint32_t *hi, int32_t v) {
  atomicAdd(lo, (uint32_t)v & 0xffffu);
  atomicAdd(hi, (uint32_t)(v >> 16));
}
__device__ __forceinline__ long long get_fixed(const uint32_t *lo, const uint32_t *hi) {
  return (long long)(int32_t)*hi * 65536ll + (long long)*lo;
}

// Accumulator of a deposit brick: its BR x BR x BZ cells, rows padded by one word so
// that neighbouring rows do not fall on the same shared-memory banks.
template <int BR, int BZ> struct Acc {
  static constexpr int kRow = BR + 1, kSlots = kRow * BR * BZ;
  static __device__ __forceinline__ int slot(int x, int y, int z) { return (z * BR + y) * kRow + x; }
};

// The source window of the deposit brick at (bx, by, bz) -- its cells and two
// around them -- as SW^2 x SEG row segments: per (y, z) row, x in [b-2, b-1], then
// BR/8 runs of 8 cells, then [b+BR, b+BR+1]. Each segment lies in one 8^3 sort
// brick along one x-row, so its particles are one contiguous range
// [cell_start[id], cell_start[id + len]) of the sorted order.
template <int BR, int BZ> struct Window {
  static constexpr int kSeg = 2 + BR / kBr, kSideY = BR + 2 * kHalo, kSideZ = BZ + 2 * kHalo,
                       kRanges = kSideY * kSideZ * kSeg;
  static __device__ __forceinline__ void segment(const Geom &G, int bx, int by, int bz, int r, uint32_t &id,
                                                 int &len) {
    const int sg = r % kSeg, row = r / kSeg;
    int j = by - kHalo + row % kSideY, k = bz - kHalo + row / kSideY;
    j += j < 0 ? G.n[1] : 0; j -= j >= G.n[1] ? G.n[1] : 0;
    k += k < 0 ? G.n[2] : 0; k -= k >= G.n[2] ? G.n[2] : 0;
    int x0;
    if (sg == 0) { x0 = bx - kHalo; len = kHalo; }
    else if (sg == kSeg - 1) { x0 = bx + BR; len = kHalo; }
    else { x0 = bx + (sg - 1) * kBr; len = kBr; }
    x0 += x0 < 0 ? G.n[0] : 0; x0 -= x0 >= G.n[0] ? G.n[0] : 0;
    id = brick_id(G, x0, j, k);
  }
};

// deposit brick b's origin (cells)
template <int BR, int BZ>
__device__ __forceinline__ void brick_origin(const Geom &G, int b, int &bx, int &by, int &bz) {
  const int ndx = G.n[0] / BR, ndy = G.n[1] / BR;
  bx = (b % ndx) * BR;
  by = ((b / ndx) % ndy) * BR;
  bz = (b / (ndx * ndy)) * BZ;
}

// per deposit brick: the particles of its source window (one warp per brick) and
// from that the number of work items, each at most kChunkMax particles
template <int BR, int BZ>
__global__ void k_work_count(Geom G, const int32_t *__restrict__ cs, Work w, int nb) {
  const int lane = threadIdx.x & 31;
  const int b = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (b >= nb) return;  // whole warps
  int bx, by, bz;
  brick_origin<BR, BZ>(G, b, bx, by, bz);
  long long total = 0;
  for (int r = lane; r < Window<BR, BZ>::kRanges; r += 32) {
    uint32_t id;
    int len;
    Window<BR, BZ>::segment(G, bx, by, bz, r, id, len);
    total += cs[id + len] - cs[id];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
  if (lane == 0) {
    const int c = (int)((total + kChunkMax - 1) / kChunkMax);
    const bool split = c > 1;
    w.cnt_a[b] = split ? c : 0;
    w.cnt_b[b] = split ? 0 : 1;
    w.cnt_s[b] = split ? 1 : 0;
    w.nchunk[b] = split ? c : 1;
  }
}

__global__ void k_work_fill(Work w, int nb) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t total_a = w.off_a[nb];
  if (b == 0) *w.n_items = total_a + w.off_b[nb];
  if (b >= nb) return;
  const int c = w.nchunk[b];
  if (c > 1) {
    // the slot count bounds the split bricks (see f32_create); a brick past it is
    // reported and left out rather than run as one oversized item
    const bool ok = w.off_s[b] < w.slot_cap;
    w.slot[b] = ok ? w.off_s[b] : -1;
    for (int q = 0; q < c; ++q) w.items[w.off_a[b] + q] = ok ? ((long long)b << 32 | q) : -1ll;
    if (!ok) atomicOr(w.err, kErrCapacity);
  } else {
    w.items[total_a + w.off_b[b]] = (long long)b << 32;
    w.slot[b] = -1;
  }
}

// trilinear deposit (particle.cpp:526-559, :586-658) of a particle with in-cell offsets
// o3 whose round() node is `node` (brick-relative) and value `val` (already times the
// field's fixed-point scale): of the 8 cells node - 1 .. node, which get products of
// x_l / (1 - x_l), those inside the brick are added (the others belong to the
// neighbouring bricks, which add them themselves); lanes with no target there issue
// no shared-memory access for it
template <int BR, int BZ>
__device__ __forceinline__ void deposit_trilinear(uint32_t *lo, uint32_t *hi, const int node[3], const float o3[3],
                                                  float val) {
  using A = Acc<BR, BZ>;
  float w[3][2];
  bool ok[3][2];
  const int ext[3] = {BR, BR, BZ};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float xl = o3[d] - (o3[d] >= 0.5f ? 1.f : 0.f) + 0.5f;
    w[d][0] = 1.f - xl;  // cell node - 1
    w[d][1] = xl;        // cell node
    ok[d][0] = (unsigned)(node[d] - 1) < (unsigned)ext[d];
    ok[d][1] = (unsigned)node[d] < (unsigned)ext[d];
  }
  const int base = A::slot(node[0] - 1, node[1] - 1, node[2] - 1);
#pragma unroll
  for (int oz = 0; oz < 2; ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
      const float wyz = w[2][oz] * w[1][oy] * val;
      const bool pyz = ok[2][oz] && ok[1][oy];
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int sl = base + (oz * BR + oy) * A::kRow + ox;
        const int32_t v = __float2int_rn(w[0][ox] * wyz);
        if (pyz && ok[0][ox]) add_fixed32(lo + sl, hi + sl, v);
      }
    }
}

// face-normal deposits (particle.cpp:498-524) of a particle in brick-relative cell r3:
// along d, face r3[d] gets (1 - x_l) R_d and face r3[d] + 1 gets x_l R_d, at the
// particle's cell across; the faces inside the brick are added. lo[d]/hi[d]: field d's words.
template <int BR, int BZ>
__device__ __forceinline__ void deposit_faces(uint32_t *const *lo, uint32_t *const *hi, const int r3[3],
                                              const float o3[3], const float ru[3], const float *scale) {
  using A = Acc<BR, BZ>;
  const int ext[3] = {BR, BR, BZ};
  bool in[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) in[d] = (unsigned)r3[d] < (unsigned)ext[d];
  const bool across[3] = {in[1] && in[2], in[0] && in[2], in[0] && in[1]};
  const int sl0 = A::slot(r3[0], r3[1], r3[2]);
  constexpr int step[3] = {1, A::kRow, BR * A::kRow};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float r = ru[d] * scale[1 + d];
    const int32_t v0 = __float2int_rn((1.f - o3[d]) * r), v1 = __float2int_rn(o3[d] * r);
    if (across[d] && in[d]) add_fixed32(lo[d] + sl0, hi[d] + sl0, v0);
    if (across[d] && (unsigned)(r3[d] + 1) < (unsigned)ext[d])
      add_fixed32(lo[d] + sl0 + step[d], hi[d] + sl0 + step[d], v1);
  }
}

// exclusive prefix of n <= 2 * blockDim.x int32 counts in place: a[0..n] (a[n] = total);
// every thread of the block calls it
__device__ __forceinline__ void block_exclusive_scan2(int32_t *a, int n, int32_t *warp_sums) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  const int i0 = 2 * t, i1 = 2 * t + 1;
  const int32_t v0 = i0 < n ? a[i0] : 0, v1 = i1 < n ? a[i1] : 0;
  int32_t x = v0 + v1;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int32_t ws = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += y;
    }
    if (lane < nw) warp_sums[lane] = ws;  // inclusive warp totals
  }
  __syncthreads();
  const int32_t before = (wid ? warp_sums[wid - 1] : 0) + x - (v0 + v1);
  if (i0 < n) a[i0] = before;
  if (i1 < n) a[i1] = before + v0;
  if (t == (int)blockDim.x - 1) a[n] = warp_sums[nw - 1];
  __syncthreads();
}

// Shared memory of the deposit CTA for bricks BR x BR x BZ: the accumulators of the NF
// fields (two words per slot; a multiple of 8 bytes), each warp's running field sums,
// maxima and minima (32 x 5 x 3 int64), the window's row-segment prefix and starts,
// misc words. Whatever shared memory the CTA takes is the L1's loss: at 1024 threads
// per SM the deposit's loads want every KB of L1 (measured: 40 KB more shared memory,
// 24% slower), so nothing per thread lives here.
template <int BR, int BZ, int NF> struct DepSmem {
  static constexpr int kRanges = Window<BR, BZ>::kRanges;
  static constexpr size_t kAcc = sizeof(uint32_t) * NF * Acc<BR, BZ>::kSlots;
  static constexpr size_t kBytes = 2 * kAcc + sizeof(long long) * 32 * 5 * 3 +
                                   sizeof(int32_t) * (2 * kRanges + 1) + sizeof(int32_t) * 40;
  static_assert(kRanges <= 2 * DepTraits<BR, BZ>::kThreads, "ranges exceed the block scan");
  static_assert(kBytes <= 227 * 1024, "deposit shared memory exceeds the per-block limit");
};

// warp sum, maximum and minimum of an int64 with 32-bit warp reductions. The sum: three
// pieces of the two's-complement value (bits 0-20 and 21-41 unsigned, 42-63 signed),
// whose 32-lane sums cannot overflow, recombined exactly. The maximum and minimum: the
// high words (signed), then the low words (unsigned) of the lanes holding that high word.
__device__ __forceinline__ long long warp_sum_i64(long long v) {
  const unsigned lo = (unsigned)(v & 0x1fffffll), mid = (unsigned)((v >> 21) & 0x1fffffll);
  const int hi = (int)(v >> 42);
  const unsigned slo = __reduce_add_sync(0xffffffffu, lo), smid = __reduce_add_sync(0xffffffffu, mid);
  const int shi = __reduce_add_sync(0xffffffffu, hi);
  return (long long)shi * (1ll << 42) + (long long)smid * (1ll << 21) + (long long)slo;
}
__device__ __forceinline__ long long warp_max_i64(long long v) {
  const int hi = (int)(v >> 32);
  const int mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? (unsigned)v : 0u);
  return (long long)(((unsigned long long)(unsigned)mh << 32) | ml);
}
__device__ __forceinline__ long long warp_min_i64(long long v) {
  const int hi = (int)(v >> 32);
  const int mh = __reduce_min_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_min_sync(0xffffffffu, hi == mh ? (unsigned)v : 0xffffffffu);
  return (long long)(((unsigned long long)(unsigned)mh << 32) | ml);
}

// Deposit into bricks of BR x BR x BZ interior cells, one walk over each brick's
// source window (the particles whose step-start cell lies within two cells of the
// brick). Per particle, every value the walk may need is loaded at once; then
//   DO_INT: the concentration and the face momentum at the *_int position (fields
//     C, RHS_RU x/y/z), when its x_int cell lies within one cell of the brick: the
//     targets inside the brick;
//   DO_NEW: RHS_T at the *_new position (RHS_Part_Temp), the same way.
// Field slots: 0 C, 1-3 RHS_RU x/y/z, 4 (FE) RHS_Part_Temp; scale exponents f.se[0..4].
// The flush also gathers the launch's exact field statistics into `totals` (15 int64
// words: sums, maxima, minima of the five fields; k_dep_stats_init sets them before the
// launch): each warp folds the sums, maxima and minima of the cells it flushes into its
// own running words (warp reductions, no block barrier), and at the end of the launch
// the block reduces them once. They are the momentum and energy balance sums and the
// field statistics, exact and independent of the order of the work.
template <bool DO_INT, bool DO_NEW, int BR, int BZ>
__global__ void __launch_bounds__(DepTraits<BR, BZ>::kThreads)
    k_dep32(Geom G, F32Form f, Set32 SI, Set32 SN, Work w, int twc, double *__restrict__ outC,
            double *__restrict__ outX, double *__restrict__ outY, double *__restrict__ outZ,
            double *__restrict__ outE, unsigned long long *__restrict__ totals, int ext) {
  constexpr int NF = (DO_INT ? 4 : 0) + (DO_NEW ? 1 : 0);
  constexpr int FE = DO_INT ? 4 : 0;  // accumulator index of RHS_Part_Temp
  constexpr int NB = BR * BR * BZ;
  constexpr int SLOTS = Acc<BR, BZ>::kSlots;
  constexpr int NR = Window<BR, BZ>::kRanges;
  extern __shared__ __align__(16) uint8_t dsm[];
  uint32_t *acc_lo = reinterpret_cast<uint32_t *>(dsm);
  uint32_t *acc_hi = acc_lo + NF * SLOTS;
  constexpr int T = DepTraits<BR, BZ>::kThreads;
  long long *wsum = reinterpret_cast<long long *>(acc_hi + NF * SLOTS);  // 32 x 5 (8-byte aligned)
  long long *wmax = wsum + 32 * 5;                                       // 32 x 5
  long long *wmin = wmax + 32 * 5;                                       // 32 x 5
  int32_t *pre = reinterpret_cast<int32_t *>(wmin + 32 * 5);             // NR + 1
  int32_t *beg = pre + NR + 1;                                          // NR
  int32_t *misc = beg + NR;                                             // 32 warp sums, item, last
  uint32_t *lo_f[5], *hi_f[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    lo_f[q] = acc_lo + (q < NF ? q : 0) * SLOTS;
    hi_f[q] = acc_hi + (q < NF ? q : 0) * SLOTS;
  }
  const int32_t n_items = *w.n_items;
  float scale[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) scale[q] = ldexpf(1.0f, f.se[q]);  // exact powers of two
  int se[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) se[q] = f.se[q];
  const bool ru_on = DO_INT && twc;
  if ((threadIdx.x & 31) < 5) {  // this warp's own words
    wsum[(threadIdx.x >> 5) * 5 + (threadIdx.x & 31)] = 0;
    wmax[(threadIdx.x >> 5) * 5 + (threadIdx.x & 31)] = LLONG_MIN;
    wmin[(threadIdx.x >> 5) * 5 + (threadIdx.x & 31)] = LLONG_MAX;
  }
  while (true) {
    if (threadIdx.x == 0) misc[32] = atomicAdd(&w.next[0], 1);
    __syncthreads();
    const int32_t item_idx = misc[32];
    if (item_idx >= n_items) break;
    const long long item = w.items[item_idx];
    if (item < 0) { __syncthreads(); continue; }
    const int brick = (int)(item >> 32), chunk = (int)(item & 0xffffffffll);
    const int nch = w.nchunk[brick];
    int bx, by, bz;
    brick_origin<BR, BZ>(G, brick, bx, by, bz);
    const int slot_idx = nch > 1 ? w.slot[brick] : -1;
    long long *tile = slot_idx >= 0 ? w.tiles + (int64_t)slot_idx * 5 * NB : nullptr;
    static_assert((2 * NF * SLOTS) % 4 == 0, "whole 16-byte vectors");
    for (int s = threadIdx.x; s < 2 * NF * SLOTS / 4; s += blockDim.x)
      reinterpret_cast<uint4 *>(acc_lo)[s] = make_uint4(0u, 0u, 0u, 0u);  // the lo and hi words, contiguous
    for (int r = threadIdx.x; r < NR; r += blockDim.x) {
      uint32_t id;
      int len;
      Window<BR, BZ>::segment(G, bx, by, bz, r, id, len);
      const int32_t a0 = f.cell_start[id];
      beg[r] = a0;
      pre[r] = f.cell_start[id + len] - a0;
    }
    __syncthreads();
    block_exclusive_scan2(pre, NR, misc);
    const int32_t total = pre[NR];
    const int32_t t0 = (int32_t)(((int64_t)total * chunk) / nch);
    const int32_t t1 = (int32_t)(((int64_t)total * (chunk + 1)) / nch);
    // Lane groups of 8 walk their own sub-range of the slice, 8 consecutive
    // particles per pass (one 32-byte sector of each 4-byte array), and the 4
    // groups of a warp take sub-ranges a quarter of the slice apart. Sorted
    // particles in a dense cell would otherwise put all 32 lanes of a warp on the
    // same accumulator slots, where the shared-memory atomics serialise.
    const int ngroups = (int)blockDim.x >> 3;
    const int grp = (int)(threadIdx.x >> 5) + ((int)blockDim.x >> 5) * (int)((threadIdx.x >> 3) & 3);
    const int32_t g0 = t0 + (int32_t)(((int64_t)(t1 - t0) * grp) / ngroups);
    const int32_t g1 = t0 + (int32_t)(((int64_t)(t1 - t0) * (grp + 1)) / ngroups);
    // segment of the thread's first particle: the last r with pre[r] <= t (binary
    // search); later particles only move forward (pre[NR] = total > t ends the scan)
    int seg = 0;
    {
      const int32_t tf = g0 + (int32_t)(threadIdx.x & 7);
      int hi = NR;
      while (hi - seg > 1) {
        const int mid = (seg + hi) >> 1;
        if (pre[mid] <= tf) seg = mid; else hi = mid;
      }
    }
    for (int32_t t = g0 + (int32_t)(threadIdx.x & 7); t < g1; t += 8) {
      while (pre[seg + 1] <= t) ++seg;
      const int32_t p = beg[seg] + (t - pre[seg]);
      // all loads first: one memory round trip per particle
      uint32_t ci = 0, cn = 0;
      float oi[3] = {0.f, 0.f, 0.f}, on3[3] = {0.f, 0.f, 0.f}, ru[3] = {0.f, 0.f, 0.f}, rt = 0.f;
      if (DO_INT) {
        ci = SI.cell[p];
#pragma unroll
        for (int d = 0; d < 3; ++d) oi[d] = SI.o[d][p];
        if (ru_on) {
#pragma unroll
          for (int d = 0; d < 3; ++d) ru[d] = f.rhs_u[d][p];
        }
      }
      if (DO_NEW) {
        cn = SN.cell[p];
#pragma unroll
        for (int d = 0; d < 3; ++d) on3[d] = SN.o[d][p];
        rt = f.rhs_t[p];
      }
      if (DO_INT) {
        const int r3[3] = {rel_local(ci_(ci), bx, G.n[0]), rel_local(cj_(ci), by, G.n[1]),
                           rel_local(ck_(ci), bz, G.n[2])};
        // only a cell within one of the brick reaches it
        if ((unsigned)(r3[0] + 1) <= (unsigned)(BR + 1) && (unsigned)(r3[1] + 1) <= (unsigned)(BR + 1) &&
            (unsigned)(r3[2] + 1) <= (unsigned)(BZ + 1)) {
          const int node[3] = {r3[0] + (oi[0] >= 0.5f ? 1 : 0), r3[1] + (oi[1] >= 0.5f ? 1 : 0),
                               r3[2] + (oi[2] >= 0.5f ? 1 : 0)};
          deposit_trilinear<BR, BZ>(lo_f[0], hi_f[0], node, oi, scale[0]);
          if (ru_on) deposit_faces<BR, BZ>(&lo_f[1], &hi_f[1], r3, oi, ru, scale);
        }
      }
      if (DO_NEW) {
        const int r3[3] = {rel_local(ci_(cn), bx, G.n[0]), rel_local(cj_(cn), by, G.n[1]),
                           rel_local(ck_(cn), bz, G.n[2])};
        if ((unsigned)(r3[0] + 1) <= (unsigned)(BR + 1) && (unsigned)(r3[1] + 1) <= (unsigned)(BR + 1) &&
            (unsigned)(r3[2] + 1) <= (unsigned)(BZ + 1)) {
          const int node[3] = {r3[0] + (on3[0] >= 0.5f ? 1 : 0), r3[1] + (on3[1] >= 0.5f ? 1 : 0),
                               r3[2] + (on3[2] >= 0.5f ? 1 : 0)};
          deposit_trilinear<BR, BZ>(lo_f[FE], hi_f[FE], node, on3, rt * scale[4]);
        }
      }
    }
    __syncthreads();
    if (tile) {
      // split brick: add this slice into the brick's global tile; the last slice writes the cells
      for (int s = threadIdx.x; s < NF * NB; s += blockDim.x) {
        const int q = s / NB, r = s % NB;
        const int sl = q * SLOTS + Acc<BR, BZ>::slot(r % BR, (r / BR) % BR, r / (BR * BR));
        const long long v = get_fixed(&acc_lo[sl], &acc_hi[sl]);
        const int fld = DO_INT ? q : 4;
        if (v) atomicAdd((unsigned long long *)&tile[fld * NB + r], (unsigned long long)v);
      }
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) misc[33] = (atomicAdd(&w.done[slot_idx], 1) == nch - 1);
      __syncthreads();
      const int last = misc[33];
      if (!last) continue;
      __threadfence();
    }
    long long tot[5] = {0, 0, 0, 0, 0}, vmax[5], vmin[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) { vmax[q] = LLONG_MIN; vmin[q] = LLONG_MAX; }
    for (int s = threadIdx.x; s < NB; s += blockDim.x) {
      const int lx = s % BR, ly = (s / BR) % BR, lz = s / (BR * BR);
      const long long g = glin3(G, bx + lx + 1, by + ly + 1, bz + lz + 1);
      const int sl = Acc<BR, BZ>::slot(lx, ly, lz);
#pragma unroll
      for (int fld = 0; fld < 5; ++fld) {
        if (fld < 4 ? !DO_INT : !DO_NEW) continue;
        const int q = fld < 4 ? fld : FE;
        long long v;
        if (tile) {
          v = __ldcg(&tile[fld * NB + s]);
          tile[fld * NB + s] = 0;  // ready for the next launch
        } else {
          v = get_fixed(&lo_f[q][sl], &hi_f[q][sl]);
        }
        const bool zero_ru = fld >= 1 && fld <= 3 && !twc;  // RHS_RU = 0 without TWC (grid.cpp:671)
        double *out = fld == 0 ? outC : (fld == 1 ? outX : (fld == 2 ? outY : (fld == 3 ? outZ : outE)));
        if (zero_ru) v = 0;
        out[g] = fixed_to_f64(v, se[fld]);
        tot[fld] += v;
        if (ext) {
          vmax[fld] = max(vmax[fld], v);
          vmin[fld] = min(vmin[fld], v);
        }
      }
    }
    {
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
      for (int fld = 0; fld < 5; ++fld) {
        if (fld < 4 ? !DO_INT : !DO_NEW) continue;
        const long long sm = warp_sum_i64(tot[fld]);
        if (lane == 0) wsum[wid * 5 + fld] += sm;
        if (ext) {  // the same for every thread of the launch
          const long long mx = warp_max_i64(vmax[fld]), mn = warp_min_i64(vmin[fld]);
          if (lane == 0) {
            wmax[wid * 5 + fld] = max(wmax[wid * 5 + fld], mx);
            wmin[wid * 5 + fld] = min(wmin[wid * 5 + fld], mn);
          }
        }
      }
    }
    if (tile && threadIdx.x == 0) w.done[slot_idx] = 0;
    __syncthreads();
  }
  // the launch's exact field statistics (integer order is the fp64 order at one scale):
  // one block reduction of the warps' running words, three atomics per field and block
  {
    const int q = threadIdx.x;
    if (q < NF) {
      const int fld = DO_INT ? q : 4;
      long long r = 0, mx = LLONG_MIN, mn = LLONG_MAX;
      for (int w2 = 0; w2 < T / 32; ++w2) {
        r += wsum[w2 * 5 + fld];
        mx = max(mx, wmax[w2 * 5 + fld]);
        mn = min(mn, wmin[w2 * 5 + fld]);
      }
      if (r) atomicAdd(&totals[fld], (unsigned long long)r);
      if (ext) {
        atomicMax(reinterpret_cast<long long *>(&totals[5 + fld]), mx);
        atomicMin(reinterpret_cast<long long *>(&totals[10 + fld]), mn);
      }
    }
  }
}

// statistics words of the fields a deposit launch writes: sums 0, maxima and minima at
// the ends of the int64 range
__global__ void k_dep_stats_init(unsigned long long *__restrict__ totals, int do_int, int do_new) {
  const int q = threadIdx.x;
  if (q >= 15 || !(q % 5 < 4 ? do_int : do_new)) return;
  totals[q] = q < 5 ? 0ull : (q < 10 ? (unsigned long long)LLONG_MIN : (unsigned long long)LLONG_MAX);
}

// The balance sums and field statistics of the last deposit, from the exact integer
// words as fp64 (correctly rounded): the momentum components' sums, the interior mean
// of RHS_Part_Temp (grid.cpp:541), and per field max, min and interior sum
// (fstat[3 q .. 3 q + 2]) for the fields this launch wrote.
__global__ void k_totals(F32Form f, const unsigned long long *__restrict__ totals, int do_int, int do_new, int ext,
                         double inv_cells, double *__restrict__ mom, double *__restrict__ emean,
                         double *__restrict__ fstat) {
  const int q = threadIdx.x;
  if (q >= 5 || !(q < 4 ? do_int : do_new)) return;
  const int se = f.se[q];
  if (ext) {
    fstat[3 * q + 0] = fixed_to_f64((long long)totals[5 + q], se);
    fstat[3 * q + 1] = fixed_to_f64((long long)totals[10 + q], se);
  }
  fstat[3 * q + 2] = fixed_to_f64((long long)totals[q], se);
  if (q >= 1 && q <= 3) mom[q - 1] = fstat[3 * q + 2];
  if (q == 4) *emean = fstat[3 * q + 2] * inv_cells;
}

__global__ void k_to_f32(const double *__restrict__ src, int64_t n, double shift, float *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)(src[i] - shift);
}

// upload: absolute fp64 positions -> cell + fp32 offset (the reference's trunc cell)
// particles p0 .. p0 + n - 1 from fp64 arrays holding them from index 0
__global__ void k_from_f64(Geom G, F32Form f, const double *__restrict__ x, const double *__restrict__ y,
                           const double *__restrict__ z, const double *__restrict__ u, const double *__restrict__ v,
                           const double *__restrict__ w, const double *__restrict__ t, double tref, int64_t p0,
                           int64_t n, int32_t *__restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t p = p0 + i;
  const double X[3] = {x[i], y[i], z[i]};
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
  B.v[0][p] = (float)u[i];
  B.v[1][p] = (float)v[i];
  B.v[2][p] = (float)w[i];
  B.v[3][p] = (float)(t[i] - tref);
}

// download: one array of a set as fp64 (positions back to absolute coordinates)
// particles p0 .. p0 + n - 1 into dst[0 .. n)
__global__ void k_to_f64_arr(Geom G, Set32 S, int comp, double tref, int64_t p0, int64_t n,
                             double *__restrict__ dst) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int64_t p = p0 + q;
  if (comp < 3) {
    const uint32_t c = S.cell[p];
    const int i = comp == 0 ? ci_(c) : (comp == 1 ? cj_(c) : ck_(c));
    dst[q] = ((double)i + (double)S.o[comp][p]) * (G.l[comp] / G.n[comp]);
  } else if (comp < 6) {
    dst[q] = (double)S.v[comp - 3][p];
  } else {
    dst[q] = (double)S.v[3][p] + tref;
  }
}

__global__ void k_keys32(Geom G, Set32 S, int64_t n, uint32_t *__restrict__ key) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t c = S.cell[p];
  key[p] = brick_id(G, ci_(c), cj_(c), ck_(c));
}

// any key above its successor: the storage is not in key order
__global__ void k_keys_unsorted(const uint32_t *__restrict__ key, int64_t n, int32_t *__restrict__ flag) {
  int unsorted = 0;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p + 1 < n; p += (int64_t)gridDim.x * blockDim.x)
    unsorted |= key[p] > key[p + 1];
  if (__syncthreads_or(unsorted) && threadIdx.x == 0) atomicOr(flag, 1);
}

// Per-particle arrays gathered through the sort permutation, up to kPermBatch
// arrays of one element type per launch: the permutation is read once per batch
// and every thread keeps one independent load per array in flight (a gather of
// one array per launch is bound by load latency, not bandwidth).
constexpr int kPermBatch = 8;
template <typename T> struct PermBatch {
  const T *src[kPermBatch];
  T *dst[kPermBatch];
};
template <typename T, int K>
__global__ void __launch_bounds__(256) k_perm_batch(PermBatch<T> b, const int32_t *__restrict__ idx, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t j = __ldcs(idx + i);
    T v[K];
#pragma unroll
    for (int a = 0; a < K; ++a) v[a] = __ldcs(b.src[a] + j);
#pragma unroll
    for (int a = 0; a < K; ++a) __stcs(b.dst[a] + i, v[a]);
  }
}

__global__ void k_f32_to_f64(const float *__restrict__ src, int64_t n, double *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}

__global__ void k_to_f32_shift(const float *__restrict__ src, int64_t n, double shift, double *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i] + shift;
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
  c.is = (float)iS;
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

int dep_launch(pstep_ctx *h, bool do_int, bool do_new, Set32 SI, Set32 SN, bool ext);

// check_sorted: first test whether the storage is in key order already (a population
// uploaded as an earlier step left it, e.g. a host round trip), and then only build the
// cell-start table; one 4-byte read-back
int sort_step(pstep_ctx *h, bool check_sorted = false) {
  // particles by brick-major cell of the base position; storage reordered; per-cell CSR kept
  F32Form &f = *h->f32;
  const Geom &G = h->geom;
  const int64_t n = h->np;
  const int64_t ncell = (int64_t)G.n[0] * G.n[1] * G.n[2];
  if (n > 0) {
    k_keys32<<<nb(n), kThreads, 0, h->stream>>>(G, f.set[SBASE], n, f.key);
    PSTEP_LAUNCHED(h);
  }
  bool in_order = false;
  if (check_sorted && n > 1) {
    PSTEP_CUDA(cudaMemsetAsync(f.unsorted, 0, sizeof(int32_t), h->stream));
    k_keys_unsorted<<<h->num_sms * 8, kThreads, 0, h->stream>>>(f.key, n, f.unsorted);
    PSTEP_LAUNCHED(h);
    int32_t u = 1;
    PSTEP_CUDA(cudaMemcpyAsync(&u, f.unsorted, sizeof u, cudaMemcpyDeviceToHost, h->stream));
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    in_order = u == 0;
  }
  // The order inside a cell is left as the scatter makes it: every result of this form
  // (integer deposit sums, per-particle states by id) is independent of storage order.
  if (in_order)
    TRY32(csr_count(h, f.key, 0, ncell, f.cell_start));
  else
    TRY32(csr_sort(h, f.key, 0, ncell, h->s.flag, f.cell_start, f.sidx, 0));
  if (n > 0 && !in_order) {
    Set32 &B = f.set[SBASE];
    // every 4-byte per-particle array that lives across steps; the addresses of their
    // pointer fields (float *, uint32_t *, int32_t *), swapped through memcpy
    void *arrs[32];
    int na = 0;
    for (int d = 0; d < 3; ++d) arrs[na++] = &B.o[d];
    for (int q = 0; q < 4; ++q) arrs[na++] = &B.v[q];
    arrs[na++] = &B.cell;
    arrs[na++] = &h->s.flag;
    arrs[na++] = &f.rhs_t;
    if (f.itp) arrs[na++] = &f.itp;
    for (int q = 0; q < 7; ++q)
      if (f.pp[q]) arrs[na++] = &f.pp[q];
    for (int q = 0; q < 4; ++q)
      if (f.gas[q]) arrs[na++] = &f.gas[q];
    // Scratch: the *_np1 set's 8 arrays. After the step's last stage the base set
    // holds the new positions and every *_int, *_new and *_np1 query reads the base
    // set, so the stage sets carry nothing across the step boundary.
    Set32 &S = f.set[SNP1];
    void *scr[kPermBatch] = {&S.cell, &S.o[0], &S.o[1], &S.o[2], &S.v[0], &S.v[1], &S.v[2], &S.v[3]};
    auto get = [](void *field) { void *p; memcpy(&p, field, sizeof p); return p; };
    auto put = [](void *field, void *p) { memcpy(field, &p, sizeof p); };
    const int pgrid = h->num_sms * 8;
    for (int a0 = 0; a0 < na; a0 += kPermBatch) {
      const int k = na - a0 < kPermBatch ? na - a0 : kPermBatch;
      PermBatch<uint32_t> pb{};
      for (int a = 0; a < k; ++a) {
        pb.src[a] = (const uint32_t *)get(arrs[a0 + a]);
        pb.dst[a] = (uint32_t *)get(scr[a]);
      }
      switch (k) {
        case 1: k_perm_batch<uint32_t, 1><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
        case 2: k_perm_batch<uint32_t, 2><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
        case 3: k_perm_batch<uint32_t, 3><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
        case 4: k_perm_batch<uint32_t, 4><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
        case 5: k_perm_batch<uint32_t, 5><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
        case 6: k_perm_batch<uint32_t, 6><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
        case 7: k_perm_batch<uint32_t, 7><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
        default: k_perm_batch<uint32_t, 8><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n); break;
      }
      PSTEP_LAUNCHED(h);
      for (int a = 0; a < k; ++a) {  // the gathered copy takes the array's place; the old one is scratch
        void *old = get(arrs[a0 + a]);
        put(arrs[a0 + a], pb.dst[a]);
        put(scr[a], old);
      }
    }
    // f.corr_y (the network output) is not carried: stage 0 rewrites it for every
    // particle before stages 1-3 read it, so it is the drive state's scratch here
    if (f.drive) {
      PermBatch<uint2> pb{};
      pb.src[0] = f.drive;
      pb.dst[0] = f.corr_y;
      k_perm_batch<uint2, 1><<<pgrid, 256, 0, h->stream>>>(pb, f.sidx, n);
      PSTEP_LAUNCHED(h);
      uint2 *t = f.drive;
      f.drive = f.corr_y;
      f.corr_y = t;
    }
  }
  if (n > 0) {
    PSTEP_CUDA(cudaMemsetAsync(&f.bounds[4], 0, sizeof(uint32_t), h->stream));
    k_max_count<<<1024, kThreads, 0, h->stream>>>(f.cell_start, ncell, &f.bounds[4]);
    PSTEP_LAUNCHED(h);
  }
  {  // deposit work list for this step's particle distribution
    Work &w = f.work;
    const int nbk = w.nbd;
    const int wblocks = (int)(((int64_t)nbk * 32 + kThreads - 1) / kThreads);  // one warp per brick
    if (w.br == 16)
      k_work_count<16, 16><<<wblocks, kThreads, 0, h->stream>>>(G, f.cell_start, w, nbk);
    else
      k_work_count<8, 8><<<wblocks, kThreads, 0, h->stream>>>(G, f.cell_start, w, nbk);
    PSTEP_LAUNCHED(h);
    TRY32(exclusive_scan(h, w.cnt_a, nbk, w.off_a, nullptr));
    TRY32(exclusive_scan(h, w.cnt_b, nbk, w.off_b, nullptr));
    TRY32(exclusive_scan(h, w.cnt_s, nbk, w.off_s, nullptr));
    k_work_fill<<<nb(nbk), kThreads, 0, h->stream>>>(w, nbk);
    PSTEP_LAUNCHED(h);
  }
  f.sorted = 1;
  return PSTEP_OK;
}

}  // namespace

int f32_create(pstep_ctx *h) {
  const Geom &G = h->geom;
  for (int d = 0; d < 3; ++d) {
    if (G.n[d] > kMaxN || G.n[d] % kBr != 0 || G.n[d] < 2 * kBr) {
      snprintf(h->err, sizeof h->err, "FP32 form needs cells per side a multiple of %d in [%d, %d]", kBr, 2 * kBr,
               kMaxN);
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
    // zeros (cell 0, offset 0) until a stage writes them: a stage that stopped early
    // (a device-side error) leaves nothing unwritten behind it
    PSTEP_CUDA(cudaMemsetAsync(f->set[s].cell, 0, sizeof(uint32_t) * cap, h->stream));
    for (int d = 0; d < 3; ++d) PSTEP_CUDA(cudaMemsetAsync(f->set[s].o[d], 0, sizeof(float) * cap, h->stream));
    for (int q = 0; q < 4; ++q) PSTEP_CUDA(cudaMemsetAsync(f->set[s].v[q], 0, sizeof(float) * cap, h->stream));
  }
  TRY32(dalloc32(h, f->rhs_t, cap));
  PSTEP_CUDA(cudaMemsetAsync(f->rhs_t, 0, sizeof(float) * cap, h->stream));
  for (int d = 0; d < 3; ++d) {
    TRY32(dalloc32(h, f->rhs_u[d], cap));
    PSTEP_CUDA(cudaMemsetAsync(f->rhs_u[d], 0, sizeof(float) * cap, h->stream));
  }
  if (h->cfg.flags & PSTEP_KEEP_GAS)
    for (int q = 0; q < 4; ++q) {
      TRY32(dalloc32(h, f->gas[q], cap));
      PSTEP_CUDA(cudaMemsetAsync(f->gas[q], 0, sizeof(float) * cap, h->stream));
    }
  const size_t gs = (size_t)G.gsize;
  for (int d = 0; d < 3; ++d) TRY32(dalloc32(h, f->uf[d], gs));
  TRY32(dalloc32(h, f->tf, gs));
  TRY32(dalloc32(h, f->key, cap));
  const size_t ncell = (size_t)G.n[0] * G.n[1] * G.n[2];
  TRY32(dalloc32(h, f->cell_start, ncell + 1));
  TRY32(dalloc32(h, f->sidx, cap));
  {  // deposit work list
    Work &w = f->work;
    // 16^3 where the grid allows (the window of a brick and two cells must not wrap
    // onto itself), else 8^3
    bool big = true;
    for (int d = 0; d < 3; ++d) big = big && G.n[d] % 16 == 0 && G.n[d] >= 32;
    w.br = big ? 16 : 8;
    w.bz = w.br;
    const int64_t nbk = (int64_t)(G.n[0] / w.br) * (G.n[1] / w.br) * (G.n[2] / w.bz);
    w.nbd = (int)nbk;
    // a split brick's window holds more than kChunkMax particles and the windows
    // hold at most kVisit * cap particles in all
    const int64_t visit = w.br == 16 ? DepTraits<16, 16>::kVisit : DepTraits<8, 8>::kVisit;
    w.slot_cap = visit * (int64_t)h->cap / kChunkMax + 1;
    w.err = h->err_word;
    const int64_t br3 = (int64_t)w.br * w.br * w.bz;
    // items: one per unsplit brick plus ceil(window / kChunkMax) <= 2 window / kChunkMax
    // per split brick, so at most nbk + 2 * kVisit * cap / kChunkMax
    TRY32(dalloc32(h, w.items, (size_t)(nbk + 2 * w.slot_cap + 64)));
    TRY32(dalloc32(h, w.nchunk, (size_t)nbk));
    TRY32(dalloc32(h, w.slot, (size_t)nbk));
    int32_t **scan_arrays[6] = {&w.cnt_a, &w.cnt_b, &w.cnt_s, &w.off_a, &w.off_b, &w.off_s};
    for (int q = 0; q < 6; ++q) TRY32(dalloc32(h, *scan_arrays[q], (size_t)nbk + 1));
    TRY32(dalloc32(h, w.n_items, 1));
    TRY32(dalloc32(h, w.next, 64));
    TRY32(dalloc32(h, w.done, (size_t)w.slot_cap));
    TRY32(dalloc32(h, w.tiles, (size_t)(w.slot_cap * 5 * br3)));
    PSTEP_CUDA(cudaMemsetAsync(w.done, 0, sizeof(int32_t) * w.slot_cap, h->stream));
    PSTEP_CUDA(cudaMemsetAsync(w.tiles, 0, sizeof(long long) * w.slot_cap * 5 * br3, h->stream));
    PSTEP_CUDA(cudaMemsetAsync(w.n_items, 0, sizeof(int32_t), h->stream));
  }
  TRY32(dalloc32(h, f->bounds, 8));
  TRY32(dalloc32(h, f->slots, kBoundSlots * 4));
  PSTEP_CUDA(cudaMemsetAsync(f->slots, 0, kBoundSlots * 4 * sizeof(uint32_t), h->stream));
  TRY32(dalloc32(h, f->pslots, kBoundSlots * 2));
  TRY32(dalloc32(h, f->unsorted, 1));
  f->pmax_state = 0;
  TRY32(dalloc32(h, f->se, 8));
  TRY32(dalloc32(h, f->totals, 16));
  TRY32(dalloc32(h, f->fstat, 16));
  PSTEP_CUDA(cudaMemsetAsync(f->fstat, 0, 16 * sizeof(double), h->stream));
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
  if (f->corr_mem) cudaFree(f->corr_mem);
  for (int q = 0; q < 7; ++q) dfree32(f->pp[q]);
  for (int q = 0; q < 4; ++q) dfree32(f->gas[q]);
  dfree32(f->drive);
  dfree32(f->corr_y);
  for (int d = 0; d < 3; ++d) { dfree32(f->rhs_u[d]); dfree32(f->uf[d]); }
  dfree32(f->tf); dfree32(f->key); dfree32(f->cell_start); dfree32(f->sidx);
  dfree32(f->bounds); dfree32(f->se); dfree32(f->slots); dfree32(f->pslots); dfree32(f->unsorted); dfree32(f->totals); dfree32(f->fstat);
  {
    Work &w = f->work;
    dfree32(w.items); dfree32(w.nchunk); dfree32(w.slot); dfree32(w.cnt_a); dfree32(w.cnt_b); dfree32(w.cnt_s);
    dfree32(w.off_a); dfree32(w.off_b); dfree32(w.off_s); dfree32(w.n_items); dfree32(w.next); dfree32(w.done);
    dfree32(w.tiles);
  }
  if (f->stage[0]) {
    cudaStreamSynchronize(f->copy_stream);
    for (int sl = 0; sl < 2; ++sl) {
      dfree32(f->stage[sl]);
      cudaEventDestroy(f->ev_copied[sl]);
      cudaEventDestroy(f->ev_used[sl]);
    }
    cudaStreamDestroy(f->copy_stream);
  }
  delete f;
  h->f32 = nullptr;
  return PSTEP_OK;
}

// the host-transfer staging of the FP32 form (first use)
static int stage_init(pstep_ctx *h) {
  F32Form &f = *h->f32;
  if (f.stage[0]) return PSTEP_OK;
  for (int sl = 0; sl < 2; ++sl) TRY32(dalloc32(h, f.stage[sl], (size_t)(kStageArrays * kStageChunk)));
  PSTEP_CUDA(cudaStreamCreateWithFlags(&f.copy_stream, cudaStreamNonBlocking));
  for (int sl = 0; sl < 2; ++sl) {
    PSTEP_CUDA(cudaEventCreateWithFlags(&f.ev_copied[sl], cudaEventDisableTiming));
    PSTEP_CUDA(cudaEventCreateWithFlags(&f.ev_used[sl], cudaEventDisableTiming));
  }
  return PSTEP_OK;
}

int f32_upload(pstep_ctx *h, const double *x, const double *y, const double *z, const double *u, const double *v,
               const double *w, const double *t, int on_device) {
  F32Form &f = *h->f32;
  const int64_t n = h->np;
  dfree32(f.itp);
  for (int q = 0; q < 7; ++q) dfree32(f.pp[q]);
  if (f.drive) PSTEP_CUDA(cudaMemsetAsync(f.drive, 0, sizeof(uint2) * (size_t)h->cap, h->stream));
  if (f.corr_y) PSTEP_CUDA(cudaMemsetAsync(f.corr_y, 0, sizeof(uint2) * (size_t)h->cap, h->stream));
  f.sorted = 0;
  f.pmax_state = 0;
  if (n == 0) return PSTEP_OK;
  if (!f.tref_set) {
    double t0 = 0.0;
    if (on_device) PSTEP_CUDA(cudaMemcpy(&t0, t, sizeof(double), cudaMemcpyDeviceToHost));
    else t0 = t[0];
    f.tref = (double)(float)t0;
    f.tref_set = 1;
  }
  const double *src[7] = {x, y, z, u, v, w, t};
  if (on_device) {
    k_from_f64<<<nb(n), kThreads, 0, h->stream>>>(h->geom, f, src[0], src[1], src[2], src[3], src[4], src[5],
                                                  src[6], f.tref, 0, n, h->err_word);
    PSTEP_LAUNCHED(h);
    return PSTEP_OK;
  }
  // host arrays: chunks of kStageChunk particles copied into the two staging slots in
  // turn on the copy stream, each converted on the handle's stream once it has landed
  TRY32(stage_init(h));
  for (int64_t c = 0, p0 = 0; p0 < n; ++c, p0 += kStageChunk) {
    const int sl = (int)(c & 1);
    const int64_t len = n - p0 < kStageChunk ? n - p0 : kStageChunk;
    // the slot's last conversion (of this upload, or of an earlier upload or read-back
    // still running on the handle's stream) is done; an event never recorded is complete
    PSTEP_CUDA(cudaStreamWaitEvent(f.copy_stream, f.ev_used[sl], 0));
    double *b = f.stage[sl];
    for (int q = 0; q < 7; ++q)
      PSTEP_CUDA(cudaMemcpyAsync(b + q * kStageChunk, src[q] + p0, sizeof(double) * len, cudaMemcpyHostToDevice,
                                 f.copy_stream));
    PSTEP_CUDA(cudaEventRecord(f.ev_copied[sl], f.copy_stream));
    PSTEP_CUDA(cudaStreamWaitEvent(h->stream, f.ev_copied[sl], 0));
    k_from_f64<<<nb(len), kThreads, 0, h->stream>>>(h->geom, f, b, b + kStageChunk, b + 2 * kStageChunk,
                                                    b + 3 * kStageChunk, b + 4 * kStageChunk, b + 5 * kStageChunk,
                                                    b + 6 * kStageChunk, f.tref, p0, len, h->err_word);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaEventRecord(f.ev_used[sl], h->stream));
  }
  // the host arrays may be reused when this returns: every copy has been read
  PSTEP_CUDA(cudaStreamSynchronize(f.copy_stream));
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

__global__ void k_d2f(const double *__restrict__ src, int64_t n, float *__restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)src[i];
}

int f32_set_props(pstep_ctx *h, const pstep_particle_props *pr, int on_device) {
  F32Form &f = *h->f32;
  if (f.sorted) {
    snprintf(h->err, sizeof h->err, "particle properties must be set before pstep_prime");
    return PSTEP_ERR_STATE;
  }
  TRY32(f32_set_tau(h, pr->tau_p, on_device));
  const double *src[7] = {pr->mass_ratio, pr->itth, pr->heat_is, pr->alpha, pr->accel[0], pr->accel[1], pr->accel[2]};
  const int64_t n = h->np;
  double *tmp = nullptr;
  if (!on_device && n > 0) TRY32(dalloc32(h, tmp, (size_t)n));
  for (int q = 0; q < 7; ++q) {
    if (!src[q]) {
      dfree32(f.pp[q]);
      continue;
    }
    if (!f.pp[q]) TRY32(dalloc32(h, f.pp[q], (size_t)h->cap));
    if (n == 0) continue;
    const double *s = src[q];
    if (!on_device) {
      PSTEP_CUDA(cudaMemcpyAsync(tmp, src[q], sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
      s = tmp;
    }
    k_d2f<<<nb(n), kThreads, 0, h->stream>>>(s, n, f.pp[q]);
    PSTEP_LAUNCHED(h);
  }
  if (tmp) {
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    dfree32(tmp);
  }
  return PSTEP_OK;
}

// host round-to-nearest-even fp32 -> bf16 bits (finite values)
static uint16_t bf16_bits(float v) {
  uint32_t u;
  memcpy(&u, &v, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

int f32_set_correction(pstep_ctx *h, const pstep_correction *pc) {
  F32Form &f = *h->f32;
  if (f.corr_mem) {
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    cudaFree(f.corr_mem);
    f.corr_mem = nullptr;
  }
  h->corr_on = 0;
  if (!pc) return PSTEP_OK;
  if (!pc->params || !(pc->nu_gas > 0)) {
    snprintf(h->err, sizeof h->err, "correction needs parameters and a positive gas viscosity");
    return PSTEP_ERR_ARG;
  }
  const Geom &G = h->geom;
  if (G.n[0] != G.n[1] || G.n[0] != G.n[2] || G.l[0] != G.l[1] || G.l[0] != G.l[2]) {
    snprintf(h->err, sizeof h->err, "the correction's d_p/dx needs a cubic grid");
    return PSTEP_ERR_CONFIG;
  }
  // weight tiles in the canonical K-major layout (tc05.cuh), then fp32 biases
  const size_t bias_off = corr::kImage;
  const size_t bytes = bias_off + sizeof(float) * (corr::kHid + corr::kHid + corr::kOutP);
  uint8_t *img = (uint8_t *)calloc(1, bytes);
  const float *P = pc->params;
  for (int o = 0; o < corr::kHid; ++o)
    for (int j = 0; j < corr::kInP; ++j)
      *(uint16_t *)(img + corr::W1 + tc05::tile_off(o, j, corr::kInP)) = bf16_bits(P[o * corr::kInP + j]);
  for (int o = 0; o < corr::kHid; ++o)
    for (int i = 0; i < corr::kHid; ++i)
      *(uint16_t *)(img + corr::W2 + tc05::tile_off(o, i, corr::kHid)) = bf16_bits(P[1088 + o * corr::kHid + i]);
  for (int o = 0; o < corr::kOutP; ++o)
    for (int i = 0; i < corr::kHid; ++i)
      *(uint16_t *)(img + corr::W3 + tc05::tile_off(o, i, corr::kHid)) = bf16_bits(P[5248 + o * corr::kHid + i]);
  float *bias = (float *)(img + bias_off);
  for (int q = 0; q < corr::kHid; ++q) bias[q] = P[1024 + q];
  for (int q = 0; q < corr::kHid; ++q) bias[corr::kHid + q] = P[5184 + q];
  for (int q = 0; q < corr::kOutP; ++q) bias[2 * corr::kHid + q] = P[6272 + q];
  cudaError_t e = cudaMalloc(&f.corr_mem, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(f.corr_mem, img, bytes, cudaMemcpyHostToDevice);
  free(img);
  if (e != cudaSuccess) {
    cudaGetLastError();
    f.corr_mem = nullptr;
    snprintf(h->err, sizeof h->err, "correction upload: %s", cudaGetErrorString(e));
    return PSTEP_ERR_CUDA;
  }
  CorrDev &cd = *reinterpret_cast<CorrDev *>(h->corr_dev);
  cd.image = (const uint4 *)f.corr_mem;
  cd.bias = (const float *)((const uint8_t *)f.corr_mem + bias_off);
  for (int q = 0; q < 10; ++q) { cd.shift[q] = pc->shift[q]; cd.scale[q] = pc->scale[q]; }
  for (int q = 0; q < 4; ++q) { cd.lo[q] = pc->lo[q]; cd.hi[q] = pc->hi[q]; }
  cd.inv_nu = (float)(1.0 / pc->nu_gas);
  cd.inv_prior_re = pc->prior_re > 0.f ? 1.f / pc->prior_re : 0.f;
  const pstep_config &cfg = h->cfg;
  cd.dp_per_itth = (cfg.nu > 0 && cfg.k > 0) ? (float)(1.0 / (cfg.nu * kPi * cfg.k)) : 0.f;
  cd.dp = (float)cfg.dp;
  cd.idx = (float)G.idx[0];
  h->corr_every_stage = pc->every_stage ? 1 : 0;
  cd.drive_cap = pc->drive_cap > 0.f ? pc->drive_cap : kDriveCap;
  if (!f.drive) TRY32(dalloc32(h, f.drive, (size_t)h->cap));
  PSTEP_CUDA(cudaMemsetAsync(f.drive, 0, sizeof(uint2) * (size_t)h->cap, h->stream));
  if (!f.corr_y) TRY32(dalloc32(h, f.corr_y, (size_t)h->cap));
  PSTEP_CUDA(cudaMemsetAsync(f.corr_y, 0, sizeof(uint2) * (size_t)h->cap, h->stream));
  h->corr_on = 1;
  return PSTEP_OK;
}

// fp32 copies of the fields just bound: which = 1 the velocity (3 fields), 2 the temperature
int f32_bind_fields(pstep_ctx *h, int which) {
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
    if (!src[q] || !(which & (q < 3 ? 1 : 2))) continue;
    k_to_f32<<<nb(gs), kThreads, 0, h->stream>>>(src[q], gs, q == 3 ? f.tref : 0.0, dst[q]);
    PSTEP_LAUNCHED(h);
  }
  return PSTEP_OK;
}

int f32_prime(pstep_ctx *h) {
  F32Form &f = *h->f32;
  TRY32(sort_step(h, true));
  const C32 c = make_c32(h, 0, 0.5, 1. / 6.);
  if (h->np > 0) {
    k_prime32<<<nb(h->np), kThreads, 0, h->stream>>>(h->geom, f, c.itth, h->np);
    PSTEP_LAUNCHED(h);
  }
  // part2gas_Temp_int at the base positions
  return dep_launch(h, false, true, f.set[SBASE], f.set[SBASE], true);
}

int f32_stage(pstep_ctx *h, int k, double pre, double post) {
  F32Form &f = *h->f32;
  const C32 c = make_c32(h, k, pre, post);
  const int64_t n = h->np;
  CorrDev cd = *reinterpret_cast<const CorrDev *>(h->corr_dev);
  cd.wait_limit = h->wait_limit;
  cd.idle_first = h->wait_idle ? 1u : 0u;
  if (n > 0 && h->corr_on && (k == 0 || h->corr_every_stage)) {
    // the network at this stage's x_int: persistent CTAs of two warpgroups, 4 per SM,
    // tiles of 128 particles
    prof_begin(h, PSTEP_PHASE_NETWORK);
    const int64_t pairs = (n + 2 * corr::kRows - 1) / (2 * corr::kRows);
    const unsigned grid = (unsigned)(pairs < 4 * (int64_t)h->num_sms ? pairs : 4 * (int64_t)h->num_sms);
    auto net = k == 0 ? k_corr_net<0> : (k == 1 ? k_corr_net<1> : (k == 2 ? k_corr_net<2> : k_corr_net<3>));
    // the shared-memory opt-in belongs to the current (launch) device: set it per launch
    PSTEP_CUDA(cudaFuncSetAttribute(net, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)corr::kAlloc));
    net<<<grid, corr::kThreads, corr::kAlloc, h->stream>>>(h->geom, f, c, n, h->err_word, cd);
    PSTEP_LAUNCHED(h);
    prof_end(h, PSTEP_PHASE_NETWORK);
  }
  if (k == 3) {  // the last stage gathers the step result's max u and max ug
    PSTEP_CUDA(cudaMemsetAsync(f.pslots, 0, sizeof(uint32_t) * kBoundSlots * 2, h->stream));
    f.pmax_state = 1;
  } else if (f.pmax_state == 1) {
    f.pmax_state = 0;  // a stage after the last one without the step's end
  }
  prof_begin(h, PSTEP_PHASE_ADVANCE);
  if (n > 0 && h->corr_on) {
    switch (k) {
      case 0: k_advance32_corr<0><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word, cd); break;
      case 1: k_advance32_corr<1><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word, cd); break;
      case 2: k_advance32_corr<2><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word, cd); break;
      default: k_advance32_corr<3><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word, cd); break;
    }
    PSTEP_LAUNCHED(h);
  } else if (n > 0) {
    switch (k) {
      case 0: k_advance32<0><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
      case 1: k_advance32<1><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
      case 2: k_advance32<2><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
      default: k_advance32<3><<<nb(n), 256, 0, h->stream>>>(h->geom, f, c, h->cfg.twc, n, h->err_word); break;
    }
    PSTEP_LAUNCHED(h);
  }
  prof_end(h, PSTEP_PHASE_ADVANCE);
  // one walk: concentration + momentum at *_int (the base itself at stage 0), RHS_T at *_new;
  // the field extrema (pstep_field_stats) only in the step's last stage, whose fields the
  // step leaves
  prof_begin(h, PSTEP_PHASE_DEPOSIT_INT);
  TRY32(dep_launch(h, true, true, f.set[h->int_is_base ? SBASE : SINT], f.set[SNEW], k == 3));
  prof_end(h, PSTEP_PHASE_DEPOSIT_INT);
  return PSTEP_OK;
}

namespace {
// one launch of the deposit variant for (do_int, do_new) with bricks BR x BR x BZ:
// persistent CTAs (as many as fit on the SMs) pulling work items
template <bool DO_INT, bool DO_NEW, int BR, int BZ>
int dep_run1(pstep_ctx *h, Set32 SI, Set32 SN, double *C, double *X, double *Y, double *Z, double *E, int ext) {
  constexpr int NF = (DO_INT ? 4 : 0) + (DO_NEW ? 1 : 0);
  constexpr size_t smem = DepSmem<BR, BZ, NF>::kBytes;
  auto kern = k_dep32<DO_INT, DO_NEW, BR, BZ>;
  PSTEP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  PSTEP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, DepTraits<BR, BZ>::kThreads, smem));
  if (per_sm < 1) {
    snprintf(h->err, sizeof h->err, "deposit kernel does not fit on an SM (%zu B shared memory)", smem);
    return PSTEP_ERR_CUDA;
  }
  F32Form &f = *h->f32;
  kern<<<h->num_sms * per_sm, DepTraits<BR, BZ>::kThreads, smem, h->stream>>>(h->geom, f, SI, SN, f.work,
                                                                               h->cfg.twc, C, X, Y, Z, E, f.totals, ext);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

template <int BR, int BZ>
int dep_run(pstep_ctx *h, bool do_int, bool do_new, Set32 SI, Set32 SN, double *C, double *X, double *Y, double *Z,
            double *E, int ext) {
  if (do_int && do_new) return dep_run1<true, true, BR, BZ>(h, SI, SN, C, X, Y, Z, E, ext);
  if (do_int) return dep_run1<true, false, BR, BZ>(h, SI, SN, C, X, Y, Z, E, ext);
  return dep_run1<false, true, BR, BZ>(h, SI, SN, C, X, Y, Z, E, ext);
}

int dep_launch(pstep_ctx *h, bool do_int, bool do_new, Set32 SI, Set32 SN, bool ext) {
  F32Form &f = *h->f32;
  k_scales<<<1, 32, 0, h->stream>>>(f);  // fold this advance's maxima into the fixed-point scales
  PSTEP_LAUNCHED(h);
  PSTEP_CUDA(cudaMemsetAsync(f.work.next, 0, sizeof(int32_t), h->stream));
  k_dep_stats_init<<<1, 32, 0, h->stream>>>(f.totals, do_int ? 1 : 0, do_new ? 1 : 0);
  PSTEP_LAUNCHED(h);
  double *C = h->dep[PSTEP_FIELD_C], *X = h->dep[PSTEP_FIELD_RU_X], *Y = h->dep[PSTEP_FIELD_RU_Y],
         *Z = h->dep[PSTEP_FIELD_RU_Z], *E = h->dep[PSTEP_FIELD_PART_TEMP];
  if (f.work.br == 16) {
    TRY32((dep_run<16, 16>(h, do_int, do_new, SI, SN, C, X, Y, Z, E, ext ? 1 : 0)));
  } else {
    TRY32((dep_run<8, 8>(h, do_int, do_new, SI, SN, C, X, Y, Z, E, ext ? 1 : 0)));
  }
  for (int q = 0; q < 5; ++q)
    if (q < 4 ? do_int : do_new) f.ext_ok[q] = ext ? 1 : 0;
  // interior values are final (periodic targets): refresh the ghost layers only
  if (do_int) {
    double *all[4] = {C, X, Y, Z};
    TRY32(fold_fields(h, all, 4, 2));
  }
  if (do_new) {
    double *e[1] = {E};
    TRY32(fold_fields(h, e, 1, 2));
  }
  // balance sums from the deposit's exact integer totals: the momentum components and
  // the interior mean of RHS_Part_Temp (grid.cpp:541)
  const Geom &G = h->geom;
  k_totals<<<1, 32, 0, h->stream>>>(f, f.totals, do_int ? 1 : 0, do_new ? 1 : 0, ext ? 1 : 0,
                                    1.0 / ((double)G.n[0] * G.n[1] * G.n[2]), h->mom_dev, h->emean_dev, f.fstat);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}
}  // namespace

// particle::max of u or ug (grid.cpp:726-727) as the last stage gathered them, when they
// describe the current base state (the step's result): PSTEP_OK with *out set, or -1
// when they are not available (the caller then makes a pass over the array)
int f32_fused_max(pstep_ctx *h, int id, double *out) {
  F32Form &f = *h->f32;
  if (f.pmax_state != 2 || (id != PSTEP_U && id != PSTEP_UG)) return -1;
  uint32_t keys[kBoundSlots * 2];
  PSTEP_CUDA(cudaMemcpyAsync(keys, f.pslots, sizeof keys, cudaMemcpyDeviceToHost, h->stream));
  PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  const int q = id == PSTEP_U ? 0 : 1;
  uint32_t best = 0;
  for (int s = 0; s < kBoundSlots; ++s) best = keys[2 * s + q] > best ? keys[2 * s + q] : best;
  if (best == 0) return -1;
  const uint32_t bits = (best & 0x80000000u) ? (best & 0x7fffffffu) : ~best;
  float v;
  memcpy(&v, &bits, sizeof v);
  *out = (double)v;
  return PSTEP_OK;
}

// a deposited field's max, min and interior sum as the last deposit that wrote it
// gathered them (FP32 form): PSTEP_OK with r set, or -1 when that deposit did not gather
// the extrema (a stage other than a step's last; the caller then makes a pass)
int f32_field_stats(pstep_ctx *h, int field, double r[3]) {
  F32Form &f = *h->f32;
  if (!f.ext_ok[field]) return -1;
  PSTEP_CUDA(cudaMemcpyAsync(r, f.fstat + 3 * field, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  return PSTEP_OK;
}

int f32_end_stage(pstep_ctx *h) {
  F32Form &f = *h->f32;
  Set32 t = f.set[SINT];
  f.set[SINT] = f.set[SNEW];
  f.set[SNEW] = t;
  return PSTEP_OK;
}

int f32_end_step(pstep_ctx *h) {
  F32Form &f = *h->f32;
  f.pmax_state = f.pmax_state == 1 ? 2 : 0;  // the last stage's maxima describe the new base
  Set32 t = f.set[SBASE];
  f.set[SBASE] = f.set[SNP1];
  f.set[SNP1] = t;
  prof_begin(h, PSTEP_PHASE_REORDER);
  int rc = sort_step(h);
  prof_end(h, PSTEP_PHASE_REORDER);
  return rc;
}

namespace {
__global__ void k_positions32(Geom G, Set32 S, const int32_t *__restrict__ idx, int32_t n, double *__restrict__ xyz) {
  const int32_t i = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n) return;
  const int32_t p = idx[i];
  if (p < 0) return;
  const uint32_t c = S.cell[p];
  const int cc[3] = {ci_(c), cj_(c), ck_(c)};
#pragma unroll
  for (int d = 0; d < 3; ++d) xyz[3 * i + d] = ((double)cc[d] + (double)S.o[d][p]) * (G.l[d] / G.n[d]);
}
}  // namespace

// positions (as pstep_get_particle_array returns them) of the particles at storage
// indices idx[0 .. n) (negative: skipped) into xyz (device, 3 per particle)
int f32_positions(pstep_ctx *h, const int32_t *idx, int32_t n, double *xyz) {
  F32Form &f = *h->f32;
  if (n <= 0) return PSTEP_OK;
  k_positions32<<<(n + kThreads - 1) / kThreads, kThreads, 0, h->stream>>>(h->geom, f.set[SBASE], idx, n, xyz);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

namespace {
// the base state of particles p0 .. p0 + n - 1 as fp64 (absolute positions, velocities,
// temperature) into dst[q][0 .. n): the arrays pstep_get_particle_array returns for
// PSTEP_X .. PSTEP_T, all seven from one read of each particle
__global__ void k_to_f64_all(Geom G, Set32 S, double tref, int64_t p0, int64_t n, double *__restrict__ x,
                             double *__restrict__ y, double *__restrict__ z, double *__restrict__ u,
                             double *__restrict__ v, double *__restrict__ w, double *__restrict__ t) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int64_t p = p0 + q;
  const uint32_t c = S.cell[p];
  x[q] = ((double)ci_(c) + (double)S.o[0][p]) * (G.l[0] / G.n[0]);
  y[q] = ((double)cj_(c) + (double)S.o[1][p]) * (G.l[1] / G.n[1]);
  z[q] = ((double)ck_(c) + (double)S.o[2][p]) * (G.l[2] / G.n[2]);
  u[q] = (double)S.v[0][p];
  v[q] = (double)S.v[1][p];
  w[q] = (double)S.v[2][p];
  t[q] = (double)S.v[3][p] + tref;
}
}  // namespace

// pstep_download_particles, FP32 form: the base state and the ids in storage order. Host
// destinations: chunks converted into the two staging slots in turn and copied out on the
// copy stream, all seven arrays per chunk, so one pipeline serves the whole download.
int f32_download(pstep_ctx *h, double *const dst[7], int32_t *flag, int on_device) {
  F32Form &f = *h->f32;
  const int64_t n = h->np;
  if (n == 0) return PSTEP_OK;
  const Set32 &B = f.set[SBASE];
  if (on_device) {
    k_to_f64_all<<<nb(n), kThreads, 0, h->stream>>>(h->geom, B, f.tref, 0, n, dst[0], dst[1], dst[2], dst[3],
                                                    dst[4], dst[5], dst[6]);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaMemcpyAsync(flag, h->s.flag, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, h->stream));
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    return PSTEP_OK;
  }
  TRY32(stage_init(h));
  for (int64_t c = 0, p0 = 0; p0 < n; ++c, p0 += kStageChunk) {
    const int sl = (int)(c & 1);
    const int64_t len = n - p0 < kStageChunk ? n - p0 : kStageChunk;
    double *b = f.stage[sl];
    PSTEP_CUDA(cudaStreamWaitEvent(h->stream, f.ev_copied[sl], 0));  // the slot's last copy (any call) is done
    k_to_f64_all<<<nb(len), kThreads, 0, h->stream>>>(h->geom, B, f.tref, p0, len, b, b + kStageChunk,
                                                      b + 2 * kStageChunk, b + 3 * kStageChunk, b + 4 * kStageChunk,
                                                      b + 5 * kStageChunk, b + 6 * kStageChunk);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaEventRecord(f.ev_used[sl], h->stream));
    PSTEP_CUDA(cudaStreamWaitEvent(f.copy_stream, f.ev_used[sl], 0));
    for (int q = 0; q < 7; ++q)
      PSTEP_CUDA(cudaMemcpyAsync(dst[q] + p0, b + q * kStageChunk, sizeof(double) * len, cudaMemcpyDeviceToHost,
                                 f.copy_stream));
    PSTEP_CUDA(cudaEventRecord(f.ev_copied[sl], f.copy_stream));
  }
  // the ids need no conversion: one copy behind the chunks, after everything enqueued on
  // the handle's stream so far
  PSTEP_CUDA(cudaEventRecord(f.ev_used[0], h->stream));
  PSTEP_CUDA(cudaStreamWaitEvent(f.copy_stream, f.ev_used[0], 0));
  PSTEP_CUDA(cudaMemcpyAsync(flag, h->s.flag, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, f.copy_stream));
  PSTEP_CUDA(cudaStreamSynchronize(f.copy_stream));
  return PSTEP_OK;
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
  if (id >= PSTEP_UG && !f.gas[0]) {
    snprintf(h->err, sizeof h->err, "gas values per particle need the PSTEP_KEEP_GAS flag");
    return PSTEP_ERR_CONFIG;
  }
  // particles p0 .. p0 + len - 1 as fp64 into out[0 .. len)
  auto convert = [&](int64_t p0, int64_t len, double *out) {
    if (set >= 0) {
      k_to_f64_arr<<<nb(len), kThreads, 0, h->stream>>>(h->geom, f.set[set], comp, f.tref, p0, len, out);
    } else if (id >= PSTEP_UG) {
      k_to_f32_shift<<<nb(len), kThreads, 0, h->stream>>>(f.gas[id - PSTEP_UG] + p0, len,
                                                          id == PSTEP_TG ? f.tref : 0.0, out);
    } else {
      k_f32_to_f64<<<nb(len), kThreads, 0, h->stream>>>(f.rhs_t + p0, len, out);  // RHS_T
    }
  };
  if (on_device) {
    convert(0, n, (double *)dst);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));  // complete on return, as for host destinations
    return PSTEP_OK;
  }
  // host destination: chunks converted into the staging slots in turn and copied out on
  // the copy stream, the copy of one overlapping the conversion of the next
  TRY32(stage_init(h));
  double *out = (double *)dst;
  for (int64_t c = 0, p0 = 0; p0 < n; ++c, p0 += kStageChunk) {
    const int sl = (int)(c & 1);
    const int64_t len = n - p0 < kStageChunk ? n - p0 : kStageChunk;
    PSTEP_CUDA(cudaStreamWaitEvent(h->stream, f.ev_copied[sl], 0));  // the slot's last copy (any call) is done
    convert(p0, len, f.stage[sl]);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaEventRecord(f.ev_used[sl], h->stream));
    PSTEP_CUDA(cudaStreamWaitEvent(f.copy_stream, f.ev_used[sl], 0));
    PSTEP_CUDA(cudaMemcpyAsync(out + p0, f.stage[sl], sizeof(double) * len, cudaMemcpyDeviceToHost, f.copy_stream));
    PSTEP_CUDA(cudaEventRecord(f.ev_copied[sl], f.copy_stream));
  }
  PSTEP_CUDA(cudaStreamSynchronize(f.copy_stream));
  return PSTEP_OK;
}

}  // namespace pstep
