// The reference's box gas step (grid.cpp) on the GPU, FP64, coupled to a pstep
// handle: the two-way-coupled gas response that turns the particle step's
// deposits into the gas disturbance (the learned correction's training runs).
//
// Every operation is its own kernel over the reference's loop range (ghost
// layers included where tensor0.cpp/tensor1.cpp include them), each element
// computed with the reference's operand order and no FMA contraction (this
// file is compiled with -fmad=false). Stencil results get their periodic ghost
// layers from one refresh kernel (each ghost cell copies its periodic image,
// which is what communicator.cpp:177-278's x, y, z passes leave). The Poisson
// solve is the reference's fixed-point iteration on constant-coefficient FFT
// solves (poisson.cpp:391-462); the FFT is an iterative radix-2 transform, one
// CTA per line in shared memory, with host-computed twiddles and
// modified-wavenumber tables. Interior sums (mean) and maxima are two-pass
// reductions in a fixed order of their own, so they round differently from
// the reference's sequential i-outer loop: that is the only source of
// difference from the CPU restatement.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "pstep_gas.h"
#include "pstep_internal.cuh"

namespace pgas {

constexpr double kPre[4] = {0.5, 0.5, 1., 1. / 6.};  // grid.cpp:16-23
constexpr double kPost[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};
constexpr int kT = 256;

enum {
  F_RU = 0, F_RU_INT = 3, F_RU_NEW = 6, F_RU_NP1 = 9, F_RHS_RU = 12, F_U = 15, F_RHO_FACE = 18, F_DUMMY = 21,
  F_DUMMY2 = 24, F_PDUMMY = 27, F_P = 30, F_RHS_POIS, F_C, F_RHO, F_RHO_INT, F_RHO_NEW, F_RHO_NP1, F_RHS_RHO, F_T,
  F_DIV, F_RHS_PT, F_CENTER, F_RHS_NEW, F_NF
};
// device scalars: P0 and its stage copies, dP0/dt, mean of RHS_Part_Temp, scratch mean, solve error
enum { S_P0, S_P0_INT, S_P0_NEW, S_P0_NP1, S_DP0, S_MEAN_E, S_MEAN, S_ERR, S_N };

struct Dim {
  int n, G;
  double idx, idx2;
};

__device__ __forceinline__ size_t ix(const Dim &d, int i, int j, int k) {
  return ((size_t)k * d.G + (size_t)j) * d.G + (size_t)i;
}

__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }

// element e of the box [lo, lo+ext)
__device__ __forceinline__ bool in_box(int64_t e, int l0, int l1, int l2, int e0, int e1, int e2, int &i, int &j,
                                       int &k) {
  if (e >= (int64_t)e0 * e1 * e2) return false;
  i = l0 + (int)(e % e0);
  j = l1 + (int)((e / e0) % e1);
  k = l2 + (int)(e / ((int64_t)e0 * e1));
  return true;
}

// tensor0::Equal_Div_F2C (tensor0.cpp:303-310), i, j, k in [0, n]
__global__ void k_div_f2c(Dim d, double *out, const double *tx, const double *ty, const double *tz) {
  int i, j, k;
  if (!in_box(gtid(), 0, 0, 0, d.n + 1, d.n + 1, d.n + 1, i, j, k)) return;
  out[ix(d, i, j, k)] = (tx[ix(d, i + 1, j, k)] - tx[ix(d, i, j, k)]) * d.idx +
                        (ty[ix(d, i, j + 1, k)] - ty[ix(d, i, j, k)]) * d.idx +
                        (tz[ix(d, i, j, k + 1)] - tz[ix(d, i, j, k)]) * d.idx;
}

// tensor0::Equal_Del2 (tensor0.cpp:312-320), interior
__global__ void k_del2(Dim d, double *out, const double *t) {
  int i, j, k;
  if (!in_box(gtid(), 1, 1, 1, d.n, d.n, d.n, i, j, k)) return;
  const size_t c = ix(d, i, j, k);
  out[c] = (t[ix(d, i + 1, j, k)] - 2 * t[c] + t[ix(d, i - 1, j, k)]) * d.idx2 +
           (t[ix(d, i, j + 1, k)] - 2 * t[c] + t[ix(d, i, j - 1, k)]) * d.idx2 +
           (t[ix(d, i, j, k + 1)] - 2 * t[c] + t[ix(d, i, j, k - 1)]) * d.idx2;
}

// tensor0::Equal_I{x,y,z}_C2F (tensor0.cpp:353-378): (t(c) + t(c - e_axis)) * 0.5
// with the axis index in [1, n+1] and the others over the ghosted range;
// with grad != 0, tensor1::Equal_Grad_C2F's component (t(c) - t(c - e_axis)) * idx
__global__ void k_c2f(Dim d, double *out, const double *t, int axis, int grad) {
  int i, j, k;
  const int a0 = axis == 0, a1 = axis == 1, a2 = axis == 2;
  if (!in_box(gtid(), a0, a1, a2, d.G - a0, d.G - a1, d.G - a2, i, j, k)) return;
  const size_t c = ix(d, i, j, k), m = ix(d, i - a0, j - a1, k - a2);
  out[c] = grad ? (t[c] - t[m]) * d.idx : (t[c] + t[m]) * 0.5;
}

// tensor0::Equal_I_F2C(tensor1) (tensor0.cpp:408-416), [0, n]^3
__global__ void k_i_f2c_vec(Dim d, double *out, const double *tx, const double *ty, const double *tz) {
  int i, j, k;
  if (!in_box(gtid(), 0, 0, 0, d.n + 1, d.n + 1, d.n + 1, i, j, k)) return;
  const double third = 1. / 3.;
  const size_t c = ix(d, i, j, k);
  out[c] = third * ((tx[c] + tx[ix(d, i + 1, j, k)]) * 0.5 + (ty[c] + ty[ix(d, i, j + 1, k)]) * 0.5 +
                    (tz[c] + tz[ix(d, i, j, k + 1)]) * 0.5);
}

// periodic ghost layers: every ghost cell takes its periodic image
__global__ void k_refresh(Dim d, double *f) {
  int i, j, k;
  if (!in_box(gtid(), 0, 0, 0, d.G, d.G, d.G, i, j, k)) return;
  const int n = d.n;
  const int si = i == 0 ? n : (i == n + 1 ? 1 : i);
  const int sj = j == 0 ? n : (j == n + 1 ? 1 : j);
  const int sk = k == 0 ? n : (k == n + 1 ? 1 : k);
  if (si != i || sj != j || sk != k) f[ix(d, i, j, k)] = f[ix(d, si, sj, sk)];
}

// ------------------------------------------------------------ elementwise
__global__ void k_lin2(double *out, double a, const double *x, double b, const double *y, int64_t n) {
  int64_t q = gtid();
  if (q < n) out[q] = a * x[q] + b * y[q];
}
__global__ void k_lin3(double *out, double a, const double *x, double b, const double *y, double c, const double *z,
                       int64_t n) {
  int64_t q = gtid();
  if (q < n) out[q] = a * x[q] + b * y[q] + c * z[q];
}
__global__ void k_axpy(double *y, double a, const double *x, int64_t n) {
  int64_t q = gtid();
  if (q < n) y[q] += a * x[q];
}
__global__ void k_div(double *out, const double *x, const double *y, int64_t n) {
  int64_t q = gtid();
  if (q < n) out[q] = x[q] / y[q];
}
__global__ void k_sdiv(double *out, double a, const double *y, int64_t n) {
  int64_t q = gtid();
  if (q < n) out[q] = a / y[q];
}
__global__ void k_mul(double *x, const double *y, int64_t n) {
  int64_t q = gtid();
  if (q < n) x[q] *= y[q];
}
__global__ void k_sub(double *x, const double *y, int64_t n) {
  int64_t q = gtid();
  if (q < n) x[q] -= y[q];
}
__global__ void k_add(double *x, const double *y, int64_t n) {
  int64_t q = gtid();
  if (q < n) x[q] += y[q];
}
__global__ void k_adds(double *x, double s, int64_t n) {
  int64_t q = gtid();
  if (q < n) x[q] += s;
}
__global__ void k_subs_dev(double *x, const double *s, int64_t n) {
  int64_t q = gtid();
  if (q < n) x[q] -= *s;
}
__global__ void k_muls(double *x, double s, int64_t n) {
  int64_t q = gtid();
  if (q < n) x[q] *= s;
}
__global__ void k_mul_to(double *out, const double *x, double s, int64_t n) {
  int64_t q = gtid();
  if (q < n) out[q] = x[q] * s;
}
__global__ void k_fill(double *x, double s, int64_t n) {
  int64_t q = gtid();
  if (q < n) x[q] = s;
}
// T = (P0_x / R) / rho (grid.cpp:221, :676)
__global__ void k_t_from_rho(double *T, const double *rho, const double *sc, int which, double R, int64_t n) {
  int64_t q = gtid();
  if (q < n) {
    const double a = sc[which] / R;
    T[q] = a / rho[q];
  }
}
// divergence = k/Cp * del2(1/rho_new) - R/(Cp*P0_new*Vcell) * RHS_Part_Temp (grid.cpp:562)
__global__ void k_div_u(double *div, const double *dy, const double *dz, const double *sc, double a, double R, double cp,
                        double vcell, int64_t n) {
  int64_t q = gtid();
  if (q < n) {
    const double b = -R / (cp * sc[S_P0_NEW] * vcell);
    div[q] = a * dy[q] + b * dz[q];
  }
}
// Update_P0 (grid.cpp:539-554); the mean is already in sc[S_MEAN_E]
__global__ void k_update_p0(double *sc, int k3, double dt_post, double dt_pre, double R, double cv, int cooling) {
  const double dp0 = cooling ? 0.0 : -R / cv * sc[S_MEAN_E];
  sc[S_DP0] = dp0;
  sc[S_P0_NP1] += dt_post * dp0;
  sc[S_P0_NEW] = k3 ? sc[S_P0_NP1] : sc[S_P0] + dt_pre * dp0;
}
__global__ void k_scalar_copy(double *sc, int dst, int src) { sc[dst] = sc[src]; }

// ----------------------------------------------------------- reductions
// one warp per (j, k) interior row
__global__ void k_rows(Dim d, const double *f, int mode, double *rows) {
  const int64_t w = gtid() >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nr = (int64_t)d.n * d.n;
  if (w >= nr) return;
  const int j = (int)(w % d.n) + 1, k = (int)(w / d.n) + 1;
  const double *r = f + ix(d, 0, j, k);
  double s = 0.0;
  for (int i = lane + 1; i <= d.n; i += 32) s = mode ? fmax(s, fabs(r[i])) : s + r[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_down_sync(0xffffffffu, s, o);
    s = mode ? fmax(s, v) : s + v;
  }
  if (lane == 0) rows[w] = s;
}
// one block: sum (mode 0, times inv) or maximum (mode 1) of the row values
__global__ void k_rows_total(const double *rows, int64_t nr, int mode, double inv, double *out) {
  __shared__ double sm[256];
  double s = 0.0;
  for (int64_t r = threadIdx.x; r < nr; r += blockDim.x) s = mode ? fmax(s, rows[r]) : s + rows[r];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] = mode ? fmax(sm[threadIdx.x], sm[threadIdx.x + o]) : sm[threadIdx.x] + sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = mode ? sm[0] : sm[0] * inv;
}

// ------------------------------------------------------------------ FFT
__global__ void k_pack(Dim d, double2 *z, const double *rhs) {
  int i, j, k;
  if (!in_box(gtid(), 0, 0, 0, d.n, d.n, d.n, i, j, k)) return;
  z[((size_t)k * d.n + j) * d.n + i] = make_double2(rhs[ix(d, i + 1, j + 1, k + 1)], 0.0);
}

// one CTA per line along `axis`; radix-2 decimation in time after a bit-reversal load
__global__ void k_fft_line(double2 *z, int n, int logn, int axis, const double2 *__restrict__ tw) {
  extern __shared__ double2 s[];
  const int64_t l = blockIdx.x;
  const int64_t nn = (int64_t)n * n;
  int64_t base, stride;
  if (axis == 0) { base = l * n; stride = 1; }
  else if (axis == 1) { base = (l / n) * nn + (l % n); stride = n; }
  else { base = l; stride = nn; }
  for (int e = threadIdx.x; e < n; e += blockDim.x) s[__brev((unsigned)e) >> (32 - logn)] = z[base + e * stride];
  __syncthreads();
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int q = threadIdx.x; q < n / 2; q += blockDim.x) {
      const int kk = q % half, ia = (q / half) * len + kk, ib = ia + half;
      const double2 w = tw[kk * step];
      const double2 a = s[ia], b = s[ib];
      const double tr = b.x * w.x - b.y * w.y;
      const double ti = b.x * w.y + b.y * w.x;
      s[ib] = make_double2(a.x - tr, a.y - ti);
      s[ia] = make_double2(a.x + tr, a.y + ti);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < n; e += blockDim.x) z[base + e * stride] = s[e];
}

__global__ void k_kmod_div(int n, double2 *z, const double *kmod) {
  const int64_t c = gtid();
  if (c >= (int64_t)n * n * n) return;
  const int i = (int)(c % n), j = (int)((c / n) % n), k = (int)(c / ((int64_t)n * n));
  if (i + j + k > 0) {
    const double den = kmod[i] + kmod[j] + kmod[k];
    double2 v = z[c];
    v.y /= den;
    v.x /= den;
    z[c] = v;
  }
}

__global__ void k_scatter(Dim d, double *out, const double *lin) {
  int i, j, k;
  if (!in_box(gtid(), 0, 0, 0, d.n, d.n, d.n, i, j, k)) return;
  out[ix(d, i + 1, j + 1, k + 1)] = lin[((size_t)k * d.n + j) * d.n + i];
}

__global__ void k_unpack(Dim d, double *out, const double2 *z, double tot) {
  int i, j, k;
  if (!in_box(gtid(), 0, 0, 0, d.n, d.n, d.n, i, j, k)) return;
  out[ix(d, i + 1, j + 1, k + 1)] = (-1) * z[((size_t)k * d.n + j) * d.n + i].x / tot;
}

}  // namespace pgas

struct pgas_ctx {
  pgas_config c;
  pgas::Dim d;
  int device;
  cudaStream_t stream;
  double *f[pgas::F_NF];
  double *sc;      // device scalars
  double *rows;    // reduction scratch (n^2)
  double2 *z;      // FFT buffer (n^3)
  double2 *tw[2];  // twiddles: forward, backward
  double *kmod;
  double r, vcell;
  int logn, last_iterations;
  int64_t size;
  char msg[256];
};

namespace {

using namespace pgas;

int gfail(pgas_ctx *g, int code, const char *what, cudaError_t e = cudaSuccess) {
  if (g) {
    if (e != cudaSuccess) snprintf(g->msg, sizeof g->msg, "%s: %s", what, cudaGetErrorString(e));
    else snprintf(g->msg, sizeof g->msg, "%s", what);
  }
  cudaGetLastError();
  return code;
}

#define GCUDA(g, x)                                                 \
  do {                                                              \
    cudaError_t e_ = (x);                                           \
    if (e_ != cudaSuccess) return gfail(g, PSTEP_ERR_CUDA, #x, e_); \
  } while (0)
#define GTRY(x)                      \
  do {                               \
    int rc_ = (x);                   \
    if (rc_ != PSTEP_OK) return rc_; \
  } while (0)

inline unsigned nblk(int64_t n) { return (unsigned)((n + kT - 1) / kT); }

struct Ops {
  pgas_ctx *g;
  cudaStream_t s;
  int64_t S;
  Dim d;
  explicit Ops(pgas_ctx *g_) : g(g_), s(g_->stream), S(g_->size), d(g_->d) {}
  double *F(int q) const { return g->f[q]; }
  void refresh(double *f) const { k_refresh<<<nblk(S), kT, 0, s>>>(d, f); }
  void div_f2c(double *out, const double *x, const double *y, const double *z) const {
    k_div_f2c<<<nblk((int64_t)(d.n + 1) * (d.n + 1) * (d.n + 1)), kT, 0, s>>>(d, out, x, y, z);
    refresh(out);
  }
  void del2(double *out, const double *t) const {
    k_del2<<<nblk((int64_t)d.n * d.n * d.n), kT, 0, s>>>(d, out, t);
    refresh(out);
  }
  void c2f(double *out, const double *t, int axis, int grad) const {
    k_c2f<<<nblk(S), kT, 0, s>>>(d, out, t, axis, grad);
    refresh(out);
  }
  void grad(double *const *o, const double *t) const {
    for (int a = 0; a < 3; ++a) k_c2f<<<nblk(S), kT, 0, s>>>(d, o[a], t, a, 1);
    for (int a = 0; a < 3; ++a) refresh(o[a]);
  }
  void copy(double *dst, const double *src) const {
    cudaMemcpyAsync(dst, src, sizeof(double) * S, cudaMemcpyDeviceToDevice, s);
  }
  // interior mean (mode 0) or max |.| (mode 1) into sc[slot]
  void reduce(const double *f, int mode, int slot) const {
    const int64_t nr = (int64_t)d.n * d.n;
    k_rows<<<nblk(nr * 32), kT, 0, s>>>(d, f, mode, g->rows);
    k_rows_total<<<1, 256, 0, s>>>(g->rows, nr, mode, 1.0 / ((double)d.n * d.n * d.n), g->sc + slot);
  }
  void mean_zero(double *f) const {
    reduce(f, 0, S_MEAN);
    k_subs_dev<<<nblk(S), kT, 0, s>>>(f, g->sc + S_MEAN, S);
  }
};

void ccp_fft(const Ops &o, const double *rhs, double *out) {
  pgas_ctx *g = o.g;
  const int n = g->c.n;
  const int64_t n3 = (int64_t)n * n * n;
  k_pack<<<nblk(n3), kT, 0, o.s>>>(o.d, g->z, rhs);
  const int th = n / 2 < 256 ? n / 2 : 256;
  const size_t sh = sizeof(double2) * (size_t)n;
  for (int a = 0; a < 3; ++a) k_fft_line<<<(unsigned)((int64_t)n * n), th, sh, o.s>>>(g->z, n, g->logn, a, g->tw[0]);
  k_kmod_div<<<nblk(n3), kT, 0, o.s>>>(n, g->z, g->kmod);
  for (int a = 0; a < 3; ++a) k_fft_line<<<(unsigned)((int64_t)n * n), th, sh, o.s>>>(g->z, n, g->logn, a, g->tw[1]);
  k_unpack<<<nblk(n3), kT, 0, o.s>>>(o.d, out, g->z, (double)n3);
}

int solve_poisson(pgas_ctx *g) {
  Ops o(g);
  double *C[3] = {o.F(F_DUMMY), o.F(F_DUMMY + 1), o.F(F_DUMMY + 2)};
  for (int a = 0; a < 3; ++a) k_sdiv<<<nblk(o.S), kT, 0, o.s>>>(C[a], 1., o.F(F_RHO_FACE + a), o.S);
  double *cc = o.F(F_CENTER), *rn = o.F(F_RHS_NEW), *P = o.F(F_P);
  double *pd[3] = {o.F(F_PDUMMY), o.F(F_PDUMMY + 1), o.F(F_PDUMMY + 2)};
  k_i_f2c_vec<<<nblk((int64_t)(g->c.n + 1) * (g->c.n + 1) * (g->c.n + 1)), kT, 0, o.s>>>(o.d, cc, C[0], C[1], C[2]);
  o.refresh(cc);
  k_sdiv<<<nblk(o.S), kT, 0, o.s>>>(cc, -1., cc, o.S);
  int it = 0;
  double error = 100;
  while (it < g->c.iterations && error > g->c.epsilon) {
    o.grad(pd, P);
    for (int a = 0; a < 3; ++a) k_mul<<<nblk(o.S), kT, 0, o.s>>>(pd[a], C[a], o.S);
    o.div_f2c(rn, pd[0], pd[1], pd[2]);
    k_sub<<<nblk(o.S), kT, 0, o.s>>>(rn, o.F(F_RHS_POIS), o.S);
    k_mul<<<nblk(o.S), kT, 0, o.s>>>(rn, cc, o.S);
    ccp_fft(o, rn, pd[0]);
    k_add<<<nblk(o.S), kT, 0, o.s>>>(P, pd[0], o.S);
    o.refresh(P);
    o.reduce(pd[0], 1, S_ERR);
    GCUDA(g, cudaMemcpyAsync(&error, g->sc + S_ERR, sizeof(double), cudaMemcpyDeviceToHost, o.s));
    GCUDA(g, cudaStreamSynchronize(o.s));
    it++;
  }
  g->last_iterations = it;
  return PSTEP_OK;
}

int update_particle(pgas_ctx *g, pstep_handle h, int k) {
  Ops o(g);
  for (int a = 0; a < 3; ++a) k_div<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_U + a), o.F(F_RU_INT + a), o.F(F_RHO_FACE + a), o.S);
  k_t_from_rho<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_T), o.F(F_RHO_NEW), g->sc, S_P0_NEW, g->r, o.S);
  if (!h) {
    k_fill<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_C), 0.0, o.S);
    for (int a = 0; a < 3; ++a) k_fill<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_RHS_RU + a), 0.0, o.S);
    k_fill<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_RHS_PT), 0.0, o.S);
    return PSTEP_OK;
  }
  GTRY(pstep_bind_velocity(h, o.F(F_U), o.F(F_U + 1), o.F(F_U + 2), 1));
  GTRY(pstep_bind_temperature(h, o.F(F_T), 1));
  GTRY(pstep_stage(h, k, kPre[k], kPost[k]));
  GTRY(pstep_get_field(h, PSTEP_FIELD_C, o.F(F_C), 1));
  if (g->c.twc) {
    for (int a = 0; a < 3; ++a) GTRY(pstep_get_field(h, PSTEP_FIELD_RU_X + a, o.F(F_RHS_RU + a), 1));
  } else {
    for (int a = 0; a < 3; ++a) k_fill<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_RHS_RU + a), 0.0, o.S);  // grid.cpp:671
  }
  GTRY(pstep_get_field(h, PSTEP_FIELD_PART_TEMP, o.F(F_RHS_PT), 1));
  return PSTEP_OK;
}

int stage(pgas_ctx *g, pstep_handle h, int k) {
  Ops o(g);
  const pgas_config &c = g->c;
  const double dt = c.dt;
  const int64_t S = o.S;
  // Update_Rho (grid.cpp:327-333)
  o.div_f2c(o.F(F_RHS_RHO), o.F(F_RU_INT), o.F(F_RU_INT + 1), o.F(F_RU_INT + 2));
  k_axpy<<<nblk(S), kT, 0, o.s>>>(o.F(F_RHO_NP1), -(dt * kPost[k]), o.F(F_RHS_RHO), S);
  if (k != 3) k_lin2<<<nblk(S), kT, 0, o.s>>>(o.F(F_RHO_NEW), 1, o.F(F_RHO), -dt * kPre[k], o.F(F_RHS_RHO), S);
  else o.copy(o.F(F_RHO_NEW), o.F(F_RHO_NP1));
  // Update_P0 (grid.cpp:539-554)
  o.reduce(o.F(F_RHS_PT), 0, S_MEAN_E);
  k_update_p0<<<1, 1, 0, o.s>>>(g->sc, k == 3, dt * kPost[k], dt * kPre[k], g->r, c.cv, c.cooling);
  // Update_Particle (grid.cpp:659-680)
  GTRY(update_particle(g, h, k));
  // Update_RU_WOP (grid.cpp:387-425)
  {
    double *U[3] = {o.F(F_U), o.F(F_U + 1), o.F(F_U + 2)};
    double *D[3] = {o.F(F_DUMMY), o.F(F_DUMMY + 1), o.F(F_DUMMY + 2)};
    double *D2[3] = {o.F(F_DUMMY2), o.F(F_DUMMY2 + 1), o.F(F_DUMMY2 + 2)};
    double *R[3] = {o.F(F_RHS_RU), o.F(F_RHS_RU + 1), o.F(F_RHS_RU + 2)};
    double *RUI[3] = {o.F(F_RU_INT), o.F(F_RU_INT + 1), o.F(F_RU_INT + 2)};
    o.div_f2c(o.F(F_DIV), U[0], U[1], U[2]);
    o.grad(D2, o.F(F_DIV));
    for (int a = 0; a < 3; ++a) o.del2(D[a], U[a]);
    for (int a = 0; a < 3; ++a)
      k_lin3<<<nblk(S), kT, 0, o.s>>>(R[a], -c.mp / g->vcell, R[a], c.mu0 / 3., D2[a], c.mu0, D[a], S);
    for (int e = 0; e < 3; ++e) {
      for (int a = 0; a < 3; ++a) o.c2f(D[a], U[e], a, 0);
      for (int a = 0; a < 3; ++a) o.c2f(D2[a], RUI[a], e, 0);
      for (int a = 0; a < 3; ++a) k_mul<<<nblk(S), kT, 0, o.s>>>(D[a], D2[a], S);
      o.div_f2c(D2[e], D[0], D[1], D[2]);
      k_sub<<<nblk(S), kT, 0, o.s>>>(R[e], D2[e], S);
    }
    for (int a = 0; a < 3; ++a) k_axpy<<<nblk(S), kT, 0, o.s>>>(R[a], c.a_force, RUI[a], S);
    k_adds<<<nblk(S), kT, 0, o.s>>>(R[0], -(c.a_force * c.rho0 * c.u0), S);
    const double gv[3] = {c.gx, c.gy, c.gz};
    for (int a = 0; a < 3; ++a) {
      k_adds<<<nblk(S), kT, 0, o.s>>>(o.F(F_RHO_FACE + a), -c.rho0, S);
      k_mul_to<<<nblk(S), kT, 0, o.s>>>(D[a], o.F(F_RHO_FACE + a), gv[a], S);
      k_add<<<nblk(S), kT, 0, o.s>>>(R[a], D[a], S);
    }
    for (int a = 0; a < 3; ++a) k_axpy<<<nblk(S), kT, 0, o.s>>>(o.F(F_RU_NP1 + a), dt * kPost[k], R[a], S);
    if (k != 3) {
      for (int a = 0; a < 3; ++a)
        k_lin2<<<nblk(S), kT, 0, o.s>>>(o.F(F_RU_NEW + a), 1, o.F(F_RU + a), dt * kPre[k], R[a], S);
    } else {
      for (int a = 0; a < 3; ++a) o.copy(o.F(F_RU_NEW + a), o.F(F_RU_NP1 + a));
    }
  }
  // Compute_Div_U_new (grid.cpp:556-563)
  k_sdiv<<<nblk(S), kT, 0, o.s>>>(o.F(F_DUMMY), 1., o.F(F_RHO_NEW), S);
  o.del2(o.F(F_DUMMY + 1), o.F(F_DUMMY));
  o.copy(o.F(F_DUMMY + 2), o.F(F_RHS_PT));
  if (c.cooling) o.mean_zero(o.F(F_DUMMY + 2));
  k_div_u<<<nblk(S), kT, 0, o.s>>>(o.F(F_DIV), o.F(F_DUMMY + 1), o.F(F_DUMMY + 2), g->sc, c.k / c.cp, g->r, c.cp,
                                   g->vcell, S);
  // Compute_RHS_Pois (grid.cpp:629-637)
  for (int a = 0; a < 3; ++a) o.c2f(o.F(F_RHO_FACE + a), o.F(F_RHO_NEW), a, 0);
  for (int a = 0; a < 3; ++a) k_div<<<nblk(S), kT, 0, o.s>>>(o.F(F_U + a), o.F(F_RU_NEW + a), o.F(F_RHO_FACE + a), S);
  o.div_f2c(o.F(F_RHS_POIS), o.F(F_U), o.F(F_U + 1), o.F(F_U + 2));
  k_sub<<<nblk(S), kT, 0, o.s>>>(o.F(F_RHS_POIS), o.F(F_DIV), S);
  k_muls<<<nblk(S), kT, 0, o.s>>>(o.F(F_RHS_POIS), 1. / (dt * kPre[k]), S);
  o.mean_zero(o.F(F_RHS_POIS));
  GCUDA(g, cudaGetLastError());
  // Solve_Poisson (grid.cpp:639-643)
  GTRY(solve_poisson(g));
  // Update_RU_WP (grid.cpp:651-657)
  {
    double *D[3] = {o.F(F_DUMMY), o.F(F_DUMMY + 1), o.F(F_DUMMY + 2)};
    o.grad(D, o.F(F_P));
    for (int a = 0; a < 3; ++a) k_axpy<<<nblk(S), kT, 0, o.s>>>(o.F(F_RU_NP1 + a), -(dt * kPost[k]), D[a], S);
    if (k != 3) {
      for (int a = 0; a < 3; ++a) k_axpy<<<nblk(S), kT, 0, o.s>>>(o.F(F_RU_NEW + a), -(dt * kPre[k]), D[a], S);
    } else {
      for (int a = 0; a < 3; ++a) o.copy(o.F(F_RU_NEW + a), o.F(F_RU_NP1 + a));
    }
  }
  // TimeAdvance_RK4 (grid.cpp:705-712)
  o.copy(o.F(F_RHO_INT), o.F(F_RHO_NEW));
  for (int a = 0; a < 3; ++a) o.copy(o.F(F_RU_INT + a), o.F(F_RU_NEW + a));
  k_scalar_copy<<<1, 1, 0, o.s>>>(g->sc, S_P0_INT, S_P0_NEW);
  if (h) GTRY(pstep_end_stage(h));
  GCUDA(g, cudaGetLastError());
  return PSTEP_OK;
}

}  // namespace

extern "C" {

int pgas_create(const pgas_config *cfg, pgas_handle *out) {
  if (!cfg || !out) return PSTEP_ERR_ARG;
  *out = nullptr;
  const int n = cfg->n;
  int logn = 0;
  while ((1 << logn) < n) ++logn;
  if (n < 8 || n > 1024 || (1 << logn) != n) return PSTEP_ERR_CONFIG;
  if (!(cfg->l > 0) || !(cfg->dt > 0) || cfg->iterations < 1) return PSTEP_ERR_CONFIG;
  pgas_ctx *g = new pgas_ctx();
  memset((void *)g, 0, sizeof(pgas_ctx));
  g->c = *cfg;
  g->logn = logn;
  g->d.n = n;
  g->d.G = n + 2;
  const double dx = cfg->l / (double)n;
  g->d.idx = 1. / dx;
  g->d.idx2 = 1. / (dx * dx);
  g->vcell = dx * dx * dx;
  g->r = cfg->cp - cfg->cv;
  g->size = (int64_t)(n + 2) * (n + 2) * (n + 2);
  cudaGetDevice(&g->device);
  auto alloc = [&](void **p, size_t bytes) {
    if (cudaMalloc(p, bytes) != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      return false;
    }
    return true;
  };
  bool ok = true;
  for (int q = 0; q < F_NF && ok; ++q) {
    ok = alloc((void **)&g->f[q], sizeof(double) * g->size);
    if (ok) cudaMemset(g->f[q], 0, sizeof(double) * g->size);
  }
  ok = ok && alloc((void **)&g->sc, sizeof(double) * S_N) && alloc((void **)&g->rows, sizeof(double) * n * n) &&
       alloc((void **)&g->z, sizeof(double2) * (size_t)n * n * n) && alloc((void **)&g->tw[0], sizeof(double2) * n) &&
       alloc((void **)&g->tw[1], sizeof(double2) * n) && alloc((void **)&g->kmod, sizeof(double) * n);
  if (!ok) {
    pgas_destroy(g);
    return PSTEP_ERR_NOMEM;
  }
  // twiddles (cos, -/+ sin of 2 pi m / n) and modified wavenumbers (poisson.cpp:428-448)
  const double two_pi = 2 * 3.141592653589793;
  double2 *tw = (double2 *)malloc(sizeof(double2) * n);
  for (int sgn = 0; sgn < 2; ++sgn) {
    for (int m = 0; m < n / 2; ++m) {
      const double a = two_pi * (double)m / (double)n;
      tw[m] = make_double2(cos(a), (sgn == 0 ? -1 : 1) * sin(a));
    }
    cudaMemcpy(g->tw[sgn], tw, sizeof(double2) * n, cudaMemcpyHostToDevice);
  }
  free(tw);
  double *km = (double *)malloc(sizeof(double) * n);
  {
    const double two_pi_over_l = two_pi / cfg->l;
    const double d2 = 2. / (dx * dx);
    for (int i = 0; i < n; ++i) {
      const double kk = ((i < n / 2) ? i : i - n) * two_pi_over_l;
      km[i] = (d2) * (1 - cos(kk * dx));
    }
  }
  cudaMemcpy(g->kmod, km, sizeof(double) * n, cudaMemcpyHostToDevice);
  free(km);
  if (cudaGetLastError() != cudaSuccess) {
    pgas_destroy(g);
    return PSTEP_ERR_CUDA;
  }
  *out = g;
  return PSTEP_OK;
}

int pgas_destroy(pgas_handle g) {
  if (!g) return PSTEP_ERR_ARG;
  if (g->stream) cudaStreamSynchronize(g->stream);
  else cudaDeviceSynchronize();
  for (int q = 0; q < F_NF; ++q)
    if (g->f[q]) cudaFree(g->f[q]);
  void *ps[6] = {g->sc, g->rows, g->z, g->tw[0], g->tw[1], g->kmod};
  for (void *p : ps)
    if (p) cudaFree(p);
  delete g;
  return PSTEP_OK;
}

int pgas_set_stream(pgas_handle g, void *stream) {
  if (!g) return PSTEP_ERR_ARG;
  g->stream = (cudaStream_t)stream;
  return PSTEP_OK;
}

int pgas_init(pgas_handle g, pstep_handle h, const double *ru_x, const double *ru_y, const double *ru_z, const double *rho,
              double p0, int on_device) {
  if (!g || !ru_x || !ru_y || !ru_z || !rho) return PSTEP_ERR_ARG;
  Ops o(g);
  const int n = g->c.n;
  const int64_t n3 = (int64_t)n * n * n;
  const double *src[4] = {ru_x, ru_y, ru_z, rho};
  const int dst[4] = {F_RU, F_RU + 1, F_RU + 2, F_RHO};
  // interior n^3 (i fastest) -> ghosted, staged through the FFT buffer
  for (int q = 0; q < 4; ++q) {
    GCUDA(g, cudaMemcpyAsync(g->z, src[q], sizeof(double) * n3,
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, o.s));
    k_scatter<<<nblk(n3), kT, 0, o.s>>>(o.d, o.F(dst[q]), (const double *)g->z);
    o.refresh(o.F(dst[q]));
    GCUDA(g, cudaStreamSynchronize(o.s));  // the buffer is reused for the next field
  }
  k_fill<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_P), 0.0, o.S);
  double sc[S_N] = {0};
  sc[S_P0] = sc[S_P0_INT] = sc[S_P0_NP1] = sc[S_P0_NEW] = p0;
  GCUDA(g, cudaMemcpyAsync(g->sc, sc, sizeof sc, cudaMemcpyHostToDevice, o.s));
  for (int a = 0; a < 3; ++a) {
    o.copy(o.F(F_RU_INT + a), o.F(F_RU + a));
    o.copy(o.F(F_RU_NP1 + a), o.F(F_RU + a));
  }
  o.copy(o.F(F_RHO_INT), o.F(F_RHO));
  o.copy(o.F(F_RHO_NP1), o.F(F_RHO));
  for (int a = 0; a < 3; ++a) o.c2f(o.F(F_RHO_FACE + a), o.F(F_RHO), a, 0);
  k_t_from_rho<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_T), o.F(F_RHO_INT), g->sc, S_P0_INT, g->r, o.S);
  for (int a = 0; a < 3; ++a) k_div<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_U + a), o.F(F_RU + a), o.F(F_RHO_FACE + a), o.S);
  if (h) {
    GTRY(pstep_set_stream(h, g->stream));
    GTRY(pstep_bind_velocity(h, o.F(F_U), o.F(F_U + 1), o.F(F_U + 2), 1));
    GTRY(pstep_bind_temperature(h, o.F(F_T), 1));
    GTRY(pstep_prime(h));
    GTRY(pstep_get_field(h, PSTEP_FIELD_PART_TEMP, o.F(F_RHS_PT), 1));
  } else {
    k_fill<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_RHS_PT), 0.0, o.S);
  }
  GCUDA(g, cudaGetLastError());
  GCUDA(g, cudaStreamSynchronize(o.s));
  return PSTEP_OK;
}

int pgas_stage(pgas_handle g, pstep_handle h, int k) {
  if (!g || k < 0 || k > 3) return PSTEP_ERR_ARG;
  if (h) GTRY(pstep_set_stream(h, g->stream));
  return stage(g, h, k);
}

int pgas_end_step(pgas_handle g, pstep_handle h) {
  if (!g) return PSTEP_ERR_ARG;
  Ops o(g);
  // Correct_mean_RU (grid.cpp:566-572, box)
  for (int a = 0; a < 3; ++a) o.mean_zero(o.F(F_RU_NP1 + a));
  k_adds<<<nblk(o.S), kT, 0, o.s>>>(o.F(F_RU_NP1), g->c.rho0 * g->c.u0, o.S);
  // TimeAdvance (grid.cpp:315-325)
  o.copy(o.F(F_RHO), o.F(F_RHO_NP1));
  for (int a = 0; a < 3; ++a) o.copy(o.F(F_RU + a), o.F(F_RU_NP1 + a));
  k_scalar_copy<<<1, 1, 0, o.s>>>(g->sc, S_P0, S_P0_NP1);
  if (h) GTRY(pstep_end_step(h));
  GCUDA(g, cudaGetLastError());
  return PSTEP_OK;
}

int pgas_step(pgas_handle g, pstep_handle h) {
  if (!g) return PSTEP_ERR_ARG;
  for (int k = 0; k < 4; ++k) GTRY(pgas_stage(g, h, k));
  return pgas_end_step(g, h);
}

int pgas_get_field(pgas_handle g, int id, double *dst, int on_device) {
  if (!g || !dst || id < 0 || id >= PGAS_NUM_FIELDS) return PSTEP_ERR_ARG;
  static const int map[PGAS_NUM_FIELDS] = {F_RU, F_RU + 1, F_RU + 2, F_RHO, F_P, F_T, F_U, F_U + 1, F_U + 2, F_C,
                                           F_RHS_RU, F_RHS_RU + 1, F_RHS_RU + 2, F_RHS_PT, F_DIV, F_RHO_NEW};
  GCUDA(g, cudaMemcpyAsync(dst, g->f[map[id]], sizeof(double) * g->size,
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, g->stream));
  if (!on_device) GCUDA(g, cudaStreamSynchronize(g->stream));
  return PSTEP_OK;
}

int pgas_p0(pgas_handle g, double *p0) {
  if (!g || !p0) return PSTEP_ERR_ARG;
  GCUDA(g, cudaMemcpyAsync(p0, g->sc + S_P0, sizeof(double), cudaMemcpyDeviceToHost, g->stream));
  GCUDA(g, cudaStreamSynchronize(g->stream));
  return PSTEP_OK;
}

int pgas_last_iterations(pgas_handle g) { return g ? g->last_iterations : -1; }
const char *pgas_last_error(pgas_handle g) { return g ? g->msg : "null handle"; }

}  // extern "C"
