/*
 * CPU restatement of the reference's box gas step, FP64, single rank.
 * TEST INFRASTRUCTURE (the checker of the GPU gas step). Built with
 * -ffp-contract=off: every expression is the IEEE sequence the reference
 * writes, in its operand order and over its loop ranges (ghost cells
 * included where the reference includes them).
 *
 * Reference map:
 *   grid.cpp:194-226 Initialize (given fields), :315-325 TimeAdvance,
 *   :327-333 Update_Rho, :387-425 Update_RU_WOP, :539-554 Update_P0,
 *   :556-563 Compute_Div_U_new, :566-572 Correct_mean_RU (box),
 *   :629-637 Compute_RHS_Pois, :639-643 Solve_Poisson, :651-657 Update_RU_WP,
 *   :659-680 Update_Particle, :705-712 TimeAdvance_RK4;
 *   poisson.cpp:391-411 (iterative constant-coefficient FFT solve) and
 *   :413-462 (CCP_FFT, modified wavenumber);
 *   tensor0.cpp:243-460, tensor1.cpp:170-330 (stencils, interpolations, sums);
 *   communicator.cpp:177-278 (periodic ghost refresh);
 *   simulation.cpp:38-66 (stage order).
 * Local index = global + 1, ghosted extent n+2 (tensor0.cpp:72-80).
 */
#include "gas_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double RK_PRE[4] = {0.5, 0.5, 1., 1. / 6.};   /* grid.cpp:16-19 */
static const double RK_POST[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};

enum {
  F_RU = 0, F_RU_INT = 3, F_RU_NEW = 6, F_RU_NP1 = 9, F_RHS_RU = 12, F_U = 15, F_RHO_FACE = 18, F_DUMMY = 21,
  F_DUMMY2 = 24, F_PDUMMY = 27, /* poisson's own tensor1 */
  F_P = 30, F_RHS_POIS, F_C, F_RHO, F_RHO_INT, F_RHO_NEW, F_RHO_NP1, F_RHS_RHO, F_T, F_DIV, F_RHS_PT,
  F_CENTER, F_RHS_NEW, F_NF
};

struct pgo_state {
  pgo_config c;
  pso_state *part;
  int n, G;
  size_t size;
  double dx, inv_dx, inv_dx2, vcell, r;
  double *f[F_NF];
  double p0, p0_int, p0_new, p0_np1, dp0_dt, mean_e;
  int last_iterations;
  double *fft;        /* n^3 complex */
  double *kmod;       /* per-axis modified wavenumber terms */
};

#define IX(g, i, j, k) (((size_t)(k) * (size_t)(g)->G + (size_t)(j)) * (size_t)(g)->G + (size_t)(i))

/* ------------------------------------------------------------------ FFT */
void gas_twiddles(double *w, int n, int sign) {
  const double two_pi = 2 * 3.141592653589793;
  for (int m = 0; m < n / 2; ++m) {
    const double a = two_pi * (double)m / (double)n;
    w[2 * m] = cos(a);
    w[2 * m + 1] = sign * sin(a);
  }
}

static void fft_line(double *x, int n, size_t stride, const double *w) {
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double *a = x + 2 * stride * (size_t)i, *b = x + 2 * stride * (size_t)j;
      double t0 = a[0], t1 = a[1];
      a[0] = b[0]; a[1] = b[1];
      b[0] = t0; b[1] = t1;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int i = 0; i < n; i += len)
      for (int k = 0; k < half; ++k) {
        const double wr = w[2 * (k * step)], wi = w[2 * (k * step) + 1];
        double *a = x + 2 * stride * (size_t)(i + k), *b = x + 2 * stride * (size_t)(i + k + half);
        const double tr = b[0] * wr - b[1] * wi;
        const double ti = b[0] * wi + b[1] * wr;
        const double ar = a[0], ai = a[1];
        b[0] = ar - tr;
        b[1] = ai - ti;
        a[0] = ar + tr;
        a[1] = ai + ti;
      }
  }
}

void gas_fft3d(double *data, int n, int sign) {
  double *w = (double *)malloc(sizeof(double) * (size_t)n);
  gas_twiddles(w, n, sign);
  const size_t nn = (size_t)n * n;
  for (size_t l = 0; l < nn; ++l) fft_line(data + 2 * l * n, n, 1, w);                      /* x */
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < n; ++i) fft_line(data + 2 * ((size_t)k * nn + i), n, (size_t)n, w);  /* y */
  for (size_t l = 0; l < nn; ++l) fft_line(data + 2 * l, n, nn, w);                          /* z */
  free(w);
}

void gas_mod_wavenumber(double *out, int n, double l) {
  const double two_pi = 2 * 3.141592653589793;
  const double two_pi_over_l = two_pi / l;
  const double d = l / (double)n;
  const double d2 = 2. / (d * d);
  for (int i = 0; i < n; ++i) {
    const double kk = ((i < n / 2) ? i : i - n) * two_pi_over_l;
    out[i] = (d2) * (1 - cos(kk * d));
  }
}

/* ------------------------------------------------------- tensor helpers */
static void refresh(const pgo_state *g, double *f) {
  const int N = g->n, G = g->G;
  for (int k = 0; k < G; ++k)
    for (int j = 0; j < G; ++j) {
      f[IX(g, 0, j, k)] = f[IX(g, N, j, k)];
      f[IX(g, N + 1, j, k)] = f[IX(g, 1, j, k)];
    }
  for (int k = 0; k < G; ++k)
    for (int i = 0; i < G; ++i) {
      f[IX(g, i, 0, k)] = f[IX(g, i, N, k)];
      f[IX(g, i, N + 1, k)] = f[IX(g, i, 1, k)];
    }
  for (int j = 0; j < G; ++j)
    for (int i = 0; i < G; ++i) {
      f[IX(g, i, j, 0)] = f[IX(g, i, j, N)];
      f[IX(g, i, j, N + 1)] = f[IX(g, i, j, 1)];
    }
}

static void copy(const pgo_state *g, double *d, const double *s) { memcpy(d, s, sizeof(double) * g->size); }
static void setv(const pgo_state *g, double *d, double v) {
  for (size_t q = 0; q < g->size; ++q) d[q] = v;
}

/* tensor0::Equal_Div_F2C (tensor0.cpp:303-310): i,j,k in [0, n] */
static void div_f2c(const pgo_state *g, double *out, const double *tx, const double *ty, const double *tz) {
  const int N = g->n;
  const double idx = g->inv_dx;
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N; ++j)
      for (int k = 0; k <= N; ++k)
        out[IX(g, i, j, k)] = (tx[IX(g, i + 1, j, k)] - tx[IX(g, i, j, k)]) * idx +
                              (ty[IX(g, i, j + 1, k)] - ty[IX(g, i, j, k)]) * idx +
                              (tz[IX(g, i, j, k + 1)] - tz[IX(g, i, j, k)]) * idx;
  refresh(g, out);
}

/* tensor0::Equal_Del2 (tensor0.cpp:312-320): interior */
static void del2(const pgo_state *g, double *out, const double *t) {
  const int N = g->n;
  const double i2 = g->inv_dx2;
  for (int i = 1; i <= N; ++i)
    for (int j = 1; j <= N; ++j)
      for (int k = 1; k <= N; ++k) {
        const size_t c = IX(g, i, j, k);
        out[c] = (t[IX(g, i + 1, j, k)] - 2 * t[c] + t[IX(g, i - 1, j, k)]) * i2 +
                 (t[IX(g, i, j + 1, k)] - 2 * t[c] + t[IX(g, i, j - 1, k)]) * i2 +
                 (t[IX(g, i, j, k + 1)] - 2 * t[c] + t[IX(g, i, j, k - 1)]) * i2;
      }
  refresh(g, out);
}

/* tensor0::Equal_I{x,y,z}_C2F (tensor0.cpp:353-378): out(i) = (t(i) + t(i-1)) * 0.5 along axis,
 * index along the axis in [1, n+1], the others over the whole ghosted range */
static void i_c2f(const pgo_state *g, double *out, const double *t, int axis) {
  const int G = g->G;
  for (int i = (axis == 0); i < G; ++i)
    for (int j = (axis == 1); j < G; ++j)
      for (int k = (axis == 2); k < G; ++k) {
        const size_t m = axis == 0 ? IX(g, i - 1, j, k) : axis == 1 ? IX(g, i, j - 1, k) : IX(g, i, j, k - 1);
        out[IX(g, i, j, k)] = (t[IX(g, i, j, k)] + t[m]) * 0.5;
      }
  refresh(g, out);
}

/* tensor1::Equal_Grad_C2F (tensor1.cpp:212-227) */
static void grad_c2f(const pgo_state *g, double *ox, double *oy, double *oz, const double *t) {
  const int G = g->G;
  const double idx = g->inv_dx;
  for (int i = 1; i < G; ++i)
    for (int j = 0; j < G; ++j)
      for (int k = 0; k < G; ++k) ox[IX(g, i, j, k)] = (t[IX(g, i, j, k)] - t[IX(g, i - 1, j, k)]) * idx;
  for (int i = 0; i < G; ++i)
    for (int j = 1; j < G; ++j)
      for (int k = 0; k < G; ++k) oy[IX(g, i, j, k)] = (t[IX(g, i, j, k)] - t[IX(g, i, j - 1, k)]) * idx;
  for (int i = 0; i < G; ++i)
    for (int j = 0; j < G; ++j)
      for (int k = 1; k < G; ++k) oz[IX(g, i, j, k)] = (t[IX(g, i, j, k)] - t[IX(g, i, j, k - 1)]) * idx;
  refresh(g, ox);
  refresh(g, oy);
  refresh(g, oz);
}

/* tensor0::Equal_I_F2C(tensor1) (tensor0.cpp:408-416) */
static void i_f2c_vec(const pgo_state *g, double *out, const double *tx, const double *ty, const double *tz) {
  const int N = g->n;
  const double third = 1. / 3.;
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N; ++j)
      for (int k = 0; k <= N; ++k)
        out[IX(g, i, j, k)] = third * ((tx[IX(g, i, j, k)] + tx[IX(g, i + 1, j, k)]) * 0.5 +
                                       (ty[IX(g, i, j, k)] + ty[IX(g, i, j + 1, k)]) * 0.5 +
                                       (tz[IX(g, i, j, k)] + tz[IX(g, i, j, k + 1)]) * 0.5);
  refresh(g, out);
}

/* tensor0::sum / mean (tensor0.cpp:418-435): interior, i outer, k inner */
static double mean(const pgo_state *g, const double *t) {
  const int N = g->n;
  double s = 0;
  for (int i = 1; i <= N; ++i)
    for (int j = 1; j <= N; ++j)
      for (int k = 1; k <= N; ++k) s += t[IX(g, i, j, k)];
  return s / (double)((int64_t)N * N * N);
}

static void make_mean_zero(const pgo_state *g, double *t) {
  const double m = mean(g, t);
  for (size_t q = 0; q < g->size; ++q) t[q] -= m;
}

/* tensor0::max_abs (tensor0.cpp:478-490) */
static double max_abs(const pgo_state *g, const double *t) {
  const int N = g->n;
  double m = fabs(t[IX(g, 1, 1, 1)]);
  for (int i = 1; i <= N; ++i)
    for (int j = 1; j <= N; ++j)
      for (int k = 1; k <= N; ++k) {
        const double a = t[IX(g, i, j, k)] >= 0 ? t[IX(g, i, j, k)] : -t[IX(g, i, j, k)];
        if (a > m) m = a;
      }
  return m;
}

/* ------------------------------------------------------------- lifecycle */
pgo_state *pgo_create(const pgo_config *cfg, pso_state *particles) {
  pgo_state *g = (pgo_state *)calloc(1, sizeof(pgo_state));
  g->c = *cfg;
  g->part = particles;
  g->n = cfg->n;
  g->G = cfg->n + 2;
  g->size = (size_t)g->G * g->G * g->G;
  g->dx = cfg->l / (double)cfg->n;
  g->inv_dx = 1. / g->dx;
  g->inv_dx2 = 1. / (g->dx * g->dx);
  g->vcell = g->dx * g->dx * g->dx;
  g->r = cfg->cp - cfg->cv; /* params.cpp:50 */
  for (int q = 0; q < F_NF; ++q) g->f[q] = (double *)calloc(g->size, sizeof(double));
  g->fft = (double *)malloc(sizeof(double) * 2 * (size_t)cfg->n * cfg->n * cfg->n);
  g->kmod = (double *)malloc(sizeof(double) * (size_t)cfg->n);
  gas_mod_wavenumber(g->kmod, cfg->n, cfg->l);
  return g;
}

void pgo_destroy(pgo_state *g) {
  if (!g) return;
  for (int q = 0; q < F_NF; ++q) free(g->f[q]);
  free(g->fft);
  free(g->kmod);
  free(g);
}

int pgo_init(pgo_state *g, const double *ru_x, const double *ru_y, const double *ru_z, const double *rho, double p0) {
  const int N = g->n;
  const double *src[4] = {ru_x, ru_y, ru_z, rho};
  double *dst[4] = {g->f[F_RU], g->f[F_RU + 1], g->f[F_RU + 2], g->f[F_RHO]};
  for (int q = 0; q < 4; ++q) {
    for (int k = 0; k < N; ++k)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) dst[q][IX(g, i + 1, j + 1, k + 1)] = src[q][((size_t)k * N + j) * N + i];
    refresh(g, dst[q]);
  }
  setv(g, g->f[F_P], 0.0);
  g->p0 = p0;
  /* grid.cpp:194-226 */
  for (int d = 0; d < 3; ++d) {
    copy(g, g->f[F_RU_INT + d], g->f[F_RU + d]);
    copy(g, g->f[F_RU_NP1 + d], g->f[F_RU + d]);
  }
  copy(g, g->f[F_RHO_INT], g->f[F_RHO]);
  copy(g, g->f[F_RHO_NP1], g->f[F_RHO]);
  g->p0_int = g->p0;
  g->p0_np1 = g->p0;
  for (int d = 0; d < 3; ++d) i_c2f(g, g->f[F_RHO_FACE + d], g->f[F_RHO], d);
  {
    const double a = g->p0_int / g->r;
    double *T = g->f[F_T], *R = g->f[F_RHO_INT];
    for (size_t q = 0; q < g->size; ++q) T[q] = a / R[q];
  }
  if (g->part) pso_prime(g->part, g->f[F_T], g->f[F_RHS_PT]);
  else setv(g, g->f[F_RHS_PT], 0.0);
  for (int d = 0; d < 3; ++d)
    for (size_t q = 0; q < g->size; ++q) g->f[F_U + d][q] = g->f[F_RU + d][q] / g->f[F_RHO_FACE + d][q];
  return 0;
}

/* grid.cpp:327-333 */
static void update_rho(pgo_state *g, int k) {
  const double dt = g->c.dt;
  double *R = g->f[F_RHS_RHO];
  div_f2c(g, R, g->f[F_RU_INT], g->f[F_RU_INT + 1], g->f[F_RU_INT + 2]);
  const double a = -(dt * RK_POST[k]);
  double *np1 = g->f[F_RHO_NP1];
  for (size_t q = 0; q < g->size; ++q) np1[q] += a * R[q];
  if (k != 3) {
    const double b = -dt * RK_PRE[k];
    double *nw = g->f[F_RHO_NEW], *rho = g->f[F_RHO];
    for (size_t q = 0; q < g->size; ++q) nw[q] = 1 * rho[q] + b * R[q];
  } else {
    copy(g, g->f[F_RHO_NEW], g->f[F_RHO_NP1]);
  }
}

/* grid.cpp:539-554 */
static void update_p0(pgo_state *g, int k) {
  g->mean_e = mean(g, g->f[F_RHS_PT]);
  if (g->c.cooling) g->dp0_dt = 0;
  else g->dp0_dt = -g->r / g->c.cv * g->mean_e;
  g->p0_np1 += g->c.dt * RK_POST[k] * g->dp0_dt;
  if (k != 3) g->p0_new = g->p0 + g->c.dt * RK_PRE[k] * g->dp0_dt;
  else g->p0_new = g->p0_np1;
}

/* grid.cpp:659-680 */
static void update_particle(pgo_state *g, int k) {
  for (int d = 0; d < 3; ++d)
    for (size_t q = 0; q < g->size; ++q) g->f[F_U + d][q] = g->f[F_RU_INT + d][q] / g->f[F_RHO_FACE + d][q];
  {
    const double a = g->p0_new / g->r;
    double *T = g->f[F_T], *R = g->f[F_RHO_NEW];
    for (size_t q = 0; q < g->size; ++q) T[q] = a / R[q];
  }
  if (g->part) {
    pso_stage(g->part, k, g->f[F_U], g->f[F_U + 1], g->f[F_U + 2], g->f[F_T], g->f[F_C], g->f[F_RHS_RU],
              g->f[F_RHS_RU + 1], g->f[F_RHS_RU + 2], g->f[F_RHS_PT]);
  } else {
    setv(g, g->f[F_C], 0.0);
    for (int d = 0; d < 3; ++d) setv(g, g->f[F_RHS_RU + d], 0.0);
    setv(g, g->f[F_RHS_PT], 0.0);
  }
}

/* grid.cpp:387-425 */
static void update_ru_wop(pgo_state *g, int k) {
  double **f = g->f;
  const size_t S = g->size;
  double *U[3] = {f[F_U], f[F_U + 1], f[F_U + 2]};
  double *D[3] = {f[F_DUMMY], f[F_DUMMY + 1], f[F_DUMMY + 2]};
  double *D2[3] = {f[F_DUMMY2], f[F_DUMMY2 + 1], f[F_DUMMY2 + 2]};
  double *RHS[3] = {f[F_RHS_RU], f[F_RHS_RU + 1], f[F_RHS_RU + 2]};
  double *RUI[3] = {f[F_RU_INT], f[F_RU_INT + 1], f[F_RU_INT + 2]};
  div_f2c(g, f[F_DIV], U[0], U[1], U[2]);
  grad_c2f(g, D2[0], D2[1], D2[2], f[F_DIV]);
  for (int d = 0; d < 3; ++d) del2(g, D[d], U[d]);
  {
    const double a = -g->c.mp / g->vcell, b = g->c.mu0 / 3., c = g->c.mu0;
    for (int d = 0; d < 3; ++d)
      for (size_t q = 0; q < S; ++q) RHS[d][q] = a * RHS[d][q] + b * D2[d][q] + c * D[d][q];
  }
  /* convection along axis e: dummy = I_C2F(U.e) (components x,y,z), dummy2 = I_e_C2F(RU_int) */
  for (int e = 0; e < 3; ++e) {
    for (int d = 0; d < 3; ++d) i_c2f(g, D[d], U[e], d);
    for (int d = 0; d < 3; ++d) i_c2f(g, D2[d], RUI[d], e);
    for (int d = 0; d < 3; ++d)
      for (size_t q = 0; q < S; ++q) D[d][q] *= D2[d][q];
    div_f2c(g, D2[e], D[0], D[1], D[2]);
    for (size_t q = 0; q < S; ++q) RHS[e][q] -= D2[e][q];
  }
  {
    const double A = g->c.a_force;
    for (int d = 0; d < 3; ++d)
      for (size_t q = 0; q < S; ++q) RHS[d][q] += A * RUI[d][q];
    const double s = g->c.a_force * g->c.rho0 * g->c.u0;
    for (size_t q = 0; q < S; ++q) RHS[0][q] -= s;
  }
  {
    const double gv[3] = {g->c.gx, g->c.gy, g->c.gz};
    for (int d = 0; d < 3; ++d) {
      double *RF = f[F_RHO_FACE + d];
      for (size_t q = 0; q < S; ++q) RF[q] -= g->c.rho0;
      for (size_t q = 0; q < S; ++q) D[d][q] = RF[q] * gv[d];
      for (size_t q = 0; q < S; ++q) RHS[d][q] += D[d][q];
    }
  }
  {
    const double a = g->c.dt * RK_POST[k];
    for (int d = 0; d < 3; ++d)
      for (size_t q = 0; q < S; ++q) f[F_RU_NP1 + d][q] += a * RHS[d][q];
    if (k != 3) {
      const double b = g->c.dt * RK_PRE[k];
      for (int d = 0; d < 3; ++d)
        for (size_t q = 0; q < S; ++q) f[F_RU_NEW + d][q] = 1 * f[F_RU + d][q] + b * RHS[d][q];
    } else {
      for (int d = 0; d < 3; ++d) copy(g, f[F_RU_NEW + d], f[F_RU_NP1 + d]);
    }
  }
}

/* grid.cpp:556-563 */
static void compute_div_u_new(pgo_state *g) {
  double **f = g->f;
  const size_t S = g->size;
  for (size_t q = 0; q < S; ++q) f[F_DUMMY][q] = 1. / f[F_RHO_NEW][q];
  del2(g, f[F_DUMMY + 1], f[F_DUMMY]);
  copy(g, f[F_DUMMY + 2], f[F_RHS_PT]);
  if (g->c.cooling) make_mean_zero(g, f[F_DUMMY + 2]);
  const double a = g->c.k / g->c.cp;
  const double b = -g->r / (g->c.cp * g->p0_new * g->vcell);
  for (size_t q = 0; q < S; ++q) f[F_DIV][q] = a * f[F_DUMMY + 1][q] + b * f[F_DUMMY + 2][q];
}

/* grid.cpp:629-637 */
static void compute_rhs_pois(pgo_state *g, int k) {
  double **f = g->f;
  const size_t S = g->size;
  for (int d = 0; d < 3; ++d) i_c2f(g, f[F_RHO_FACE + d], f[F_RHO_NEW], d);
  for (int d = 0; d < 3; ++d)
    for (size_t q = 0; q < S; ++q) f[F_U + d][q] = f[F_RU_NEW + d][q] / f[F_RHO_FACE + d][q];
  div_f2c(g, f[F_RHS_POIS], f[F_U], f[F_U + 1], f[F_U + 2]);
  for (size_t q = 0; q < S; ++q) f[F_RHS_POIS][q] -= f[F_DIV][q];
  const double s = 1. / (g->c.dt * RK_PRE[k]);
  for (size_t q = 0; q < S; ++q) f[F_RHS_POIS][q] *= s;
  make_mean_zero(g, f[F_RHS_POIS]);
}

/* poisson.cpp:413-462: constant-coefficient solve of del2 out = rhs, interiors only */
static void ccp_fft(pgo_state *g, const double *rhs, double *out) {
  const int N = g->n;
  const size_t nn = (size_t)N * N, tot = nn * N;
  double *d = g->fft;
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const size_t c = ((size_t)k * N + j) * N + i;
        d[2 * c + 1] = 0;
        d[2 * c] = rhs[IX(g, i + 1, j + 1, k + 1)];
      }
  gas_fft3d(d, N, -1);
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const size_t c = ((size_t)k * N + j) * N + i;
        if (i + j + k > 0) {
          const double den = g->kmod[i] + g->kmod[j] + g->kmod[k];
          d[2 * c + 1] /= den;
          d[2 * c] /= den;
        }
      }
  gas_fft3d(d, N, +1);
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i)
        out[IX(g, i + 1, j + 1, k + 1)] = (-1) * d[2 * (((size_t)k * N + j) * N + i)] / (double)tot;
}

/* grid.cpp:639-643 and poisson.cpp:391-411 */
static void solve_poisson(pgo_state *g) {
  double **f = g->f;
  const size_t S = g->size;
  double *C[3] = {f[F_DUMMY], f[F_DUMMY + 1], f[F_DUMMY + 2]};
  for (int d = 0; d < 3; ++d)
    for (size_t q = 0; q < S; ++q) C[d][q] = 1. / f[F_RHO_FACE + d][q];
  double *cc = f[F_CENTER], *rn = f[F_RHS_NEW], *P = f[F_P];
  double *pd[3] = {f[F_PDUMMY], f[F_PDUMMY + 1], f[F_PDUMMY + 2]};
  i_f2c_vec(g, cc, C[0], C[1], C[2]);
  for (size_t q = 0; q < S; ++q) cc[q] = -1. / cc[q];
  int it = 0;
  double error = 100;
  while (it < g->c.iterations && error > g->c.epsilon) {
    grad_c2f(g, pd[0], pd[1], pd[2], P);
    for (int d = 0; d < 3; ++d)
      for (size_t q = 0; q < S; ++q) pd[d][q] *= C[d][q];
    div_f2c(g, rn, pd[0], pd[1], pd[2]);
    for (size_t q = 0; q < S; ++q) rn[q] -= f[F_RHS_POIS][q];
    for (size_t q = 0; q < S; ++q) rn[q] *= cc[q];
    ccp_fft(g, rn, pd[0]);
    for (size_t q = 0; q < S; ++q) P[q] += pd[0][q];
    refresh(g, P);
    error = max_abs(g, pd[0]);
    it++;
  }
  g->last_iterations = it;
}

/* grid.cpp:651-657 */
static void update_ru_wp(pgo_state *g, int k) {
  double **f = g->f;
  const size_t S = g->size;
  double *D[3] = {f[F_DUMMY], f[F_DUMMY + 1], f[F_DUMMY + 2]};
  grad_c2f(g, D[0], D[1], D[2], f[F_P]);
  const double a = -(g->c.dt * RK_POST[k]);
  for (int d = 0; d < 3; ++d)
    for (size_t q = 0; q < S; ++q) f[F_RU_NP1 + d][q] += a * D[d][q];
  if (k != 3) {
    const double b = -(g->c.dt * RK_PRE[k]);
    for (int d = 0; d < 3; ++d)
      for (size_t q = 0; q < S; ++q) f[F_RU_NEW + d][q] += b * D[d][q];
  } else {
    for (int d = 0; d < 3; ++d) copy(g, f[F_RU_NEW + d], f[F_RU_NP1 + d]);
  }
}

int pgo_step(pgo_state *g) {
  double **f = g->f;
  for (int k = 0; k < 4; ++k) {
    update_rho(g, k);
    update_p0(g, k);
    update_particle(g, k);
    update_ru_wop(g, k);
    compute_div_u_new(g);
    compute_rhs_pois(g, k);
    solve_poisson(g);
    update_ru_wp(g, k);
    /* TimeAdvance_RK4 (grid.cpp:705-712) */
    copy(g, f[F_RHO_INT], f[F_RHO_NEW]);
    for (int d = 0; d < 3; ++d) copy(g, f[F_RU_INT + d], f[F_RU_NEW + d]);
    g->p0_int = g->p0_new;
    if (g->part) pso_end_stage(g->part);
  }
  /* Correct_mean_RU (grid.cpp:566-572, box) */
  for (int d = 0; d < 3; ++d) make_mean_zero(g, f[F_RU_NP1 + d]);
  {
    const double s = g->c.rho0 * g->c.u0;
    for (size_t q = 0; q < g->size; ++q) f[F_RU_NP1][q] += s;
  }
  /* TimeAdvance (grid.cpp:315-325) */
  copy(g, f[F_RHO], f[F_RHO_NP1]);
  for (int d = 0; d < 3; ++d) copy(g, f[F_RU + d], f[F_RU_NP1 + d]);
  g->p0 = g->p0_np1;
  if (g->part) pso_end_step(g->part);
  return 0;
}

double *pgo_field(pgo_state *g, int id) {
  switch (id) {
    case PGO_RU_X: return g->f[F_RU];
    case PGO_RU_Y: return g->f[F_RU + 1];
    case PGO_RU_Z: return g->f[F_RU + 2];
    case PGO_RHO: return g->f[F_RHO];
    case PGO_P: return g->f[F_P];
    case PGO_T: return g->f[F_T];
    case PGO_U_X: return g->f[F_U];
    case PGO_U_Y: return g->f[F_U + 1];
    case PGO_U_Z: return g->f[F_U + 2];
    case PGO_C: return g->f[F_C];
    case PGO_RHS_RU_X: return g->f[F_RHS_RU];
    case PGO_RHS_RU_Y: return g->f[F_RHS_RU + 1];
    case PGO_RHS_RU_Z: return g->f[F_RHS_RU + 2];
    case PGO_RHS_PART_TEMP: return g->f[F_RHS_PT];
    case PGO_DIVERGENCE: return g->f[F_DIV];
    case PGO_RHO_NEW: return g->f[F_RHO_NEW];
    default: return 0;
  }
}

double pgo_scalar(const pgo_state *g, int id) {
  switch (id) {
    case PGO_P0: return g->p0;
    case PGO_P0_NEW: return g->p0_new;
    case PGO_MEAN_E: return g->mean_e;
    case PGO_LAST_ITERATIONS: return (double)g->last_iterations;
    default: return 0;
  }
}
