/*
 * CPU restatement of the reference particle step, FP64, single rank.
 * TEST INFRASTRUCTURE (the checker): only tests, smoke() and bench.py's CPU
 * baseline use it. Built with -ffp-contract=off so every expression is the
 * IEEE sequence written below, in the reference's operand order.
 *
 * Reference map (particle.cpp unless noted):
 *   x2i/y2j/z2k :106-119, x2i_round... :121-134, MODE_Lx/y/z :58-104,
 *   SortValidX/Y/Z :150-250, ToBuf/FromBuf/SWAP/RESIZE :136-311,
 *   update_position :314-338, gas2part_velocity :340-360,
 *   update_velocity :362-399, gas2part_Temp_int/new :402-456,
 *   Compute_RHS_Temp_int/new :460-478, update_Temp :480-496,
 *   part2gas_velocity :498-524, part2gas_concentration :526-559,
 *   part2gas_Temp_int/new :586-658, Send_Recv_X/Y/Z + Send_Recv :745-858,
 *   communicator.cpp:422-511 (cumulative ghost fold, z then y then x),
 *   communicator.cpp:177-278 (ghost refresh, x then y then z),
 *   tensor0.cpp:418-435 (sum/mean), grid.cpp:207-226, 315-325, 659-680, 705-712.
 * Single rank: il = jl = kl = 0, bs = 1, xl = 0, xh = (ih+1)*dx = N*dx,
 * every neighbour is this rank.
 */
#include "pstep_oracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define PSO_PI 3.141592653589793 /* params.h:5 */

struct pso_state {
  pso_config c;
  int64_t cap, np, edge_hits;
  double idx, dx, xh; /* idx = 1./dx (particle.cpp:19); xh = (ih+1)*dx (gridsize.cpp:83-88) */
  double *a[PSO_NARRAYS];
  int32_t *flag;
  double *rec0, *rec1; /* leaver records: 29 doubles each (ToBuf layout) */
  double *prop[8];      /* per-particle properties by id (pso_set_props) or NULL */
  int64_t nprop;
};

enum { PR_TAU, PR_MASS, PR_ITTH, PR_HEAT_IS, PR_ALPHA, PR_AX, PR_AY, PR_AZ };

/* property q of the particle at storage index i, or the scalar fallback */
static double prop_or(const pso_state *s, int q, int64_t i, double scalar) {
  if (!s->prop[q]) return scalar;
  const int32_t id = s->flag[i];
  return (id >= 0 && id < s->nprop) ? s->prop[q][id] : scalar;
}

#define G(s) ((s)->c.n + 2)
#define AT(f, s, i, j, k) (f)[((size_t)(k) * G(s) + (size_t)(j)) * G(s) + (size_t)(i)]

pso_state *pso_create(const pso_config *cfg, int64_t capacity) {
  pso_state *s = (pso_state *)calloc(1, sizeof(pso_state));
  if (!s) return 0;
  s->c = *cfg;
  s->cap = capacity;
  s->dx = s->c.l / (double)s->c.n;
  s->idx = 1. / s->dx;
  s->xh = (double)((s->c.n - 1) + 1) * s->dx;
  for (int i = 0; i < PSO_NARRAYS; ++i) s->a[i] = (double *)calloc((size_t)(capacity > 0 ? capacity : 1), sizeof(double));
  s->flag = (int32_t *)calloc((size_t)(capacity > 0 ? capacity : 1), sizeof(int32_t));
  s->rec0 = (double *)malloc(sizeof(double) * 29 * (size_t)(capacity > 0 ? capacity : 1));
  s->rec1 = (double *)malloc(sizeof(double) * 29 * (size_t)(capacity > 0 ? capacity : 1));
  return s;
}

void pso_destroy(pso_state *s) {
  if (!s) return;
  for (int i = 0; i < PSO_NARRAYS; ++i) free(s->a[i]);
  for (int q = 0; q < 8; ++q) free(s->prop[q]);
  free(s->flag); free(s->rec0); free(s->rec1);
  free(s);
}

double *pso_array(pso_state *s, int id) { return (id >= 0 && id < PSO_NARRAYS) ? s->a[id] : 0; }
int32_t *pso_flag(pso_state *s) { return s->flag; }
int64_t pso_np(const pso_state *s) { return s->np; }
int64_t pso_edge_hits(const pso_state *s) { return s->edge_hits; }

int pso_load(pso_state *s, int64_t n, const double *x, const double *y, const double *z, const double *u,
             const double *v, const double *w, const double *t, const int32_t *flag) {
  if (n < 0 || n > s->cap) return -1;
  s->np = n;
  size_t b = (size_t)n * sizeof(double);
  memcpy(s->a[PSO_X], x, b); memcpy(s->a[PSO_Y], y, b); memcpy(s->a[PSO_Z], z, b);
  memcpy(s->a[PSO_U], u, b); memcpy(s->a[PSO_V], v, b); memcpy(s->a[PSO_W], w, b);
  memcpy(s->a[PSO_T], t, b);
  memcpy(s->flag, flag, (size_t)n * sizeof(int32_t));
  return 0;
}

static void copy_arr(pso_state *s, int dst, int src) { memcpy(s->a[dst], s->a[src], (size_t)s->np * sizeof(double)); }

/* communicator.cpp:422-511 on one rank: z planes (all i,j), then y rows (all i, interior k),
 * then x columns (interior j,k); each ghost layer is added into the opposite interior layer. */
static void fold_cum(const pso_state *s, double *f) {
  const int G = G(s), N = s->c.n;
  for (int i = 0; i < G; ++i)
    for (int j = 0; j < G; ++j) {
      double top = AT(f, s, i, j, G - 1), bot = AT(f, s, i, j, 0);
      AT(f, s, i, j, G - 2) += bot;
      AT(f, s, i, j, 1) += top;
    }
  for (int i = 0; i < G; ++i)
    for (int k = 1; k <= N; ++k) {
      double top = AT(f, s, i, G - 1, k), bot = AT(f, s, i, 0, k);
      AT(f, s, i, G - 2, k) += bot;
      AT(f, s, i, 1, k) += top;
    }
  for (int j = 1; j <= N; ++j)
    for (int k = 1; k <= N; ++k) {
      double top = AT(f, s, G - 1, j, k), bot = AT(f, s, 0, j, k);
      AT(f, s, G - 2, j, k) += bot;
      AT(f, s, 1, j, k) += top;
    }
}

/* communicator.cpp:177-278 on one rank: x (interior j,k), y (all i, interior k), z (all i,j) */
static void refresh(const pso_state *s, double *f) {
  const int G = G(s), N = s->c.n;
  for (int j = 1; j <= N; ++j)
    for (int k = 1; k <= N; ++k) {
      AT(f, s, G - 1, j, k) = AT(f, s, 1, j, k);
      AT(f, s, 0, j, k) = AT(f, s, G - 2, j, k);
    }
  for (int i = 0; i < G; ++i)
    for (int k = 1; k <= N; ++k) {
      AT(f, s, i, G - 1, k) = AT(f, s, i, 1, k);
      AT(f, s, i, 0, k) = AT(f, s, i, G - 2, k);
    }
  for (int i = 0; i < G; ++i)
    for (int j = 0; j < G; ++j) {
      AT(f, s, i, j, G - 1) = AT(f, s, i, j, 1);
      AT(f, s, i, j, 0) = AT(f, s, i, j, G - 2);
    }
}

static void zero(const pso_state *s, double *f) {
  size_t n = (size_t)G(s) * G(s) * G(s);
  for (size_t i = 0; i < n; ++i) f[i] = 0.0;
}

/* a node index past the ghost layer (x_new == L exactly) would be read or written out of
 * bounds by the reference; count it and clamp so the restatement itself stays in bounds */
static int guard(pso_state *s, int i) {
  if (i < 1 || i > s->c.n + 1) { s->edge_hits++; return i < 1 ? 1 : s->c.n + 1; }
  return i;
}
static int guard_face(pso_state *s, int i) {
  if (i < 1 || i > s->c.n) { s->edge_hits++; return i < 1 ? 1 : s->c.n; }
  return i;
}

/* particle.cpp:402-456 at positions (px,py,pz) */
static void gas2part_temp(pso_state *s, int px, int py, int pz, const double *T) {
  double *X = s->a[px], *Y = s->a[py], *Z = s->a[pz], *Tg = s->a[PSO_TG];
  const double idx = s->idx;
  for (int64_t i = 0; i < s->np; ++i) {
    int ii = (int)(round(X[i] * idx)), jj = (int)(round(Y[i] * idx)), kk = (int)(round(Z[i] * idx));
    double x_l = X[i] * idx - ii + 0.5, y_l = Y[i] * idx - jj + 0.5, z_l = Z[i] * idx - kk + 0.5;
    ii = guard(s, ii + 1); jj = guard(s, jj + 1); kk = guard(s, kk + 1);
    Tg[i] = x_l * y_l * z_l * AT(T, s, ii, jj, kk) +
            (1 - x_l) * y_l * z_l * AT(T, s, ii - 1, jj, kk) + x_l * (1 - y_l) * z_l * AT(T, s, ii, jj - 1, kk) +
            x_l * y_l * (1 - z_l) * AT(T, s, ii, jj, kk - 1) +
            (1 - x_l) * (1 - y_l) * z_l * AT(T, s, ii - 1, jj - 1, kk) +
            (1 - x_l) * y_l * (1 - z_l) * AT(T, s, ii - 1, jj, kk - 1) +
            x_l * (y_l - 1) * (z_l - 1) * AT(T, s, ii, jj - 1, kk - 1) +
            (1 - x_l) * (1 - y_l) * (1 - z_l) * AT(T, s, ii - 1, jj - 1, kk - 1);
  }
}

/* particle.cpp:460-478 */
static void compute_rhs_temp(pso_state *s, int tid) {
  double iTth = s->c.nu * PSO_PI * s->c.dp * s->c.k;
  double *Tg = s->a[PSO_TG], *Tp = s->a[tid], *R = s->a[PSO_RHS_T];
  for (int64_t i = 0; i < s->np; ++i) R[i] = (Tg[i] - Tp[i]) * prop_or(s, PR_ITTH, i, iTth);
}

int pso_set_props(pso_state *s, int64_t n, const double *tau_p, const double *mass_ratio, const double *itth,
                  const double *heat_is, const double *alpha, const double *ax, const double *ay, const double *az) {
  const double *src[8] = {tau_p, mass_ratio, itth, heat_is, alpha, ax, ay, az};
  for (int q = 0; q < 8; ++q) {
    free(s->prop[q]);
    s->prop[q] = 0;
    if (!src[q] || n <= 0) continue;
    s->prop[q] = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(s->prop[q], src[q], sizeof(double) * (size_t)n);
  }
  s->nprop = n;
  return 0;
}

/* particle.cpp:526-559 (weights w) and :586-658 (weights w * RHS_T), trilinear at round() nodes */
static void part2gas_trilinear(pso_state *s, int px, int py, int pz, const double *val, double *A, int do_refresh) {
  double *X = s->a[px], *Y = s->a[py], *Z = s->a[pz];
  const double idx = s->idx;
  zero(s, A);
  for (int64_t i = 0; i < s->np; ++i) {
    int ii = (int)(round(X[i] * idx)), jj = (int)(round(Y[i] * idx)), kk = (int)(round(Z[i] * idx));
    double x_l = X[i] * idx - ii + 0.5, y_l = Y[i] * idx - jj + 0.5, z_l = Z[i] * idx - kk + 0.5;
    ii = guard(s, ii + 1); jj = guard(s, jj + 1); kk = guard(s, kk + 1);
    if (!val) {
      AT(A, s, ii, jj, kk) += (x_l * y_l * z_l);
      AT(A, s, ii - 1, jj, kk) += (1 - x_l) * y_l * z_l;
      AT(A, s, ii, jj - 1, kk) += x_l * (1 - y_l) * z_l;
      AT(A, s, ii, jj, kk - 1) += x_l * y_l * (1 - z_l);
      AT(A, s, ii - 1, jj - 1, kk) += (1 - x_l) * (1 - y_l) * z_l;
      AT(A, s, ii - 1, jj, kk - 1) += (1 - x_l) * y_l * (1 - z_l);
      AT(A, s, ii, jj - 1, kk - 1) += x_l * (1 - y_l) * (1 - z_l);
      AT(A, s, ii - 1, jj - 1, kk - 1) += (1 - x_l) * (1 - y_l) * (1 - z_l);
    } else {
      double r = val[i];
      AT(A, s, ii, jj, kk) += x_l * y_l * z_l * r;
      AT(A, s, ii - 1, jj, kk) += (1 - x_l) * y_l * z_l * r;
      AT(A, s, ii, jj - 1, kk) += x_l * (1 - y_l) * z_l * r;
      AT(A, s, ii, jj, kk - 1) += x_l * y_l * (1 - z_l) * r;
      AT(A, s, ii - 1, jj - 1, kk) += (1 - x_l) * (1 - y_l) * z_l * r;
      AT(A, s, ii - 1, jj, kk - 1) += (1 - x_l) * y_l * (1 - z_l) * r;
      AT(A, s, ii, jj - 1, kk - 1) += x_l * (1 - y_l) * (1 - z_l) * r;
      AT(A, s, ii - 1, jj - 1, kk - 1) += (1 - x_l) * (1 - y_l) * (1 - z_l) * r;
    }
  }
  fold_cum(s, A);
  if (do_refresh) refresh(s, A);
}

int pso_prime(pso_state *s, const double *tfield, double *e) {
  copy_arr(s, PSO_X_INT, PSO_X); copy_arr(s, PSO_Y_INT, PSO_Y); copy_arr(s, PSO_Z_INT, PSO_Z);
  copy_arr(s, PSO_U_INT, PSO_U); copy_arr(s, PSO_V_INT, PSO_V); copy_arr(s, PSO_W_INT, PSO_W);
  copy_arr(s, PSO_T_INT, PSO_T);
  copy_arr(s, PSO_X_NP1, PSO_X); copy_arr(s, PSO_Y_NP1, PSO_Y); copy_arr(s, PSO_Z_NP1, PSO_Z);
  copy_arr(s, PSO_U_NP1, PSO_U); copy_arr(s, PSO_V_NP1, PSO_V); copy_arr(s, PSO_W_NP1, PSO_W);
  copy_arr(s, PSO_T_NP1, PSO_T);
  gas2part_temp(s, PSO_X_INT, PSO_Y_INT, PSO_Z_INT, tfield);
  compute_rhs_temp(s, PSO_T_INT);
  part2gas_trilinear(s, PSO_X_INT, PSO_Y_INT, PSO_Z_INT, s->a[PSO_RHS_T], e, 1);
  return 0;
}

/* particle.cpp:136-311: SWAP and ToBuf act on the 29 transported values only */
static const int rec_ids[28] = {PSO_X, PSO_X_INT, PSO_X_NEW, PSO_X_NP1, PSO_Y, PSO_Y_INT, PSO_Y_NEW, PSO_Y_NP1,
                                PSO_Z, PSO_Z_INT, PSO_Z_NEW, PSO_Z_NP1, PSO_U, PSO_U_INT, PSO_U_NEW, PSO_U_NP1,
                                PSO_V, PSO_V_INT, PSO_V_NEW, PSO_V_NP1, PSO_W, PSO_W_INT, PSO_W_NEW, PSO_W_NP1,
                                PSO_T, PSO_T_INT, PSO_T_NEW, PSO_T_NP1};

static void to_buf(pso_state *s, int64_t i, double *b) {
  for (int q = 0; q < 28; ++q) b[q] = s->a[rec_ids[q]][i];
  b[28] = (double)s->flag[i];
}
static void swap_p(pso_state *s, int64_t i, int64_t j) {
  for (int q = 0; q < 28; ++q) {
    double *v = s->a[rec_ids[q]];
    double t = v[i]; v[i] = v[j]; v[j] = t;
  }
  int32_t t = s->flag[i]; s->flag[i] = s->flag[j]; s->flag[j] = t;
}
static void from_buf(pso_state *s, const double *b, int64_t nrec) {
  for (int64_t r = 0; r < nrec; ++r) {
    const double *q = b + 29 * r;
    int64_t i = s->np++;
    for (int t = 0; t < 28; ++t) s->a[rec_ids[t]][i] = q[t];
    s->flag[i] = (int32_t)q[28];
  }
}

/* MODE_L* (particle.cpp:58-104): shifts base, new and np1 of dimension d */
static void mode_l(pso_state *s, int64_t i, int d) {
  double *base = s->a[PSO_X + d], *nw = s->a[PSO_X_NEW + d], *np1 = s->a[PSO_X_NP1 + d];
  const double L = s->c.l;
  if (nw[i] > L) { nw[i] -= L; base[i] -= L; np1[i] -= L; }
  else if (nw[i] < 0) { nw[i] += L; base[i] += L; np1[i] += L; }
}

/* SortValid{X,Y,Z} + the loopback exchange + FromBuf (particle.cpp:150-311, 745-812):
 * leavers are swap-removed in scan order; the ones that crossed the low side come back
 * first (Rbuf0 <- Sbuf1 by tag), then the ones that crossed the high side. */
static void send_recv_dim(pso_state *s, int d) {
  double *nw = s->a[PSO_X_NEW + d];
  const double lo = 0.0, hi = s->xh;
  int64_t i = 0, s0 = 0, s1 = 0;
  while (i < s->np) {
    if (nw[i] > hi) {
      mode_l(s, i, d);
      to_buf(s, i, s->rec0 + 29 * s0); s0++;
      swap_p(s, i, s->np - 1); s->np--; i--;
    } else if (nw[i] < lo) {
      mode_l(s, i, d);
      to_buf(s, i, s->rec1 + 29 * s1); s1++;
      swap_p(s, i, s->np - 1); s->np--; i--;
    }
    i++;
  }
  /* RESIZE() (particle.cpp:136-148) shrinks to the stayers and, after FromBuf, grows
   * back: the tails of the work vectors it resizes come back as zeros (wg and Tg are
   * only reserved and keep their values) */
  if (s0 + s1 > 0) {
    static const int resized[6] = {PSO_RHS_U, PSO_RHS_V, PSO_RHS_W, PSO_RHS_T, PSO_UG, PSO_VG};
    for (int q = 0; q < 6; ++q)
      for (int64_t t = s->np; t < s->np + s0 + s1; ++t) s->a[resized[q]][t] = 0.0;
  }
  from_buf(s, s->rec1, s1);
  from_buf(s, s->rec0, s0);
}

int pso_stage(pso_state *s, int k, const double *ux, const double *uy, const double *uz, const double *tfield,
              double *c, double *ax, double *ay, double *az, double *e) {
  static const double pre[4] = {0.5, 0.5, 1., 1. / 6.};
  static const double post[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};
  if (k < 0 || k > 3) return -1;
  const double idx = s->idx, dt = s->c.dt, P = pre[k], Q = post[k];
  const int64_t n = s->np;
  double *xi = s->a[PSO_X_INT], *yi = s->a[PSO_Y_INT], *zi = s->a[PSO_Z_INT];
  double *ug = s->a[PSO_UG], *vg = s->a[PSO_VG], *wg = s->a[PSO_WG];

  /* gas2part_velocity :340-360 */
  for (int64_t i = 0; i < n; ++i) {
    int ii = (int)(xi[i] * idx) + 1, jj = (int)(yi[i] * idx) + 1, kk = (int)(zi[i] * idx) + 1;
    double x_l = (xi[i] * idx - ((int)(xi[i] * idx)));
    double y_l = (yi[i] * idx - ((int)(yi[i] * idx)));
    double z_l = (zi[i] * idx - ((int)(zi[i] * idx)));
    ii = guard_face(s, ii); jj = guard_face(s, jj); kk = guard_face(s, kk);
    ug[i] = x_l * AT(ux, s, ii + 1, jj, kk) + (1 - x_l) * AT(ux, s, ii, jj, kk);
    vg[i] = y_l * AT(uy, s, ii, jj + 1, kk) + (1 - y_l) * AT(uy, s, ii, jj, kk);
    wg[i] = z_l * AT(uz, s, ii, jj, kk + 1) + (1 - z_l) * AT(uz, s, ii, jj, kk);
  }
  /* update_position :314-338 */
  for (int d = 0; d < 3; ++d) {
    double *np1 = s->a[PSO_X_NP1 + d], *nw = s->a[PSO_X_NEW + d], *b = s->a[PSO_X + d], *vel = s->a[PSO_U_INT + d];
    for (int64_t i = 0; i < n; ++i) np1[i] += dt * Q * vel[i];
    if (k != 3) for (int64_t i = 0; i < n; ++i) nw[i] = b[i] + dt * P * vel[i];
    else for (int64_t i = 0; i < n; ++i) nw[i] = np1[i];
  }
  /* update_velocity :362-399 */
  {
    double iTp = 0.0;
    if (s->c.tp != 0) iTp = 1. / s->c.tp;
    const double g[3] = {s->c.particle_gravity * s->c.gx, s->c.particle_gravity * s->c.gy,
                         s->c.particle_gravity * s->c.gz};
    double *gas[3] = {ug, vg, wg};
    for (int d = 0; d < 3; ++d) {
      double *rhs = s->a[PSO_RHS_U + d], *vin = s->a[PSO_U_INT + d], *np1 = s->a[PSO_U_NP1 + d],
             *nw = s->a[PSO_U_NEW + d], *b = s->a[PSO_U + d];
      if (!s->prop[PR_TAU] && !s->prop[PR_AX + d]) {
        for (int64_t i = 0; i < n; ++i) rhs[i] = (gas[d][i] - vin[i]) * iTp;
        for (int64_t i = 0; i < n; ++i) np1[i] += dt * Q * (rhs[i] + g[d]);
        if (k != 3) for (int64_t i = 0; i < n; ++i) nw[i] = b[i] + dt * P * (rhs[i] + g[d]);
        else for (int64_t i = 0; i < n; ++i) nw[i] = np1[i];
      } else {
        for (int64_t i = 0; i < n; ++i) {
          const double itp_i = s->prop[PR_TAU] ? 1. / prop_or(s, PR_TAU, i, 0.0) : iTp;
          const double g_i = prop_or(s, PR_AX + d, i, g[d]);
          rhs[i] = (gas[d][i] - vin[i]) * itp_i;
          np1[i] += dt * Q * (rhs[i] + g_i);
          nw[i] = (k != 3) ? b[i] + dt * P * (rhs[i] + g_i) : np1[i];
        }
      }
    }
  }
  /* update_Temp :480-496 */
  {
    double alpha = 0.25 * s->c.epsilonp * PSO_PI * s->c.dp * s->c.dp * s->c.i0;
    double iS = 1. / (s->c.mp * s->c.cvp);
    double *np1 = s->a[PSO_T_NP1], *nw = s->a[PSO_T_NEW], *b = s->a[PSO_T], *R = s->a[PSO_RHS_T];
    if (!s->prop[PR_HEAT_IS] && !s->prop[PR_ALPHA]) {
      for (int64_t i = 0; i < n; ++i) np1[i] += dt * Q * iS * (R[i] + alpha);
      if (k != 3) for (int64_t i = 0; i < n; ++i) nw[i] = b[i] + dt * P * iS * (R[i] + alpha);
      else for (int64_t i = 0; i < n; ++i) nw[i] = np1[i];
    } else {
      for (int64_t i = 0; i < n; ++i) {
        const double is_i = prop_or(s, PR_HEAT_IS, i, iS), a_i = prop_or(s, PR_ALPHA, i, alpha);
        np1[i] += dt * Q * is_i * (R[i] + a_i);
        nw[i] = (k != 3) ? b[i] + dt * P * is_i * (R[i] + a_i) : np1[i];
      }
    }
  }
  /* part2gas_concentration :526-559 (no refresh) */
  part2gas_trilinear(s, PSO_X_INT, PSO_Y_INT, PSO_Z_INT, 0, c, 0);
  /* part2gas_velocity :498-524, or RHS_RU = 0 (grid.cpp:671) */
  zero(s, ax); zero(s, ay); zero(s, az);
  if (s->c.twc) {
    double *ru = s->a[PSO_RHS_U], *rv = s->a[PSO_RHS_V], *rw = s->a[PSO_RHS_W];
    for (int64_t i = 0; i < n; ++i) {
      int ii = (int)(xi[i] * idx) + 1, jj = (int)(yi[i] * idx) + 1, kk = (int)(zi[i] * idx) + 1;
      double x_l = (xi[i] * idx - ((int)(xi[i] * idx)));
      double y_l = (yi[i] * idx - ((int)(yi[i] * idx)));
      double z_l = (zi[i] * idx - ((int)(zi[i] * idx)));
      ii = guard_face(s, ii); jj = guard_face(s, jj); kk = guard_face(s, kk);
      double r0 = ru[i], r1 = rv[i], r2 = rw[i];
      if (s->prop[PR_MASS]) {
        const double m = prop_or(s, PR_MASS, i, 1.0);
        r0 *= m; r1 *= m; r2 *= m;
      }
      AT(ax, s, ii + 1, jj, kk) += x_l * r0;
      AT(ax, s, ii, jj, kk) += (1 - x_l) * r0;
      AT(ay, s, ii, jj + 1, kk) += y_l * r1;
      AT(ay, s, ii, jj, kk) += (1 - y_l) * r1;
      AT(az, s, ii, jj, kk + 1) += z_l * r2;
      AT(az, s, ii, jj, kk) += (1 - z_l) * r2;
    }
    fold_cum(s, ax); fold_cum(s, ay); fold_cum(s, az);
    refresh(s, ax); refresh(s, ay); refresh(s, az);
  }
  /* Send_Recv :853-858: z, then y, then x */
  send_recv_dim(s, 2);
  send_recv_dim(s, 1);
  send_recv_dim(s, 0);
  /* gas2part_Temp_new, Compute_RHS_Temp_new, part2gas_Temp_new :430-456, :470-478, :624-658 */
  gas2part_temp(s, PSO_X_NEW, PSO_Y_NEW, PSO_Z_NEW, tfield);
  compute_rhs_temp(s, PSO_T_NEW);
  part2gas_trilinear(s, PSO_X_NEW, PSO_Y_NEW, PSO_Z_NEW, s->a[PSO_RHS_T], e, 1);
  return 0;
}

void pso_end_stage(pso_state *s) {
  copy_arr(s, PSO_X_INT, PSO_X_NEW); copy_arr(s, PSO_Y_INT, PSO_Y_NEW); copy_arr(s, PSO_Z_INT, PSO_Z_NEW);
  copy_arr(s, PSO_U_INT, PSO_U_NEW); copy_arr(s, PSO_V_INT, PSO_V_NEW); copy_arr(s, PSO_W_INT, PSO_W_NEW);
  copy_arr(s, PSO_T_INT, PSO_T_NEW);
}

void pso_end_step(pso_state *s) {
  copy_arr(s, PSO_X, PSO_X_NP1); copy_arr(s, PSO_Y, PSO_Y_NP1); copy_arr(s, PSO_Z, PSO_Z_NP1);
  copy_arr(s, PSO_U, PSO_U_NP1); copy_arr(s, PSO_V, PSO_V_NP1); copy_arr(s, PSO_W, PSO_W_NP1);
  copy_arr(s, PSO_T, PSO_T_NP1);
}

double pso_mean(const double *f, int32_t n) {
  const int G = n + 2;
  double sum = 0;
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= n; ++j)
      for (int k = 1; k <= n; ++k) sum += f[((size_t)k * G + j) * G + i];
  return sum / (double)((int64_t)n * n * n);
}

int pso_run(pso_state *s, int nsteps, const double *ux, const double *uy, const double *uz, const double *tfield,
            double *c, double *ax, double *ay, double *az, double *e) {
  for (int st = 0; st < nsteps; ++st) {
    for (int k = 0; k < 4; ++k) {
      int rc = pso_stage(s, k, ux, uy, uz, tfield, c, ax, ay, az, e);
      if (rc) return rc;
      pso_end_stage(s);
    }
    pso_end_step(s);
  }
  return 0;
}
