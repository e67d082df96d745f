// FP64 drop-in particle kernels: gas->particle interpolation, RK4 stage advance,
// periodic wrap, temperature interpolation and heat-transfer RHS.
//
// Compiled with -fmad=false: every expression is evaluated as the separate IEEE
// operations the reference writes, in its operand order, so particle states are
// bit-identical to the reference's particle.cpp (built without FMA contraction).
//
// Positions are absolute FP64 (as in the reference). For each position the
// kernels derive, exactly as the reference does:
//   trunc cell  t = (int)(x*idx)              particle.cpp:106-119, 346-352
//   round node  r = (int)round(x*idx)         particle.cpp:121-134, 409-415
//   fraction    f = x*idx - t  (exact: x*idx and t are within one unit)
// and store (f, node key) as the position's deposit record: x_l of the
// face-normal interpolation is f, x_l of the trilinear one is
// (x*idx - r) + 0.5 = (h ? (f - 1) : f) + 0.5 with h = r - t, both exact
// reconstructions of the reference's values.
#include "pstep_internal.cuh"

namespace pstep {
namespace {

struct PosRec {
  int node[3];     // ghosted node index r+1 per dimension
  int h[3];        // r - t
  double frac[3];  // x*idx - t
  bool bad;        // index clamped (x outside [0, L] or at the x == L edge)
  bool nonfinite;
};

__device__ inline void position_record(const Geom &G, const double x[3], PosRec &r) {
  r.bad = false;
  r.nonfinite = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double xi = x[d] * G.idx[d];
    if (!isfinite(xi)) {
      r.nonfinite = true;
      xi = 0.0;
    }
    int t = __double2int_rz(xi);
    int rn = __double2int_rz(round(xi));
    double f = xi - (double)t;
    int h = rn - t;
    // the trilinear stencil is in bounds for round nodes 0..n; a position at x == L
    // (t == n) is legal here but makes the next stage's face-normal gather read
    // past the ghost layer in the reference (checked where that gather happens)
    if (xi < 0.0 || t < 0 || rn > G.n[d]) {
      r.bad = true;
      t = t < 0 ? 0 : G.n[d] - 1;
      rn = t;
      h = 0;
      f = 0.0;
    }
    r.node[d] = rn + 1;
    r.h[d] = h;
    r.frac[d] = f;
  }
}

__device__ inline uint32_t node_key(const Geom &G, const PosRec &r) {
  long long lin = glin(G, r.node[0], r.node[1], r.node[2]);
  return ((uint32_t)lin << 3) | (uint32_t)(r.h[0] << 2 | r.h[1] << 1 | r.h[2]);
}

// particle.cpp:430-456: trilinear T at the round() node, the reference's term order
__device__ inline double gather_t(const Geom &G, const double *__restrict__ T, const PosRec &r) {
  const double x_l = (r.h[0] ? (r.frac[0] - 1.0) : r.frac[0]) + 0.5;
  const double y_l = (r.h[1] ? (r.frac[1] - 1.0) : r.frac[1]) + 0.5;
  const double z_l = (r.h[2] ? (r.frac[2] - 1.0) : r.frac[2]) + 0.5;
  const int ii = r.node[0], jj = r.node[1], kk = r.node[2];
  return x_l * y_l * z_l * T[glin(G, ii, jj, kk)] +
         (1 - x_l) * y_l * z_l * T[glin(G, ii - 1, jj, kk)] + x_l * (1 - y_l) * z_l * T[glin(G, ii, jj - 1, kk)] +
         x_l * y_l * (1 - z_l) * T[glin(G, ii, jj, kk - 1)] +
         (1 - x_l) * (1 - y_l) * z_l * T[glin(G, ii - 1, jj - 1, kk)] +
         (1 - x_l) * y_l * (1 - z_l) * T[glin(G, ii - 1, jj, kk - 1)] +
         x_l * (y_l - 1) * (z_l - 1) * T[glin(G, ii, jj - 1, kk - 1)] +
         (1 - x_l) * (1 - y_l) * (1 - z_l) * T[glin(G, ii - 1, jj - 1, kk - 1)];
}

// grid.cpp:223-226 at the base positions (x_int = x after Initialize)
__global__ void k_prime(Geom G, F64State s, const double *__restrict__ T, double itth, int64_t n,
                        int32_t *__restrict__ err) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3] = {s.base[0][i], s.base[1][i], s.base[2][i]};
  PosRec r;
  position_record(G, x, r);
  if (r.bad || r.nonfinite) atomicOr(err, r.nonfinite ? kErrNonFinite : kErrRange);
  double tg = gather_t(G, T, r);
  double tp = s.base[6][i];
  s.rhs_t[i] = (tg - tp) * itth;  // particle.cpp:460-468
#pragma unroll
  for (int d = 0; d < 3; ++d) s.frac_new[d][i] = r.frac[d];
  s.key_new[i] = node_key(G, r);
}

// order-preserving 64-bit key of a double (larger double, larger key; 0 is below every key)
__device__ __forceinline__ unsigned long long order_key64(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | (1ull << 63));
}

// warp maximum of 64-bit keys over the warp's active lanes (two 32-bit reductions)
__device__ __forceinline__ unsigned long long warp_max_key(unsigned mask, unsigned long long k) {
  const unsigned hi = (unsigned)(k >> 32);
  const unsigned mh = __reduce_max_sync(mask, hi);
  const unsigned ml = __reduce_max_sync(mask, hi == mh ? (unsigned)k : 0u);
  return ((unsigned long long)mh << 32) | ml;
}

// One RK4 stage for every particle (particle.cpp:314-399, 480-496, 58-104, 430-478).
// Reads the stage's x_int record (fraction + key, computed when x_int was made).
template <int K>
__global__ void __launch_bounds__(kThreads) k_advance(Geom G, F64State s, StageConst c, const double *__restrict__ Ux,
                                                      const double *__restrict__ Uy, const double *__restrict__ Uz,
                                                      const double *__restrict__ T, int twc, int64_t n,
                                                      uint8_t *__restrict__ leave, int32_t *__restrict__ err,
                                                      unsigned long long *__restrict__ pmax) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // stage inputs: at k = 0 the *_int and *_np1 values equal the base state
  double b[7], vin[7], acc[7];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    b[q] = s.base[q][i];
    vin[q] = (K == 0) ? b[q] : s.sint[q][i];
    acc[q] = (K == 0) ? b[q] : s.np1[q][i];
  }
  const double rhs_t_old = s.rhs_t[i];
  const double itp = s.itp ? s.itp[i] : c.itp;

  // gas2part_velocity (particle.cpp:340-360) from the x_int record
  const uint32_t key = s.key_prev[i];
  const long long lin = key >> 3;
  const int hx = (key >> 2) & 1, hy = (key >> 1) & 1, hz = key & 1;
  const int nx = (int)(lin % G.g[0]);
  const int ny = (int)((lin / G.g[0]) % G.g[1]);
  const int nz = (int)(lin / ((long long)G.g[0] * G.g[1]));
  int ii = nx - hx, jj = ny - hy, kk = nz - hz;  // trunc cell + 1 (ghosted)
  bool bad = false;
  if (ii > G.n[0]) { ii = G.n[0]; bad = true; }
  if (jj > G.n[1]) { jj = G.n[1]; bad = true; }
  if (kk > G.n[2]) { kk = G.n[2]; bad = true; }
  const double x_l = s.frac_prev[0][i], y_l = s.frac_prev[1][i], z_l = s.frac_prev[2][i];
  const double ug = x_l * Ux[glin(G, ii + 1, jj, kk)] + (1 - x_l) * Ux[glin(G, ii, jj, kk)];
  const double vg = y_l * Uy[glin(G, ii, jj + 1, kk)] + (1 - y_l) * Uy[glin(G, ii, jj, kk)];
  const double wg = z_l * Uz[glin(G, ii, jj, kk + 1)] + (1 - z_l) * Uz[glin(G, ii, jj, kk)];

  // at k = 0, *_int aliases the base state, which the wrap below may shift: keep the
  // unshifted positions as *_int (the reference's MODE_L* leaves x_int alone)
  if (K == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) s.sint[d][i] = b[d];
  }
  double nw[7];
  // update_position (particle.cpp:314-338)
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    acc[d] += c.dt_post * vin[3 + d];
    nw[d] = (K != 3) ? b[d] + c.dt_pre * vin[3 + d] : acc[d];
  }
  // update_velocity (particle.cpp:362-399)
  const double g[3] = {c.gx, c.gy, c.gz};
  const double gas[3] = {ug, vg, wg};
  double rhs[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rhs[d] = (gas[d] - vin[3 + d]) * itp;
    acc[3 + d] += c.dt_post * (rhs[d] + g[d]);
    nw[3 + d] = (K != 3) ? b[3 + d] + c.dt_pre * (rhs[d] + g[d]) : acc[3 + d];
  }
  // update_Temp (particle.cpp:480-496); RHS_T is the previous stage's
  acc[6] += c.dt_post_is * (rhs_t_old + c.alpha);
  nw[6] = (K != 3) ? b[6] + c.dt_pre_is * (rhs_t_old + c.alpha) : acc[6];

  // Send_Recv on one rank: MODE_Lz, MODE_Ly, MODE_Lx (particle.cpp:58-104) with the
  // leave test of SortValid* (x_new > xh or x_new < xl = 0, particle.cpp:150-250)
  uint8_t code = 0;
  bool wrapped[3] = {false, false, false};
#pragma unroll
  for (int d = 2; d >= 0; --d) {
    // only particles that leave the slab pass through MODE_L*
    const double xv = nw[d];
    if (xv > G.xh[d]) {
      code |= (uint8_t)(1 << (2 * d));
      if (xv > G.l[d]) { nw[d] -= G.l[d]; b[d] -= G.l[d]; acc[d] -= G.l[d]; wrapped[d] = true; }
    } else if (xv < 0.0) {
      code |= (uint8_t)(2 << (2 * d));
      nw[d] += G.l[d]; b[d] += G.l[d]; acc[d] += G.l[d]; wrapped[d] = true;
    }
  }
  if (leave) leave[i] = code;

  // gas2part_Temp_new + Compute_RHS_Temp_new (particle.cpp:430-456, 470-478)
  PosRec r;
  position_record(G, nw, r);
  const double tg = gather_t(G, T, r);
  const double rhs_t_new = (tg - nw[6]) * c.itth;

  bool nonfinite = r.nonfinite;
#pragma unroll
  for (int q = 3; q < 7; ++q) nonfinite |= !isfinite(nw[q]);
  if (bad || r.bad || nonfinite) atomicOr(err, nonfinite ? kErrNonFinite : kErrRange);

  // stores
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    s.snew[q][i] = nw[q];
    s.np1[q][i] = acc[q];
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (wrapped[d]) s.base[d][i] = b[d];
    s.frac_new[d][i] = r.frac[d];
  }
  if (twc) {
#pragma unroll
    for (int d = 0; d < 3; ++d) s.rhs_u[d][i] = rhs[d];
  }
  s.rhs_t[i] = rhs_t_new;
  s.key_new[i] = node_key(G, r);
  // the last stage: max u of the step's result and max ug (grid.cpp:726-727), per warp
  // into one of 1024 slot pairs
  if (K == 3 && pmax) {
    const unsigned mask = __activemask();
    const unsigned long long ku = warp_max_key(mask, order_key64(acc[3])), kg = warp_max_key(mask, order_key64(ug));
    if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) {
      const int slot = (int)((((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) % 1024);
      atomicMax(&pmax[2 * slot], ku);
      atomicMax(&pmax[2 * slot + 1], kg);
    }
  }
}

// gas2part_Temp_new + Compute_RHS_Temp_new from the x_new record, for a temperature
// field bound after the advance kernel ran
__global__ void k_temp_gather(Geom G, F64State s, const double *__restrict__ T, double itth, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t key = s.key_new[i];
  const long long lin = key >> 3;
  PosRec r;
  r.node[0] = (int)(lin % G.g[0]);
  r.node[1] = (int)((lin / G.g[0]) % G.g[1]);
  r.node[2] = (int)(lin / ((long long)G.g[0] * G.g[1]));
  r.h[0] = (key >> 2) & 1;
  r.h[1] = (key >> 1) & 1;
  r.h[2] = key & 1;
#pragma unroll
  for (int d = 0; d < 3; ++d) r.frac[d] = s.frac_new[d][i];
  const double tg = gather_t(G, T, r);
  s.rhs_t[i] = (tg - s.snew[6][i]) * itth;
}

}  // namespace

StageConst make_stage_const(const pstep_config &cfg, int k, double pre, double post) {
  StageConst c;
  c.k = k;
  const double dt = cfg.dt;
  const double iS = 1. / (cfg.mp * cfg.cvp);                         // particle.cpp:486
  c.dt_pre = dt * pre;                                                // dt*RK4_pre*...
  c.dt_post = dt * post;
  c.dt_pre_is = dt * pre * iS;
  c.dt_post_is = dt * post * iS;
  c.itp = 0.0;
  if (cfg.tp != 0) c.itp = 1. / cfg.tp;                               // particle.cpp:365-366
  c.gx = cfg.particle_gravity * cfg.gx;                               // particle.cpp:376-378
  c.gy = cfg.particle_gravity * cfg.gy;
  c.gz = cfg.particle_gravity * cfg.gz;
  c.alpha = 0.25 * cfg.epsilonp * kPi * cfg.dp * cfg.dp * cfg.i0;     // particle.cpp:484
  c.itth = cfg.nu * kPi * cfg.dp * cfg.k;                             // particle.cpp:462, 473
  return c;
}

int f64_prime_kernel(pstep_ctx *h) {
  if (h->np == 0) return PSTEP_OK;
  StageConst c = make_stage_const(h->cfg, 0, 0.5, 1. / 6.);
  const int blocks = (int)((h->np + kThreads - 1) / kThreads);
  k_prime<<<blocks, kThreads, 0, h->stream>>>(h->geom, h->s, h->tf, c.itth, h->np, h->err_word);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

int f64_advance(pstep_ctx *h, int k, double pre, double post) {
  if (h->np == 0) return PSTEP_OK;
  StageConst c = make_stage_const(h->cfg, k, pre, post);
  const int blocks = (int)((h->np + kThreads - 1) / kThreads);
  uint8_t *leave = (h->cfg.flags & PSTEP_TRACK_ORDER) ? h->leave_code : nullptr;
  const int twc = h->cfg.twc;
#define PSTEP_ADV(KK)                                                                                   \
  k_advance<KK><<<blocks, kThreads, 0, h->stream>>>(h->geom, h->s, c, h->ux, h->uy, h->uz, h->tf, twc, \
                                                    h->np, leave, h->err_word, h->pmax64)
  switch (k) {
    case 0: PSTEP_ADV(0); break;
    case 1: PSTEP_ADV(1); break;
    case 2: PSTEP_ADV(2); break;
    default: PSTEP_ADV(3); break;
  }
#undef PSTEP_ADV
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}

}  // namespace pstep

namespace pstep {
// particle::max of u or ug (grid.cpp:726-727) as the FP64 form's last stage gathered
// them, when they describe the current base state: PSTEP_OK with *out set, or -1
int f64_fused_max(pstep_ctx *h, int id, double *out) {
  if (h->pmax64_state != 2 || !h->pmax64 || (id != PSTEP_U && id != PSTEP_UG)) return -1;
  unsigned long long keys[2 * 1024];
  PSTEP_CUDA(cudaMemcpyAsync(keys, h->pmax64, sizeof keys, cudaMemcpyDeviceToHost, h->stream));
  PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  const int q = id == PSTEP_U ? 0 : 1;
  unsigned long long best = 0;
  for (int s = 0; s < 1024; ++s) best = keys[2 * s + q] > best ? keys[2 * s + q] : best;
  if (best == 0) return -1;
  const unsigned long long bits = (best >> 63) ? (best & ~(1ull << 63)) : ~best;
  memcpy(out, &bits, sizeof bits);
  return PSTEP_OK;
}

int f64_temp_gather(pstep_ctx *h) {
  if (h->np == 0) return PSTEP_OK;
  StageConst c = make_stage_const(h->cfg, 0, 0.5, 1. / 6.);
  const int blocks = (int)((h->np + kThreads - 1) / kThreads);
  k_temp_gather<<<blocks, kThreads, 0, h->stream>>>(h->geom, h->s, h->tf, c.itth, h->np);
  PSTEP_LAUNCHED(h);
  return PSTEP_OK;
}
}  // namespace pstep
