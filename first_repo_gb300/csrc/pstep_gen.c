/*
 * Seeded synthetic inputs for the particle step: gas fields on the periodic
 * staggered mesh and particle clouds. Host C, compiled without FMA
 * contraction and using only +,-,*,/ and sqrt (all correctly rounded in
 * IEEE-754), so the x86 build and the Arm build produce bit-identical inputs.
 * sin/cos/log are evaluated by the series below, not by libm (whose last-bit
 * results differ between platforms).
 *
 * Field layout: interior arrays of N^3 doubles, index (k*N + j)*N + i.
 * Placement follows the reference mesh (particle.cpp:346-355, tensor0.cpp:72-80):
 *   u.x(i,j,k) on the left x-face of cell i:  x = i*dx, y = (j+1/2)dx, z = (k+1/2)dx
 *   u.y on the lower y-face, u.z on the lower z-face, T at cell centres.
 *
 * Velocity: random-phase solenoidal Fourier modes, integer wavevectors with
 * round(|k|) in 1..8 (units of 2*pi/L), shell energy E(k) ~ k^(-5/3) split
 * evenly over the shell's modes, scaled analytically to u_rms = 1 per component.
 * Temperature: T = 1 + 0.05 * boxfilter3(N(0,1)) (periodic 3x3x3 mean).
 * Particles: uniform in [0,L)^3, or half uniform and half from Gaussian blobs
 * (seeded centres, sigma in cells), wrapped periodically into [0,L).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define GEN_TWO_PI 6.283185307179586
#define GEN_PI_4 0.7853981633974483
#define GEN_LN2 0.6931471805599453

/* ---------------- deterministic RNG ---------------- */
static uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static uint64_t rng_u64(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed ^ mix64(stream * 0x632BE59BD9B4E019ull)) + i);
}
/* uniform in [0,1) with 53 random bits */
static double rng_u01(uint64_t seed, uint64_t stream, uint64_t i) {
  return (double)(rng_u64(seed, stream, i) >> 11) * (1.0 / 9007199254740992.0);
}

/* ---------------- deterministic elementary functions ---------------- */
/* sin and cos of r in [0, pi/4] by Taylor series (|error| < 1e-17) */
static void sincos_small(double r, double *s, double *c) {
  double r2 = r * r;
  double ts = r, tc = 1.0, ss = r, cc = 1.0;
  for (int n = 1; n <= 12; ++n) {
    ts = -ts * r2 / (double)((2 * n) * (2 * n + 1));
    tc = -tc * r2 / (double)((2 * n - 1) * (2 * n));
    ss += ts;
    cc += tc;
  }
  *s = ss;
  *c = cc;
}
/* sin/cos of theta >= 0 via octant reduction */
static void det_sincos(double theta, double *s, double *c) {
  double q = floor(theta / GEN_PI_4);
  double r = theta - q * GEN_PI_4;
  long oct = ((long)q) & 7;
  if (r < 0) r = 0;
  double a, b;
  /* within an octant, map to [0, pi/4] */
  if (oct & 1) sincos_small(GEN_PI_4 - r, &a, &b); else sincos_small(r, &a, &b);
  /* a = sin(rr), b = cos(rr) for the reduced angle; rebuild by octant */
  double sv, cv;
  switch (oct) {
    case 0: sv = a; cv = b; break;
    case 1: sv = b; cv = a; break;
    case 2: sv = b; cv = -a; break;
    case 3: sv = a; cv = -b; break;
    case 4: sv = -a; cv = -b; break;
    case 5: sv = -b; cv = -a; break;
    case 6: sv = -b; cv = a; break;
    default: sv = -a; cv = b; break;
  }
  *s = sv;
  *c = cv;
}
/* natural log of x > 0 via frexp (exact) and the atanh series */
static double det_log(double x) {
  int e;
  double m = frexp(x, &e); /* x = m * 2^e, m in [0.5,1) */
  if (m < 0.7071067811865476) { m *= 2.0; e -= 1; }
  double s = (m - 1.0) / (m + 1.0), s2 = s * s, t = s, acc = s;
  for (int n = 1; n <= 14; ++n) {
    t *= s2;
    acc += t / (double)(2 * n + 1);
  }
  return (double)e * GEN_LN2 + 2.0 * acc;
}
/* standard normal by Box-Muller from two uniforms */
static double det_normal(uint64_t seed, uint64_t stream, uint64_t i) {
  double u1 = rng_u01(seed, stream, 2 * i);
  double u2 = rng_u01(seed, stream, 2 * i + 1);
  if (u1 < 1e-300) u1 = 1e-300;
  double r = sqrt(-2.0 * det_log(u1));
  double s, c;
  det_sincos(GEN_TWO_PI * u2, &s, &c);
  return r * c;
}

double pstep_gen_log(double x) { return det_log(x); }
void pstep_gen_sincos(double t, double *s, double *c) { det_sincos(t, s, c); }
double pstep_gen_normal(uint64_t seed, uint64_t stream, uint64_t i) { return det_normal(seed, stream, i); }

/* ---------------- velocity field ---------------- */
typedef struct { int kx, ky, kz; double ar[3], ai[3]; } gen_mode;

static int build_modes(uint64_t seed, int kmax, gen_mode **out) {
  int cap = (2 * kmax + 1) * (2 * kmax + 1) * (2 * kmax + 1);
  gen_mode *m = (gen_mode *)calloc((size_t)cap, sizeof(gen_mode));
  int count[64] = {0};
  int n = 0;
  for (int pass = 0; pass < 2; ++pass) {
    n = 0;
    for (int kx = 0; kx <= kmax; ++kx)
      for (int ky = -kmax; ky <= kmax; ++ky)
        for (int kz = -kmax; kz <= kmax; ++kz) {
          /* one of each +-k pair */
          if (kx == 0 && (ky < 0 || (ky == 0 && kz <= 0))) continue;
          double k2 = (double)(kx * kx + ky * ky + kz * kz);
          double kk = sqrt(k2);
          int shell = (int)floor(kk + 0.5);
          if (shell < 1 || shell > kmax) continue;
          if (pass == 0) { count[shell]++; continue; }
          gen_mode *g = &m[n];
          g->kx = kx; g->ky = ky; g->kz = kz;
          /* random direction perpendicular to k */
          double rx = det_normal(seed, 11, 3 * (uint64_t)n), ry = det_normal(seed, 11, 3 * (uint64_t)n + 1),
                 rz = det_normal(seed, 11, 3 * (uint64_t)n + 2);
          double dot = (rx * kx + ry * ky + rz * kz) / k2;
          rx -= dot * kx; ry -= dot * ky; rz -= dot * kz;
          double rn = sqrt(rx * rx + ry * ry + rz * rz);
          if (rn < 1e-12) { rx = 1; ry = 0; rz = 0; rn = 1; }
          /* energy per mode: E(shell)/count with E ~ shell^(-5/3); amplitude a with <u.u> = a^2/2 */
          double e53 = 1.0;
          { /* shell^(-5/3) with det functions */
            double l = det_log((double)shell) * (-5.0 / 3.0);
            /* exp by squaring of e^(l/64) series */
            double y = l / 64.0, t = 1.0, acc = 1.0;
            for (int q = 1; q <= 16; ++q) { t *= y / (double)q; acc += t; }
            for (int q = 0; q < 6; ++q) acc *= acc;
            e53 = acc;
          }
          double amp = sqrt(2.0 * e53 / (double)count[shell]);
          double s, c;
          det_sincos(GEN_TWO_PI * rng_u01(seed, 12, (uint64_t)n), &s, &c);
          g->ar[0] = amp * c * rx / rn; g->ai[0] = amp * s * rx / rn;
          g->ar[1] = amp * c * ry / rn; g->ai[1] = amp * s * ry / rn;
          g->ar[2] = amp * c * rz / rn; g->ai[2] = amp * s * rz / rn;
          n++;
        }
  }
  /* analytic normalisation: sum of a^2/2 over modes = 3 (u_rms = 1 per component) */
  double e = 0;
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) e += 0.5 * (m[i].ar[d] * m[i].ar[d] + m[i].ai[d] * m[i].ai[d]);
  double sc = sqrt(3.0 / e);
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) { m[i].ar[d] *= sc; m[i].ai[d] *= sc; }
  *out = m;
  return n;
}

/*
 * Evaluate component d of sum_k Re[a_k exp(i 2pi k.p / N)] at staggered
 * positions p = (i + sx/2, j + sy/2, k + sz/2) (s* in {0,1}), in three
 * separable passes over a table of exp(i 2pi m/(2N)).
 */
static void eval_component(const gen_mode *m, int nm, int kmax, int N, int d, int sx, int sy, int sz, double *dst) {
  const int M = 2 * N;
  double *cs = (double *)malloc(sizeof(double) * M), *sn = (double *)malloc(sizeof(double) * M);
  for (int q = 0; q < M; ++q) det_sincos(GEN_TWO_PI * (double)q / (double)M, &sn[q], &cs[q]);
  const int KX = kmax + 1, KY = 2 * kmax + 1;
  /* g[kx][ky][z] = sum_kz a * e(kz pz) */
  double *gr = (double *)calloc((size_t)KX * KY * N, sizeof(double));
  double *gi = (double *)calloc((size_t)KX * KY * N, sizeof(double));
  for (int t = 0; t < nm; ++t) {
    int ix = m[t].kx, iy = m[t].ky + kmax;
    for (int z = 0; z < N; ++z) {
      long ph = ((long)m[t].kz * (2 * z + sz)) % M;
      if (ph < 0) ph += M;
      double c = cs[ph], s = sn[ph];
      size_t o = ((size_t)ix * KY + iy) * N + z;
      gr[o] += m[t].ar[d] * c - m[t].ai[d] * s;
      gi[o] += m[t].ar[d] * s + m[t].ai[d] * c;
    }
  }
  /* h[kx][y][z] = sum_ky g * e(ky py) */
  double *hr = (double *)calloc((size_t)KX * N * N, sizeof(double));
  double *hi = (double *)calloc((size_t)KX * N * N, sizeof(double));
#pragma omp parallel for schedule(static)
  for (int kx = 0; kx < KX; ++kx)
    for (int ky = 0; ky < KY; ++ky)
      for (int y = 0; y < N; ++y) {
        long ph = ((long)(ky - kmax) * (2 * y + sy)) % M;
        if (ph < 0) ph += M;
        double c = cs[ph], s = sn[ph];
        const double *ar = gr + ((size_t)kx * KY + ky) * N, *ai = gi + ((size_t)kx * KY + ky) * N;
        double *or_ = hr + ((size_t)kx * N + y) * N, *oi = hi + ((size_t)kx * N + y) * N;
        for (int z = 0; z < N; ++z) {
          or_[z] += ar[z] * c - ai[z] * s;
          oi[z] += ar[z] * s + ai[z] * c;
        }
      }
  /* f[z][y][x] = Re sum_kx h * e(kx px) */
#pragma omp parallel for schedule(static)
  for (int z = 0; z < N; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        double acc = 0;
        for (int kx = 0; kx < KX; ++kx) {
          long ph = ((long)kx * (2 * x + sx)) % M;
          double c = cs[ph], s = sn[ph];
          size_t o = ((size_t)kx * N + y) * N + z;
          acc += hr[o] * c - hi[o] * s;
        }
        dst[((size_t)z * N + y) * N + x] = acc;
      }
  free(cs); free(sn); free(gr); free(gi); free(hr); free(hi);
}

/* velocity on faces (interior arrays), u_rms = 1; returns the number of modes */
int pstep_gen_velocity(int N, uint64_t seed, double *ux, double *uy, double *uz) {
  if (N < 2) return -1;
  const int kmax = 8;
  gen_mode *m = 0;
  int nm = build_modes(seed, kmax, &m);
  eval_component(m, nm, kmax, N, 0, 0, 1, 1, ux);
  eval_component(m, nm, kmax, N, 1, 1, 0, 1, uy);
  eval_component(m, nm, kmax, N, 2, 1, 1, 0, uz);
  free(m);
  return nm;
}

/* T = 1 + amp * periodic 3x3x3 box mean of N(0,1) noise (interior array) */
int pstep_gen_temperature(int N, uint64_t seed, double amp, double *T) {
  if (N < 1) return -1;
  size_t N3 = (size_t)N * N * N;
  double *w = (double *)malloc(sizeof(double) * N3);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)N3; ++c) w[c] = det_normal(seed, 21, (uint64_t)c);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        double acc = 0;
        for (int dk = -1; dk <= 1; ++dk)
          for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
              int kk = (k + dk + N) % N, jj = (j + dj + N) % N, ii = (i + di + N) % N;
              acc += w[((size_t)kk * N + jj) * N + ii];
            }
        T[((size_t)k * N + j) * N + i] = 1.0 + amp * (acc / 27.0);
      }
  free(w);
  return 0;
}

static double wrap01(double x, double L) {
  while (x < 0) x += L;
  while (x >= L) x -= L;
  return x;
}

/*
 * Particle positions. clustered == 0: uniform. clustered == 1: particles with
 * index < n/2 uniform, the rest from nblobs Gaussian blobs (std sigma_cells*L/N).
 */
int pstep_gen_positions(int N, double L, uint64_t seed, int64_t n, int clustered, int nblobs, double sigma_cells,
                        double *x, double *y, double *z) {
  if (n < 0 || N < 1) return -1;
  double sig = sigma_cells * L / (double)N;
  int64_t nu = clustered ? n / 2 : n;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    if (p < nu) {
      x[p] = wrap01(L * rng_u01(seed, 31, 3 * (uint64_t)p), L);
      y[p] = wrap01(L * rng_u01(seed, 31, 3 * (uint64_t)p + 1), L);
      z[p] = wrap01(L * rng_u01(seed, 31, 3 * (uint64_t)p + 2), L);
    } else {
      uint64_t b = rng_u64(seed, 32, (uint64_t)p) % (uint64_t)(nblobs > 0 ? nblobs : 1);
      double cx = L * rng_u01(seed, 33, 3 * b), cy = L * rng_u01(seed, 33, 3 * b + 1), cz = L * rng_u01(seed, 33, 3 * b + 2);
      x[p] = wrap01(cx + sig * det_normal(seed, 34, 3 * (uint64_t)p), L);
      y[p] = wrap01(cy + sig * det_normal(seed, 34, 3 * (uint64_t)p + 1), L);
      z[p] = wrap01(cz + sig * det_normal(seed, 34, 3 * (uint64_t)p + 2), L);
    }
  }
  return 0;
}

/*
 * Gas velocity at particle positions by the reference's face-normal linear
 * interpolation (particle.cpp:340-360), periodic, from interior face arrays.
 */
int pstep_gen_interp_velocity(int N, double L, int64_t n, const double *x, const double *y, const double *z,
                              const double *ux, const double *uy, const double *uz, double *u, double *v, double *w) {
  double idx = 1. / (L / (double)N);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    double px = x[p] * idx, py = y[p] * idx, pz = z[p] * idx;
    int i = (int)px, j = (int)py, k = (int)pz;
    double xl = px - i, yl = py - j, zl = pz - k;
    int i0 = i % N, j0 = j % N, k0 = k % N;
    int i1 = (i + 1) % N, j1 = (j + 1) % N, k1 = (k + 1) % N;
    u[p] = xl * ux[((size_t)k0 * N + j0) * N + i1] + (1 - xl) * ux[((size_t)k0 * N + j0) * N + i0];
    v[p] = yl * uy[((size_t)k0 * N + j1) * N + i0] + (1 - yl) * uy[((size_t)k0 * N + j0) * N + i0];
    w[p] = zl * uz[((size_t)k1 * N + j0) * N + i0] + (1 - zl) * uz[((size_t)k0 * N + j0) * N + i0];
  }
  return 0;
}

/* interior N^3 -> ghosted (N+2)^3 with periodic ghosts (what the reference's Update_Ghosts leaves) */
int pstep_gen_ghost(int N, const double *src, double *dst) {
  const int G = N + 2;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < G; ++k)
    for (int j = 0; j < G; ++j)
      for (int i = 0; i < G; ++i) {
        int kk = (k - 1 + N) % N, jj = (j - 1 + N) % N, ii = (i - 1 + N) % N;
        dst[((size_t)k * G + j) * G + i] = src[((size_t)kk * N + jj) * N + ii];
      }
  return 0;
}

/* uniform random doubles in [lo, hi) (per-particle parameters such as tau_p ranges) */
int pstep_gen_uniform(uint64_t seed, uint64_t stream, int64_t n, double lo, double hi, double *out) {
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) out[p] = lo + (hi - lo) * rng_u01(seed, stream, (uint64_t)p);
  return 0;
}

/* log-uniform doubles in [lo, hi) */
int pstep_gen_loguniform(uint64_t seed, uint64_t stream, int64_t n, double lo, double hi, double *out) {
  double a = det_log(lo), b = det_log(hi);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    double l = a + (b - a) * rng_u01(seed, stream, (uint64_t)p);
    /* exp(l) = 2^(l/ln2): integer part by ldexp, fraction by series */
    double t = l / GEN_LN2;
    double fi = floor(t);
    double f = (t - fi) * GEN_LN2, term = 1.0, acc = 1.0;
    for (int q = 1; q <= 20; ++q) { term *= f / (double)q; acc += term; }
    out[p] = ldexp(acc, (int)fi);
  }
  return 0;
}
