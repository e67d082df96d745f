/*
 * CPU restatement of the reference's box gas step (grid.cpp, low-Mach
 * variable-density projection on the staggered periodic mesh), FP64, single
 * rank, coupled to the particle-step restatement (pstep_oracle.h).
 * TEST INFRASTRUCTURE: the checker of the GPU gas step; the product never links it.
 *
 * Pinning: tests compare it bit for bit with the reference's own grid.cpp
 * compiled with the single-rank MPI stub and a Poisson stub (oracle/poisson_stub)
 * that restates poisson.cpp's iterative FFT solve on gas_fft3d below (the
 * Sandia FFT and HYPRE libraries the reference links are not vendored).
 */
#ifndef PSTEP_GAS_ORACLE_H
#define PSTEP_GAS_ORACLE_H
#include <stdint.h>
#include "pstep_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* params.h values the box gas step reads (params.cpp:22-56) */
typedef struct {
  int32_t n;           /* cells per side */
  int32_t cooling;     /* Is_Cooling (grid.cpp:544, 561) */
  int32_t iterations;  /* Iteration(): Poisson iterations (poisson.cpp:396) */
  int32_t twc;         /* TWC */
  double l;            /* box side */
  double dt, mu0, k, cp, cv, rho0, u0, a_force, gx, gy, gz, mp, epsilon;
} pgo_config;

typedef struct pgo_state pgo_state;

/* field ids for pgo_field (ghosted (n+2)^3 arrays) */
enum {
  PGO_RU_X, PGO_RU_Y, PGO_RU_Z, PGO_RHO, PGO_P, PGO_T, PGO_U_X, PGO_U_Y, PGO_U_Z, PGO_C,
  PGO_RHS_RU_X, PGO_RHS_RU_Y, PGO_RHS_RU_Z, PGO_RHS_PART_TEMP, PGO_DIVERGENCE, PGO_RHO_NEW,
  PGO_NFIELDS_OUT
};
/* scalar ids for pgo_scalar */
enum { PGO_P0, PGO_P0_NEW, PGO_MEAN_E, PGO_LAST_ITERATIONS };

/* the particles may be NULL (gas only); the state keeps the pointer */
pgo_state *pgo_create(const pgo_config *cfg, pso_state *particles);
void pgo_destroy(pgo_state *g);
/* grid::Initialize (grid.cpp:194-226) with the given interior fields (n^3, i fastest):
 * RU, Rho, P = 0, P0; *_int = *_np1 copies, Rho_face, the particle prime */
int pgo_init(pgo_state *g, const double *ru_x, const double *ru_y, const double *ru_z, const double *rho, double p0);
/* one time step (simulation.cpp:38-66, box part): 4 RK4 stages of
 * Update_Rho, Update_P0, Update_Particle, Update_RU_WOP, Compute_Div_U_new,
 * Compute_RHS_Pois, Solve_Poisson, Update_RU_WP, TimeAdvance_RK4; then
 * Correct_mean_RU and TimeAdvance */
int pgo_step(pgo_state *g);
double *pgo_field(pgo_state *g, int id);
double pgo_scalar(const pgo_state *g, int id);

/* In-place complex 3D DFT of an n^3 array (i fastest) of interleaved
 * (re, im) doubles, n a power of two; sign -1 forward, +1 backward; no
 * scaling. Iterative radix-2, twiddles from gas_twiddles. */
void gas_fft3d(double *data, int n, int sign);
/* twiddles w[m] = (cos(2 pi m / n), sign * sin(2 pi m / n)), m < n/2 (libm) */
void gas_twiddles(double *w, int n, int sign);
/* the modified-wavenumber denominators of poisson.cpp:428-448 per axis:
 * out[i] = (2/(d*d)) * (1 - cos(kk*d)), kk = ((i < n/2) ? i : i - n) * 2 pi / L */
void gas_mod_wavenumber(double *out, int n, double l);

#ifdef __cplusplus
}
#endif
#endif
