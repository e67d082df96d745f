/* pstep_gas.h -- the reference's box gas step (grid.cpp: low-Mach
 * variable-density projection on the staggered periodic mesh) on the GPU,
 * FP64, coupled to a particle-step handle (pstep.h).
 *
 * It is the two-way-coupled gas response the learned correction is trained on:
 * it turns the particle step's deposited momentum and energy into the gas
 * disturbance (quiescent-gas runs generate the training data). It restates
 * one time step of simulation.cpp:38-66 for the box:
 *   per RK4 stage  Update_Rho (grid.cpp:327-333), Update_P0 (:539-554),
 *                  Update_Particle (:659-680, through the pstep handle),
 *                  Update_RU_WOP (:387-425), Compute_Div_U_new (:556-563),
 *                  Compute_RHS_Pois (:629-637), Solve_Poisson (:639-643 with the
 *                  iterative FFT solve of poisson.cpp:391-462), Update_RU_WP
 *                  (:651-657), TimeAdvance_RK4 (:705-712);
 *   then           Correct_mean_RU (:566-572) and TimeAdvance (:315-325).
 * Fields use the reference's ghosted layout (pstep.h). Every entry point
 * returns a pstep_status. The particle handle runs on the gas handle's stream
 * (pgas_init and pgas_step set it).
 */
#ifndef PSTEP_GAS_H
#define PSTEP_GAS_H
#include <stdint.h>
#include "pstep.h"

#ifdef __cplusplus
extern "C" {
#endif

/* params.h values the box gas step reads (params.cpp:22-56) */
typedef struct pgas_config {
  int32_t n;           /* cells per side (a power of two, 8..1024) */
  int32_t cooling;     /* Is_Cooling */
  int32_t iterations;  /* Iteration(): Poisson iterations at most */
  int32_t twc;         /* TWC (momentum coupling) */
  double l;            /* box side */
  double dt, mu0, k, cp, cv, rho0, u0, a_force, gx, gy, gz;
  double mp;           /* particle mass: the momentum source is -mp/Vcell * RHS_RU */
  double epsilon;      /* Poisson convergence criterion */
} pgas_config;

typedef struct pgas_ctx *pgas_handle;

/* field ids for pgas_get_field (ghosted (n+2)^3 doubles) */
enum {
  PGAS_RU_X = 0, PGAS_RU_Y, PGAS_RU_Z, PGAS_RHO, PGAS_P, PGAS_T, PGAS_U_X, PGAS_U_Y, PGAS_U_Z, PGAS_C,
  PGAS_RHS_RU_X, PGAS_RHS_RU_Y, PGAS_RHS_RU_Z, PGAS_RHS_PART_TEMP, PGAS_DIVERGENCE, PGAS_RHO_NEW,
  PGAS_NUM_FIELDS
};

int pgas_create(const pgas_config *cfg, pgas_handle *out);
int pgas_destroy(pgas_handle g);
int pgas_set_stream(pgas_handle g, void *cuda_stream);
/* grid::Initialize (grid.cpp:194-226) from interior fields (n^3 each, i fastest):
 * RU, Rho, P = 0, P0; with a particle handle (or NULL) whose particles are
 * uploaded, also the particle prime (pstep_prime) */
int pgas_init(pgas_handle g, pstep_handle particles, const double *ru_x, const double *ru_y, const double *ru_z,
              const double *rho, double p0, int on_device);
/* one time step of gas and particles: pgas_stage for k = 0..3, then pgas_end_step */
int pgas_step(pgas_handle g, pstep_handle particles);
/* RK4 stage k (simulation.cpp:40-48 and grid.cpp:705-712 for one k) */
int pgas_stage(pgas_handle g, pstep_handle particles, int k);
/* Correct_mean_RU and TimeAdvance (grid.cpp:566-572, 315-325) after stage 3 */
int pgas_end_step(pgas_handle g, pstep_handle particles);
int pgas_get_field(pgas_handle g, int id, double *dst, int on_device);
/* thermodynamic pressure P0 after the last step */
int pgas_p0(pgas_handle g, double *p0);
/* Poisson iterations of the last solve */
int pgas_last_iterations(pgas_handle g);
const char *pgas_last_error(pgas_handle g);

#ifdef __cplusplus
}
#endif
#endif
