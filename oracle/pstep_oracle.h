/*
 * CPU restatement of the reference solver's Lagrangian particle step
 * (particle.cpp + the single-rank behaviour of communicator.cpp), FP64,
 * for use as the CHECKER in tests, smoke() and bench.py's CPU-baseline leg.
 * It is test infrastructure: the product never links or calls it.
 *
 * Pinning: tests compare this restatement bit-for-bit with the reference's
 * own sources compiled with a single-rank MPI stub (oracle/_ref, built by
 * oracle/Makefile) and with the golden fixtures in tests/golden made from it.
 */
#ifndef PSTEP_ORACLE_H
#define PSTEP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scalar inputs of the step; names as in params.h of the reference. */
typedef struct {
  int32_t n;          /* cells per side (Nx_tot = Ny_tot = Nz_tot) */
  int32_t particle_gravity, twc, pad;
  double l;           /* box side (Lx = Ly = Lz) */
  double dt, tp, mp, dp, nu, k, epsilonp, i0, cvp, gx, gy, gz;
} pso_config;

typedef struct pso_state pso_state;

/* array ids for pso_array() */
enum {
  PSO_X, PSO_Y, PSO_Z, PSO_X_INT, PSO_Y_INT, PSO_Z_INT, PSO_X_NEW, PSO_Y_NEW, PSO_Z_NEW,
  PSO_X_NP1, PSO_Y_NP1, PSO_Z_NP1, PSO_U, PSO_V, PSO_W, PSO_U_INT, PSO_V_INT, PSO_W_INT,
  PSO_U_NEW, PSO_V_NEW, PSO_W_NEW, PSO_U_NP1, PSO_V_NP1, PSO_W_NP1, PSO_T, PSO_T_INT, PSO_T_NEW,
  PSO_T_NP1, PSO_RHS_U, PSO_RHS_V, PSO_RHS_W, PSO_RHS_T, PSO_UG, PSO_VG, PSO_WG, PSO_TG,
  PSO_NARRAYS
};

pso_state *pso_create(const pso_config *cfg, int64_t capacity);
void pso_destroy(pso_state *s);
/* particle.cpp load_random/Load_All stand-in: set x,u,T,flag for n particles */
int pso_load(pso_state *s, int64_t n, const double *x, const double *y, const double *z, const double *u,
             const double *v, const double *w, const double *t, const int32_t *flag);
/* Per-particle properties (no reference counterpart; the library's
 * pstep_set_particle_props): arrays indexed by particle id (flag, 0..n-1), so
 * they follow each particle through the reference's reordering; NULL keeps the
 * scalar. tau_p replaces Tp, mass_ratio weights the momentum deposit, itth
 * replaces Nu*PI*Dp*k, heat_is 1/(mp*Cvp), alpha the absorbed power, accel
 * ParticleGravity*g. Call after pso_load. */
int pso_set_props(pso_state *s, int64_t n, const double *tau_p, const double *mass_ratio, const double *itth,
                  const double *heat_is, const double *alpha, const double *ax, const double *ay, const double *az);
/* grid.cpp:207-226: *_int = *_np1 = base; gas2part_Temp_int; Compute_RHS_Temp_int; part2gas_Temp_int -> e */
int pso_prime(pso_state *s, const double *tfield, double *e);
/* grid.cpp:659-680 for RK4 stage k with fixed ghosted fields; deposits into c, ax/ay/az, e ((n+2)^3 each) */
int pso_stage(pso_state *s, int k, const double *ux, const double *uy, const double *uz, const double *tfield,
              double *c, double *ax, double *ay, double *az, double *e);
/* grid.cpp:705-712 (particle part) */
void pso_end_stage(pso_state *s);
/* grid.cpp:315-325 (particle part) */
void pso_end_step(pso_state *s);
/* pointer to an internal array (length pso_np) */
double *pso_array(pso_state *s, int id);
int32_t *pso_flag(pso_state *s);
int64_t pso_np(const pso_state *s);
/* number of particles found at x_new == L (an index the reference reads past its ghost layer) */
int64_t pso_edge_hits(const pso_state *s);
/* tensor0::mean over the interior, summed i-outer, k-inner (tensor0.cpp:418-435) */
double pso_mean(const double *field, int32_t n);
/* full steps (4 stages each) with fixed fields; the deposits of the last stage are left in c..e */
int pso_run(pso_state *s, int nsteps, const double *ux, const double *uy, const double *uz, const double *tfield,
            double *c, double *ax, double *ay, double *az, double *e);

#ifdef __cplusplus
}
#endif
#endif
