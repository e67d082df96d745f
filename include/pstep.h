/*
 * pstep.h -- C ABI of the GB300 (sm_103a) Lagrangian particle step.
 *
 * A drop-in for the particle stage of the reference solver (ggeraci/first_repo):
 * the reference's `class particle` (particle.h:12-155) keeps its call surface in
 * a replacement particle.cpp that forwards to these entry points, and gas fields
 * keep the reference's ghosted tensor layout (tensor0.cpp:72-80):
 *
 *     field[(k*(ny+2) + j)*(nx+2) + i],  local index = global index + 1 (bs = 1)
 *
 * with u.x on the left x-face of cell i, u.y on the lower y-face, u.z on the
 * lower z-face and T at cell centres (particle.cpp:346-355, :409-415).
 *
 * Conventions:
 *  - every entry point returns a pstep_status (0 = PSTEP_OK); nothing traps;
 *  - pointers are plain host or device pointers, sizes are element counts;
 *    `on_device` says which (1 = device pointer on the handle's device);
 *  - work is enqueued on the handle's stream (pstep_set_stream); calls that
 *    return data to host memory synchronise that stream;
 *  - one handle = one device = one rank's particles; the reference's MPI
 *    migration is replaced by periodic wrap on the single GPU.
 *
 * Precisions:
 *  - PSTEP_FP64: the plain drop-in. Particle states, cell indices, the wrap and
 *    the particle order (the permutation that Send_Recv, particle.cpp:745-858,
 *    leaves behind) are bit-identical to the reference; deposited fields match
 *    it to round-off of a different (fixed, deterministic) summation order, or
 *    bit for bit with PSTEP_REFERENCE_SUMS.
 *  - PSTEP_FP32: mixed form. Positions as int32 cell + fp32 offset, fields and
 *    ODE arithmetic in fp32; deposits accumulated in fp64-class precision and
 *    written as fp64; balance reductions in fp64.
 */
#ifndef PSTEP_H
#define PSTEP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pstep_ctx *pstep_handle;

typedef enum {
  PSTEP_OK = 0,
  PSTEP_ERR_ARG = 1,        /* null handle/pointer, bad id, bad stage index */
  PSTEP_ERR_CONFIG = 2,     /* unsupported configuration (bs != 1, n < 2, ...) */
  PSTEP_ERR_CAPACITY = 3,   /* more particles than the handle was created for */
  PSTEP_ERR_STATE = 4,      /* call out of order (e.g. stage before fields are bound) */
  PSTEP_ERR_CUDA = 5,       /* a CUDA runtime call failed; see pstep_last_error */
  PSTEP_ERR_NONFINITE = 6,  /* NaN/Inf found in particle state or fields */
  PSTEP_ERR_RANGE = 7,      /* a particle position outside [0, L] (or at L, where the
                               reference indexes past its ghost layer) */
  PSTEP_ERR_MOVE = 8,       /* FP32 form: a particle's stage position more than one cell from
                               its step-start cell along some axis (the deposit gathers each
                               brick's sources from two cells around it, which holds only for
                               moves of at most one cell per stage); the stage's deposits are
                               then incomplete */
  PSTEP_ERR_NOMEM = 9,      /* device allocation failed */
  PSTEP_ERR_TIMEOUT = 10,   /* a bounded device-side wait gave up */
  PSTEP_ERR_IO = 11         /* a snapshot file could not be created, read or written */
} pstep_status;

enum { PSTEP_FP64 = 0, PSTEP_FP32 = 1 };

/* config.flags */
enum {
  PSTEP_TRACK_ORDER = 1,     /* keep the reference's particle order for downloads (FP64 only) */
  PSTEP_CHECK_INPUTS = 2,    /* validate uploads (finite, in range) before use */
  PSTEP_REFERENCE_SUMS = 4,  /* with TRACK_ORDER: add every deposit in the reference's particle
                                order, so deposited fields are bit-identical to the reference
                                (slower; without it the order is fixed but different) */
  PSTEP_KEEP_GAS = 8         /* FP32: keep the gas values each particle's update used (the
                                reference's public ug/vg/wg/Tg, particle.h:110-113) for
                                pstep_get_particle_array (16 bytes per particle and stage) */
};

/* Scalars of params.h that the particle step reads (params.cpp:22-56). The
 * derived values Tp and mp are passed as the reference computes them. */
typedef struct pstep_config {
  int32_t nx, ny, nz;        /* global cells per side: Nx_tot, Ny_tot, Nz_tot */
  int32_t bs;                /* ghost width; the reference's periodic box uses 1 */
  int32_t twc;               /* TWC: deposit momentum (particle.cpp:498, grid.cpp:671) */
  int32_t particle_gravity;  /* ParticleGravity (particle.cpp:376-378) */
  int32_t precision;         /* PSTEP_FP64 or PSTEP_FP32 */
  int32_t flags;             /* PSTEP_TRACK_ORDER | PSTEP_CHECK_INPUTS */
  int64_t capacity;          /* maximum number of particles */
  double lx, ly, lz;         /* box size */
  double dt;                 /* time step */
  double tp;                 /* momentum relaxation time Tp = Rhop*Dp^2/(18*Mu0) */
  double mp;                 /* particle mass mp = Rhop*PI*Dp^3/6 */
  double dp, nu, k, epsilonp, i0, cvp;  /* Dp, Nu, k, epsilon_p, I0, Cvp */
  double gx, gy, gz;         /* gravity (used when particle_gravity != 0) */
} pstep_config;

/* particle array ids for pstep_get_particle_array / pstep_set_particle_array */
enum {
  PSTEP_X = 0, PSTEP_Y, PSTEP_Z, PSTEP_U, PSTEP_V, PSTEP_W, PSTEP_T,                 /* base state */
  PSTEP_X_INT, PSTEP_Y_INT, PSTEP_Z_INT, PSTEP_U_INT, PSTEP_V_INT, PSTEP_W_INT, PSTEP_T_INT,
  PSTEP_X_NEW, PSTEP_Y_NEW, PSTEP_Z_NEW, PSTEP_U_NEW, PSTEP_V_NEW, PSTEP_W_NEW, PSTEP_T_NEW,
  PSTEP_X_NP1, PSTEP_Y_NP1, PSTEP_Z_NP1, PSTEP_U_NP1, PSTEP_V_NP1, PSTEP_W_NP1, PSTEP_T_NP1,
  PSTEP_RHS_T,               /* particle.h:116 */
  PSTEP_FLAG,                /* int32 particle id (particle.h:119) */
  PSTEP_UG, PSTEP_VG, PSTEP_WG, /* gas velocity at x_int used by the last stage (gas2part_velocity,
                                   particle.cpp:340-360); FP32 with PSTEP_KEEP_GAS */
  PSTEP_TG,                  /* gas temperature at x_new used by the last stage (particle.cpp:430-456) */
  PSTEP_NUM_ARRAYS
};

/* deposited field ids for pstep_get_field (ghosted (nx+2)(ny+2)(nz+2) doubles) */
enum {
  PSTEP_FIELD_C = 0,         /* concentration, part2gas_concentration (particle.cpp:526-559) */
  PSTEP_FIELD_RU_X,          /* RHS_RU.x, part2gas_velocity (particle.cpp:498-524) */
  PSTEP_FIELD_RU_Y,
  PSTEP_FIELD_RU_Z,
  PSTEP_FIELD_PART_TEMP,     /* RHS_Part_Temp, part2gas_Temp_int/new (particle.cpp:586-658) */
  PSTEP_NUM_FIELDS
};

/* Create a handle on the current CUDA device (replaces particle::particle,
 * particle.cpp:14-40; allocates all device storage up front). */
int pstep_create(const pstep_config *cfg, pstep_handle *out);
/* Release everything (particle::~particle, particle.cpp:42-56). */
int pstep_destroy(pstep_handle h);
/* Stream for all work of this handle (cudaStream_t; 0 = legacy default). */
int pstep_set_stream(pstep_handle h, void *cuda_stream);
/* Update the scalar parameters (dt, tp, mp, dp, nu, k, epsilonp, i0, cvp, gravity,
 * twc) that params::update switches after its threshold (params.cpp:66-77).
 * Sizes, precision, flags and capacity must not change. */
int pstep_update_params(pstep_handle h, const pstep_config *cfg);

/* Set the base particle state x,u,T and flag for n particles (the reference's
 * load_random / Load_All leave these in the public vectors, particle.cpp:919-999).
 * Also does the particle part of grid::Initialize (grid.cpp:207-221):
 * *_int = *_np1 = base. */
int pstep_upload_particles(pstep_handle h, int64_t n, const double *x, const double *y, const double *z,
                           const double *u, const double *v, const double *w, const double *t,
                           const int32_t *flag, int on_device);
/* Read the base particle state x,u,T and the ids back (the reference's public vectors
 * after grid::TimeAdvance, grid.cpp:315-325): the same arrays as pstep_get_particle_array
 * with PSTEP_X .. PSTEP_T and PSTEP_FLAG, in the same order, from one pass over the
 * particles. Host destinations are complete when the call returns. */
int pstep_download_particles(pstep_handle h, double *x, double *y, double *z, double *u, double *v, double *w,
                             double *t, int32_t *flag, int on_device);
/* Optional per-particle momentum relaxation time (same order as the upload);
 * replaces the scalar Tp for every particle. NULL restores the scalar. */
int pstep_set_tau_p(pstep_handle h, const double *tau_p, int on_device);

/* Per-particle physical properties. No reference counterpart: the reference's
 * particles share the scalars of params.h. Each pointer holds one value per
 * particle in upload order, or is NULL to keep the config's scalar. Set after
 * pstep_upload_particles and before pstep_prime; FP32 form (the FP64 form
 * accepts tau_p alone). */
typedef struct pstep_particle_props {
  const double *tau_p;       /* momentum relaxation time (replaces Tp, particle.cpp:365) */
  const double *mass_ratio;  /* m_p / cfg.mp: weight of the momentum deposit (the gas scales
                                RHS_RU by -mp/Vcell, grid.cpp:393) */
  const double *itth;        /* heat-transfer coefficient Nu*PI*Dp*k (particle.cpp:462) */
  const double *heat_is;     /* 1/(m_p*Cvp) (particle.cpp:485) */
  const double *alpha;       /* absorbed power 0.25*epsilonp*PI*Dp^2*I0 (particle.cpp:484) */
  const double *accel[3];    /* body acceleration, replaces ParticleGravity*g (particle.cpp:376-378) */
} pstep_particle_props;
int pstep_set_particle_props(pstep_handle h, const pstep_particle_props *props, int on_device);

/* Learned correction of the interpolated gas state (FP32 form; no reference
 * counterpart: the reference uses the disturbed interpolation, particle.cpp:340-360,
 * 430-456). A network in the layout of pstep_mlp.h predicts, for every particle
 * and stage, its own disturbance of the gas at x_int in units of the slip that
 * drives it, y = d / |s| (learned where the drag used the disturbed slip s =
 * u_int - u_plain). The step uses u_gas = u_plain - y[0..2] |s_drive| and
 * Tg = Tg_plain - y[3] dT_drive, where s_drive and dT_drive are the slip and the
 * T_new - Tg the particle's drag and heat transfer used in the previous stage
 * (the plain values at the first stage; capped at 10x the plain ones): a fixed-
 * point iteration across stages towards the self-consistent correction, which
 * leaves the drag's dependence on the current gas value as in the plain step.
 * The network runs on the tensor cores inside the advance kernel. Features,
 * each mapped to (value - shift[i]) * scale[i]:
 *   0-2 offset of x_int in its cell (cell units), 3-5 s_drive/|s_drive|, 6 d_p/dx,
 *   7 ln Re_p with Re_p = |s_drive| d_p / nu_gas, 8 Q = alpha/(m_p Cvp), 9 ln tau_p;
 * d_p is itth/(Nu*PI*k) with per-particle itth, else Dp. Particles with zero slip
 * or with d_p/dx, Re_p, Q or tau_p outside [lo, hi] keep the plain values. */
typedef struct pstep_correction {
  const float *params;       /* PMLP_NPARAM floats, host memory */
  float shift[10], scale[10];
  float lo[4], hi[4];        /* ranges of d_p/dx, Re_p, Q, tau_p */
  float prior_re;            /* > 0: the network's outputs are in units of the prior
                                (d_p/dx) / (1 + Re_p / ((d_p/dx) prior_re)), the disturbance's
                                dependence on size and cell Reynolds number; 0: no prior */
  double nu_gas;             /* kinematic viscosity of the gas */
  int32_t every_stage;       /* 0: the network runs at stage 0 and its output serves the step's
                                four stages (each with its own drive slip and prior); 1: it runs
                                at every stage, at that stage's x_int */
  float drive_cap;           /* the drive slip is at most drive_cap times the plain slip (a bound
                                on the lagged iteration; output y < 1 converges to a drive of
                                plain / (1 - y), so the cap admits y up to 1 - 1/drive_cap);
                                0: 10 */
} pstep_correction;
/* NULL switches the correction off */
int pstep_set_correction(pstep_handle h, const pstep_correction *c);
/* The fused inference's tensor-core completion waits are bounded: after `polls` polls
 * of an MMA's mbarrier (0: the default, 2^22) a warpgroup gives up, the kernel sets
 * PSTEP_ERR_TIMEOUT in the check word (pstep_check), waits for the MMAs it has issued
 * (always with the default bound), frees its tensor memory and returns. With
 * idle_first != 0 each warpgroup's first wait polls a barrier that nothing signals, so
 * the timeout path runs as it would for a completion that never arrives (for testing
 * that path; the stage's results are then incomplete). No reference counterpart. */
int pstep_set_wait_limit(pstep_handle h, uint32_t polls, int idle_first);
int64_t pstep_num_particles(pstep_handle h);

/* Gas fields, ghosted layout. The velocity is U = RU_int/Rho_face (grid.cpp:662),
 * the temperature T = (P0_new/R)/Rho_new (grid.cpp:676); both are formed by the
 * caller as in the reference. Host pointers are copied; device pointers are
 * read in place and must stay valid until the next bind. */
int pstep_bind_velocity(pstep_handle h, const double *ux, const double *uy, const double *uz, int on_device);
int pstep_bind_temperature(pstep_handle h, const double *t, int on_device);

/* grid.cpp:223-226: gas2part_Temp_int + Compute_RHS_Temp_int + part2gas_Temp_int
 * (RHS_Part_Temp is then available through pstep_get_field). Needs the bound
 * temperature. */
int pstep_prime(pstep_handle h);

/* One RK4 stage (k = 0..3) of grid::Update_Particle (grid.cpp:659-680), split as
 * the reference's particle.h calls group:
 *   interp_advance_deposit  gas2part_velocity, update_position, update_velocity,
 *                           update_Temp, part2gas_concentration, part2gas_velocity
 *   wrap                    Send_Recv (periodic wrap + the reference's reordering)
 *   stage_temp              gas2part_Temp_new, Compute_RHS_Temp_new,
 *                           part2gas_Temp_new, and the interior mean of
 *                           RHS_Part_Temp (grid.cpp:541)
 * pre/post are the RK4 coefficients of grid.cpp:16-23 for stage k. */
int pstep_stage_interp_advance_deposit(pstep_handle h, int k, double pre, double post);
int pstep_wrap(pstep_handle h);
int pstep_stage_temp(pstep_handle h);
/* the three above in order */
int pstep_stage(pstep_handle h, int k, double pre, double post);
/* grid::TimeAdvance_RK4, particle part (grid.cpp:705-712): *_int = *_new */
int pstep_end_stage(pstep_handle h);
/* grid::TimeAdvance, particle part (grid.cpp:315-325): base = *_np1; the
 * particles are then reordered in device memory by cell (downloads keep the
 * reference order when PSTEP_TRACK_ORDER is set). */
int pstep_end_step(pstep_handle h);
/* nsteps full steps with the bound fields held fixed (4 x stage + end_stage,
 * then end_step), standard RK4 coefficients. */
int pstep_run(pstep_handle h, int nsteps);

/* Copy a deposited field (ghosted layout) to dst. */
int pstep_get_field(pstep_handle h, int field_id, double *dst, int on_device);
/* RHS_Part_Temp.mean() of the last stage_temp/prime (tensor0.cpp:418-435, grid.cpp:541). */
int pstep_energy_mean(pstep_handle h, double *out);
/* The momentum balance of the last stage's deposit: the interior sums of RHS_RU.x,
 * .y, .z (the particles' momentum source; the gas adds it times -mp/Vcell,
 * grid.cpp:393, and keeps the box's mean momentum with Correct_mean_RU,
 * grid.cpp:565-577), out[0..2], in fp64. PSTEP_FP64: a fixed-order fp64 sum of the
 * deposited values; PSTEP_FP32: the exact integer sum of the fixed-point deposits,
 * correctly rounded (its energy mean, pstep_energy_mean, comes from the same exact
 * totals). Zeros without TWC. Synchronises the stream. No reference counterpart as an
 * entry point (the reference forms these means on the host inside grid). */
int pstep_momentum_sums(pstep_handle h, double *out);
/* Copy one particle array (PSTEP_X ... PSTEP_FLAG) to dst (int32 for PSTEP_FLAG),
 * in the reference's order when PSTEP_TRACK_ORDER is set. */
int pstep_get_particle_array(pstep_handle h, int array_id, void *dst, int on_device);

/* Interior mean of a ghosted field ((nx+2)(ny+2)(nz+2) doubles, device pointer),
 * written to *out (device pointer), enqueued on `stream`; the same quantity as
 * pstep_energy_mean. No counterpart in the reference (whose tensor0::mean runs on
 * the host): this entry point allocates no device memory, for callers that cannot
 * call cudaMalloc (work recorded during CUDA stream capture, applications whose own
 * pool owns device memory, loops that must not synchronise the device). Its
 * scratch is a fixed device array of 2^20 row sums (8 MiB, held by every GPU that
 * loads the library until the process exits): ny*nz above 2^20 returns
 * PSTEP_ERR_CAPACITY. The first call on a device looks up that array's address
 * (make it before any stream capture: a first call on a capturing stream returns
 * PSTEP_ERR_STATE and launches nothing). Every call writes all the scratch it reads,
 * so nothing needs clearing, but all calls share the array: calls that overlap on
 * the GPU race. Messages: pstep_noalloc_last_error(), per calling thread. */
int pstep_field_mean_noalloc(const double *field, int32_t nx, int32_t ny, int32_t nz, double *out, void *stream);
const char *pstep_noalloc_last_error(void);

/* Error reporting */
const char *pstep_last_error(pstep_handle h);
const char *pstep_status_string(int status);
/* Device-side check word: the OR of PSTEP_ERR_* conditions seen by the kernels
 * since the last call (non-finite values, out-of-range positions, moves of more
 * than one cell). Synchronises the stream and clears the word. */
int pstep_check(pstep_handle h, int32_t *flags_out);

/* Per-phase kernel timing with CUDA events on the handle's stream (no host
 * synchronisation while enabled). Phases: PSTEP_PHASE_*. pstep_profile_read
 * synchronises, returns total ms and event-pair counts per phase, and resets. */
enum {
  PSTEP_PHASE_ADVANCE = 0,     /* interpolation + RK4 advance + wrap + T interpolation */
  PSTEP_PHASE_DEPOSIT_INT,     /* concentration + momentum deposits, fold, refresh */
  PSTEP_PHASE_ORDER,           /* reference-order bookkeeping of Send_Recv */
  PSTEP_PHASE_SORT,            /* counting sort by node (CSR) */
  PSTEP_PHASE_DEPOSIT_TEMP,    /* energy deposit, fold, refresh, interior mean */
  PSTEP_PHASE_REORDER,         /* per-step reorder of particle storage */
  PSTEP_PHASE_NETWORK,         /* FP32 learned correction: the tensor-core network */
  PSTEP_NUM_PHASES
};
int pstep_profile(pstep_handle h, int enable);
int pstep_profile_read(pstep_handle h, double *ms, int64_t *counts, int nphases);

/* Timing of the last pstep_run on the handle's stream (CUDA events): total ms. */
int pstep_last_run_ms(pstep_handle h, double *ms);
/* Number of kernel launches enqueued by this handle since creation. */
int64_t pstep_launch_count(pstep_handle h);

/* ---- Diagnostics: the reference's particle statistics and the extrema of the
 * deposited fields that its statistics output takes (grid.cpp:715-735). All
 * synchronise the stream; results are for this handle (one rank). ---- */
/* particle::NP_TOT (particle.cpp:662-669): the particle count (summed over ranks) */
int pstep_np_tot(pstep_handle h, int64_t *out);
/* particle::max (particle.cpp:671-685) of one particle array (PSTEP_X ... PSTEP_TG, not
 * PSTEP_FLAG), as pstep_get_particle_array would return it: its largest value, or -1e9
 * when there are no particles. After pstep_end_step (or pstep_run), both forms: the
 * maxima of u and ug that grid::Statistics asks for (grid.cpp:726-727) are gathered by
 * the step's last stage in its epilogue, so PSTEP_U and PSTEP_UG read them without a
 * pass over the particles (PSTEP_UG then needs no PSTEP_KEEP_GAS, and the FP64 form,
 * which keeps no per-particle gas values, answers it only this way); other arrays, and
 * any state not left by a full step, take a pass. */
int pstep_max(pstep_handle h, int id, double *out);
/* particle::Balance_Index (particle.cpp:730-741): largest over smallest per-rank particle
 * count; one rank: Np / Np (NaN when there are no particles) */
int pstep_balance_index(pstep_handle h, double *out);
/* tensor0::max, ::min and ::mean (tensor0.cpp:452-463, 492-503, 418-435) of a deposited
 * field (PSTEP_FIELD_*), over the interior cells. The maximum and minimum are exact; the
 * mean is the interior sum (taken in a fixed order, not the reference's i-j-k loop
 * order, so it can differ in the last bits) over n^3. PSTEP_FP32, after pstep_end_step
 * (or pstep_run) or pstep_prime: gathered by the last deposit as it wrote the field
 * (exact integer maximum, minimum and sum, the sum rounded once), so the call reads three
 * numbers and makes no pass over the grid; after a stage other than a step's last, a
 * pass. Any of the outputs may be NULL. */
int pstep_field_stats(pstep_handle h, int field, double *max, double *min, double *mean);
/* particle::find_tag (particle.cpp:721-731) for n ids: xyz[3 i .. 3 i + 2] = the position of
 * the particle with id tags[i] and found[i] = 1, or found[i] = 0 (xyz untouched) when no
 * particle has it. particle::trajectory (:687-719) asks it for ids 0, K, 2K, ... */
int pstep_find_tags(pstep_handle h, const int32_t *tags, int32_t n, double *xyz, int32_t *found);

/* ---- Snapshot files: particle::Store_All / Load_All (particle.cpp:867-1025), one rank.
 * Raw native-endian arrays, one file per quantity: doubles for x y z u v w T, int32 for
 * the ids. ---- */
/* writes <data_dir>Part_{x,y,z,u,v,w,T,flag}_<num_ts>.bin (data_dir is a prefix, as
 * params.data_dir(); include the trailing '/'), in the order pstep_get_particle_array
 * returns (with PSTEP_TRACK_ORDER: the reference's order, byte-identical to its files).
 * A file that exists already is an error (MPI_MODE_EXCL), PSTEP_ERR_IO. */
int pstep_store_all(pstep_handle h, const char *data_dir, int num_ts);
/* reads n0 particles from <dir>Restart_Part_{x,...,flag}.bin (box != 0) or
 * <dir>Restart_Part_{x,...,flag}_IO.bin (the IO duct's files) and uploads them as
 * pstep_upload_particles does; a missing or short file is PSTEP_ERR_IO. The reference
 * then runs Send_Recv, which on one rank changes nothing for positions inside the box. */
int pstep_load_all(pstep_handle h, const char *dir, int64_t n0, int box);

#ifdef __cplusplus
}
#endif
#endif
