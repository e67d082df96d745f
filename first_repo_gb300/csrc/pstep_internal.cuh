// Internal definitions shared by the pstep translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include "pstep.h"

namespace pstep {

constexpr double kPi = 3.141592653589793;  // params.h:5
constexpr int kThreads = 256;

// device error word bits (pstep_check)
enum : int32_t {
  kErrNonFinite = 1 << 0,
  kErrRange = 1 << 1,
  kErrMove = 1 << 2,
  kErrTimeout = 1 << 3,
  kErrCapacity = 1 << 4,
};

// Grid geometry as the kernels see it (single rank: il = jl = kl = 0, bs = 1).
struct Geom {
  int n[3];         // interior cells per dimension
  int g[3];         // ghosted extents n+2
  long long gsize;  // g0*g1*g2
  double l[3];      // box size
  double idx[3];    // 1./dx (particle.cpp:19-21)
  double xh[3];     // (ih+1)*dx = n*dx, upper bound of the rank's slab (gridsize.cpp:83-88)
};

__host__ __device__ inline long long glin(const Geom &G, int i, int j, int k) {
  return ((long long)k * G.g[1] + j) * G.g[0] + i;
}

// Per-stage particle-stage constants (particle.cpp:365-379, 462, 484-486).
struct StageConst {
  int k;
  double dt_pre, dt_post;             // dt*RK4_pre, dt*RK4_post (left-to-right as in the reference)
  double dt_pre_is, dt_post_is;       // dt*RK4_pre*iS, dt*RK4_post*iS
  double itp;                         // 1./Tp (scalar)
  double gx, gy, gz;                  // ParticleGravity*g
  double alpha;                       // 0.25*epsilonp*PI*Dp*Dp*I0
  double itth;                        // Nu*PI*Dp*k
};

// FP64 particle storage: structure of arrays.
struct F64State {
  double *base[7];   // x y z u v w T
  double *sint[7];   // *_int
  double *snew[7];   // *_new
  double *np1[7];    // *_np1
  double *rhs_t;     // RHS_T
  double *itp;       // per-particle 1/tau_p (nullptr: scalar)
  int32_t *flag;
  // deposit records (positions -> exact in-cell fraction, node key)
  double *frac_prev[3], *frac_new[3];
  uint32_t *key_prev, *key_new;  // node linear index << 3 | h bits
  double *rhs_u[3];              // RHS_u at x_int of the current stage
};

struct F32Form;

// Counting-sort CSR by node key.
struct Csr {
  int32_t *cell_start;  // gsize + 1
  int32_t *sidx;        // sorted physical indices
  int identity;         // sidx[i] == i (after the per-step reorder)
};

}  // namespace pstep

struct pstep_ctx {
  pstep_config cfg;
  pstep::Geom geom;
  int device;
  cudaStream_t stream;
  int64_t np;
  int64_t cap;
  int num_sms;
  int corr_on;                              // learned correction active (FP32 form)
  int corr_every_stage;                     // run the network at every stage (else stage 0 only)
  uint32_t wait_limit;                      // polls of the tensor-core completion waits (0: default)
  int wait_idle;                            // timeout test: first wait polls a barrier nothing signals
  alignas(16) unsigned char corr_dev[256];  // its kernel constants (stage_f32.cu)

  // FP64 state
  pstep::F64State s;
  pstep::Csr csr_prev, csr_new;
  int new_is_zero;  // no stage has run since the upload: *_new read as zeros
  int int_is_base;  // *_int equal base (start of step): read base
  int np1_is_base;  // *_np1 equal base

  // counting sort scratch
  int32_t *counts;      // gsize
  int32_t *cursor;      // gsize
  int32_t *scan_blocks; // block sums
  int32_t *big_list;    // nodes with long segments (gsize)
  int32_t *big_count;   // device counter
  int64_t scan_nblocks;
  // permutation scratch (per-step reorder)
  void *perm_tmp;
  size_t perm_tmp_bytes;

  // fields (device pointers; own_* when copied from host)
  const double *ux, *uy, *uz, *tf;
  double *own_u[3], *own_t;
  double *dep[PSTEP_NUM_FIELDS];
  double *emean_dev;       // device scalar
  double *mom_dev;         // device: interior sums of the three deposited momentum fields (last stage)
  double *red_partials;    // reduction scratch (4 x 1024)
  double emean_host;
  double mom_host[3];

  // reference-order bookkeeping
  int32_t *ref_of_phys, *phys_of_ref;
  uint8_t *leave_code;      // per particle: bit 2d = high side, bit 2d+1 = low side, dimension d
  unsigned long long *pmax64;  // FP64 form: 1024 x 2 order keys of the last stage's max u and max ug
  int pmax64_state;            // 0: none; 1: filled by this step's last stage; 2: valid for the base state
  int32_t *leavers;         // compaction scratch
  uint32_t *bitmap;         // n bits
  int32_t *ord_scratch;     // misc scratch for the order passes
  int32_t *ord_count;       // device counters
  int64_t ord_scratch_len;

  int32_t *err_word;  // device

  // state machine
  int fields_u, fields_t, primed;
  int fields_t_at_advance;  // temperature binding seen by the fused advance kernel
  int64_t stages_done;
  int timed;
  int phase;  // 0: idle, 1: after interp_advance_deposit, 2: after wrap, 3: after stage_temp
  int cur_k;

  // FP32 form (stage_f32.cu)
  pstep::F32Form *f32;

  struct Prof *prof;  // per-phase event pairs (pstep_profile)

  cudaEvent_t ev0, ev1;
  double last_run_ms;
  int64_t launches;
  char err[512];
};

#define PSTEP_CUDA(call)                                                                    \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      snprintf(h->err, sizeof h->err, "%s:%d %s: %s", __FILE__, __LINE__, #call,            \
               cudaGetErrorString(e_));                                                     \
      return PSTEP_ERR_CUDA;                                                                \
    }                                                                                       \
  } while (0)

#define PSTEP_LAUNCHED(h)                                                                   \
  do {                                                                                      \
    (h)->launches++;                                                                        \
    cudaError_t e_ = cudaGetLastError();                                                    \
    if (e_ != cudaSuccess) {                                                                \
      snprintf((h)->err, sizeof (h)->err, "%s:%d launch: %s", __FILE__, __LINE__,           \
               cudaGetErrorString(e_));                                                     \
      return PSTEP_ERR_CUDA;                                                                \
    }                                                                                       \
  } while (0)

// entry points implemented per translation unit (return pstep_status)
namespace pstep {
void prof_begin(pstep_ctx *h, int phase);
void prof_end(pstep_ctx *h, int phase);
int f64_prime(pstep_ctx *h);
int f64_advance(pstep_ctx *h, int k, double pre, double post);
int f64_deposit_int(pstep_ctx *h);
int f64_stage_temp(pstep_ctx *h);
int f64_reorder(pstep_ctx *h);
int sort_by_node(pstep_ctx *h, const uint32_t *keys, Csr &out);
int csr_sort(pstep_ctx *h, const uint32_t *keys, int shift, int64_t nkeys, const int32_t *order, int32_t *cell_start,
             int32_t *sidx, int order_within);
int csr_count(pstep_ctx *h, const uint32_t *keys, int shift, int64_t nkeys, int32_t *cell_start);
template <typename T>
__global__ void k_gather(const T *__restrict__ src, const int32_t *__restrict__ idx, int64_t n, T *__restrict__ dst);
int fold_cum(pstep_ctx *h, double *f);
int refresh_ghosts(pstep_ctx *h, double *f);
int interior_mean(pstep_ctx *h, const double *f, double *out_dev);
int momentum_sums(pstep_ctx *h);
int f32_download(pstep_ctx *h, double *const dst[7], int32_t *flag, int on_device);
int f32_field_stats(pstep_ctx *h, int field, double r[3]);
int f32_fused_max(pstep_ctx *h, int id, double *out);
int f64_fused_max(pstep_ctx *h, int id, double *out);
int order_passes(pstep_ctx *h);
int order_init(pstep_ctx *h);
int order_permute(pstep_ctx *h, const int32_t *sidx);
}  // namespace pstep
