// C ABI of the particle step (include/pstep.h): storage, call sequencing and
// host<->device plumbing around the kernels. Every entry point returns a
// pstep_status; nothing here synchronises except calls that hand data to the host.
#include <stdlib.h>
#include <string.h>
#include <new>
#include <vector>
#include "pstep_internal.cuh"

struct Prof {
  int enabled = 0;
  std::vector<cudaEvent_t> pool;  // created on demand, reused
  std::vector<int> phase;         // phase of each recorded pair
  size_t used = 0;                // events in use (pairs * 2)
  int open_phase = -1;
  double ms[PSTEP_NUM_PHASES] = {0};
  int64_t count[PSTEP_NUM_PHASES] = {0};
};

namespace pstep {
static cudaEvent_t prof_event(pstep_ctx *h) {
  Prof *p = h->prof;
  if (p->used == p->pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    p->pool.push_back(e);
  }
  return p->pool[p->used++];
}
void prof_begin(pstep_ctx *h, int phase) {
  if (!h->prof || !h->prof->enabled) return;
  cudaEvent_t e = prof_event(h);
  if (e) {
    cudaEventRecord(e, h->stream);
    h->prof->phase.push_back(phase);
  }
}
void prof_end(pstep_ctx *h, int phase) {
  if (!h->prof || !h->prof->enabled) return;
  (void)phase;
  cudaEvent_t e = prof_event(h);
  if (e) cudaEventRecord(e, h->stream);
}
}  // namespace pstep

namespace pstep {
StageConst make_stage_const(const pstep_config &cfg, int k, double pre, double post);
int f64_prime_kernel(pstep_ctx *h);
int deposit_temperature(pstep_ctx *h, const Csr &csr, double *const frac[3], const uint32_t *key);
int f64_temp_gather(pstep_ctx *h);
int exclusive_scan(pstep_ctx *h, const int32_t *in, int64_t n, int32_t *out, int32_t *out2);
int64_t scan_blocks_needed(int64_t n);
int64_t order_scratch_words(int64_t cap);
int f32_create(pstep_ctx *h);
int f32_destroy(pstep_ctx *h);
int f32_upload(pstep_ctx *h, const double *x, const double *y, const double *z, const double *u, const double *v,
               const double *w, const double *t, int on_device);
int f32_set_tau(pstep_ctx *h, const double *tau, int on_device);
int f32_set_props(pstep_ctx *h, const pstep_particle_props *props, int on_device);
int f32_set_correction(pstep_ctx *h, const pstep_correction *c);
int f32_bind_fields(pstep_ctx *h, int which);
int f32_prime(pstep_ctx *h);
int f32_stage(pstep_ctx *h, int k, double pre, double post);
int f32_end_stage(pstep_ctx *h);
int f32_end_step(pstep_ctx *h);
int f32_get_array(pstep_ctx *h, int id, void *dst, int on_device);
}  // namespace pstep

using namespace pstep;

namespace {

const double kPre[4] = {0.5, 0.5, 1., 1. / 6.};             // grid.cpp:16-19
const double kPost[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};  // grid.cpp:20-23

int fail(pstep_ctx *h, int code, const char *msg) {
  if (h) snprintf(h->err, sizeof h->err, "%s", msg);
  return code;
}

template <typename T>
int dalloc(pstep_ctx *h, T *&p, size_t count) {
  p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void **)&p, sizeof(T) * count);
  if (e != cudaSuccess) {
    p = nullptr;
    snprintf(h->err, sizeof h->err, "cudaMalloc(%zu bytes): %s", sizeof(T) * count, cudaGetErrorString(e));
    cudaGetLastError();
    return PSTEP_ERR_NOMEM;
  }
  return PSTEP_OK;
}

template <typename T>
void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

cudaMemcpyKind kind_in(int on_device) { return on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }
cudaMemcpyKind kind_out(int on_device) { return on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost; }

__global__ void k_recip(const double *__restrict__ tau, int64_t n, double *__restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = 1. / tau[i];
}

__global__ void k_gather_ref(const double *__restrict__ src, const int32_t *__restrict__ phys_of_ref, int64_t n,
                             double *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[phys_of_ref ? phys_of_ref[i] : i];
}
__global__ void k_gather_ref_i(const int32_t *__restrict__ src, const int32_t *__restrict__ phys_of_ref, int64_t n,
                               int32_t *__restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[phys_of_ref ? phys_of_ref[i] : i];
}
__global__ void k_fill_i32(int32_t *a, int64_t n, int32_t v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

int blocks_for(int64_t n) { return (int)((n + kThreads - 1) / kThreads); }

bool is_f32(const pstep_ctx *h) { return h->cfg.precision == PSTEP_FP32; }

void release(pstep_ctx *h) {
  for (int q = 0; q < 7; ++q) {
    dfree(h->s.base[q]); dfree(h->s.sint[q]); dfree(h->s.snew[q]); dfree(h->s.np1[q]);
  }
  dfree(h->s.rhs_t); dfree(h->s.itp); dfree(h->s.flag);
  for (int d = 0; d < 3; ++d) { dfree(h->s.frac_prev[d]); dfree(h->s.frac_new[d]); dfree(h->s.rhs_u[d]); }
  dfree(h->s.key_prev); dfree(h->s.key_new);
  dfree(h->csr_prev.cell_start); dfree(h->csr_prev.sidx); dfree(h->csr_new.cell_start); dfree(h->csr_new.sidx);
  dfree(h->counts); dfree(h->cursor); dfree(h->scan_blocks); dfree(h->big_list); dfree(h->big_count);
  void *pt = h->perm_tmp; if (pt) cudaFree(pt); h->perm_tmp = nullptr;
  for (int d = 0; d < 3; ++d) dfree(h->own_u[d]);
  dfree(h->own_t);
  for (int f = 0; f < PSTEP_NUM_FIELDS; ++f) dfree(h->dep[f]);
  dfree(h->emean_dev); dfree(h->mom_dev); dfree(h->red_partials);
  dfree(h->pmax64);
  dfree(h->ref_of_phys); dfree(h->phys_of_ref); dfree(h->leave_code); dfree(h->ord_scratch); dfree(h->ord_count);
  dfree(h->err_word);
  if (is_f32(h)) f32_destroy(h);
}

#define TRY(x)                  \
  do {                          \
    int rc_ = (x);              \
    if (rc_ != PSTEP_OK) return rc_; \
  } while (0)

int alloc_all(pstep_ctx *h) {
  const size_t cap = (size_t)h->cap;
  const size_t gs = (size_t)h->geom.gsize;
  if (!is_f32(h)) {
    for (int q = 0; q < 7; ++q) {
      TRY(dalloc(h, h->s.base[q], cap)); TRY(dalloc(h, h->s.sint[q], cap));
      TRY(dalloc(h, h->s.snew[q], cap)); TRY(dalloc(h, h->s.np1[q], cap));
    }
    TRY(dalloc(h, h->s.rhs_t, cap));
    TRY(dalloc(h, h->s.flag, cap));
    for (int d = 0; d < 3; ++d) {
      TRY(dalloc(h, h->s.frac_prev[d], cap)); TRY(dalloc(h, h->s.frac_new[d], cap));
      TRY(dalloc(h, h->s.rhs_u[d], cap));
    }
    TRY(dalloc(h, h->s.key_prev, cap)); TRY(dalloc(h, h->s.key_new, cap));
    TRY(dalloc(h, h->csr_prev.sidx, cap)); TRY(dalloc(h, h->csr_new.sidx, cap));
    TRY(dalloc(h, h->pmax64, 2 * 1024));
    if (h->cfg.flags & PSTEP_TRACK_ORDER) {
      TRY(dalloc(h, h->ref_of_phys, cap)); TRY(dalloc(h, h->phys_of_ref, cap));
      TRY(dalloc(h, h->leave_code, cap));
      h->ord_scratch_len = (int64_t)cap + 64;
      TRY(dalloc(h, h->ord_scratch, (size_t)order_scratch_words((int64_t)cap)));
      TRY(dalloc(h, h->ord_count, 8));
      // anchor slots start empty (-1); the order passes restore them after use
      int32_t *slots = h->ord_scratch + 5 * h->ord_scratch_len;
      k_fill_i32<<<blocks_for(h->ord_scratch_len), kThreads, 0, h->stream>>>(slots, h->ord_scratch_len, -1);
      PSTEP_LAUNCHED(h);
    }
  }
  {  // permutation / download scratch, both forms
    double *pt = nullptr;
    TRY(dalloc(h, pt, cap));
    h->perm_tmp = pt;
  }
  TRY(dalloc(h, h->csr_prev.cell_start, gs + 1)); TRY(dalloc(h, h->csr_new.cell_start, gs + 1));
  TRY(dalloc(h, h->counts, gs)); TRY(dalloc(h, h->cursor, gs));
  TRY(dalloc(h, h->big_list, gs)); TRY(dalloc(h, h->big_count, 1));
  int64_t scan_n = (int64_t)gs + 1;
  if ((int64_t)cap > scan_n) scan_n = (int64_t)cap;
  h->scan_nblocks = scan_blocks_needed(scan_n) + 1;
  TRY(dalloc(h, h->scan_blocks, (size_t)h->scan_nblocks));
  for (int f = 0; f < PSTEP_NUM_FIELDS; ++f) {
    TRY(dalloc(h, h->dep[f], gs));
    PSTEP_CUDA(cudaMemsetAsync(h->dep[f], 0, sizeof(double) * gs, h->stream));
  }
  TRY(dalloc(h, h->emean_dev, 1));
  TRY(dalloc(h, h->mom_dev, 3));
  PSTEP_CUDA(cudaMemsetAsync(h->mom_dev, 0, 3 * sizeof(double), h->stream));
  TRY(dalloc(h, h->red_partials, 4 * 1024));
  TRY(dalloc(h, h->err_word, 1));
  PSTEP_CUDA(cudaMemsetAsync(h->err_word, 0, sizeof(int32_t), h->stream));
  PSTEP_CUDA(cudaMemsetAsync(h->emean_dev, 0, sizeof(double), h->stream));
  if (is_f32(h)) TRY(f32_create(h));
  return PSTEP_OK;
}

int copy_field_in(pstep_ctx *h, const double *src, int on_device, double *&own, const double *&bound) {
  const size_t gs = (size_t)h->geom.gsize;
  if (!src) return fail(h, PSTEP_ERR_ARG, "null field pointer");
  if (on_device) {
    bound = src;
    return PSTEP_OK;
  }
  if (!own) TRY(dalloc(h, own, gs));
  PSTEP_CUDA(cudaMemcpyAsync(own, src, sizeof(double) * gs, cudaMemcpyHostToDevice, h->stream));
  bound = own;
  return PSTEP_OK;
}

}  // namespace

extern "C" {

const char *pstep_status_string(int s) {
  switch (s) {
    case PSTEP_OK: return "ok";
    case PSTEP_ERR_ARG: return "invalid argument";
    case PSTEP_ERR_CONFIG: return "unsupported configuration";
    case PSTEP_ERR_CAPACITY: return "capacity exceeded";
    case PSTEP_ERR_STATE: return "call out of sequence";
    case PSTEP_ERR_CUDA: return "CUDA error";
    case PSTEP_ERR_NONFINITE: return "non-finite value";
    case PSTEP_ERR_RANGE: return "position out of range";
    case PSTEP_ERR_MOVE: return "particle moved more than one cell";
    case PSTEP_ERR_NOMEM: return "device memory exhausted";
    case PSTEP_ERR_TIMEOUT: return "device wait timed out";
    case PSTEP_ERR_IO: return "snapshot file error";
    default: return "unknown status";
  }
}

const char *pstep_last_error(pstep_handle h) { return h ? h->err : "null handle"; }

int pstep_create(const pstep_config *cfg, pstep_handle *out) {
  if (!cfg || !out) return PSTEP_ERR_ARG;
  *out = nullptr;
  if (cfg->bs != 1) return PSTEP_ERR_CONFIG;
  if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2) return PSTEP_ERR_CONFIG;
  if (!(cfg->lx > 0 && cfg->ly > 0 && cfg->lz > 0 && cfg->dt > 0)) return PSTEP_ERR_CONFIG;
  if (cfg->capacity < 0 || cfg->capacity > INT32_MAX - 64) return PSTEP_ERR_CONFIG;
  if (cfg->precision != PSTEP_FP64 && cfg->precision != PSTEP_FP32) return PSTEP_ERR_CONFIG;
  const long long gsize = (long long)(cfg->nx + 2) * (cfg->ny + 2) * (cfg->nz + 2);
  if (gsize >= (1ll << 29)) return PSTEP_ERR_CONFIG;  // node keys carry 3 extra bits in 32
  pstep_ctx *h = new (std::nothrow) pstep_ctx();
  if (!h) return PSTEP_ERR_NOMEM;
  memset((void *)h, 0, sizeof(pstep_ctx));
  h->cfg = *cfg;
  h->cfg.particle_gravity = cfg->particle_gravity ? 1 : 0;
  h->cfg.twc = cfg->twc ? 1 : 0;
  if (h->cfg.precision == PSTEP_FP32) h->cfg.flags &= ~PSTEP_TRACK_ORDER;
  h->cap = cfg->capacity;
  cudaGetDevice(&h->device);
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  Geom &G = h->geom;
  const int n3[3] = {cfg->nx, cfg->ny, cfg->nz};
  const double l3[3] = {cfg->lx, cfg->ly, cfg->lz};
  for (int d = 0; d < 3; ++d) {
    G.n[d] = n3[d];
    G.g[d] = n3[d] + 2;
    G.l[d] = l3[d];
    const double dx = l3[d] / n3[d];           // gridsize.cpp:26-28
    G.idx[d] = 1. / dx;                        // particle.cpp:19-21
    G.xh[d] = (double)((n3[d] - 1) + 1) * dx;  // gridsize.cpp:83-88 with ih = Nx_tot - 1
  }
  G.gsize = gsize;
  h->stream = 0;
  int rc = alloc_all(h);
  if (rc == PSTEP_OK) {
    if (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) rc = PSTEP_ERR_CUDA;
  }
  if (rc == PSTEP_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = PSTEP_ERR_CUDA;
  if (rc != PSTEP_OK) {
    release(h);
    delete h;
    return rc;
  }
  *out = h;
  return PSTEP_OK;
}

int pstep_destroy(pstep_handle h) {
  if (!h) return PSTEP_ERR_ARG;
  cudaStreamSynchronize(h->stream);
  release(h);
  if (h->prof) {
    for (cudaEvent_t e : h->prof->pool) cudaEventDestroy(e);
    delete h->prof;
    h->prof = nullptr;
  }
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  delete h;
  return PSTEP_OK;
}

int pstep_update_params(pstep_handle h, const pstep_config *c) {
  if (!h || !c) return PSTEP_ERR_ARG;
  if (c->nx != h->cfg.nx || c->ny != h->cfg.ny || c->nz != h->cfg.nz || c->bs != h->cfg.bs ||
      c->precision != h->cfg.precision || c->capacity != h->cfg.capacity || c->lx != h->cfg.lx ||
      c->ly != h->cfg.ly || c->lz != h->cfg.lz)
    return fail(h, PSTEP_ERR_CONFIG, "sizes, box, precision and capacity cannot change");
  if (!(c->dt > 0)) return fail(h, PSTEP_ERR_CONFIG, "dt must be positive");
  h->cfg.dt = c->dt; h->cfg.tp = c->tp; h->cfg.mp = c->mp; h->cfg.dp = c->dp; h->cfg.nu = c->nu;
  h->cfg.k = c->k; h->cfg.epsilonp = c->epsilonp; h->cfg.i0 = c->i0; h->cfg.cvp = c->cvp;
  h->cfg.gx = c->gx; h->cfg.gy = c->gy; h->cfg.gz = c->gz;
  h->cfg.particle_gravity = c->particle_gravity ? 1 : 0;
  h->cfg.twc = c->twc ? 1 : 0;
  return PSTEP_OK;
}

int pstep_set_stream(pstep_handle h, void *stream) {
  if (!h) return PSTEP_ERR_ARG;
  h->stream = (cudaStream_t)stream;
  return PSTEP_OK;
}

int64_t pstep_num_particles(pstep_handle h) { return h ? h->np : -1; }
int64_t pstep_launch_count(pstep_handle h) { return h ? h->launches : -1; }

int pstep_upload_particles(pstep_handle h, int64_t n, const double *x, const double *y, const double *z,
                           const double *u, const double *v, const double *w, const double *t, const int32_t *flag,
                           int on_device) {
  if (!h) return PSTEP_ERR_ARG;
  if (n < 0) return fail(h, PSTEP_ERR_ARG, "negative particle count");
  if (n > h->cap) return fail(h, PSTEP_ERR_CAPACITY, "more particles than capacity");
  if (n > 0 && (!x || !y || !z || !u || !v || !w || !t || !flag)) return fail(h, PSTEP_ERR_ARG, "null particle array");
  h->np = n;
  h->primed = 0;
  h->phase = 0;
  h->pmax64_state = 0;
  if (is_f32(h)) {
    TRY(f32_upload(h, x, y, z, u, v, w, t, on_device));
  } else {
    const double *src[7] = {x, y, z, u, v, w, t};
    for (int q = 0; q < 7 && n > 0; ++q)
      PSTEP_CUDA(cudaMemcpyAsync(h->s.base[q], src[q], sizeof(double) * n, kind_in(on_device), h->stream));
  }
  // flag lives in the FP64 storage for both forms
  if (!h->s.flag) TRY(dalloc(h, h->s.flag, (size_t)h->cap));
  if (n > 0) PSTEP_CUDA(cudaMemcpyAsync(h->s.flag, flag, sizeof(int32_t) * n, kind_in(on_device), h->stream));
  if (h->s.itp) dfree(h->s.itp);  // a new population drops any per-particle tau_p
  h->int_is_base = 1;
  h->np1_is_base = 1;
  h->new_is_zero = 1;  // the reference's *_new vectors are zero-filled until the first stage writes them
  h->csr_prev.identity = 0;
  if (h->cfg.flags & PSTEP_TRACK_ORDER) TRY(order_init(h));
  // host arrays may be reused or freed when this returns: every copy from them has completed
  if (!on_device) PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  if (h->cfg.flags & PSTEP_CHECK_INPUTS && !on_device) {
    for (int64_t i = 0; i < n; ++i) {
      const double p[3] = {x[i], y[i], z[i]};
      const double L[3] = {h->cfg.lx, h->cfg.ly, h->cfg.lz};
      for (int d = 0; d < 3; ++d) {
        if (!(p[d] == p[d]) || p[d] - p[d] != 0.0) return fail(h, PSTEP_ERR_NONFINITE, "non-finite position");
        if (p[d] < 0.0 || p[d] >= L[d]) return fail(h, PSTEP_ERR_RANGE, "position outside [0, L)");
      }
      if (u[i] - u[i] != 0.0 || v[i] - v[i] != 0.0 || w[i] - w[i] != 0.0 || t[i] - t[i] != 0.0)
        return fail(h, PSTEP_ERR_NONFINITE, "non-finite velocity or temperature");
    }
  }
  return PSTEP_OK;
}

int pstep_download_particles(pstep_handle h, double *x, double *y, double *z, double *u, double *v, double *w,
                             double *t, int32_t *flag, int on_device) {
  if (!h) return PSTEP_ERR_ARG;
  if (h->np > 0 && (!x || !y || !z || !u || !v || !w || !t || !flag)) return fail(h, PSTEP_ERR_ARG, "null array");
  double *dst[7] = {x, y, z, u, v, w, t};
  if (is_f32(h)) return pstep::f32_download(h, dst, flag, on_device);
  for (int q = 0; q < 7; ++q) TRY(pstep_get_particle_array(h, PSTEP_X + q, dst[q], on_device));
  return pstep_get_particle_array(h, PSTEP_FLAG, flag, on_device);
}

int pstep_set_tau_p(pstep_handle h, const double *tau, int on_device) {
  if (!h) return PSTEP_ERR_ARG;
  if (is_f32(h)) return f32_set_tau(h, tau, on_device);
  if (!tau) {
    dfree(h->s.itp);
    return PSTEP_OK;
  }
  if (!h->s.itp) TRY(dalloc(h, h->s.itp, (size_t)h->cap));
  if (h->np == 0) return PSTEP_OK;
  const double *src = tau;
  double *tmp = nullptr;
  if (!on_device) {
    TRY(dalloc(h, tmp, (size_t)h->np));
    PSTEP_CUDA(cudaMemcpyAsync(tmp, tau, sizeof(double) * h->np, cudaMemcpyHostToDevice, h->stream));
    src = tmp;
  }
  k_recip<<<blocks_for(h->np), kThreads, 0, h->stream>>>(src, h->np, h->s.itp);
  PSTEP_LAUNCHED(h);
  if (tmp) {
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    dfree(tmp);
  }
  if (h->primed) return fail(h, PSTEP_ERR_STATE, "tau_p must be set before pstep_prime");
  return PSTEP_OK;
}

int pstep_set_particle_props(pstep_handle h, const pstep_particle_props *props, int on_device) {
  if (!h || !props) return PSTEP_ERR_ARG;
  if (is_f32(h)) return f32_set_props(h, props, on_device);
  if (props->mass_ratio || props->itth || props->heat_is || props->alpha || props->accel[0] || props->accel[1] ||
      props->accel[2])
    return fail(h, PSTEP_ERR_CONFIG, "per-particle properties other than tau_p need the FP32 form");
  return pstep_set_tau_p(h, props->tau_p, on_device);
}

int pstep_set_correction(pstep_handle h, const pstep_correction *c) {
  if (!h) return PSTEP_ERR_ARG;
  if (!is_f32(h)) return c ? fail(h, PSTEP_ERR_CONFIG, "the learned correction needs the FP32 form") : PSTEP_OK;
  return f32_set_correction(h, c);
}

int pstep_bind_velocity(pstep_handle h, const double *ux, const double *uy, const double *uz, int on_device) {
  if (!h) return PSTEP_ERR_ARG;
  TRY(copy_field_in(h, ux, on_device, h->own_u[0], h->ux));
  TRY(copy_field_in(h, uy, on_device, h->own_u[1], h->uy));
  TRY(copy_field_in(h, uz, on_device, h->own_u[2], h->uz));
  h->fields_u++;
  if (is_f32(h)) TRY(f32_bind_fields(h, 1));
  return PSTEP_OK;
}

int pstep_bind_temperature(pstep_handle h, const double *t, int on_device) {
  if (!h) return PSTEP_ERR_ARG;
  TRY(copy_field_in(h, t, on_device, h->own_t, h->tf));
  h->fields_t++;
  if (is_f32(h)) TRY(f32_bind_fields(h, 2));
  return PSTEP_OK;
}

int pstep_prime(pstep_handle h) {
  if (!h) return PSTEP_ERR_ARG;
  if (!h->fields_t) return fail(h, PSTEP_ERR_STATE, "prime needs a bound temperature field");
  if (is_f32(h)) {
    TRY(f32_prime(h));
    h->primed = 1;
    return PSTEP_OK;
  }
  // grid.cpp:207-226: Tg and RHS_T at x_int = x, part2gas_Temp_int
  TRY(f64_prime_kernel(h));
  TRY(sort_by_node(h, h->s.key_new, h->csr_new));
  TRY(deposit_temperature(h, h->csr_new, h->s.frac_new, h->s.key_new));
  // the first stage deposits at x_int = x: the primed records become the stage's x_int records,
  // and storage is reordered by them
  for (int d = 0; d < 3; ++d) { double *t = h->s.frac_prev[d]; h->s.frac_prev[d] = h->s.frac_new[d]; h->s.frac_new[d] = t; }
  { uint32_t *t = h->s.key_prev; h->s.key_prev = h->s.key_new; h->s.key_new = t; }
  { Csr t = h->csr_prev; h->csr_prev = h->csr_new; h->csr_new = t; }
  TRY(f64_reorder(h));
  h->int_is_base = 1;
  h->np1_is_base = 1;
  h->primed = 1;
  h->phase = 0;
  return PSTEP_OK;
}

int pstep_stage_interp_advance_deposit(pstep_handle h, int k, double pre, double post) {
  if (!h) return PSTEP_ERR_ARG;
  if (k < 0 || k > 3) return fail(h, PSTEP_ERR_ARG, "stage index must be 0..3");
  if (!h->primed) return fail(h, PSTEP_ERR_STATE, "pstep_prime must run before the first stage");
  if (!h->fields_u || !h->fields_t) return fail(h, PSTEP_ERR_STATE, "fields are not bound");
  if (h->phase != 0) return fail(h, PSTEP_ERR_STATE, "previous stage not finished (pstep_end_stage)");
  if ((k == 0) != (h->int_is_base != 0)) return fail(h, PSTEP_ERR_STATE, "stage index out of sequence");
  h->cur_k = k;
  h->new_is_zero = 0;
  h->np1_is_base = 0;  // the stage writes *_np1
  if (is_f32(h)) {
    TRY(f32_stage(h, k, pre, post));
    h->phase = 1;
    return PSTEP_OK;
  }
  h->fields_t_at_advance = h->fields_t;
  if (k == 3) {  // the last stage gathers the step result's max u and max ug
    PSTEP_CUDA(cudaMemsetAsync(h->pmax64, 0, sizeof(unsigned long long) * 2 * 1024, h->stream));
    h->pmax64_state = 1;
  }
  prof_begin(h, PSTEP_PHASE_ADVANCE);
  TRY(f64_advance(h, k, pre, post));
  prof_end(h, PSTEP_PHASE_ADVANCE);
  prof_begin(h, PSTEP_PHASE_DEPOSIT_INT);
  TRY(f64_deposit_int(h));
  prof_end(h, PSTEP_PHASE_DEPOSIT_INT);
  h->phase = 1;
  return PSTEP_OK;
}

int pstep_wrap(pstep_handle h) {
  if (!h) return PSTEP_ERR_ARG;
  if (h->phase != 1) return fail(h, PSTEP_ERR_STATE, "wrap must follow interp_advance_deposit");
  if (!is_f32(h) && (h->cfg.flags & PSTEP_TRACK_ORDER)) {
    prof_begin(h, PSTEP_PHASE_ORDER);
    TRY(order_passes(h));
    prof_end(h, PSTEP_PHASE_ORDER);
  }
  h->phase = 2;
  return PSTEP_OK;
}

int pstep_stage_temp(pstep_handle h) {
  if (!h) return PSTEP_ERR_ARG;
  if (h->phase != 2) return fail(h, PSTEP_ERR_STATE, "stage_temp must follow wrap");
  if (!is_f32(h)) {
    // the fused advance kernel interpolated T with the field bound at that time; a
    // temperature bound since then (the reference forms it after Send_Recv,
    // grid.cpp:676) is interpolated here
    if (h->fields_t != h->fields_t_at_advance) TRY(f64_temp_gather(h));
    prof_begin(h, PSTEP_PHASE_SORT);
    TRY(sort_by_node(h, h->s.key_new, h->csr_new));
    prof_end(h, PSTEP_PHASE_SORT);
    prof_begin(h, PSTEP_PHASE_DEPOSIT_TEMP);
    TRY(deposit_temperature(h, h->csr_new, h->s.frac_new, h->s.key_new));
    prof_end(h, PSTEP_PHASE_DEPOSIT_TEMP);
  }
  h->phase = 3;
  return PSTEP_OK;
}

int pstep_stage(pstep_handle h, int k, double pre, double post) {
  TRY(pstep_stage_interp_advance_deposit(h, k, pre, post));
  TRY(pstep_wrap(h));
  return pstep_stage_temp(h);
}

int pstep_end_stage(pstep_handle h) {
  if (!h) return PSTEP_ERR_ARG;
  if (h->phase != 3) return fail(h, PSTEP_ERR_STATE, "end_stage must follow stage_temp");
  if (is_f32(h)) {
    TRY(f32_end_stage(h));
  } else {
    for (int q = 0; q < 7; ++q) { double *t = h->s.sint[q]; h->s.sint[q] = h->s.snew[q]; h->s.snew[q] = t; }
    for (int d = 0; d < 3; ++d) { double *t = h->s.frac_prev[d]; h->s.frac_prev[d] = h->s.frac_new[d]; h->s.frac_new[d] = t; }
    { uint32_t *t = h->s.key_prev; h->s.key_prev = h->s.key_new; h->s.key_new = t; }
    { Csr t = h->csr_prev; h->csr_prev = h->csr_new; h->csr_new = t; }
  }
  h->int_is_base = 0;
  h->np1_is_base = 0;
  h->phase = 0;
  h->stages_done++;
  return PSTEP_OK;
}

int pstep_end_step(pstep_handle h) {
  if (!h) return PSTEP_ERR_ARG;
  if (h->phase != 0 || h->cur_k != 3 || h->int_is_base) return fail(h, PSTEP_ERR_STATE, "end_step must follow stage 3");
  if (is_f32(h)) {
    TRY(f32_end_step(h));
  } else {
    // base = np1 (TimeAdvance); then reorder storage by the cell sort of these positions
    for (int q = 0; q < 7; ++q) { double *t = h->s.base[q]; h->s.base[q] = h->s.np1[q]; h->s.np1[q] = t; }
    h->pmax64_state = h->pmax64_state == 1 ? 2 : 0;  // the last stage's maxima describe the new base
    prof_begin(h, PSTEP_PHASE_REORDER);
    TRY(f64_reorder(h));
    prof_end(h, PSTEP_PHASE_REORDER);
  }
  h->int_is_base = 1;
  h->np1_is_base = 1;
  return PSTEP_OK;
}

int pstep_run(pstep_handle h, int nsteps) {
  if (!h) return PSTEP_ERR_ARG;
  if (nsteps < 0) return fail(h, PSTEP_ERR_ARG, "negative step count");
  PSTEP_CUDA(cudaEventRecord(h->ev0, h->stream));
  for (int s = 0; s < nsteps; ++s) {
    for (int k = 0; k < 4; ++k) {
      TRY(pstep_stage(h, k, kPre[k], kPost[k]));
      TRY(pstep_end_stage(h));
    }
    TRY(pstep_end_step(h));
  }
  PSTEP_CUDA(cudaEventRecord(h->ev1, h->stream));
  h->timed = 1;
  return PSTEP_OK;
}

int pstep_profile(pstep_handle h, int enable) {
  if (!h) return PSTEP_ERR_ARG;
  if (!h->prof) h->prof = new (std::nothrow) Prof();
  if (!h->prof) return PSTEP_ERR_NOMEM;
  h->prof->enabled = enable ? 1 : 0;
  return PSTEP_OK;
}

int pstep_profile_read(pstep_handle h, double *ms, int64_t *counts, int nphases) {
  if (!h || nphases < 0) return PSTEP_ERR_ARG;
  Prof *p = h->prof;
  if (p) {
    PSTEP_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i + 1 < p->used && i / 2 < p->phase.size(); i += 2) {
      float f = 0;
      PSTEP_CUDA(cudaEventElapsedTime(&f, p->pool[i], p->pool[i + 1]));
      int ph = p->phase[i / 2];
      p->ms[ph] += f;
      p->count[ph] += 1;
    }
    p->used = 0;
    p->phase.clear();
  }
  for (int q = 0; q < nphases && q < PSTEP_NUM_PHASES; ++q) {
    if (ms) ms[q] = p ? p->ms[q] : 0.0;
    if (counts) counts[q] = p ? p->count[q] : 0;
  }
  if (p) {
    for (int q = 0; q < PSTEP_NUM_PHASES; ++q) { p->ms[q] = 0; p->count[q] = 0; }
  }
  return PSTEP_OK;
}

int pstep_last_run_ms(pstep_handle h, double *ms) {
  if (!h || !ms) return PSTEP_ERR_ARG;
  if (!h->timed) return fail(h, PSTEP_ERR_STATE, "no timed run");
  PSTEP_CUDA(cudaEventSynchronize(h->ev1));
  float f = 0;
  PSTEP_CUDA(cudaEventElapsedTime(&f, h->ev0, h->ev1));
  *ms = f;
  return PSTEP_OK;
}

int pstep_get_field(pstep_handle h, int id, double *dst, int on_device) {
  if (!h || !dst || id < 0 || id >= PSTEP_NUM_FIELDS) return PSTEP_ERR_ARG;
  PSTEP_CUDA(cudaMemcpyAsync(dst, h->dep[id], sizeof(double) * h->geom.gsize, kind_out(on_device), h->stream));
  if (!on_device) PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  return PSTEP_OK;
}

int pstep_energy_mean(pstep_handle h, double *out) {
  if (!h || !out) return PSTEP_ERR_ARG;
  PSTEP_CUDA(cudaMemcpyAsync(&h->emean_host, h->emean_dev, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  *out = h->emean_host;
  return PSTEP_OK;
}

int pstep_set_wait_limit(pstep_handle h, uint32_t polls, int idle_first) {
  if (!h) return PSTEP_ERR_ARG;
  h->wait_limit = polls;
  h->wait_idle = idle_first ? 1 : 0;
  return PSTEP_OK;
}

int pstep_momentum_sums(pstep_handle h, double *out) {
  if (!h || !out) return PSTEP_ERR_ARG;
  PSTEP_CUDA(cudaMemcpyAsync(h->mom_host, h->mom_dev, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  for (int d = 0; d < 3; ++d) out[d] = h->mom_host[d];
  return PSTEP_OK;
}

int pstep_get_particle_array(pstep_handle h, int id, void *dst, int on_device) {
  if (!h || !dst || id < 0 || id >= PSTEP_NUM_ARRAYS) return PSTEP_ERR_ARG;
  const int64_t n = h->np;
  if (n == 0) return PSTEP_OK;
  if (is_f32(h) && id != PSTEP_FLAG) return f32_get_array(h, id, dst, on_device);
  if (id >= PSTEP_UG) return fail(h, PSTEP_ERR_CONFIG, "gas values per particle are kept by the FP32 form");
  const int32_t *perm = (h->cfg.flags & PSTEP_TRACK_ORDER) ? h->phys_of_ref : nullptr;
  if (id == PSTEP_FLAG) {
    int32_t *tmp = (int32_t *)h->perm_tmp;
    k_gather_ref_i<<<blocks_for(n), kThreads, 0, h->stream>>>(h->s.flag, perm, n, tmp);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaMemcpyAsync(dst, tmp, sizeof(int32_t) * n, kind_out(on_device), h->stream));
  } else {
    const double *src = nullptr;
    if (id <= PSTEP_T) {
      src = h->s.base[id - PSTEP_X];
    } else if (id <= PSTEP_T_INT) {
      int q = id - PSTEP_X_INT;
      // during stage 0 the unshifted *_int positions are in sint (the base may be wrapped)
      src = (h->int_is_base && !(q < 3 && h->phase != 0)) ? h->s.base[q] : h->s.sint[q];
    } else if (id <= PSTEP_T_NEW) {
      int q = id - PSTEP_X_NEW;
      if (h->new_is_zero) {
        PSTEP_CUDA(cudaMemsetAsync(h->perm_tmp, 0, sizeof(double) * n, h->stream));
        PSTEP_CUDA(cudaMemcpyAsync(dst, h->perm_tmp, sizeof(double) * n, kind_out(on_device), h->stream));
        if (!on_device) PSTEP_CUDA(cudaStreamSynchronize(h->stream));
        return PSTEP_OK;
      }
      // within a stage: the new values; after end_stage the reference's *_new equal *_int;
      // at the start of a step, the base
      if (h->phase != 0) src = h->s.snew[q];
      else src = h->int_is_base ? h->s.base[q] : h->s.sint[q];
    } else if (id <= PSTEP_T_NP1) {
      int q = id - PSTEP_X_NP1;
      src = h->np1_is_base ? h->s.base[q] : h->s.np1[q];
    } else {
      src = h->s.rhs_t;
    }
    double *tmp = (double *)h->perm_tmp;
    k_gather_ref<<<blocks_for(n), kThreads, 0, h->stream>>>(src, perm, n, tmp);
    PSTEP_LAUNCHED(h);
    PSTEP_CUDA(cudaMemcpyAsync(dst, tmp, sizeof(double) * n, kind_out(on_device), h->stream));
  }
  if (!on_device) PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  return PSTEP_OK;
}

int pstep_check(pstep_handle h, int32_t *flags_out) {
  if (!h) return PSTEP_ERR_ARG;
  int32_t w = 0;
  PSTEP_CUDA(cudaMemcpyAsync(&w, h->err_word, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  PSTEP_CUDA(cudaMemsetAsync(h->err_word, 0, sizeof(int32_t), h->stream));
  PSTEP_CUDA(cudaStreamSynchronize(h->stream));
  if (flags_out) *flags_out = w;
  if (w & kErrNonFinite) return PSTEP_ERR_NONFINITE;
  if (w & kErrRange) return PSTEP_ERR_RANGE;
  if (w & kErrMove) return PSTEP_ERR_MOVE;
  if (w & kErrTimeout) return PSTEP_ERR_TIMEOUT;
  if (w & kErrCapacity) return PSTEP_ERR_CAPACITY;
  return PSTEP_OK;
}

}  // extern "C"
