// Drop-in replacement for the reference solver's particle.cpp: every method of
// `class particle` (particle.h, unchanged) forwards to the GB300 C ABI in
// include/pstep.h. Build it in place of particle.cpp and link libpstep.so.
//
// The particle state lives on the GPU. The public vectors of `particle` are
// synchronised lazily:
//  - host -> device once, at the first gas2part_Temp_int (grid::Initialize
//    fills x, u, T, flag and copies *_int / *_np1 just before, grid.cpp:207-226);
//  - device -> host when the reference reads them element by element. The
//    statistics (NP_TOT, max, Balance_Index, trajectory) and Store_All run on
//    the device state directly (pstep_np_tot, pstep_max, pstep_balance_index,
//    pstep_find_tags, pstep_store_all) without a download. The interpolation
//    work arrays ug, vg, wg, Tg and RHS_u/v/w are internal to the device step
//    and are not synchronised.
// grid::TimeAdvance_RK4 and grid::TimeAdvance copy the public vectors
// (grid.cpp:705-712, 315-325); on the device these copies happen when the next
// stage starts (the next gas2part_velocity), inferred from the stage index.
//
// Call mapping (particle.h method -> C ABI):
//   gas2part_velocity(U)        close the previous stage/step; bind U
//   update_position(k,pre,post) remembered (update_velocity/update_Temp fused)
//   part2gas_concentration(C)   pstep_stage_interp_advance_deposit, copy C
//   part2gas_velocity(A)        copy RHS_RU.x/y/z
//   Send_Recv()                 pstep_wrap
//   gas2part_Temp_new(T)        bind T
//   part2gas_Temp_new(A)        pstep_stage_temp, copy RHS_Part_Temp
//   gas2part_Temp_int(T) ... part2gas_Temp_int(A)   upload + pstep_prime
// Single rank per device: the MPI exchange of Send_Recv becomes the periodic
// wrap on the device (the reference's particle order is kept).
#include "particle.h"
#include "gridsize.h"
#include "params.h"
#include "proc.h"
#include "tensor0.h"
#include "tensor1.h"
#include "mpi.h"
#include "pstep.h"

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <map>
#include <sstream>
#include <string>

namespace {

struct GpuState {
  pstep_handle h = nullptr;
  int k = -1;  // stage of the last update_position call
  double pre = 0, post = 0;
  int stage_open = 0;  // a stage ran to part2gas_Temp_new and was not closed yet
  int uploaded = 0;
  int host_stale = 0;  // host vectors older than the device state
};

std::map<const particle *, GpuState> &states() {
  static std::map<const particle *, GpuState> m;
  return m;
}

GpuState &state(const particle *p) { return states()[p]; }

void check(pstep_handle h, int rc, const char *what) {
  if (rc != PSTEP_OK) {
    std::cerr << "pstep: " << what << " failed: " << pstep_status_string(rc) << " ("
              << (h ? pstep_last_error(h) : "") << ")" << std::endl;
    std::abort();
  }
}

void unsupported(const char *what) {
  std::cerr << "pstep: " << what << " is not part of the GPU particle step" << std::endl;
  std::abort();
}

pstep_config make_config(params *p, gridsize *s, int64_t capacity) {
  pstep_config c = {};
  c.nx = p->Nx_tot();
  c.ny = p->Ny_tot();
  c.nz = p->Nz_tot();
  c.bs = s->bs();
  c.twc = p->TWC() ? 1 : 0;
  c.particle_gravity = p->ParticleGravity() ? 1 : 0;
  c.precision = PSTEP_FP64;
  c.flags = PSTEP_TRACK_ORDER;
  c.capacity = capacity;
  c.lx = p->Lx();
  c.ly = p->Ly();
  c.lz = p->Lz();
  c.dt = p->dt();
  c.tp = p->Tp();
  c.mp = p->mp();
  c.dp = p->Dp();
  c.nu = p->Nu();
  c.k = p->k();
  c.epsilonp = p->epsilonp();
  c.i0 = p->I0();
  c.cvp = p->Cvp();
  c.gx = p->gx();
  c.gy = p->gy();
  c.gz = p->gz();
  return c;
}

void resize_all(particle *q, int n) {
  std::vector<double> *v[] = {&q->x, &q->x_int, &q->x_new, &q->x_np1, &q->y, &q->y_int, &q->y_new, &q->y_np1,
                              &q->z, &q->z_int, &q->z_new, &q->z_np1, &q->u, &q->u_int, &q->u_new, &q->u_np1,
                              &q->v, &q->v_int, &q->v_new, &q->v_np1, &q->w, &q->w_int, &q->w_new, &q->w_np1,
                              &q->T, &q->T_int, &q->T_new, &q->T_np1, &q->RHS_u, &q->RHS_v, &q->RHS_w,
                              &q->RHS_T, &q->ug, &q->vg, &q->wg, &q->Tg};
  for (auto *a : v) a->resize(n);
  q->flag.resize(n);
}

// host vectors <- device, in the reference's order
void pull(particle *q) {
  GpuState &g = state(q);
  if (!g.host_stale) return;
  const int64_t n = pstep_num_particles(g.h);
  q->Np = (int)n;
  resize_all(q, q->Np);
  struct { int id; std::vector<double> *v; } m[] = {
      {PSTEP_X, &q->x}, {PSTEP_Y, &q->y}, {PSTEP_Z, &q->z}, {PSTEP_U, &q->u}, {PSTEP_V, &q->v},
      {PSTEP_W, &q->w}, {PSTEP_T, &q->T}, {PSTEP_X_INT, &q->x_int}, {PSTEP_Y_INT, &q->y_int},
      {PSTEP_Z_INT, &q->z_int}, {PSTEP_U_INT, &q->u_int}, {PSTEP_V_INT, &q->v_int}, {PSTEP_W_INT, &q->w_int},
      {PSTEP_T_INT, &q->T_int}, {PSTEP_X_NEW, &q->x_new}, {PSTEP_Y_NEW, &q->y_new}, {PSTEP_Z_NEW, &q->z_new},
      {PSTEP_U_NEW, &q->u_new}, {PSTEP_V_NEW, &q->v_new}, {PSTEP_W_NEW, &q->w_new}, {PSTEP_T_NEW, &q->T_new},
      {PSTEP_X_NP1, &q->x_np1}, {PSTEP_Y_NP1, &q->y_np1}, {PSTEP_Z_NP1, &q->z_np1}, {PSTEP_U_NP1, &q->u_np1},
      {PSTEP_V_NP1, &q->v_np1}, {PSTEP_W_NP1, &q->w_np1}, {PSTEP_T_NP1, &q->T_np1}, {PSTEP_RHS_T, &q->RHS_T}};
  if (n > 0) {
    for (auto &e : m) check(g.h, pstep_get_particle_array(g.h, e.id, e.v->data(), 0), "download");
    check(g.h, pstep_get_particle_array(g.h, PSTEP_FLAG, q->flag.data(), 0), "download flag");
  }
  g.host_stale = 0;
}

// grid::TimeAdvance_RK4 / TimeAdvance happened since the last stage: apply them on the device
void close_stage(GpuState &g) {
  if (!g.stage_open) return;
  check(g.h, pstep_end_stage(g.h), "end_stage");
  if (g.k == 3) check(g.h, pstep_end_step(g.h), "end_step");
  g.stage_open = 0;
}

}  // namespace

particle::particle(params *p, proc *pc, gridsize *s) {
  param_ = p;
  pc_ = pc;
  size_ = s;
  idx = 1. / size_->dx();
  idy = 1. / size_->dy();
  idz = 1. / size_->dz();
  OFF_SET = 0;
  // the MPI migration buffers are not used on one device; keep them valid and small
  Buffer_max_size = 29;
  Sbuf0 = new double[Buffer_max_size];
  Sbuf1 = new double[Buffer_max_size];
  Rbuf0 = new double[Buffer_max_size];
  Rbuf1 = new double[Buffer_max_size];
  Snum0 = Snum1 = Rnum0 = Rnum1 = 0;
  Np = 0;
  Nps = nullptr;
  if (pc_->TOT() != 1) unsupported("more than one MPI rank per particle population");
  if (pc_->IsRoot()) {
    Nps = new int[pc_->TOT()];
    if (param_->Statistics()) {
      std::ostringstream fn;
      fn << param_->stat_dir() << "Part_trajectory" << ".dat";
      stat_trajectory.open(fn.str().c_str(), std::ios::out | std::ios::app);
    }
  }
  GpuState &g = state(this);
  const int64_t capacity = (int64_t)param_->N0() + 64;
  pstep_config c = make_config(param_, size_, capacity);
  check(nullptr, pstep_create(&c, &g.h), "pstep_create");
}

particle::~particle() {
  delete[] Sbuf0;
  delete[] Sbuf1;
  delete[] Rbuf0;
  delete[] Rbuf1;
  delete[] Nps;
  if (pc_->IsRoot() && param_->Statistics()) stat_trajectory.close();
  auto it = states().find(this);
  if (it != states().end()) {
    pstep_destroy(it->second.h);
    states().erase(it);
  }
}

void particle::RESIZE() { resize_all(this, Np); }

// ---- prime (grid.cpp:223-226) ----
void particle::gas2part_Temp_int(tensor0 &Tf) {
  GpuState &g = state(this);
  if (!g.uploaded) {
    Np = (int)x.size();
    check(g.h, pstep_upload_particles(g.h, Np, x.data(), y.data(), z.data(), u.data(), v.data(), w.data(), T.data(),
                                      flag.data(), 0), "upload");
    g.uploaded = 1;
  }
  check(g.h, pstep_bind_temperature(g.h, Tf.pointer(), 0), "bind T");
}
void particle::Compute_RHS_Temp_int() {}
void particle::part2gas_Temp_int(tensor0 &A) {
  GpuState &g = state(this);
  check(g.h, pstep_prime(g.h), "prime");
  check(g.h, pstep_get_field(g.h, PSTEP_FIELD_PART_TEMP, A.pointer(), 0), "RHS_Part_Temp");
  g.host_stale = 1;
}

// ---- one RK4 stage (grid.cpp:659-680) ----
void particle::gas2part_velocity(tensor1 &U) {
  GpuState &g = state(this);
  close_stage(g);
  pstep_config c = make_config(param_, size_, (int64_t)param_->N0() + 64);  // params::update may have switched I0, g
  check(g.h, pstep_update_params(g.h, &c), "update params");
  check(g.h, pstep_bind_velocity(g.h, U.x.pointer(), U.y.pointer(), U.z.pointer(), 0), "bind U");
}
void particle::update_position(int k, double pre, double post) {
  GpuState &g = state(this);
  g.k = k;
  g.pre = pre;
  g.post = post;
}
void particle::update_velocity(int, double, double) {}
void particle::update_Temp(int, double, double) {}
void particle::part2gas_concentration(tensor0 &A) {
  GpuState &g = state(this);
  check(g.h, pstep_stage_interp_advance_deposit(g.h, g.k, g.pre, g.post), "interp/advance/deposit");
  check(g.h, pstep_get_field(g.h, PSTEP_FIELD_C, A.pointer(), 0), "C");
  g.host_stale = 1;
}
void particle::part2gas_velocity(tensor1 &A) {
  GpuState &g = state(this);
  check(g.h, pstep_get_field(g.h, PSTEP_FIELD_RU_X, A.x.pointer(), 0), "RHS_RU.x");
  check(g.h, pstep_get_field(g.h, PSTEP_FIELD_RU_Y, A.y.pointer(), 0), "RHS_RU.y");
  check(g.h, pstep_get_field(g.h, PSTEP_FIELD_RU_Z, A.z.pointer(), 0), "RHS_RU.z");
}
void particle::Send_Recv() {
  GpuState &g = state(this);
  check(g.h, pstep_wrap(g.h), "wrap");
}
void particle::gas2part_Temp_new(tensor0 &Tf) {
  GpuState &g = state(this);
  check(g.h, pstep_bind_temperature(g.h, Tf.pointer(), 0), "bind T");
}
void particle::Compute_RHS_Temp_new() {}
void particle::part2gas_Temp_new(tensor0 &A) {
  GpuState &g = state(this);
  check(g.h, pstep_stage_temp(g.h), "stage_temp");
  check(g.h, pstep_get_field(g.h, PSTEP_FIELD_PART_TEMP, A.pointer(), 0), "RHS_Part_Temp");
  g.stage_open = 1;
  g.host_stale = 1;
}

// ---- statistics and storage ----
// particle.cpp:662-669
int particle::NP_TOT() {
  GpuState &g = state(this);
  if (!g.uploaded) return Np;
  int64_t n = 0;
  check(g.h, pstep_np_tot(g.h, &n), "np_tot");
  return (int)n;
}

// the device array a public vector of the reference stands for, or -1
static int array_id(const particle *q, const std::vector<double> *v) {
  const std::vector<double> *m[] = {&q->x, &q->y, &q->z, &q->u, &q->v, &q->w, &q->T};
  for (int i = 0; i < 7; ++i)
    if (m[i] == v) return PSTEP_X + i;
  if (v == &q->RHS_T) return PSTEP_RHS_T;
  if (v == &q->ug) return PSTEP_UG;
  if (v == &q->vg) return PSTEP_VG;
  if (v == &q->wg) return PSTEP_WG;
  if (v == &q->Tg) return PSTEP_TG;
  return -1;
}

// particle.cpp:671-685: on the device when the vector is one the device keeps
double particle::max(std::vector<double> &V) {
  GpuState &g = state(this);
  const int id = array_id(this, &V);
  double m = 0;
  if (g.uploaded && id >= 0 && pstep_max(g.h, id, &m) == PSTEP_OK) return m;
  pull(this);
  if (Np == 0) return -1e9;
  m = V[0];
  for (int i = 1; i < Np; ++i)
    if (V[i] > m) m = V[i];
  return m;
}

// particle.cpp:730-741
double particle::Balance_Index() {
  GpuState &g = state(this);
  if (!g.uploaded) return (double)Np / (double)Np;
  double b = 0;
  check(g.h, pstep_balance_index(g.h, &b), "balance_index");
  return b;
}

bool particle::find_tag(int tag, double &xx, double &yy, double &zz) {
  GpuState &g = state(this);
  if (g.uploaded) {
    double xyz[3];
    int32_t found = 0;
    const int32_t t = tag;
    check(g.h, pstep_find_tags(g.h, &t, 1, xyz, &found), "find_tag");
    if (found) { xx = xyz[0]; yy = xyz[1]; zz = xyz[2]; }
    return found != 0;
  }
  for (int i = 0; i < Np; ++i)
    if (flag[i] == tag) {
      xx = x[i];
      yy = y[i];
      zz = z[i];
      return true;
    }
  return false;
}

// particle.cpp:687-719 for one rank: every tracked id located in one device pass
void particle::trajectory(double t) {
  if (param_->Np_track() == 0) return;
  const int K = (param_->N0() + param_->Np_track() - 1) / param_->Np_track();
  std::vector<int32_t> ids;
  for (int i = 0; i < param_->N0(); i += K) ids.push_back(i);
  std::vector<double> xyz(3 * ids.size());
  std::vector<int32_t> found(ids.size(), 0);
  GpuState &g = state(this);
  if (g.uploaded) {
    check(g.h, pstep_find_tags(g.h, ids.data(), (int32_t)ids.size(), xyz.data(), found.data()), "trajectory");
  } else {
    for (size_t q = 0; q < ids.size(); ++q)
      found[q] = find_tag(ids[q], xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]);
  }
  stat_trajectory << t << " ";
  for (size_t q = 0; q < ids.size(); ++q)
    if (found[q]) stat_trajectory << xyz[3 * q] << " " << xyz[3 * q + 1] << " " << xyz[3 * q + 2] << " ";
  stat_trajectory << std::endl;
}

void particle::Store(char *name, int num_ts, double *p) {
  std::ostringstream fn;
  fn << param_->data_dir() << name << "_" << num_ts << ".bin";
  FILE *f = fopen(fn.str().c_str(), "wbx");  // MPI_MODE_EXCL
  if (!f) {
    std::cerr << "pstep: cannot create " << fn.str() << " (Store_All never overwrites a file)" << std::endl;
    std::abort();
  }
  fwrite(p, sizeof(double), (size_t)Np, f);
  fclose(f);
}

void particle::Store(char *name, int num_ts, int *p) {
  std::ostringstream fn;
  fn << param_->data_dir() << name << "_" << num_ts << ".bin";
  FILE *f = fopen(fn.str().c_str(), "wbx");  // MPI_MODE_EXCL
  if (!f) {
    std::cerr << "pstep: cannot create " << fn.str() << " (Store_All never overwrites a file)" << std::endl;
    std::abort();
  }
  fwrite(p, sizeof(int), (size_t)Np, f);
  fclose(f);
}

// particle.cpp:867-890: straight from the device state once it lives there
void particle::Store_All(int num_ts) {
  GpuState &g = state(this);
  if (g.uploaded) {
    check(g.h, pstep_store_all(g.h, param_->data_dir().c_str(), num_ts), "store_all");
    return;
  }
  Store((char *)"Part_x", num_ts, x.data());
  Store((char *)"Part_y", num_ts, y.data());
  Store((char *)"Part_z", num_ts, z.data());
  Store((char *)"Part_u", num_ts, u.data());
  Store((char *)"Part_v", num_ts, v.data());
  Store((char *)"Part_w", num_ts, w.data());
  Store((char *)"Part_T", num_ts, T.data());
  Store((char *)"Part_flag", num_ts, flag.data());
}

// ---- initial particles (host, before the upload) ----
// load_random restates particle.cpp:919-958 for one rank: the same rand() sequence.
void particle::load_random() {
  const double U0 = param_->U0(), T0 = param_->T0();
  Np = param_->N0();
  int flag_number = 0;
  for (int i = 0; i < Np; ++i) {
    double r = ((double)(rand()) / (double)(RAND_MAX)) * (size_->xh() - size_->xl()) + size_->xl();
    x.push_back(r);
    u.push_back(U0);
    r = ((double)(rand()) / (double)(RAND_MAX)) * (size_->yh() - size_->yl()) + size_->yl();
    y.push_back(r);
    v.push_back(0);
    r = ((double)(rand()) / (double)(RAND_MAX)) * (size_->zh() - size_->zl()) + size_->zl();
    z.push_back(r);
    w.push_back(0);
    T.push_back(T0);
    flag.push_back(flag_number++);
  }
  RESIZE();
}

void particle::Load(char *name, double *p) {
  std::ostringstream fn;
  fn << "Restart_" << name << ".bin";
  FILE *f = fopen(fn.str().c_str(), "rb");
  if (!f || fread(p, sizeof(double), (size_t)Np, f) != (size_t)Np) unsupported("reading a restart file");
  fclose(f);
}

void particle::Load(char *name, int *p) {
  std::ostringstream fn;
  fn << "Restart_" << name << ".bin";
  FILE *f = fopen(fn.str().c_str(), "rb");
  if (!f || fread(p, sizeof(int), (size_t)Np, f) != (size_t)Np) unsupported("reading a restart file");
  fclose(f);
}

// particle.cpp:961-999 for one rank (no redistribution needed)
void particle::Load_All() {
  Np = param_->N0();
  RESIZE();
  const bool box = param_->IsBox();
  Load((char *)(box ? "Part_x" : "Part_x_IO"), x.data());
  Load((char *)(box ? "Part_y" : "Part_y_IO"), y.data());
  Load((char *)(box ? "Part_z" : "Part_z_IO"), z.data());
  Load((char *)(box ? "Part_u" : "Part_u_IO"), u.data());
  Load((char *)(box ? "Part_v" : "Part_v_IO"), v.data());
  Load((char *)(box ? "Part_w" : "Part_w_IO"), w.data());
  Load((char *)(box ? "Part_T" : "Part_T_IO"), T.data());
  Load((char *)(box ? "Part_flag" : "Part_flag_IO"), flag.data());
  x_new = x;
  y_new = y;
  z_new = z;
}

// ---- outside the GPU particle step ----
void particle::part2gas_concentration2(tensor0 &) { unsupported("part2gas_concentration2 (count deposit)"); }
void particle::Send_Recv(particle &) { unsupported("the inflow/outflow duct hand-off"); }
