// Harness that runs the REFERENCE solver's own box gas step (its grid.cpp, with
// particle.cpp, tensor0/1.cpp, communicator.cpp, gridsize.cpp, proc.cpp and
// params.cpp, compiled from source with the single-rank MPI stub and the
// Poisson stand-in in oracle/poisson_stub) from given initial fields and
// particles. TEST INFRASTRUCTURE ONLY: the checker of oracle/gas_oracle.c.
//
// Replayed (reference file:line): grid::Initialize's tail with the given
// fields (grid.cpp:194-226), then per step the box part of simulation.cpp:38-66
// (4 x Update_Rho, Update_P0, Update_Particle, Update_RU_WOP, Compute_Div_U_new,
// Compute_RHS_Pois, Solve_Poisson, Update_RU_WP, TimeAdvance_RK4; then
// Correct_mean_RU, TimeAdvance).
//
// usage: gas_harness params.in input.bin output.bin nsteps
// input:  int64 np, int32 n, double P0, RU.x RU.y RU.z Rho (n^3 each, i fastest),
//         particles x y z u v w T (np each), int32 flag (np)
// output: one record per step: int32 step, int32 np, ghosted RU.x RU.y RU.z Rho P T
//         RHS_Part_Temp C RHS_RU.x RHS_RU.y RHS_RU.z ((n+2)^3 each), double P0,
//         int32 Poisson iterations, particles x y z u v w T (np each), int32 flag (np)
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "mpi.h"
#include "params.h"
#include "proc.h"
#include "gridsize.h"
#include "communicator.h"
#include "tensor0.h"
#include "tensor1.h"
#include "grid.h"

static void die(const char *m) {
  fprintf(stderr, "gas_harness: %s\n", m);
  exit(2);
}

static void read_exact(FILE *f, void *p, size_t n) {
  if (n && fread(p, 1, n, f) != n) die("short read");
}

static void fill_interior(tensor0 &t, const double *src, int N) {
  const int G = N + 2;
  double *p = t.pointer();
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i)
        p[(size_t)(k + 1) * G * G + (size_t)(j + 1) * G + (i + 1)] = src[(size_t)k * N * N + (size_t)j * N + i];
  t.Update_Ghosts();
}

int main(int argc, char **argv) {
  if (argc < 5) die("usage: gas_harness params.in input.bin output.bin nsteps");
  const int nsteps = atoi(argv[4]);
  MPI_Init(&argc, &argv);
  params P(argv[1]);
  proc PC;
  gridsize S(&P, &PC);
  communicator COM(&S, &P, &PC);
  const int N = P.Nx_tot();
  if (P.Ny_tot() != N || P.Nz_tot() != N || P.bs() != 1 || !P.IsBox()) die("harness expects a cubic periodic box, bs=1");
  grid g(&S, &P, &PC, &COM);

  FILE *in = fopen(argv[2], "rb");
  if (!in) die("cannot open input");
  int64_t np64 = 0;
  int32_t nn = 0;
  double p0 = 0;
  read_exact(in, &np64, sizeof np64);
  read_exact(in, &nn, sizeof nn);
  read_exact(in, &p0, sizeof p0);
  if (nn != N) die("input grid size does not match params");
  const size_t N3 = (size_t)N * N * N;
  std::vector<double> buf(N3);
  tensor0 *dst[4] = {&g.RU.x, &g.RU.y, &g.RU.z, &g.Rho};
  for (int q = 0; q < 4; ++q) {
    read_exact(in, buf.data(), N3 * 8);
    fill_interior(*dst[q], buf.data(), N);
  }
  particle &part = g.part;
  const int n = (int)np64;
  part.Np = n;
  std::vector<double> *pv[7] = {&part.x, &part.y, &part.z, &part.u, &part.v, &part.w, &part.T};
  for (int a = 0; a < 7; ++a) {
    pv[a]->resize(n);
    read_exact(in, pv[a]->data(), (size_t)n * 8);
  }
  part.flag.resize(n);
  read_exact(in, part.flag.data(), (size_t)n * 4);
  fclose(in);
  // size every work vector (RESIZE, particle.cpp:136-148, only reserves wg and Tg)
  std::vector<double> *work[] = {&part.x_int, &part.y_int, &part.z_int, &part.x_new, &part.y_new, &part.z_new,
                                 &part.x_np1, &part.y_np1, &part.z_np1, &part.u_int, &part.v_int, &part.w_int,
                                 &part.u_new, &part.v_new, &part.w_new, &part.u_np1, &part.v_np1, &part.w_np1,
                                 &part.T_int, &part.T_new, &part.T_np1, &part.RHS_u, &part.RHS_v, &part.RHS_w,
                                 &part.RHS_T, &part.ug, &part.vg, &part.wg, &part.Tg};
  for (auto *w : work) w->assign(n, 0.0);

  // grid.cpp:194-226 with the given fields
  g.P = 0;
  g.P0 = p0;
  g.T_cur = 0;
  g.num_timestep = 0;
  g.RU_int = g.RU;
  g.RU_np1 = g.RU;
  g.Rho_int = g.Rho;
  g.Rho_np1 = g.Rho;
  g.P0_int = g.P0;
  g.P0_np1 = g.P0;
  g.Rho_face.Equal_I_C2F(g.Rho);
  part.x_int = part.x; part.y_int = part.y; part.z_int = part.z;
  part.u_int = part.u; part.v_int = part.v; part.w_int = part.w; part.T_int = part.T;
  part.x_np1 = part.x; part.y_np1 = part.y; part.z_np1 = part.z;
  part.u_np1 = part.u; part.v_np1 = part.v; part.w_np1 = part.w; part.T_np1 = part.T;
  g.T.Equal_Divide(g.P0_int / P.R(), g.Rho_int);
  part.gas2part_Temp_int(g.T);
  part.Compute_RHS_Temp_int();
  part.part2gas_Temp_int(g.RHS_Part_Temp);
  g.U.Equal_Divide(g.RU, g.Rho_face);

  FILE *out = fopen(argv[3], "wb");
  if (!out) die("cannot open output");
  const size_t G3 = (size_t)(N + 2) * (N + 2) * (N + 2);
  for (int s = 0; s < nsteps; ++s) {
    for (g.RK4_count = 0; g.RK4_count < 4; g.RK4_count++) {
      g.Update_Rho();
      g.Update_P0();
      g.Update_Particle();
      g.Update_RU_WOP();
      g.Compute_Div_U_new();
      g.Compute_RHS_Pois();
      g.Solve_Poisson();
      g.Update_RU_WP();
      g.TimeAdvance_RK4();
    }
    g.Correct_mean_RU();
    g.TimeAdvance();
    int32_t hdr[2] = {s, part.Np};
    fwrite(hdr, sizeof(int32_t), 2, out);
    tensor0 *fs[11] = {&g.RU.x, &g.RU.y, &g.RU.z, &g.Rho, &g.P, &g.T, &g.RHS_Part_Temp, &g.C,
                       &g.RHS_RU.x, &g.RHS_RU.y, &g.RHS_RU.z};
    for (auto *f : fs) fwrite(f->pointer(), sizeof(double), G3, out);
    fwrite(&g.P0, sizeof(double), 1, out);
    int32_t its = 0;  // the stand-in's iteration count is private; recorded as 0
    fwrite(&its, sizeof(int32_t), 1, out);
    for (int a = 0; a < 7; ++a)
      if (part.Np) fwrite(pv[a]->data(), sizeof(double), (size_t)part.Np, out);
    if (part.Np) fwrite(part.flag.data(), sizeof(int), (size_t)part.Np, out);
  }
  fclose(out);
  MPI_Finalize();
  return 0;
}
