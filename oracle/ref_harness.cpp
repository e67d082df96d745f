// Harness that runs the REFERENCE solver's own particle step (its particle.cpp,
// tensor0/1.cpp, communicator.cpp, gridsize.cpp, proc.cpp, params.cpp compiled
// from source with the single-rank MPI stub in oracle/mpi_stub) on fixed gas
// fields. Test infrastructure only: it is the checker for oracle/pstep_oracle.c
// and the source of the golden fixtures; the product never links it.
//
// Call order replayed (reference file:line):
//   prime    grid.cpp:207-226  (x_int=x_np1=x ..., gas2part_Temp_int,
//                               Compute_RHS_Temp_int, part2gas_Temp_int)
//   stage k  grid.cpp:659-680  (gas2part_velocity, update_position/velocity/
//                               Temp, part2gas_concentration, part2gas_velocity
//                               or RHS_RU=0, Send_Recv, gas2part_Temp_new,
//                               Compute_RHS_Temp_new, part2gas_Temp_new)
//   between  grid.cpp:705-712  (TimeAdvance_RK4: *_int = *_new)
//   step end grid.cpp:315-325  (TimeAdvance: x = x_np1 ...)
//   energy   grid.cpp:541      (mean_energy_transferred = RHS_Part_Temp.mean())
// RK4 coefficients as grid.cpp:16-23.
//
// The fields are held fixed: U and T are given directly (the caller's
// Equal_Divide forming, grid.cpp:662 and :676, is outside the step).
//
// Optional, for the snapshot files and the statistics (particle.cpp:662-741, 867-1025):
//   load     1: the particles come from the reference's Load_All (Restart_Part_*.bin in
//            the working directory, N0 from params) instead of input.bin
//   store_ts >= 0: after the run, Store_All(store_ts) (Part_*_<store_ts>.bin under the
//            params data directory), trajectory(nsteps) when params track particles
//            (Part_trajectory.dat under the statistics directory: the positions of ids
//            0, K, 2K, ... through find_tag) and one line "STATS {json}" on stdout:
//            NP_TOT, Balance_Index, max of x y z u v w T, C and RHS_Part_Temp
//            max/min/mean
//
// dump_all: 0 = records after the prime and at the end only, 1 = also after every
// stage, 2 = also after every step (grid.cpp:315-325 done; tag 100000 + step)
//
// usage: ref_harness params.in input.bin output.bin nsteps dump_all [time [store_ts [load]]]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <chrono>
#include "mpi.h"
#include "params.h"
#include "proc.h"
#include "gridsize.h"
#include "communicator.h"
#include "tensor0.h"
#include "tensor1.h"
#include "particle.h"

static void die(const char *m) { fprintf(stderr, "ref_harness: %s\n", m); exit(2); }

static void read_exact(FILE *f, void *p, size_t n) {
  if (n && fread(p, 1, n, f) != n) die("short read");
}

// interior N^3 array (k,j,i with i fastest) -> ghosted tensor, then periodic ghost refresh
static void fill_interior(tensor0 &t, const double *src, int N) {
  const int G = N + 2;
  double *p = t.pointer();
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i)
        p[(size_t)(k + 1) * G * G + (size_t)(j + 1) * G + (i + 1)] = src[(size_t)k * N * N + (size_t)j * N + i];
  t.Update_Ghosts();
}

static void put(FILE *f, const std::vector<double> &v, int n) {
  if (n) fwrite(v.data(), sizeof(double), (size_t)n, f);
}

static void dump(FILE *f, int tag, particle &p, tensor0 &C, tensor1 &A, tensor0 &E, int N) {
  int32_t hdr[2] = {tag, p.Np};
  fwrite(hdr, sizeof(int32_t), 2, f);
  const int n = p.Np;
  put(f, p.x, n); put(f, p.y, n); put(f, p.z, n);
  put(f, p.x_int, n); put(f, p.y_int, n); put(f, p.z_int, n);
  put(f, p.x_new, n); put(f, p.y_new, n); put(f, p.z_new, n);
  put(f, p.x_np1, n); put(f, p.y_np1, n); put(f, p.z_np1, n);
  put(f, p.u, n); put(f, p.v, n); put(f, p.w, n);
  put(f, p.u_int, n); put(f, p.v_int, n); put(f, p.w_int, n);
  put(f, p.u_new, n); put(f, p.v_new, n); put(f, p.w_new, n);
  put(f, p.u_np1, n); put(f, p.v_np1, n); put(f, p.w_np1, n);
  put(f, p.T, n); put(f, p.T_int, n); put(f, p.T_new, n); put(f, p.T_np1, n);
  put(f, p.RHS_u, n); put(f, p.RHS_v, n); put(f, p.RHS_w, n); put(f, p.RHS_T, n);
  if (n) fwrite(p.flag.data(), sizeof(int), (size_t)n, f);
  const size_t G3 = (size_t)(N + 2) * (N + 2) * (N + 2);
  fwrite(C.pointer(), sizeof(double), G3, f);
  fwrite(A.x.pointer(), sizeof(double), G3, f);
  fwrite(A.y.pointer(), sizeof(double), G3, f);
  fwrite(A.z.pointer(), sizeof(double), G3, f);
  fwrite(E.pointer(), sizeof(double), G3, f);
  double mean_e = E.mean();
  fwrite(&mean_e, sizeof(double), 1, f);
}

int main(int argc, char **argv) {
  if (argc < 6) die("usage: ref_harness params.in input.bin output.bin nsteps dump_all [time]");
  const int nsteps = atoi(argv[4]);
  const int dump_all = atoi(argv[5]);
  const int timing = argc > 6 ? atoi(argv[6]) : 0;
  const int store_ts = argc > 7 ? atoi(argv[7]) : -1;
  const int load = argc > 8 ? atoi(argv[8]) : 0;
  MPI_Init(&argc, &argv);
  params P(argv[1]);
  proc PC;
  gridsize S(&P, &PC);
  communicator COM(&S, &P, &PC);
  const int N = P.Nx_tot();
  if (P.Ny_tot() != N || P.Nz_tot() != N) die("harness expects a cubic grid");
  if (P.bs() != 1) die("harness expects bs=1");

  FILE *in = fopen(argv[2], "rb");
  if (!in) die("cannot open input");
  int64_t np64 = 0;
  int32_t nn = 0;
  read_exact(in, &np64, sizeof np64);
  read_exact(in, &nn, sizeof nn);
  if (nn != N) die("input grid size does not match params");
  int n = (int)np64;
  const size_t N3 = (size_t)N * N * N;
  std::vector<double> buf(N3);

  tensor1 U(&S, &COM);
  tensor0 T(&S, &COM);
  tensor0 C(&S, &COM);
  tensor1 RHS_RU(&S, &COM);
  tensor0 RHS_Part_Temp(&S, &COM);
  read_exact(in, buf.data(), N3 * 8); fill_interior(U.x, buf.data(), N);
  read_exact(in, buf.data(), N3 * 8); fill_interior(U.y, buf.data(), N);
  read_exact(in, buf.data(), N3 * 8); fill_interior(U.z, buf.data(), N);
  read_exact(in, buf.data(), N3 * 8); fill_interior(T, buf.data(), N);
  C = 0.; RHS_RU = 0.; RHS_Part_Temp = 0.;

  particle part(&P, &PC, &S);
  if (load) {
    fclose(in);
    part.Load_All();  // particle.cpp:948-985
    n = part.Np;
  } else {
    part.Np = n;
    std::vector<double> *dst[7] = {&part.x, &part.y, &part.z, &part.u, &part.v, &part.w, &part.T};
    for (int a = 0; a < 7; ++a) {
      dst[a]->resize(n);
      read_exact(in, dst[a]->data(), (size_t)n * 8);
    }
    part.flag.resize(n);
    read_exact(in, part.flag.data(), (size_t)n * 4);
    fclose(in);
  }
  // RESIZE() (particle.cpp:136-148) reserves wg and Tg instead of resizing them;
  // size every work vector here so the reference's writes stay in bounds.
  std::vector<double> *work[] = {&part.x_int, &part.y_int, &part.z_int, &part.x_new, &part.y_new, &part.z_new,
                                 &part.x_np1, &part.y_np1, &part.z_np1, &part.u_int, &part.v_int, &part.w_int,
                                 &part.u_new, &part.v_new, &part.w_new, &part.u_np1, &part.v_np1, &part.w_np1,
                                 &part.T_int, &part.T_new, &part.T_np1, &part.RHS_u, &part.RHS_v, &part.RHS_w,
                                 &part.RHS_T, &part.ug, &part.vg, &part.wg, &part.Tg};
  for (auto *w : work) w->assign(n, 0.0);

  const double pre[4] = {0.5, 0.5, 1., 1. / 6.};
  const double post[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};

  FILE *out = fopen(argv[3], "wb");
  if (!out) die("cannot open output");

  // grid.cpp:207-226 (particle part of Initialize)
  part.x_int = part.x; part.y_int = part.y; part.z_int = part.z;
  part.u_int = part.u; part.v_int = part.v; part.w_int = part.w; part.T_int = part.T;
  part.x_np1 = part.x; part.y_np1 = part.y; part.z_np1 = part.z;
  part.u_np1 = part.u; part.v_np1 = part.v; part.w_np1 = part.w; part.T_np1 = part.T;
  part.gas2part_Temp_int(T);
  part.Compute_RHS_Temp_int();
  part.part2gas_Temp_int(RHS_Part_Temp);
  dump(out, -1, part, C, RHS_RU, RHS_Part_Temp, N);

  auto t0 = std::chrono::steady_clock::now();
  for (int s = 0; s < nsteps; ++s) {
    for (int k = 0; k < 4; ++k) {
      // grid.cpp:659-680
      part.gas2part_velocity(U);
      part.update_position(k, pre[k], post[k]);
      part.update_velocity(k, pre[k], post[k]);
      part.update_Temp(k, pre[k], post[k]);
      part.part2gas_concentration(C);
      if (P.TWC()) part.part2gas_velocity(RHS_RU); else RHS_RU = 0.;
      part.Send_Recv();
      part.gas2part_Temp_new(T);
      part.Compute_RHS_Temp_new();
      part.part2gas_Temp_new(RHS_Part_Temp);
      if (dump_all == 1) dump(out, s * 4 + k, part, C, RHS_RU, RHS_Part_Temp, N);
      // grid.cpp:705-712
      part.x_int = part.x_new; part.y_int = part.y_new; part.z_int = part.z_new;
      part.u_int = part.u_new; part.v_int = part.v_new; part.w_int = part.w_new; part.T_int = part.T_new;
    }
    // grid.cpp:315-325 (particle part)
    part.x = part.x_np1; part.y = part.y_np1; part.z = part.z_np1;
    part.u = part.u_np1; part.v = part.v_np1; part.w = part.w_np1; part.T = part.T_np1;
    if (dump_all == 2) dump(out, 100000 + s, part, C, RHS_RU, RHS_Part_Temp, N);
  }
  auto t1 = std::chrono::steady_clock::now();
  if (timing) {
    double sec = std::chrono::duration<double>(t1 - t0).count();
    printf("{\"particle_steps\": %.0f, \"seconds\": %.6f, \"particle_steps_per_s\": %.6e}\n",
           (double)n * nsteps, sec, (double)n * nsteps / sec);
  }
  dump(out, 1000000 + nsteps, part, C, RHS_RU, RHS_Part_Temp, N);
  fclose(out);
  if (store_ts >= 0) {
    part.Store_All(store_ts);
    printf("STATS {\"np_tot\": %d, \"balance_index\": %.17g, \"max\": {", part.NP_TOT(), part.Balance_Index());
    const char *nm[7] = {"x", "y", "z", "u", "v", "w", "T"};
    std::vector<double> *arr[7] = {&part.x, &part.y, &part.z, &part.u, &part.v, &part.w, &part.T};
    for (int a = 0; a < 7; ++a) printf("%s\"%s\": %.17g", a ? ", " : "", nm[a], part.max(*arr[a]));
    printf("}, \"C\": [%.17g, %.17g, %.17g]", C.max(), C.min(), C.mean());
    printf(", \"RHS_Part_Temp\": [%.17g, %.17g, %.17g]}\n", RHS_Part_Temp.max(), RHS_Part_Temp.min(),
           RHS_Part_Temp.mean());
    if (P.Np_track() > 0) part.trajectory((double)nsteps);
  }
  MPI_Finalize();
  return 0;
}
