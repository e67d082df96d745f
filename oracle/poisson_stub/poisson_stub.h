// Stand-in for the reference's poisson.h and poisson_IO.h, force-included
// (g++ -include) when the reference's grid.cpp is compiled for the checker.
// TEST INFRASTRUCTURE ONLY.
//
// The reference's Poisson headers pull in the Sandia parallel FFT and HYPRE,
// which the reference does not vendor. Defining their include guards here
// makes grid.h skip them; the classes below keep the members grid.cpp uses.
// poisson::Solve restates the box's iterative FFT solve (poisson.cpp:115-117
// with Solver() == 0, :391-411, and CCP_FFT :413-462) on the oracle's own
// radix-2 FFT (gas_fft3d in oracle/gas_oracle.c), the same one the C
// restatement of the gas step uses. The inflow/outflow solver is not stubbed.
#ifndef PSTEP_POISSON_STUB_H
#define PSTEP_POISSON_STUB_H
#define poisson_h
#define poissonIO_h
#include "tensor0.h"
#include "tensor1.h"

class params;
class proc;
class gridsize;
class communicator;

class poisson {
 public:
  poisson() {}
  poisson(params *, proc *, gridsize *, communicator *);
  ~poisson();
  void Solve(tensor1 &C, tensor0 &P, tensor0 &RHS);
  int num_iteration() const { return num_iteration_; }

 private:
  void ccp_fft(tensor0 &rhs, tensor0 &out);
  params *param_ = nullptr;
  gridsize *size_ = nullptr;
  tensor0 *center_coeff_ = nullptr, *rhs_new_ = nullptr;
  tensor1 *dummy_ = nullptr;
  double *fft_ = nullptr, *kmod_ = nullptr;
  int num_iteration_ = 0;
};

class poisson_IO {
 public:
  poisson_IO() {}
  poisson_IO(params *, proc *, gridsize *, communicator *) {}
  void Solve(tensor1 &, tensor0 &, tensor0 &);
  int num_iteration1() const { return 0; }
  int num_iteration2() const { return 0; }
  double FFT_TIME = 0, SOLVER_TIME = 0;
};
#endif
