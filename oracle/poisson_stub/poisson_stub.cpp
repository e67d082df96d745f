// Implementation of the Poisson stand-in (see poisson_stub.h). TEST INFRASTRUCTURE ONLY.
#include "poisson_stub.h"
#include <cstdio>
#include <cstdlib>
#include "gas_oracle.h"
#include "gridsize.h"
#include "params.h"

poisson::poisson(params *p, proc *, gridsize *s, communicator *com) : param_(p), size_(s) {
  center_coeff_ = new tensor0(s, com);
  rhs_new_ = new tensor0(s, com);
  dummy_ = new tensor1(s, com);
  const int n = s->Nx_tot();
  fft_ = new double[2 * (size_t)n * n * n];
  kmod_ = new double[n];
  gas_mod_wavenumber(kmod_, n, s->Lx());
}

poisson::~poisson() {
  delete center_coeff_;
  delete rhs_new_;
  delete dummy_;
  delete[] fft_;
  delete[] kmod_;
}

// del2 out = rhs with the modified wavenumber (poisson.cpp:413-462), interior of out only
void poisson::ccp_fft(tensor0 &rhs, tensor0 &out) {
  const int n = size_->Nx_tot(), G = n + 2;
  const size_t tot = (size_t)n * n * n;
  const double *r = rhs.pointer();
  double *o = out.pointer();
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t c = ((size_t)k * n + j) * n + i;
        fft_[2 * c + 1] = 0;
        fft_[2 * c] = r[((size_t)(k + 1) * G + (j + 1)) * G + (i + 1)];
      }
  gas_fft3d(fft_, n, -1);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t c = ((size_t)k * n + j) * n + i;
        if (i + j + k > 0) {
          const double den = kmod_[i] + kmod_[j] + kmod_[k];
          fft_[2 * c + 1] /= den;
          fft_[2 * c] /= den;
        }
      }
  gas_fft3d(fft_, n, +1);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        o[((size_t)(k + 1) * G + (j + 1)) * G + (i + 1)] = (-1) * fft_[2 * (((size_t)k * n + j) * n + i)] / (double)tot;
}

// div(C grad P) = RHS by fixed-point iteration on constant-coefficient solves
void poisson::Solve(tensor1 &C, tensor0 &P, tensor0 &RHS) {
  if (param_->Solver() != 0) {
    fprintf(stderr, "poisson stub: only the FFT solver (Solver 0) is available\n");
    abort();
  }
  tensor0 &cc = *center_coeff_, &rn = *rhs_new_;
  tensor1 &d = *dummy_;
  cc.Equal_I_F2C(C);
  cc.Equal_Divide(-1., cc);
  int it = 0;
  double error = 100;
  while (it < param_->Iteration() && error > param_->epsilon()) {
    d.Equal_Grad_C2F(P);
    d *= C;
    rn.Equal_Div_F2C(d);
    rn -= RHS;
    rn *= cc;
    ccp_fft(rn, d.x);
    P += d.x;
    P.Update_Ghosts();
    error = d.x.max_abs();
    it++;
  }
  num_iteration_ = it;
}

void poisson_IO::Solve(tensor1 &, tensor0 &, tensor0 &) {
  fprintf(stderr, "poisson stub: the inflow/outflow solver is not available\n");
  abort();
}
