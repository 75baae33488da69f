// Device-resident Krylov solvers (CG, BiCGStab, GMRES, FGMRES).
#pragma once

#include "gp_pc.h"

namespace gp {

enum KspType : int { KSP_CG = 2, KSP_BCGS = 6, KSP_GMRES = 12, KSP_FGMRES = 40 };

struct KspOptions {
  int type = KSP_GMRES;
  double rtol = 1e-5, atol = 1e-50, divtol = 1e4;
  double haptol = 1e-30, breakdowntol = 0.1;
  int normtype = 2;  // resolved: 1 none, 2 preconditioned, 3 unpreconditioned, 4 natural
  int pc_side = 0;   // 0 left, 1 right, 2 symmetric
  int guess_zero = 1;
  int min_it = 0;
  int chknorm = -1;
  int convmaxits = 0;
  int max_it = 1000;
  int restart = 30;
  int orthog = 0;    // 0 classical, 1 modified
  int cgstype = 0;   // 0 never, 1 if needed, 2 always
  int seed_rhs = 0;  // nonzero guess: rnorm0 from rhs_norm
  double rhs_norm = 0.0;
};

// Scalars of a running solve, in device memory.  Field names follow the
// reference drivers (src/ksp.mojo).
struct KspState {
  // configuration copy
  double rtol, atol, divtol, haptol, breakdowntol, rhs_norm;
  int normtype, pc_side, guess_zero, min_it, chknorm, convmaxits, max_it, m, seed_rhs;
  int cgstype;
  // KSPConvergedDefault bookkeeping
  double rnorm0, ttol;
  int seeded;
  // result
  double rnorm;
  int its, reason;
  // loop control and gate words
  int active;       // 1 while the solve runs (CG, BCGS)
  int phase;        // GMRES / FGMRES phase
  int trips;
  int g[16];        // per-driver conditional gates
  // CG
  double beta, betaold, dpi, dpiold, a, dp, bcoef;
  int i, bmode;
  // BCGS
  double rho, rhoold, alpha, omega, omegaold, d1, d2, bbeta, c_omb, c_one, c_nalpha, c_nomega;
  // GMRES / FGMRES
  int it, itcount, kcount, hapend, itb;
  double res, prev_rnorm, tt, cfg8, inv;
  double* vv_it;    // basis vector `it`
  double* vv_it1;   // basis vector `it + 1`
  double* pv_it;    // FGMRES prevec `it`
  double* vv_scale; // FGMRES: the vector the step's scale applies to
  double red[4];
  int mgs_on[64];    // modified Gram-Schmidt: projection k runs while k <= it
  double mgs_d;      // the current projection
};

struct Ksp {
  KspOptions opt;
  int device = -1;
  int n = 0;
  cudaStream_t stream = nullptr;
  // workspace
  double* work = nullptr;     // 7n (CG/BCGS) or 2n (GMRES family)
  double* vv = nullptr;       // (m+1) n
  double* prevec = nullptr;   // (m+2) n
  double* hs = nullptr;       // GMRES scalar block
  double* lhh = nullptr;      // CGS coefficients (m+2)
  double* hist = nullptr;     // max_it + 2
  int hist_cap = 0;
  KspState* st = nullptr;
  KspState* h_st = nullptr;   // pinned mirror
  RedSlot slot{};
  size_t work_n = 0, vv_n = 0, pv_n = 0, hs_n = 0;
  // captured loop
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  // what the graph was captured for
  const void* cap_A = nullptr;
  const void* cap_pc = nullptr;
  unsigned long long cap_A_uid = 0;  // Csr::uid of the captured operator
  unsigned long long cap_pc_gen = 0;  // Pc::generation of the captured PC
  const void* cap_b = nullptr;
  const void* cap_x = nullptr;
  int cap_key[13] = {0};
  cudaStream_t stream2 = nullptr;  // body capture stream
  int64_t top_kernels = 0;         // kernels outside the loop body
  int64_t body_kernels = 0;        // kernels per loop trip
  int64_t last_trips = 0;
  int launch_form = -1;  // -1 the environment's (GPETSC_KSP_GRAPH), 0 graph, 1 host loop
  int transpose = 0;     // solve A^T x = b (A^T multiply, transposed preconditioner)
};

struct KspResult {
  int its;
  int reason;
  double rnorm;
};

int ksp_create(Ksp** out);
int ksp_destroy(Ksp* k);
// b, x: device vectors of length A->n.  hist_out (host) receives min(hist_len,
// its + 1) residual norms.  Synchronous.
int ksp_solve(Ksp* k, Csr* A, Pc* pc, const double* b, double* x, KspResult* res,
              double* hist_out, int64_t hist_len, cudaStream_t caller);

}  // namespace gp
