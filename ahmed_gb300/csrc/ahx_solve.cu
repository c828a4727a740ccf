// Iterative solvers on the device product and the multi-instance batch.
#include "ahx_hmat.hpp"

using namespace ahx;

extern "C" {

int ahx_gmres(ahx_hmat* H, int precision, uint32_t p, const double* B, uint64_t ldB, double* X,
              uint64_t ldX, double tol, uint32_t m, uint32_t maxit, uint32_t* iters,
              double* resid) {
  (void)H; (void)precision; (void)p; (void)B; (void)ldB; (void)X; (void)ldX; (void)tol; (void)m;
  (void)maxit; (void)iters; (void)resid;
  set_error("ahx_gmres: not built yet");
  return AHX_ERR_STATE;
}

int ahx_cg(ahx_hmat* H, uint32_t p, const double* B, uint64_t ldB, double* X, uint64_t ldX,
           double tol, uint32_t maxit, uint32_t* iters, double* resid) {
  (void)H; (void)p; (void)B; (void)ldB; (void)X; (void)ldX; (void)tol; (void)maxit; (void)iters;
  (void)resid;
  set_error("ahx_cg: not built yet");
  return AHX_ERR_STATE;
}

int ahx_batch_create(ahx_hmat* const* mats, uint32_t count, int precision, ahx_batch** out) {
  (void)mats; (void)count; (void)precision; (void)out;
  set_error("ahx_batch_create: not built yet");
  return AHX_ERR_STATE;
}
int ahx_batch_destroy(ahx_batch* b) { (void)b; return AHX_OK; }
uint64_t ahx_batch_n(const ahx_batch* b) { (void)b; return 0; }
int ahx_batch_matvec(ahx_batch* b, double d, uint32_t p, const double* X, double* Y) {
  (void)b; (void)d; (void)p; (void)X; (void)Y;
  set_error("ahx_batch_matvec: not built yet");
  return AHX_ERR_STATE;
}
int ahx_batch_gmres(ahx_batch* b, const double* B, double* X, double tol, uint32_t m,
                    uint32_t maxit, uint32_t* iters, double* resid) {
  (void)b; (void)B; (void)X; (void)tol; (void)m; (void)maxit; (void)iters; (void)resid;
  set_error("ahx_batch_gmres: not built yet");
  return AHX_ERR_STATE;
}
}
