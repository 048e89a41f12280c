/*
 * apply_A_T_mex -- MATLAB / GNU Octave gateway of the adjoint of apply_A and of the gradients
 * with respect to the 1-D operators.  No counterpart in the reference (the prototype has no
 * adjoint); the operator it differentiates is the one apply_A.m:1-252 applies.
 *
 *   fbar      = apply_A_T_mex(ops, idx1d, deg, f, r)
 *   [fbar, G] = apply_A_T_mex(ops, idx1d, deg, f, r)
 *   ...       = apply_A_T_mex(ops, idx1d, deg, f, r, row_ptr, cols)
 *
 * With y = A*f and a cotangent r = dL/dy (for L = 1/2 ||A f - y*||^2, r = A f - y*):
 *   fbar = A' * r = dL/df                               (asg_apply_T_host_f64)
 *   G{t,k} = dL/d ops{t,k}, a matrix the size of ops{t,k} (asg_grad_ops_host_f64): the blocks
 *            some listed pair reaches hold the gradient, the others are zero; a factor the
 *            structure analysis found to be the identity is not differentiated and its G{t,k}
 *            is [] (empty).
 * Arguments as in apply_A_mex; f and r are DOF x 1 real doubles.  The plan cache is this
 * gateway's own (a MEX file is its own shared object).
 */
#include "asgkron_mex.h"

static asgm_cache g_cache;

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  static const char* gw = "apply_A_T_mex";
  if (nrhs != 5 && nrhs != 7)
    asgm_args(gw, "expected (ops, idx1d, deg, f, r) or (ops, idx1d, deg, f, r, row_ptr, cols)");
  if (nlhs > 2) asgm_args(gw, "at most two outputs (fbar, G)");
  asg_plan* plan = asgm_plan(gw, &g_cache, prhs[0], prhs[1], prhs[2], nrhs == 7 ? prhs[5] : NULL,
                             nrhs == 7 ? prhs[6] : NULL);
  asgm_check_vector(gw, prhs[3], "f", &g_cache);
  asgm_check_vector(gw, prhs[4], "r", &g_cache);
  const size_t n = mxGetNumberOfElements(prhs[4]);
  plhs[0] = mxCreateDoubleMatrix(n, 1, mxREAL);
  asg_status st = asg_apply_T_host_f64(plan, mxGetDoubles(prhs[4]), mxGetDoubles(plhs[0]));
  if (st != ASG_OK) asgm_fail(gw, st);
  if (nlhs < 2) return;
  const int T = g_cache.T, d = g_cache.d;
  unsigned masks[16];
  st = asg_plan_active(plan, masks);
  if (st != ASG_OK) asgm_fail(gw, st);
  double* G[ASGM_MAX_OPS];
  int ld[ASGM_MAX_OPS];
  mxArray* cell = mxCreateCellMatrix((size_t)T, (size_t)d);
  for (int t = 0; t < T; ++t)
    for (int m = 0; m < d; ++m) {
      const mxArray* a = mxGetCell(prhs[0], (size_t)t + (size_t)m * (size_t)T);
      const size_t n1 = mxGetM(a);
      const int applied = (masks[t] >> m) & 1u;
      mxArray* g = mxCreateDoubleMatrix(applied ? n1 : 0, applied ? n1 : 0, mxREAL); /* zero-filled */
      mxSetCell(cell, (size_t)t + (size_t)m * (size_t)T, g);
      G[t * d + m] = applied ? mxGetDoubles(g) : NULL;
      ld[t * d + m] = (int)n1;
    }
  plhs[1] = cell;
  st = asg_grad_ops_host_f64(plan, mxGetDoubles(prhs[3]), mxGetDoubles(prhs[4]), G, ld);
  if (st != ASG_OK) asgm_fail(gw, st);
}
