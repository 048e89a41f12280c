/*
 * apply_A_mex -- MATLAB / GNU Octave gateway of y = A*f on the GPU (apply_A.m:1-252, the
 * matrix-free branch: ftmp = sum over row elements, their connected column elements and the
 * selected terms of kron_multd(d, blocks, f_col), apply_A.m:102-236).
 *
 *   ftmp = apply_A_mex(ops, idx1d, deg, f)                  all element pairs
 *   ftmp = apply_A_mex(ops, idx1d, deg, f, row_ptr, cols)   pde.connectivity pairs
 *
 * ops, idx1d, deg, row_ptr and cols are described in asgkron_mex.h; f is the DOF x 1 real
 * double state (element-major in table order, apply_A.m:116).  The result is FP64, computed
 * by asg_apply_host_f64 (copy f in, one kernel, copy y out).  Errors: "asgkron:args" for bad
 * arguments, "asgkron:apply" for a library failure, with asg_last_error's text.
 *
 * Build: mex -R2018a apply_A_mex.c -I<repo>/include -L<lib dir> -lasgkron
 *        mkoctfile --mex apply_A_mex.c -I<repo>/include -L<lib dir> -lasgkron
 */
#include "asgkron_mex.h"

static asgm_cache g_cache;

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  static const char* gw = "apply_A_mex";
  if (nrhs != 4 && nrhs != 6) asgm_args(gw, "expected (ops, idx1d, deg, f) or (ops, idx1d, deg, f, row_ptr, cols)");
  if (nlhs > 1) asgm_args(gw, "one output (ftmp)");
  asg_plan* plan = asgm_plan(gw, &g_cache, prhs[0], prhs[1], prhs[2], nrhs == 6 ? prhs[4] : NULL,
                             nrhs == 6 ? prhs[5] : NULL);
  asgm_check_vector(gw, prhs[3], "f", &g_cache);
  const size_t n = mxGetNumberOfElements(prhs[3]);
  plhs[0] = mxCreateDoubleMatrix(n, 1, mxREAL);
  const asg_status st = asg_apply_host_f64(plan, mxGetDoubles(prhs[3]), mxGetDoubles(plhs[0]));
  if (st != ASG_OK) asgm_fail(gw, st);
}
