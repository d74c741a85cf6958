/* Thin C driver around the reference's own OpenCL FNNLS kernel source
 * (multifit_ocl/device/regression_inplace_fnnls.cl: inplace_fnnls with the
 * incremental Cholesky row addition and in-between removal, N = K = 10, row-major
 * matrices), compiled as C on the host -- TEST INFRASTRUCTURE ONLY (it pins the
 * oracle's FNNLS loop; nothing on the engine's path uses it).
 *
 * The .cl file is included unmodified. The OpenCL address-space and kernel
 * qualifiers become empty macros and get_global_id() a constant (the facade
 * kernel is compiled but not called). Built twice by oracle/build_oracle.py:
 * as written (data_type float) and with MF_REF_OCL_DOUBLE, where the keyword
 * float is mapped to double before the file's `typedef float data_type`, so
 * that the same loop runs in the oracle's FP64. */
#include <float.h>
#include <math.h>
#include <stdio.h>

#define __global
#define __kernel
#define get_global_id(dim) 0

#ifdef MF_REF_OCL_DOUBLE
#define float double
#endif
#include "regression_inplace_fnnls.cl"
#ifdef MF_REF_OCL_DOUBLE
#undef float
#endif

/* A: 10 x 10 row-major, b: 10, x: 10 in/out (the warm start, as the kernel's
 * final_s is initialised from x). */
void ref_ocl_inplace_fnnls(const data_type* A, const data_type* b, data_type* x, double eps,
                           unsigned int max_iter) {
  inplace_fnnls(A, b, x, eps, max_iter);
}

int ref_ocl_data_type_bytes(void) { return (int)sizeof(data_type); }
