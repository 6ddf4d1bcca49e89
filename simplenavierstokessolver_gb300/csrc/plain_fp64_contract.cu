// The plain FP64 kernels compiled with fused multiply-add contraction, for
// the parallel form of the plain path (sns_set_form(SNS_FORM_PARALLEL)): the
// same expressions and operation order as plain_fp64.cu, with a * b + c
// evaluated as one rounding where the compiler pairs them. Fewer FP64
// instructions (GB300's FP64 issue rate bounds the step) and shorter
// dependent chains in the Crank-Nicolson sweeps; results differ from the
// reference's by rounding and are held to the path's 1e-12 tolerance.
#define SNS_PLAIN_CONTRACT 1
#include "plain_fp64.cu"
