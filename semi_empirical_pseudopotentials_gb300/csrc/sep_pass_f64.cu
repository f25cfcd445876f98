// sep_pass_f64.cu -- complex128 line passes (the FP64 filter path).
#define SEP_T double
#include "sep_pass_impl.cuh"
