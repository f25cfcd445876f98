// sep_pass_f32.cu -- complex64 line passes (the mixed-precision filter path).
#define SEP_T float
#include "sep_pass_impl.cuh"
