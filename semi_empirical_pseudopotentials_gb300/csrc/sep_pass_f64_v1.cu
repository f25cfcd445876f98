// sep_pass_f64_v1.cu -- line passes, tile shape 1, for double.
#define SEP_T double
#define SEP_V 1
#include "sep_pass_impl.cuh"
