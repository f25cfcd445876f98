// sep_pass_f32_v1.cu -- line passes, tile shape 1, for float.
#define SEP_T float
#define SEP_V 1
#include "sep_pass_impl.cuh"
