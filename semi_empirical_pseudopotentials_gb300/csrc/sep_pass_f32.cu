// sep_pass_f32.cu -- line passes, tile shape 0, and the dispatch for float.
#define SEP_T float
#define SEP_V 0
#define SEP_DISPATCH
#include "sep_pass_impl.cuh"
