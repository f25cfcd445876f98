// sep_pass_f64.cu -- line passes, tile shape 0, and the dispatch for double.
#define SEP_T double
#define SEP_V 0
#define SEP_DISPATCH
#include "sep_pass_impl.cuh"
