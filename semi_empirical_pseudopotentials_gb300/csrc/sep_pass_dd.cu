// sep_pass_dd.cu -- the dispatch for ddf, the double-float form of the FP64
// passes (sep_dd.cuh); the passes themselves are in sep_pass_dd_g0..3.cu.
#define SEP_T ddf
#define SEP_IS_DD
#define SEP_DISPATCH
#include "sep_pass_impl.cuh"
