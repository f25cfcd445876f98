// sep_pass_dd_g1.cu -- double-float line passes, length group 1.
#define SEP_T ddf
#define SEP_DD_G 1
#define SEP_DD_LIST SEP_DD_GROUP1
#include "sep_pass_impl.cuh"
