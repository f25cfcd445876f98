// sep_pass_dd_g0.cu -- double-float line passes, length group 0.
#define SEP_T ddf
#define SEP_DD_G 0
#define SEP_DD_LIST SEP_DD_GROUP0
#include "sep_pass_impl.cuh"
