// sep_pass_dd_g3.cu -- double-float line passes, length group 3.
#define SEP_T ddf
#define SEP_DD_G 3
#define SEP_DD_LIST SEP_DD_GROUP3
#include "sep_pass_impl.cuh"
