// sep_pass_dd_g2.cu -- double-float line passes, length group 2.
#define SEP_T ddf
#define SEP_DD_G 2
#define SEP_DD_LIST SEP_DD_GROUP2
#include "sep_pass_impl.cuh"
