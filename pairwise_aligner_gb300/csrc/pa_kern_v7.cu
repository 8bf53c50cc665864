// pa_kern_v7.cu -- instantiations of dp_kernel for inner-loop variant 7.
#include "pa_dp.cuh"
#include "pa_launch.h"

namespace pa {

#define PA_VARIANT 7
#include "pa_kern_inst.cuh"

}  // namespace pa
