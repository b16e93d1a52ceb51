// Scalar RT instantiation for 4 half-space streams.
#include "rt_launch.cuh"
AERORT_INSTANTIATE_RT(4)
