// Scalar RT instantiation for 8 half-space streams.
#include "rt_launch.cuh"
AERORT_INSTANTIATE_RT(8)
