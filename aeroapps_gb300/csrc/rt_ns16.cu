// Scalar RT instantiation for 16 half-space streams.
#include "rt_launch.cuh"
AERORT_INSTANTIATE_RT(16)
