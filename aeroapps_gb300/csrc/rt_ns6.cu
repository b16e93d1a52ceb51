// Scalar RT instantiation for 6 half-space streams.
#include "rt_launch.cuh"
AERORT_INSTANTIATE_RT(6)
