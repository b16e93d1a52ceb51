// Scalar RT instantiation for 12 half-space streams.
#include "rt_launch.cuh"
AERORT_INSTANTIATE_RT(12)
