/* Mixed-precision FIRE kernels (FP32 bulk, FP64 anchors and reductions). */
#include "nr_device.cuh"
