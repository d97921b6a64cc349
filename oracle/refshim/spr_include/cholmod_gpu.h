/* Stand-in for the one CHOLMOD GPU call sparse_relax.cpp makes (with -g). */
#ifndef NR_REFSHIM_CHOLMOD_GPU_H
#define NR_REFSHIM_CHOLMOD_GPU_H
#include "SuiteSparseQR.hpp"
int cholmod_l_gpu_memorysize(size_t *total_mem, size_t *available_mem, cholmod_common *cc);
#endif
