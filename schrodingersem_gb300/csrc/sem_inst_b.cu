// Explicit instantiations of the kernel launchers for N = 7 8 (p = N-1).
// The degrees are split over several units so they compile in parallel.
#include "sem_kernels.cuh"
SEM_INSTANTIATE(7)
SEM_INSTANTIATE(8)
