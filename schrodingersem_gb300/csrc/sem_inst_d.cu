// Explicit instantiations of the kernel launchers for N = 11 12 13 (p = N-1).
// The degrees are split over several units so they compile in parallel.
#include "sem_kernels.cuh"
SEM_INSTANTIATE(11)
SEM_INSTANTIATE(12)
SEM_INSTANTIATE(13)
