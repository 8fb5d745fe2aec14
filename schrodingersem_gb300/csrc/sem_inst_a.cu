// Explicit instantiations of the kernel launchers for N = 2 3 4 5 6 (p = N-1).
// The degrees are split over several units so they compile in parallel.
#include "sem_kernels.cuh"
SEM_INSTANTIATE(2)
SEM_INSTANTIATE(3)
SEM_INSTANTIATE(4)
SEM_INSTANTIATE(5)
SEM_INSTANTIATE(6)
