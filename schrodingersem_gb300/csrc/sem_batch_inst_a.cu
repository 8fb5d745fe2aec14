// Batched-ensemble kernels for N = 3, 4, 5 (sem_batch.cuh).
#define SEM_BATCH_DEFINE_KERNELS
#include "sem_batch.cuh"

SEM_BATCH_INSTANTIATE(3)
SEM_BATCH_INSTANTIATE(4)
SEM_BATCH_INSTANTIATE(5)
