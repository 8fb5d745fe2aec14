// Batched-ensemble kernels for N = 8, 9 (sem_batch.cuh).
#define SEM_BATCH_DEFINE_KERNELS
#include "sem_batch.cuh"

SEM_BATCH_INSTANTIATE(8)
SEM_BATCH_INSTANTIATE(9)
