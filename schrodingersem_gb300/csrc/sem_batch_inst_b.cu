// Batched-ensemble kernels for N = 6, 7 (sem_batch.cuh).
#define SEM_BATCH_DEFINE_KERNELS
#include "sem_batch.cuh"

SEM_BATCH_INSTANTIATE(6)
SEM_BATCH_INSTANTIATE(7)
