// Instantiations of the on-chip resident inner solver (sem_resident.cuh) for
// the odd N (even degrees p = 4, 6, 8, 10): odd line strides keep the line
// passes free of shared-memory bank conflicts.  Other degrees use the staged
// kernel (k_minres_mixed).
#include "sem_resident.cuh"

namespace semgb {
SEM_INSTANTIATE_RESIDENT(5)
SEM_INSTANTIATE_RESIDENT(7)
SEM_INSTANTIATE_RESIDENT(9)
SEM_INSTANTIATE_RESIDENT(11)
}  // namespace semgb
