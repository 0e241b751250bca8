// Instantiation of the lattice-gauge kernels for SU2 (float and double,
// 2 to 4 dimensions); one translation unit per group keeps builds parallel.
#include "kernels.cuh"

namespace meshgb {
MESH_OPS_GETTER(ops_su2, SU2)
} // namespace meshgb
