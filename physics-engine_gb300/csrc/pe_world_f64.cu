// World<double>: double-precision step (the reference's default PE_USE_DOUBLE build).
#include "pe_world_impl.cuh"
namespace pe { template class World<double>; }
