// World<float>: single-precision step (the reference built with pe::Real = float).
#include "pe_world_impl.cuh"
namespace pe { template class World<float>; }
