// World<R> member definitions; included by exactly one translation unit per precision.  They live in
// four parts, each including the one before it: pe_world_setup, pe_world_step, pe_world_io,
// pe_world_repack.
#pragma once
#include "pe_world_repack.cuh"
