// Kernels of the rigid-body step.  One thread per body for integration, a project-written
// LSD radix sort plus a sweep for the broadphase, one thread per collision pair for the
// narrowphase (pairs bucketed by shape pairing), and sequential-impulse solver kernels
// (serial replay of the reference order per scene, or graph-coloured Gauss-Seidel).
// The kernels live in six parts, each including the one before it:
// pe_k_integrate, pe_k_broadphase, pe_k_narrowphase, pe_k_sat, pe_k_solver, pe_k_state.
#pragma once
#include "pe_k_state.cuh"
