// Kernels of the rigid-body step.  One thread per body for integration, a project-written
// LSD radix sort plus a warp-per-position sweep for the broadphase, one thread per pair for the
// closed-form pair algorithms and one warp (one block for heavy pairs) per pair for the staged
// convex SAT, and sequential-impulse solver kernels (the reference's order kept per island by
// level schedules, or graph-coloured Gauss-Seidel).
// The kernels live in six parts, each including the one before it:
// pe_k_integrate, pe_k_broadphase, pe_k_narrowphase, pe_k_sat, pe_k_solver, pe_k_state.
#pragma once
#include "pe_k_state.cuh"
