// prgpu_solver_lean.cu -- k_world_solve<false> (steps without joints or
// recording), compiled apart from the rest of prgpu_solver.cu so the two build
// in parallel.
#define PRGPU_SOLVER_PART 2
#include "prgpu_solver.cu"
