// prgpu_solver_lean.cu -- k_world_solve without joint or recording code (steps
// with neither), compiled apart from the rest of prgpu_solver.cu so the instances
// build in parallel.
#define PRGPU_SOLVER_PART 2
#include "prgpu_solver.cu"
