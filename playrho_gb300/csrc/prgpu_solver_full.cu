// prgpu_solver_full.cu -- k_world_solve<true> (steps with joints or recording),
// compiled apart from the rest of prgpu_solver.cu so the two build in parallel.
#define PRGPU_SOLVER_PART 1
#include "prgpu_solver.cu"
