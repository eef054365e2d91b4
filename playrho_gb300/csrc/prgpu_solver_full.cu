// prgpu_solver_full.cu -- k_world_solve with joint and recording code (steps with joints),
// compiled apart from the rest of prgpu_solver.cu so the instances build in parallel.
#define PRGPU_SOLVER_PART 1
#include "prgpu_solver.cu"
