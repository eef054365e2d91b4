// prgpu_solver_tape.cu -- k_world_solve for recorded steps without joints,
// compiled apart from the rest of prgpu_solver.cu so the instances build in
// parallel.
#define PRGPU_SOLVER_PART 3
#include "prgpu_solver.cu"
