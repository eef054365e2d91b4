// prgpu_kernels.cuh -- launchers of the world-step kernels (one stream, all
// counts in device memory so the whole step can be captured in a CUDA graph).
#pragma once

#include "prgpu_internal.cuh"

namespace prgpu {

struct Launch {
    Prims prims;
    int threads;       // block size of element-wise kernels
    int grid;          // grid of element-wise (grid-stride) kernels
    int coop_grid;     // grid of the cooperative colouring / solver kernels
    int coop_threads;
    bool per_world;    // sweeps run one CTA per world (batches of many worlds)
    int world_grid;    // persistent CTAs of the per-world sweep kernel
};

// contacts / broadphase (prgpu_contacts.cu)
void launch_pre_proxies(const DW& d, const Launch& L, cudaStream_t s);
void launch_destroy_contacts(const DW& d, const Launch& L, cudaStream_t s);
void launch_update_contacts(const DW& d, const Launch& L, uint32_t body_mask, cudaStream_t s);
void launch_find_contacts(const DW& d, const Launch& L, cudaStream_t s);
void launch_synchronize(const DW& d, const Launch& L, cudaStream_t s);
void launch_init_bodies(const DW& d, const Launch& L, cudaStream_t s);
// solver (prgpu_solver.cu)
void launch_solve(const DW& d, const Launch& L, cudaStream_t s);
void launch_islands_colour(const DW& d, const Launch& L, cudaStream_t s);
void launch_build_constraints(const DW& d, const Launch& L, cudaStream_t s);
void launch_solve_sweeps(const DW& d, const Launch& L, cudaStream_t s);
void launch_solve_finish(const DW& d, const Launch& L, cudaStream_t s);
void launch_reset_step(const DW& d, const Launch& L, cudaStream_t s);
void launch_clear_dirty(const DW& d, const Launch& L, cudaStream_t s);
int coop_blocks_per_sm(int threads);
// Sets k_world_solve's dynamic shared memory to stage_bytes; returns its CTAs per SM.
int world_blocks_per_sm(uint32_t stage_bytes);

}  // namespace prgpu
