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
    bool sensors;      // the batch has sensor shapes (their update pass runs)
    bool isl_big_worlds;  // a world has more bodies than the islands' shared-memory pass holds
};
// bodies of the largest world whose islands are found in shared memory
constexpr uint32_t kIslSmemBodiesMax = 8192;

// contacts / broadphase (prgpu_contacts.cu)
void launch_pre_proxies(const DW& d, const Launch& L, cudaStream_t s);
void launch_destroy_contacts(const DW& d, const Launch& L, cudaStream_t s);
void launch_update_contacts(const DW& d, const Launch& L, uint32_t body_mask, cudaStream_t s);
void launch_set_upd_phase(const DW& d, uint32_t phase, cudaStream_t s);
void launch_post_record(const DW& d, const Launch& L, cudaStream_t s);
// spatial queries over the step's LBVH (prgpu_query.cu)
void launch_query_boxes(const DW& d, const Launch& L, uint32_t n, const uint32_t* worlds, const float4* boxes,
                        uint32_t cap, uint32_t* counts, uint32_t* out, uint32_t* status, cudaStream_t s);
void launch_ray_nearest(const DW& d, const Launch& L, uint32_t n, const uint32_t* worlds, const float* rays5,
                        int32_t* shape_out, float* hit5, uint32_t* status, cudaStream_t s);
void launch_ray_all(const DW& d, uint32_t w, const float* ray5, uint32_t cap, uint32_t* count, int32_t* shapes,
                    float* hit5, uint32_t* status, cudaStream_t s);
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
// time-of-impact phase (prgpu_toi.cu): set-up with round 0's times of impact,
// one event per world per round (with the contact search of the moved proxies),
// and the final contact update
void launch_toi_begin(const DW& d, const Launch& L, cudaStream_t s);
void launch_toi_round(const DW& d, const Launch& L, cudaStream_t s);
void launch_toi_end(const DW& d, const Launch& L, cudaStream_t s);
// GetToiViaSat over n pairs of (proxy, sweep) records
cudaError_t launch_toi_pairs(uint32_t n, const float4* vtx, const uint32_t* meta, const float* sweeps,
                             const DConf& c, float* time, int32_t* iout, cudaStream_t s);
// recording for the adjoint (prgpu_adjoint.cu)
void launch_tape_body_start(const DW& d, const Launch& L, cudaStream_t s);
void launch_tape_body_flags(const DW& d, const Launch& L, cudaStream_t s);
void launch_tape_constraints(const DW& d, const Launch& L, cudaStream_t s);

// adjoint and tangent passes over recorded steps (prgpu_adjoint.cu)
struct AdjState {
    float4* pbar;     // [N] d(loss)/d(centre x, y, angle)
    float4* vbar;     // [N] d(loss)/d(velocity)
    float4* vibar;    // [N] through the velocity bias: d(loss)/d(velocity at the start of the solve)
    float4* vi;       // [N] velocity at the start of the solve (recomputed)
    double* pvacc;    // [N*6] k_adj_local's adjoints of each body's position and start velocity, in FP64
    float4* lbar;     // [K] d(loss)/d(impulses ni0 ti0 ni1 ti1) of each constraint
    float* gbar;      // [K * kGeomWords] d(loss)/d(geometry)
    float* gval;      // [K * kGeomWords] geometry values
    float4* mbar;     // [C] d(loss)/d(stored manifold impulses) per slot
    float4* mtmp;     // [C]
    float* fbar;      // [S] d(loss)/d(shape friction)
    float4* jbar;     // [J] d(loss)/d(stored joint impulse x y)
    uint32_t* err;    // tape overflow count
    uint32_t grid;           // blocks of the parallel passes
    uint32_t sweep_threads;  // threads of the per-world sweep block
};

constexpr uint32_t kAdjSweepMaxThreads = 512;
constexpr int kAdjGeomWords = 28;  // words per recorded constraint in gbar, gval and gdot

struct TanState {
    double* pdot;   // [N*3]
    double* vdot;   // [N*3]
    double* vidot;  // [N*3] at the start of the solve
    double* ldot;   // [K*4]
    double* gdot;   // [K*kGeomWords]
    double* mdot;   // [C*4]
    double* mtmp;   // [C*4]
    const double* fdot;  // [S] tangent of shape friction
    double* jdot;   // [J*2] tangent of the stored joint impulses
};

// blocks of the adjoint's parallel passes on this device (0: no device)
uint32_t adj_parallel_grid();
// threads of the reverse sweeps' block (one a world), from the largest world's bodies
uint32_t adj_sweep_threads(uint32_t most, uint32_t n_worlds);
cudaError_t launch_adj_step(const DW& d, const StepTape* tp, const AdjState& a, uint32_t n_slots, cudaStream_t s);
cudaError_t launch_tan_step(const DW& d, const StepTape* tp, const TanState& t, float* gval, uint32_t n_slots,
                            cudaStream_t s);
// Sets k_world_solve's dynamic shared memory to stage_bytes; returns its CTAs per SM.
int world_blocks_per_sm(uint32_t stage_bytes);
// The k_world_solve instances with joint and recording code (full), with
// neither (lean) and with recording code only (tape), each in a translation
// unit of its own: launch on the per-world grid, raise the dynamic shared
// memory limit (false if refused), CTAs per SM at that staging size.
void world_solve_full_launch(const DW& d, unsigned grid, cudaStream_t s);
bool world_solve_full_allow_smem(uint32_t stage_bytes);
int world_solve_full_blocks_per_sm(uint32_t stage_bytes);
void world_solve_lean_launch(const DW& d, unsigned grid, cudaStream_t s);
bool world_solve_lean_allow_smem(uint32_t stage_bytes);
int world_solve_lean_blocks_per_sm(uint32_t stage_bytes);
void world_solve_tape_launch(const DW& d, unsigned grid, cudaStream_t s);
bool world_solve_tape_allow_smem(uint32_t stage_bytes);
int world_solve_tape_blocks_per_sm(uint32_t stage_bytes);

}  // namespace prgpu
