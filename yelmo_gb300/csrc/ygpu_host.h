// ygpu_host.h -- host-side declarations shared by the library's translation units.
#pragma once
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/yelmo_gpu.h"

// An NVTX range over a C++ scope: the solve, a batch, a chunk of Picard
// iterations, the host staging copies, a serving tick. NVTX3 is header-only and
// does nothing unless a profiler or an NVTX injection library is attached.
struct YgRange {
    explicit YgRange(const char* name) { nvtxRangePushA(name); }
    ~YgRange() { nvtxRangePop(); }
    YgRange(const YgRange&) = delete;
    YgRange& operator=(const YgRange&) = delete;
};

#ifndef YG_BLOCK
#define YG_BLOCK 256
#endif

struct Inst;
struct InstOut;
struct TeamCtl;

// error message of the calling thread (ygpu_last_error)
void ygpu_set_error(const char* fmt, ...);

// ygpu_solver.cu

int ygpu_solver_max_ctas(int device);
size_t ygpu_solver_stack_bytes();

// Step kernels of the Picard loop (one cooperative launch each)
enum { YG_STEP_SETUP = 0, YG_STEP_PRE = 1, YG_STEP_KRYLOV = 2, YG_STEP_POST = 3, YG_STEP_FINAL = 4 };
struct StepShape {
    int grid, team_ctas;           // heavy steps: CTAs, CTAs per team
    int kgrid, ktc;                // Krylov step: CTAs, CTAs per team
    const int* map = nullptr;      // device team map of the heavy steps (NULL: uniform teams)
    const int* kmap = nullptr;     // device team map of the Krylov step
    int kcl = 0;                   // > 0: the Krylov teams are thread-block clusters of kcl CTAs
                                   // (kgrid = clusters x kcl), see ygpu_krylov_cluster_plan
    int wide_pre = 0;              // mixed pre step on the wide kernel (ygpu_step_shape_wide)
    int kslots = 0;                // mixed Krylov step: cells per thread whose CG records stay in
                                   // shared memory (ygpu_step_shape_wide sets it)
};
// The mixed pre step runs on 1024-thread CTAs (64 registers) when its CTAs hold
// more than two cells per thread of the 512-thread kernel: twice the warps per SM
// for the latency-bound passes; fewer cells leave the extra threads idle and the
// register cap costs more than it saves. total_unknowns: of all the instances.
void ygpu_step_shape_wide(StepShape* sh, size_t total_unknowns);
// Cluster size and count for the Krylov step of n_inst instances: req CTAs per
// cluster (2..16; anything else: no clusters), one instance per resident cluster
// or the instances round-robin over the resident clusters. Returns the size (0:
// use the global teams) and the cluster count.
int ygpu_krylov_cluster_plan(int device, int n_inst, size_t max_nu, int req, int* n_clusters);
int ygpu_init_constants(int device);
void ygpu_count_launches(unsigned long long n);
void ygpu_step_timing_flush();
int ygpu_step_shape(int device, int n_teams, int team_ctas, StepShape* sh);
// one team per instance, CTA counts from a plan (ygpu_plan_teams) already on the device
int ygpu_step_shape_mapped(int device, int grid, const int* d_map, StepShape* sh);
// CTAs per instance in proportion to its unknowns (at least one, at most its
// single-solve team); false when the instances outnumber max_ctas. map gets
// the layout run_step reads: [grid] CTA -> instance, then (first, count) pairs.
bool ygpu_plan_teams(int max_ctas, int n_inst, const size_t* nu, std::vector<int>& map, int* grid,
                     int unknowns_per_cta = 0);
int ygpu_launch_step(int step, cudaStream_t s, const StepShape& sh, const Inst* d_insts, int n_inst,
                     const ygpu_dyn_par& P, TeamCtl* ctls, int* d_done, int* d_abort);

// A CUDA graph of one chunk of Picard iterations, reused while the key matches.
struct GraphKey {
    const Inst* insts;
    int n_inst;
    StepShape sh;
    ygpu_dyn_par P;
    TeamCtl* ctls;
    int *done, *abort_;
    int check;
    int* h_flags;
    bool timed;                    // step timing events inside the graph
};
struct GraphEvents {
    cudaEvent_t a, b;
    int kind;
};
struct GraphCache {
    bool valid = false;
    GraphKey key;
    cudaGraphExec_t exec = nullptr;
    std::vector<GraphEvents> ev;   // event pairs of the timed launches
};
void ygpu_step_timing_add(int kind, double ms);
void ygpu_graph_cache_clear(GraphCache* gc);
bool ygpu_step_timing_on();

// A host hook between Picard iterations (neff_hook) of a single-instance solve
struct NeffRun {
    ygpu_neff_hook fn;
    void* user;
    int nx, ny;
    InstOut* d_out;                // the instance's outputs (defer is set)
    double *d_cbed, *d_uxb, *d_uyb;
    double *h_cbed, *h_uxb, *h_uyb, *h_prev;   // host buffers of nx*ny
};

// The whole solve of n_inst instances on `stream`: setup, the Picard loop as
// step launches (or chunk graphs with gc and pinned h_flags[2]; or one
// iteration at a time around a host hook), final passes.
int ygpu_launch_solver(int device, cudaStream_t stream, const Inst* d_insts, int n_inst, const ygpu_dyn_par& P,
                       TeamCtl* d_ctls, int n_teams, int team_ctas, int* d_done, int* d_abort,
                       const int* d_map = nullptr, int map_grid = 0, GraphCache* gc = nullptr,
                       int* h_flags = nullptr, int check_every = 4, const NeffRun* hook = nullptr,
                       int spin_log2 = 0, int cluster_req = 0, size_t max_nu = 0);
int ygpu_sm_count(int device);
size_t ygpu_teamctl_bytes();
size_t ygpu_inst_bytes();
int ygpu_launch_csr(cudaStream_t stream, int n, const int* ptr, const int* idx, const double* val, const double* b,
                    double* x, double* work, int method, int precond, int maxiter, double tol, int initx_zeros,
                    int* d_out_i, double* d_out_d, TeamCtl* d_ctl, int* d_abort, int n_ctas);
int ygpu_csr_max_ctas(int device);
int ygpu_adv_max_ctas(int device);
int ygpu_launch_advect(cudaStream_t stream, int nx, int ny, int code, double dx, double dy, double dt,
                       const double* var, const double* ux, const double* uy, const double* F, const double* Href,
                       const int* mask, double* dvdt, double* work, int* d_out_i, double* d_out_d, TeamCtl* d_ctl,
                       int* d_abort, int n_ctas);
int ygpu_dyn_inputs_device(cudaStream_t s, const double* H, const double* zb, const double* zsl, double* f_ice,
                           double* H_grnd, double* z_srf, double* f_grnd, double* fgx, double* fgy, int* mf,
                           double* dzsdx, double* dzsdy, double* tdx, double* tdy, double* tlx, double* tly,
                           double dx, double grad_lim, double taud_lim, double rho_ice, double rho_sw, double g,
                           int bc, int nx, int ny, double slope_bg_x = 0.0, double slope_bg_y = 0.0);
int ygpu_dyn_diagnostics_device(cudaStream_t s, const ygpu_dyn_diag& D, int bc);
int ygpu_gradient_column_device(cudaStream_t s, double* gx_c, double* gy_c, const double* gx, const double* gy,
                                const double* f_ice, const int* mask_ocn, int bc, int nx, int ny);
int ygpu_jacobian_device(cudaStream_t s, const ygpu_jvel& J, int bc, int terms);
int ygpu_uz3d_device(cudaStream_t s, const ygpu_uz3d& U, int bc, int method);
// ygpu_post.cu: uz_method 2 and 3, the strain-rate tensor
int ygpu_uz3d_quad_device(cudaStream_t s, const ygpu_uz3d& U, int bc, int method);
int ygpu_strain3d_device(cudaStream_t s, const ygpu_strain3d& S, int bc);
int ygpu_ssa_masks_device(cudaStream_t s, int* mx, int* my, const int* mf, const double* f_ice, const double* f_grnd,
                          int lat, int bc, int nx, int ny);

// ygpu_api.cu internals shared with the other translation units
struct ygpu_fields;
int ygpu_check_par(const ygpu_dyn_par* p);
// a neff hook is set on the calling thread (ygpu_set_neff_hook)
bool ygpu_neff_hook_is_set();
int ygpu_fields_check(int kind, const ygpu_fields* f);
void ygpu_fill_inst(Inst& I, int kind, const ygpu_fields* f);
// block: scratch for the tile-block preconditioner (mixed mode, -p ilu)
// ilu: scratch for the ILU(0) factors of the residual form (-p ilu)
size_t ygpu_inst_scratch_bytes(int nx, int ny, int nz, bool mixed, bool block = false, bool ilu = false);
void ygpu_inst_scratch_carve(Inst& I, char* base, int nx, int ny, int nz, bool mixed, bool block = false,
                             bool ilu = false);
inline bool ygpu_wants_block(const ygpu_dyn_par& p) {
    return p.lin_precond == YGPU_PRE_ILU0 && p.ssa_solver == YGPU_SSA_ENERGY && p.lin_solver != YGPU_LIN_BICGSTAB;
}
// lin_solver_run / lin_precond_run of a solve on an nx x ny grid (0: unknown)
void ygpu_lin_method_run_grid(const ygpu_dyn_par* p, int nx, int ny, int* solver, int* precond);
inline bool ygpu_wants_ilu(const ygpu_dyn_par& p) {
    return p.lin_precond == YGPU_PRE_ILU0 && p.ssa_solver != YGPU_SSA_ENERGY;
}
// the six-colour ordering of the ILU(0) leaves no two coupled unknowns in one
// colour unless a periodic direction has a length that is not a multiple of 3
inline bool ygpu_ilu_colourable(int nx, int ny, int bc) {
    const bool px = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_X);
    const bool py = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_Y || bc == YGPU_BND_MISMIP3D ||
                     bc == YGPU_BND_TROUGH);
    return !(px && nx % 3 != 0) && !(py && ny % 3 != 0);
}
size_t ygpu_align256(size_t b);
int ygpu_single_team_ctas(int max_ctas, size_t nu, int unknowns_per_cta = 0);
void ygpu_choose_teams(int max_ctas, int n_inst, size_t max_nu, int* n_teams, int* team_ctas, int upc = 0);
