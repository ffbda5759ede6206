/*
 * yelmo_oracle.h -- CPU FP64 restatement of Yelmo's SSA/DIVA velocity solve.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle of the GPU solver: only the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it. The
 * product (libyelmo_gpu.so) never links or calls it.
 *
 * Provenance: restated from the reference Fortran sources, routine by routine
 * (file:line cited at each function in yelmo_oracle.c). Two third-party pieces
 * the reference does not vendor are restated from their published algorithms:
 *   - LIS (linear solver library, version not pinned: fesm-utils:stable): CG
 *     (Hestenes-Stiefel), BiCGSTAB (van der Vorst 1992), MINRES (Paige-Saunders
 *     1975), Jacobi and ILU(0) (Saad, Iterative Methods, 10.3), with LIS's
 *     relative-residual stopping rule ||b-Ax||_2 / ||b||_2 < tol;
 *   - fesm-utils gaussian_quadrature (gq2D_*, gq3D_*): 2x2 (2x2x2)
 *     Gauss-Legendre nodes at +-1/sqrt(3) of the cell (cell-layer box), node
 *     values bilinear (trilinear) from corner means (masked by the `act`
 *     faces/cells when given; in 3D also averaged over the two layers or ac
 *     levels meeting at a corner), equal weights.
 * Pinning: the assembly is pinned by the reference's known-answer tests
 * (tests/test_ssa_energy*.f90), the converged solve by the reference's
 * analytic benchmarks (A2 radial shelf, tests/bench/src/shelf.jl). The
 * quadrature rule and LIS iterates are restated and unpinned; only converged
 * solutions are compared. The routines around the solve (post-solve diagnostics,
 * column gradients, velocity Jacobian, vertical velocity, implicit advection)
 * have no known-answer test in the reference; they are pinned by independent
 * restatements in the tests and by analytic cases (exactness of the difference
 * formulas on polynomials, incompressible flow, column mass balance).
 */
#ifndef YELMO_ORACLE_H
#define YELMO_ORACLE_H

#include "../include/yelmo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CSR matrix, 0-based, with the reference's unknown numbering
   (solver_linear.F90:131-143): cell q = i*ny + j, ux -> 2q, uy -> 2q+1. */
typedef struct orc_csr {
    int nmax, nnz, cap;
    int *ptr, *idx;
    double *val, *b, *x;
    int *copy_from;            /* -1: none, else row whose solution this row takes */
} orc_csr;

void orc_csr_free(orc_csr* A);

/* assemblers: residual (solver_ssa_ac.f90:73) and energy (solver_ssa_ac_energy.f90:70) */
int orc_assemble_residual(orc_csr* A, const double* ux, const double* uy,
        const double* beta_acx, const double* beta_acy, const double* N_aa,
        const int* mask_acx, const int* mask_acy, const double* H_ice, const double* f_ice,
        const double* z_bed, const double* z_sl, const double* taud_acx, const double* taud_acy,
        const double* taul_acx, const double* taul_acy, double dx, double dy, int bc,
        const double* lim_k_acx, const double* lim_k_acy, const double* lim_r_acx,
        const double* lim_r_acy, int nx, int ny);
int orc_assemble_energy(orc_csr* A, const double* ux, const double* uy,
        const double* beta_acx, const double* beta_acy, const double* N_aa,
        const int* mask_acx, const int* mask_acy, const double* H_ice, const double* f_ice,
        const double* z_bed, const double* z_sl, const double* taud_acx, const double* taud_acy,
        const double* taul_acx, const double* taul_acy, double dx, double dy, int bc,
        const double* lim_k_acx, const double* lim_k_acy, const double* lim_r_acx,
        const double* lim_r_acy, int nx, int ny);

/* Assemble into caller arrays (for the tests): returns nnz, or -needed if cap too small. */
int orc_assemble_csr(int energy, int nx, int ny, double dx, double dy, int bc,
        const double* ux, const double* uy, const double* beta_acx, const double* beta_acy,
        const double* N_aa, const int* mask_acx, const int* mask_acy, const double* H_ice,
        const double* f_ice, const double* z_bed, const double* z_sl,
        const double* taud_acx, const double* taud_acy, const double* taul_acx,
        const double* taul_acy, int cap, int* ptr, int* idx, double* val, double* b,
        double* x, int* copy_from);

/* Linear solve (LIS stand-in). Returns status 0/2/4; *iters, *relres out. */
int orc_linear_solve(int n, const int* ptr, const int* idx, const double* val,
        const double* b, double* x, int method, int precond, int maxiter, double tol,
        int initx_zeros, int* iters, double* relres);

/* Velocity solves: same argument order as the ABI functions of yelmo_gpu.h. */
int orc_calc_velocity_ssa(
    double* ux_b, double* uy_b, double* taub_acx, double* taub_acy,
    double* visc_eff, double* visc_eff_int, int* ssa_mask_acx, int* ssa_mask_acy,
    double* ssa_err_acx, double* ssa_err_acy,
    int* ssa_iter_now, int* ssa_lin_iter, int* ssa_lin_fail, int* ssa_lim_n,
    double* beta, double* beta_acx, double* beta_acy,
    const double* c_bed, const double* f_slide,
    const double* taud_acx, const double* taud_acy,
    const double* taul_int_acx, const double* taul_int_acy,
    const double* H_ice, const double* f_ice, const double* H_grnd, const double* f_grnd,
    const double* f_grnd_acx, const double* f_grnd_acy,
    const double* ATT, const double* zeta_aa,
    const double* z_sl, const double* z_bed, const double* z_srf,
    double dx, double dy, double n_glen,
    int nx, int ny, int nz, const ygpu_dyn_par* par);

int orc_calc_velocity_diva(
    double* ux, double* uy, double* ux_bar, double* uy_bar,
    double* ux_b, double* uy_b, double* ux_i, double* uy_i,
    double* taub_acx, double* taub_acy,
    double* beta, double* beta_acx, double* beta_acy, double* beta_eff,
    double* visc_eff, double* visc_eff_int, double* duxdz, double* duydz,
    int* ssa_mask_acx, int* ssa_mask_acy, double* ssa_err_acx, double* ssa_err_acy,
    int* ssa_iter_now, int* ssa_lin_iter, int* ssa_lin_fail, int* ssa_lim_n,
    const double* c_bed, const double* f_slide,
    const double* taud_acx, const double* taud_acy,
    const double* taul_int_acx, const double* taul_int_acy,
    const double* H_ice, const double* f_ice, const double* H_grnd, const double* f_grnd,
    const double* f_grnd_acx, const double* f_grnd_acy,
    const double* ATT, const double* zeta_aa,
    const double* z_sl, const double* z_bed, const double* z_srf,
    double dx, double dy, double n_glen,
    int nx, int ny, int nz, const ygpu_dyn_par* par);

/* neff_hook of calc_velocity_diva: c_bed (in/out) from the basal velocity */
typedef void (*orc_neff_hook)(void* user, double* c_bed, const double* ux_b, const double* uy_b, int nx, int ny);
int orc_calc_velocity_diva_hook(
    double* ux, double* uy, double* ux_bar, double* uy_bar,
    double* ux_b, double* uy_b, double* ux_i, double* uy_i,
    double* taub_acx, double* taub_acy,
    double* beta, double* beta_acx, double* beta_acy, double* beta_eff,
    double* visc_eff, double* visc_eff_int, double* duxdz, double* duydz,
    int* ssa_mask_acx, int* ssa_mask_acy, double* ssa_err_acx, double* ssa_err_acy,
    int* ssa_iter_now, int* ssa_lin_iter, int* ssa_lin_fail, int* ssa_lim_n,
    double* c_bed, const double* f_slide,
    const double* taud_acx, const double* taud_acy,
    const double* taul_int_acx, const double* taul_int_acy,
    const double* H_ice, const double* f_ice, const double* H_grnd, const double* f_grnd,
    const double* f_grnd_acx, const double* f_grnd_acy,
    const double* ATT, const double* zeta_aa,
    const double* z_sl, const double* z_bed, const double* z_srf,
    double dx, double dy, double n_glen,
    int nx, int ny, int nz, const ygpu_dyn_par* par, orc_neff_hook hook, void* user);


int orc_set_ssa_masks(int* mask_acx, int* mask_acy, const int* mask_frnt,
                      const double* f_ice, const double* f_grnd, int lateral_bc, int bc,
                      int nx, int ny);

int orc_calc_dyn_inputs(const double* H_ice, const double* z_bed, const double* z_sl,
                        double* f_ice, double* H_grnd, double* z_srf,
                        double* f_grnd, double* f_grnd_acx, double* f_grnd_acy,
                        int* mask_frnt, double* dzsdx, double* dzsdy,
                        double* taud_acx, double* taud_acy,
                        double* taul_int_acx, double* taul_int_acy,
                        double dx, double grad_lim, double taud_lim,
                        double rho_ice, double rho_sw, double g, int bc, int nx, int ny);
/* the same with the uniform background slope added to dzsdx, dzsdy before the
   limit (calc_gradient_acx/acy slope_bg, yelmo_tools.f90:401,470) */
int orc_calc_dyn_inputs_bg(const double* H_ice, const double* z_bed, const double* z_sl,
                           double* f_ice, double* H_grnd, double* z_srf,
                           double* f_grnd, double* f_grnd_acx, double* f_grnd_acy,
                           int* mask_frnt, double* dzsdx, double* dzsdy,
                           double* taud_acx, double* taud_acy,
                           double* taul_int_acx, double* taul_int_acy,
                           double dx, double grad_lim, double taud_lim,
                           double rho_ice, double rho_sw, double g,
                           double slope_bg_x, double slope_bg_y, int bc, int nx, int ny);

/* sigma grid, calc_zeta (yelmo_grid.f90:41): scale 0 linear, 1 exp, 2 exp-inv, 3 tanh */
void orc_calc_zeta(int nz, int scale, double zeta_exp, double* zeta_aa);

/* rate factor, calc_rate_factor (deformation.f90:305) */
double orc_rate_factor(double T_ice, double T_pmp, double enh, double T0);

/* Oracle's own parameter helpers (same semantics as the library's). */
void orc_dyn_par_defaults(ygpu_dyn_par* par);
int  orc_parse_lis_opt(const char* opts, ygpu_dyn_par* par);
void orc_set_threads(int n);

/* Post-solve diagnostics of calc_ydyn (yelmo_dynamics.f90:304-336, :642-644):
   depth averages, ice and grounding-line fluxes, magnitudes, surface fields,
   f_vbvs; the same groups and NULL conventions as ygpu_calc_dyn_diagnostics. */
int orc_calc_dyn_diagnostics(const ygpu_dyn_diag* D, int boundaries);

/* calc_gradient_column_ac (yelmo_tools.f90:479-571) and the velocity Jacobian
   (calc_jacobian_vel_3D_uxyterms / _uzterms, deformation.f90:397-961), in the
   reference's two passes per routine; the same arguments as the ygpu_ entries. */
int orc_calc_gradient_column_ac(double* dvdx_c, double* dvdy_c, const double* dvdx, const double* dvdy,
                                const double* f_ice, const int* mask_ocn, int boundaries, int nx, int ny);
int orc_calc_jacobian_vel_3D(const ygpu_jvel* J, int boundaries, int terms);

/* Vertical velocity by uz_method (calc_uz_3D_aa, calc_uz_3D, calc_uz_3D_jac,
   calc_uz_3D_flux, velocity_general.f90:41-1116) and uz_srf_err; the arguments of
   ygpu_calc_uz_3D. */
int orc_calc_uz_3D(const ygpu_uz3d* U, int boundaries, int method);
/* calc_strain_rate_tensor_jac_quad3D (deformation.f90:963-1183) */
int orc_calc_strain_rate_tensor(const ygpu_strain3d* S, int boundaries);

/* calc_advec2D(solver = "impl-lis"), solver_advection.f90:20-145: the CSR system of
   linear_solver_matrix_advection_csr_2D (:171-487) solved with this oracle's BiCGSTAB
   and Jacobi to 1e-12, calc_fixed_cell_transport (:489-546), dvdt. Same arguments as
   ygpu_calc_advec2D_impl_lis. */
int orc_calc_advec2D_impl_lis(double* dvdt, const double* var, const double* ux, const double* uy,
                              const double* var_dot, const int* mask_ice, const double* var_ref,
                              double dx, double dy, double dt, int boundaries, int nx, int ny,
                              int* lin_iter, int* lin_status);

#ifdef __cplusplus
}
#endif
#endif
