/*
 * yelmo_gpu.h -- C ABI of the GB300 (sm_103a) SSA/DIVA ice-velocity solver.
 *
 * Drop-in for Yelmo's velocity-solver entry points:
 *   calc_velocity_ssa   (src/physics/velocity_ssa.f90:60, called from src/yelmo_dynamics.f90:504)
 *   calc_velocity_diva  (src/physics/velocity_diva.f90:59, called from src/yelmo_dynamics.f90:630)
 * and the lower linear-solver seam
 *   linear_solver_matrix_solve (src/physics/solver_linear.F90:151).
 *
 * Conventions (those of Yelmo's own C API, docs/c-api.md:28-36):
 *   - every array is caller owned, Fortran column-major: 2D fields (nx,ny) with x
 *     fastest, 3D fields (nx,ny,nz) with k=1 at the ice base;
 *   - staggered fields share the cell shape: ux(i,j) lives on the right face of
 *     cell (i,j) (acx), uy(i,j) on its top face (acy), corner (i,j) is top-right;
 *   - reals are double precision (Fortran real(c_double)), masks are C int;
 *   - functions return an int status: 0 OK, 2 linear-solve breakdown, 4 linear
 *     solve hit its iteration limit (the LIS codes of solver_linear.F90:36-39),
 *     negative values for errors (see YGPU_ERR_*). Nothing here calls exit().
 */
#ifndef YELMO_GPU_H
#define YELMO_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define YGPU_OK               0
#define YGPU_BREAKDOWN        2   /* LGS_BREAKDOWN, solver_linear.F90:38            */
#define YGPU_MAXITER          4   /* LGS_MAXITER,   solver_linear.F90:39            */
#define YGPU_ERR_NONFINITE   -1   /* velocity not finite (velocity_general.f90:2114) */
#define YGPU_ERR_BAD_ARG     -2   /* bad size / option / method code               */
#define YGPU_ERR_CUDA        -3   /* CUDA runtime error (message: ygpu_last_error)  */
#define YGPU_ERR_TIMEOUT     -4   /* a device-side wait hit its iteration limit     */
#define YGPU_ERR_ADMISSION   -5   /* serving: request rejected by the HBM budget    */
#define YGPU_ERR_NOMEM       -6   /* device allocation failed                       */
#define YGPU_ERR_BUSY        -7   /* serving: no free slot, try again               */

/* ---- boundary codes: yelmo_tools.f90:14-20 (BND_*), boundary_code() :248 ---- */
#define YGPU_BND_ZEROS        0
#define YGPU_BND_INFINITE     1   /* also "mask" */
#define YGPU_BND_MISMIP3D     2
#define YGPU_BND_TROUGH       3
#define YGPU_BND_PERIODIC     4
#define YGPU_BND_PERIODIC_X   5
#define YGPU_BND_PERIODIC_Y   6
#define YGPU_BND_MASK         7   /* "mask": INFINITE for the velocity solve; own border rows in advection */

/* ---- ydyn.ssa_solver ("residual" | "energy"), velocity_ssa.f90:25 ---- */
#define YGPU_SSA_RESIDUAL     0
#define YGPU_SSA_ENERGY       1

/* ---- ydyn.ssa_vel_lim_method ("clip" | "drag") ---- */
#define YGPU_VEL_LIM_CLIP     0
#define YGPU_VEL_LIM_DRAG     1

/* ---- ydyn.ssa_lat_bc for set_ssa_masks (solver_ssa_ac.f90:985-994) ---- */
#define YGPU_LATBC_NONE       0
#define YGPU_LATBC_FLOATING   1
#define YGPU_LATBC_MARINE     2
#define YGPU_LATBC_ALL        3

/* ---- LIS option string "-i ... -p ..." (input/yelmo_defaults.nml:160-161) ---- */
#define YGPU_LIN_CG           0
#define YGPU_LIN_BICGSTAB     1
#define YGPU_LIN_MINRES       2
#define YGPU_PRE_NONE         0
#define YGPU_PRE_JACOBI       1
#define YGPU_PRE_ILU0         2   /* "-p ilu". With BiCGSTAB on the residual form the GPU runs
                                     ILU(0) of the operator in a six-colour ordering (cell
                                     colour (i - j) mod 3, then the component), which needs
                                     periodic directions in multiples of 3 cells (else Jacobi),
                                     with FP64 factors and BiCGSTAB in both precisions; the
                                     other forms run what ygpu_stats.lin_precond_run says      */
#define YGPU_PRE_TILE_BLOCK   3   /* run only (never parsed): block Jacobi with the exact inverse
                                     of each 4x4-cell tile block (32 unknowns, inverted in FP32),
                                     what "-p ilu" runs for CG on the energy form             */

/* ---- arithmetic of the GPU solve ---- */
#define YGPU_PREC_FP64        0   /* plain FP64 solve: the drop-in                         */
#define YGPU_PREC_MIXED       1   /* FP32 viscosity/operator/preconditioner/Krylov inside an
                                     FP64 defect-correction loop                             */

/*
 * Parameters of one velocity solve. Mirrors ssa_param_class
 * (velocity_ssa.f90:23-52) and diva_param_class (velocity_diva.f90:22-51), with
 * the character fields replaced by the codes above and ssa_lis_opt parsed into
 * the lin_* fields (ygpu_parse_lis_opt).
 */
typedef struct ygpu_dyn_par {
    int    ssa_solver;          /* YGPU_SSA_*                                   */
    int    boundaries;          /* YGPU_BND_*                                   */
    int    no_slip;             /* DIVA only: solver = "diva-noslip"            */
    int    visc_method;         /* 0 const, 1 quadrature nodes, 2 aa-nodes      */
    double visc_const;          /* [Pa a]                                       */
    int    beta_method;         /* -1 imposed, 0 const, 1 linear, 2 power, 3 reg. Coulomb, 4/5 centred */
    double beta_const;          /* [Pa a m-1]                                   */
    double beta_q;
    double beta_u0;             /* [m a-1]                                      */
    int    beta_gl_scale;       /* 0 fraction, 1 H_grnd, 2 zstar, 3 f_grnd      */
    int    beta_gl_stag;        /* -1 imposed, 0 mean, 1 upstream, 2 downstream, 3 subgrid, 4 flux */
    double beta_gl_f;
    double H_grnd_lim;          /* [m]                                          */
    double beta_min;            /* [Pa a m-1]                                   */
    double eps_0;               /* [a-1]                                        */
    int    ssa_vel_lim_method;  /* YGPU_VEL_LIM_*                               */
    double ssa_vel_lim_tau;     /* [Pa]                                         */
    double ssa_vel_max;         /* [m a-1]                                      */
    int    ssa_iter_max;
    double ssa_iter_rel;
    double ssa_iter_conv;
    int    ssa_write_log;       /* print the per-iteration "ssa:" line          */
    double rho_ice;
    double rho_sw;
    double g;
    /* parsed ssa_lis_opt */
    int    lin_solver;          /* YGPU_LIN_*                                   */
    int    lin_precond;         /* YGPU_PRE_*                                   */
    int    lin_maxiter;
    double lin_tol;             /* relative residual ||b-Ax||/||b||             */
    int    lin_initx_zeros;     /* 1: start the Krylov solve from x=0           */
    /* GPU solve only */
    int    precision;           /* YGPU_PREC_*                                  */
    int    inner_maxiter;       /* mixed: FP32 iterations per defect-correction step (0: default) */
    double inner_tol;           /* mixed: FP32 relative tolerance per step (0: default)          */
} ygpu_dyn_par;

/* Iteration counters of one solve (ydyn%par%ssa_iter_now etc., yelmo_defs.f90:483-486) */
typedef struct ygpu_stats {
    int    ssa_iter_now;        /* Picard iterations done                       */
    int    ssa_lin_iter;        /* linear iterations, summed over Picard        */
    int    ssa_lin_fail;        /* linear solves that ended at breakdown/maxiter */
    int    ssa_lim_n;           /* faces at the velocity limit (count_vel_lim_faces) */
    double ssa_resid;           /* last Picard L2 relative change               */
    double lin_resid;           /* last linear relative residual                */
    int    outer_iter;          /* mixed: defect-correction steps, summed       */
    int    status;              /* YGPU_* of the solve                          */
    double device_ms;           /* device time of the solve (CUDA events)       */
    double phase_ms[10];        /* device time per phase of the solve: setup, strain rates,
                                   column (viscosity, integrals, beta), faces, linear system,
                                   Krylov, epilogue, final passes; then the time spent in
                                   team all-reduces over the solve and within the Krylov phase */
    int    active_cells;        /* cells with a non-identity row: the cells the Krylov iterations visit */
    int    lin_solver_run;      /* YGPU_LIN_* the GPU ran for the requested method: MINRES
                                   requests run CG (energy form) or BiCGSTAB (residual form) */
    int    lin_precond_run;     /* YGPU_PRE_* the GPU ran for the requested preconditioner   */
} ygpu_stats;

/* The Krylov method and preconditioner the GPU runs for a parameter set (the
   values ygpu_stats.lin_solver_run / lin_precond_run report; a solve on a
   periodic grid that the ILU(0) colouring does not fit reports Jacobi). */
void ygpu_lin_method_run(const ygpu_dyn_par* par, int* lin_solver_run, int* lin_precond_run);

/* ---- parameter helpers -------------------------------------------------- */
/* Defaults of input/yelmo_defaults.nml &ydyn (:140-172) and &Earth constants. */
void ygpu_dyn_par_defaults(ygpu_dyn_par* par);
/* Parse a LIS option string such as "-i cg -p jacobi -maxiter 200 -tol 1.0e-2
   -initx_zeros false" into par->lin_*. Returns YGPU_OK or YGPU_ERR_BAD_ARG. */
int  ygpu_parse_lis_opt(const char* opts, ygpu_dyn_par* par);
/* boundary_code() of yelmo_tools.f90:248; -1 if not recognised. */
int  ygpu_boundary_code(const char* boundaries);
/* Message of the last error on this thread (empty string if none). */
const char* ygpu_last_error(void);
/* Library version string. */
const char* ygpu_version(void);

/*
 * ygpu_calc_velocity_ssa -- GPU replacement of calc_velocity_ssa
 * (src/physics/velocity_ssa.f90:60-357). Same arguments in the same order,
 * with the array extents appended (Fortran assumed shape). Host pointers; the
 * call copies inputs to the device, runs the whole Picard loop there and copies
 * the INOUT/OUT fields back. ssa_mask_acx/acy are read (as set by set_ssa_masks).
 * Returns the status of the last linear solve (0/2/4) or a negative error.
 */
int ygpu_calc_velocity_ssa(
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

/*
 * ygpu_calc_velocity_diva -- GPU replacement of calc_velocity_diva
 * (src/physics/velocity_diva.f90:59-429), without the optional neff_hook.
 * Same arguments in the same order, extents appended. c_bed is read only.
 */
int ygpu_calc_velocity_diva(
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

/*
 * ygpu_set_ssa_masks -- set_ssa_masks (src/physics/solver_ssa_ac.f90:851-943)
 * on the GPU; integer result, bit-exact. lateral_bc is YGPU_LATBC_*.
 */
int ygpu_set_ssa_masks(int* ssa_mask_acx, int* ssa_mask_acy, const int* mask_frnt,
                       const double* f_ice, const double* f_grnd,
                       int lateral_bc, int boundaries, int nx, int ny);

/*
 * ygpu_calc_dyn_inputs -- the fields calc_ydyn builds before the solve, on the
 * GPU, from H_ice, z_bed, z_sl with a binary ice mask (front_subgrid = "none",
 * gl_sep = 1):
 *   f_ice = 1 where H_ice > 0                      (yelmo_topography.f90:1348)
 *   H_grnd                                         calc_H_grnd, topography.f90:876 (use_f_ice=.FALSE.)
 *   z_srf                                          calc_z_srf_max, topography.f90:820
 *   f_grnd, f_grnd_acx, f_grnd_acy                 calc_f_grnd_subgrid_linear, topography.f90:977
 *   mask_frnt                                      calc_ice_front, topography.f90:724
 *   dzsdx, dzsdy                                   calc_gradient_acx/acy, yelmo_tools.f90:341,405
 *   taud_acx, taud_acy                             calc_driving_stress, velocity_general.f90:1118
 *   taul_int_acx, taul_int_acy                     calc_lateral_bc_stress_2D, velocity_general.f90:1453
 * The flotation test and every mask are computed in FP64 without contraction
 * (bit-exact with a CPU evaluation of the same expressions).
 */
int ygpu_calc_dyn_inputs(const double* H_ice, const double* z_bed, const double* z_sl,
                         double* f_ice, double* H_grnd, double* z_srf,
                         double* f_grnd, double* f_grnd_acx, double* f_grnd_acy,
                         int* mask_frnt, double* dzsdx, double* dzsdy,
                         double* taud_acx, double* taud_acy,
                         double* taul_int_acx, double* taul_int_acy,
                         double dx, double grad_lim, double taud_lim,
                         double rho_ice, double rho_sw, double g,
                         int boundaries, int nx, int ny);

/*
 * ygpu_calc_dyn_inputs_bg -- ygpu_calc_dyn_inputs with a uniform background
 * slope (ytopo slope_bg_x, slope_bg_y; yelmo_topography.f90:1373-1374) that
 * z_srf does not contain: it is added to dzsdx and dzsdy before the grad_lim
 * limit (calc_gradient_acx/acy, yelmo_tools.f90:401,470) and so enters the
 * driving stress. The inclined-plane domains (ISMIP-HOM, tests/yelmo_ismiphom.f90:
 * 102-106) carry their mean slope this way on a periodic grid.
 * ygpu_calc_dyn_inputs is this call with both slopes 0.
 */
int ygpu_calc_dyn_inputs_bg(const double* H_ice, const double* z_bed, const double* z_sl,
                            double* f_ice, double* H_grnd, double* z_srf,
                            double* f_grnd, double* f_grnd_acx, double* f_grnd_acy,
                            int* mask_frnt, double* dzsdx, double* dzsdy,
                            double* taud_acx, double* taud_acy,
                            double* taul_int_acx, double* taul_int_acy,
                            double dx, double grad_lim, double taud_lim,
                            double rho_ice, double rho_sw, double g,
                            double slope_bg_x, double slope_bg_y,
                            int boundaries, int nx, int ny);

/*
 * Post-solve diagnostics of calc_ydyn (src/yelmo_dynamics.f90:304-336 and the
 * DIVA depth averages of :642-644), on the GPU. All arrays are (nx,ny) or
 * (nx,ny,nz) column-major like the solver fields; f_ice is f_ice_dyn.
 *   ux_i_bar, uy_i_bar    calc_vertical_integrated_2D(ux_i / uy_i, zeta_aa), yelmo_tools.f90:1064
 *   qq_acx, qq_acy        calc_ice_flux (upwind thickness), velocity_general.f90:1752
 *   qq_gl_acx, qq_gl_acy  calc_grounding_line_flux, velocity_general.f90:1825
 *   qq, taub, taud, uxy_b, uxy_i_bar, uxy_bar, uxy(:,:,k)
 *                         calc_magnitude_from_staggered, yelmo_tools.f90:287
 *   ux_s, uy_s, uxy_s     the top layer of ux, uy, uxy (yelmo_dynamics.f90:330-333)
 *   f_vbvs                calc_vel_ratio(uxy_b, uxy_s), velocity_general.f90:1888
 * Optional groups: ux_i/uy_i/zeta_aa NULL skips the depth averages (ux_i_bar
 * and uy_i_bar are then inputs, or NULL to skip uxy_i_bar); ux/uy NULL skips
 * uxy, the surface fields and f_vbvs. Computed in FP64 without contraction:
 * bit-exact with a CPU evaluation of the same expressions.
 */
typedef struct ygpu_dyn_diag {
    int nx, ny, nz;
    double dx, dy;
    /* inputs */
    const double *ux_bar, *uy_bar, *ux_b, *uy_b, *taub_acx, *taub_acy, *taud_acx, *taud_acy;
    const double *H_ice, *f_ice, *f_grnd;
    const double *ux_i, *uy_i, *zeta_aa;   /* 3D shear velocity (DIVA) and the layers */
    const double *ux, *uy;                 /* 3D velocity */
    /* outputs (ux_i_bar / uy_i_bar: outputs with ux_i, else inputs) */
    double *ux_i_bar, *uy_i_bar;
    double *qq_acx, *qq_acy, *qq, *qq_gl_acx, *qq_gl_acy;
    double *taub, *taud, *uxy_b, *uxy_i_bar, *uxy_bar, *uxy;
    double *ux_s, *uy_s, *uxy_s, *f_vbvs;
} ygpu_dyn_diag;

/* host arrays (staged through the calling thread's default context) */
int ygpu_calc_dyn_diagnostics(const ygpu_dyn_diag* fields, int boundaries);
/* device arrays, on `stream` (a cudaStream_t; NULL: the default stream); asynchronous */
int ygpu_calc_dyn_diagnostics_device(void* stream, const ygpu_dyn_diag* fields, int boundaries);

/*
 * ygpu_calc_gradient_column_ac -- calc_gradient_column_ac
 * (src/yelmo_tools.f90:479-571): the surface or base gradient on the faces for
 * the sigma-coordinate transform, with the cliff at faces to ice-free ocean
 * replaced by the ice-side neighbour face. mask_ocn is nonzero where the bed
 * lies below sea level (calc_ydyn passes z_bed < z_sl,
 * src/yelmo_dynamics.f90:243-246). Host arrays; the _device form takes device
 * arrays and runs on `stream` asynchronously.
 */
int ygpu_calc_gradient_column_ac(double* dvdx_c, double* dvdy_c, const double* dvdx, const double* dvdy,
                                 const double* f_ice, const int* mask_ocn, int boundaries, int nx, int ny);
int ygpu_calc_gradient_column_ac_device(void* stream, double* dvdx_c, double* dvdy_c, const double* dvdx,
                                        const double* dvdy, const double* f_ice, const int* mask_ocn,
                                        int boundaries, int nx, int ny);

/*
 * Velocity Jacobian of calc_ydyn (src/yelmo_dynamics.f90:248-296):
 *   YGPU_JAC_UXY  calc_jacobian_vel_3D_uxyterms (src/physics/deformation.f90:397-716):
 *                 dxz, dyz (three-point unequal-spacing derivatives in z on the faces,
 *                 where the face thickness is positive), dxx, dxy, dyx, dyy (centred,
 *                 one-sided at the ice margin, cross derivatives over faces with a
 *                 velocity solution) with the sigma-transform corrections; dzx, dzy,
 *                 dzz are zeroed (if given), as that routine does.
 *   YGPU_JAC_UZ   calc_jacobian_vel_3D_uzterms (:718-961): dzz, dzx, dzy of uz on
 *                 the fully ice-covered cells, zero elsewhere.
 * Both flags: the two routines in that order, as calc_ydyn runs them for a given uz.
 * ux, uy and the six ux/uy components are (nx,ny,nz_aa); uz and dzx, dzy, dzz are
 * (nx,ny,nz_ac). dzsdx ... dzbdy are the column gradients
 * (ygpu_calc_gradient_column_ac). f_grnd, an argument of both reference routines,
 * is read by neither and is not taken. 3 <= nz_aa, nz_ac <= 1000. FP64; the
 * layer loops carry no division (the vertical derivative in difference form with
 * per-layer weights, reciprocals of dx, dy and H), so results agree with the
 * reference expressions to rounding, not bit for bit.
 */
#define YGPU_JAC_UXY 1
#define YGPU_JAC_UZ  2
typedef struct ygpu_jvel {
    int nx, ny, nz_aa, nz_ac;
    double dx, dy;
    /* inputs */
    const double *ux, *uy, *uz, *H_ice, *f_ice;
    const double *dzsdx, *dzsdy, *dzbdx, *dzbdy;
    const double *zeta_aa, *zeta_ac;
    /* outputs */
    double *dxx, *dxy, *dxz, *dyx, *dyy, *dyz, *dzx, *dzy, *dzz;
} ygpu_jvel;

/*
 * Vertical velocity of calc_ydyn (src/yelmo_dynamics.f90:259-290), by uz_method:
 *   YGPU_UZ_AA   (1) calc_uz_3D_aa (src/physics/velocity_general.f90:683-945): uz
 *                    integrated upward from the kinematic base value with the
 *                    sigma-corrected horizontal divergence, and the advective
 *                    uz_star = uz + coordinate terms;
 *   YGPU_UZ_FLUX (4) calc_uz_3D_flux (:947-1116): uz_star from the layer mass budgets
 *                    with upwind face thicknesses, corrected to the applied transport
 *                    -dHidt_dyn where mask_kin == 1, and uz = uz_star - coordinate terms.
 *   YGPU_UZ_NODES (2) calc_uz_3D (:346-681): the same integration with the base and
 *                    surface gradients, the velocities and the per-layer horizontal
 *                    strain rates (calc_strain_rate_horizontal_2D, deformation.f90:
 *                    1393-1507) taken to the cell centre by the 2D Gauss quadrature;
 *   YGPU_UZ_JAC  (3) calc_uz_3D_jac (:41-344), the namelist default: the divergence
 *                    from the velocity Jacobian's dxx and dyy (jac_dxx, jac_dyy, the
 *                    ux/uy terms of ygpu_calc_jacobian_vel_3D) by the 3D quadrature.
 * The quadratures restate fesm-utils' gq2D/gq3D, which the reference does not vendor:
 * corner values are means of the active faces (acx/acy fields) or of the four cells
 * (aa fields) around each cell corner, and at vertical corners also of the two layers
 * (or ac levels) that meet there; the 2 (2D) or 8 (3D) Gauss-Legendre nodes at
 * +-1/sqrt(3) of the half cell interpolate them bilinearly (trilinearly) and the
 * equal-weight node mean is the cell value. Ice-free cells take dzbdt - max(smb, 0).
 * nz_ac = nz_aa + 1, 2 <= nz_aa <= 1000. ux_bar, uy_bar, dHidt_dyn and mask_kin are
 * read by YGPU_UZ_FLUX only, jac_dxx and jac_dyy by YGPU_UZ_JAC only. uz_srf_err
 * (optional, NULL to skip) is uz_star(:,:,nz_ac) + smb on the fully ice-covered cells
 * and 0 elsewhere (yelmo_dynamics.f90:283-290). FP64, agreeing with the reference
 * expressions to rounding.
 */
#define YGPU_UZ_AA    1
#define YGPU_UZ_NODES 2
#define YGPU_UZ_JAC   3
#define YGPU_UZ_FLUX  4
typedef struct ygpu_uz3d {
    int nx, ny, nz_aa, nz_ac;
    double dx, dy;
    int use_bmb;
    /* inputs */
    const double *ux, *uy, *H_ice, *f_ice, *smb, *bmb, *dzbdt, *dzsdt;
    const double *dzsdx, *dzsdy, *dzbdx, *dzbdy, *zeta_aa, *zeta_ac;
    const double *ux_bar, *uy_bar, *dHidt_dyn;
    const int* mask_kin;
    /* outputs */
    double *uz, *uz_star, *uz_srf_err;
    /* YGPU_UZ_JAC: jvel%dxx, jvel%dyy (nx,ny,nz_aa) */
    const double *jac_dxx, *jac_dyy;
} ygpu_uz3d;

int ygpu_calc_uz_3D(const ygpu_uz3d* f, int boundaries, int method);
int ygpu_calc_uz_3D_device(void* stream, const ygpu_uz3d* f, int boundaries, int method);

/*
 * Strain-rate tensor of calc_ydyn: calc_strain_rate_tensor_jac_quad3D
 * (src/physics/deformation.f90:963-1183, called at src/yelmo_dynamics.f90:299-300)
 * from the velocity Jacobian (the outputs of ygpu_calc_jacobian_vel_3D). On the
 * fully ice-covered cells, per layer: dxx, dyy, dxy = (dxy + dyx)/2, dxz = (dxz +
 * dzx)/2, dyz = (dyz + dzy)/2 at the cell centre by the 3D quadrature of
 * ygpu_calc_uz_3D's note (acx fields with the active x faces, acy fields with the
 * active y faces, dzx and dzy on the two ac levels bounding the layer); the
 * effective strain rate de = sqrt(dxx^2 + dyy^2 + dxx dyy + dxy^2 + dxz^2 + dyz^2),
 * capped at de_max; the divergence div = dxx + dyy; the shear fraction
 * sqrt(dxz^2 + dyz^2)/de (1 where de = 0, 0 on floating cells, clipped to [0,1]).
 * Zero elsewhere. Then the vertical trapezoid integrals of the eight fields over
 * zeta_aa (calc_vertical_integrated_2D, yelmo_tools.f90:1064-1122) and the two
 * eigenvalues of the averaged horizontal tensor, larger first, or 0 when they are
 * not real and distinct (calc_2D_eigen_values, deformation.f90:1542-1595).
 * jvel: dxx, dxy, dxz, dyx, dyy, dyz (nx,ny,nz_aa), dzx, dzy (nx,ny,nz_ac). The 2D
 * outputs may be NULL (skipped). 2 <= nz_aa <= 1000, nz_ac = nz_aa + 1. FP64.
 */
typedef struct ygpu_strain3d {
    int nx, ny, nz_aa, nz_ac;
    double dx, dy;
    double de_max;              /* [a-1] cap of the effective strain rate (ymat de_max) */
    /* inputs */
    const double *dxx, *dxy, *dxz, *dyx, *dyy, *dyz, *dzx, *dzy;
    const double *H_ice, *f_ice, *f_grnd, *zeta_aa, *zeta_ac;
    /* outputs, (nx,ny,nz_aa): strn%dxx ... strn%f_shear */
    double *s_dxx, *s_dyy, *s_dxy, *s_dxz, *s_dyz, *s_de, *s_div, *s_f_shear;
    /* outputs, (nx,ny): strn2D%dxx ... strn2D%f_shear, eps_eig_1, eps_eig_2 */
    double *a_dxx, *a_dyy, *a_dxy, *a_dxz, *a_dyz, *a_de, *a_div, *a_f_shear, *eps_eig_1, *eps_eig_2;
} ygpu_strain3d;

/* host arrays (staged through the calling thread's default context) */
int ygpu_calc_strain_rate_tensor(const ygpu_strain3d* s, int boundaries);
/* device arrays, on `stream` (a cudaStream_t; NULL: the default stream); asynchronous */
int ygpu_calc_strain_rate_tensor_device(void* stream, const ygpu_strain3d* s, int boundaries);

/* host arrays (staged through the calling thread's default context) */
int ygpu_calc_jacobian_vel_3D(const ygpu_jvel* jvel, int boundaries, int terms);
/* device arrays, on `stream` (a cudaStream_t; NULL: the default stream); asynchronous */
int ygpu_calc_jacobian_vel_3D_device(void* stream, const ygpu_jvel* jvel, int boundaries, int terms);

/*
 * ygpu_calc_advec2D_impl_lis -- calc_advec2D with solver = "impl-lis"
 * (src/physics/solver_advection.f90:20-145) on the GPU: the implicit upwind
 * system of linear_solver_matrix_advection_csr_2D (:171-487), assembled on the
 * device, solved with BiCGSTAB and Jacobi to a relative residual of 1e-12
 * (:119), the transport of the MASK_ICE_FIXED cells (calc_fixed_cell_transport,
 * :489-546) and dvdt = (var_new - var)/dt. mask_ice holds MASK_ICE_* (0 none,
 * 1 fixed, 2 dynamic). boundaries is YGPU_BND_* or YGPU_BND_MASK ("mask",
 * whose advection borders are Neumann rows). lin_iter / lin_status: the
 * Krylov iterations and the LIS-style status (0, 2, 4; negative on error).
 */
int ygpu_calc_advec2D_impl_lis(double* dvdt, const double* var, const double* ux, const double* uy,
                               const double* var_dot, const int* mask_ice, const double* var_ref,
                               double dx, double dy, double dt, int boundaries, int nx, int ny,
                               int* lin_iter, int* lin_status);
struct ygpu_ctx;
/*
 * ygpu_calc_dyn_inputs_bg and ygpu_set_ssa_masks on DEVICE arrays, enqueued on
 * ctx's stream without synchronising (same arguments after ctx). A time loop
 * that keeps every field on the device chains them with
 * ygpu_advec2D_impl_lis_device and ygpu_solve_device on the same stream.
 */
int ygpu_calc_dyn_inputs_bg_device(struct ygpu_ctx* ctx, const double* H_ice, const double* z_bed,
                                   const double* z_sl, double* f_ice, double* H_grnd, double* z_srf,
                                   double* f_grnd, double* f_grnd_acx, double* f_grnd_acy, int* mask_frnt,
                                   double* dzsdx, double* dzsdy, double* taud_acx, double* taud_acy,
                                   double* taul_int_acx, double* taul_int_acy, double dx, double grad_lim,
                                   double taud_lim, double rho_ice, double rho_sw, double g,
                                   double slope_bg_x, double slope_bg_y, int boundaries, int nx, int ny);
int ygpu_set_ssa_masks_device(struct ygpu_ctx* ctx, int* ssa_mask_acx, int* ssa_mask_acy, const int* mask_frnt,
                              const double* f_ice, const double* f_grnd, int lateral_bc, int boundaries,
                              int nx, int ny);
/* the same on device arrays, on ctx's stream (scratch from its arena); synchronises */
int ygpu_advec2D_impl_lis_device(struct ygpu_ctx* ctx, double* dvdt, const double* var, const double* ux,
                                 const double* uy, const double* var_dot, const int* mask_ice,
                                 const double* var_ref, double dx, double dy, double dt, int boundaries,
                                 int nx, int ny, int* lin_iter, int* lin_status);

/*
 * ygpu_linear_solver_matrix_solve -- GPU Krylov solve of a CSR system, the
 * drop-in for linear_solver_matrix_solve (solver_linear.F90:151-190) with the
 * linear_solver_class arrays (1-based a_ptr/a_index as Fortran holds them).
 * x_value is the start vector on entry (unless -initx_zeros true) and the
 * solution on return. b == 0 gives x = 0 without iterating (:162-174).
 */
int ygpu_linear_solver_matrix_solve(int nmax, const int* a_ptr, const int* a_index,
                                    const double* a_value, const double* b_value,
                                    double* x_value, const char* lis_opt,
                                    int* lin_iter, int* status, double* L2_rel_norm);

/*
 * neff_hook of calc_velocity_diva (velocity_diva.f90:390-400; the hook of
 * calc_ydyn, src/yelmo_dynamics.f90:357-411): after every Picard iteration the
 * hook recomputes c_bed (in place) from the iteration's basal velocity ux_b,
 * uy_b (host arrays, nx*ny, Fortran order), as a steady hydrology does for the
 * effective pressure; the solve has converged only when c_bed also changed by
 * less than ssa_iter_conv (relative L1). ygpu_set_neff_hook sets the hook of
 * the calling thread (NULL clears it); it applies to the DIVA solves of
 * ygpu_calc_velocity_diva (c_bed is then in/out: the hook receives the caller's
 * array) and of ygpu_solve_device (the hook receives a library buffer and the
 * device c_bed is updated).
 */
typedef void (*ygpu_neff_hook)(void* user, double* c_bed, const double* ux_b, const double* uy_b, int nx, int ny);
void ygpu_set_neff_hook(ygpu_neff_hook hook, void* user);

/* ======================================================================== */
/* Device-resident API: the solve on fields already in GPU memory.           */
/* ======================================================================== */

/* Device pointers of one instance (all FP64, same layout as above). Fields the
   solver kind does not use may be NULL (ux,uy,ux_i,uy_i,duxdz,duydz,beta_eff for
   SSA). */
typedef struct ygpu_fields {
    int nx, ny, nz;
    double dx, dy, n_glen;
    /* in/out state */
    double *ux, *uy, *ux_bar, *uy_bar, *ux_b, *uy_b, *ux_i, *uy_i;
    double *taub_acx, *taub_acy, *beta, *beta_acx, *beta_acy, *beta_eff;
    double *visc_eff, *visc_eff_int, *duxdz, *duydz;
    double *ssa_err_acx, *ssa_err_acy;
    int    *ssa_mask_acx, *ssa_mask_acy;
    /* inputs */
    const double *c_bed, *f_slide, *taud_acx, *taud_acy, *taul_int_acx, *taul_int_acy;
    const double *H_ice, *f_ice, *H_grnd, *f_grnd, *f_grnd_acx, *f_grnd_acy;
    const double *ATT, *zeta_aa, *z_sl, *z_bed, *z_srf;
} ygpu_fields;

typedef struct ygpu_ctx ygpu_ctx;

/* A context owns one CUDA stream and the scratch of its solves. */
ygpu_ctx* ygpu_ctx_create(int device);
void      ygpu_ctx_destroy(ygpu_ctx* ctx);
/* The context's stream, as a cudaStream_t cast to void*. */
void*     ygpu_ctx_stream(ygpu_ctx* ctx);

/* kind: 0 = SSA (calc_velocity_ssa), 1 = DIVA (calc_velocity_diva). */
#define YGPU_KIND_SSA   0
#define YGPU_KIND_DIVA  1

/*
 * Launch tuning of a context (no counterpart in the reference): how often the
 * host checks for finished solves, whether each chunk of Picard iterations
 * between checks runs as one CUDA graph (captured once per launch shape and
 * parameters, then replayed), and the team size (unknowns per CTA of a solve;
 * smaller teams synchronise faster, larger ones have more threads per row).
 * yelmo_gb300/autotune.py picks these by measurement for a workload.
 */
typedef struct ygpu_tuning {
    int check_every;            /* Picard iterations between host checks (1..64), default 4 */
    int use_graphs;             /* 1: chunk graphs (default), 0: one launch per step        */
    int unknowns_per_cta;       /* team sizing, default 512                                 */
    unsigned long long max_active_unknowns; /* batches with more unknowns run as a queue:
                                   continuous batching with at most this many unknowns on the
                                   GPU at once (default 1.5 M; 0: always one lockstep batch)  */
    int spin_log2;              /* for tests of the timeout path: a wait of a team of CTAs
                                   gives up after 2^spin_log2 polls (1..22) instead of 2^22
                                   (0, the default), and the solve returns YGPU_ERR_TIMEOUT */
    int cluster_ctas;           /* 2..16: the Krylov step on thread-block clusters of this
                                   many CTAs (one team = one cluster, the barrier and the
                                   all-reduce inside the cluster); 0 (default) or -1: teams
                                   of CTAs with a global-memory barrier, which measured
                                   faster on the marine DIVA workloads                     */
} ygpu_tuning;
void ygpu_tuning_defaults(ygpu_tuning* t);
int  ygpu_ctx_set_tuning(ygpu_ctx* ctx, const ygpu_tuning* t);

/* One solve on device-resident fields; enqueued on the context stream and
   synchronised before return (stats filled). */
int ygpu_solve_device(ygpu_ctx* ctx, int kind, const ygpu_dyn_par* par,
                      const ygpu_fields* f, ygpu_stats* stats);

/*
 * Batched solve: n_inst independent instances of uneven size. A batch within
 * the context's max_active_unknowns runs in lockstep (every instance on the GPU,
 * one team of CTAs each); a larger one runs as a queue: instances are admitted
 * largest first as others finish, each tick advancing the active ones by one
 * Picard iteration (continuous batching). stats may be NULL or an array of
 * n_inst entries.
 */
int ygpu_solve_batch_device(ygpu_ctx* ctx, int kind, const ygpu_dyn_par* par,
                            int n_inst, const ygpu_fields* inst, ygpu_stats* stats);

/*
 * Batched solve on HOST arrays (no counterpart in the reference): `host` holds
 * n ygpu_fields of host pointers with the layouts and directions of
 * ygpu_calc_velocity_ssa / _diva; the library copies them to the device, solves
 * the batch as ygpu_solve_batch_device on the calling thread's default context
 * and copies the in/out fields back. A single DIVA instance (n_inst = 1) with a
 * neff hook set runs the hook as ygpu_calc_velocity_diva does, and c_bed comes
 * back with the hook's last update.
 */
int ygpu_solve_batch_host(int kind, const ygpu_dyn_par* par, int n_inst, const ygpu_fields* host,
                          ygpu_stats* stats);

/*
 * ygpu_solve_device_noalloc -- no counterpart in the reference.
 * One solve on device-resident fields, like ygpu_solve_device, for callers that
 * cannot allocate device memory: a host whose device memory belongs to another
 * runtime or to a pool allocator that must account for every byte, or a server
 * that must not grow after start-up. The call allocates nothing: its scratch is
 * a fixed array of YGPU_NOALLOC_SCRATCH_BYTES inside the library, held by every
 * GPU that loads the library until the process exits. Instances whose scratch
 * does not fit are rejected with YGPU_ERR_BAD_ARG (a 161x161x10 FP64 solve needs
 * about 24 MB). The first call on a device looks up the array's device address
 * and checks that the kernels' stack (up to about 1.3 KB per thread) fits the
 * context's stack limit, which it does not raise. The call reads the count of finished
 * solves back and synchronises its stream, so it cannot be recorded into a CUDA
 * graph: on a stream that is being captured it returns YGPU_ERR_BAD_ARG and
 * enqueues nothing. All calls share the array and it keeps the last call's contents:
 * calls that overlap on the GPU race, so serialise them. A neff hook is not run
 * here: with one set on the calling thread a DIVA solve returns YGPU_ERR_BAD_ARG.
 * stream is a cudaStream_t (NULL: the legacy default stream); the call returns
 * after that stream has finished the solve. stats->device_ms is 0 (no events
 * are created).
 */
#define YGPU_NOALLOC_SCRATCH_BYTES (64u << 20)
int ygpu_solve_device_noalloc(int kind, const ygpu_dyn_par* par, const ygpu_fields* f,
                              ygpu_stats* stats, void* stream);

/* ======================================================================== */
/* Serving: velocity-solve requests from many ensemble members.              */
/* ======================================================================== */
/*
 * No counterpart in the reference, which solves one domain per call
 * (calc_ydyn -> calc_velocity_*, src/yelmo_dynamics.f90:415,544). A server
 * keeps the state of every registered member on the device (thickness, bed,
 * friction, rate factor, viscosity and the previous velocity) and solves the
 * requests it is sent with continuous batching: a loop on a host thread runs
 * one Picard iteration of every solve on the GPU per tick (the pre / Krylov /
 * post step kernels over all of them), retires the solves that converged and
 * admits waiting requests into the freed slots between ticks, so requests that
 * arrive while others are on the GPU join them at the next tick.
 *
 * A request advances its member by one step: H_ice += dH where H_ice > 0
 * (dH ~ N(0, dH_sigma^2) per cell, drawn from (seed, member, step) with a
 * counter-based generator and clamped at 0), rebuilds the inputs of the solve
 * on the device (ygpu_calc_dyn_inputs, ygpu_set_ssa_masks) and solves warm
 * from the member's previous velocity and viscosity. Requests of one member
 * run in submission order, one at a time.
 *
 * Admission by device memory: the server never holds more than hbm_budget
 * bytes. Admission by load: at most max_slots solves and max_active_unknowns
 * unknowns are on the GPU at once. A member that does not fit is refused (YGPU_ERR_ADMISSION); a request
 * waits until a slot (the scratch of one solve, sized for the largest member)
 * is free or can be allocated within the budget.
 */
typedef struct ygpu_server ygpu_server;

typedef struct ygpu_server_cfg {
    int    device;              /* CUDA device                                   */
    int    kind;                /* YGPU_KIND_SSA or YGPU_KIND_DIVA               */
    ygpu_dyn_par par;           /* solver parameters of every request            */
    double grad_lim;            /* surface-gradient limit (ytopo grad_lim)       */
    double taud_lim;            /* driving-stress clamp (Pa)                     */
    int    lateral_bc;          /* YGPU_LATBC_*                                  */
    double dH_sigma;            /* standard deviation of the per-step dH (m)     */
    unsigned long long hbm_budget; /* device bytes the server may hold         */
    int    max_slots;           /* solves on the GPU at once (0: one per SM)     */
    unsigned long long max_active_unknowns; /* admission also stops at this many unknowns
                                   on the GPU (0: 1.5 M)                           */
} ygpu_server_cfg;

typedef struct ygpu_server_info {
    int    members, slots, active, pending;
    long long ticks, completed;
    unsigned long long bytes_held;
} ygpu_server_info;

/* fields for ygpu_server_fetch */
#define YGPU_SRV_UX    0        /* solve velocity x: ux_bar (DIVA) / ux_b (SSA)  */
#define YGPU_SRV_UY    1
#define YGPU_SRV_VISC  2        /* visc_eff, nx*ny*nz                            */
#define YGPU_SRV_H     3        /* H_ice                                         */
#define YGPU_SRV_UXB   4        /* ux_b                                          */
#define YGPU_SRV_UYB   5
#define YGPU_SRV_TAUBX 6        /* taub_acx                                      */
#define YGPU_SRV_TAUBY 7        /* taub_acy                                      */
#define YGPU_SRV_BETA  8        /* beta (aa-nodes)                               */
#define YGPU_SRV_BETAX 9        /* beta_acx                                      */
#define YGPU_SRV_BETAY 10       /* beta_acy                                      */

/* NULL on error (ygpu_last_error). Starts the serving thread. */
ygpu_server* ygpu_server_create(const ygpu_server_cfg* cfg);
/* Stops the thread after the solves on the GPU finish; frees everything. */
void ygpu_server_destroy(ygpu_server* srv);
/*
 * Registers a member from HOST arrays laid out like ygpu_fields (nx, ny, nz,
 * dx, dy, n_glen set). Read: H_ice, z_bed, z_sl, c_bed, f_slide, ATT, zeta_aa,
 * and where not NULL the initial beta, visc_eff (else 1e5 Pa a), velocities and
 * basal stress (else 0). The other inputs are built on the device per request.
 */
int ygpu_server_add_member(ygpu_server* srv, const ygpu_fields* host, int* member_id);
/* Queues one step of a member; thread-safe. */
int ygpu_server_submit(ygpu_server* srv, int member, unsigned long long seed, int* request_id);
/* 1 when the request has finished, 0 while it waits or runs, <0 on a bad id. */
int ygpu_server_poll(ygpu_server* srv, int request_id);
/* Waits up to timeout_s (<0: no limit); returns the solve status, or
   YGPU_ERR_BUSY on timeout. latency_ms: submit to completion. */
int ygpu_server_wait(ygpu_server* srv, int request_id, double timeout_s, ygpu_stats* stats,
                     double* latency_ms);
/* Copies a member field to a host buffer; YGPU_ERR_BUSY while it is solving. */
int ygpu_server_fetch(ygpu_server* srv, int member, int field, double* host);
/*
 * Checkpoint and restart of a member. Its evolving state is the thickness and
 * the warm start of its next solve: YGPU_SRV_H, _UX, _UY, _UXB, _UYB, _VISC,
 * _TAUBX, _TAUBY, _BETA, _BETAX, _BETAY (fetched while it is idle), plus the
 * count of its requests admitted so far. Registering those arrays with the
 * member's fixed inputs (z_bed, z_sl, c_bed, f_slide, ATT, zeta_aa) through
 * ygpu_server_add_member, under the same member id (members added in the same
 * order: the id keys the thickness perturbations), and setting the count with
 * ygpu_server_set_member_steps resumes it: its next request solves the state
 * the uninterrupted server's would. The step count can only be set while the
 * member is idle with no request of it waiting (else YGPU_ERR_BUSY).
 */
int ygpu_server_member_steps(ygpu_server* srv, int member, unsigned long long* steps);
int ygpu_server_set_member_steps(ygpu_server* srv, int member, unsigned long long steps);
int ygpu_server_get_info(ygpu_server* srv, ygpu_server_info* info);

/* ======================================================================== */
/* Launch accounting (no counterpart in the reference; for benchmarks).      */
/* ======================================================================== */
/* Kernels this library has launched in the process so far. */
unsigned long long ygpu_kernel_launches(void);
/* on != 0: time every solver step launch with CUDA events on its stream (and
   clear the totals); 0: stop. Steps: 0 setup, 1 pre, 2 Krylov, 3 post, 4 final. */
void ygpu_step_timing(int on);
/* Device milliseconds and launch counts per step since ygpu_step_timing(1). */
void ygpu_step_timing_get(double ms[5], long long count[5]);

#ifdef __cplusplus
}
#endif

#endif /* YELMO_GPU_H */
