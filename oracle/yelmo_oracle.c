/*
 * yelmo_oracle.c -- CPU FP64 restatement of Yelmo's SSA/DIVA velocity solve.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): used by tests/, the smoke check of
 * __graft_entry__.py and the CPU-baseline leg of bench.py. The GPU library
 * never links or calls this file. See yelmo_oracle.h for provenance and pinning.
 *
 * Indexing: 0-based (i,j) with column-major storage, idx = i + nx*j; 3D fields
 * idx = i + nx*(j + ny*k), k = 0 at the ice base. Built with
 * -ffp-contract=off so that every expression rounds as written.
 */
#include "yelmo_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ID2(i, j) ((size_t)(i) + (size_t)nx * (size_t)(j))
#define ID3(i, j, k) ((size_t)(i) + (size_t)nx * ((size_t)(j) + (size_t)ny * (size_t)(k)))

static const double TOL_UNDERFLOW = 1e-15;   /* yelmo_defs.f90:65 */
static const double VISC_MIN = 1e5;          /* velocity_*.f90 visc_min */

enum { MASK_FRNT_ICE_FREE = -1, MASK_FRNT_ICE_FREE_LAND = -2, MASK_FRNT_NONE = 0,
       MASK_FRNT_FLOAT = 1, MASK_FRNT_MARINE = 2, MASK_FRNT_GRND = 3 }; /* yelmo_defs.f90:75-80 */

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ======================================================================== */
/* Grid helpers                                                             */
/* ======================================================================== */

/* get_neighbor_indices_bc_codes, yelmo_tools.f90:118-201 (0-based) */
static inline void nbr(int i, int j, int nx, int ny, int bc, int* im1, int* ip1, int* jm1, int* jp1) {
    int wrapx = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_X);
    int wrapy = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_Y || bc == YGPU_BND_MISMIP3D ||
                 bc == YGPU_BND_TROUGH);
    if (wrapx) {
        *im1 = (i == 0) ? nx - 1 : i - 1;
        *ip1 = (i == nx - 1) ? 0 : i + 1;
    } else {
        *im1 = (i > 0) ? i - 1 : 0;
        *ip1 = (i < nx - 1) ? i + 1 : nx - 1;
    }
    if (wrapy) {
        *jm1 = (j == 0) ? ny - 1 : j - 1;
        *jp1 = (j == ny - 1) ? 0 : j + 1;
    } else {
        *jm1 = (j > 0) ? j - 1 : 0;
        *jp1 = (j < ny - 1) ? j + 1 : ny - 1;
    }
}

/* get_periodic_directions, yelmo_tools.f90:203-246 */
static void periodic_dirs(int bc, int* px, int* py) {
    *px = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_X);
    *py = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_Y || bc == YGPU_BND_MISMIP3D ||
           bc == YGPU_BND_TROUGH);
}

/* Border types of the assemblers (solver_ssa_ac.f90:149-210): index 0..3 = bcs(1..4):
   1 right (x), 2 upper (y), 3 left (x), 4 lower (y). */
static void border_types(int bc, int per[4], int fre[4]) {
    /* 0 no-slip, 1 free-slip, 2 periodic */
    int t[4];
    switch (bc) {
        case YGPU_BND_MISMIP3D:
        case YGPU_BND_TROUGH: t[0] = 1; t[1] = 2; t[2] = 0; t[3] = 2; break;
        case YGPU_BND_PERIODIC: t[0] = t[1] = t[2] = t[3] = 2; break;
        case YGPU_BND_PERIODIC_X: t[0] = 2; t[1] = 1; t[2] = 2; t[3] = 1; break;
        case YGPU_BND_PERIODIC_Y: t[0] = 1; t[1] = 2; t[2] = 1; t[3] = 2; break;
        case YGPU_BND_INFINITE: t[0] = t[1] = t[2] = t[3] = 1; break;
        default: t[0] = t[1] = t[2] = t[3] = 0; break;
    }
    for (int k = 0; k < 4; k++) {
        per[k] = (t[k] == 2);
        fre[k] = (t[k] == 1);
    }
}

/* integrate_trapezoid1D_pt, yelmo_tools.f90:1092-1122 */
static double trapz_pt(const double* v, const double* z, int nk, size_t stride) {
    double s = 0.0;
    for (int k = 1; k < nk; k++) {
        double mid = 0.5 * (v[k * stride] + v[(k - 1) * stride]);
        s = s + mid * (z[k] - z[k - 1]);
    }
    return s;
}

/* calc_staggered_margin, velocity_diva.f90:1052-1082 */
static inline double stag_margin(double v0, double v1, double f0, double f1) {
    if (f0 == 1.0 && f1 < 1.0) return v0;
    if (f0 < 1.0 && f1 == 1.0) return v1;
    return 0.5 * (v0 + v1);
}

/* ======================================================================== */
/* Gaussian quadrature (fesm-utils gq2D, restated; see yelmo_oracle.h)      */
/* ======================================================================== */

/* Node q (0 SW, 1 SE, 2 NE, 3 NW) at (sx*g, sy*g), g = 1/sqrt(3); bilinear
   weight of corner c (same order) = (1 + sx_q*sx_c*g)*(1 + sy_q*sy_c*g)/4. */
static double GQW[4][4];
static int gq_ready = 0;
static const int GQ_SX[4] = {-1, 1, 1, -1};
static const int GQ_SY[4] = {-1, -1, 1, 1};

static void gq_init(void) {
    if (gq_ready) return;
    double g = 1.0 / sqrt(3.0);
    for (int q = 0; q < 4; q++)
        for (int c = 0; c < 4; c++) {
            double ax = 1.0 + (double)(GQ_SX[q] * GQ_SX[c]) * g;
            double ay = 1.0 + (double)(GQ_SY[q] * GQ_SY[c]) * g;
            GQW[q][c] = (ax * ay) * 0.25;
        }
    gq_ready = 1;
}

static inline void gq_corners_to_nodes(const double c[4], double v[4]) {
    for (int q = 0; q < 4; q++) {
        double s = GQW[q][0] * c[0];
        s = s + GQW[q][1] * c[1];
        s = s + GQW[q][2] * c[2];
        s = s + GQW[q][3] * c[3];
        v[q] = s;
    }
}

static inline double mean2_act(double a, double b, int aa, int ab) {
    int n = aa + ab;
    if (n == 0) return 0.0;
    double s = (aa ? a : 0.0) + (ab ? b : 0.0);
    return s / (double)n;
}

static inline double mean4_act(double a, double b, double c, double d, int aa, int ab, int ac, int ad) {
    /* mean4_active, deformation.f90:1370-1391 */
    int n = aa + ab + ac + ad;
    if (n == 0) return 0.0;
    double s = (aa ? a : 0.0) + (ab ? b : 0.0);
    s = s + (ac ? c : 0.0);
    s = s + (ad ? d : 0.0);
    return s / (double)n;
}

/* gq2D_to_nodes_aa: corner = mean of the 4 cells around it (act: active only) */
static void gq_nodes_aa(const double* var, const unsigned char* act, int i, int j, int im1, int ip1,
                        int jm1, int jp1, int nx, double v[4]) {
    double c[4];
    int ii[4][4] = {{im1, i, im1, i}, {i, ip1, i, ip1}, {i, ip1, i, ip1}, {im1, i, im1, i}};
    int jj[4][4] = {{jm1, jm1, j, j}, {jm1, jm1, j, j}, {j, j, jp1, jp1}, {j, j, jp1, jp1}};
    for (int q = 0; q < 4; q++) {
        double a0 = var[ID2(ii[q][0], jj[q][0])], a1 = var[ID2(ii[q][1], jj[q][1])];
        double a2 = var[ID2(ii[q][2], jj[q][2])], a3 = var[ID2(ii[q][3], jj[q][3])];
        if (act) {
            c[q] = mean4_act(a0, a1, a2, a3, act[ID2(ii[q][0], jj[q][0])], act[ID2(ii[q][1], jj[q][1])],
                             act[ID2(ii[q][2], jj[q][2])], act[ID2(ii[q][3], jj[q][3])]);
        } else {
            double s = a0 + a1;
            s = s + a2;
            s = s + a3;
            c[q] = 0.25 * s;
        }
    }
    gq_corners_to_nodes(c, v);
}

/* gq2D_to_nodes_acx: corner = mean of the two acx faces above/below it */
static void gq_nodes_acx(const double* var, const unsigned char* act, int i, int j, int im1, int jm1,
                         int jp1, int nx, double v[4]) {
    double c[4];
    int ic[4] = {im1, i, i, im1};
    int ja[4] = {jm1, jm1, j, j};
    int jb[4] = {j, j, jp1, jp1};
    for (int q = 0; q < 4; q++) {
        double a = var[ID2(ic[q], ja[q])], b = var[ID2(ic[q], jb[q])];
        if (act)
            c[q] = mean2_act(a, b, act[ID2(ic[q], ja[q])], act[ID2(ic[q], jb[q])]);
        else
            c[q] = 0.5 * (a + b);
    }
    gq_corners_to_nodes(c, v);
}

/* gq2D_to_nodes_acy: corner = mean of the two acy faces left/right of it */
static void gq_nodes_acy(const double* var, const unsigned char* act, int i, int j, int im1, int ip1,
                         int jm1, int nx, double v[4]) {
    double c[4];
    int ia[4] = {im1, i, i, im1};
    int ib[4] = {i, ip1, ip1, i};
    int jc[4] = {jm1, jm1, j, j};
    for (int q = 0; q < 4; q++) {
        double a = var[ID2(ia[q], jc[q])], b = var[ID2(ib[q], jc[q])];
        if (act)
            c[q] = mean2_act(a, b, act[ID2(ia[q], jc[q])], act[ID2(ib[q], jc[q])]);
        else
            c[q] = 0.5 * (a + b);
    }
    gq_corners_to_nodes(c, v);
}

static inline double gq_mean(const double v[4]) {
    double s = v[0] + v[1];
    s = s + v[2];
    s = s + v[3];
    return s / 4.0;
}

/* ======================================================================== */
/* Strain rates and viscosity                                               */
/* ======================================================================== */

/* calc_active_faces, deformation.f90:1316-1344 */
static void active_faces(unsigned char* ax, unsigned char* ay, const double* f_ice, int bc, int nx, int ny) {
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            ax[ID2(i, j)] = (f_ice[ID2(i, j)] == 1.0 || f_ice[ID2(ip1, j)] == 1.0);
            ay[ID2(i, j)] = (f_ice[ID2(i, j)] == 1.0 || f_ice[ID2(i, jp1)] == 1.0);
        }
}

/* deriv_active, deformation.f90:1346-1368 */
static inline double deriv_active(double vm, double v0, double vp, int am, int ap, double h) {
    if (am && ap) return (vp - vm) / (2.0 * h);
    if (ap) return (vp - v0) / h;
    if (am) return (v0 - vm) / h;
    return 0.0;
}

/* calc_strain_rate_horizontal_2D, deformation.f90:1393-1507 */
static void strain_rate_2D(double* dudx, double* dudy, double* dvdx, double* dvdy, const double* ux,
                           const double* uy, const double* f_ice, const unsigned char* ax,
                           const unsigned char* ay, double dx, double dy, int bc, int nx, int ny) {
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1, im2, ip2, jm2, jp2, d1, d2, d3;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            dudx[c] = (ux[ID2(ip1, j)] - ux[ID2(im1, j)]) / (2.0 * dx);
            dudy[c] = deriv_active(ux[ID2(i, jm1)], ux[c], ux[ID2(i, jp1)], ax[ID2(i, jm1)], ax[ID2(i, jp1)], dy);
            dvdx[c] = deriv_active(uy[ID2(im1, j)], uy[c], uy[ID2(ip1, j)], ay[ID2(im1, j)], ay[ID2(ip1, j)], dx);
            dvdy[c] = (uy[ID2(i, jp1)] - uy[ID2(i, jm1)]) / (2.0 * dy);

            if (f_ice[c] == 1.0 && f_ice[ID2(ip1, j)] < 1.0) {
                nbr(im1, j, nx, ny, bc, &im2, &d1, &d2, &d3);
                if (f_ice[ID2(im1, j)] == 1.0 && im2 != im1)
                    dudx[c] = (1.0 * ux[ID2(im2, j)] - 4.0 * ux[ID2(im1, j)] + 3.0 * ux[c]) / (2.0 * dx);
                else
                    dudx[c] = (ux[c] - ux[ID2(im1, j)]) / dx;
            } else if (f_ice[c] < 1.0 && f_ice[ID2(ip1, j)] == 1.0) {
                nbr(ip1, j, nx, ny, bc, &d1, &ip2, &d2, &d3);
                if (ip2 != ip1 && f_ice[ID2(ip2, j)] == 1.0)
                    dudx[c] = -(1.0 * ux[ID2(ip2, j)] - 4.0 * ux[ID2(ip1, j)] + 3.0 * ux[c]) / (2.0 * dx);
                else
                    dudx[c] = (ux[ID2(ip1, j)] - ux[c]) / dx;
            }

            if (f_ice[c] == 1.0 && f_ice[ID2(i, jp1)] < 1.0) {
                nbr(i, jm1, nx, ny, bc, &d1, &d2, &jm2, &d3);
                if (f_ice[ID2(i, jm1)] == 1.0 && jm2 != jm1)
                    dvdy[c] = (1.0 * uy[ID2(i, jm2)] - 4.0 * uy[ID2(i, jm1)] + 3.0 * uy[c]) / (2.0 * dy);
                else
                    dvdy[c] = (uy[c] - uy[ID2(i, jm1)]) / dy;
            } else if (f_ice[c] < 1.0 && f_ice[ID2(i, jp1)] == 1.0) {
                nbr(i, jp1, nx, ny, bc, &d1, &d2, &d3, &jp2);
                if (jp2 != jp1 && f_ice[ID2(i, jp2)] == 1.0)
                    dvdy[c] = -(1.0 * uy[ID2(i, jp2)] - 4.0 * uy[ID2(i, jp1)] + 3.0 * uy[c]) / (2.0 * dy);
                else
                    dvdy[c] = (uy[ID2(i, jp1)] - uy[c]) / dy;
            }
        }
}

/* calc_visc_eff_3D_nodes: SSA velocity_ssa.f90:359-488 (duxdz == NULL),
   DIVA velocity_diva.f90:573-710 (with duxdz/duydz) */
static void visc_3D_nodes(double* visc, const double* ux, const double* uy, const double* duxdz,
                          const double* duydz, const double* ATT, const double* f_ice, double dx,
                          double dy, double n_glen, double eps_0, int bc, int nx, int ny, int nz) {
    gq_init();
    size_t n2 = (size_t)nx * ny;
    unsigned char* ax = malloc(n2);
    unsigned char* ay = malloc(n2);
    double* dudx = malloc(n2 * sizeof(double));
    double* dudy = malloc(n2 * sizeof(double));
    double* dvdx = malloc(n2 * sizeof(double));
    double* dvdy = malloc(n2 * sizeof(double));
    active_faces(ax, ay, f_ice, bc, nx, ny);
    double p1 = (1.0 - n_glen) / (2.0 * n_glen);
    double p2 = -1.0 / n_glen;
    double eps0sq = eps_0 * eps_0;
    strain_rate_2D(dudx, dudy, dvdx, dvdy, ux, uy, f_ice, ax, ay, dx, dy, bc, nx, ny);
#pragma omp parallel for collapse(2) schedule(dynamic, 64)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            if (f_ice[ID2(i, j)] == 1.0) {
                int im1, ip1, jm1, jp1;
                nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
                double dudxn[4], dudyn[4], dvdxn[4], dvdyn[4], dudzn[4], dvdzn[4], ATTn[4], vn[4], e2[4];
                gq_nodes_acx(dudx, ax, i, j, im1, jm1, jp1, nx, dudxn);
                gq_nodes_acx(dudy, ax, i, j, im1, jm1, jp1, nx, dudyn);
                gq_nodes_acy(dvdx, ay, i, j, im1, ip1, jm1, nx, dvdxn);
                gq_nodes_acy(dvdy, ay, i, j, im1, ip1, jm1, nx, dvdyn);
                for (int k = 0; k < nz; k++) {
                    if (duxdz) {
                        gq_nodes_acx(duxdz + (size_t)k * n2, ax, i, j, im1, jm1, jp1, nx, dudzn);
                        gq_nodes_acy(duydz + (size_t)k * n2, ay, i, j, im1, ip1, jm1, nx, dvdzn);
                    }
                    for (int q = 0; q < 4; q++) {
                        double sh = dudyn[q] + dvdxn[q];
                        double e = dudxn[q] * dudxn[q] + dvdyn[q] * dvdyn[q];
                        e = e + dudxn[q] * dvdyn[q];
                        e = e + 0.25 * (sh * sh);
                        if (duxdz) {
                            e = e + 0.25 * (dudzn[q] * dudzn[q]);
                            e = e + 0.25 * (dvdzn[q] * dvdzn[q]);
                        }
                        e2[q] = e + eps0sq;
                    }
                    gq_nodes_aa(ATT + (size_t)k * n2, NULL, i, j, im1, ip1, jm1, jp1, nx, ATTn);
                    for (int q = 0; q < 4; q++) vn[q] = 0.5 * pow(e2[q], p1) * pow(ATTn[q], p2);
                    visc[ID3(i, j, k)] = gq_mean(vn);
                }
            } else {
                for (int k = 0; k < nz; k++) visc[ID3(i, j, k)] = VISC_MIN;
            }
        }
    free(ax); free(ay); free(dudx); free(dudy); free(dvdx); free(dvdy);
}

/* calc_visc_eff_3D_aa: SSA velocity_ssa.f90:490-586, DIVA velocity_diva.f90:712-822 */
static void visc_3D_aa(double* visc, const double* ux, const double* uy, const double* duxdz,
                       const double* duydz, const double* ATT, const double* f_ice, double dx, double dy,
                       double n_glen, double eps_0, int bc, int nx, int ny, int nz) {
    double p1 = (1.0 - n_glen) / (2.0 * n_glen);
    double p2 = -1.0 / n_glen;
    double eps0sq = eps_0 * eps_0;
    size_t n2 = (size_t)nx * ny;
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            if (f_ice[ID2(i, j)] != 1.0) {
                for (int k = 0; k < nz; k++) visc[ID3(i, j, k)] = VISC_MIN;
                continue;
            }
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            double dudx = (ux[ID2(i, j)] - ux[ID2(im1, j)]) / dx;
            double dvdy = (uy[ID2(i, j)] - uy[ID2(i, jm1)]) / dy;
            double dudy1 = (ux[ID2(i, jp1)] - ux[ID2(i, jm1)]) / (2.0 * dy);
            double dudy2 = (ux[ID2(im1, jp1)] - ux[ID2(im1, jm1)]) / (2.0 * dy);
            double dudy = 0.5 * (dudy1 + dudy2);
            double dvdx1 = (uy[ID2(ip1, j)] - uy[ID2(im1, j)]) / (2.0 * dx);
            double dvdx2 = (uy[ID2(ip1, jm1)] - uy[ID2(im1, jm1)]) / (2.0 * dx);
            double dvdx = 0.5 * (dvdx1 + dvdx2);
            double sh = dudy + dvdx;
            double e0 = dudx * dudx + dvdy * dvdy;
            e0 = e0 + dudx * dvdy;
            e0 = e0 + 0.25 * (sh * sh);
            for (int k = 0; k < nz; k++) {
                double e = e0;
                if (duxdz) {
                    double dzx = 0.5 * (duxdz[k * n2 + ID2(i, j)] + duxdz[k * n2 + ID2(im1, j)]);
                    double dzy = 0.5 * (duydz[k * n2 + ID2(i, j)] + duydz[k * n2 + ID2(i, jm1)]);
                    e = e + 0.25 * (dzx * dzx);
                    e = e + 0.25 * (dzy * dzy);
                }
                e = e + eps0sq;
                visc[ID3(i, j, k)] = 0.5 * pow(e, p1) * pow(ATT[ID3(i, j, k)], p2);
            }
        }
}

/* picard_relax_visc, velocity_general.f90:2188-2213 */
static void relax_visc(double* visc, const double* visc_prev, double rel, size_t n) {
#pragma omp parallel for
    for (size_t c = 0; c < n; c++) visc[c] = exp((1.0 - rel) * log(visc_prev[c]) + rel * log(visc[c]));
}

/* calc_visc_eff_int, velocity_general.f90:2215-2261 */
static void visc_eff_int_calc(double* vint, const double* visc, const double* H, const double* f_ice,
                              const double* zeta, int nx, int ny, int nz) {
    size_t n2 = (size_t)nx * ny;
#pragma omp parallel for
    for (size_t c = 0; c < n2; c++) {
        double v;
        if (f_ice[c] == 1.0)
            v = trapz_pt(visc + c, zeta, nz, n2) * H[c];
        else
            v = VISC_MIN;
        if (v < VISC_MIN) v = VISC_MIN;
        vint[c] = v;
    }
}

/* ======================================================================== */
/* Basal friction (basal_dragging.f90)                                      */
/* ======================================================================== */

/* calc_beta_aa_power_plastic :949-1068 (coulomb=0), calc_beta_aa_reg_coulomb :1070-1194 (coulomb=1) */
static void beta_law(double* beta, const double* ux_b, const double* uy_b, const double* c_bed,
                     const double* f_ice, const double* f_grnd, double q, double u0, int bc, int simple,
                     int coulomb, int nx, int ny) {
    gq_init();
    const double ub_min = 1e-3, ub_sq_min = ub_min * ub_min;
    size_t n2 = (size_t)nx * ny;
    unsigned char* ax = malloc(n2);
    unsigned char* ay = malloc(n2);
    unsigned char* aa = malloc(n2);
    active_faces(ax, ay, f_ice, bc, nx, ny);
    for (size_t c = 0; c < n2; c++) aa[c] = (f_ice[c] == 1.0 && f_grnd[c] > 0.0);
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            if (f_ice[c] == 1.0) {
                double cbn[4], uxn[4], uyn[4], bn[4];
                if (simple) {
                    double ucx = 0.5 * (ux_b[c] + ux_b[ID2(im1, j)]);
                    double ucy = 0.5 * (uy_b[c] + uy_b[ID2(i, jm1)]);
                    for (int k = 0; k < 4; k++) { cbn[k] = c_bed[c]; uxn[k] = ucx; uyn[k] = ucy; }
                } else {
                    gq_nodes_aa(c_bed, aa, i, j, im1, ip1, jm1, jp1, nx, cbn);
                    gq_nodes_acx(ux_b, ax, i, j, im1, jm1, jp1, nx, uxn);
                    gq_nodes_acy(uy_b, ay, i, j, im1, ip1, jm1, nx, uyn);
                }
                for (int k = 0; k < 4; k++) {
                    double s = uxn[k] * uxn[k] + uyn[k] * uyn[k];
                    double uxy = sqrt(s + ub_sq_min);
                    double fac = coulomb ? pow(uxy / (uxy + u0), q) : pow(uxy / u0, q);
                    bn[k] = cbn[k] * fac * (1.0 / uxy);
                }
                beta[c] = gq_mean(bn);
            } else {
                double uxy = ub_min;
                double fac = coulomb ? pow(uxy / (uxy + u0), q) : pow(uxy / u0, q);
                beta[c] = c_bed[c] * fac * (1.0 / uxy);
            }
        }
    free(ax); free(ay); free(aa);
}

/* calc_beta, basal_dragging.f90:384-579 */
static void calc_beta(double* beta, const double* c_bed, const double* f_slide, const double* ux_b,
                      const double* uy_b, const double* H_ice, const double* f_ice, const double* H_grnd,
                      const double* f_grnd, const double* z_bed, const double* z_sl, const ygpu_dyn_par* p,
                      int nx, int ny) {
    size_t n2 = (size_t)nx * ny;
    int bc = p->boundaries;
    if (p->beta_method == -1) return;
    switch (p->beta_method) {
        case 0: for (size_t c = 0; c < n2; c++) beta[c] = p->beta_const; break;
        case 1: beta_law(beta, ux_b, uy_b, c_bed, f_ice, f_grnd, 1.0, p->beta_u0, bc, 0, 0, nx, ny); break;
        case 2: beta_law(beta, ux_b, uy_b, c_bed, f_ice, f_grnd, p->beta_q, p->beta_u0, bc, 0, 0, nx, ny); break;
        case 3: beta_law(beta, ux_b, uy_b, c_bed, f_ice, f_grnd, p->beta_q, p->beta_u0, bc, 0, 1, nx, ny); break;
        case 4: beta_law(beta, ux_b, uy_b, c_bed, f_ice, f_grnd, p->beta_q, p->beta_u0, bc, 1, 0, nx, ny); break;
        case 5: beta_law(beta, ux_b, uy_b, c_bed, f_ice, f_grnd, p->beta_q, p->beta_u0, bc, 1, 1, nx, ny); break;
        default: return;
    }
    double q_frz = (p->beta_method == 0 || p->beta_method == 1) ? 1.0 : p->beta_q;
    for (size_t c = 0; c < n2; c++) beta[c] = beta[c] * pow(f_slide[c], -q_frz);

    switch (p->beta_gl_scale) {
        case 0: { /* scale_beta_gl_fraction :1202-1254 */
            double* tmp = malloc(n2 * sizeof(double));
            memcpy(tmp, beta, n2 * sizeof(double));
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    int im1, ip1, jm1, jp1;
                    nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
                    if (f_grnd[ID2(i, j)] > 0.0 &&
                        (f_grnd[ID2(im1, j)] == 0.0 || f_grnd[ID2(ip1, j)] == 0.0 ||
                         f_grnd[ID2(i, jm1)] == 0.0 || f_grnd[ID2(i, jp1)] == 0.0))
                        tmp[ID2(i, j)] = beta[ID2(i, j)] * p->beta_gl_f;
                }
            memcpy(beta, tmp, n2 * sizeof(double));
            free(tmp);
        } break;
        case 1: /* scale_beta_gl_Hgrnd :1256-1294 */
            for (size_t c = 0; c < n2; c++) {
                double hg = H_grnd[c] < p->H_grnd_lim ? H_grnd[c] : p->H_grnd_lim;
                double f = hg / p->H_grnd_lim;
                if (f < 0.0) f = 0.0;
                beta[c] = beta[c] * f;
            }
            break;
        case 2: { /* scale_beta_gl_zstar :1296-1352 */
            double rsi = p->rho_sw / p->rho_ice;
            for (size_t c = 0; c < n2; c++) {
                if (f_ice[c] > 0.0) {
                    double Heff = (f_ice[c] > 0.0) ? H_ice[c] / f_ice[c] : H_ice[c];
                    if (f_ice[c] < 1.0) Heff = 0.0;
                    double f;
                    if (z_bed[c] > z_sl[c]) f = Heff;
                    else {
                        f = Heff - (z_sl[c] - z_bed[c]) * rsi;
                        if (f < 0.0) f = 0.0;
                    }
                    if (Heff > 0.0) f = f / Heff;
                    beta[c] = beta[c] * f;
                }
            }
        } break;
        case 3:
            for (size_t c = 0; c < n2; c++) beta[c] = f_grnd[c] * beta[c];
            break;
        default: break;
    }
    for (size_t c = 0; c < n2; c++)
        if (f_grnd[c] == 0.0) beta[c] = 0.0;
    if (bc == YGPU_BND_MISMIP3D) {
        for (int j = 0; j < ny; j++) beta[ID2(0, j)] = beta[ID2(1, j)];
    } else if (bc == YGPU_BND_INFINITE) {
        for (int j = 0; j < ny; j++) beta[ID2(0, j)] = beta[ID2(1, j)];
        for (int j = 0; j < ny; j++) beta[ID2(nx - 1, j)] = beta[ID2(nx - 2, j)];
        for (int i = 0; i < nx; i++) beta[ID2(i, 0)] = beta[ID2(i, 1)];
        for (int i = 0; i < nx; i++) beta[ID2(i, ny - 1)] = beta[ID2(i, ny - 2)];
    }
    for (size_t c = 0; c < n2; c++)
        if (beta[c] > 0.0 && beta[c] < p->beta_min) beta[c] = p->beta_min;
}

/* calc_beta_gl_flux_weight, basal_dragging.f90:1760-1845 */
static double beta_gl_flux_weight(double beta_a, double ux_a, double ux_b, double H_a, double H_b,
                                  double f_grnd_ac) {
    double q_a = ux_a * H_a, q_b = ux_b * H_b;
    double ug = 0.0, ut = 0.0;
    for (int n = 1; n <= 100; n++) {
        double lam = ((double)n - 0.5) / 100.0;
        double Hn = H_a * lam + H_b * (1.0 - lam);
        double qn = q_a * lam + q_b * (1.0 - lam);
        double un = (Hn > 0.0) ? qn / Hn : 0.0;
        ut = ut + fabs(un);
        if (lam > (1.0 - f_grnd_ac)) ug = ug + fabs(un);
    }
    double w = (ut > 0.0) ? ug / ut : 0.0;
    return beta_a * w;
}

/* stagger_beta, basal_dragging.f90:581-704 (with the variants :1360-1758) */
static void stagger_beta(double* bx, double* by, const double* beta, const double* H_ice,
                         const double* f_ice, const double* ux, const double* uy, const double* f_grnd,
                         const double* fgx, const double* fgy, int gl_stag, double beta_min, int limit,
                         int bc, int nx, int ny) {
    size_t n2 = (size_t)nx * ny;
    if (gl_stag != -1) {
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) { /* stagger_beta_aa_mean :1360 */
                int im1, ip1, jm1, jp1;
                nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
                size_t c = ID2(i, j);
                if (f_grnd[c] == 0.0 && f_grnd[ID2(ip1, j)] == 0.0) bx[c] = 0.0;
                else if (f_ice[c] == 1.0 && f_ice[ID2(ip1, j)] < 1.0) bx[c] = beta[c];
                else if (f_ice[c] < 1.0 && f_ice[ID2(ip1, j)] == 1.0) bx[c] = beta[ID2(ip1, j)];
                else bx[c] = 0.5 * (beta[c] + beta[ID2(ip1, j)]);
                if (f_grnd[c] == 0.0 && f_grnd[ID2(i, jp1)] == 0.0) by[c] = 0.0;
                else if (f_ice[c] == 1.0 && f_ice[ID2(i, jp1)] < 1.0) by[c] = beta[c];
                else if (f_ice[c] < 1.0 && f_ice[ID2(i, jp1)] == 1.0) by[c] = beta[ID2(i, jp1)];
                else by[c] = 0.5 * (beta[c] + beta[ID2(i, jp1)]);
            }
        if (gl_stag >= 1 && gl_stag <= 4) {
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    int im1, ip1, jm1, jp1;
                    nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
                    size_t c = ID2(i, j), cx = ID2(ip1, j), cy = ID2(i, jp1);
                    /* x faces */
                    if (f_ice[c] == 1.0 && f_ice[cx] == 1.0) {
                        int gl_r = (f_grnd[c] > 0.0 && f_grnd[cx] == 0.0);
                        int gl_l = (f_grnd[c] == 0.0 && f_grnd[cx] > 0.0);
                        if (gl_stag == 1) {
                            if (gl_r) bx[c] = beta[c]; else if (gl_l) bx[c] = beta[cx];
                        } else if (gl_stag == 2) {
                            if (gl_r) bx[c] = beta[cx]; else if (gl_l) bx[c] = beta[c];
                        } else if (gl_stag == 3) {
                            double wt = fgx[c] * fgx[c];
                            if (gl_r) bx[c] = wt * beta[c] + (1.0 - wt) * beta[cx];
                            else if (gl_l) bx[c] = (1.0 - wt) * beta[c] + wt * beta[cx];
                        } else {
                            if (gl_r) {
                                double ua = 0.5 * (ux[ID2(im1, j)] + ux[c]);
                                double ub = 0.5 * (ux[ID2(ip1, j)] + ux[c]);
                                bx[c] = beta_gl_flux_weight(beta[c], ua, ub, H_ice[c], H_ice[cx], fgx[c]);
                            } else if (gl_l) {
                                double ua = 0.5 * (ux[ID2(ip1, j)] + ux[c]);
                                double ub = 0.5 * (ux[ID2(im1, j)] + ux[c]);
                                bx[c] = beta_gl_flux_weight(beta[cx], ua, ub, H_ice[cx], H_ice[c], fgx[c]);
                            }
                        }
                    }
                    /* y faces */
                    if (f_ice[c] == 1.0 && f_ice[cy] == 1.0) {
                        int gl_t = (f_grnd[c] > 0.0 && f_grnd[cy] == 0.0);
                        int gl_b = (f_grnd[c] == 0.0 && f_grnd[cy] > 0.0);
                        if (gl_stag == 1) {
                            if (gl_t) by[c] = beta[c]; else if (gl_b) by[c] = beta[cy];
                        } else if (gl_stag == 2) {
                            if (gl_t) by[c] = beta[cy]; else if (gl_b) by[c] = beta[c];
                        } else if (gl_stag == 3) {
                            double wt = fgy[c] * fgy[c];
                            if (gl_t) by[c] = wt * beta[c] + (1.0 - wt) * beta[cy];
                            else if (gl_b) by[c] = (1.0 - wt) * beta[c] + wt * beta[cy];
                        } else {
                            if (gl_t) {
                                double ua = 0.5 * (uy[ID2(i, jm1)] + uy[c]);
                                double ub = 0.5 * (uy[ID2(i, jp1)] + uy[c]);
                                by[c] = beta_gl_flux_weight(beta[c], ua, ub, H_ice[c], H_ice[cy], fgy[c]);
                            } else if (gl_b) {
                                double ua = 0.5 * (uy[ID2(i, jp1)] + uy[c]);
                                double ub = 0.5 * (uy[ID2(i, jm1)] + uy[c]);
                                by[c] = beta_gl_flux_weight(beta[cy], ua, ub, H_ice[cy], H_ice[c], fgy[c]);
                            }
                        }
                    }
                }
        }
        if (bc == YGPU_BND_INFINITE || bc == YGPU_BND_MISMIP3D) {
            for (int j = 0; j < ny; j++) {
                bx[ID2(0, j)] = bx[ID2(1, j)];
                bx[ID2(nx - 2, j)] = bx[ID2(nx - 3, j)];
                bx[ID2(nx - 1, j)] = bx[ID2(nx - 3, j)];
                by[ID2(0, j)] = by[ID2(1, j)];
                by[ID2(nx - 1, j)] = by[ID2(nx - 2, j)];
            }
        }
        if (bc == YGPU_BND_INFINITE) {
            for (int i = 0; i < nx; i++) {
                bx[ID2(i, 0)] = bx[ID2(i, 1)];
                bx[ID2(i, ny - 1)] = bx[ID2(i, ny - 2)];
                by[ID2(i, 0)] = by[ID2(i, 1)];
                by[ID2(i, ny - 2)] = by[ID2(i, ny - 3)];
                by[ID2(i, ny - 1)] = by[ID2(i, ny - 3)];
            }
        }
    }
    if (limit) {
        for (size_t c = 0; c < n2; c++) {
            if (bx[c] > 0.0 && bx[c] < beta_min) bx[c] = beta_min;
            if (by[c] > 0.0 && by[c] < beta_min) by[c] = beta_min;
        }
    }
}

/* set_beta_min_grounded, basal_dragging.f90:706-780 */
static void set_beta_min_grounded(double* bx, double* by, const int* mx, const int* my, double beta_min,
                                  size_t n2) {
    for (size_t c = 0; c < n2; c++) {
        if (mx[c] == 1 && bx[c] == 0.0) bx[c] = beta_min;
        if (my[c] == 1 && by[c] == 0.0) by[c] = beta_min;
    }
}

/* ======================================================================== */
/* DIVA helpers (velocity_diva.f90)                                         */
/* ======================================================================== */

/* calc_vertical_shear_3D :510-571 */
static void vertical_shear_3D(double* duxdz, double* duydz, const double* tbx, const double* tby,
                              const double* visc, const double* f_ice, const double* zeta, int bc, int nx,
                              int ny, int nz) {
    size_t n2 = (size_t)nx * ny;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int im1, ip1, jm1, jp1;
                nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
                size_t c = ID2(i, j);
                double va = stag_margin(visc[k * n2 + c], visc[k * n2 + ID2(ip1, j)], f_ice[c], f_ice[ID2(ip1, j)]);
                duxdz[k * n2 + c] = (va != 0.0) ? (tbx[c] / va) * (1.0 - zeta[k]) : 0.0;
                va = stag_margin(visc[k * n2 + c], visc[k * n2 + ID2(i, jp1)], f_ice[c], f_ice[ID2(i, jp1)]);
                duydz[k * n2 + c] = (va != 0.0) ? (tby[c] / va) * (1.0 - zeta[k]) : 0.0;
            }
}

/* calc_F_integral :824-869 with n = 2 */
static void F_integral2(double* F2, const double* visc, const double* H, const double* f_ice,
                        const double* zeta, int nx, int ny, int nz) {
    size_t n2 = (size_t)nx * ny;
    double* tmp = malloc((size_t)nz * sizeof(double));
    for (size_t c = 0; c < n2; c++) {
        if (f_ice[c] == 1.0) {
            for (int k = 0; k < nz; k++) {
                double o = 1.0 - zeta[k];
                tmp[k] = (H[c] / visc[k * n2 + c]) * (o * o);
            }
            F2[c] = trapz_pt(tmp, zeta, nz, 1);
        } else {
            F2[c] = 0.0;
        }
    }
    free(tmp);
}

/* stagger_F_integral :871-910 */
static void stagger_F(double* Fx, double* Fy, const double* F, const double* f_ice, int bc, int nx, int ny) {
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            Fx[c] = stag_margin(F[c], F[ID2(ip1, j)], f_ice[c], f_ice[ID2(ip1, j)]);
            Fy[c] = stag_margin(F[c], F[ID2(i, jp1)], f_ice[c], f_ice[ID2(i, jp1)]);
        }
}

/* calc_beta_eff :912-958 */
static void beta_eff_calc(double* be, const double* b, const double* F2, int no_slip, size_t n2) {
    for (size_t c = 0; c < n2; c++) {
        if (no_slip) be[c] = (F2[c] > 0.0) ? 1.0 / F2[c] : 0.0;
        else be[c] = b[c] / (1.0 + b[c] * F2[c]);
    }
}

/* calc_vel_horizontal_3D :431-508 */
static void vel_horizontal_3D(double* ux, double* uy, const double* ux_b, const double* uy_b,
                              const double* tbx, const double* tby, const double* visc, const double* H,
                              const double* f_ice, const double* zeta, int bc, int nx, int ny, int nz) {
    size_t n2 = (size_t)nx * ny;
    double* F1 = calloc(n2 * nz, sizeof(double));
    for (size_t c = 0; c < n2; c++) {
        if (f_ice[c] == 1.0) {
            double acc = 0.0;
            F1[c] = 0.0;
            for (int k = 1; k < nz; k++) {
                double vk = (H[c] / visc[k * n2 + c]) * (1.0 - zeta[k]);
                double vkm = (H[c] / visc[(k - 1) * n2 + c]) * (1.0 - zeta[k - 1]);
                double mid = 0.5 * (vk + vkm);
                acc = acc + mid * (zeta[k] - zeta[k - 1]);
                F1[k * n2 + c] = acc;
            }
        }
    }
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int im1, ip1, jm1, jp1;
                nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
                size_t c = ID2(i, j);
                double fa = stag_margin(F1[k * n2 + c], F1[k * n2 + ID2(ip1, j)], f_ice[c], f_ice[ID2(ip1, j)]);
                ux[k * n2 + c] = ux_b[c] + tbx[c] * fa;
                fa = stag_margin(F1[k * n2 + c], F1[k * n2 + ID2(i, jp1)], f_ice[c], f_ice[ID2(i, jp1)]);
                uy[k * n2 + c] = uy_b[c] + tby[c] * fa;
            }
    free(F1);
}

/* ======================================================================== */
/* Picard helpers (solver_ssa_ac.f90, velocity_general.f90)                 */
/* ======================================================================== */

/* calc_vel_lim_drag, solver_ssa_ac.f90:1095-1199 */
static void lim_face(double* k, double* r, double u, double uc, int mask, double s0, double inv_du,
                     double tau_c) {
    *k = 0.0;
    *r = 0.0;
    if (mask < 1) return;
    double s = sqrt(u * u + uc * uc);
    if (s <= s0) return;
    double x = (s - s0) * inv_du;
    double tau = tau_c * x * x;
    double dtds = 2.0 * tau_c * x * inv_du;
    double b = tau / s;
    double w = (u / s) * (u / s);
    *k = b * (1.0 - w) + dtds * w;
    *r = (*k - b) * u;
}

static void vel_lim_drag(double* kx, double* ky, double* rx, double* ry, const double* ux, const double* uy,
                         const int* mx, const int* my, double u_max, double tau_c, int bc, int nx, int ny) {
    double s0 = 0.8 * u_max;
    double inv_du = 1.0 / (u_max - s0);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            double uc = 0.25 * (uy[c] + uy[ID2(ip1, j)] + uy[ID2(i, jm1)] + uy[ID2(ip1, jm1)]);
            lim_face(&kx[c], &rx[c], ux[c], uc, mx[c], s0, inv_du, tau_c);
            uc = 0.25 * (ux[c] + ux[ID2(im1, j)] + ux[ID2(i, jp1)] + ux[ID2(im1, jp1)]);
            lim_face(&ky[c], &ry[c], uy[c], uc, my[c], s0, inv_du, tau_c);
        }
}

/* count_vel_lim_faces, solver_ssa_ac.f90:1201-1262 */
static int count_lim_faces(const double* ux, const double* uy, const int* mx, const int* my, double u_max,
                           int drag, int bc, int nx, int ny) {
    double s0 = 0.8 * u_max;
    int n = 0;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            if (mx[c] >= 1) {
                if (drag) {
                    double uc = 0.25 * (uy[c] + uy[ID2(ip1, j)] + uy[ID2(i, jm1)] + uy[ID2(ip1, jm1)]);
                    if (ux[c] * ux[c] + uc * uc > s0 * s0) n++;
                } else if (fabs(ux[c]) >= u_max) n++;
            }
            if (my[c] >= 1) {
                if (drag) {
                    double uc = 0.25 * (ux[c] + ux[ID2(im1, j)] + ux[ID2(i, jp1)] + ux[ID2(im1, jp1)]);
                    if (uy[c] * uy[c] + uc * uc > s0 * s0) n++;
                } else if (fabs(uy[c]) >= u_max) n++;
            }
        }
    return n;
}

/* ssa_vel_clip / limit_vel, solver_ssa_ac.f90:1069-1093,1264-1280 */
static void vel_clip(double* ux, double* uy, double lim, size_t n2) {
    for (size_t c = 0; c < n2; c++) {
        if (ux[c] > lim) ux[c] = lim;
        if (ux[c] < -lim) ux[c] = -lim;
        if (uy[c] > lim) uy[c] = lim;
        if (uy[c] < -lim) uy[c] = -lim;
    }
}

/* picard_relax_vel, velocity_general.f90:2160-2186 */
static void relax_vel(double* ux, double* uy, const double* uxp, const double* uyp, double rel, size_t n2) {
    for (size_t c = 0; c < n2; c++) {
        ux[c] = uxp[c] + rel * (ux[c] - uxp[c]);
        uy[c] = uyp[c] + rel * (uy[c] - uyp[c]);
    }
}

/* picard_calc_convergence_l2, velocity_general.f90:1950-2158. Returns 1 if
   converged (or iter == iter_max), -1 if the velocity is not finite. */
static int conv_l2(double* resid, const double* ux, const double* uy, const double* uxp, const double* uyp,
                   const int* mx, const int* my, double tol, int iter, int iter_max, int nx, int ny) {
    const double vel_tol = 1e-5, du_reg = 1e-10;
    double r1 = 0.0, r2 = 0.0, r3 = 0.0;
    int ncheck = 0, bad = 0;
    for (int j = 0; j < ny; j++) {
        double a = 0.0, b = 0.0, c3 = 0.0;
        for (int i = 0; i < nx; i++) {
            size_t c = ID2(i, j);
            if (fabs(ux[c]) > vel_tol && mx[c] > 0) {
                ncheck++;
                double t = ux[c] - uxp[c];
                if (fabs(t) < TOL_UNDERFLOW) t = 0.0;
                a = a + t * t;
                t = uxp[c];
                if (fabs(t) < TOL_UNDERFLOW) t = 0.0;
                b = b + t * t;
                t = ux[c] + uxp[c];
                c3 = c3 + t * t;
            }
            if (fabs(uy[c]) > vel_tol && my[c] > 0) {
                ncheck++;
                double t = uy[c] - uyp[c];
                if (fabs(t) < TOL_UNDERFLOW) t = 0.0;
                a = a + t * t;
                t = uyp[c];
                if (fabs(t) < TOL_UNDERFLOW) t = 0.0;
                b = b + t * t;
                t = uy[c] + uyp[c];
                c3 = c3 + t * t;
            }
            if ((mx[c] > 0 && !isfinite(ux[c])) || (my[c] > 0 && !isfinite(uy[c]))) bad = 1;
        }
        r1 = r1 + a;
        r2 = r2 + b;
        r3 = r3 + c3;
    }
    (void)r3;
    double res = (ncheck > 0) ? sqrt(r1) / (sqrt(r2) + du_reg) : 0.0;
    *resid = res;
    if (bad || !isfinite(res)) return -1;
    if (res < tol) return 1;
    if (iter == iter_max) return 1;
    return 0;
}

/* picard_calc_convergence_l1rel_matrix, velocity_general.f90:1907-1948 */
static void conv_l1rel(double* ex, double* ey, const double* ux, const double* uy, const double* uxp,
                       const double* uyp, size_t n2) {
    const double vt = 1e-2, tol = 1e-5;
    for (size_t c = 0; c < n2; c++) {
        ex[c] = (fabs(ux[c]) > vt) ? 2.0 * fabs(ux[c] - uxp[c]) / fabs(ux[c] + uxp[c] + tol) : 0.0;
        ey[c] = (fabs(uy[c]) > vt) ? 2.0 * fabs(uy[c] - uyp[c]) / fabs(uy[c] + uyp[c] + tol) : 0.0;
    }
}

/* set_inactive_margins (no a_front), velocity_general.f90:1687-1750 */
static void set_inactive_margins(double* ux, double* uy, const double* f_ice, int bc, int nx, int ny) {
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            double fa = f_ice[ID2(i, j)], fb = f_ice[ID2(ip1, j)];
            if ((fb == 0.0 && fa < 1.0) || (fa == 0.0 && fb < 1.0)) ux[ID2(i, j)] = 0.0;
            fb = f_ice[ID2(i, jp1)];
            if ((fb == 0.0 && fa < 1.0) || (fa == 0.0 && fb < 1.0)) uy[ID2(i, j)] = 0.0;
        }
}

/* stagger_visc_aa_ab, solver_ssa_ac.f90:1000-1067 */
static void stagger_visc_ab(double* Nab, const double* N, const double* f_ice, const double* z_bed,
                            const double* z_sl, int bc, int nx, int ny) {
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t cc[4] = {ID2(i, j), ID2(ip1, j), ID2(i, jp1), ID2(ip1, jp1)};
            int nice = 0, anyocn = 0;
            double v[4];
            for (int q = 0; q < 4; q++) {
                int ice = (f_ice[cc[q]] == 1.0);
                int ocn = (!ice) && (z_bed[cc[q]] < z_sl[cc[q]]);
                nice += ice;
                anyocn |= ocn;
                v[q] = ice ? N[cc[q]] : 0.0;
            }
            if (anyocn || nice == 0) Nab[ID2(i, j)] = 0.0;
            else Nab[ID2(i, j)] = ((v[0] + v[1]) + (v[2] + v[3])) / (double)nice;
        }
}

/* ======================================================================== */
/* CSR container                                                            */
/* ======================================================================== */

void orc_csr_free(orc_csr* A) {
    free(A->ptr); free(A->idx); free(A->val); free(A->b); free(A->x); free(A->copy_from);
    memset(A, 0, sizeof(*A));
}

static void csr_alloc(orc_csr* A, int nmax, int cap) {
    if (A->nmax != nmax || A->cap < cap) {
        orc_csr_free(A);
        A->nmax = nmax;
        A->cap = cap;
        A->ptr = malloc((size_t)(nmax + 1) * sizeof(int));
        A->idx = malloc((size_t)cap * sizeof(int));
        A->val = malloc((size_t)cap * sizeof(double));
        A->b = malloc((size_t)nmax * sizeof(double));
        A->x = malloc((size_t)nmax * sizeof(double));
        A->copy_from = malloc((size_t)nmax * sizeof(int));
    }
    for (int n = 0; n < nmax; n++) A->copy_from[n] = -1;
}

/* ======================================================================== */
/* Residual assembler, solver_ssa_ac.f90:73-848                             */
/* ======================================================================== */

int orc_assemble_residual(orc_csr* A, const double* ux, const double* uy, const double* bx,
                          const double* by, const double* N, const int* mx, const int* my,
                          const double* H_ice, const double* f_ice, const double* z_bed, const double* z_sl,
                          const double* tdx, const double* tdy, const double* tlx, const double* tly,
                          double dx, double dy, int bc, const double* lkx, const double* lky,
                          const double* lrx, const double* lry, int nx, int ny) {
    (void)H_ice;
    int nmax = 2 * nx * ny;
    csr_alloc(A, nmax, 9 * nmax);
    int per[4], fre[4];
    border_types(bc, per, fre);
    int use_lim = (lkx && lky && lrx && lry);
    double inv_dx = 1.0 / dx, inv_dxdx = 1.0 / (dx * dx), inv_dy = 1.0 / dy, inv_dydy = 1.0 / (dy * dy);
    double inv_dxdy = 1.0 / (dx * dy);
    size_t n2 = (size_t)nx * ny;
    double* Nab = malloc(n2 * sizeof(double));
    stagger_visc_ab(Nab, N, f_ice, z_bed, z_sl, bc, nx, ny);
#define UXC(i, j) (2 * ((i) * ny + (j)))
#define UYC(i, j) (2 * ((i) * ny + (j)) + 1)
    int k = 0;
    A->ptr[0] = 0;
    for (int n = 0; n < nmax; n += 2) {
        int q = n / 2, i = q / ny, j = q % ny;
        int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
        int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
        size_t c = ID2(i, j);
#define ADD(col, v) do { A->idx[k] = (col); A->val[k] = (v); k++; } while (0)
        /* ---- ux row ---- */
        int nr = n;
        if (mx[c] == 0) {
            ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0;
        } else if (mx[c] == -1) {
            ADD(nr, 1.0); A->b[nr] = ux[c]; A->x[nr] = ux[c];
        } else if (i == 0 && !per[2]) {
            if (fre[2]) { ADD(UXC(i, j), 1.0); ADD(UXC(ip1, j), -1.0); A->b[nr] = 0.0; A->x[nr] = ux[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (i == nx - 1 && !per[0]) {
            if (fre[0]) { ADD(UXC(i, j), 1.0); ADD(UXC(nx - 2, j), -1.0); A->b[nr] = 0.0; A->x[nr] = ux[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (j == 0 && !per[3]) {
            if (fre[3]) { ADD(UXC(i, j), 1.0); ADD(UXC(i, jp1), -1.0); A->b[nr] = 0.0; A->x[nr] = ux[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (j == ny - 1 && !per[1]) {
            if (fre[1]) { ADD(UXC(i, j), 1.0); ADD(UXC(i, ny - 2), -1.0); A->b[nr] = 0.0; A->x[nr] = ux[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (mx[c] == 3) {
            if (f_ice[c] == 1.0 && f_ice[ID2(ip1, j)] < 1.0) {
                double Nn = N[c];
                ADD(UXC(im1, j), -4.0 * inv_dx * Nn);
                ADD(UYC(i, jm1), -2.0 * inv_dy * Nn);
                ADD(UXC(i, j), 4.0 * inv_dx * Nn);
                ADD(UYC(i, j), 2.0 * inv_dy * Nn);
            } else {
                double Nn = N[ID2(ip1, j)];
                ADD(UXC(i, j), -4.0 * inv_dx * Nn);
                ADD(UYC(ip1, jm1), -2.0 * inv_dy * Nn);
                ADD(UXC(ip1, j), 4.0 * inv_dx * Nn);
                ADD(UYC(ip1, j), 2.0 * inv_dy * Nn);
            }
            A->b[nr] = tlx[c];
            A->x[nr] = ux[c];
        } else {
            double w = (mx[c] == 4) ? 0.5 : 1.0;
            double bn = w * bx[c], lr = 0.0;
            if (use_lim) { bn = bn + w * lkx[c]; lr = w * lrx[c]; }
            ADD(UXC(i, j), -4.0 * inv_dxdx * (N[ID2(ip1, j)] + N[c]) - 1.0 * inv_dydy * (Nab[c] + Nab[ID2(i, jm1)]) - bn);
            ADD(UXC(ip1, j), 4.0 * inv_dxdx * N[ID2(ip1, j)]);
            ADD(UXC(im1, j), 4.0 * inv_dxdx * N[c]);
            ADD(UXC(i, jp1), 1.0 * inv_dydy * Nab[c]);
            ADD(UXC(i, jm1), 1.0 * inv_dydy * Nab[ID2(i, jm1)]);
            ADD(UYC(i, j), -2.0 * inv_dxdy * N[c] - 1.0 * inv_dxdy * Nab[c]);
            ADD(UYC(ip1, j), 2.0 * inv_dxdy * N[ID2(ip1, j)] + 1.0 * inv_dxdy * Nab[c]);
            ADD(UYC(ip1, jm1), -2.0 * inv_dxdy * N[ID2(ip1, j)] - 1.0 * inv_dxdy * Nab[ID2(i, jm1)]);
            ADD(UYC(i, jm1), 2.0 * inv_dxdy * N[c] + 1.0 * inv_dxdy * Nab[ID2(i, jm1)]);
            A->b[nr] = tdx[c] - lr;
            A->x[nr] = ux[c];
        }
        A->ptr[nr + 1] = k;
        /* ---- uy row ---- */
        nr = n + 1;
        if (my[c] == 0) {
            ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0;
        } else if (my[c] == -1) {
            ADD(nr, 1.0); A->b[nr] = uy[c]; A->x[nr] = uy[c];
        } else if (j == 0 && !per[3]) {
            if (fre[3]) { ADD(UYC(i, j), 1.0); ADD(UYC(i, jp1), -1.0); A->b[nr] = 0.0; A->x[nr] = uy[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (j == ny - 1 && !per[1]) {
            if (fre[1]) { ADD(UYC(i, j), 1.0); ADD(UYC(i, ny - 2), -1.0); A->b[nr] = 0.0; A->x[nr] = uy[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (i == 0 && !per[2]) {
            if (fre[2]) { ADD(UYC(i, j), 1.0); ADD(UYC(ip1, j), -1.0); A->b[nr] = 0.0; A->x[nr] = uy[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (i == nx - 1 && !per[0]) {
            if (fre[0]) { ADD(UYC(i, j), 1.0); ADD(UYC(nx - 2, j), -1.0); A->b[nr] = 0.0; A->x[nr] = uy[c]; }
            else { ADD(nr, 1.0); A->b[nr] = 0.0; A->x[nr] = 0.0; }
        } else if (my[c] == 3) {
            if (f_ice[c] == 1.0 && f_ice[ID2(i, jp1)] < 1.0) {
                double Nn = N[c];
                ADD(UXC(im1, j), -2.0 * inv_dx * Nn);
                ADD(UYC(i, jm1), -4.0 * inv_dy * Nn);
                ADD(UXC(i, j), 2.0 * inv_dx * Nn);
                ADD(UYC(i, j), 4.0 * inv_dy * Nn);
            } else {
                double Nn = N[ID2(i, jp1)];
                ADD(UXC(im1, jp1), -2.0 * inv_dx * Nn);
                ADD(UYC(i, j), -4.0 * inv_dy * Nn);
                ADD(UXC(i, jp1), 2.0 * inv_dx * Nn);
                ADD(UYC(i, jp1), 4.0 * inv_dy * Nn);
            }
            A->b[nr] = tly[c];
            A->x[nr] = uy[c];
        } else {
            double w = (my[c] == 4) ? 0.5 : 1.0;
            double bn = w * by[c], lr = 0.0;
            if (use_lim) { bn = bn + w * lky[c]; lr = w * lry[c]; }
            ADD(UYC(i, j), -4.0 * inv_dydy * (N[ID2(i, jp1)] + N[c]) - 1.0 * inv_dxdx * (Nab[c] + Nab[ID2(im1, j)]) - bn);
            ADD(UYC(i, jp1), 4.0 * inv_dydy * N[ID2(i, jp1)]);
            ADD(UYC(i, jm1), 4.0 * inv_dydy * N[c]);
            ADD(UYC(ip1, j), 1.0 * inv_dxdx * Nab[c]);
            ADD(UYC(im1, j), 1.0 * inv_dxdx * Nab[ID2(im1, j)]);
            ADD(UXC(i, j), -2.0 * inv_dxdy * N[c] - 1.0 * inv_dxdy * Nab[c]);
            ADD(UXC(i, jp1), 2.0 * inv_dxdy * N[ID2(i, jp1)] + 1.0 * inv_dxdy * Nab[c]);
            ADD(UXC(im1, jp1), -2.0 * inv_dxdy * N[ID2(i, jp1)] - 1.0 * inv_dxdy * Nab[ID2(im1, j)]);
            ADD(UXC(im1, j), 2.0 * inv_dxdy * N[c] + 1.0 * inv_dxdy * Nab[ID2(im1, j)]);
            A->b[nr] = tdy[c] - lr;
            A->x[nr] = uy[c];
        }
        A->ptr[nr + 1] = k;
#undef ADD
    }
    A->nnz = k;
    free(Nab);
    return 0;
}

/* ======================================================================== */
/* Energy assembler, solver_ssa_ac_energy.f90:70-708                        */
/* ======================================================================== */

enum { DOF_FREE = 0, DOF_DIR = 1, DOF_TIED = 2 };
#define NNZ_ROW_MAX 48

typedef struct {
    int nx, ny, per_x, per_y;
    int per[4], fre[4];
    const int *mx, *my;
    const double *ux, *uy, *bx, *by, *N, *Nab, *f_ice, *tdx, *tdy, *tlx, *tly, *lkx, *lky, *lrx, *lry;
    double dx, dy, dxdy, dyodx, dxody;
    int use_lim;
    int *kind, *part, *root, *mem_ptr, *mem_list;
    double* dval;
} egy_t;

static int wrap_index(int* k, int nk, int periodic, int free_lo, int free_hi) {
    if (*k < 0) {
        if (periodic) *k += nk;
        else if (free_lo) *k = 0;
        else return 0;
    } else if (*k > nk - 1) {
        if (periodic) *k -= nk;
        else if (free_hi) *k = nk - 1;
        else return 0;
    }
    return 1;
}

static int element_index(int* k, int nk, int periodic) {
    if (*k < 0 || *k > nk - 1) {
        if (!periodic) return 0;
        *k = ((*k % nk) + nk) % nk;
    }
    return 1;
}

static int dof_ux(const egy_t* E, int ii, int jj) {
    if (!wrap_index(&ii, E->nx, E->per_x, E->fre[2], E->fre[0])) return -1;
    if (!wrap_index(&jj, E->ny, E->per_y, E->fre[3], E->fre[1])) return -1;
    return 2 * (ii * E->ny + jj);
}
static int dof_uy(const egy_t* E, int ii, int jj) {
    if (!wrap_index(&ii, E->nx, E->per_x, E->fre[2], E->fre[0])) return -1;
    if (!wrap_index(&jj, E->ny, E->per_y, E->fre[3], E->fre[1])) return -1;
    return 2 * (ii * E->ny + jj) + 1;
}

static int cell_elem(const egy_t* E, int ci, int cj, int d[4], double H[4][4]) {
    if (!element_index(&ci, E->nx, E->per_x)) return 0;
    if (!element_index(&cj, E->ny, E->per_y)) return 0;
    d[0] = dof_ux(E, ci - 1, cj);
    d[1] = dof_ux(E, ci, cj);
    d[2] = dof_uy(E, ci, cj - 1);
    d[3] = dof_uy(E, ci, cj);
    int nx = E->nx;
    double Nc = E->N[ID2(ci, cj)];
    double hx = 4.0 * Nc * E->dyodx, hy = 4.0 * Nc * E->dxody, hc = 2.0 * Nc;
    double h[4][4] = {{hx, -hx, hc, -hc}, {-hx, hx, -hc, hc}, {hc, -hc, hy, -hy}, {-hc, hc, -hy, hy}};
    memcpy(H, h, sizeof(h));
    return 1;
}

static int corner_elem(const egy_t* E, int ci, int cj, int d[4], double H[4][4]) {
    if (!element_index(&ci, E->nx, E->per_x)) return 0;
    if (!element_index(&cj, E->ny, E->per_y)) return 0;
    d[0] = dof_ux(E, ci, cj);
    d[1] = dof_ux(E, ci, cj + 1);
    d[2] = dof_uy(E, ci, cj);
    d[3] = dof_uy(E, ci + 1, cj);
    int nx = E->nx;
    double Nc = E->Nab[ID2(ci, cj)];
    double hx = Nc * E->dxody, hy = Nc * E->dyodx;
    double h[4][4] = {{hx, -hx, Nc, -Nc}, {-hx, hx, -Nc, Nc}, {Nc, -Nc, hy, -hy}, {-Nc, Nc, -hy, hy}};
    memcpy(H, h, sizeof(h));
    return 1;
}

static int add_entry(int c, double v, int* nb, int* cols, double* vals) {
    for (int k = 0; k < *nb; k++)
        if (cols[k] == c) { vals[k] += v; return 0; }
    if (*nb >= NNZ_ROW_MAX) return -1;
    cols[*nb] = c;
    vals[*nb] = v;
    (*nb)++;
    return 0;
}

static int add_element(const egy_t* E, int mm, const int d[4], double H[4][4], int* nb, int* cols,
                       double* vals, double* bval) {
    for (int l = 0; l < 4; l++) {
        if (d[l] != mm) continue;
        for (int k = 0; k < 4; k++) {
            int c = d[k];
            if (c < 0) continue;
            switch (E->kind[c]) {
                case DOF_FREE: if (add_entry(c, H[l][k], nb, cols, vals)) return -1; break;
                case DOF_TIED: if (add_entry(E->root[c], H[l][k], nb, cols, vals)) return -1; break;
                default: *bval = *bval - H[l][k] * E->dval[c]; break;
            }
        }
    }
    return 0;
}

static int add_member(const egy_t* E, int mm, int r, int* nb, int* cols, double* vals, double* bval) {
    int nx = E->nx, ny = E->ny;
    int q = mm / 2, i = q / ny, j = q % ny;
    int ip1 = (i + 1 == nx) ? 0 : i + 1, jp1 = (j + 1 == ny) ? 0 : j + 1;
    size_t c = ID2(i, j);
    int d[4];
    double H[4][4];
    if (mm % 2 == 0) {
        int mask = E->mx[c];
        double bn = E->bx[c];
        double w = (mask == 3 || mask == 4) ? 0.5 : 1.0;
        if (E->use_lim) {
            bn = bn + E->lkx[c];
            *bval = *bval + w * E->lrx[c] * E->dxdy;
        }
        if (add_entry(r, w * bn * E->dxdy, nb, cols, vals)) return -1;
        if (mask == 3) {
            if (E->f_ice[c] == 1.0 && E->f_ice[ID2(ip1, j)] < 1.0) *bval = *bval + E->tlx[c] * E->dy;
            else *bval = *bval - E->tlx[c] * E->dy;
        } else {
            *bval = *bval - E->tdx[c] * E->dxdy;
        }
        if (cell_elem(E, i, j, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
        if (cell_elem(E, i + 1, j, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
        if (corner_elem(E, i, j, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
        if (corner_elem(E, i, j - 1, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
    } else {
        int mask = E->my[c];
        double bn = E->by[c];
        double w = (mask == 3 || mask == 4) ? 0.5 : 1.0;
        if (E->use_lim) {
            bn = bn + E->lky[c];
            *bval = *bval + w * E->lry[c] * E->dxdy;
        }
        if (add_entry(r, w * bn * E->dxdy, nb, cols, vals)) return -1;
        if (mask == 3) {
            if (E->f_ice[c] == 1.0 && E->f_ice[ID2(i, jp1)] < 1.0) *bval = *bval + E->tly[c] * E->dx;
            else *bval = *bval - E->tly[c] * E->dx;
        } else {
            *bval = *bval - E->tdy[c] * E->dxdy;
        }
        if (cell_elem(E, i, j, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
        if (cell_elem(E, i, j + 1, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
        if (corner_elem(E, i, j, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
        if (corner_elem(E, i - 1, j, d, H) && add_element(E, mm, d, H, nb, cols, vals, bval)) return -1;
    }
    return 0;
}

static int assemble_row(const egy_t* E, int r, int* nb, int* cols, double* vals, double* bval) {
    *nb = 0;
    *bval = 0.0;
    if (add_member(E, r, r, nb, cols, vals, bval)) return -1;
    for (int k = E->mem_ptr[r]; k < E->mem_ptr[r + 1]; k++)
        if (add_member(E, E->mem_list[k], r, nb, cols, vals, bval)) return -1;
    return 0;
}

static void sort_row(int nb, int* cols, double* vals) {
    for (int k = 1; k < nb; k++) {
        int c = cols[k];
        double v = vals[k];
        int l = k - 1;
        while (l >= 0 && cols[l] > c) {
            cols[l + 1] = cols[l];
            vals[l + 1] = vals[l];
            l--;
        }
        cols[l + 1] = c;
        vals[l + 1] = v;
    }
}

static void classify(const egy_t* E, int n) {
    int nx = E->nx, ny = E->ny, q = n / 2, i = q / ny, j = q % ny;
    size_t c = ID2(i, j);
    int kind = DOF_FREE, part = -1;
    double val = 0.0;
#define EDGE(fr, inner) do { if (fr) { kind = DOF_TIED; part = (inner); } else { kind = DOF_DIR; part = -1; } } while (0)
    if (n % 2 == 0) {
        if (E->mx[c] == 0) kind = DOF_DIR;
        else if (E->mx[c] == -1) { kind = DOF_DIR; val = E->ux[c]; }
        else if (i == 0 && !E->per[2]) EDGE(E->fre[2], 2 * (1 * ny + j));
        else if (i == nx - 1 && !E->per[0]) EDGE(E->fre[0], 2 * ((nx - 2) * ny + j));
        else if (j == 0 && !E->per[3]) EDGE(E->fre[3], 2 * (i * ny + 1));
        else if (j == ny - 1 && !E->per[1]) EDGE(E->fre[1], 2 * (i * ny + ny - 2));
    } else {
        if (E->my[c] == 0) kind = DOF_DIR;
        else if (E->my[c] == -1) { kind = DOF_DIR; val = E->uy[c]; }
        else if (j == 0 && !E->per[3]) EDGE(E->fre[3], 2 * (i * ny + 1) + 1);
        else if (j == ny - 1 && !E->per[1]) EDGE(E->fre[1], 2 * (i * ny + ny - 2) + 1);
        else if (i == 0 && !E->per[2]) EDGE(E->fre[2], 2 * (1 * ny + j) + 1);
        else if (i == nx - 1 && !E->per[0]) EDGE(E->fre[0], 2 * ((nx - 2) * ny + j) + 1);
    }
#undef EDGE
    E->kind[n] = kind;
    E->part[n] = part;
    E->dval[n] = val;
}

int orc_assemble_energy(orc_csr* A, const double* ux, const double* uy, const double* bx,
                        const double* by, const double* N, const int* mx, const int* my,
                        const double* H_ice, const double* f_ice, const double* z_bed, const double* z_sl,
                        const double* tdx, const double* tdy, const double* tlx, const double* tly,
                        double dx, double dy, int bc, const double* lkx, const double* lky,
                        const double* lrx, const double* lry, int nx, int ny) {
    (void)H_ice;
    int nmax = 2 * nx * ny;
    size_t n2 = (size_t)nx * ny;
    egy_t E;
    memset(&E, 0, sizeof(E));
    E.nx = nx; E.ny = ny;
    border_types(bc, E.per, E.fre);
    E.per_x = E.per[0] && E.per[2];
    E.per_y = E.per[1] && E.per[3];
    E.mx = mx; E.my = my; E.ux = ux; E.uy = uy; E.bx = bx; E.by = by; E.N = N; E.f_ice = f_ice;
    E.tdx = tdx; E.tdy = tdy; E.tlx = tlx; E.tly = tly; E.lkx = lkx; E.lky = lky; E.lrx = lrx; E.lry = lry;
    E.use_lim = (lkx && lky && lrx && lry);
    E.dx = dx; E.dy = dy; E.dxdy = dx * dy; E.dyodx = dy / dx; E.dxody = dx / dy;
    double* Nab = malloc(n2 * sizeof(double));
    stagger_visc_ab(Nab, N, f_ice, z_bed, z_sl, bc, nx, ny);
    E.Nab = Nab;
    E.kind = malloc((size_t)nmax * sizeof(int));
    E.part = malloc((size_t)nmax * sizeof(int));
    E.root = malloc((size_t)nmax * sizeof(int));
    E.dval = malloc((size_t)nmax * sizeof(double));
    int* row_nnz = malloc((size_t)nmax * sizeof(int));
    int err = 0;
    for (int n = 0; n < nmax; n++) classify(&E, n);
    for (int n = 0; n < nmax && !err; n++) {
        int m = n, depth = 0;
        while (E.kind[m] == DOF_TIED) {
            m = E.part[m];
            if (++depth > 8) { err = YGPU_ERR_BAD_ARG; break; }
        }
        E.root[n] = m;
    }
    if (!err) {
        for (int n = 0; n < nmax; n++)
            if (E.kind[n] == DOF_TIED && E.kind[E.root[n]] == DOF_DIR) {
                E.kind[n] = DOF_DIR;
                E.dval[n] = E.dval[E.root[n]];
                E.root[n] = n;
            }
        int* fill = calloc((size_t)nmax, sizeof(int));
        E.mem_ptr = malloc((size_t)(nmax + 1) * sizeof(int));
        for (int n = 0; n < nmax; n++)
            if (E.kind[n] == DOF_TIED) fill[E.root[n]]++;
        E.mem_ptr[0] = 0;
        for (int n = 0; n < nmax; n++) E.mem_ptr[n + 1] = E.mem_ptr[n] + fill[n];
        E.mem_list = malloc((size_t)(E.mem_ptr[nmax] > 0 ? E.mem_ptr[nmax] : 1) * sizeof(int));
        memset(fill, 0, (size_t)nmax * sizeof(int));
        for (int n = 0; n < nmax; n++)
            if (E.kind[n] == DOF_TIED) {
                int m = E.root[n];
                E.mem_list[E.mem_ptr[m] + fill[m]] = n;
                fill[m]++;
            }
        free(fill);
        /* count */
        int bad = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : bad)
        for (int n = 0; n < nmax; n++) {
            int cols[NNZ_ROW_MAX], nb;
            double vals[NNZ_ROW_MAX], bval;
            if (E.kind[n] == DOF_FREE) {
                if (assemble_row(&E, n, &nb, cols, vals, &bval)) bad = 1;
                row_nnz[n] = nb;
            } else {
                row_nnz[n] = 1;
            }
        }
        if (bad) err = YGPU_ERR_BAD_ARG;
    }
    if (!err) {
        int total = 0;
        for (int n = 0; n < nmax; n++) total += row_nnz[n];
        csr_alloc(A, nmax, total > 9 * nmax ? total : 9 * nmax);
        A->ptr[0] = 0;
        for (int n = 0; n < nmax; n++) A->ptr[n + 1] = A->ptr[n] + row_nnz[n];
        A->nnz = A->ptr[nmax];
#pragma omp parallel for schedule(dynamic, 1024)
        for (int n = 0; n < nmax; n++) {
            int q = n / 2, i = q / ny, j = q % ny;
            int p0 = A->ptr[n];
            if (E.kind[n] == DOF_FREE) {
                int cols[NNZ_ROW_MAX], nb;
                double vals[NNZ_ROW_MAX], bval;
                assemble_row(&E, n, &nb, cols, vals, &bval);
                sort_row(nb, cols, vals);
                for (int k = 0; k < nb; k++) { A->idx[p0 + k] = cols[k]; A->val[p0 + k] = vals[k]; }
                A->b[n] = bval;
                A->copy_from[n] = -1;
                A->x[n] = (n % 2 == 0) ? ux[ID2(i, j)] : uy[ID2(i, j)];
            } else if (E.kind[n] == DOF_DIR) {
                A->idx[p0] = n; A->val[p0] = 1.0;
                A->b[n] = E.dval[n]; A->x[n] = E.dval[n];
                A->copy_from[n] = -1;
            } else {
                A->idx[p0] = n; A->val[p0] = 1.0;
                A->b[n] = 0.0; A->x[n] = 0.0;
                A->copy_from[n] = E.root[n];
            }
        }
    }
    free(Nab); free(E.kind); free(E.part); free(E.root); free(E.dval); free(row_nnz);
    free(E.mem_ptr); free(E.mem_list);
    return err;
}

int orc_assemble_csr(int energy, int nx, int ny, double dx, double dy, int bc, const double* ux,
                     const double* uy, const double* bx, const double* by, const double* N, const int* mx,
                     const int* my, const double* H_ice, const double* f_ice, const double* z_bed,
                     const double* z_sl, const double* tdx, const double* tdy, const double* tlx,
                     const double* tly, int cap, int* ptr, int* idx, double* val, double* b, double* x,
                     int* copy_from) {
    orc_csr A;
    memset(&A, 0, sizeof(A));
    int err = energy ? orc_assemble_energy(&A, ux, uy, bx, by, N, mx, my, H_ice, f_ice, z_bed, z_sl, tdx, tdy,
                                           tlx, tly, dx, dy, bc, NULL, NULL, NULL, NULL, nx, ny)
                     : orc_assemble_residual(&A, ux, uy, bx, by, N, mx, my, H_ice, f_ice, z_bed, z_sl, tdx,
                                             tdy, tlx, tly, dx, dy, bc, NULL, NULL, NULL, NULL, nx, ny);
    if (err) { orc_csr_free(&A); return err; }
    int nnz = A.nnz;
    if (nnz > cap) { orc_csr_free(&A); return -nnz; }
    memcpy(ptr, A.ptr, (size_t)(A.nmax + 1) * sizeof(int));
    memcpy(idx, A.idx, (size_t)nnz * sizeof(int));
    memcpy(val, A.val, (size_t)nnz * sizeof(double));
    memcpy(b, A.b, (size_t)A.nmax * sizeof(double));
    memcpy(x, A.x, (size_t)A.nmax * sizeof(double));
    memcpy(copy_from, A.copy_from, (size_t)A.nmax * sizeof(int));
    orc_csr_free(&A);
    return nnz;
}

/* ======================================================================== */
/* Krylov solvers (LIS stand-in)                                            */
/* ======================================================================== */

static void spmv(int n, const int* ptr, const int* idx, const double* val, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; r++) {
        double s = 0.0;
        for (int k = ptr[r]; k < ptr[r + 1]; k++) s = s + val[k] * x[idx[k]];
        y[r] = s;
    }
}

/* Deterministic dot: 256 fixed chunks summed serially, then in order. */
static double dotp(int n, const double* a, const double* b) {
    enum { NCH = 256 };
    double part[NCH];
    int chunk = (n + NCH - 1) / NCH;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < NCH; c++) {
        double s = 0.0;
        int lo = c * chunk, hi = lo + chunk < n ? lo + chunk : n;
        for (int r = lo; r < hi; r++) s = s + a[r] * b[r];
        part[c] = s;
    }
    double s = 0.0;
    for (int c = 0; c < NCH; c++) s = s + part[c];
    return s;
}

typedef struct {
    int n, kind;          /* 0 none, 1 jacobi, 2 ilu0 */
    double* dinv;
    int *lptr, *lidx, *diag;  /* sorted copy with ILU factors */
    double* lval;
} precond_t;

static int pc_setup(precond_t* P, int n, const int* ptr, const int* idx, const double* val, int kind,
                    int absdiag) {
    memset(P, 0, sizeof(*P));
    P->n = n;
    P->kind = kind;
    if (kind == YGPU_PRE_JACOBI) {
        /* absdiag: |diag| (MINRES needs a positive definite preconditioner, and
           a residual-form matrix has rows of both diagonal signs) */
        P->dinv = malloc((size_t)n * sizeof(double));
        for (int r = 0; r < n; r++) {
            double d = 0.0;
            for (int k = ptr[r]; k < ptr[r + 1]; k++)
                if (idx[k] == r) d += val[k];
            if (absdiag) d = fabs(d);
            P->dinv[r] = (d != 0.0) ? 1.0 / d : 1.0;
        }
    } else if (kind == YGPU_PRE_ILU0) {
        int nnz = ptr[n];
        P->lptr = malloc((size_t)(n + 1) * sizeof(int));
        P->lidx = malloc((size_t)nnz * sizeof(int));
        P->lval = malloc((size_t)nnz * sizeof(double));
        P->diag = malloc((size_t)n * sizeof(int));
        /* sorted, duplicate-free copy */
        int k2 = 0;
        P->lptr[0] = 0;
        int cols[NNZ_ROW_MAX * 2];
        double vals[NNZ_ROW_MAX * 2];
        for (int r = 0; r < n; r++) {
            int nb = 0;
            for (int k = ptr[r]; k < ptr[r + 1]; k++) {
                int f = 0;
                for (int m = 0; m < nb; m++)
                    if (cols[m] == idx[k]) { vals[m] += val[k]; f = 1; break; }
                if (!f) { cols[nb] = idx[k]; vals[nb] = val[k]; nb++; }
            }
            sort_row(nb, cols, vals);
            P->diag[r] = -1;
            for (int m = 0; m < nb; m++) {
                if (cols[m] == r) P->diag[r] = k2;
                P->lidx[k2] = cols[m];
                P->lval[k2] = vals[m];
                k2++;
            }
            P->lptr[r + 1] = k2;
            if (P->diag[r] < 0) return YGPU_BREAKDOWN;
        }
        /* ILU(0), IKJ variant (Saad 10.3.2) */
        /* A pivot that cancels to zero (possible with uniform coefficients and
           the mixed-sign rows of the residual form) is replaced by the row's
           original diagonal entry, so the factorization always exists. */
        double* d0 = malloc((size_t)n * sizeof(double));
        for (int r = 0; r < n; r++) d0[r] = P->lval[P->diag[r]];
        int* pos = malloc((size_t)n * sizeof(int));
        for (int r = 0; r < n; r++) pos[r] = -1;
        int bad = 0;
        for (int i = 0; i < n && !bad; i++) {
            for (int k = P->lptr[i]; k < P->lptr[i + 1]; k++) pos[P->lidx[k]] = k;
            for (int k = P->lptr[i]; k < P->lptr[i + 1]; k++) {
                int c = P->lidx[k];
                if (c >= i) break;
                double piv = P->lval[P->diag[c]];
                double lik = P->lval[k] / piv;
                P->lval[k] = lik;
                for (int m = P->diag[c] + 1; m < P->lptr[c + 1]; m++) {
                    int cc = P->lidx[m];
                    if (pos[cc] >= 0) P->lval[pos[cc]] -= lik * P->lval[m];
                }
            }
            for (int k = P->lptr[i]; k < P->lptr[i + 1]; k++) pos[P->lidx[k]] = -1;
            if (fabs(P->lval[P->diag[i]]) <= 1e-14 * fabs(d0[i])) P->lval[P->diag[i]] = d0[i];
            if (P->lval[P->diag[i]] == 0.0) bad = 1;
        }
        free(pos);
        free(d0);
        if (bad) return YGPU_BREAKDOWN;
    }
    return 0;
}

static void pc_apply(const precond_t* P, const double* r, double* z) {
    int n = P->n;
    if (P->kind == YGPU_PRE_JACOBI) {
#pragma omp parallel for
        for (int i = 0; i < n; i++) z[i] = P->dinv[i] * r[i];
    } else if (P->kind == YGPU_PRE_ILU0) {
        for (int i = 0; i < n; i++) {
            double s = r[i];
            for (int k = P->lptr[i]; k < P->diag[i]; k++) s -= P->lval[k] * z[P->lidx[k]];
            z[i] = s;
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = z[i];
            for (int k = P->diag[i] + 1; k < P->lptr[i + 1]; k++) s -= P->lval[k] * z[P->lidx[k]];
            z[i] = s / P->lval[P->diag[i]];
        }
    } else {
        memcpy(z, r, (size_t)n * sizeof(double));
    }
}

static void pc_free(precond_t* P) {
    free(P->dinv); free(P->lptr); free(P->lidx); free(P->lval); free(P->diag);
}

int orc_linear_solve(int n, const int* ptr, const int* idx, const double* val, const double* b, double* x,
                     int method, int precond, int maxiter, double tol, int initx_zeros, int* iters,
                     double* relres) {
    *iters = 0;
    *relres = 0.0;
    double bnrm = sqrt(dotp(n, b, b));
    if (bnrm == 0.0) { /* solver_linear.F90:162-174 */
        memset(x, 0, (size_t)n * sizeof(double));
        return YGPU_OK;
    }
    if (initx_zeros) memset(x, 0, (size_t)n * sizeof(double));
    precond_t P;
    int st = pc_setup(&P, n, ptr, idx, val, precond, method == YGPU_LIN_MINRES);
    if (st) { pc_free(&P); return st; }
    size_t bytes = (size_t)n * sizeof(double);
    double *r = malloc(bytes), *z = malloc(bytes), *p = malloc(bytes), *q = malloc(bytes);
    double *s = malloc(bytes), *t = malloc(bytes), *v = malloc(bytes), *w = malloc(bytes);
    double *rt = malloc(bytes), *ph = malloc(bytes), *sh = malloc(bytes);
    spmv(n, ptr, idx, val, x, q);
#pragma omp parallel for
    for (int i = 0; i < n; i++) r[i] = b[i] - q[i];
    double rel = sqrt(dotp(n, r, r)) / bnrm;
    *relres = rel;
    int status = YGPU_MAXITER, it = 0;
    if (rel <= tol) { status = YGPU_OK; goto done; }

    if (method == YGPU_LIN_CG) {
        pc_apply(&P, r, z);
        memcpy(p, z, bytes);
        double rz = dotp(n, r, z);
        for (it = 1; it <= maxiter; it++) {
            spmv(n, ptr, idx, val, p, q);
            double pq = dotp(n, p, q);
            if (pq == 0.0 || !isfinite(pq)) { status = YGPU_BREAKDOWN; break; }
            double alpha = rz / pq;
            for (int i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
            rel = sqrt(dotp(n, r, r)) / bnrm;
            *relres = rel;
            if (rel <= tol) { status = YGPU_OK; break; }
            pc_apply(&P, r, z);
            double rz1 = dotp(n, r, z);
            double beta = rz1 / rz;
            rz = rz1;
            for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        }
    } else if (method == YGPU_LIN_BICGSTAB) {
        memcpy(rt, r, bytes);
        double rho_old = 1.0, alpha = 1.0, omega = 1.0;
        memset(p, 0, bytes);
        memset(v, 0, bytes);
        for (it = 1; it <= maxiter; it++) {
            double rho = dotp(n, rt, r);
            if (rho == 0.0 || !isfinite(rho)) { status = YGPU_BREAKDOWN; break; }
            if (it == 1) memcpy(p, r, bytes);
            else {
                double beta = (rho / rho_old) * (alpha / omega);
                for (int i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - omega * v[i]);
            }
            pc_apply(&P, p, ph);
            spmv(n, ptr, idx, val, ph, v);
            double tv = dotp(n, rt, v);
            if (tv == 0.0 || !isfinite(tv)) { status = YGPU_BREAKDOWN; break; }
            alpha = rho / tv;
            for (int i = 0; i < n; i++) s[i] = r[i] - alpha * v[i];
            rel = sqrt(dotp(n, s, s)) / bnrm;
            if (rel <= tol) {
                for (int i = 0; i < n; i++) x[i] += alpha * ph[i];
                *relres = rel;
                status = YGPU_OK;
                break;
            }
            pc_apply(&P, s, sh);
            spmv(n, ptr, idx, val, sh, t);
            double tt = dotp(n, t, t);
            if (tt == 0.0 || !isfinite(tt)) { status = YGPU_BREAKDOWN; break; }
            omega = dotp(n, t, s) / tt;
            for (int i = 0; i < n; i++) {
                x[i] += alpha * ph[i] + omega * sh[i];
                r[i] = s[i] - omega * t[i];
            }
            rel = sqrt(dotp(n, r, r)) / bnrm;
            *relres = rel;
            if (rel <= tol) { status = YGPU_OK; break; }
            if (omega == 0.0) { status = YGPU_BREAKDOWN; break; }
            rho_old = rho;
        }
    } else { /* MINRES, Paige-Saunders with preconditioner (Choi/Saunders form) */
        double *r1 = s, *r2 = t, *y = z, *wv = w, *w1 = q, *w2 = sh, *vv = v;
        memcpy(r1, r, bytes);
        pc_apply(&P, r1, y);
        double beta1 = dotp(n, r1, y);
        if (beta1 <= 0.0 || !isfinite(beta1)) { status = YGPU_BREAKDOWN; goto done; }
        beta1 = sqrt(beta1);
        double oldb = 0.0, beta = beta1, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0;
        memset(wv, 0, bytes);
        memset(w2, 0, bytes);
        memcpy(r2, r1, bytes);
        for (it = 1; it <= maxiter; it++) {
            double sc = 1.0 / beta;
            for (int i = 0; i < n; i++) vv[i] = sc * y[i];
            spmv(n, ptr, idx, val, vv, y);
            if (it >= 2)
                for (int i = 0; i < n; i++) y[i] -= (beta / oldb) * r1[i];
            double alfa = dotp(n, vv, y);
            for (int i = 0; i < n; i++) y[i] -= (alfa / beta) * r2[i];
            memcpy(r1, r2, bytes);
            memcpy(r2, y, bytes);
            pc_apply(&P, r2, y);
            oldb = beta;
            double bb = dotp(n, r2, y);
            if (bb < 0.0) { status = YGPU_BREAKDOWN; break; }
            beta = sqrt(bb);
            double oldeps = epsln;
            double delta = cs * dbar + sn * alfa;
            double gbar = sn * dbar - cs * alfa;
            epsln = sn * beta;
            dbar = -cs * beta;
            double gamma = sqrt(gbar * gbar + beta * beta);
            if (gamma < 1e-300) gamma = 1e-300;
            cs = gbar / gamma;
            sn = beta / gamma;
            double phi = cs * phibar;
            phibar = sn * phibar;
            double denom = 1.0 / gamma;
            memcpy(w1, w2, bytes);
            memcpy(w2, wv, bytes);
            for (int i = 0; i < n; i++) {
                wv[i] = (vv[i] - oldeps * w1[i] - delta * w2[i]) * denom;
                x[i] += phi * wv[i];
            }
            spmv(n, ptr, idx, val, x, ph);
            for (int i = 0; i < n; i++) ph[i] = b[i] - ph[i];
            rel = sqrt(dotp(n, ph, ph)) / bnrm;
            *relres = rel;
            if (rel <= tol) { status = YGPU_OK; break; }
            if (beta == 0.0) { status = YGPU_BREAKDOWN; break; }
        }
    }
    if (it > maxiter) it = maxiter;
done:
    *iters = it;
    free(r); free(z); free(p); free(q); free(s); free(t); free(v); free(w); free(rt); free(ph); free(sh);
    pc_free(&P);
    return status;
}

/* ======================================================================== */
/* Masks and the fields calc_ydyn builds before the solve                   */
/* ======================================================================== */

/* front_face_mask, solver_ssa_ac.f90:945-996 */
static int front_face_mask(int a, int b, int lat_bc) {
    int ice, fre;
    if (a > 0 && b < 0) { ice = a; fre = b; }
    else if (a < 0 && b > 0) { ice = b; fre = a; }
    else return -1;
    if (fre == MASK_FRNT_ICE_FREE_LAND) {
        if (ice == MASK_FRNT_FLOAT) return 0;
        ice = MASK_FRNT_GRND;
    }
    switch (lat_bc) {
        case YGPU_LATBC_NONE: return 4;
        case YGPU_LATBC_FLOATING: return (ice == MASK_FRNT_FLOAT) ? 3 : 4;
        case YGPU_LATBC_MARINE: return (ice == MASK_FRNT_FLOAT || ice == MASK_FRNT_MARINE) ? 3 : 4;
        case YGPU_LATBC_ALL: return 3;
        default: return -1;
    }
}

/* set_ssa_masks, solver_ssa_ac.f90:851-943 */
int orc_set_ssa_masks(int* mx, int* my, const int* mf, const double* f_ice, const double* f_grnd, int lat_bc,
                      int bc, int nx, int ny) {
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j), cx = ID2(ip1, j), cy = ID2(i, jp1);
            int m = 0;
            if (f_ice[c] == 1.0 || f_ice[cx] == 1.0) m = (f_grnd[c] > 0.0 || f_grnd[cx] > 0.0) ? 1 : 2;
            int ml = front_face_mask(mf[c], mf[cx], lat_bc);
            if (ml >= 0) m = ml;
            mx[c] = m;
            m = 0;
            if (f_ice[c] == 1.0 || f_ice[cy] == 1.0) m = (f_grnd[c] > 0.0 || f_grnd[cy] > 0.0) ? 1 : 2;
            ml = front_face_mask(mf[c], mf[cy], lat_bc);
            if (ml >= 0) m = ml;
            my[c] = m;
        }
    return 0;
}

int orc_calc_dyn_inputs(const double* H_ice, const double* z_bed, const double* z_sl, double* f_ice,
                        double* H_grnd, double* z_srf, double* f_grnd, double* fgx, double* fgy, int* mf,
                        double* dzsdx, double* dzsdy, double* tdx, double* tdy, double* tlx, double* tly,
                        double dx, double grad_lim, double taud_lim, double rho_ice, double rho_sw, double g,
                        int bc, int nx, int ny) {
    return orc_calc_dyn_inputs_bg(H_ice, z_bed, z_sl, f_ice, H_grnd, z_srf, f_grnd, fgx, fgy, mf, dzsdx, dzsdy, tdx,
                                  tdy, tlx, tly, dx, grad_lim, taud_lim, rho_ice, rho_sw, g, 0.0, 0.0, bc, nx, ny);
}

int orc_calc_dyn_inputs_bg(const double* H_ice, const double* z_bed, const double* z_sl, double* f_ice,
                           double* H_grnd, double* z_srf, double* f_grnd, double* fgx, double* fgy, int* mf,
                           double* dzsdx, double* dzsdy, double* tdx, double* tdy, double* tlx, double* tly,
                           double dx, double grad_lim, double taud_lim, double rho_ice, double rho_sw, double g,
                           double slope_bg_x, double slope_bg_y, int bc, int nx, int ny) {
    size_t n2 = (size_t)nx * ny;
    double rsi = rho_sw / rho_ice, ris = rho_ice / rho_sw, rhog = rho_ice * g;
    for (size_t c = 0; c < n2; c++) {
        f_ice[c] = (H_ice[c] > 0.0) ? 1.0 : 0.0;
        /* calc_H_grnd, topography.f90:876-931, use_f_ice = .FALSE. */
        double d = z_sl[c] - z_bed[c];
        H_grnd[c] = (d > 0.0) ? H_ice[c] - rsi * d : H_ice[c] + (z_bed[c] - z_sl[c]);
        /* calc_z_srf_max, topography.f90:820-849 (binary f_ice: H_eff = H_ice) */
        double He = (f_ice[c] < 1.0) ? 0.0 : H_ice[c];
        double a = z_bed[c] + He, b = z_sl[c] + (1.0 - ris) * He;
        z_srf[c] = (a > b) ? a : b;
        /* calc_f_grnd_subgrid_linear: central aa-node */
        f_grnd[c] = (H_grnd[c] < 0.0) ? 0.0 : 1.0;
    }
    int px, py;
    periodic_dirs(bc, &px, &py);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            for (int dir = 0; dir < 2; dir++) {
                size_t cn = dir == 0 ? ID2(ip1, j) : ID2(i, jp1);
                double h1 = H_grnd[c], h2 = H_grnd[cn], f;
                if (h1 > 0.0 && h2 <= 0.0) f = -h1 / (h2 - h1);
                else if (h1 <= 0.0 && h2 > 0.0) f = -h2 / (h1 - h2);
                else if (h1 <= 0.0 && h2 <= 0.0) f = 0.0;
                else f = 1.0;
                (dir == 0 ? fgx : fgy)[c] = f;
            }
        }
    if (!px)
        for (int j = 0; j < ny; j++) fgx[ID2(nx - 1, j)] = fgx[ID2(nx - 2, j)];
    if (!py)
        for (int i = 0; i < nx; i++) fgy[ID2(i, ny - 1)] = fgy[ID2(i, ny - 2)];
    /* calc_ice_front, topography.f90:724-818 */
    for (size_t c = 0; c < n2; c++) mf[c] = MASK_FRNT_NONE;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            size_t nb[4] = {ID2(im1, j), ID2(ip1, j), ID2(i, jm1), ID2(i, jp1)};
            int nfree = 0;
            for (int q = 0; q < 4; q++) nfree += (f_ice[nb[q]] < 1.0);
            if (f_ice[c] == 1.0 && nfree > 0) {
                if (f_grnd[c] > 0.0 && z_sl[c] <= z_bed[c]) mf[c] = MASK_FRNT_GRND;
                else if (f_grnd[c] > 0.0) mf[c] = MASK_FRNT_MARINE;
                else mf[c] = MASK_FRNT_FLOAT;
                for (int q = 0; q < 4; q++)
                    if (f_ice[nb[q]] < 1.0)
                        mf[nb[q]] = (z_bed[nb[q]] < z_sl[nb[q]]) ? MASK_FRNT_ICE_FREE : MASK_FRNT_ICE_FREE_LAND;
            }
        }
    /* calc_gradient_acx/acy (zero_outside = .FALSE.; the background slope is added below) */
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            dzsdx[ID2(i, j)] = (z_srf[ID2(ip1, j)] - z_srf[ID2(i, j)]) / dx;
            dzsdy[ID2(i, j)] = (z_srf[ID2(i, jp1)] - z_srf[ID2(i, j)]) / dx;
        }
    if (bc == YGPU_BND_INFINITE || bc == YGPU_BND_MISMIP3D || bc == YGPU_BND_TROUGH || bc == YGPU_BND_PERIODIC_Y)
        for (int j = 0; j < ny; j++) {
            dzsdx[ID2(0, j)] = dzsdx[ID2(1, j)];
            dzsdx[ID2(nx - 1, j)] = dzsdx[ID2(nx - 2, j)];
        }
    if (bc == YGPU_BND_INFINITE || bc == YGPU_BND_PERIODIC_X)
        for (int i = 0; i < nx; i++) {
            dzsdy[ID2(i, 0)] = dzsdy[ID2(i, 1)];
            dzsdy[ID2(i, ny - 1)] = dzsdy[ID2(i, ny - 2)];
        }
    for (size_t c = 0; c < n2; c++) {
        /* the background slope, then the limit (yelmo_tools.f90:400-404) */
        dzsdx[c] = dzsdx[c] + slope_bg_x;
        dzsdy[c] = dzsdy[c] + slope_bg_y;
        if (dzsdx[c] < -grad_lim) dzsdx[c] = -grad_lim; else if (dzsdx[c] > grad_lim) dzsdx[c] = grad_lim;
        if (dzsdy[c] < -grad_lim) dzsdy[c] = -grad_lim; else if (dzsdy[c] > grad_lim) dzsdy[c] = grad_lim;
    }
    /* calc_driving_stress, velocity_general.f90:1118-1205 (dy = dx) */
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            for (int dir = 0; dir < 2; dir++) {
                size_t cn = dir == 0 ? ID2(ip1, j) : ID2(i, jp1);
                double Hm;
                if (f_ice[c] == 1.0 && f_ice[cn] < 1.0) Hm = 0.5 * (H_ice[c] + 0.0);
                else if (f_ice[c] < 1.0 && f_ice[cn] == 1.0) Hm = 0.5 * (0.0 + H_ice[cn]);
                else Hm = 0.5 * (H_ice[c] + H_ice[cn]);
                double t = rhog * Hm * (dir == 0 ? dzsdx[c] : dzsdy[c]);
                if (t > taud_lim) t = taud_lim;
                if (t < -taud_lim) t = -taud_lim;
                (dir == 0 ? tdx : tdy)[c] = t;
            }
        }
    /* calc_lateral_bc_stress_2D, velocity_general.f90:1453-1609 */
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            size_t c = ID2(i, j);
            for (int dir = 0; dir < 2; dir++) {
                size_t cn = dir == 0 ? ID2(ip1, j) : ID2(i, jp1);
                double tl = 0.0;
                if ((mf[c] > 0 && mf[cn] < 0) || (mf[c] < 0 && mf[cn] > 0)) {
                    size_t ci = (mf[c] < 0) ? cn : c;
                    double Hn = H_ice[ci], zs = z_srf[ci], zl = z_sl[ci];
                    if (mf[c] == MASK_FRNT_ICE_FREE_LAND || mf[cn] == MASK_FRNT_ICE_FREE_LAND) zl = zs - Hn;
                    double r = (zs - zl) / Hn;
                    double fs = 1.0 - (r < 1.0 ? r : 1.0);
                    double Ho = Hn * fs;
                    tl = 0.5 * rho_ice * g * (Hn * Hn) - 0.5 * rho_sw * g * (Ho * Ho);
                }
                (dir == 0 ? tlx : tly)[c] = tl;
            }
        }
    return 0;
}

/* calc_zeta, yelmo_grid.f90:41-121 (zeta_aa only) */
void orc_calc_zeta(int nz, int scale, double zeta_exp, double* z) {
    for (int k = 0; k < nz; k++) z[k] = 0.0 + 1.0 * (double)k / (double)(nz - 1);
    if (scale == 1) {
        for (int k = 0; k < nz; k++) z[k] = pow(z[k], zeta_exp);
    } else if (scale == 2) {
        double* t = malloc((size_t)nz * sizeof(double));
        for (int k = 0; k < nz; k++) t[k] = 1.0 - pow(z[k], zeta_exp);
        for (int k = 0; k < nz; k++) z[k] = t[nz - 1 - k];
        free(t);
    } else if (scale == 3) {
        const double pi = 3.14159265358979323846;
        for (int k = 0; k < nz; k++) z[k] = tanh(1.0 * pi * (z[k] - 0.5));
        double mn = z[0], mx;
        for (int k = 0; k < nz; k++) if (z[k] < mn) mn = z[k];
        for (int k = 0; k < nz; k++) z[k] -= mn;
        mx = z[0];
        for (int k = 0; k < nz; k++) if (z[k] > mx) mx = z[k];
        for (int k = 0; k < nz; k++) z[k] /= mx;
    }
}

/* calc_rate_factor, deformation.f90:305-341 */
double orc_rate_factor(double T_ice, double T_pmp, double enh, double T0) {
    const double T_prime_lim = 263.15, A0_1 = 1.25671e-05, A0_2 = 6.0422976e10, Q_1 = 60.e3, Q_2 = 139.e3,
                 R = 8.314;
    double Tp = T_ice - T_pmp + T0;
    if (Tp < 220.0) Tp = 220.0;
    if (Tp > T0) Tp = T0;
    if (Tp <= T_prime_lim) return enh * A0_1 * exp(-Q_1 / (R * Tp));
    return enh * A0_2 * exp(-Q_2 / (R * Tp));
}

/* ======================================================================== */
/* Parameters                                                               */
/* ======================================================================== */

void orc_dyn_par_defaults(ygpu_dyn_par* p) {
    memset(p, 0, sizeof(*p));
    p->ssa_solver = YGPU_SSA_ENERGY;
    p->boundaries = YGPU_BND_ZEROS;
    p->visc_method = 1;
    p->visc_const = 1e7;
    p->beta_method = 1;
    p->beta_const = 1e3;
    p->beta_q = 1.0;
    p->beta_u0 = 100.0;
    p->beta_gl_scale = 0;
    p->beta_gl_stag = 1;
    p->beta_gl_f = 1.0;
    p->H_grnd_lim = 500.0;
    p->beta_min = 100.0;
    p->eps_0 = 1e-6;
    p->ssa_vel_lim_method = YGPU_VEL_LIM_DRAG;
    p->ssa_vel_max = 10000.0;
    p->ssa_vel_lim_tau = 1e5;
    p->ssa_iter_max = 20;
    p->ssa_iter_rel = 0.7;
    p->ssa_iter_conv = 1e-2;
    p->rho_ice = 910.0;
    p->rho_sw = 1028.0;
    p->g = 9.81;
    p->lin_solver = YGPU_LIN_CG;
    p->lin_precond = YGPU_PRE_JACOBI;
    p->lin_maxiter = 200;
    p->lin_tol = 1e-2;
    p->lin_initx_zeros = 0;
}

int orc_parse_lis_opt(const char* opts, ygpu_dyn_par* p) {
    char buf[512];
    if (!opts) return YGPU_ERR_BAD_ARG;
    strncpy(buf, opts, sizeof(buf) - 1);
    buf[sizeof(buf) - 1] = 0;
    char* save = NULL;
    char* tok = strtok_r(buf, " \t", &save);
    while (tok) {
        char* val = strtok_r(NULL, " \t", &save);
        if (!val) return YGPU_ERR_BAD_ARG;
        if (!strcmp(tok, "-i")) {
            if (!strcmp(val, "cg") || !strcmp(val, "1")) p->lin_solver = YGPU_LIN_CG;
            else if (!strcmp(val, "bicgstab") || !strcmp(val, "3")) p->lin_solver = YGPU_LIN_BICGSTAB;
            else if (!strcmp(val, "minres") || !strcmp(val, "5")) p->lin_solver = YGPU_LIN_MINRES;
            else return YGPU_ERR_BAD_ARG;
        } else if (!strcmp(tok, "-p")) {
            if (!strcmp(val, "none") || !strcmp(val, "0")) p->lin_precond = YGPU_PRE_NONE;
            else if (!strcmp(val, "jacobi") || !strcmp(val, "1")) p->lin_precond = YGPU_PRE_JACOBI;
            else if (!strcmp(val, "ilu") || !strcmp(val, "2")) p->lin_precond = YGPU_PRE_ILU0;
            else return YGPU_ERR_BAD_ARG;
        } else if (!strcmp(tok, "-maxiter")) {
            p->lin_maxiter = atoi(val);
        } else if (!strcmp(tok, "-tol")) {
            p->lin_tol = atof(val);
        } else if (!strcmp(tok, "-initx_zeros")) {
            p->lin_initx_zeros = (!strcmp(val, "true") || !strcmp(val, "1"));
        }
        tok = strtok_r(NULL, " \t", &save);
    }
    return YGPU_OK;
}

/* ======================================================================== */
/* Picard drivers                                                           */
/* ======================================================================== */

static int linear_solve_csr(orc_csr* A, const ygpu_dyn_par* p, int* iters, double* relres) {
    return orc_linear_solve(A->nmax, A->ptr, A->idx, A->val, A->b, A->x, p->lin_solver, p->lin_precond,
                            p->lin_maxiter, p->lin_tol, p->lin_initx_zeros, iters, relres);
}

/* linear_solver_save_velocity, solver_ssa_ac.f90:33-71 */
static void save_velocity(double* ux, double* uy, const orc_csr* A, int nx, int ny) {
    for (int n = 0; n < A->nmax; n += 2) {
        int q = n / 2, i = q / ny, j = q % ny;
        int r = (A->copy_from[n] >= 0) ? A->copy_from[n] : n;
        ux[ID2(i, j)] = A->x[r];
        r = (A->copy_from[n + 1] >= 0) ? A->copy_from[n + 1] : n + 1;
        uy[ID2(i, j)] = A->x[r];
    }
    size_t n2 = (size_t)nx * ny;
    for (size_t c = 0; c < n2; c++) {
        if (fabs(ux[c]) < TOL_UNDERFLOW) ux[c] = 0.0;
        if (fabs(uy[c]) < TOL_UNDERFLOW) uy[c] = 0.0;
    }
}

static int assemble(orc_csr* A, const ygpu_dyn_par* p, const double* ux, const double* uy, const double* bx,
                    const double* by, const double* N, const int* mx, const int* my, const double* H,
                    const double* f_ice, const double* z_bed, const double* z_sl, const double* tdx,
                    const double* tdy, const double* tlx, const double* tly, double dx, double dy,
                    const double* lkx, const double* lky, const double* lrx, const double* lry, int nx, int ny) {
    if (p->ssa_solver == YGPU_SSA_ENERGY)
        return orc_assemble_energy(A, ux, uy, bx, by, N, mx, my, H, f_ice, z_bed, z_sl, tdx, tdy, tlx, tly, dx,
                                   dy, p->boundaries, lkx, lky, lrx, lry, nx, ny);
    return orc_assemble_residual(A, ux, uy, bx, by, N, mx, my, H, f_ice, z_bed, z_sl, tdx, tdy, tlx, tly, dx,
                                 dy, p->boundaries, lkx, lky, lrx, lry, nx, ny);
}

static void log_iter(const ygpu_dyn_par* p, int conv, int iter, double resid, int lin_it, int st) {
    if (!p->ssa_write_log) return;
    printf("ssa: %s %4d %12.4g | lin %6d %d\n", conv == 1 ? "C" : "", iter, resid, lin_it, st);
}

int orc_calc_velocity_ssa(double* ux_b, double* uy_b, double* taub_acx, double* taub_acy, double* visc_eff,
                          double* visc_eff_int, int* mx, int* my, double* ssa_err_acx, double* ssa_err_acy,
                          int* ssa_iter_now, int* ssa_lin_iter, int* ssa_lin_fail, int* ssa_lim_n,
                          double* beta, double* beta_acx, double* beta_acy, const double* c_bed,
                          const double* f_slide, const double* taud_acx, const double* taud_acy,
                          const double* taul_int_acx, const double* taul_int_acy, const double* H_ice,
                          const double* f_ice, const double* H_grnd, const double* f_grnd,
                          const double* f_grnd_acx, const double* f_grnd_acy, const double* ATT,
                          const double* zeta_aa, const double* z_sl, const double* z_bed, const double* z_srf,
                          double dx, double dy, double n_glen, int nx, int ny, int nz, const ygpu_dyn_par* p) {
    (void)z_srf;
    if (nx < 3 || ny < 3 || nz < 2) return YGPU_ERR_BAD_ARG;
    size_t n2 = (size_t)nx * ny, n3 = n2 * nz;
    int bc = p->boundaries;
    double* visc_nm1 = malloc(n3 * sizeof(double));
    double* uxp = malloc(n2 * sizeof(double));
    double* uyp = malloc(n2 * sizeof(double));
    double* bsx = malloc(n2 * sizeof(double));
    double* bsy = malloc(n2 * sizeof(double));
    double* lkx = calloc(n2, sizeof(double));
    double* lky = calloc(n2, sizeof(double));
    double* lrx = calloc(n2, sizeof(double));
    double* lry = calloc(n2, sizeof(double));
    int drag = (p->ssa_vel_lim_method == YGPU_VEL_LIM_DRAG);
    memcpy(bsx, beta_acx, n2 * sizeof(double));
    memcpy(bsy, beta_acy, n2 * sizeof(double));
    for (size_t c = 0; c < n2; c++) ssa_err_acx[c] = ssa_err_acy[c] = 1.0;
    set_inactive_margins(ux_b, uy_b, f_ice, bc, nx, ny);
    orc_csr A;
    memset(&A, 0, sizeof(A));
    *ssa_lin_iter = 0;
    *ssa_lin_fail = 0;
    *ssa_iter_now = 0;
    int status = YGPU_OK;
    for (int iter = 1; iter <= p->ssa_iter_max; iter++) {
        memcpy(visc_nm1, visc_eff, n3 * sizeof(double));
        memcpy(uxp, ux_b, n2 * sizeof(double));
        memcpy(uyp, uy_b, n2 * sizeof(double));
        if (p->visc_method == 0) {
            for (size_t c = 0; c < n3; c++) visc_eff[c] = p->visc_const;
        } else if (p->visc_method == 1) {
            visc_3D_nodes(visc_eff, ux_b, uy_b, NULL, NULL, ATT, f_ice, dx, dy, n_glen, p->eps_0, bc, nx, ny, nz);
            relax_visc(visc_eff, visc_nm1, p->ssa_iter_rel, n3);
        } else if (p->visc_method == 2) {
            visc_3D_aa(visc_eff, ux_b, uy_b, NULL, NULL, ATT, f_ice, dx, dy, n_glen, p->eps_0, bc, nx, ny, nz);
            relax_visc(visc_eff, visc_nm1, p->ssa_iter_rel, n3);
        } else { status = YGPU_ERR_BAD_ARG; break; }
        visc_eff_int_calc(visc_eff_int, visc_eff, H_ice, f_ice, zeta_aa, nx, ny, nz);
        calc_beta(beta, c_bed, f_slide, ux_b, uy_b, H_ice, f_ice, H_grnd, f_grnd, z_bed, z_sl, p, nx, ny);
        stagger_beta(beta_acx, beta_acy, beta, H_ice, f_ice, ux_b, uy_b, f_grnd, f_grnd_acx, f_grnd_acy,
                     p->beta_gl_stag, p->beta_min, p->beta_method != -1 && p->beta_gl_stag != -1, bc, nx, ny);
        memcpy(bsx, beta_acx, n2 * sizeof(double));
        memcpy(bsy, beta_acy, n2 * sizeof(double));
        set_beta_min_grounded(bsx, bsy, mx, my, p->beta_min, n2);
        if (drag) vel_lim_drag(lkx, lky, lrx, lry, ux_b, uy_b, mx, my, p->ssa_vel_max, p->ssa_vel_lim_tau, bc, nx, ny);
        int err = assemble(&A, p, ux_b, uy_b, bsx, bsy, visc_eff_int, mx, my, H_ice, f_ice, z_bed, z_sl, taud_acx,
                           taud_acy, taul_int_acx, taul_int_acy, dx, dy, lkx, lky, lrx, lry, nx, ny);
        if (err) { status = err; break; }
        int it;
        double rr;
        int st = linear_solve_csr(&A, p, &it, &rr);
        *ssa_lin_iter += it;
        if (st != YGPU_OK) (*ssa_lin_fail)++;
        status = st;
        save_velocity(ux_b, uy_b, &A, nx, ny);
        vel_clip(ux_b, uy_b, p->ssa_vel_max, n2);
        relax_vel(ux_b, uy_b, uxp, uyp, p->ssa_iter_rel, n2);
        double resid;
        int conv = conv_l2(&resid, ux_b, uy_b, uxp, uyp, mx, my, p->ssa_iter_conv, iter, p->ssa_iter_max, nx, ny);
        log_iter(p, conv, iter, resid, it, st);
        conv_l1rel(ssa_err_acx, ssa_err_acy, ux_b, uy_b, uxp, uyp, n2);
        *ssa_iter_now = iter;
        if (conv < 0) { status = YGPU_ERR_NONFINITE; break; }
        if (conv) break;
    }
    if (status >= 0) {
        *ssa_lim_n = count_lim_faces(ux_b, uy_b, mx, my, p->ssa_vel_max, drag, bc, nx, ny);
        for (size_t c = 0; c < n2; c++) { /* calc_basal_stress, velocity_ssa.f90:588-617 */
            taub_acx[c] = bsx[c] * ux_b[c];
            taub_acy[c] = bsy[c] * uy_b[c];
            if (fabs(taub_acx[c]) < 1e-5) taub_acx[c] = 0.0;
            if (fabs(taub_acy[c]) < 1e-5) taub_acy[c] = 0.0;
        }
        if (p->visc_method == 0)
            visc_3D_nodes(visc_eff, ux_b, uy_b, NULL, NULL, ATT, f_ice, dx, dy, n_glen, p->eps_0, bc, nx, ny, nz);
    }
    orc_csr_free(&A);
    free(visc_nm1); free(uxp); free(uyp); free(bsx); free(bsy); free(lkx); free(lky); free(lrx); free(lry);
    return status;
}

/* calc_velocity_diva with the optional neff_hook (velocity_diva.f90:390-400):
   after every Picard iteration the hook recomputes c_bed from the basal velocity,
   and the iteration has converged only if c_bed also changed by less than
   ssa_iter_conv in relative L1 */
static int diva_solve(double* ux, double* uy, double* ux_bar, double* uy_bar, double* ux_b, double* uy_b,
                      double* ux_i, double* uy_i, double* taub_acx, double* taub_acy, double* beta,
                      double* beta_acx, double* beta_acy, double* beta_eff, double* visc_eff, double* visc_eff_int,
                      double* duxdz, double* duydz, int* mx, int* my, double* ssa_err_acx, double* ssa_err_acy,
                      int* ssa_iter_now, int* ssa_lin_iter, int* ssa_lin_fail, int* ssa_lim_n, double* c_bed,
                      const double* f_slide, const double* taud_acx, const double* taud_acy,
                      const double* taul_int_acx, const double* taul_int_acy, const double* H_ice,
                      const double* f_ice, const double* H_grnd, const double* f_grnd, const double* f_grnd_acx,
                      const double* f_grnd_acy, const double* ATT, const double* zeta_aa, const double* z_sl,
                      const double* z_bed, double dx, double dy, double n_glen, int nx, int ny, int nz,
                      const ygpu_dyn_par* p, orc_neff_hook hook, void* user);

int orc_calc_velocity_diva_hook(double* ux, double* uy, double* ux_bar, double* uy_bar, double* ux_b, double* uy_b,
                                double* ux_i, double* uy_i, double* taub_acx, double* taub_acy, double* beta,
                                double* beta_acx, double* beta_acy, double* beta_eff, double* visc_eff,
                                double* visc_eff_int, double* duxdz, double* duydz, int* mx, int* my,
                                double* ssa_err_acx, double* ssa_err_acy, int* ssa_iter_now, int* ssa_lin_iter,
                                int* ssa_lin_fail, int* ssa_lim_n, double* c_bed, const double* f_slide,
                                const double* taud_acx, const double* taud_acy, const double* taul_int_acx,
                                const double* taul_int_acy, const double* H_ice, const double* f_ice,
                                const double* H_grnd, const double* f_grnd, const double* f_grnd_acx,
                                const double* f_grnd_acy, const double* ATT, const double* zeta_aa,
                                const double* z_sl, const double* z_bed, const double* z_srf, double dx, double dy,
                                double n_glen, int nx, int ny, int nz, const ygpu_dyn_par* p, orc_neff_hook hook,
                                void* user) {
    (void)z_srf;
    return diva_solve(ux, uy, ux_bar, uy_bar, ux_b, uy_b, ux_i, uy_i, taub_acx, taub_acy, beta, beta_acx, beta_acy,
                      beta_eff, visc_eff, visc_eff_int, duxdz, duydz, mx, my, ssa_err_acx, ssa_err_acy, ssa_iter_now,
                      ssa_lin_iter, ssa_lin_fail, ssa_lim_n, c_bed, f_slide, taud_acx, taud_acy, taul_int_acx,
                      taul_int_acy, H_ice, f_ice, H_grnd, f_grnd, f_grnd_acx, f_grnd_acy, ATT, zeta_aa, z_sl, z_bed,
                      dx, dy, n_glen, nx, ny, nz, p, hook, user);
}

int orc_calc_velocity_diva(double* ux, double* uy, double* ux_bar, double* uy_bar, double* ux_b, double* uy_b,
                           double* ux_i, double* uy_i, double* taub_acx, double* taub_acy, double* beta,
                           double* beta_acx, double* beta_acy, double* beta_eff, double* visc_eff,
                           double* visc_eff_int, double* duxdz, double* duydz, int* mx, int* my,
                           double* ssa_err_acx, double* ssa_err_acy, int* ssa_iter_now, int* ssa_lin_iter,
                           int* ssa_lin_fail, int* ssa_lim_n, const double* c_bed, const double* f_slide,
                           const double* taud_acx, const double* taud_acy, const double* taul_int_acx,
                           const double* taul_int_acy, const double* H_ice, const double* f_ice,
                           const double* H_grnd, const double* f_grnd, const double* f_grnd_acx,
                           const double* f_grnd_acy, const double* ATT, const double* zeta_aa, const double* z_sl,
                           const double* z_bed, const double* z_srf, double dx, double dy, double n_glen, int nx,
                           int ny, int nz, const ygpu_dyn_par* p) {
    (void)z_srf;
    /* without a hook c_bed is only read */
    return diva_solve(ux, uy, ux_bar, uy_bar, ux_b, uy_b, ux_i, uy_i, taub_acx, taub_acy, beta, beta_acx, beta_acy,
                      beta_eff, visc_eff, visc_eff_int, duxdz, duydz, mx, my, ssa_err_acx, ssa_err_acy, ssa_iter_now,
                      ssa_lin_iter, ssa_lin_fail, ssa_lim_n, (double*)c_bed, f_slide, taud_acx, taud_acy,
                      taul_int_acx, taul_int_acy, H_ice, f_ice, H_grnd, f_grnd, f_grnd_acx, f_grnd_acy, ATT, zeta_aa,
                      z_sl, z_bed, dx, dy, n_glen, nx, ny, nz, p, NULL, NULL);
}

static int diva_solve(double* ux, double* uy, double* ux_bar, double* uy_bar, double* ux_b, double* uy_b,
                      double* ux_i, double* uy_i, double* taub_acx, double* taub_acy, double* beta,
                      double* beta_acx, double* beta_acy, double* beta_eff, double* visc_eff, double* visc_eff_int,
                      double* duxdz, double* duydz, int* mx, int* my, double* ssa_err_acx, double* ssa_err_acy,
                      int* ssa_iter_now, int* ssa_lin_iter, int* ssa_lin_fail, int* ssa_lim_n, double* c_bed,
                      const double* f_slide, const double* taud_acx, const double* taud_acy,
                      const double* taul_int_acx, const double* taul_int_acy, const double* H_ice,
                      const double* f_ice, const double* H_grnd, const double* f_grnd, const double* f_grnd_acx,
                      const double* f_grnd_acy, const double* ATT, const double* zeta_aa, const double* z_sl,
                      const double* z_bed, double dx, double dy, double n_glen, int nx, int ny, int nz,
                      const ygpu_dyn_par* p, orc_neff_hook hook, void* user) {
    if (nx < 3 || ny < 3 || nz < 2) return YGPU_ERR_BAD_ARG;
    size_t n2 = (size_t)nx * ny, n3 = n2 * nz;
    int bc = p->boundaries;
    double* visc_nm1 = malloc(n3 * sizeof(double));
    double* cb_nm1 = hook ? malloc(n2 * sizeof(double)) : NULL;
    double* uxp = malloc(n2 * sizeof(double));
    double* uyp = malloc(n2 * sizeof(double));
    double* bex = malloc(n2 * sizeof(double));
    double* bey = malloc(n2 * sizeof(double));
    double* lkx = calloc(n2, sizeof(double));
    double* lky = calloc(n2, sizeof(double));
    double* lrx = calloc(n2, sizeof(double));
    double* lry = calloc(n2, sizeof(double));
    double* F2 = malloc(n2 * sizeof(double));
    double* F2x = malloc(n2 * sizeof(double));
    double* F2y = malloc(n2 * sizeof(double));
    int drag = (p->ssa_vel_lim_method == YGPU_VEL_LIM_DRAG);
    for (size_t c = 0; c < n2; c++) ssa_err_acx[c] = ssa_err_acy[c] = 1.0;
    orc_csr A;
    memset(&A, 0, sizeof(A));
    *ssa_lin_iter = 0;
    *ssa_lin_fail = 0;
    *ssa_iter_now = 0;
    int status = YGPU_OK;
    for (int iter = 1; iter <= p->ssa_iter_max; iter++) {
        memcpy(visc_nm1, visc_eff, n3 * sizeof(double));
        memcpy(uxp, ux_bar, n2 * sizeof(double));
        memcpy(uyp, uy_bar, n2 * sizeof(double));
        vertical_shear_3D(duxdz, duydz, taub_acx, taub_acy, visc_eff, f_ice, zeta_aa, bc, nx, ny, nz);
        if (p->visc_method == 0) {
            for (size_t c = 0; c < n3; c++) visc_eff[c] = p->visc_const;
        } else if (p->visc_method == 1) {
            visc_3D_nodes(visc_eff, ux_bar, uy_bar, duxdz, duydz, ATT, f_ice, dx, dy, n_glen, p->eps_0, bc, nx, ny, nz);
        } else if (p->visc_method == 2) {
            visc_3D_aa(visc_eff, ux_bar, uy_bar, duxdz, duydz, ATT, f_ice, dx, dy, n_glen, p->eps_0, bc, nx, ny, nz);
        } else { status = YGPU_ERR_BAD_ARG; break; }
        relax_visc(visc_eff, visc_nm1, p->ssa_iter_rel, n3);
        visc_eff_int_calc(visc_eff_int, visc_eff, H_ice, f_ice, zeta_aa, nx, ny, nz);
        calc_beta(beta, c_bed, f_slide, ux_b, uy_b, H_ice, f_ice, H_grnd, f_grnd, z_bed, z_sl, p, nx, ny);
        F_integral2(F2, visc_eff, H_ice, f_ice, zeta_aa, nx, ny, nz);
        stagger_F(F2x, F2y, F2, f_ice, bc, nx, ny);
        stagger_beta(beta_acx, beta_acy, beta, H_ice, f_ice, ux_bar, uy_bar, f_grnd, f_grnd_acx, f_grnd_acy,
                     p->beta_gl_stag, p->beta_min, p->beta_method != -1 && p->beta_gl_stag != -1, bc, nx, ny);
        beta_eff_calc(bex, beta_acx, F2x, p->no_slip, n2);
        beta_eff_calc(bey, beta_acy, F2y, p->no_slip, n2);
        set_beta_min_grounded(bex, bey, mx, my, p->beta_min, n2);
        if (drag) vel_lim_drag(lkx, lky, lrx, lry, ux_bar, uy_bar, mx, my, p->ssa_vel_max, p->ssa_vel_lim_tau, bc, nx, ny);
        beta_eff_calc(beta_eff, beta, F2, p->no_slip, n2);
        int err = assemble(&A, p, ux_bar, uy_bar, bex, bey, visc_eff_int, mx, my, H_ice, f_ice, z_bed, z_sl,
                           taud_acx, taud_acy, taul_int_acx, taul_int_acy, dx, dy, lkx, lky, lrx, lry, nx, ny);
        if (err) { status = err; break; }
        int it;
        double rr;
        int st = linear_solve_csr(&A, p, &it, &rr);
        *ssa_lin_iter += it;
        if (st != YGPU_OK) (*ssa_lin_fail)++;
        status = st;
        save_velocity(ux_bar, uy_bar, &A, nx, ny);
        vel_clip(ux_bar, uy_bar, p->ssa_vel_max, n2);
        relax_vel(ux_bar, uy_bar, uxp, uyp, p->ssa_iter_rel, n2);
        double resid;
        int conv = conv_l2(&resid, ux_bar, uy_bar, uxp, uyp, mx, my, p->ssa_iter_conv, iter, p->ssa_iter_max, nx, ny);
        log_iter(p, conv, iter, resid, it, st);
        conv_l1rel(ssa_err_acx, ssa_err_acy, ux_bar, uy_bar, uxp, uyp, n2);
        *ssa_iter_now = iter;
        for (size_t c = 0; c < n2; c++) { /* calc_basal_stress :1011-1050 */
            taub_acx[c] = bex[c] * ux_bar[c];
            if (fabs(taub_acx[c]) < TOL_UNDERFLOW) taub_acx[c] = 0.0;
            taub_acy[c] = bey[c] * uy_bar[c];
            if (fabs(taub_acy[c]) < TOL_UNDERFLOW) taub_acy[c] = 0.0;
        }
        for (size_t c = 0; c < n2; c++) { /* calc_vel_basal :960-1009 */
            if (p->no_slip) { ux_b[c] = 0.0; uy_b[c] = 0.0; }
            else {
                ux_b[c] = ux_bar[c] - taub_acx[c] * F2x[c];
                uy_b[c] = uy_bar[c] - taub_acy[c] * F2y[c];
            }
        }
        if (conv < 0) { status = YGPU_ERR_NONFINITE; break; }
        if (hook) {
            /* neff_hook: c_bed from this iteration's basal velocity; converged only
               if c_bed changed by less than ssa_iter_conv (relative L1) */
            memcpy(cb_nm1, c_bed, n2 * sizeof(double));
            hook(user, c_bed, ux_b, uy_b, nx, ny);
            double dsum = 0.0, csum = 0.0;
            for (size_t c = 0; c < n2; c++) {
                dsum += fabs(c_bed[c] - cb_nm1[c]);
                csum += fabs(c_bed[c]);
            }
            if (dsum > p->ssa_iter_conv * (csum > TOL_UNDERFLOW ? csum : TOL_UNDERFLOW) && iter < p->ssa_iter_max)
                conv = 0;
        }
        if (conv) break;
    }
    free(cb_nm1);
    if (status >= 0) {
        *ssa_lim_n = count_lim_faces(ux_bar, uy_bar, mx, my, p->ssa_vel_max, drag, bc, nx, ny);
        vel_horizontal_3D(ux, uy, ux_b, uy_b, taub_acx, taub_acy, visc_eff, H_ice, f_ice, zeta_aa, bc, nx, ny, nz);
        for (int k = 0; k < nz; k++)
            for (size_t c = 0; c < n2; c++) {
                ux_i[k * n2 + c] = ux[k * n2 + c] - ux_b[c];
                uy_i[k * n2 + c] = uy[k * n2 + c] - uy_b[c];
            }
    }
    orc_csr_free(&A);
    free(visc_nm1); free(uxp); free(uyp); free(bex); free(bey); free(lkx); free(lky); free(lrx); free(lry);
    free(F2); free(F2x); free(F2y);
    return status;
}


/* ======================================================================== */
/* Post-solve diagnostics (yelmo_dynamics.f90:304-336, :642-644)            */
/* ======================================================================== */

#define ORC_TOL_UNDERFLOW 1e-15

/* integrate_trapezoid1D_pt, yelmo_tools.f90:1092-1122 */
static double diag_trapz(const double* v, const double* zeta, size_t c, size_t n2, int nz) {
    double s = 0.0;
    for (int k = 1; k < nz; k++) {
        double mid = 0.5 * (v[(size_t)k * n2 + c] + v[(size_t)(k - 1) * n2 + c]);
        s = s + mid * (zeta[k] - zeta[k - 1]);
    }
    return s;
}

/* calc_magnitude_from_staggered, yelmo_tools.f90:287-339 */
static double diag_mag(const double* u, const double* v, const double* f_ice, size_t c, size_t cxm, size_t cym) {
    double unow = 0.0, vnow = 0.0;
    if (f_ice[c] == 1.0) {
        unow = 0.5 * (u[cxm] + u[c]);
        vnow = 0.5 * (v[cym] + v[c]);
        if (fabs(unow) < ORC_TOL_UNDERFLOW) unow = 0.0;
        if (fabs(vnow) < ORC_TOL_UNDERFLOW) vnow = 0.0;
    }
    double m = sqrt(unow * unow + vnow * vnow);
    if (fabs(m) < ORC_TOL_UNDERFLOW) m = 0.0;
    return m;
}

/* is_gl_face, velocity_general.f90:1873-1882 */
static int diag_gl_face(double fg0, double fg1, double fi0, double fi1) {
    return (fg0 > 0.0 && fg1 == 0.0 && fi1 > 0.0) || (fg1 > 0.0 && fg0 == 0.0 && fi0 > 0.0);
}

int orc_calc_dyn_diagnostics(const ygpu_dyn_diag* D, int bc) {
    if (!D || D->nx < 2 || D->ny < 2) return YGPU_ERR_BAD_ARG;
    const int nx = D->nx, ny = D->ny, nz = D->nz;
    const size_t n2 = (size_t)nx * ny;
    int px, py;
    periodic_dirs(bc, &px, &py);
    /* depth averages of the shear velocity (calc_ydyn_diva, yelmo_dynamics.f90:642-644) */
    if (D->ux_i)
        for (size_t c = 0; c < n2; c++) {
            D->ux_i_bar[c] = diag_trapz(D->ux_i, D->zeta_aa, c, n2, nz);
            D->uy_i_bar[c] = diag_trapz(D->uy_i, D->zeta_aa, c, n2, nz);
        }
    /* calc_ice_flux, velocity_general.f90:1752-1823 (upwind thickness; the last
       face of a non-periodic direction stays 0) */
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = (size_t)i + (size_t)nx * j;
            double qx = 0.0, qy = 0.0;
            if (i < nx - 1 || px) {
                double area = (D->ux_bar[c] >= 0.0) ? D->H_ice[c] * D->dy : D->H_ice[ip1 + (size_t)nx * j] * D->dy;
                qx = area * D->ux_bar[c];
            }
            if (j < ny - 1 || py) {
                double area = (D->uy_bar[c] >= 0.0) ? D->H_ice[c] * D->dx : D->H_ice[i + (size_t)nx * jp1] * D->dx;
                qy = area * D->uy_bar[c];
            }
            D->qq_acx[c] = qx;
            D->qq_acy[c] = qy;
        }
    /* calc_grounding_line_flux, velocity_general.f90:1825-1886; magnitudes */
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = (size_t)i + (size_t)nx * j, cx = ip1 + (size_t)nx * j, cy = i + (size_t)nx * jp1;
            const size_t cxm = im1 + (size_t)nx * j, cym = i + (size_t)nx * jm1;
            D->qq_gl_acx[c] = diag_gl_face(D->f_grnd[c], D->f_grnd[cx], D->f_ice[c], D->f_ice[cx]) ? D->qq_acx[c] : 0.0;
            D->qq_gl_acy[c] = diag_gl_face(D->f_grnd[c], D->f_grnd[cy], D->f_ice[c], D->f_ice[cy]) ? D->qq_acy[c] : 0.0;
            D->qq[c] = diag_mag(D->qq_acx, D->qq_acy, D->f_ice, c, cxm, cym);
            D->taub[c] = diag_mag(D->taub_acx, D->taub_acy, D->f_ice, c, cxm, cym);
            D->taud[c] = diag_mag(D->taud_acx, D->taud_acy, D->f_ice, c, cxm, cym);
            const double ub = diag_mag(D->ux_b, D->uy_b, D->f_ice, c, cxm, cym);
            D->uxy_b[c] = ub;
            if (D->uxy_i_bar && D->ux_i_bar) D->uxy_i_bar[c] = diag_mag(D->ux_i_bar, D->uy_i_bar, D->f_ice, c, cxm, cym);
            D->uxy_bar[c] = diag_mag(D->ux_bar, D->uy_bar, D->f_ice, c, cxm, cym);
            if (D->ux) {
                double us = 0.0;
                for (int k = 0; k < nz; k++) {
                    const size_t o = (size_t)k * n2;
                    us = diag_mag(D->ux + o, D->uy + o, D->f_ice, c, cxm, cym);
                    D->uxy[o + c] = us;
                }
                const size_t top = (size_t)(nz - 1) * n2;
                D->ux_s[c] = D->ux[top + c];
                D->uy_s[c] = D->uy[top + c];
                D->uxy_s[c] = us;
                /* calc_vel_ratio, velocity_general.f90:1888-1905 */
                D->f_vbvs[c] = (us > 0.0) ? fmin(1.0, ub / us) : 1.0;
            }
        }
    return YGPU_OK;
}


/* ======================================================================== */
/* Column gradients and the velocity Jacobian (calc_ydyn,                   */
/* yelmo_dynamics.f90:243-296)                                              */
/* ======================================================================== */

/* calc_gradient_column_ac, yelmo_tools.f90:479-571 */
int orc_calc_gradient_column_ac(double* dvdx_c, double* dvdy_c, const double* dvdx, const double* dvdy,
                                const double* f_ice, const int* mask_ocn, int bc, int nx, int ny) {
    if (nx < 2 || ny < 2) return YGPU_ERR_BAD_ARG;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1, im2, ip2, jm2, jp2;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = ID2(i, j);
            int ice_0 = f_ice[c] == 1.0, ice_1 = f_ice[ID2(ip1, j)] == 1.0;
            dvdx_c[c] = 0.0;
            if (ice_0 && ice_1) {
                dvdx_c[c] = dvdx[c];
            } else if ((ice_0 && !mask_ocn[ID2(ip1, j)]) || (ice_1 && !mask_ocn[c])) {
                dvdx_c[c] = dvdx[c];
            } else if (ice_0) {
                if (im1 != i && f_ice[ID2(im1, j)] == 1.0) dvdx_c[c] = dvdx[ID2(im1, j)];
            } else if (ice_1) {
                nbr(ip1, j, nx, ny, bc, &im2, &ip2, &jm2, &jp2);
                if (ip2 != ip1 && f_ice[ID2(ip2, j)] == 1.0) dvdx_c[c] = dvdx[ID2(ip1, j)];
            }
            ice_1 = f_ice[ID2(i, jp1)] == 1.0;
            dvdy_c[c] = 0.0;
            if (ice_0 && ice_1) {
                dvdy_c[c] = dvdy[c];
            } else if ((ice_0 && !mask_ocn[ID2(i, jp1)]) || (ice_1 && !mask_ocn[c])) {
                dvdy_c[c] = dvdy[c];
            } else if (ice_0) {
                if (jm1 != j && f_ice[ID2(i, jm1)] == 1.0) dvdy_c[c] = dvdy[ID2(i, jm1)];
            } else if (ice_1) {
                nbr(i, jp1, nx, ny, bc, &im2, &ip2, &jm2, &jp2);
                if (jp2 != jp1 && f_ice[ID2(i, jp2)] == 1.0) dvdy_c[c] = dvdy[ID2(i, jp1)];
            }
        }
    return YGPU_OK;
}

/* The unequal-spacing first derivatives of the Jacobian routines (Singh and
   Bhadauria): 3-point forward at the base, centred inside, 3-point backward at
   the top (or, for uz, first order). u is one column, stride n2. */
static double jac_vderiv(const double* u, size_t c, size_t n2, const double* z, int k, int nz, double Hn,
                         int top3) {
#define U_(kk) u[(size_t)(kk) * n2 + c]
    double h1, h2;
    if (k == 0) {
        h1 = Hn * (z[1] - z[0]);
        h2 = Hn * (z[2] - z[1]);
        return -(2.0 * h1 + h2) / (h1 * (h1 + h2)) * U_(0) + (h1 + h2) / (h1 * h2) * U_(1) -
               h1 / (h2 * (h1 + h2)) * U_(2);
    }
    if (k < nz - 1) {
        h1 = Hn * (z[k] - z[k - 1]);
        h2 = Hn * (z[k + 1] - z[k]);
        return -h2 / (h1 * (h1 + h2)) * U_(k - 1) - (h1 - h2) / (h1 * h2) * U_(k) + h1 / (h2 * (h1 + h2)) * U_(k + 1);
    }
    if (!top3) return (U_(k) - U_(k - 1)) / (Hn * (z[k] - z[k - 1]));
    h1 = Hn * (z[k - 1] - z[k - 2]);
    h2 = Hn * (z[k] - z[k - 1]);
    return h2 / (h1 * (h1 + h2)) * U_(k - 2) - (h1 + h2) / (h1 * h2) * U_(k - 1) +
           (h1 + 2.0 * h2) / (h2 * (h1 + h2)) * U_(k);
#undef U_
}

/* calc_jacobian_vel_3D_uxyterms, deformation.f90:397-716 */
static void jac_uxyterms(const ygpu_jvel* J, int bc) {
    const int nx = J->nx, ny = J->ny, nz = J->nz_aa;
    const size_t n2 = (size_t)nx * ny;
    const double *f = J->f_ice, *H = J->H_ice, *ux = J->ux, *uy = J->uy, *za = J->zeta_aa;
    const double dx = J->dx, dy = J->dy;
    memset(J->dxx, 0, n2 * nz * sizeof(double));
    memset(J->dxy, 0, n2 * nz * sizeof(double));
    memset(J->dxz, 0, n2 * nz * sizeof(double));
    memset(J->dyx, 0, n2 * nz * sizeof(double));
    memset(J->dyy, 0, n2 * nz * sizeof(double));
    memset(J->dyz, 0, n2 * nz * sizeof(double));
    if (J->dzx) {
        memset(J->dzx, 0, n2 * J->nz_ac * sizeof(double));
        memset(J->dzy, 0, n2 * J->nz_ac * sizeof(double));
        memset(J->dzz, 0, n2 * J->nz_ac * sizeof(double));
    }
    /* step 1: dxz, dyz on the faces where the staggered thickness is positive (:464-561) */
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = ID2(i, j);
            double Hx, Hy;
            if (f[c] == 1.0 && f[ID2(ip1, j)] < 1.0) Hx = H[c];
            else if (f[c] < 1.0 && f[ID2(ip1, j)] == 1.0) Hx = H[ID2(ip1, j)];
            else Hx = 0.5 * (H[c] + H[ID2(ip1, j)]);
            if (f[c] == 1.0 && f[ID2(i, jp1)] < 1.0) Hy = H[c];
            else if (f[c] < 1.0 && f[ID2(i, jp1)] == 1.0) Hy = H[ID2(i, jp1)];
            else Hy = 0.5 * (H[c] + H[ID2(i, jp1)]);
            for (int k = 0; k < nz; k++) {
                if (Hx > 0.0) J->dxz[k * n2 + c] = jac_vderiv(ux, c, n2, za, k, nz, Hx, 1);
                if (Hy > 0.0) J->dyz[k * n2 + c] = jac_vderiv(uy, c, n2, za, k, nz, Hy, 1);
            }
        }
    /* step 2: horizontal derivatives and the sigma-transform corrections (:565-710) */
    unsigned char* ax = malloc(n2);
    unsigned char* ay = malloc(n2);
    active_faces(ax, ay, f, bc, nx, ny);
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = ID2(i, j);
            for (int k = 0; k < nz; k++) {
                const size_t o = k * n2;
                const double* uxk = ux + o;
                const double* uyk = uy + o;
                double dxx = (uxk[ID2(ip1, j)] - uxk[ID2(im1, j)]) / (2.0 * dx);
                double dxy = deriv_active(uxk[ID2(i, jm1)], uxk[c], uxk[ID2(i, jp1)], ax[ID2(i, jm1)],
                                          ax[ID2(i, jp1)], dy);
                double dyx = deriv_active(uyk[ID2(im1, j)], uyk[c], uyk[ID2(ip1, j)], ay[ID2(im1, j)],
                                          ay[ID2(ip1, j)], dx);
                double dyy = (uyk[ID2(i, jp1)] - uyk[ID2(i, jm1)]) / (2.0 * dy);
                /* one-sided at the ice margin */
                if (f[c] == 1.0 && f[ID2(ip1, j)] < 1.0) {
                    if (im1 > 0 && f[ID2(im1, j)] == 1.0)
                        dxx = (1.0 * uxk[ID2(im1 - 1, j)] - 4.0 * uxk[ID2(im1, j)] + 3.0 * uxk[c]) / (2.0 * dx);
                    else
                        dxx = (uxk[c] - uxk[ID2(im1, j)]) / dx;
                } else if (f[c] < 1.0 && f[ID2(ip1, j)] == 1.0) {
                    if (ip1 < nx - 1 && f[ID2(ip1 + 1, j)] == 1.0)
                        dxx = -(1.0 * uxk[ID2(ip1 + 1, j)] - 4.0 * uxk[ID2(ip1, j)] + 3.0 * uxk[c]) / (2.0 * dx);
                    else
                        dxx = (uxk[ID2(ip1, j)] - uxk[c]) / dx;
                }
                if (f[c] == 1.0 && f[ID2(i, jp1)] < 1.0) {
                    if (jm1 > 0 && f[ID2(i, jm1)] == 1.0)
                        dyy = (1.0 * uyk[ID2(i, jm1 - 1)] - 4.0 * uyk[ID2(i, jm1)] + 3.0 * uyk[c]) / (2.0 * dy);
                    else
                        dyy = (uyk[c] - uyk[ID2(i, jm1)]) / dy;
                } else if (f[c] < 1.0 && f[ID2(i, jp1)] == 1.0) {
                    if (jp1 < ny - 1 && f[ID2(i, jp1 + 1)] == 1.0)
                        dyy = -(1.0 * uyk[ID2(i, jp1 + 1)] - 4.0 * uyk[ID2(i, jp1)] + 3.0 * uyk[c]) / (2.0 * dy);
                    else
                        dyy = (uyk[ID2(i, jp1)] - uyk[c]) / dy;
                }
                const double zk = za[k];
                const double c_x = -((1.0 - zk) * J->dzbdx[c] + zk * J->dzsdx[c]);
                const double c_y = -((1.0 - zk) * J->dzbdy[c] + zk * J->dzsdy[c]);
                const double dzbdx_acy = mean4_act(J->dzbdx[c], J->dzbdx[ID2(i, jp1)], J->dzbdx[ID2(im1, j)],
                                                   J->dzbdx[ID2(im1, jp1)], ax[c], ax[ID2(i, jp1)], ax[ID2(im1, j)],
                                                   ax[ID2(im1, jp1)]);
                const double dzsdx_acy = mean4_act(J->dzsdx[c], J->dzsdx[ID2(i, jp1)], J->dzsdx[ID2(im1, j)],
                                                   J->dzsdx[ID2(im1, jp1)], ax[c], ax[ID2(i, jp1)], ax[ID2(im1, j)],
                                                   ax[ID2(im1, jp1)]);
                const double c_x_acy = -((1.0 - zk) * dzbdx_acy + zk * dzsdx_acy);
                const double dzbdy_acx = mean4_act(J->dzbdy[c], J->dzbdy[ID2(ip1, j)], J->dzbdy[ID2(i, jm1)],
                                                   J->dzbdy[ID2(ip1, jm1)], ay[c], ay[ID2(ip1, j)], ay[ID2(i, jm1)],
                                                   ay[ID2(ip1, jm1)]);
                const double dzsdy_acx = mean4_act(J->dzsdy[c], J->dzsdy[ID2(ip1, j)], J->dzsdy[ID2(i, jm1)],
                                                   J->dzsdy[ID2(ip1, jm1)], ay[c], ay[ID2(ip1, j)], ay[ID2(i, jm1)],
                                                   ay[ID2(ip1, jm1)]);
                const double c_y_acx = -((1.0 - zk) * dzbdy_acx + zk * dzsdy_acx);
                J->dxx[o + c] = dxx + c_x * J->dxz[o + c];
                J->dxy[o + c] = dxy + c_y_acx * J->dxz[o + c];
                J->dyx[o + c] = dyx + c_x_acy * J->dyz[o + c];
                J->dyy[o + c] = dyy + c_y * J->dyz[o + c];
            }
        }
    free(ax);
    free(ay);
}

/* calc_jacobian_vel_3D_uzterms, deformation.f90:718-961 */
static void jac_uzterms(const ygpu_jvel* J, int bc) {
    const int nx = J->nx, ny = J->ny, nz = J->nz_ac;
    const size_t n2 = (size_t)nx * ny;
    const double *f = J->f_ice, *uz = J->uz, *zc = J->zeta_ac;
    memset(J->dzx, 0, n2 * nz * sizeof(double));
    memset(J->dzy, 0, n2 * nz * sizeof(double));
    memset(J->dzz, 0, n2 * nz * sizeof(double));
    /* step 1: dzz on the ice-covered cells (:782-842) */
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t c = ID2(i, j);
            if (f[c] != 1.0) continue;
            for (int k = 0; k < nz; k++) J->dzz[k * n2 + c] = jac_vderiv(uz, c, n2, zc, k, nz, J->H_ice[c], 0);
        }
    /* step 2: dzx, dzy with the corrections (:846-955) */
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = ID2(i, j);
            if (f[c] != 1.0) continue;
            for (int k = 0; k < nz; k++) {
                const size_t o = k * n2;
                const double* u = uz + o;
                double dzx = (u[ID2(ip1, j)] - u[ID2(im1, j)]) / (2.0 * J->dx);
                double dzy = (u[ID2(i, jp1)] - u[ID2(i, jm1)]) / (2.0 * J->dy);
                if (f[ID2(ip1, j)] < 1.0 && f[ID2(im1, j)] < 1.0) {
                    dzx = 0.0;
                } else if (f[ID2(ip1, j)] < 1.0 && f[ID2(im1, j)] == 1.0) {
                    if (im1 > 0 && f[ID2(im1 - 1, j)] == 1.0)
                        dzx = (1.0 * u[ID2(im1 - 1, j)] - 4.0 * u[ID2(im1, j)] + 3.0 * u[c]) / (2.0 * J->dx);
                    else
                        dzx = (u[c] - u[ID2(im1, j)]) / J->dx;
                } else if (f[ID2(ip1, j)] == 1.0 && f[ID2(im1, j)] < 1.0) {
                    if (ip1 < nx - 1 && f[ID2(ip1 + 1, j)] == 1.0)
                        dzx = -(1.0 * u[ID2(ip1 + 1, j)] - 4.0 * u[ID2(ip1, j)] + 3.0 * u[c]) / (2.0 * J->dx);
                    else
                        dzx = (u[ID2(ip1, j)] - u[c]) / J->dx;
                }
                if (f[ID2(i, jp1)] < 1.0 && f[ID2(i, jm1)] < 1.0) {
                    dzy = 0.0;
                } else if (f[ID2(i, jp1)] < 1.0 && f[ID2(i, jm1)] == 1.0) {
                    if (jm1 > 0 && f[ID2(i, jm1 - 1)] == 1.0)
                        dzy = (1.0 * u[ID2(i, jm1 - 1)] - 4.0 * u[ID2(i, jm1)] + 3.0 * u[c]) / (2.0 * J->dy);
                    else
                        dzy = (u[c] - u[ID2(i, jm1)]) / J->dy;
                } else if (f[ID2(i, jp1)] == 1.0 && f[ID2(i, jm1)] < 1.0) {
                    if (jp1 < ny - 1 && f[ID2(i, jp1 + 1)] == 1.0)
                        dzy = -(1.0 * u[ID2(i, jp1 + 1)] - 4.0 * u[ID2(i, jp1)] + 3.0 * u[c]) / (2.0 * J->dy);
                    else
                        dzy = (u[ID2(i, jp1)] - u[c]) / J->dy;
                }
                const double dzbdx_aa = 0.5 * (J->dzbdx[c] + J->dzbdx[ID2(im1, j)]);
                const double dzbdy_aa = 0.5 * (J->dzbdy[c] + J->dzbdy[ID2(i, jm1)]);
                const double dzsdx_aa = 0.5 * (J->dzsdx[c] + J->dzsdx[ID2(im1, j)]);
                const double dzsdy_aa = 0.5 * (J->dzsdy[c] + J->dzsdy[ID2(i, jm1)]);
                const double c_x = -((1.0 - zc[k]) * dzbdx_aa + zc[k] * dzsdx_aa);
                const double c_y = -((1.0 - zc[k]) * dzbdy_aa + zc[k] * dzsdy_aa);
                J->dzx[o + c] = dzx + c_x * J->dzz[o + c];
                J->dzy[o + c] = dzy + c_y * J->dzz[o + c];
            }
        }
}

int orc_calc_jacobian_vel_3D(const ygpu_jvel* J, int bc, int terms) {
    if (!J || J->nx < 2 || J->ny < 2 || terms < 1 || terms > 3) return YGPU_ERR_BAD_ARG;
    if ((terms & YGPU_JAC_UXY) && J->nz_aa < 3) return YGPU_ERR_BAD_ARG;
    if ((terms & YGPU_JAC_UZ) && J->nz_ac < 3) return YGPU_ERR_BAD_ARG;
    if (terms & YGPU_JAC_UXY) jac_uxyterms(J, bc);
    if (terms & YGPU_JAC_UZ) jac_uzterms(J, bc);
    return YGPU_OK;
}

/* ======================================================================== */
/* Vertical velocity (calc_ydyn, yelmo_dynamics.f90:259-290)                */
/* ======================================================================== */

static inline double flush_tiny(double v) { return fabs(v) < TOL_UNDERFLOW ? 0.0 : v; }

/* calc_uz_3D_aa, velocity_general.f90:683-945 (0-based: ac level kc, aa layer ka) */
static void uz_aa(const ygpu_uz3d* U, int bc) {
    const int nx = U->nx, ny = U->ny, nza = U->nz_aa, nzc = U->nz_ac;
    const size_t n2 = (size_t)nx * ny;
    const double *za = U->zeta_aa, *zc = U->zeta_ac, *ux = U->ux, *uy = U->uy;
    const double f_bmb = U->use_bmb ? 1.0 : 0.0;
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = ID2(i, j), cxm = ID2(im1, j), cym = ID2(i, jm1);
            const double dzsdt_now = U->dzsdt[c], dzbdt_now = U->dzbdt[c];
#define UX(ii, k) ux[(size_t)(k) * n2 + (ii)]
#define UY(ii, k) uy[(size_t)(k) * n2 + (ii)]
            if (U->f_ice[c] == 1.0) {
                const double H_now = U->H_ice[c], H_inv = 1.0 / H_now;
                const double dzbdx_aa = 0.5 * (U->dzbdx[c] + U->dzbdx[cxm]);
                const double dzbdy_aa = 0.5 * (U->dzbdy[c] + U->dzbdy[cym]);
                const double dzsdx_aa = 0.5 * (U->dzsdx[c] + U->dzsdx[cxm]);
                const double dzsdy_aa = 0.5 * (U->dzsdy[c] + U->dzsdy[cym]);
                double ux_aa = 0.5 * (UX(cxm, 0) + UX(c, 0));
                double uy_aa = 0.5 * (UY(cym, 0) + UY(c, 0));
                const double uz_grid = 0.0;
                /* basal value, Greve and Blatter (2009) Eq. 5.31 */
                double u0 = dzbdt_now + uz_grid + f_bmb * U->bmb[c] + ux_aa * dzbdx_aa + uy_aa * dzbdy_aa;
                U->uz[c] = flush_tiny(u0);
                for (int kc = 1; kc < nzc; kc++) {
                    const int ka = kc - 1;
                    const double duxdx_aa = (UX(c, ka) - UX(cxm, ka)) / U->dx;
                    const double duydy_aa = (UY(c, ka) - UY(cym, ka)) / U->dy;
                    double duxdz_aa, duydz_aa;
                    int hi, lo;
                    if (kc == 1) { hi = 1; lo = 0; }
                    else if (kc == nzc - 1) { hi = nza - 1; lo = nza - 2; }
                    else { hi = kc; lo = kc - 2; }
                    duxdz_aa = (0.5 * (UX(c, hi) + UX(cxm, hi)) - 0.5 * (UX(c, lo) + UX(cxm, lo))) / (za[hi] - za[lo]);
                    duydz_aa = (0.5 * (UY(c, hi) + UY(cym, hi)) - 0.5 * (UY(c, lo) + UY(cym, lo))) / (za[hi] - za[lo]);
                    const double c_x = -H_inv * ((1.0 - zc[kc]) * dzbdx_aa + zc[kc] * dzsdx_aa);
                    const double c_y = -H_inv * ((1.0 - zc[kc]) * dzbdy_aa + zc[kc] * dzsdy_aa);
                    const double duxdx_now = duxdx_aa + c_x * duxdz_aa;
                    const double duydy_now = duydy_aa + c_y * duydz_aa;
                    const double u = U->uz[(size_t)(kc - 1) * n2 + c] - H_now * (zc[kc] - zc[kc - 1]) * (duxdx_now + duydy_now);
                    U->uz[(size_t)kc * n2 + c] = flush_tiny(u);
                }
                /* uz_star, Greve and Blatter (2009) Eq. 5.148 (no 1/H) */
                for (int kc = 0; kc < nzc; kc++) {
                    if (kc == 0) {
                        ux_aa = 0.5 * (UX(cxm, 0) + UX(c, 0));
                        uy_aa = 0.5 * (UY(cym, 0) + UY(c, 0));
                    } else if (kc == nzc - 1) {
                        ux_aa = 0.5 * (UX(cxm, kc - 1) + UX(c, kc - 1));
                        uy_aa = 0.5 * (UY(cym, kc - 1) + UY(c, kc - 1));
                    } else {
                        ux_aa = 0.25 * (UX(cxm, kc) + UX(c, kc) + UX(cxm, kc - 1) + UX(c, kc - 1));
                        uy_aa = 0.25 * (UY(cym, kc) + UY(c, kc) + UY(cym, kc - 1) + UY(c, kc - 1));
                    }
                    const double z = zc[kc];
                    const double c_x = -ux_aa * ((1.0 - z) * dzbdx_aa + z * dzsdx_aa);
                    const double c_y = -uy_aa * ((1.0 - z) * dzbdy_aa + z * dzsdy_aa);
                    const double c_t = -((1.0 - z) * dzbdt_now + z * dzsdt_now);
                    U->uz_star[(size_t)kc * n2 + c] = flush_tiny(U->uz[(size_t)kc * n2 + c] + c_x + c_y + c_t);
                }
            } else {
                for (int kc = 0; kc < nzc; kc++) {
                    const double u = flush_tiny(dzbdt_now - fmax(U->smb[c], 0.0));
                    U->uz[(size_t)kc * n2 + c] = u;
                    U->uz_star[(size_t)kc * n2 + c] = u;
                }
            }
        }
}

/* calc_uz_3D_flux, velocity_general.f90:947-1116 */
static void uz_flux(const ygpu_uz3d* U, int bc) {
    const int nx = U->nx, ny = U->ny, nza = U->nz_aa, nzc = U->nz_ac;
    const size_t n2 = (size_t)nx * ny;
    const double *zc = U->zeta_ac, *ux = U->ux, *uy = U->uy, *H = U->H_ice;
    const double f_bmb = U->use_bmb ? 1.0 : 0.0;
    double* dzeta = malloc((size_t)nza * sizeof(double));
    for (int k = 0; k < nza; k++) dzeta[k] = zc[k + 1] - zc[k];
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = ID2(i, j), cxm = ID2(im1, j), cym = ID2(i, jm1);
            const size_t cxp = ID2(ip1, j), cyp = ID2(i, jp1);
            if (U->f_ice[c] == 1.0) {
                const double Hx_w = (U->ux_bar[cxm] >= 0.0) ? H[cxm] : H[c];
                const double Hx_e = (U->ux_bar[c] >= 0.0) ? H[c] : H[cxp];
                const double Hy_s = (U->uy_bar[cym] >= 0.0) ? H[cym] : H[c];
                const double Hy_n = (U->uy_bar[c] >= 0.0) ? H[c] : H[cyp];
                double D[1001];
                for (int k = 0; k < nza; k++)
                    D[k] = dzeta[k] * ((Hx_e * UX(c, k) - Hx_w * UX(cxm, k)) / U->dx +
                                       (Hy_n * UY(c, k) - Hy_s * UY(cym, k)) / U->dy);
                if (U->mask_kin[c] == 1) {
                    double tot = 0.0;
                    for (int k = 0; k < nza; k++) tot += D[k];
                    const double corr = -U->dHidt_dyn[c] - tot;
                    for (int k = 0; k < nza; k++) D[k] = D[k] + dzeta[k] * corr;
                }
                const double dHdt = U->dzsdt[c] - U->dzbdt[c];
                double* us = U->uz_star;
                us[c] = f_bmb * U->bmb[c];
                for (int k = 0; k < nza; k++)
                    us[(size_t)(k + 1) * n2 + c] = us[(size_t)k * n2 + c] - dzeta[k] * dHdt - D[k];
                const double dzbdx_aa = 0.5 * (U->dzbdx[c] + U->dzbdx[cxm]);
                const double dzbdy_aa = 0.5 * (U->dzbdy[c] + U->dzbdy[cym]);
                const double dzsdx_aa = 0.5 * (U->dzsdx[c] + U->dzsdx[cxm]);
                const double dzsdy_aa = 0.5 * (U->dzsdy[c] + U->dzsdy[cym]);
                for (int kc = 0; kc < nzc; kc++) {
                    double ux_aa, uy_aa;
                    if (kc == 0) {
                        ux_aa = 0.5 * (UX(cxm, 0) + UX(c, 0));
                        uy_aa = 0.5 * (UY(cym, 0) + UY(c, 0));
                    } else if (kc == nzc - 1) {
                        ux_aa = 0.5 * (UX(cxm, kc - 1) + UX(c, kc - 1));
                        uy_aa = 0.5 * (UY(cym, kc - 1) + UY(c, kc - 1));
                    } else {
                        ux_aa = 0.25 * (UX(cxm, kc) + UX(c, kc) + UX(cxm, kc - 1) + UX(c, kc - 1));
                        uy_aa = 0.25 * (UY(cym, kc) + UY(c, kc) + UY(cym, kc - 1) + UY(c, kc - 1));
                    }
                    const double z = zc[kc];
                    const double c_x = -ux_aa * ((1.0 - z) * dzbdx_aa + z * dzsdx_aa);
                    const double c_y = -uy_aa * ((1.0 - z) * dzbdy_aa + z * dzsdy_aa);
                    const double c_t = -((1.0 - z) * U->dzbdt[c] + z * U->dzsdt[c]);
                    const size_t o = (size_t)kc * n2 + c;
                    U->uz[o] = flush_tiny(us[o] - (c_x + c_y + c_t));
                    us[o] = flush_tiny(us[o]);
                }
            } else {
                for (int kc = 0; kc < nzc; kc++) {
                    const double u = flush_tiny(U->dzbdt[c] - fmax(U->smb[c], 0.0));
                    U->uz[(size_t)kc * n2 + c] = u;
                    U->uz_star[(size_t)kc * n2 + c] = u;
                }
            }
#undef UX
#undef UY
        }
    free(dzeta);
}


/* ------------------------------------------------------------------------ */
/* 3D Gaussian quadrature (fesm-utils gq3D, restated as gq2D above; unpinned) */
/* ------------------------------------------------------------------------ */
/* Node q = (qx, qy, qz) in bits 0, 1, 2 (0: -, 1: +) at (sx*g, sy*g, sz*g),
   g = 1/sqrt(3); corner c likewise; trilinear weight of corner c at node q =
   prod over the axes of (1 + s_q*s_c*g)/2. The corners are the 8 corners of the
   cell-layer box: horizontally as gq2D's (SW, SE, NE, NW), vertically the lower
   and upper face of the layer. The dz arguments of the reference's gq3D calls do
   not enter the mapping. */
static double GQ3W[8][8];
static int gq3_ready = 0;

static void gq3_init(void) {
    if (gq3_ready) return;
    double g = 1.0 / sqrt(3.0);
    for (int q = 0; q < 8; q++)
        for (int c = 0; c < 8; c++) {
            double w = 1.0;
            for (int a = 0; a < 3; a++) {
                double sq = ((q >> a) & 1) ? 1.0 : -1.0, sc = ((c >> a) & 1) ? 1.0 : -1.0;
                w = w * ((1.0 + sq * sc * g) * 0.5);
            }
            GQ3W[q][c] = w;
        }
    gq3_ready = 1;
}

/* horizontal corner h (0 SW, 1 SE, 2 NE, 3 NW) and level l (0 lower, 1 upper) ->
   corner index c with bits (x, y, z) */
static inline int gq3_corner(int h, int l) {
    static const int hx[4] = {0, 1, 1, 0}, hy[4] = {0, 0, 1, 1};
    return hx[h] | (hy[h] << 1) | (l << 2);
}

static inline void gq3_corners_to_nodes(const double c[8], double v[8]) {
    for (int q = 0; q < 8; q++) {
        double s = 0.0;
        for (int k = 0; k < 8; k++) s = s + GQ3W[q][k] * c[k];
        v[q] = s;
    }
}

/* sum(v*wt)/wt_tot with the equal Gauss-Legendre weights */
static inline double gq3_mean(const double v[8]) {
    double s = 0.0;
    for (int q = 0; q < 8; q++) s = s + v[q];
    return s / 8.0;
}

/* gq3D_to_nodes_acx on layer k (0-based) with the layers km1, kp1 below and above
   (clamped by the caller): a lower corner is the mean of the two acx faces beside
   it on layers km1 and k (active faces only), an upper corner on layers k and kp1 */
static void gq3_nodes_acx(const double* var, const unsigned char* act, int i, int j, int k, int km1, int kp1,
                          int im1, int jm1, int jp1, int nx, size_t n2, double v[8]) {
    double c[8];
    const int ic[4] = {im1, i, i, im1};
    const int ja[4] = {jm1, jm1, j, j};
    const int jb[4] = {j, j, jp1, jp1};
    const int lay[2][2] = {{km1, k}, {k, kp1}};
    for (int h = 0; h < 4; h++)
        for (int l = 0; l < 2; l++) {
            const double* p0 = var + (size_t)lay[l][0] * n2;
            const double* p1 = var + (size_t)lay[l][1] * n2;
            const size_t a = ID2(ic[h], ja[h]), b = ID2(ic[h], jb[h]);
            double m0 = mean2_act(p0[a], p0[b], act[a], act[b]);
            double m1 = mean2_act(p1[a], p1[b], act[a], act[b]);
            c[gq3_corner(h, l)] = 0.5 * (m0 + m1);
        }
    gq3_corners_to_nodes(c, v);
}

/* gq3D_to_nodes_acy: as acx with the two acy faces left and right of a corner */
static void gq3_nodes_acy(const double* var, const unsigned char* act, int i, int j, int k, int km1, int kp1,
                          int im1, int ip1, int jm1, int nx, size_t n2, double v[8]) {
    double c[8];
    const int ia[4] = {im1, i, i, im1};
    const int ib[4] = {i, ip1, ip1, i};
    const int jc[4] = {jm1, jm1, j, j};
    const int lay[2][2] = {{km1, k}, {k, kp1}};
    for (int h = 0; h < 4; h++)
        for (int l = 0; l < 2; l++) {
            const double* p0 = var + (size_t)lay[l][0] * n2;
            const double* p1 = var + (size_t)lay[l][1] * n2;
            const size_t a = ID2(ia[h], jc[h]), b = ID2(ib[h], jc[h]);
            double m0 = mean2_act(p0[a], p0[b], act[a], act[b]);
            double m1 = mean2_act(p1[a], p1[b], act[a], act[b]);
            c[gq3_corner(h, l)] = 0.5 * (m0 + m1);
        }
    gq3_corners_to_nodes(c, v);
}

/* gq3D_to_nodes_acz: a field on the vertical faces (ac levels) and the horizontal
   cell centres; the lower corners are the means of the four cells around each
   corner on ac level klo, the upper ones on level khi */
static void gq3_nodes_acz(const double* var, int i, int j, int klo, int khi, int im1, int ip1, int jm1, int jp1,
                          int nx, size_t n2, double v[8]) {
    double c[8];
    const int ii[4][4] = {{im1, i, im1, i}, {i, ip1, i, ip1}, {i, ip1, i, ip1}, {im1, i, im1, i}};
    const int jj[4][4] = {{jm1, jm1, j, j}, {jm1, jm1, j, j}, {j, j, jp1, jp1}, {j, j, jp1, jp1}};
    const int lev[2] = {klo, khi};
    for (int h = 0; h < 4; h++)
        for (int l = 0; l < 2; l++) {
            const double* p = var + (size_t)lev[l] * n2;
            double s = p[ID2(ii[h][0], jj[h][0])] + p[ID2(ii[h][1], jj[h][1])];
            s = s + p[ID2(ii[h][2], jj[h][2])];
            s = s + p[ID2(ii[h][3], jj[h][3])];
            c[gq3_corner(h, l)] = 0.25 * s;
        }
    gq3_corners_to_nodes(c, v);
}

/* the 2D quadrature value of an acx / acy field at cell (i, j) */
static inline double gq_acx_value(const double* var, const unsigned char* act, int i, int j, int im1, int jm1,
                                  int jp1, int nx) {
    double v[4];
    gq_nodes_acx(var, act, i, j, im1, jm1, jp1, nx, v);
    return gq_mean(v);
}
static inline double gq_acy_value(const double* var, const unsigned char* act, int i, int j, int im1, int ip1,
                                  int jm1, int nx) {
    double v[4];
    gq_nodes_acy(var, act, i, j, im1, ip1, jm1, nx, v);
    return gq_mean(v);
}

/* calc_uz_3D (uz_method 2), velocity_general.f90:346-681, and calc_uz_3D_jac
   (uz_method 3), :41-344 (0-based: ac level kc, aa layer ka) */
static void uz_quad(const ygpu_uz3d* U, int bc, int jac) {
    const int nx = U->nx, ny = U->ny, nza = U->nz_aa, nzc = U->nz_ac;
    const size_t n2 = (size_t)nx * ny;
    const double *za = U->zeta_aa, *zc = U->zeta_ac, *ux = U->ux, *uy = U->uy;
    const double f_bmb = U->use_bmb ? 1.0 : 0.0;
    gq_init();
    gq3_init();
    unsigned char* ax = malloc(n2);
    unsigned char* ay = malloc(n2);
    active_faces(ax, ay, U->f_ice, bc, nx, ny);
    double *dudx = NULL, *dvdy = NULL;
    if (!jac) {
        /* the per-layer horizontal strain rates (:453-458), no sigma correction */
        dudx = malloc(n2 * (size_t)nza * sizeof(double));
        dvdy = malloc(n2 * (size_t)nza * sizeof(double));
        double* dudy = malloc(n2 * sizeof(double));
        double* dvdx = malloc(n2 * sizeof(double));
        for (int k = 0; k < nza; k++)
            strain_rate_2D(dudx + (size_t)k * n2, dudy, dvdx, dvdy + (size_t)k * n2, ux + (size_t)k * n2,
                           uy + (size_t)k * n2, U->f_ice, ax, ay, U->dx, U->dy, bc, nx, ny);
        free(dudy);
        free(dvdx);
    }
#pragma omp parallel for collapse(2)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = ID2(i, j);
            const double dzsdt_now = U->dzsdt[c], dzbdt_now = U->dzbdt[c];
            if (U->f_ice[c] == 1.0) {
                const double H_now = U->H_ice[c], H_inv = 1.0 / H_now;
                const double dzbdx_aa = gq_acx_value(U->dzbdx, ax, i, j, im1, jm1, jp1, nx);
                const double dzbdy_aa = gq_acy_value(U->dzbdy, ay, i, j, im1, ip1, jm1, nx);
                const double dzsdx_aa = gq_acx_value(U->dzsdx, ax, i, j, im1, jm1, jp1, nx);
                const double dzsdy_aa = gq_acy_value(U->dzsdy, ay, i, j, im1, ip1, jm1, nx);
                double ux_aa = gq_acx_value(ux, ax, i, j, im1, jm1, jp1, nx);
                double uy_aa = gq_acy_value(uy, ay, i, j, im1, ip1, jm1, nx);
                const double uz_grid = 0.0;
                /* basal value, Greve and Blatter (2009) Eq. 5.31 */
                U->uz[c] = flush_tiny(dzbdt_now + uz_grid + f_bmb * U->bmb[c] + ux_aa * dzbdx_aa + uy_aa * dzbdy_aa);
                for (int kc = 1; kc < nzc; kc++) {
                    double dudx_aa, dvdy_aa;
                    if (jac) {
                        /* :218-233: layer kmid below the level, its neighbours clamped */
                        const int kmid = kc - 1;
                        const int km1 = kmid > 0 ? kmid - 1 : 0, kp1 = kmid < nza - 1 ? kmid + 1 : nza - 1;
                        double v[8];
                        gq3_nodes_acx(U->jac_dxx, ax, i, j, kmid, km1, kp1, im1, jm1, jp1, nx, n2, v);
                        dudx_aa = gq3_mean(v);
                        gq3_nodes_acy(U->jac_dyy, ay, i, j, kmid, km1, kp1, im1, ip1, jm1, nx, n2, v);
                        dvdy_aa = gq3_mean(v);
                    } else {
                        /* :535-579 */
                        const double zeta_now = za[kc - 1];
                        const double c_x = -H_inv * ((1.0 - zeta_now) * dzbdx_aa + zeta_now * dzsdx_aa);
                        const double c_y = -H_inv * ((1.0 - zeta_now) * dzbdy_aa + zeta_now * dzsdy_aa);
                        int kup, kdn;
                        if (kc == 1) { kup = 1; kdn = 0; }
                        else if (kc == nzc - 1) { kup = kc - 1; kdn = kc - 2; }
                        else { kup = kc; kdn = kc - 2; }
                        double vu[4], vd[4], dn[4];
                        gq_nodes_acx(ux + (size_t)kup * n2, ax, i, j, im1, jm1, jp1, nx, vu);
                        gq_nodes_acx(ux + (size_t)kdn * n2, ax, i, j, im1, jm1, jp1, nx, vd);
                        for (int q = 0; q < 4; q++) dn[q] = (vu[q] - vd[q]) / (za[kup] - za[kdn]);
                        const double dudz_aa = gq_mean(dn);
                        gq_nodes_acy(uy + (size_t)kup * n2, ay, i, j, im1, ip1, jm1, nx, vu);
                        gq_nodes_acy(uy + (size_t)kdn * n2, ay, i, j, im1, ip1, jm1, nx, vd);
                        for (int q = 0; q < 4; q++) dn[q] = (vu[q] - vd[q]) / (za[kup] - za[kdn]);
                        const double dvdz_aa = gq_mean(dn);
                        dudx_aa = gq_acx_value(dudx + (size_t)(kc - 1) * n2, ax, i, j, im1, jm1, jp1, nx) +
                                  c_x * dudz_aa;
                        dvdy_aa = gq_acy_value(dvdy + (size_t)(kc - 1) * n2, ay, i, j, im1, ip1, jm1, nx) +
                                  c_y * dvdz_aa;
                    }
                    /* Greve and Blatter (2009) Eq. 5.95 */
                    const double u = U->uz[(size_t)(kc - 1) * n2 + c] - H_now * (zc[kc] - zc[kc - 1]) * (dudx_aa + dvdy_aa);
                    U->uz[(size_t)kc * n2 + c] = flush_tiny(u);
                }
                /* uz_star, Greve and Blatter (2009) Eq. 5.148 (no 1/H) */
                for (int kc = 0; kc < nzc; kc++) {
                    int kup, kdn;
                    if (kc == 0) { kup = 0; kdn = 0; }
                    else if (kc == nzc - 1) { kup = kc - 1; kdn = kc - 1; }
                    else { kup = kc; kdn = kc - 1; }
                    double vu[4], vd[4], vn[4];
                    gq_nodes_acx(ux + (size_t)kup * n2, ax, i, j, im1, jm1, jp1, nx, vu);
                    gq_nodes_acx(ux + (size_t)kdn * n2, ax, i, j, im1, jm1, jp1, nx, vd);
                    for (int q = 0; q < 4; q++) vn[q] = 0.5 * (vu[q] + vd[q]);
                    ux_aa = gq_mean(vn);
                    gq_nodes_acy(uy + (size_t)kup * n2, ay, i, j, im1, ip1, jm1, nx, vu);
                    gq_nodes_acy(uy + (size_t)kdn * n2, ay, i, j, im1, ip1, jm1, nx, vd);
                    for (int q = 0; q < 4; q++) vn[q] = 0.5 * (vu[q] + vd[q]);
                    uy_aa = gq_mean(vn);
                    const double z = zc[kc];
                    const double c_x = -((1.0 - z) * dzbdx_aa + z * dzsdx_aa);
                    const double c_y = -((1.0 - z) * dzbdy_aa + z * dzsdy_aa);
                    const double c_t = -((1.0 - z) * dzbdt_now + z * dzsdt_now);
                    const size_t o = (size_t)kc * n2 + c;
                    double us;
                    if (jac) us = ux_aa * c_x + uy_aa * c_y + U->uz[o] * 1.0 + c_t;
                    else us = U->uz[o] + ux_aa * c_x + uy_aa * c_y + c_t;
                    U->uz_star[o] = flush_tiny(us);
                }
            } else {
                for (int kc = 0; kc < nzc; kc++) {
                    const double u = flush_tiny(dzbdt_now - fmax(U->smb[c], 0.0));
                    U->uz[(size_t)kc * n2 + c] = u;
                    U->uz_star[(size_t)kc * n2 + c] = u;
                }
            }
        }
    free(ax);
    free(ay);
    free(dudx);
    free(dvdy);
}

int orc_calc_uz_3D(const ygpu_uz3d* U, int bc, int method) {
    if (!U || U->nx < 2 || U->ny < 2 || U->nz_aa < 2 || U->nz_aa > 1000 || U->nz_ac != U->nz_aa + 1)
        return YGPU_ERR_BAD_ARG;
    if (method == YGPU_UZ_JAC && (!U->jac_dxx || !U->jac_dyy)) return YGPU_ERR_BAD_ARG;
    if (method == YGPU_UZ_AA) uz_aa(U, bc);
    else if (method == YGPU_UZ_FLUX) uz_flux(U, bc);
    else if (method == YGPU_UZ_NODES) uz_quad(U, bc, 0);
    else if (method == YGPU_UZ_JAC) uz_quad(U, bc, 1);
    else return YGPU_ERR_BAD_ARG;
    if (U->uz_srf_err) {
        const size_t n2 = (size_t)U->nx * U->ny, top = (size_t)(U->nz_ac - 1) * n2;
        for (size_t c = 0; c < n2; c++)
            U->uz_srf_err[c] = (U->f_ice[c] == 1.0) ? U->uz_star[top + c] + U->smb[c] : 0.0;
    }
    return YGPU_OK;
}

/* ======================================================================== */
/* Strain-rate tensor (calc_ydyn, yelmo_dynamics.f90:299-300)              */
/* ======================================================================== */

/* calc_2D_eigen_values, deformation.f90:1542-1595 */
static void eigen_2D(double* e1, double* e2, double txx, double tyy, double txy) {
    const double a = 1.0, b = -(txx + tyy), c = txx * tyy - txy * txy;
    if (b * b - 4.0 * a * c > 0.0) {
        const double root = sqrt(b * b - 4.0 * a * c);
        const double l1 = (-b + root) / (2.0 * a), l2 = (-b - root) / (2.0 * a);
        if (l1 > l2) { *e1 = l1; *e2 = l2; }
        else { *e1 = l2; *e2 = l1; }
    } else {
        *e1 = 0.0;
        *e2 = 0.0;
    }
}

/* calc_strain_rate_tensor_jac_quad3D, deformation.f90:963-1183 (0-based layer k) */
int orc_calc_strain_rate_tensor(const ygpu_strain3d* S, int bc) {
    if (!S || S->nx < 2 || S->ny < 2 || S->nz_aa < 2 || S->nz_aa > 1000 || S->nz_ac != S->nz_aa + 1)
        return YGPU_ERR_BAD_ARG;
    const int nx = S->nx, ny = S->ny, nza = S->nz_aa;
    const size_t n2 = (size_t)nx * ny, n3 = n2 * (size_t)nza;
    gq3_init();
    unsigned char* ax = malloc(n2);
    unsigned char* ay = malloc(n2);
    active_faces(ax, ay, S->f_ice, bc, nx, ny);
    double* out3[8] = {S->s_dxx, S->s_dyy, S->s_dxy, S->s_dxz, S->s_dyz, S->s_de, S->s_div, S->s_f_shear};
    for (int q = 0; q < 8; q++) memset(out3[q], 0, n3 * sizeof(double));
#pragma omp parallel for collapse(2) schedule(dynamic, 64)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t c = ID2(i, j);
            if (!(S->f_ice[c] == 1.0)) continue;
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            for (int k = 0; k < nza; k++) {
                const int km1 = k > 0 ? k - 1 : 0, kp1 = k < nza - 1 ? k + 1 : nza - 1;
                double dn[8], an[8], bn[8];
                const size_t o = (size_t)k * n2 + c;
                gq3_nodes_acx(S->dxx, ax, i, j, k, km1, kp1, im1, jm1, jp1, nx, n2, dn);
                const double dxx = gq3_mean(dn);
                gq3_nodes_acx(S->dxy, ax, i, j, k, km1, kp1, im1, jm1, jp1, nx, n2, an);
                gq3_nodes_acy(S->dyx, ay, i, j, k, km1, kp1, im1, ip1, jm1, nx, n2, bn);
                for (int q = 0; q < 8; q++) dn[q] = 0.5 * (an[q] + bn[q]);
                const double dxy = gq3_mean(dn);
                /* dzx on the ac levels k (below) and k+1 (above) of layer k */
                gq3_nodes_acx(S->dxz, ax, i, j, k, km1, kp1, im1, jm1, jp1, nx, n2, an);
                gq3_nodes_acz(S->dzx, i, j, k, k + 1, im1, ip1, jm1, jp1, nx, n2, bn);
                for (int q = 0; q < 8; q++) dn[q] = 0.5 * (an[q] + bn[q]);
                const double dxz = gq3_mean(dn);
                gq3_nodes_acy(S->dyz, ay, i, j, k, km1, kp1, im1, ip1, jm1, nx, n2, an);
                gq3_nodes_acz(S->dzy, i, j, k, k + 1, im1, ip1, jm1, jp1, nx, n2, bn);
                for (int q = 0; q < 8; q++) dn[q] = 0.5 * (an[q] + bn[q]);
                const double dyz = gq3_mean(dn);
                gq3_nodes_acy(S->dyy, ay, i, j, k, km1, kp1, im1, ip1, jm1, nx, n2, dn);
                const double dyy = gq3_mean(dn);
                double de = sqrt(dxx * dxx + dyy * dyy + dxx * dyy + dxy * dxy + dxz * dxz + dyz * dyz);
                if (de > S->de_max) de = S->de_max;
                double fs;
                if (de > 0.0) fs = sqrt(dxz * dxz + dyz * dyz) / de;
                else fs = 1.0;
                if (S->f_grnd[c] == 0.0) fs = 0.0;
                fs = fmin(fmax(fs, 0.0), 1.0);
                S->s_dxx[o] = dxx; S->s_dyy[o] = dyy; S->s_dxy[o] = dxy; S->s_dxz[o] = dxz;
                S->s_dyz[o] = dyz; S->s_de[o] = de; S->s_div[o] = dxx + dyy; S->s_f_shear[o] = fs;
            }
        }
    /* vertical averages (calc_vertical_integrated_2D) and the eigenvalues */
    double* out2[8] = {S->a_dxx, S->a_dyy, S->a_dxy, S->a_dxz, S->a_dyz, S->a_de, S->a_div, S->a_f_shear};
    for (int q = 0; q < 8; q++) {
        if (!out2[q]) continue;
        for (size_t c = 0; c < n2; c++) out2[q][c] = trapz_pt(out3[q] + c, S->zeta_aa, nza, n2);
    }
    if (S->eps_eig_1 && S->eps_eig_2 && S->a_dxx && S->a_dyy && S->a_dxy)
        for (size_t c = 0; c < n2; c++) eigen_2D(&S->eps_eig_1[c], &S->eps_eig_2[c], S->a_dxx[c], S->a_dyy[c], S->a_dxy[c]);
    free(ax);
    free(ay);
    return YGPU_OK;
}

/* ======================================================================== */
/* Implicit upwind advection, calc_advec2D(solver = "impl-lis")             */
/* ======================================================================== */

enum { ADV_PERIODIC = 0, ADV_ZERO = 1, ADV_INFINITE = 2, ADV_OUTFLOW = 3 };

/* define_advection_bcs, solver_advection.f90:548-622 (right, upper, left, lower) */
static void adv_kinds(int code, int k[4]) {
    switch (code) {
        case YGPU_BND_MISMIP3D:
        case YGPU_BND_TROUGH: k[0] = ADV_ZERO; k[1] = ADV_PERIODIC; k[2] = ADV_INFINITE; k[3] = ADV_PERIODIC; break;
        case YGPU_BND_INFINITE: k[0] = k[1] = k[2] = k[3] = ADV_OUTFLOW; break;
        case YGPU_BND_MASK: k[0] = k[1] = k[2] = k[3] = ADV_INFINITE; break;
        case YGPU_BND_PERIODIC: k[0] = k[1] = k[2] = k[3] = ADV_PERIODIC; break;
        case YGPU_BND_PERIODIC_X: k[0] = ADV_PERIODIC; k[1] = ADV_OUTFLOW; k[2] = ADV_PERIODIC; k[3] = ADV_OUTFLOW; break;
        case YGPU_BND_PERIODIC_Y: k[0] = ADV_OUTFLOW; k[1] = ADV_PERIODIC; k[2] = ADV_OUTFLOW; k[3] = ADV_PERIODIC; break;
        default: k[0] = k[1] = k[2] = k[3] = ADV_ZERO; break;
    }
}

/* calc_upwind_faces (:670-755) of all cells, after limit_border_inflow (:646-668)
   on copies of ux, uy */
static void adv_upwind_faces(int nx, int ny, int code, const int* k, const double* ux, const double* uy,
                             const double* H, double* u1, double* u2, double* v1, double* v2, double* Hx1,
                             double* Hx2, double* Hy1, double* Hy2) {
    const size_t n = (size_t)nx * ny;
    double* uxl = malloc(n * sizeof(double));
    double* uyl = malloc(n * sizeof(double));
    memcpy(uxl, ux, n * sizeof(double));
    memcpy(uyl, uy, n * sizeof(double));
    for (int j = 0; j < ny; j++) {
        if (k[2] == ADV_OUTFLOW && uxl[0 + (size_t)nx * j] > 0.0) uxl[0 + (size_t)nx * j] = 0.0;
        if (k[0] == ADV_OUTFLOW && uxl[(nx - 2) + (size_t)nx * j] < 0.0) uxl[(nx - 2) + (size_t)nx * j] = 0.0;
    }
    for (int i = 0; i < nx; i++) {
        if (k[3] == ADV_OUTFLOW && uyl[i] > 0.0) uyl[i] = 0.0;
        if (k[1] == ADV_OUTFLOW && uyl[i + (size_t)nx * (ny - 2)] < 0.0) uyl[i + (size_t)nx * (ny - 2)] = 0.0;
    }
    const int bc = (code == YGPU_BND_MASK) ? YGPU_BND_INFINITE : code;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            int im1, ip1, jm1, jp1;
            nbr(i, j, nx, ny, bc, &im1, &ip1, &jm1, &jp1);
            const size_t c = (size_t)i + (size_t)nx * j;
            u1[c] = uxl[im1 + (size_t)nx * j];
            u2[c] = uxl[c];
            v1[c] = uyl[i + (size_t)nx * jm1];
            v2[c] = uyl[c];
            if (i == 0 && k[2] != ADV_PERIODIC) u1[c] = 0.0;
            if (i == nx - 1 && k[0] != ADV_PERIODIC) u2[c] = 0.0;
            if (j == 0 && k[3] != ADV_PERIODIC) v1[c] = 0.0;
            if (j == ny - 1 && k[1] != ADV_PERIODIC) v2[c] = 0.0;
            Hx1[c] = (u1[c] >= 0.0) ? H[im1 + (size_t)nx * j] : H[c];
            Hx2[c] = (u2[c] >= 0.0) ? H[c] : H[ip1 + (size_t)nx * j];
            Hy1[c] = (v1[c] >= 0.0) ? H[i + (size_t)nx * jm1] : H[c];
            Hy2[c] = (v2[c] >= 0.0) ? H[c] : H[i + (size_t)nx * jp1];
        }
    free(uxl);
    free(uyl);
}

int orc_calc_advec2D_impl_lis(double* dvdt, const double* var, const double* ux, const double* uy,
                              const double* F, const int* mask, const double* Href, double dx, double dy, double dt,
                              int code, int nx, int ny, int* lin_iter, int* lin_status) {
    if (nx < 3 || ny < 3 || !(dt > 0.0)) return YGPU_ERR_BAD_ARG;
    const size_t n = (size_t)nx * ny;
    int k[4];
    adv_kinds(code, k);
    int row_bc[4];
    for (int q = 0; q < 4; q++) row_bc[q] = (k[q] == ADV_ZERO || k[q] == ADV_INFINITE);
    const double dt_darea = dt / (dx * dy), WOVI = 1.0;
    double* buf = calloc(8 * n, sizeof(double));
    double *u1 = buf, *u2 = buf + n, *v1 = buf + 2 * n, *v2 = buf + 3 * n;
    double *Hx1 = buf + 4 * n, *Hx2 = buf + 5 * n, *Hy1 = buf + 6 * n, *Hy2 = buf + 7 * n;
    adv_upwind_faces(nx, ny, code, k, ux, uy, var, u1, u2, v1, v2, Hx1, Hx2, Hy1, Hy2);
    int* ptr = malloc((n + 1) * sizeof(int));
    int* idx = malloc(5 * n * sizeof(int));
    double* val = calloc(5 * n, sizeof(double));
    double* b = malloc(n * sizeof(double));
    double* x = malloc(n * sizeof(double));
    int kk = 0;
    ptr[0] = 0;
    /* rows of linear_solver_matrix_advection_csr_2D (:258-481), row r = i + nx j */
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t r = (size_t)i + (size_t)nx * j;
            const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
            const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
            const int use_border_bc = (mask[r] != 0);
            const double H = var[r];
            if (mask[r] == 1) {
                idx[kk] = (int)r; val[kk++] = 1.0;
                b[r] = Href[r]; x[r] = Href[r];
            } else if (use_border_bc && row_bc[0] && i == nx - 1) {
                if (k[0] == ADV_INFINITE) {
                    idx[kk] = (int)r; val[kk++] = 1.0;
                    idx[kk] = im1 + nx * j; val[kk++] = -1.0;
                    b[r] = 0.0; x[r] = H;
                } else { idx[kk] = (int)r; val[kk++] = 1.0; b[r] = 0.0; x[r] = 0.0; }
            } else if (use_border_bc && row_bc[1] && j == ny - 1) {
                if (k[1] == ADV_INFINITE) {
                    idx[kk] = (int)r; val[kk++] = 1.0;
                    idx[kk] = i + nx * jm1; val[kk++] = -1.0;
                    b[r] = 0.0; x[r] = H;
                } else { idx[kk] = (int)r; val[kk++] = 1.0; b[r] = 0.0; x[r] = 0.0; }
            } else if (use_border_bc && row_bc[2] && i == 0) {
                if (k[2] == ADV_INFINITE) {
                    idx[kk] = (int)r; val[kk++] = 1.0;
                    idx[kk] = ip1 + nx * j; val[kk++] = -1.0;
                    b[r] = 0.0; x[r] = H;
                } else { idx[kk] = (int)r; val[kk++] = 1.0; b[r] = 0.0; x[r] = 0.0; }
            } else if (use_border_bc && row_bc[3] && j == 0) {
                if (k[3] == ADV_INFINITE) {
                    idx[kk] = (int)r; val[kk++] = 1.0;
                    idx[kk] = i + nx * jp1; val[kk++] = -1.0;
                    b[r] = 0.0; x[r] = H;
                } else { idx[kk] = (int)r; val[kk++] = 1.0; b[r] = 0.0; x[r] = 0.0; }
            } else {
                double aS = 0.0, aW = 0.0, aC = 1.0, aE = 0.0, aN = 0.0;
                if (v1[r] > 0.0) aS = -(dt_darea * v1[r] * dx * WOVI);
                if (u1[r] > 0.0) aW = -(dt_darea * u1[r] * dy * WOVI);
                if (v1[r] < 0.0) aC = aC - dt_darea * v1[r] * dx * WOVI;
                if (u1[r] < 0.0) aC = aC - dt_darea * u1[r] * dy * WOVI;
                if (u2[r] > 0.0) aC = aC + dt_darea * u2[r] * dy * WOVI;
                if (v2[r] > 0.0) aC = aC + dt_darea * v2[r] * dx * WOVI;
                if (u2[r] < 0.0) aE = dt_darea * u2[r] * dy * WOVI;
                if (v2[r] < 0.0) aN = dt_darea * v2[r] * dx * WOVI;
                idx[kk] = i + nx * jm1; val[kk++] = aS;
                idx[kk] = im1 + nx * j; val[kk++] = aW;
                idx[kk] = (int)r; val[kk++] = aC;
                idx[kk] = ip1 + nx * j; val[kk++] = aE;
                idx[kk] = i + nx * jp1; val[kk++] = aN;
                const double fx = u2[r] * Hx2[r] * dy - u1[r] * Hx1[r] * dy;
                const double fy = v2[r] * Hy2[r] * dx - v1[r] * Hy1[r] * dx;
                b[r] = H + dt * F[r] - (1.0 - WOVI) * dt_darea * (fx + fy);
                x[r] = H;
            }
            ptr[r + 1] = kk;
        }
    int it = 0;
    double rr = 0.0;
    int st = orc_linear_solve((int)n, ptr, idx, val, b, x, YGPU_LIN_BICGSTAB, YGPU_PRE_JACOBI, 1000, 1e-12, 0, &it,
                              &rr);
    *lin_iter = it;
    *lin_status = st;
    /* calc_fixed_cell_transport on the solution, then dvdt */
    int any_fixed = 0;
    for (size_t c = 0; c < n; c++) any_fixed |= (mask[c] == 1);
    if (any_fixed) adv_upwind_faces(nx, ny, code, k, ux, uy, x, u1, u2, v1, v2, Hx1, Hx2, Hy1, Hy2);
    for (size_t c = 0; c < n; c++) {
        double vn = x[c];
        if (mask[c] == 1)
            vn = var[c] + dt * F[c] - dt_darea * ((u2[c] * Hx2[c] - u1[c] * Hx1[c]) * dy + (v2[c] * Hy2[c] - v1[c] * Hy1[c]) * dx);
        dvdt[c] = (vn - var[c]) / dt;
    }
    free(buf); free(ptr); free(idx); free(val); free(b); free(x);
    return st < 0 ? st : YGPU_OK;
}
